"""The preconditioner restatement (oracle/precond.py) against closed forms, on the CPU.

The GPU tests compare the engine's multicolour sweeps, factorisations and multigrid cycle
with these functions; here the functions themselves are pinned to textbook identities:
  * one block SSOR sweep pair from zero equals (D/omega + U)^-1 ((2 - omega)/omega) D
    (D/omega + L)^-1 r;
  * block SOR (forward only) equals omega (D + omega L)^-1;
  * ILU(0) on a pattern without fill is the exact LU: M^-1 A = I;
  * DILU on a block-tridiagonal matrix (no fill) is the exact LU as well;
  * a multigrid that coarsens once to a level solved densely, with the exact Galerkin
    operator, reduces to the two-grid formula.
"""

import numpy as np
import pytest

from oracle import precond as P


def tridiag_blocks(n, bs, seed, sym=False):
    rng = np.random.default_rng(seed)
    rowptr = [0]
    colidx = []
    for i in range(n):
        colidx += [j for j in (i - 1, i, i + 1) if 0 <= j < n]
        rowptr.append(len(colidx))
    rowptr = np.array(rowptr)
    colidx = np.array(colidx)
    vals = rng.uniform(-1.0, 1.0, (len(colidx), bs, bs))
    for i in range(n):
        for e in range(rowptr[i], rowptr[i + 1]):
            if colidx[e] == i:
                vals[e] += 6.0 * np.eye(bs)
    if sym:
        A = P.bsr_dense(rowptr, colidx, vals, bs)
        A = 0.5 * (A + A.T)
        for i in range(n):
            for e in range(rowptr[i], rowptr[i + 1]):
                j = colidx[e]
                vals[e] = A[i * bs:(i + 1) * bs, j * bs:(j + 1) * bs]
    return rowptr, colidx, vals


def split(A, n, bs):
    D = np.zeros_like(A)
    for i in range(n):
        D[i * bs:(i + 1) * bs, i * bs:(i + 1) * bs] = A[i * bs:(i + 1) * bs, i * bs:(i + 1) * bs]
    L = np.zeros_like(A)
    U = np.zeros_like(A)
    for i in range(n):
        for j in range(n):
            blk = A[i * bs:(i + 1) * bs, j * bs:(j + 1) * bs]
            if j < i:
                L[i * bs:(i + 1) * bs, j * bs:(j + 1) * bs] = blk
            elif j > i:
                U[i * bs:(i + 1) * bs, j * bs:(j + 1) * bs] = blk
    return D, L, U


@pytest.mark.parametrize("omega", [1.0, 1.4, 0.7])
def test_sor_and_ssor_match_closed_forms(omega):
    n, bs = 9, 2
    rowptr, colidx, vals = tridiag_blocks(n, bs, 1)
    A = P.bsr_dense(rowptr, colidx, vals, bs)
    D, L, U = split(A, n, bs)
    r = np.random.default_rng(2).standard_normal(n * bs)
    order = np.arange(n)
    z = P.sor_apply(rowptr, colidx, vals, bs, order, r, omega, 1, symmetric=False)
    assert np.allclose(z, omega * np.linalg.solve(D + omega * L, r), rtol=1e-12, atol=1e-13)
    z = P.sor_apply(rowptr, colidx, vals, bs, order, r, omega, 1, symmetric=True)
    Mf = (D + omega * L) / omega
    Mb = (D + omega * U) / omega
    want = np.linalg.solve(Mb, ((2.0 - omega) / omega) * D @ np.linalg.solve(Mf, r))
    assert np.allclose(z, want, rtol=1e-12, atol=1e-13)


def test_ilu0_and_dilu_are_exact_without_fill():
    n, bs = 11, 3
    rowptr, colidx, vals = tridiag_blocks(n, bs, 3)
    A = P.bsr_dense(rowptr, colidx, vals, bs)
    x = np.random.default_rng(4).standard_normal(n * bs)
    b = A @ x
    order = np.arange(n)
    assert np.allclose(P.ilu0_apply(rowptr, colidx, vals, bs, order, b), x, rtol=1e-12, atol=1e-12)
    # DILU on a symmetric block-tridiagonal matrix: D_i = A_ii - A_i,i-1 D_{i-1}^-1 A_i-1,i is
    # exactly the block LU pivot, so (D + L) D^-1 (D + U) = A
    rowptr, colidx, vals = tridiag_blocks(n, bs, 5, sym=True)
    A = P.bsr_dense(rowptr, colidx, vals, bs)
    b = A @ x
    assert np.allclose(P.dilu_apply(rowptr, colidx, vals, bs, order, b), x, rtol=1e-12, atol=1e-12)
    # relaxation scales the result
    z2 = P.dilu_apply(rowptr, colidx, vals, bs, order, b, omega=0.5)
    assert np.allclose(z2, 0.5 * x, rtol=1e-12, atol=1e-12)


def test_two_grid_cycle_matches_formula():
    n, bs = 12, 2
    rowptr, colidx, vals = tridiag_blocks(n, bs, 6)
    A = P.bsr_dense(rowptr, colidx, vals, bs)
    agg = np.repeat(np.arange(n // 3), 3)

    def aggregate(rp, ci, g, d):
        return agg if len(rp) - 1 == n else None, n // 3

    levels = P.amg_hierarchy(rowptr, colidx, vals, bs, None, aggregate, coarsen_target=n // 3)
    assert len(levels) == 2
    Pm = np.zeros((n * bs, (n // 3) * bs))
    for i in range(n):
        Pm[i * bs:(i + 1) * bs, agg[i] * bs:(agg[i] + 1) * bs] = np.eye(bs)
    Ac = Pm.T @ A @ Pm
    assert np.allclose(P.bsr_dense(*levels[1][:3], bs), Ac, rtol=1e-13, atol=1e-13)
    D, _L, _U = split(A, n, bs)
    S = np.linalg.inv(D)
    w = 0.85
    r = np.random.default_rng(7).standard_normal(n * bs)
    t = w * S @ r
    y = t + Pm @ np.linalg.solve(Ac, Pm.T @ (r - A @ t))
    want = y + w * S @ (r - A @ y)
    got = P.amg_apply(levels, bs, r, "jacobi", w)
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12)
