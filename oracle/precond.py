"""CPU restatement of the engine's preconditioners (test infrastructure: only tests use it;
the engine never calls it).

The reference builds its preconditioner from dune-istl (dune-istl 2.9/2.10, the version its
dune-pdelab >= 2.9 dependency pins; registry in
dune/copasi/solver/istl/factory/preconditioner.hh:88-118): SeqSSOR (the default), SeqSOR,
SeqGS, SeqILU, SeqDILU.  dune-istl is not part of the reference tree; its published
algorithms are restated here:
  * block SOR sweep over the rows in a given order:
        z_i <- z_i + omega D_i^-1 (r_i - sum_j A_ij z_j)
    SSOR = a forward then a backward sweep, `iterations` times, from z = 0; SOR and
    Gauss-Seidel = forward sweeps only;
  * block ILU(0) in the IKJ order (no fill outside the pattern): for every row i, for every
    earlier column k of row i in increasing order, L_ik = A_ik U_kk^-1 and A_ij -= L_ik U_kj
    for the later columns j of row k present in row i; z = U^-1 L^-1 (omega r);
  * block DILU: D_i = A_ii - sum over earlier k of A_ik D_k^-1 A_ki; z solves
    (D + L) D^-1 (D + U) z = omega r.
The engine sweeps the rows in the order of a colouring of the block-row graph (rows ordered
by colour, then by index); rows of one colour are never adjacent, so the engine's
colour-parallel launches compute exactly the sequential sweep in that order, which is what
these functions take as `order`.

The multigrid restatement (no reference counterpart; the engine's addition) follows
dune-copasi_gb300/csrc/amg.hpp: aggregation per level (taken as input: the engine's own
deterministic aggregation of the same graph), piecewise-constant prolongation, Galerkin
coarse operators, a V(1,1) cycle with damped block Jacobi, L1-Jacobi or Gauss-Seidel
or ILU(0) smoothing, and a dense direct solve on a coarsest level of at most 128 unknowns.
"""

import numpy as np

DENSE_MAX = 128


def block(vals, e, bs):
    return np.asarray(vals[e], dtype=np.float64).reshape(bs, bs)


def diag_index(rowptr, colidx):
    n = len(rowptr) - 1
    d = np.full(n, -1, np.int64)
    for i in range(n):
        for e in range(rowptr[i], rowptr[i + 1]):
            if colidx[e] == i:
                d[i] = e
    assert np.all(d >= 0), "every row needs its diagonal block"
    return d


def color_order(colour):
    """Rows ordered by colour, then by index."""
    colour = np.asarray(colour)
    return np.lexsort((np.arange(len(colour)), colour))


def sor_apply(rowptr, colidx, vals, bs, order, r, omega=1.0, iterations=1, symmetric=True):
    """Block SSOR (symmetric) or SOR: `iterations` sweeps from z = 0 in the row order
    `order` (backward sweeps in the reverse order)."""
    n = len(rowptr) - 1
    vals = np.asarray(vals, dtype=np.float64).reshape(-1, bs, bs)
    d = diag_index(rowptr, colidx)
    dinv = [np.linalg.inv(vals[d[i]]) for i in range(n)]
    r = np.asarray(r, dtype=np.float64).reshape(n, bs)
    z = np.zeros((n, bs))

    def sweep(rows):
        for i in rows:
            t = r[i].copy()
            for e in range(rowptr[i], rowptr[i + 1]):
                t -= vals[e] @ z[colidx[e]]
            z[i] = z[i] + omega * (dinv[i] @ t)

    for _ in range(iterations):
        sweep(order)
        if symmetric:
            sweep(order[::-1])
    return z.reshape(-1)


def ilu0_apply(rowptr, colidx, vals, bs, order, r, omega=1.0):
    """Block ILU(0) of the matrix with its rows and columns in the order `order`, applied
    to omega r."""
    n = len(rowptr) - 1
    lu = np.array(vals, dtype=np.float64).reshape(-1, bs, bs)
    pos = np.empty(n, np.int64)
    pos[np.asarray(order)] = np.arange(n)
    d = diag_index(rowptr, colidx)
    uinv = [None] * n
    for i in order:
        lower = sorted((pos[colidx[e]], e) for e in range(rowptr[i], rowptr[i + 1]) if pos[colidx[e]] < pos[i])
        for pk, e in lower:
            k = colidx[e]
            lu[e] = lu[e] @ uinv[k]
            for f in range(rowptr[k], rowptr[k + 1]):
                j = colidx[f]
                if pos[j] <= pk:
                    continue
                for g in range(rowptr[i], rowptr[i + 1]):
                    if colidx[g] == j:
                        lu[g] = lu[g] - lu[e] @ lu[f]
                        break
        uinv[i] = np.linalg.inv(lu[d[i]])
    r = np.asarray(r, dtype=np.float64).reshape(n, bs)
    z = np.zeros((n, bs))
    for i in order:  # unit lower triangle
        t = omega * r[i]
        for e in range(rowptr[i], rowptr[i + 1]):
            if pos[colidx[e]] < pos[i]:
                t = t - lu[e] @ z[colidx[e]]
        z[i] = t
    for i in order[::-1]:
        t = z[i].copy()
        for e in range(rowptr[i], rowptr[i + 1]):
            if pos[colidx[e]] > pos[i]:
                t = t - lu[e] @ z[colidx[e]]
        z[i] = uinv[i] @ t
    return z.reshape(-1)


def dilu_apply(rowptr, colidx, vals, bs, order, r, omega=1.0):
    """Block DILU in the row order `order`, applied to omega r."""
    n = len(rowptr) - 1
    vals = np.asarray(vals, dtype=np.float64).reshape(-1, bs, bs)
    pos = np.empty(n, np.int64)
    pos[np.asarray(order)] = np.arange(n)
    d = diag_index(rowptr, colidx)
    dinv = [None] * n
    for i in order:
        di = vals[d[i]].copy()
        for e in range(rowptr[i], rowptr[i + 1]):
            k = colidx[e]
            if pos[k] >= pos[i]:
                continue
            for f in range(rowptr[k], rowptr[k + 1]):
                if colidx[f] == i:
                    di = di - (vals[e] @ dinv[k]) @ vals[f]
                    break
        dinv[i] = np.linalg.inv(di)
    r = np.asarray(r, dtype=np.float64).reshape(n, bs)
    z = np.zeros((n, bs))
    for i in order:
        t = omega * r[i]
        for e in range(rowptr[i], rowptr[i + 1]):
            if pos[colidx[e]] < pos[i]:
                t = t - vals[e] @ z[colidx[e]]
        z[i] = dinv[i] @ t
    for i in order[::-1]:
        t = np.zeros(bs)
        for e in range(rowptr[i], rowptr[i + 1]):
            if pos[colidx[e]] > pos[i]:
                t = t - vals[e] @ z[colidx[e]]
        z[i] = z[i] + dinv[i] @ t
    return z.reshape(-1)


# ---------------------------------------------------------------- multigrid
def bsr_dense(rowptr, colidx, vals, bs):
    n = len(rowptr) - 1
    vals = np.asarray(vals, dtype=np.float64).reshape(-1, bs, bs)
    a = np.zeros((n * bs, n * bs))
    for i in range(n):
        for e in range(rowptr[i], rowptr[i + 1]):
            j = colidx[e]
            a[i * bs:(i + 1) * bs, j * bs:(j + 1) * bs] = vals[e]
    return a


def coarse_level(rowptr, colidx, vals, bs, agg, na, group):
    """Pattern (sorted columns), Galerkin values P^T A P and row groups of the coarse level
    of aggregation `agg`."""
    n = len(rowptr) - 1
    vals = np.asarray(vals, dtype=np.float64).reshape(-1, bs, bs)
    rows = [dict() for _ in range(na)]
    for i in range(n):
        I = agg[i]
        for e in range(rowptr[i], rowptr[i + 1]):
            J = agg[colidx[e]]
            rows[I][J] = rows[I].get(J, 0.0) + vals[e]
    crp = np.zeros(na + 1, np.int64)
    cci, cval = [], []
    for I in range(na):
        for J in sorted(rows[I]):
            cci.append(J)
            cval.append(rows[I][J])
        crp[I + 1] = len(cci)
    cgrp = np.zeros(na, np.int64)
    if group is not None:
        for i in range(n - 1, -1, -1):
            cgrp[agg[i]] = group[i]
    return crp, np.array(cci, np.int64), np.array(cval).reshape(-1, bs, bs), cgrp


def amg_hierarchy(rowptr, colidx, vals, bs, group, aggregate, distance=2, coarsen_target=0, max_levels=10):
    """Levels [(rowptr, colidx, vals, agg-to-next or None)] built with `aggregate(rowptr,
    colidx, group, distance) -> (agg, na)` (the engine's aggregation), by the engine's
    rules: stop at `coarsen_target` rows (0: the dense solve's limit, 128 unknowns), at
    max_levels, or when an aggregation keeps at least 90 % of the rows."""
    target = coarsen_target if coarsen_target > 0 else max(1, DENSE_MAX // bs)
    levels = []
    rp, ci, v, g = np.asarray(rowptr), np.asarray(colidx), np.asarray(vals, dtype=np.float64).reshape(-1, bs, bs), group
    while True:
        n = len(rp) - 1
        if len(levels) + 1 >= max_levels or n <= target:
            levels.append((rp, ci, v, None))
            break
        agg, na = aggregate(rp, ci, g, distance)
        if na >= 0.9 * n:
            levels.append((rp, ci, v, None))
            break
        levels.append((rp, ci, v, np.asarray(agg)))
        rp, ci, v, g = coarse_level(rp, ci, v, bs, np.asarray(agg), na, g)
    return levels


def amg_apply(levels, bs, r, smoother="jacobi", omega=0.8, coarse_sweeps=6, colour=None, correction=1.0,
              finest_post_smoothing=True, w_levels=0):
    """One V(1,1) cycle z = M^-1 r with the coarse-grid correction scaled by `correction`.
    colour(rowptr, colidx) -> colours (Gauss-Seidel only: the engine's colouring of the
    level's graph)."""

    def smoother_inverse(rp, ci, v):
        n = len(rp) - 1
        d = diag_index(rp, ci)
        out = []
        for i in range(n):
            a = v[d[i]].copy()
            if smoother == "l1jacobi":
                for e in range(rp[i], rp[i + 1]):
                    if e == d[i]:
                        continue
                    m = np.abs(v[e]).sum(axis=1)
                    a[np.diag_indices(bs)] += np.where(np.diag(a) < 0.0, -m, m)
            out.append(np.linalg.inv(a))
        return np.array(out)

    def matvec(rp, ci, v, x):
        n = len(rp) - 1
        x = x.reshape(n, bs)
        y = np.zeros((n, bs))
        for i in range(n):
            for e in range(rp[i], rp[i + 1]):
                y[i] += v[e] @ x[ci[e]]
        return y.reshape(-1)

    def bdiag(S, x):
        return np.einsum("nij,nj->ni", S, x.reshape(-1, bs)).reshape(-1)

    def cycle(l, rl):
        rp, ci, v, agg = levels[l]
        n = len(rp) - 1
        if agg is None:
            if n * bs <= DENSE_MAX:
                return np.linalg.solve(bsr_dense(rp, ci, v, bs), rl)
            # a coarsest level above the dense limit: damped block-Jacobi sweeps
            D = np.array([np.linalg.inv(v[e]) for e in diag_index(rp, ci)])
            x = omega * bdiag(D, rl)
            for _ in range(1, coarse_sweeps):
                x = x + omega * bdiag(D, rl - matvec(rp, ci, v, x))
            return x
        na = int(agg.max()) + 1

        def restrict(u):
            rc = np.zeros((na, bs))
            np.add.at(rc, agg, u.reshape(n, bs))
            return rc.reshape(-1)

        def prolong(xc):
            return xc.reshape(na, bs)[agg].reshape(-1)

        if smoother == "ilu0":
            order = color_order(colour(rp, ci))
            x = ilu0_apply(rp, ci, v, bs, order, rl)
            xc = cycle(l + 1, restrict(rl - matvec(rp, ci, v, x)))
            x = x + correction * prolong(xc)
            return x + ilu0_apply(rp, ci, v, bs, order, rl - matvec(rp, ci, v, x))
        if smoother == "gauss_seidel":
            order = color_order(colour(rp, ci))
            x = sor_apply(rp, ci, v, bs, order, rl, omega, 1, symmetric=False)
            xc = cycle(l + 1, restrict(rl - matvec(rp, ci, v, x)))
            x = x + correction * prolong(xc)
            # backward sweep from the corrected iterate
            xs = x.reshape(n, bs).copy()
            d = diag_index(rp, ci)
            r2 = rl.reshape(n, bs)
            for i in order[::-1]:
                t = r2[i].copy()
                for e in range(rp[i], rp[i + 1]):
                    t -= v[e] @ xs[ci[e]]
                xs[i] = xs[i] + omega * (np.linalg.inv(v[d[i]]) @ t)
            return xs.reshape(-1)
        S = smoother_inverse(rp, ci, v)
        t = omega * bdiag(S, rl)
        xc = cycle(l + 1, restrict(rl - matvec(rp, ci, v, t)))
        if l < w_levels:  # W-cycle on this level: a second coarse-grid correction
            t = t + correction * prolong(xc)
            xc = cycle(l + 1, restrict(rl - matvec(rp, ci, v, t)))
        y = t + correction * prolong(xc)
        if l == 0 and not finest_post_smoothing:
            return y
        return y + omega * bdiag(S, rl - matvec(rp, ci, v, y))

    return cycle(0, np.asarray(r, dtype=np.float64))
