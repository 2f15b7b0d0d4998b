"""Preconditioners on the GPU against their CPU restatement (oracle/precond.py).

Synthetic block matrices on the pattern of a structured triangulated grid (7 neighbours per
row, two groups of rows standing for two compartments, coupled across the interface): the
multicolour SSOR / SOR / ILU(0) / DILU and the aggregation multigrid applied once on the
device must equal the sequential restatement in the engine's row order (colour order) to
1e-12 relative (fp64) or 1e-5 (fp32, multigrid 1e-4); the colouring must be proper and the
aggregation must respect groups and the independent-set distance.  Then every registry
entry drives the time stepping of the small configurations against the oracle's direct
solves (1e-8 per species, Newton iterations per stage within +-1).
"""

import numpy as np
import pytest

import cases
from oracle import precond as P

pytestmark = pytest.mark.gpu

LS = "model.time_step_operator.linear_solver."


def grid_matrix(nx, ny, bs, seed, split=True):
    """Block matrix on an nx x ny grid with the 7-point triangulated stencil; rows with
    x < nx / 2 form group 0, the rest group 1.  Off-diagonal blocks are negative-ish and
    random, diagonal blocks dominate (nonsymmetric, well conditioned)."""
    rng = np.random.default_rng(seed)
    n = nx * ny
    offs = [(0, 0), (1, 0), (-1, 0), (0, 1), (0, -1), (1, 1), (-1, -1)]
    rowptr = [0]
    colidx = []
    for j in range(ny):
        for i in range(nx):
            cols = sorted((j + dj) * nx + (i + di) for di, dj in offs if 0 <= i + di < nx and 0 <= j + dj < ny)
            colidx += cols
            rowptr.append(len(colidx))
    rowptr = np.array(rowptr, np.int32)
    colidx = np.array(colidx, np.int32)
    vals = np.zeros((len(colidx), bs, bs))
    for r in range(n):
        dsum = np.zeros(bs)
        for e in range(rowptr[r], rowptr[r + 1]):
            if colidx[e] == r:
                continue
            b = -rng.uniform(0.1, 1.0, (bs, bs)) * rng.uniform(0.0, 1.0, (bs, bs)) ** 2
            vals[e] = b
            dsum += np.abs(b).sum(axis=1)
        for e in range(rowptr[r], rowptr[r + 1]):
            if colidx[e] == r:
                d = rng.uniform(-0.2, 0.2, (bs, bs))
                d[np.diag_indices(bs)] = dsum + np.abs(d).sum(axis=1) + rng.uniform(0.1, 1.0, bs)
                vals[e] = d
    group = np.array([0 if (r % nx) < nx // 2 else 1 for r in range(n)], np.int32) if split else None
    return rowptr, colidx, vals, group


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_colouring_is_proper_and_deterministic(dcgpu_lib):
    rowptr, colidx, _v, _g = grid_matrix(33, 21, 1, 1)
    col, nc = dcgpu_lib.color_graph(rowptr, colidx)
    col2, nc2 = dcgpu_lib.color_graph(rowptr, colidx)
    assert np.array_equal(col, col2) and nc == nc2
    assert col.min() == 0 and col.max() == nc - 1
    for i in range(len(rowptr) - 1):
        for e in range(rowptr[i], rowptr[i + 1]):
            j = colidx[e]
            assert j == i or col[i] != col[j]
    assert nc <= 7  # at most the maximal degree + 1


@pytest.mark.parametrize("distance", [1, 2])
def test_aggregation_respects_groups_and_distance(dcgpu_lib, distance):
    nx, ny = 30, 17
    rowptr, colidx, _v, group = grid_matrix(nx, ny, 1, 2)
    agg, na = dcgpu_lib.aggregate_graph(rowptr, colidx, group, distance)
    agg2, _ = dcgpu_lib.aggregate_graph(rowptr, colidx, group, distance)
    assert np.array_equal(agg, agg2)
    n = len(rowptr) - 1
    assert agg.min() == 0 and agg.max() == na - 1 and len(np.unique(agg)) == na
    assert 1 < na < n
    nbrs = [[c for c in colidx[rowptr[i]:rowptr[i + 1]] if c != i and group[c] == group[i]] for i in range(n)]
    for a in range(na):
        members = np.flatnonzero(agg == a)
        assert len(set(group[members])) == 1
        # a centre within `distance` of every member, through rows of the same group
        ok = False
        for c in members:
            reach = {c}
            front = {c}
            for _ in range(distance):
                front = {j for i in front for j in nbrs[i]} - reach
                reach |= front
            if set(members) <= reach:
                ok = True
                break
        assert ok, (a, members)


CASES = [("SSOR", "", 1), ("SSOR", "relaxation=1.3;iterations=2", 3), ("SOR", "relaxation=0.8", 2),
         ("ILU", "", 1), ("ILU", "relaxation=0.9", 4), ("DILU", "", 2), ("DILU", "relaxation=1.1", 5)]


@pytest.mark.parametrize("kind,params,bs", CASES)
@pytest.mark.parametrize("fp32", [False, True])
def test_multicolour_preconditioners_match_restatement(dcgpu_lib, kind, params, bs, fp32):
    rowptr, colidx, vals, _g = grid_matrix(17, 13, bs, 10 + bs)
    n = len(rowptr) - 1
    r = np.random.default_rng(3).standard_normal(n * bs)
    z, info = dcgpu_lib.precond_apply(kind, rowptr, colidx, vals, r, bs, params, fp32=fp32)
    col, nc = dcgpu_lib.color_graph(rowptr, colidx)
    assert info[0] == nc
    order = P.color_order(col)
    kv = dict(kv.split("=") for kv in params.split(";") if kv)
    omega = float(kv.get("relaxation", 1.0))
    its = int(kv.get("iterations", 1))
    if kind in ("SSOR", "SOR"):
        want = P.sor_apply(rowptr, colidx, vals, bs, order, r, omega, its, symmetric=kind == "SSOR")
    elif kind == "ILU":
        want = P.ilu0_apply(rowptr, colidx, vals, bs, order, r, omega)
    else:
        want = P.dilu_apply(rowptr, colidx, vals, bs, order, r, omega)
    assert rel(z, want) <= (1e-5 if fp32 else 1e-12), (kind, params, bs, rel(z, want))


def test_ilu0_is_exact_on_a_full_pattern(dcgpu_lib):
    """On a full block pattern (every row a colour of its own, nothing to drop) ILU(0) is
    the exact LU in the colour order: M^-1 A x = x."""
    n, bs = 12, 3
    rowptr = np.arange(0, n * n + 1, n, dtype=np.int32)
    colidx = np.tile(np.arange(n, dtype=np.int32), n)
    rng = np.random.default_rng(7)
    vals = rng.uniform(-1, 1, (n * n, bs, bs))
    for i in range(n):
        vals[i * n + i] += 4.0 * n * np.eye(bs)
    x = rng.standard_normal(n * bs)
    b = P.bsr_dense(rowptr, colidx, vals, bs) @ x
    z, info = dcgpu_lib.precond_apply("ILU", rowptr, colidx, vals, b, bs)
    assert info[0] == n
    assert rel(z, x) <= 1e-12


AMG_CASES = [("jacobi", 2, 1, ""), ("jacobi", 1, 2, ""), ("l1jacobi", 2, 3, ""), ("gauss_seidel", 2, 2, ""),
             ("gauss_seidel", 1, 1, ""), ("jacobi", 2, 2, "max_level=2"), ("gauss_seidel", 2, 4, "coarsen_target=3"),
             ("jacobi", 2, 5, "coarse_correction=1.6;warp_rows_below=0"),
             ("l1jacobi", 1, 3, "coarse_correction=1.3;warp_rows_below=100000"),
             ("gauss_seidel", 2, 2, "coarse_correction=1.5;warp_rows_below=200"),
             ("jacobi", 2, 3, "finest_post_smoothing=0"), ("l1jacobi", 2, 2, "finest_post_smoothing=0;warp_rows_below=0"),
             ("ilu0", 2, 2, ""), ("ilu0", 1, 3, "warp_rows_below=0"),
             ("jacobi", 2, 3, "w_levels=1"), ("l1jacobi", 1, 2, "w_levels=2;warp_rows_below=0")]
SMOOTHER_ID = {"jacobi": 0, "l1jacobi": 1, "gauss_seidel": 2, "ilu0": 3}


@pytest.mark.parametrize("smoother,distance,bs,extra", AMG_CASES)
@pytest.mark.parametrize("fp32", [False, True])
def test_multigrid_matches_restatement(dcgpu_lib, smoother, distance, bs, extra, fp32):
    nx, ny = (40, 40) if "max_level" in extra else (27, 23)
    rowptr, colidx, vals, group = grid_matrix(nx, ny, bs, 20 + bs)
    n = len(rowptr) - 1
    r = np.random.default_rng(5).standard_normal(n * bs)
    omega = 0.85 if smoother == "jacobi" else 1.0
    params = "smoother=%d;aggregation_distance=%d;%s" % (SMOOTHER_ID[smoother], distance, extra)
    z, info = dcgpu_lib.precond_apply("AMG", rowptr, colidx, vals, r, bs, params, group=group, fp32=fp32)
    kv = dict(kv.split("=") for kv in extra.split(";") if kv)

    def aggregate(rp, ci, g, d):
        return dcgpu_lib.aggregate_graph(rp, ci, g, d)

    def colour(rp, ci):
        return dcgpu_lib.color_graph(rp, ci)[0]

    levels = P.amg_hierarchy(rowptr, colidx, vals, bs, group, aggregate, distance,
                             coarsen_target=int(kv.get("coarsen_target", 0)),
                             max_levels=int(kv.get("max_level", 10)))
    assert int(info[0]) == len(levels)
    for l, lv in enumerate(levels[:6]):
        assert int(info[2 + l]) == len(lv[0]) - 1
    last_n = (len(levels[-1][0]) - 1) * bs
    assert int(info[1]) == (last_n if last_n <= P.DENSE_MAX else 0)
    if "max_level" in extra:
        assert info[1] == 0  # the coarsest level is above the dense limit: smoother sweeps
    want = P.amg_apply(levels, bs, r, smoother, omega, colour=colour,
                       correction=float(kv.get("coarse_correction", 1.0)),
                       finest_post_smoothing=kv.get("finest_post_smoothing", "1") != "0",
                       w_levels=int(kv.get("w_levels", 0)))
    assert rel(z, want) <= (1e-4 if fp32 else 1e-11), (smoother, distance, bs, extra, rel(z, want))


# ---------------------------------------------------------------- time stepping
def _steps_match(dcgpu_lib, case, overrides, mixed=False):
    from test_gpu_parity import ALL_CASES, _run_both, assert_newton_per_stage, STEP_TOL
    ini, init = ALL_CASES[case]()
    records = _run_both(dcgpu_lib, ini, init, mixed=mixed, overrides=overrides)
    assert records
    for t, errs, n_o, n_g in records:
        for name, e in errs.items():
            assert e <= STEP_TOL, (case, overrides, t, name, e)
        assert_newton_per_stage(n_o, n_g, (case, t))


REGISTRY = [("SSOR", {}), ("SSOR", {"preconditioner.relaxation": "1.2", "preconditioner.iterations": "2"}),
            ("SOR", {}), ("GaussSeidel", {}), ("ILU", {}), ("ILDL", {}), ("DILU", {}), ("Richardson", {}),
            ("BlockJacobi", {}), ("InverseOperator", {})]


@pytest.mark.parametrize("precond,extra", REGISTRY)
@pytest.mark.parametrize("case", ["two_compartment", "cross_diffusion_3d"])
def test_registry_preconditioners_match_oracle(dcgpu_lib, precond, extra, case):
    ov = {LS + "preconditioner.type": precond}
    ov.update({LS + k: v for k, v in extra.items()})
    _steps_match(dcgpu_lib, case, ov)


@pytest.mark.parametrize("precond", ["SSOR", "ILU", "DILU"])
@pytest.mark.parametrize("solver", ["BiCGSTAB", "RestartedGMRes", "mixed"])
def test_registry_preconditioners_with_solvers(dcgpu_lib, precond, solver):
    ov = {LS + "preconditioner.type": precond}
    if solver != "mixed":
        ov.update({LS + "type": solver, LS + "convergence_condition.relative_tolerance": "1e-12",
                   "model.time_step_operator.nonlinear_solver.convergence_condition.relative_tolerance": "1e-24"})
        from test_gpu_parity import ALL_CASES, _run_both, STEP_TOL
        ini, init = ALL_CASES["features_2d"]()
        records = _run_both(dcgpu_lib, ini, init, overrides=ov)
        for t, errs, n_o, n_g in records:
            for e in errs.values():
                assert e <= STEP_TOL, (precond, solver, t, e)
    else:
        _steps_match(dcgpu_lib, "gray_scott", ov, mixed=True)


@pytest.mark.timeout(300, method="thread")
@pytest.mark.parametrize("smoother,mixed", [("jacobi", False), ("l1jacobi", False), ("gauss_seidel", False),
                                            ("ilu0", False), ("jacobi", True), ("l1jacobi", True),
                                            ("gauss_seidel", True)])
@pytest.mark.parametrize("distance", ["1", "2"])
def test_multigrid_smoothers_match_oracle(dcgpu_lib, smoother, distance, mixed):
    ov = {LS + "preconditioner.type": "AMG", LS + "preconditioner.smoother": smoother,
          LS + "preconditioner.aggregation_distance": distance}
    _steps_match(dcgpu_lib, "two_compartment", ov, mixed=mixed)


def test_preconditioner_configuration_errors(dcgpu_lib):
    ini, _init = cases.small_heat()
    for key, val in [("preconditioner.type", "Multigrid"), ("preconditioner.relaxation", "2.5"),
                     ("preconditioner.iterations", "0"), ("preconditioner.smoother", "chebyshev"),
                     ("preconditioner.aggregation_distance", "3")]:
        ov = {LS + "preconditioner.type": "AMG" if "smoother" in key or "aggregation" in key else "SSOR"}
        ov[LS + key] = val
        with pytest.raises(dcgpu_lib.DcError):
            dcgpu_lib.Model(ini, ov)
