"""Request server: admission by device-memory budget, concurrent execution, and results
that are identical alone and in the mix."""

import numpy as np
import pytest

import cases

FAILING_INI = """
[grid]
cells = 6 6
[compartments.domain]
expression = 1
[model.scalar_field.u]
compartment = domain
initial.expression = 1
storage.expression = 1
reaction.expression = log(u - 2)
reaction.jacobian.u.expression = 1/(u - 2)
cross_diffusion.u.expression = 0.1
[model.time_step_operator]
type = ImplicitEuler
time_end = 1
time_step_initial = 0.1
time_step_min = 0.02
time_step_max = 0.1
"""


def _requests():
    out = []
    for ini, init in (cases.small_heat(n=20, steps=4), cases.small_gray_scott(n=20, steps=3),
                      cases.small_two_compartment(n=14, steps=3), cases.small_3d(n=4, steps=2)):
        x0 = None
        if init is not None:
            from oracle.model import OracleModel
            om = OracleModel(ini)
            x0 = om.initial_state()
            for sp in om.species:
                verts = om.comp_vertices[sp.comp]
                x0[om.dof(sp, verts)] = init(sp.name, om.mesh.coords[verts])
        out.append((ini, x0))
    return out


def _drain(server, n):
    results = {}
    while len(results) < n:
        for r in server.poll(wait=True):
            results[r["request_id"]] = r
    return results


def test_estimate_grows_with_problem_size(dcgpu_lib):
    small = dcgpu_lib.estimate_bytes(cases.small_gray_scott(n=16)[0])
    large = dcgpu_lib.estimate_bytes(cases.small_gray_scott(n=64)[0])
    assert 0 < small < large
    # 16x the cells; the estimate carries a fixed 1 MiB allowance
    assert (large - (1 << 20)) / (small - (1 << 20)) > 8


@pytest.mark.gpu
def test_results_identical_alone_and_in_the_mix(dcgpu_lib):
    reqs = _requests()
    alone = []
    srv = dcgpu_lib.Server(budget_bytes=8 << 30, max_active=1)
    for ini, x0 in reqs:
        rid = srv.submit(ini, init=x0)
        res = _drain(srv, 1)[rid]
        assert res["status"] == 0
        alone.append(srv.take_state(rid))
    srv.close()
    srv = dcgpu_lib.Server(budget_bytes=8 << 30, max_active=4)
    ids = [srv.submit(ini, init=x0) for ini, x0 in reqs]
    res = _drain(srv, len(ids))
    for k, rid in enumerate(ids):
        assert res[rid]["status"] == 0
        assert res[rid]["latency_s"] >= res[rid]["run_s"] > 0
        assert res[rid]["newton_iterations"] > 0
        assert np.array_equal(srv.take_state(rid), alone[k]), k
    srv.close()


@pytest.mark.gpu
def test_admission_respects_budget(dcgpu_lib):
    ini, _ = cases.small_heat(n=32, steps=6)
    est = dcgpu_lib.estimate_bytes(ini)
    # a budget of one estimate: a running simulation is charged its measured footprint
    # (> 0), so the next one (charged its estimate at admission) never fits beside it
    srv = dcgpu_lib.Server(budget_bytes=est, max_active=4)
    ids = [srv.submit(ini) for _ in range(3)]
    res = _drain(srv, 3)
    spans = []
    for rid in ids:
        r = res[rid]
        assert r["status"] == 0
        spans.append((r["queue_s"], r["queue_s"] + r["run_s"]))
    # only one request fits the budget at a time: the admission windows do not overlap
    spans.sort()
    for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
        assert b0 >= a1 - 1e-3
    srv.close()


@pytest.mark.gpu
def test_measured_footprint_is_reported_and_within_the_estimate(dcgpu_lib):
    """Every result carries the peak device bytes of the simulation's buffers, which the
    server charges instead of the admission estimate; the estimate bounds it."""
    srv = dcgpu_lib.Server(budget_bytes=8 << 30, max_active=3)
    # configurations whose own initial state is a proper start (no seeded perturbation)
    reqs = [cases.small_heat(n=24, steps=4)[0], cases.small_3d(n=5, steps=2)[0],
            cases.small_two_compartment(n=24, steps=3)[0]]
    ids = [srv.submit(ini) for ini in reqs]
    res = _drain(srv, len(ids))
    for rid in ids:
        r = res[rid]
        assert r["status"] == 0
        assert 0 < r["bytes_measured"] <= r["bytes_estimate"], r
    srv.close()


@pytest.mark.gpu
def test_oversized_request_rejected(dcgpu_lib):
    ini, _ = cases.small_heat(n=32, steps=2)
    srv = dcgpu_lib.Server(budget_bytes=1 << 20, max_active=2)
    rid = srv.submit(ini)
    res = _drain(srv, 1)
    assert res[rid]["status"] == 4
    srv.close()


@pytest.mark.gpu
def test_failure_is_isolated(dcgpu_lib):
    good_ini, _ = cases.small_heat(n=16, steps=3)
    srv = dcgpu_lib.Server(budget_bytes=4 << 30, max_active=1)
    rid = srv.submit(good_ini)
    _drain(srv, 1)
    ref = srv.take_state(rid)
    srv.close()
    srv = dcgpu_lib.Server(budget_bytes=4 << 30, max_active=3)
    a = srv.submit(good_ini)
    b = srv.submit(FAILING_INI)
    c = srv.submit(good_ini)
    res = _drain(srv, 3)
    assert res[b]["status"] == 2
    assert res[a]["status"] == 0 and res[c]["status"] == 0
    assert np.array_equal(srv.take_state(a), ref)
    assert np.array_equal(srv.take_state(c), ref)
    srv.close()


MIXED = {"model.time_step_operator.linear_solver.precision": "mixed"}


def _run_server(dcgpu_lib, reqs, max_active, batch_krylov, overrides=None):
    srv = dcgpu_lib.Server(budget_bytes=8 << 30, max_active=max_active, batch_krylov=batch_krylov)
    ids = [srv.submit(ini, overrides=overrides, init=x0) for ini, x0 in reqs]
    res = _drain(srv, len(ids))
    states = []
    for rid in ids:
        assert res[rid]["status"] == 0, res[rid]
        states.append(srv.take_state(rid))
    stats = srv.batch_stats()
    stats["tuned_grids"] = srv.batch_tuning()
    srv.close()
    return states, [res[rid] for rid in ids], stats


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_results_identical_alone_and_in_the_mix(dcgpu_lib, precision):
    """Continuous batching of the Krylov solves: each request's result is bitwise the same
    whether its solves ran alone in the batch or packed with other requests' solves (block
    sizes 1, 2, 3 and 5 side by side), and within 1e-8 of the unbatched server's."""
    ov = MIXED if precision == "mixed" else None
    reqs = _requests()
    alone = [_run_server(dcgpu_lib, [rq], 1, True, ov)[0][0] for rq in reqs]
    mixed_states, results, stats = _run_server(dcgpu_lib, reqs, len(reqs), True, ov)
    for k in range(len(reqs)):
        assert np.array_equal(mixed_states[k], alone[k]), k
    # the block-Jacobi BiCGSTAB solves went through the batch (a solve that switches to the
    # multigrid runs on the simulation's own stream)
    assert stats["solves"] > 0 and stats["replays"] > 0
    assert 0 < stats["iterations"] <= sum(r["linear_iterations"] for r in results)
    assert stats["slot_replays"] >= stats["replays"]
    assert 1 <= stats["max_active"] <= len(reqs)
    # the launch-shape autotuner settles on one of the captured grids per bucket it timed
    for lane in stats["tuned_grids"].values():
        assert all(g in (32, 128) or g % 4 == 0 for g in lane.values())
    unbatched, _, ustats = _run_server(dcgpu_lib, reqs, len(reqs), False, ov)
    assert ustats["solves"] == 0
    for k in range(len(reqs)):
        ref = unbatched[k]
        err = np.linalg.norm(mixed_states[k] - ref) / np.linalg.norm(ref)
        assert err <= 1e-8, (k, err)


@pytest.mark.gpu
def test_batched_server_matches_oracle(dcgpu_lib):
    """A batched request's final state against the oracle's time stepping of the same
    model (per-species relative L2 <= 1e-8), served next to three other requests."""
    from oracle.model import OracleModel
    reqs = _requests()
    states, results, _ = _run_server(dcgpu_lib, reqs, len(reqs), True, MIXED)
    for k in (1, 3):  # Gray-Scott 20^2 (bs 2) and the 3D cross-diffusion 4^3 (bs 3)
        ini, x0 = reqs[k]
        om = OracleModel(ini)
        x = om.initial_state() if x0 is None else x0.copy()
        _dec, _inc, t0, t1, _mn, _mx, dt0 = om.stepper_params()
        x, _t, _dt = om.evolve(x, t0, dt0, t1)
        for sp in om.species:
            idx = om.dof(sp, om.comp_vertices[sp.comp])
            ref = x[idx]
            err = np.linalg.norm(states[k][idx] - ref) / max(np.linalg.norm(ref), 1e-300)
            assert err <= 1e-8, (k, sp.name, err)


@pytest.mark.gpu
def test_batched_failure_is_isolated(dcgpu_lib):
    """A request whose Newton fails leaves the batch and the others' results unchanged."""
    good_ini, _ = cases.small_heat(n=16, steps=3)
    ref = _run_server(dcgpu_lib, [(good_ini, None)], 1, True)[0][0]
    srv = dcgpu_lib.Server(budget_bytes=4 << 30, max_active=3, batch_krylov=True)
    a = srv.submit(good_ini)
    b = srv.submit(FAILING_INI)
    c = srv.submit(good_ini)
    res = _drain(srv, 3)
    assert res[b]["status"] == 2
    assert res[a]["status"] == 0 and res[c]["status"] == 0
    assert np.array_equal(srv.take_state(a), ref)
    assert np.array_equal(srv.take_state(c), ref)
    srv.close()
