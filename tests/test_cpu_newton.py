"""The C++ CPU restatement (oracle/cpu_newton.cpp, the timed CPU baseline) against the
numpy oracle: the same states after whole time steps (per species relative L2 <= 1e-10;
both solve each stage to 1e-10 or better) and the same Newton iterations per stage, on
small seeded heat, Gray-Scott and 3D cross-diffusion models, with both preconditioners
and with one and several threads."""

import numpy as np
import pytest

import workloads as W
from oracle import cpu_newton
from oracle.model import OracleModel

CASES = {
    "heat": (lambda: W.heat(n=16, steps=3, dt=0.01), 3),
    "gray_scott": (lambda: W.gray_scott(n=24, steps=2, dt=1.0), 2),
    "cross_diffusion_3d": (lambda: W.cross_diffusion_3d(n=6, steps=2, dt=0.01), 2),
}


def _oracle(ini, init, steps):
    om = OracleModel(ini)
    x = om.initial_state()
    if init is not None:
        for sp in om.species:
            v = om.comp_vertices[sp.comp]
            x[om.dof(sp, v)] = init(sp.name, om.mesh.coords[v])
    t = 0.0
    dt = om.stepper_params()[6]
    per_stage = []
    for _ in range(steps):
        st = {}
        x, t, dt, _ = om.do_step(x, t, dt, st)
        per_stage += st["newton_per_stage"]
    return om, x, per_stage


@pytest.mark.parametrize("precond", ["ssor", "bjacobi"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_cpu_restatement_matches_oracle(case, precond):
    make, steps = CASES[case]
    ini, init = make()
    om, x, per_stage = _oracle(ini, init, steps)
    for threads in (1, 3):
        rep = cpu_newton.run(ini, init, steps=steps, threads=threads, want_state=True, precond=precond)
        assert rep["newton_per_stage"] == per_stage
        for sp in om.species:
            idx = om.dof(sp, om.comp_vertices[sp.comp])
            rel = np.linalg.norm(rep["state"][idx] - x[idx]) / np.linalg.norm(x[idx])
            assert rel <= 1e-10, (case, precond, threads, sp.name, rel)


def test_cpu_restatement_timing_report():
    ini, init = W.cross_diffusion_3d(n=6, steps=10, dt=0.01)
    rep = cpu_newton.run(ini, init, iterations=3, warmup=1, threads=2)
    assert rep["timed_newton_iterations"] == 3 and rep["newton_iterations"] == 4
    assert rep["value"] > 0 and rep["seconds"] > 0
    assert rep["ndof"] == 3 * 7 ** 3


def test_cpu_restatement_rejects_two_compartments():
    ini, init = W.two_compartment(n=8, steps=1)
    with pytest.raises(RuntimeError):
        cpu_newton.run(ini, init, steps=1)
