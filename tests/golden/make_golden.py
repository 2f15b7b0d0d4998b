"""Regenerate the golden fixtures of this directory from the CPU oracle.

    python tests/golden/make_golden.py

Each fixture stores, for one small seeded model of tests/cases.py, the initial state,
the state after every time step, the step times and the Newton iterations per stage, as
computed by the oracle (numpy assembly + SuperLU).  The CPU tests check that the oracle
still reproduces them; the GPU tests check the engine against them.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "dune-copasi_gb300"), os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)

import cases  # noqa: E402
from oracle.model import OracleModel  # noqa: E402

CASES = {
    "heat": cases.small_heat,
    "gray_scott": cases.small_gray_scott,
    "two_compartment": cases.small_two_compartment,
    "cross_diffusion_3d": cases.small_3d,
}


def initial(om, init):
    x = om.initial_state()
    if init is not None:
        for sp in om.species:
            verts = om.comp_vertices[sp.comp]
            x[om.dof(sp, verts)] = init(sp.name, om.mesh.coords[verts])
    return x


def run_case(name):
    ini, init = CASES[name]()
    om = OracleModel(ini)
    x = initial(om, init)
    _dec, _inc, t0, t1, _mn, _mx, dt = om.stepper_params()
    states, times, newton = [], [], []
    t = t0
    x0 = x.copy()
    while t < t1 - 1e-12:
        st = {}
        x, t, dt, _used = om.do_step(x, t, dt, st)
        states.append(x.copy())
        times.append(t)
        newton.append(st.get("newton_per_stage", []))
    return {"ini": np.array(ini), "x0": x0, "states": np.array(states), "times": np.array(times),
            "newton": np.array(newton, dtype=np.int64)}


def main():
    for name in CASES:
        data = run_case(name)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print("wrote", path, data["states"].shape)


if __name__ == "__main__":
    main()
