"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from the oracle).

CPU: the oracle reproduces the committed fixtures on this machine (pins the oracle across
numpy/scipy builds and hosts).  GPU: the engine matches the committed fixtures after every
step, per species relative L2 <= 1e-8, Newton iterations of every stage within +-1.
"""

import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
NAMES = ["heat", "gray_scott", "two_compartment", "cross_diffusion_3d"]
TOL = 1e-8


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _per_species_rel(om, a, b):
    out = {}
    for sp in om.species:
        idx = om.dof(sp, om.comp_vertices[sp.comp])
        nb = np.linalg.norm(b[idx])
        out[sp.name] = np.linalg.norm(a[idx] - b[idx]) / (nb if nb > 0 else 1.0)
    return out


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    data = load(name)
    fresh = make_golden.run_case(name)
    assert str(fresh["ini"]) == str(data["ini"])
    np.testing.assert_allclose(fresh["x0"], data["x0"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(fresh["times"], data["times"], rtol=0, atol=1e-14)
    assert np.array_equal(fresh["newton"], data["newton"])
    from oracle.model import OracleModel
    om = OracleModel(str(data["ini"]))
    for k in range(data["states"].shape[0]):
        errs = _per_species_rel(om, fresh["states"][k], data["states"][k])
        assert max(errs.values()) <= 1e-10, (name, k, errs)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_engine_matches_golden(dcgpu_lib, name):
    from oracle.model import OracleModel
    data = load(name)
    ini = str(data["ini"])
    om = OracleModel(ini)
    gm = dcgpu_lib.Model(ini)
    t0 = float(om.stepper_params()[2])
    gm.set_state(data["x0"], t0)
    dt = float(om.stepper_params()[6])
    for k in range(data["states"].shape[0]):
        info = gm.step(dt)
        dt = info["dt_next"]
        assert info["time"] == pytest.approx(float(data["times"][k]), rel=0, abs=1e-14)
        errs = _per_species_rel(om, gm.state(), data["states"][k])
        assert max(errs.values()) <= TOL, (name, k, errs)
        want = [int(v) for v in data["newton"][k]]
        got = info["newton_per_stage"]
        assert len(got) == len(want), (name, k, want, got)
        assert all(abs(a - b) <= 1 for a, b in zip(want, got)), (name, k, want, got)
    gm.close()
