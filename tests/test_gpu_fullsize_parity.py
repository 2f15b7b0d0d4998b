"""The four benchmark configurations at full size against the oracle's fixtures.

tests/golden/make_fullsize.py ran the oracle on each configuration at the size the
benchmark quotes it on (heat 128^2 for all 100 steps, Gray-Scott 512^2 for 2 Alexander2
steps, two compartments 1024^2 and cross-diffusion 128^3 x 6 tetrahedra for one step) and
stored, after every step, the Newton iterations of every stage and per species the L2 norm,
the sum and a seeded sample of vertex values.  Here the engine runs the same steps from the
same seeded state, plain FP64 and mixed precision (fp32 Krylov inside fp64 refinement), and
after every step must give:
  * per species, relative L2 over the sampled vertex values <= 1e-8, and the species'
    L2 norm within 1e-8 (relative) of the oracle's;
  * the same stage solves, with Newton iterations per stage equal within +-1.
The CPU test checks the fixtures' own consistency (shapes, initial-state norms against a
freshly built oracle state for the 2D ones).
"""

import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
NAMES = ["heat_128", "gray_scott_512", "two_compartment_1024", "cross_diffusion_3d_128"]
TOL = 1e-8


def load(name):
    path = os.path.join(GOLDEN, "fullsize_%s.npz" % name)
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated" % path)
    return np.load(path)


def workload(data):
    import workloads as W
    g = json.loads(str(data["generator"]))
    return getattr(W, g["name"])(**g["kwargs"])


@pytest.mark.parametrize("name", NAMES)
def test_fullsize_fixture_is_consistent(name):
    data = load(name)
    nsteps = data["times"].shape[0]
    nsp = data["species"].shape[0]
    assert data["norms"].shape == (nsteps, nsp)
    assert data["samples"].shape == (nsteps, nsp, data["sample_idx"].shape[1])
    assert data["newton"].shape[0] == nsteps
    assert np.all(np.diff(data["times"]) > 0)
    ini, _init = workload(data)
    assert ini == str(data["ini"])
    if name in ("heat_128", "gray_scott_512"):
        # the initial state is cheap to rebuild on the CPU for the 2D single-compartment
        # configurations: its norms pin the seeded state the engine must start from
        import sys
        from oracle.model import OracleModel
        if GOLDEN not in sys.path:
            sys.path.insert(0, GOLDEN)
        import make_fullsize as L
        om = OracleModel(ini)
        x = L.initial_state(om, _init)
        for k, nm in enumerate(data["species"]):
            v = om.species_values(x, str(nm))
            assert np.linalg.norm(v) == pytest.approx(float(data["x0_norms"][k]), rel=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", NAMES)
def test_engine_matches_fullsize_fixture(dcgpu_lib, name, precision):
    data = load(name)
    ini, init = workload(data)
    gm = dcgpu_lib.Model(ini)
    if precision == "mixed":
        gm.set_mixed_precision(True)
    gm.set_state(gm.seeded_state(init), 0.0)
    names = [str(n) for n in data["species"]]
    idx = data["sample_idx"]
    for k, nm in enumerate(names):
        assert np.linalg.norm(gm.species_values(nm)) == pytest.approx(float(data["x0_norms"][k]), rel=1e-13)
    dt = float(np.diff(np.concatenate([[0.0], data["times"]]))[0])
    for step in range(data["times"].shape[0]):
        info = gm.step(dt)
        dt = info["dt_next"]
        assert info["time"] == pytest.approx(float(data["times"][step]), rel=0, abs=1e-12)
        want = [int(v) for v in data["newton"][step]]
        got = info["newton_per_stage"]
        assert len(got) == len(want), (name, step, want, got)
        assert all(abs(a - b) <= 1 for a, b in zip(want, got)), (name, step, want, got)
        for k, nm in enumerate(names):
            v = gm.species_values(nm)
            ref = data["samples"][step, k]
            rel = np.linalg.norm(v[idx[k]] - ref) / max(np.linalg.norm(ref), 1e-300)
            assert rel <= TOL, (name, precision, step, nm, rel)
            nref = float(data["norms"][step, k])
            assert abs(np.linalg.norm(v) - nref) <= TOL * max(nref, 1e-300), (name, precision, step, nm)
    gm.close()
