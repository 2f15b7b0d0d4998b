"""Benchmark-size runs checked through size-independent properties (the CPU oracle cannot
finish these sizes in seconds):

* heat, 128^2 (16,641 DOF), implicit Euler to T = 1: total mass (sum of M x) is conserved to
  1e-12 with zero-flux boundaries, and the discrete maximum principle holds;
* Gray-Scott, 512^2 (526,338 DOF), two Alexander2 steps: the fp64 path and the fp32-Krylov /
  fp64-refinement path agree to 1e-8 per species (relative L2);
* two compartments, 1024^2 cells, 5 + 5 species (~5.3 M DOF), one implicit Euler step with the
  multigrid preconditioner: fp64 and mixed precision agree to 1e-8 per species;
* 3D, 128^3 cubes x 6 tetrahedra (6.4 M DOF), one Alexander2 step: fp64 and mixed agree to 1e-8.
"""

import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu


def _layout(model):
    """[(species names of one compartment, vertex ids, DOF offset)] in DOF order."""
    out = []
    names = model.species
    off = 0
    i = 0
    while i < len(names):
        verts = model.species_vertices(names[i])
        group = [names[i]]
        j = i + 1
        while j < len(names) and np.array_equal(model.species_vertices(names[j]), verts):
            group.append(names[j])
            j += 1
        out.append((group, verts, off))
        off += len(group) * len(verts)
        i = j
    return out


def _unit_coords(model, verts):
    """Vertex coordinates of the structured unit square / cube grid."""
    dim = model.info["dim"]
    n = int(round(model.info["n_vertices"] ** (1.0 / dim))) - 1
    idx = np.asarray(verts)
    return np.stack([(idx // (n + 1) ** d) % (n + 1) / n for d in range(dim)], axis=1)


def _seeded_state(model, init):
    x = model.state()
    if init is None:
        return x
    for group, verts, off in _layout(model):
        ns = len(group)
        cv = _unit_coords(model, verts)
        for k, name in enumerate(group):
            x[off + k: off + ns * len(verts): ns] = init(name, cv)
    return x


def _per_species_rel(model, a, b):
    errs = {}
    for group, verts, off in _layout(model):
        ns = len(group)
        for k, name in enumerate(group):
            sa = a[off + k: off + ns * len(verts): ns]
            sb = b[off + k: off + ns * len(verts): ns]
            nb = np.linalg.norm(sb)
            errs[name] = np.linalg.norm(sa - sb) / (nb if nb > 0 else 1.0)
    return errs


def test_heat_128_conserves_mass(dcgpu_lib):
    ini, _ = W.heat(n=128, steps=100, dt=0.01)
    m = dcgpu_lib.Model(ini)
    x0 = m.state()
    r0, _ = m.assemble(x0, 0.0, 1.0, 0.0, jacobian=False)
    m.evolve(1.0, 0.01)
    assert m.time() == pytest.approx(1.0, abs=1e-12)
    x1 = m.state()
    r1, _ = m.assemble(x1, 1.0, 1.0, 0.0, jacobian=False)
    assert abs(r1.sum() - r0.sum()) <= 1e-12 * abs(r0.sum())
    assert x1.min() >= -1e-10 and x1.max() <= x0.max() + 1e-10
    m.close()


def _two_precisions(dcgpu_lib, ini, init, steps, dt, overrides=None):
    finals = []
    ref_model = None
    for mixed in (False, True):
        m = dcgpu_lib.Model(ini, overrides)
        m.set_mixed_precision(mixed)
        m.set_state(_seeded_state(m, init), 0.0)
        d = dt
        for _ in range(steps):
            d = m.step(d)["dt_next"]
        finals.append(m.state())
        if ref_model is None:
            ref_model = m
        else:
            m.close()
    errs = _per_species_rel(ref_model, finals[1], finals[0])
    ref_model.close()
    return errs


def test_gray_scott_512_mixed_matches_fp64(dcgpu_lib):
    ini, init = W.gray_scott(n=512, steps=2, dt=1.0)
    errs = _two_precisions(dcgpu_lib, ini, init, 2, 1.0)
    assert max(errs.values()) <= 1e-8, errs


def test_two_compartment_1024_mixed_matches_fp64(dcgpu_lib):
    ini, init = W.two_compartment(n=1024, steps=1, dt=0.05)
    ov = {"model.time_step_operator.linear_solver.preconditioner.type": "AMG"}
    errs = _two_precisions(dcgpu_lib, ini, init, 1, 0.05, ov)
    assert max(errs.values()) <= 1e-8, errs


def test_cross_diffusion_3d_128_mixed_matches_fp64(dcgpu_lib):
    ini, init = W.cross_diffusion_3d(n=128, steps=1, dt=0.01)
    errs = _two_precisions(dcgpu_lib, ini, init, 1, 0.01)
    assert max(errs.values()) <= 1e-8, errs
