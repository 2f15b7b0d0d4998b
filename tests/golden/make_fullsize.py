"""Full-size fixtures of the four benchmark configurations, computed by the oracle.

    python tests/golden/make_fullsize.py [name ...]

Names (the configurations at the sizes the benchmark quotes them on):
  heat_128                 unit square 128 x 128 P1, one species, implicit Euler dt 0.01,
                           all 100 steps to T = 1 (SuperLU direct solve)
  gray_scott_512           Gray-Scott 512 x 512 P1, Alexander2 dt 1, the first 2 steps
                           (SuperLU direct solve)
  two_compartment_1024     two compartments on 1024 x 1024 P1, 5 + 5 species, implicit
                           Euler dt 0.05, the first step
  cross_diffusion_3d_128   unit cube 128^3 x 6 tetrahedra, 3 species, Alexander2 dt 0.01,
                           the first step

SuperLU cannot factor the last two stage systems in this machine's memory (5.26 M and
6.44 M unknowns), so the oracle solves them with BiCGSTAB + Jacobi inside iterative
refinement to a relative true residual of 1e-13, or of the rounding floor of the fp64
residual where that lies above (at most 1e-10) (OracleModel(linear="iterative")); Newton
then takes the same iterates as with an exact solve up to that residual.

Each fixture holds the configuration text, the workload generator and its arguments (so
the seeded initial state can be rebuilt), the per-species norms of the initial state, and
after every step: the time, the Newton iterations of every stage, and per species the L2
norm, the sum and a seeded sample of vertex values (2048 per species for heat_128, 10^4
otherwise; indices into the species' vertex list, ascending vertex id).
"""

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "dune-copasi_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import workloads as W  # noqa: E402
from oracle.model import OracleModel  # noqa: E402

# name -> (generator, keyword arguments, steps, oracle linear solve, sample size)
CONFIGS = {
    "heat_128": ("heat", {"n": 128, "steps": 100, "dt": 0.01}, 100, "direct", 2048),
    "gray_scott_512": ("gray_scott", {"n": 512, "steps": 2, "dt": 1.0}, 2, "direct", 10000),
    "two_compartment_1024": ("two_compartment", {"n": 1024, "steps": 1, "dt": 0.05}, 1, "iterative", 10000),
    "cross_diffusion_3d_128": ("cross_diffusion_3d", {"n": 128, "steps": 1, "dt": 0.01}, 1, "iterative", 10000),
}
SAMPLE_SEED = 20261204


def workload(name):
    gen, kw, _steps, _lin, _ns = CONFIGS[name]
    return getattr(W, gen)(**kw)


def initial_state(om, init):
    x = om.initial_state()
    if init is not None:
        for sp in om.species:
            verts = om.comp_vertices[sp.comp]
            x[om.dof(sp, verts)] = init(sp.name, om.mesh.coords[verts])
    return x


def sample_indices(sizes, n_sample):
    """Seeded sample of vertex positions per species (sorted, without repetition)."""
    rng = np.random.default_rng(SAMPLE_SEED)
    out = np.zeros((len(sizes), n_sample), np.int64)
    for k, m in enumerate(sizes):
        out[k] = np.sort(rng.choice(m, size=n_sample, replace=False))
    return out


def run(name, log=print):
    gen, kw, steps, linear, n_sample = CONFIGS[name]
    ini, init = workload(name)
    om = OracleModel(ini, linear=linear)
    x = initial_state(om, init)
    names = [sp.name for sp in om.species]
    sizes = [om.comp_vertices[sp.comp].shape[0] for sp in om.species]
    n_sample = min(n_sample, min(sizes))
    idx = sample_indices(sizes, n_sample)

    def per_species(v):
        vals = [om.species_values(v, nm) for nm in names]
        return (np.array([np.linalg.norm(a) for a in vals]), np.array([a.sum() for a in vals]),
                np.stack([a[idx[k]] for k, a in enumerate(vals)]))

    x0_norms, x0_sums, _ = per_species(x)
    _dec, _inc, t, _t1, _mn, _mx, dt = om.stepper_params()
    times, newton, norms, sums, samples = [], [], [], [], []
    for k in range(steps):
        st = {}
        t_start = time.time()
        x, t, dt, _used = om.do_step(x, t, dt, st)
        if st.get("failed_steps"):
            raise RuntimeError("%s: step %d needed a smaller dt; the fixture expects none" % (name, k))
        nrm, sm, smp = per_species(x)
        times.append(t)
        newton.append(st["newton_per_stage"])
        norms.append(nrm)
        sums.append(sm)
        samples.append(smp)
        log("%s step %d t=%.6g newton/stage=%s (%.1f s)" % (name, k + 1, t, st["newton_per_stage"],
                                                             time.time() - t_start))
    return {"ini": np.array(ini), "generator": np.array(json.dumps({"name": gen, "kwargs": kw})),
            "oracle_linear": np.array(linear), "species": np.array(names), "sample_idx": idx,
            "x0_norms": x0_norms, "x0_sums": x0_sums, "times": np.array(times),
            "newton": np.array(newton, np.int64), "norms": np.array(norms), "sums": np.array(sums),
            "samples": np.array(samples), "ndof": np.array(om.ndof)}


def main(argv):
    todo = argv or list(CONFIGS)
    for name in todo:
        t0 = time.time()
        data = run(name)
        path = os.path.join(HERE, "fullsize_%s.npz" % name)
        np.savez_compressed(path, **data)
        print("wrote %s (%.0f s)" % (path, time.time() - t0), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
