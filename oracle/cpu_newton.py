"""Driver of the C++ CPU restatement oracle/cpu_newton.cpp (test and benchmark
infrastructure; the engine never uses it).

build() compiles it with g++ into oracle/_build/cpu_newton (portable flags: the same source
builds on x86-64 and Arm hosts).  run() writes the configuration and the seeded initial
state to temporary files, runs the program and returns its JSON report.
"""

import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_newton.cpp")
BIN = os.path.join(HERE, "_build", "cpu_newton")


def build():
    """Compile the restatement if its binary is missing or older than the source."""
    if os.path.exists(BIN) and os.path.getmtime(BIN) >= os.path.getmtime(SRC):
        return BIN
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O3", "-pthread", "-o", BIN + ".tmp", SRC]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("cpu_newton build failed:\n" + p.stdout + p.stderr)
    os.replace(BIN + ".tmp", BIN)
    return BIN


def vertex_coords(ini):
    """Vertex coordinates of the configuration's structured grid, lexicographic with x
    fastest (the order of the restatement and of the oracle's mesh)."""
    from .ini import ParameterTree
    g = ParameterTree.from_text(ini).sub("grid")
    dim = g.get_int("dimension", 2)
    cells = [int(v) for v in g.get("cells").split()]
    axes = [np.linspace(0.0, 1.0, c + 1) for c in cells[:dim]]
    grids = np.meshgrid(*axes, indexing="ij")
    return np.stack([a.transpose(tuple(reversed(range(dim)))).ravel() for a in grids], axis=1)


def species_names(ini):
    from .ini import ParameterTree
    return list(ParameterTree.from_text(ini).sub("model").sub("scalar_field").sub_keys())


def initial_state(ini, init):
    """Seeded state (reference order: vertex-major, species interleaved) from
    init(species, coords), or None when the configuration's initial expressions apply."""
    if init is None:
        return None
    names = species_names(ini)
    xyz = vertex_coords(ini)
    x = np.zeros(xyz.shape[0] * len(names))
    for k, nm in enumerate(names):
        v = init(nm, xyz)
        if v is None:
            raise ValueError("init gives no values for species %r" % nm)
        x[k::len(names)] = v
    return x


def run(ini, init=None, iterations=None, warmup=0, threads=1, steps=None, want_state=False, timeout=3600,
        precond="ssor", time_budget=None):
    """Runs the restatement: `warmup` + `iterations` Newton iterations of the time-stepping
    sequence (the last `iterations` timed), or `steps` whole time steps; `precond` is "ssor"
    (the reference's iterative default) or "bjacobi"; with `time_budget` (seconds) no further
    timed iteration starts once the timed ones have taken that long.  Returns the report dict; with
    want_state the final state is under "state"."""
    exe = build()
    with tempfile.TemporaryDirectory() as tmp:
        ini_path = os.path.join(tmp, "model.ini")
        with open(ini_path, "w") as f:
            f.write(ini)
        cmd = [exe, "--ini", ini_path, "--threads", str(int(threads)), "--precond", precond]
        x0 = initial_state(ini, init)
        if x0 is not None:
            sp = os.path.join(tmp, "state.bin")
            x0.astype(np.float64).tofile(sp)
            cmd += ["--state", sp]
        if iterations is not None:
            cmd += ["--iterations", str(int(iterations)), "--warmup", str(int(warmup))]
            if time_budget is not None:
                cmd += ["--time-budget", repr(float(time_budget))]
        if steps is not None:
            cmd += ["--steps", str(int(steps))]
        out = os.path.join(tmp, "out.bin")
        if want_state:
            cmd += ["--out", out]
        p = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
        lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
        rep = json.loads(lines[-1]) if lines else {"error": p.stderr.strip()}
        if p.returncode != 0 or "error" in rep:
            raise RuntimeError(rep.get("error") or p.stderr.strip())
        if want_state:
            rep["state"] = np.fromfile(out, dtype=np.float64)
        return rep
