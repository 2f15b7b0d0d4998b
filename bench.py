"""Benchmark: DOF x Newton-steps per second of the implicit time step on one GB300.

Headline workload (the largest configuration that fits one GPU): seeded 3D
cross-diffusion, unit cube 128^3 cubes x 6 P1 tetrahedra (12,582,912 cells, 2,146,689
vertices, 3 species, 6,440,067 DOF), Michaelis-Menten reactions and a full 3 x 3
cross-diffusion matrix, Alexander2 DIRK dt = 0.01, Newton relative tolerance 1e-10 on the
squared l2 norm (as the reference), direct-solve semantics (the reference's default
UMFPack is replaced by BiCGSTAB + block Jacobi converged to a relative residual of 1e-10).
`--workload gray_scott | two_compartment | heat` selects the other configurations.

A "step" is one Alexander2 time step (2 stages x Newton iterations).  Timed per step with
CUDA events on the engine's stream (dc_step_info.device_ms); the operator (1.36 GB fp32,
3.6 GB fp64) and the element buffers are far larger than L2, and a 256 MiB write flushes L2
between timed steps as well.  value = DOF x Newton iterations of all timed steps / sum of
device step times, for the mixed-precision path (fp32 Krylov in fp64 refinement);
"plain_fp64" is the plain FP64 path on the same workload and steps, with the per-species
relative L2 deviation of the mixed state from it.  e2e = the same metric through the public
C ABI with host buffers: state upload from pinned host memory, step, state download,
host-timed.  "secondary" holds the Gray-Scott 512^2 and two-compartment 1024^2
configurations, "preconditioners" block Jacobi, the multigrid, multicolour SSOR / ILU(0) and
the engine's adaptive default side by side on heat 128^2 and two compartments 1024^2, and
"serving" a Poisson stream of random requests through the request server.

--impl reference times the CPU restatement of the reference algorithm (C++, std::thread
colour-parallel assembly, BiCGSTAB + block Jacobi, or + SSOR as the reference's iterative
default with --cpu-precond ssor; built from oracle/cpu_newton.cpp) on all host cores: each
bench step is one Newton iteration of the same time-stepping sequence on the same workload.

Multi-GPU: independent replicas (one model per rank), no collective; scaling "weak".
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "dune-copasi_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "DOF·Newton-steps/s"

# name -> (generator, default size, dt, scheme, local vertices per cell)
WORKLOADS = {
    "cross_diffusion_3d": ("cross_diffusion_3d", 128, 0.01, "Alexander2", 4),
    "gray_scott": ("gray_scott", 512, 1.0, "Alexander2", 3),
    "two_compartment": ("two_compartment", 1024, 0.05, "ImplicitEuler", 3),
    "heat": ("heat", 128, 0.01, "ImplicitEuler", 3),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cross_diffusion_3d", choices=sorted(WORKLOADS))
    # "--grid" is the spelling to use after a torchrun launcher, whose own parser reads
    # "--n" as an ambiguous abbreviation of its options
    ap.add_argument("--n", "--grid", dest="n", type=int, default=0,
                    help="mesh size (grid edge in 2D, cube edge in 3D); 0 = the configuration's own")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="mixed (default): fp32 Krylov in fp64 refinement, measured against the plain "
                         "FP64 path on the same workload; fp64: the plain path alone")
    ap.add_argument("--no-plain-fp64", action="store_true",
                    help="skip the plain FP64 comparison run of the mixed path")
    ap.add_argument("--spmv", default="auto", choices=["auto", "bsr", "sell"],
                    help="layout of the fp32 Krylov operator (linear_solver.spmv)")
    ap.add_argument("--precond", default="auto", choices=["auto", "Jacobi", "AMG", "SSOR", "ILU", "DILU"],
                    help="BiCGSTAB preconditioner (linear_solver.preconditioner.type; auto, the engine's "
                         "default: block Jacobi, the multigrid once a solve needs more than 100 iterations)")
    ap.add_argument("--no-precond-comparison", action="store_true",
                    help="skip the block-Jacobi / multigrid / SSOR comparison on heat 128^2 and two "
                         "compartments 1024^2")
    ap.add_argument("--single-launch", default="on", choices=["on", "off"],
                    help="BiCGSTAB as one cooperative launch per solve (on) or one launch per "
                         "phase from a CUDA graph (off) (linear_solver.single_launch)")
    ap.add_argument("--inner-reduction", type=float, default=None,
                    help="mixed precision: residual reduction of each fp32 correction solve "
                         "(linear_solver.inner_reduction; engine default 1e-4)")
    ap.add_argument("--override", action="append", default=[],
                    help="extra engine configuration key=value (repeatable)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-iterations", type=int, default=1,
                    help="timed Newton iterations of the CPU baseline leg (after one untimed)")
    ap.add_argument("--cpu-1core-iterations", type=int, default=0,
                    help="timed Newton iterations of the CPU baseline on one core (0: not run)")
    ap.add_argument("--minimal", action="store_true",
                    help="the timed steps only (no plain FP64, profile, end-to-end, SpMV, CPU, secondary or "
                         "serving runs): for profiling a step under ncu")
    ap.add_argument("--cpu-precond", default="bjacobi", choices=["bjacobi", "ssor"],
                    help="preconditioner of the CPU restatement's BiCGSTAB: block Jacobi (the GPU path's) "
                         "or SSOR (the reference's iterative default)")
    ap.add_argument("--no-spmv-phase", action="store_true",
                    help="skip the per-phase SpMV measurement on the headline operator")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the Gray-Scott 512^2 and two-compartment 1024^2 measurements")
    ap.add_argument("--serve-spec", action="store_true",
                    help="serving requests drawn at their specified sizes (2D N 32..512, 3D N 16..64, 20-500 "
                         "steps; mixed and FP64 both with the server's concurrency) instead of the reduced mix; "
                         "--serve-requests of them (the specification's 512 take about a GPU-hour per precision)")
    ap.add_argument("--serve-active", type=int, default=16,
                    help="simulations the request server runs at once (each on its own stream)")
    ap.add_argument("--serve-requests", type=int, default=32,
                    help="requests of the Poisson serving stream (0 disables the serving measurement)")
    return ap.parse_args()


def max_over_ranks(x, dist):
    """The largest of the ranks' values (the slowest replica sets the time); x itself when
    not distributed."""
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # one GPU per rank: restrict the rank's view before any CUDA initialisation
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    return rank, world


def workload_desc(kind, n):
    """Static description of a workload (no GPU needed): the `config` both arms print."""
    gen, n0, dt, scheme, nl = WORKLOADS[kind]
    n = n or n0
    if kind == "cross_diffusion_3d":
        desc = {"workload": "cross_diffusion_3d_%d^3x6_p1_tets_alexander2_dt0.01" % n,
                "mesh": "%d^3 cubes x 6 P1 tetrahedra" % n, "cells": 6 * n ** 3, "dof": 3 * (n + 1) ** 3,
                "species": 3}
    elif kind == "gray_scott":
        desc = {"workload": "gray_scott_%dx%d_p1_alexander2_dt1" % (n, n), "mesh": "%dx%d P1 triangles" % (n, n),
                "cells": 2 * n * n, "dof": 2 * (n + 1) ** 2, "species": 2}
    elif kind == "two_compartment":
        desc = {"workload": "two_compartment_%dx%d_p1_5+5_species_implicit_euler_dt0.05" % (n, n),
                "mesh": "%dx%d P1 triangles, disk r=0.3 + annulus" % (n, n), "cells": 2 * n * n, "species": 10}
    else:
        desc = {"workload": "heat_%dx%d_p1_implicit_euler_dt0.01" % (n, n), "mesh": "%dx%d P1 triangles" % (n, n),
                "cells": 2 * n * n, "dof": (n + 1) ** 2, "species": 1}
    desc.update({"scheme": scheme, "dt": dt, "newton_rel_tol_sq": 1e-10})
    return desc


def make_workload(kind, n):
    """(ini, init, dt, nl, description) of a workload."""
    import workloads as W
    gen, n0, dt, _scheme, nl = WORKLOADS[kind]
    n = n or n0
    kw = {"n": n, "steps": 100000, "dt": dt}
    ini, init = getattr(W, gen)(**kw)
    return ini, init, dt, nl, workload_desc(kind, n)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


# ----------------------------------------------------------------------------- CPU legs
def cpu_newton_run(kind, n, iterations, warmup, threads, precond, time_budget=None):
    """The C++ CPU restatement (oracle/cpu_newton.cpp) on the same workload: `warmup` +
    `iterations` Newton iterations of the time-stepping sequence (fewer timed ones when
    `time_budget` seconds run out first); returns its JSON report."""
    from oracle import cpu_newton
    ini, init, dt, _nl, _desc = make_workload(kind, n)
    return cpu_newton.run(ini, init, iterations=iterations, warmup=warmup, threads=threads, precond=precond,
                          time_budget=time_budget)


def cpu_baseline(kind, n, iterations, precond, one_core_iterations=0):
    """CPU baseline leg of the GPU arm: a bounded sample (Newton iterations of the same
    time-stepping sequence, after one untimed iteration) on all host cores; optionally the
    same on one core."""
    threads = os.cpu_count() or 1
    rep = cpu_newton_run(kind, n, iterations, 1, threads, precond)
    out = {"value": rep["value"], "unit": METRIC, "cores": threads, "kind": "port",
           "sample": "%d Newton iteration(s) (residual + Jacobian assembly on %d threads, BiCGSTAB + %s to "
                     "1e-10) of the %d-DOF stage systems of the first time step, after one untimed iteration"
                     % (iterations, threads, rep["precond"], rep["ndof"]),
           "seconds": rep["seconds"], "assembly_seconds": rep["assembly_seconds"],
           "solve_seconds": rep["solve_seconds"], "krylov_iterations": rep["krylov_iterations"],
           "cpu": rep.get("cpu", "")}
    if one_core_iterations > 0:
        one = cpu_newton_run(kind, n, one_core_iterations, 0, 1, precond)
        out["value_1core"] = one["value"]
    return out


# the reference arm's timed Newton iterations stop once they have taken this long, and it
# runs at most one untimed iteration first (a Newton iteration of the 128^3 workload takes
# tens of seconds on a host CPU): the whole arm then ends within a few minutes
REFERENCE_TIME_BUDGET_S = 120.0


def run_reference(args, rank, world):
    if rank != 0:
        return
    desc = workload_desc(args.workload, args.n)
    threads = os.cpu_count() or 1
    warm = min(args.warmup, 1)
    try:
        rep = cpu_newton_run(args.workload, args.n, args.steps, warm, threads, args.cpu_precond,
                             time_budget=REFERENCE_TIME_BUDGET_S)
    except Exception as e:  # the restatement covers one-compartment models only
        print(json.dumps({"impl": "reference", "unavailable": "CPU restatement: %s" % e}), flush=True)
        return
    value = rep["value"]
    done = int(rep["timed_newton_iterations"])
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": done, "warmup": warm, "requested_steps": args.steps, "requested_warmup": args.warmup,
            "ms_per_step": 1e3 * rep["seconds"] / max(done, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded initial state, no dataset)",
            "config": desc,
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": "one Newton iteration of the time-stepping sequence per step (assembly on "
                                       "%d threads, BiCGSTAB + %s to 1e-10); at most %d warm-up iteration and "
                                       "%.0f s of timed iterations" % (threads, rep["precond"], warm,
                                                                      REFERENCE_TIME_BUDGET_S),
                             "cpu": rep.get("cpu", "")},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "detail": {"assembly_seconds": rep["assembly_seconds"], "solve_seconds": rep["solve_seconds"],
                       "krylov_iterations": rep["krylov_iterations"], "setup_seconds": rep["setup_seconds"]}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- serving
SERVE_REDUCED = {"n2d": (32, 160), "n3d": (12, 32), "steps": (10, 40)}
# the serving stream at the size its specification names: 2D N log-uniform 32..512, 3D
# N log-uniform 16..64, 20-500 implicit-Euler steps (--serve-spec)
SERVE_SPEC = {"n2d": (32, 512), "n3d": (16, 64), "steps": (20, 500)}


def run_serving(dcgpu, n_requests, lam, max_active, precision, seed=20261203, budget=64 << 30, mix=None,
                batch=False):
    """Poisson stream of random requests through the request server; returns latency
    percentiles and the aggregate DOF x Newton-step throughput.  batch: the server packs
    the running simulations' Krylov solves into one continuously batched solve."""
    import workloads as W
    mix = mix or SERVE_REDUCED
    stream = W.serving_stream(n_requests, lam, seed, n2d=mix["n2d"], n3d=mix["n3d"], steps=mix["steps"])
    ov = {"model.time_step_operator.linear_solver.precision": "mixed"} if precision == "mixed" else None
    srv = dcgpu.Server(budget, max_active, batch_krylov=batch)
    t0 = time.perf_counter()
    done = {}
    for arrival, ini in stream:
        while True:
            now = time.perf_counter() - t0
            for r in srv.poll(wait=False):
                done[r["request_id"]] = r
            if now >= arrival:
                break
            time.sleep(min(arrival - now, 0.002))
        srv.submit(ini, overrides=ov)
    while len(done) < len(stream):
        for r in srv.poll(wait=True):
            done[r["request_id"]] = r
    wall = time.perf_counter() - t0
    bstats = srv.batch_stats() if batch else None
    if batch:
        bstats["tuned_grids"] = srv.batch_tuning()
    srv.close()
    lat = sorted(r["latency_s"] for r in done.values())
    ok = sum(1 for r in done.values() if r["status"] == 0)
    work = sum(r["n_dof"] * r["newton_iterations"] for r in done.values())
    import numpy as np
    return {"requests": len(stream), "ok": ok, "lambda_per_s": lam, "max_active": max_active,
            "precision": precision, "krylov_batched": batch, "batch_stats": bstats,
            "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "wall_s": wall,
            "value": work / wall, "unit": METRIC,
            "bytes_measured_max": max((r.get("bytes_measured", 0) for r in done.values()), default=0),
            "setup_s_sum": sum(r.get("setup_s", 0.0) for r in done.values()),
            "run_s_sum": sum(r["run_s"] for r in done.values()),
            "mix": "2D N log-U[%d,%d] / 3D N log-U[%d,%d], 1-2 compartments, 1-8 species, %d-%d IE steps"
                   % (mix["n2d"] + mix["n3d"] + mix["steps"])}


def run_burst(dcgpu, copies, n, steps, batch, budget=16 << 30):
    """`copies` identical 3D cross-diffusion models (n^3 x 6 tetrahedra, mixed precision)
    submitted together, so that their Krylov solves coincide; aggregate DOF x Newton-step
    throughput over the burst's wall time."""
    import workloads as W
    ini, _ = W.cross_diffusion_3d(n=n, steps=steps, dt=0.01)
    ov = {"model.time_step_operator.linear_solver.precision": "mixed"}
    srv = dcgpu.Server(budget, copies, batch_krylov=batch)
    t0 = time.perf_counter()
    for _ in range(copies):
        srv.submit(ini, overrides=ov)
    done = {}
    while len(done) < copies:
        for r in srv.poll(wait=True):
            done[r["request_id"]] = r
    wall = time.perf_counter() - t0
    bstats = srv.batch_stats() if batch else None
    if batch:
        bstats["tuned_grids"] = srv.batch_tuning()
    srv.close()
    work = sum(r["n_dof"] * r["newton_iterations"] for r in done.values())
    return {"copies": copies, "model": "cross_diffusion_3d_%d^3x6_mixed_%d_steps" % (n, steps),
            "ok": sum(1 for r in done.values() if r["status"] == 0), "wall_s": wall, "value": work / wall,
            "unit": METRIC, "krylov_batched": batch, "batch_stats": bstats}


# ----------------------------------------------------------------------------- roofline
def spmv_bytes(ndof, nnzb, bs, nrows, vbytes):
    """Algorithmic bytes of one fused BiCGSTAB SpMV launch: BSR values + block column
    indices + row pointers + x read once + y written once + the dot-product partner
    vector read once."""
    return nnzb * (bs * bs * vbytes + 4) + (nrows + 1) * 4 + 3 * ndof * vbytes


def krylov_iteration_bytes(ndof, nnzb, bs, nrows, vbytes):
    """Algorithmic bytes of one iteration of the single-launch BiCGSTAB + block Jacobi:
    two fused SpMVs (as spmv_bytes), the p update with its Jacobi apply (r, p, v read;
    p, phat written; the inverse diagonal blocks read), the s update with its Jacobi apply
    (r, v read; s, shat written; the blocks read) and the x / r update (x, phat, shat, s,
    t, rhat read; x, r written)."""
    return (2 * spmv_bytes(ndof, nnzb, bs, nrows, vbytes) + (5 + 4 + 8) * ndof * vbytes
            + 2 * nrows * bs * bs * vbytes)


def load_counters(workload):
    """ncu counters per unit of work, committed as profiles/counters_<workload>.txt: lines
    `<category> <counter> <value per unit> <unit>` (comment lines start with '#')."""
    out = {}
    path = os.path.join(ROOT, "profiles", "counters_%s.txt" % workload)
    if not os.path.exists(path):
        return out
    for line in open(path):
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        parts = line.split()
        if len(parts) >= 4:
            out.setdefault(parts[0], {})[parts[1]] = (float(parts[2]), parts[3])
    return out


def assembly_jacobian_bytes(geo, record_bytes):
    """Algorithmic bytes of one mixed-precision Jacobian pass (element kernel + covering
    gather): cell vertex and block-row indices, coordinates and state read once, the fp32
    element records written once and read once, the gather lists read once, the static
    operator read once, J (fp64) and its SELL-32 copy (fp32) written once."""
    cells, nnzb, bs, ndof = geo["cells"], geo["nnzb"], geo["bs"], geo["ndof"]
    nl = geo["nl"]
    return (cells * nl * 4 * 2 + geo["nv"] * geo["dim"] * 8 + ndof * 8 + 2 * cells * record_bytes
            + cells * nl * nl * 4 + nnzb * 8 + nnzb * bs * bs * (8 + 8 + 4))


def roofline_for(name, ms, calls, geo, peaks, counters):
    """Roofline object of one kernel category.  Residual assembly passes are bound by the FP64
    pipe (their arithmetic intensity far exceeds GB300's FP64 flop/byte balance): achieved =
    FP64 flops per launch (ncu's executed DFMA x 2 + DADD + DMUL per cell, from the committed
    counters) / average launch time, against the FP64 FMA rate measured in this run.  The
    mixed-precision Jacobian pass (fp32 element kernel + gather), the Krylov iteration and
    the SpMV are bound by HBM: achieved = algorithmic bytes per launch / average launch time,
    against the measured HBM copy bandwidth.  traffic = ncu DRAM bytes per unit x units."""
    avg_s = ms * 1e-3 / max(calls, 1)
    c = counters.get(name, {})
    dram = c.get("dram_bytes", (None, None))[0]
    if name in ("assembly_residual", "assembly_combined") or (name == "assembly_jacobian" and geo["vbytes"] == 8):
        per_cell = c.get("fp64_flops", (None, None))[0]
        flops = per_cell * geo["cells"] if per_cell is not None else None
        achieved = flops / avg_s / 1e12 if (flops and avg_s > 0) else None
        return {"kernel": name, "bound": "fp64", "achieved": achieved, "peak": peaks["fp64_tflops"],
                "unit": "TFLOP/s", "frac": achieved / peaks["fp64_tflops"] if achieved else None,
                "peak_source": "measured in this run (FMA chains, dc_selftest_fma_peaks)",
                "traffic": dram * geo["cells"] if dram is not None else None,
                "work_per_launch": flops, "avg_launch_us": avg_s * 1e6, "launches": calls,
                "per": "volume assembly pass over all cells (element kernel + gathers)"}
    if name == "assembly_jacobian":
        rec = c.get("record_bytes", (None, None))[0]
        alg = assembly_jacobian_bytes(geo, rec) if rec is not None else None
        achieved = alg / avg_s / 1e9 if (alg and avg_s > 0) else None
        return {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"] if achieved else None, "peak_source": peaks["hbm_source"],
                "traffic": dram * geo["cells"] if dram is not None else None,
                "algorithmic_bytes_per_launch": alg, "avg_launch_us": avg_s * 1e6, "launches": calls,
                "per": "fp32 element Jacobian pass + covering gather into J and its SELL-32 copy"}
    if name == "krylov_iteration":
        alg = krylov_iteration_bytes(geo["ndof"], geo["nnzb"], geo["bs"], geo["nrows"], geo["vbytes"])
        per = ("BiCGSTAB iteration inside the single-launch solve (its time includes the solve's share of "
               "the fp64 refinement residuals, which the algorithmic bytes leave out)")
    else:
        alg = spmv_bytes(geo["ndof"], geo["nnzb"], geo["bs"], geo["nrows"], geo["vbytes"])
        per = "fused SpMV launch"
    achieved = alg / avg_s / 1e9 if avg_s > 0 else 0.0
    return {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["hbm_source"],
            "traffic": dram * geo["nnzb"] if dram is not None else None,
            "algorithmic_bytes_per_launch": alg, "avg_launch_us": avg_s * 1e6, "launches": calls, "per": per}


def spmv_phase(dcgpu, ini, init, dt, precision, spmv, peaks, counters, warm_steps=1):
    """The fused SpMV kernel timed on its own on the headline operator: per-phase launches
    (linear_solver.single_launch = false), one step after a warm-up step."""
    m = dcgpu.Model(ini, {"model.time_step_operator.linear_solver.spmv": spmv,
                          "model.time_step_operator.linear_solver.single_launch": "false"})
    if precision == "mixed":
        m.set_mixed_precision(True)
    m.set_state(m.seeded_state(init), 0.0)
    d = dt
    for _ in range(warm_steps):
        d = m.step(d)["dt_next"]
    m.profile(True)
    m.step(d)
    kt = m.kernel_times()
    m.profile(False)
    mi = m.info
    fmt = m.spmv_format()
    m.close()
    geo = {"ndof": mi["n_dof"], "nnzb": mi["n_blocks"], "bs": mi["block_size"], "nrows": mi["n_block_rows"],
           "vbytes": 4 if precision == "mixed" else 8}
    ms, calls = kt["spmv"]
    r = roofline_for("spmv", ms, calls, geo, peaks, counters)
    r["spmv_layout"] = fmt["format"]
    r["tuner_us"] = {"bsr": fmt["bsr_us"], "sell": fmt["sell_us"]}
    return r


def secondary(dcgpu, kind, steps, warmup, flush):
    """Mixed and plain FP64 DOF x Newton-steps/s of another configuration (device-timed
    steps after warm-up steps, L2 flushed before each)."""
    import torch
    ini, init, dt0, _nl, desc = make_workload(kind, 0)
    out = {"config": desc, "steps": steps, "warmup": warmup}
    states = {}
    for prec in ("mixed", "fp64"):
        m = dcgpu.Model(ini)
        if prec == "mixed":
            m.set_mixed_precision(True)
        m.set_state(m.seeded_state(init), 0.0)
        d = dt0
        for _ in range(warmup):
            d = m.step(d)["dt_next"]
        tot, newton = 0.0, 0
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            inf = m.step(d)
            d = inf["dt_next"]
            tot += inf["device_ms"]
            newton += inf["newton_iterations"]
        out[prec] = {"value": m.ndof * newton / (tot * 1e-3), "ms_per_step": tot / steps, "newton_iterations": newton}
        states[prec] = (m.state(), {nm: m.species_dofs(nm) for nm in m.species})
        out["config"]["dof"] = m.ndof
        m.close()
    import numpy as np
    xm, idx = states["mixed"]
    xf, _ = states["fp64"]
    out["max_species_rel_l2_mixed_vs_fp64"] = max(
        float(np.linalg.norm(xm[i] - xf[i]) / max(np.linalg.norm(xf[i]), 1e-300)) for i in idx.values())
    out["speedup_mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def precond_comparison(dcgpu, kind, precs, steps, warmup, flush, precision="mixed"):
    """Per preconditioner on one configuration: device ms per step, Newton and Krylov
    iterations, ms per Newton iteration (per linear solve for a linear model), and the
    preconditioner's structure; steps after warm-up steps, L2 flushed before each."""
    import torch
    ini, init, dt0, _nl, desc = make_workload(kind, 0)
    out = {"config": desc, "steps": steps, "warmup": warmup, "precision": precision}
    for pc in precs:
        m = dcgpu.Model(ini, {"model.time_step_operator.linear_solver.preconditioner.type": pc})
        if precision == "mixed":
            m.set_mixed_precision(True)
        m.set_state(m.seeded_state(init), 0.0)
        d = dt0
        for _ in range(warmup):
            d = m.step(d)["dt_next"]
        s0 = m.stats()
        tot, newton = 0.0, 0
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            inf = m.step(d)
            d = inf["dt_next"]
            tot += inf["device_ms"]
            newton += inf["newton_iterations"]
        s1 = m.stats()
        lin = s1["linear_iterations"] - s0["linear_iterations"]
        solves = max(newton, 1)
        out[pc] = {"ms_per_step": tot / steps, "newton_iterations": newton, "krylov_iterations": lin,
                   "krylov_iterations_per_solve": lin / solves, "ms_per_newton_iteration": tot / solves,
                   "preconditioner": m.precond_info()}
        m.close()
    return out


def main():
    args = parse()
    rank, world = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import numpy as np
    import torch
    import __graft_entry__ as g
    g.build()
    import dcgpu

    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")

    ini, init, dt0, nl, desc = make_workload(args.workload, args.n)
    single = "true" if args.single_launch == "on" else "false"
    ov = {"model.time_step_operator.linear_solver.spmv": args.spmv,
          "model.time_step_operator.linear_solver.preconditioner.type": args.precond,
          "model.time_step_operator.linear_solver.single_launch": single}
    if args.inner_reduction is not None:
        ov["model.time_step_operator.linear_solver.inner_reduction"] = repr(args.inner_reduction)
    for kv in args.override:
        k, v = kv.split("=", 1)
        ov[k.strip()] = v.strip()

    # measured peaks: FP64 / FP32 FMA rates of this GPU now, HBM copy bandwidth from the
    # pool's measurement file
    fp64_tf, fp32_tf = dcgpu.fma_peaks()
    peaks = {"fp64_tflops": fp64_tf, "fp32_tflops": fp32_tf}
    try:
        peaks["hbm_gbs"] = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        peaks["hbm_source"] = "measured (MEASURED_PEAKS.json)"
    except Exception:
        peaks["hbm_gbs"] = 6800.0
        peaks["hbm_source"] = "fallback"
    counters = load_counters(args.workload)

    model = dcgpu.Model(ini, ov)
    if args.precision == "mixed":
        model.set_mixed_precision(True)
    x0 = model.seeded_state(init)
    ndof = model.ndof
    desc["dof"] = ndof
    model.set_state(x0, 0.0)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    dt = dt0
    for _ in range(args.warmup):
        dt = model.step(dt)["dt_next"]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()

    def timed_steps(m, d):
        """K steps, L2 flushed before each, device time of each step from its CUDA events."""
        ms, nit, lit = [], 0, 0
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            inf = m.step(d)
            d = inf["dt_next"]
            ms.append(inf["device_ms"])
            nit += inf["newton_iterations"]
            lit += inf["linear_iterations"]
        torch.cuda.synchronize()
        return sum(ms), nit, lit, d

    clocks = ClockSampler()
    clocks.start()
    launches0 = dcgpu.launch_count()
    total_ms, newton, linear, dt = timed_steps(model, dt)
    launches = dcgpu.launch_count() - launches0
    clk = clocks.stop()
    if args.minimal:
        total_ms = max_over_ranks(total_ms, dist)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": world * ndof * newton / (total_ms * 1e-3), "unit": METRIC,
                              "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                              "ms_per_step": total_ms / args.steps, "config": workload_desc(args.workload, args.n),
                              "run": {"minimal": True, "newton_iterations": newton, "krylov_iterations": linear,
                                      "volume_kernels": model.jit_status()}}), flush=True)
        model.close()
        return

    # the plain FP64 path on the same workload and steps, for the metric's comparison, and
    # the mixed path's deviation from it (per-species relative L2 after W + K steps)
    plain = None
    if args.precision == "mixed" and not args.no_plain_fp64:
        xm = model.state()
        ref = dcgpu.Model(ini, {"model.time_step_operator.linear_solver.preconditioner.type": args.precond,
                                "model.time_step_operator.linear_solver.single_launch": single})
        ref.set_state(x0, 0.0)
        d = dt0
        for _ in range(args.warmup):
            d = ref.step(d)["dt_next"]
        p_ms, p_newton, p_linear, d = timed_steps(ref, d)
        xf = ref.state()
        errs = []
        for name in ref.species:
            idx = ref.species_dofs(name)
            nb = float(np.linalg.norm(xf[idx]))
            errs.append(float(np.linalg.norm(xm[idx] - xf[idx])) / (nb if nb > 0 else 1.0))
        plain = {"value": world * ndof * p_newton / (p_ms * 1e-3), "unit": METRIC,
                 "ms_per_step": p_ms / args.steps, "newton_iterations": p_newton, "krylov_iterations": p_linear,
                 "max_species_rel_l2_mixed_vs_fp64": max(errs)}
        ref.close()

    # per-category kernel times from a second pass of the same number of steps with
    # events around each kernel group (kept out of the timed pass above)
    model.profile(True)
    prof_dt = dt
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        prof_dt = model.step(prof_dt)["dt_next"]
    torch.cuda.synchronize()
    kt = model.kernel_times()
    model.profile(False)
    total_ms = max_over_ranks(total_ms, dist)
    value = world * ndof * newton / (total_ms * 1e-3)

    # end to end through the C ABI with host buffers (upload, step, download), the state
    # living in pinned host memory
    xs = torch.empty(ndof, dtype=torch.float64, pin_memory=True).numpy()
    model.state(out=xs)
    e2e_t = 0.0
    e2e_newton = 0
    nrep = max(2, min(args.steps, 5))
    for _ in range(nrep):
        # the same L2 flush as between the device-timed steps, outside the timed region
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        model.set_state(xs, model.time())
        info = model.step(dt)
        model.state(out=xs)
        e2e_t += time.perf_counter() - t0
        e2e_newton += info["newton_iterations"]
        dt = info["dt_next"]
    e2e = {"value": world * ndof * e2e_newton / e2e_t, "unit": METRIC,
           "h2d_bytes_per_step": ndof * 8, "d2h_bytes_per_step": ndof * 8}

    # roofline of every kernel category; the headline object is the category with the
    # largest device time
    info_m = model.info
    geo = {"ndof": ndof, "nnzb": info_m["n_blocks"], "bs": info_m["block_size"], "nrows": info_m["n_block_rows"],
           "cells": info_m["n_elements"], "vbytes": 4 if args.precision == "mixed" else 8, "nl": nl,
           "nv": info_m["n_vertices"], "dim": info_m["dim"]}
    cats = {k: v for k, v in kt.items() if v[1] and k != "assembly"}
    by_cat = {k: roofline_for(k, v[0], v[1], geo, peaks, counters) for k, v in cats.items()}
    dom = max(cats, key=lambda k: cats[k][0]) if cats else "krylov_iteration"
    roof = dict(by_cat.get(dom, {}))
    roof["category_ms"] = {k: v[0] for k, v in kt.items()}
    roof["category_launches"] = {k: v[1] for k, v in kt.items()}
    roof["by_category"] = by_cat
    if not args.no_spmv_phase:
        roof["spmv_fused_kernel"] = spmv_phase(dcgpu, ini, init, dt0, args.precision, args.spmv, peaks, counters)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(args.workload, args.n, args.cpu_iterations, args.cpu_precond,
                               args.cpu_1core_iterations)
        except Exception as e:
            cpu = {"unavailable": str(e)}
    sec = None
    if not args.no_secondary and args.workload == "cross_diffusion_3d":
        sec = {"gray_scott_512": secondary(dcgpu, "gray_scott", 10, 3, flush),
               "two_compartment_1024": secondary(dcgpu, "two_compartment", 3, 2, flush)}
    pcmp = None
    if not args.no_precond_comparison and args.workload == "cross_diffusion_3d":
        pcmp = {"heat_128": precond_comparison(dcgpu, "heat", ["Jacobi", "AMG", "SSOR", "auto"], 5, 2, flush,
                                               "fp64"),
                "two_compartment_1024": precond_comparison(dcgpu, "two_compartment",
                                                           ["Jacobi", "AMG", "SSOR", "ILU", "auto"], 2, 1, flush)}
    serving = None
    if args.serve_requests > 0:
        # the same seeded stream each time: batched mixed (the served path), batched FP64,
        # the unbatched server (every simulation replays its own Krylov graphs on its own
        # stream) in mixed precision, and FP64 one simulation at a time
        mix = SERVE_SPEC if args.serve_spec else None
        ratio = lambda a, b: a["value"] / b["value"] if b["value"] > 0 else None  # noqa: E731
        batched = run_serving(dcgpu, args.serve_requests, 50.0, args.serve_active, "mixed", mix=mix, batch=True)
        batched64 = run_serving(dcgpu, args.serve_requests, 50.0, args.serve_active, "fp64", mix=mix, batch=True)
        unbatched = run_serving(dcgpu, args.serve_requests, 50.0, args.serve_active, "mixed", mix=mix)
        serving = {"spec": bool(args.serve_spec), "served_batched_mixed": batched, "batched_fp64": batched64,
                   "unbatched_mixed": unbatched,
                   # the precision's effect at the same batching, and the batching's at the same
                   # precision
                   "speedup_mixed_vs_fp64_batched": ratio(batched, batched64),
                   "speedup_batched_vs_unbatched_mixed": ratio(batched, unbatched)}
        if not args.serve_spec:
            alone = run_serving(dcgpu, args.serve_requests, 50.0, 1, "fp64")
            serving["plain_fp64_one_at_a_time"] = alone
            serving["speedup"] = ratio(batched, alone)
            # where batching pays: sixteen simulations whose solves coincide (unbatched first,
            # so neither leg pays a one-off set-up cost the other skips)
            b_un = run_burst(dcgpu, 16, 24, 10, False)
            b_ba = run_burst(dcgpu, 16, 24, 10, True)
            serving["coinciding_burst"] = {"batched": b_ba, "unbatched": b_un,
                                           "speedup_batched_vs_unbatched": ratio(b_ba, b_un)}
    # `config` names the workload only (the reference arm prints the same dict); how this
    # arm ran it is under "run"
    config = workload_desc(args.workload, args.n)
    config["dof"] = ndof
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+f32",
            "data": "synthetic (seeded initial state, no dataset)",
            "config": config,
            "run": {"precision": args.precision,
                    "linear_solver": "BiCGSTAB to 1e-10 (direct-solve semantics)",
                    "preconditioner": model.precond_info(),
                    "l2_flush": "inputs larger than L2, and a 256 MiB write between timed steps",
                    "newton_iterations": newton, "krylov_iterations": linear,
                    "spmv_layout": model.spmv_format()["format"],
                    "volume_kernels": model.jit_status(),
                    "krylov_launch": "single cooperative launch per solve" if single == "true"
                                     else "one launch per phase, CUDA graph of 8 iterations"},
            "plain_fp64": plain,
            "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
            "e2e": e2e, "roofline": roof, "peaks": peaks, "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": launches, "secondary": sec, "preconditioners": pcmp, "serving": serving}
    if rank == 0:
        print(json.dumps(line), flush=True)
    model.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
