"""Benchmark: DOF x Newton-steps per second of the implicit time step on one GB300.

Workload (the configuration the headline metric is quoted on): seeded Gray-Scott,
2 species, unit square 512 x 512 P1 triangles (526,338 DOF), Alexander2 DIRK dt = 1,
Newton relative tolerance 1e-10 (squared l2, as the reference), direct-solve semantics
(the reference's default UMFPack is replaced by BiCGSTAB converged to a relative
residual of 1e-10).

A "step" is one Alexander2 time step (2 stages x Newton iterations).  Timed per step with
CUDA events on the engine's stream (dc_step_info.device_ms); the L2 cache is flushed
between timed steps (a 256 MiB write).  value = DOF x Newton iterations of all timed
steps / sum of device step times, for the mixed-precision path (fp32 Krylov in fp64
refinement) by default; "plain_fp64" is the plain FP64 path on the same workload and steps,
with the per-species relative L2 deviation of the mixed state from it.  e2e = the same
through the public C ABI with host buffers: state upload (pinned->device), step, state
download, host-timed.  "serving" runs a Poisson stream of random requests through the
request server: served concurrently with mixed precision, and one at a time in plain FP64.

--impl reference times the CPU restatement of the reference algorithm (numpy assembly +
SuperLU direct solve, the oracle) on the host cores, one Newton iteration of the full
workload per step.

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
WORKLOAD = "gray_scott_512x512_p1_alexander2_dt1"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    # "--grid" is the spelling to use after a torchrun launcher, whose own parser reads
    # "--n" as an ambiguous abbreviation of its options
    ap.add_argument("--n", "--grid", dest="n", type=int, default=512)
    ap.add_argument("--workload", default="gray_scott", choices=["gray_scott", "cross_diffusion_3d"],
                    help="gray_scott (headline, n = grid edge) or cross_diffusion_3d (n = cube edge)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="mixed (default): fp32 Krylov in fp64 refinement, measured against the plain "
                         "FP64 path on the same workload; fp64: the plain path alone")
    ap.add_argument("--no-plain-fp64", action="store_true",
                    help="skip the plain FP64 comparison run of the mixed path")
    ap.add_argument("--spmv", default="auto", choices=["auto", "bsr", "sell"],
                    help="layout of the fp32 Krylov operator (linear_solver.spmv)")
    ap.add_argument("--precond", default="Jacobi", choices=["Jacobi", "AMG"],
                    help="BiCGSTAB preconditioner (linear_solver.preconditioner.type)")
    ap.add_argument("--single-launch", default="on", choices=["on", "off"],
                    help="BiCGSTAB as one cooperative launch per solve (on) or one launch per "
                         "phase from a CUDA graph (off) (linear_solver.single_launch)")
    ap.add_argument("--inner-reduction", type=float, default=None,
                    help="mixed precision: residual reduction of each fp32 correction solve "
                         "(linear_solver.inner_reduction; engine default 1e-4)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--large-n", type=int, default=128,
                    help="cube edge of the HBM-resident SpMV measurement (0 disables it)")
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


def make_workload(n, kind="gray_scott"):
    """(ini, init, dt, description) of the bench workload; gray_scott is the headline one."""
    import workloads as W
    if kind == "cross_diffusion_3d":
        ini, init = W.cross_diffusion_3d(n=n, steps=100000, dt=0.01)
        return ini, init, 0.01, {"workload": "cross_diffusion_3d_%d^3x6_p1_tets_alexander2_dt0.01" % n,
                                 "mesh": "%d^3 cubes x 6 P1 tetrahedra" % n, "species": 3, "nl": 4}
    ini, init = W.gray_scott(n=n, steps=100000, dt=1.0)
    name = WORKLOAD if n == 512 else "gray_scott_%dx%d_p1_alexander2_dt1" % (n, n)
    return ini, init, 1.0, {"workload": name, "mesh": "%dx%d P1 triangles" % (n, n), "species": 2, "nl": 3}


def initial_vector(om, init):
    """Seeded initial state in the reference DOF order for the CPU legs, from the oracle
    model `om` (the GPU arm builds the same vector from its own model, Model.seeded_state)."""
    x = om.initial_state()
    for sp in (om.species if init is not None else []):
        verts = om.comp_vertices[sp.comp]
        x[om.dof(sp, verts)] = init(sp.name, om.mesh.coords[verts])
    return x


def oracle_newton_iteration(om, x, dt):
    """The work of one Newton iteration of an Alexander2 stage on the CPU oracle:
    residual and Jacobian of M + gamma dt A at x, direct (SuperLU) solve, update."""
    a = (1.0 - 0.5 * 2 ** 0.5) * dt
    r = om.residual(x, 0.0, "mass") + a * om.residual(x, 0.0, "stiffness")
    J = om.jacobian(x, 0.0, "mass") + a * om.jacobian(x, 0.0, "stiffness")
    return x - om._solve(J, r)


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


def cpu_baseline(ini, init, dt, wdesc, newton_steps=1):
    """Oracle (numpy assembly + SuperLU) on the host: one Newton iteration of the full workload."""
    from oracle.model import OracleModel
    om = OracleModel(ini)
    x0 = initial_vector(om, init)
    t0 = time.perf_counter()
    for _ in range(newton_steps):
        x0 = oracle_newton_iteration(om, x0, dt)
    dt = time.perf_counter() - t0
    return {"value": om.ndof * newton_steps / dt, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": "%d Newton iteration(s) (residual + Jacobian assembly + SuperLU solve) of the "
                      "%d-DOF %s stage system, first Alexander2 stage"
                      % (newton_steps, om.ndof, wdesc["workload"]),
            "seconds": dt}


def run_reference(args, rank, world):
    if rank != 0:
        return
    ini, init, dt0, wdesc = make_workload(args.n, args.workload)
    from oracle.model import OracleModel
    om = OracleModel(ini)
    x = initial_vector(om, init)
    times = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        x = oracle_newton_iteration(om, x, dt0)
        t1 = time.perf_counter()
        if k >= args.warmup:
            times.append(t1 - t0)
    total = sum(times)
    value = om.ndof * len(times) / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded initial state)",
            "config": {"workload": wdesc["workload"], "dof": om.ndof,
                       "step": "one Newton iteration (assembly + SuperLU)"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": 1, "kind": "port",
                             "sample": "one Newton iteration of the full workload per step"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_serving(dcgpu, n_requests, lam, max_active, precision, seed=20261203, budget=64 << 30):
    """Poisson stream of random requests through the request server; returns latency
    percentiles and the aggregate DOF x Newton-step throughput."""
    import workloads as W
    stream = W.serving_stream(n_requests, lam, seed, n2d=(32, 160), n3d=(12, 32), steps=(10, 40))
    ov = {"model.time_step_operator.linear_solver.precision": "mixed"} if precision == "mixed" else None
    srv = dcgpu.Server(budget, max_active)
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
    srv.close()
    lat = sorted(r["latency_s"] for r in done.values())
    ok = sum(1 for r in done.values() if r["status"] == 0)
    work = sum(r["n_dof"] * r["newton_iterations"] for r in done.values())
    import numpy as np
    return {"requests": len(stream), "ok": ok, "lambda_per_s": lam, "max_active": max_active,
            "precision": precision, "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "wall_s": wall,
            "value": work / wall, "unit": METRIC,
            "mix": "2D N log-U[32,160] / 3D N log-U[12,32], 1-2 compartments, 1-8 species, 10-40 IE steps"}


def large_spmv(dcgpu, precision, peak_gbs, n=128, spmv="auto"):
    """SpMV roofline on an operator far larger than L2: the 3D cross-diffusion workload
    (n^3 cubes x 6 tetrahedra, 3 species, ~6.4 M DOF at n = 128), one Alexander2 step with
    per-kernel events; returns the fused-SpMV achieved bandwidth against the HBM peak."""
    import workloads as W
    ini, init = W.cross_diffusion_3d(n=n, steps=1, dt=0.01)
    vb = 4 if precision == "mixed" else 8

    def one(single):
        m = dcgpu.Model(ini, {"model.time_step_operator.linear_solver.spmv": spmv,
                              "model.time_step_operator.linear_solver.single_launch": single})
        if precision == "mixed":
            m.set_mixed_precision(True)
        m.set_state(m.seeded_state(init), 0.0)
        m.step(0.01)  # first step: tuner, graphs
        m.profile(True)
        info = m.step(0.01)
        kt = m.kernel_times()
        m.profile(False)
        fmt = m.spmv_format()
        mi = m.info
        m.close()
        return info, kt, fmt, mi

    # per-phase launches: the fused SpMV kernel timed on its own
    info, kt, fmt, mi = one("false")
    ms, calls = kt["spmv"]
    alg = spmv_bytes(mi["n_dof"], mi["n_blocks"], mi["block_size"], mi["n_block_rows"], vb)
    avg = ms * 1e-3 / max(calls, 1)
    ach = alg / avg / 1e9 if avg > 0 else 0.0
    out = {"workload": "cross_diffusion_3d_%d^3x6_tets_3_species" % n, "dof": mi["n_dof"],
           "blocks": mi["n_blocks"], "block_size": mi["block_size"], "precision": precision,
           "spmv_layout": fmt["format"], "tuner_us": {"bsr": fmt["bsr_us"], "sell": fmt["sell_us"]},
           "algorithmic_bytes_per_launch": alg, "avg_launch_us": avg * 1e6, "launches": calls,
           "achieved": ach, "peak": peak_gbs, "unit": "GB/s", "frac": ach / peak_gbs,
           "newton_iterations": info["newton_iterations"], "krylov_iterations": info["linear_iterations"]}
    # single-launch solve: whole BiCGSTAB iterations on the same operator
    info, kt, fmt, mi = one("true")
    ms, iters = kt["krylov_iteration"]
    if iters:
        alg = krylov_iteration_bytes(mi["n_dof"], mi["n_blocks"], mi["block_size"], mi["n_block_rows"], vb)
        avg = ms * 1e-3 / iters
        ach = alg / avg / 1e9 if avg > 0 else 0.0
        out["single_launch_iteration"] = {
            "algorithmic_bytes_per_iteration": alg, "avg_iteration_us": avg * 1e6, "iterations": iters,
            "achieved": ach, "peak": peak_gbs, "unit": "GB/s", "frac": ach / peak_gbs,
            "spmv_layout": fmt["format"]}
    return out


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


def assembly_bytes(ne, nl, ns, ndof, nnz, jac):
    """Algorithmic bytes of one residual (+ Jacobian) assembly pass: cell vertex and node
    indices, vertex coordinates and coefficients gathered once per cell, residual written
    once, Jacobian values written once (colour-ordered, no read-back)."""
    b = ne * (nl * 4 * 2 + nl * ns * 8) + ndof * 8
    if jac:
        b += nnz * 8 + ne * nl * nl * 4
    return b


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

    ini, init, dt0, wdesc = make_workload(args.n, args.workload)
    single = "true" if args.single_launch == "on" else "false"
    ov = {"model.time_step_operator.linear_solver.spmv": args.spmv,
          "model.time_step_operator.linear_solver.preconditioner.type": args.precond,
          "model.time_step_operator.linear_solver.single_launch": single}
    if args.inner_reduction is not None:
        ov["model.time_step_operator.linear_solver.inner_reduction"] = repr(args.inner_reduction)
    model = dcgpu.Model(ini, ov)
    if args.precision == "mixed":
        model.set_mixed_precision(True)
    x0 = model.seeded_state(init)
    ndof = model.ndof
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

    # roofline of the dominant kernel category
    import json as _j
    peaks = {}
    try:
        peaks = _j.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak_gbs = float(peaks["hbm_gbs"])
        peak_src = "measured"
    except Exception:
        peak_gbs = 6800.0
        peak_src = "fallback"
    info_m = model.info
    bs = info_m["block_size"]
    nrows = info_m["n_block_rows"]
    nnzb = info_m["n_blocks"]
    ne = info_m["n_elements"]
    vbytes = 4 if args.precision == "mixed" else 8
    cats = {}
    for name, (ms, calls) in kt.items():
        if calls:
            cats[name] = (ms, calls)
    def cat_roof(name):
        ms, calls = cats.get(name, (0.0, 1))
        avg_s = ms * 1e-3 / max(calls, 1)
        if name == "spmv":
            alg = spmv_bytes(ndof, nnzb, bs, nrows, vbytes)
        elif name == "krylov_iteration":
            alg = krylov_iteration_bytes(ndof, nnzb, bs, nrows, vbytes)
        elif name == "assembly":
            alg = assembly_bytes(ne, wdesc["nl"], wdesc["species"], ndof, nnzb * bs * bs, jac=True)
        else:
            alg = nrows * bs * bs * vbytes + 2 * ndof * vbytes
        achieved = alg / avg_s / 1e9 if avg_s > 0 else 0.0
        r = {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
             "frac": achieved / peak_gbs, "peak_source": peak_src, "traffic": None,
             "algorithmic_bytes_per_launch": alg, "avg_launch_us": avg_s * 1e6, "launches": calls}
        if name == "krylov_iteration":
            # one cooperative launch runs a whole solve: bytes and time are per iteration
            r["per"] = "BiCGSTAB iteration inside k_bicgstab_fused"
        return r

    dom = max(cats, key=lambda k: cats[k][0]) if cats else "spmv"
    roof = cat_roof(dom)
    roof["category_ms"] = {k: v[0] for k, v in cats.items()}
    roof["category_launches"] = {k: v[1] for k, v in cats.items()}
    roof["by_category"] = {k: cat_roof(k) for k in cats}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(ini, init, dt0, wdesc)
    roof["spmv_layout"] = model.spmv_format()
    if args.large_n > 0:
        roof["spmv_hbm_resident"] = large_spmv(dcgpu, args.precision, peak_gbs, args.large_n, args.spmv)
    serving = None
    if args.serve_requests > 0:
        served = run_serving(dcgpu, args.serve_requests, 50.0, args.serve_active, args.precision)
        alone = run_serving(dcgpu, args.serve_requests, 50.0, 1, "fp64")
        serving = {"served_concurrent": served, "plain_fp64_one_at_a_time": alone,
                   "speedup": served["value"] / alone["value"] if alone["value"] > 0 else None}
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+f32",
            "data": "synthetic (seeded initial state, no dataset)",
            "config": {"workload": wdesc["workload"], "mesh": wdesc["mesh"], "dof": ndof,
                       "species": wdesc["species"], "scheme": "Alexander2", "dt": dt0, "precision": args.precision,
                       "linear_solver": "BiCGSTAB+%s to 1e-10 (direct-solve semantics)"
                                        % ("block-Jacobi" if args.precond == "Jacobi" else "aggregation-AMG"),
                       "spmv_layout": model.spmv_format()["format"],
                       "krylov_launch": "single cooperative launch per solve" if single == "true"
                                        else "one launch per phase, CUDA graph of 8 iterations",
                       "newton_rel_tol_sq": 1e-10, "l2_flush": "256 MiB write between timed steps",
                       "newton_iterations": newton, "krylov_iterations": linear},
            "plain_fp64": plain,
            "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
            "serving": serving}
    if rank == 0:
        print(json.dumps(line), flush=True)
    model.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
