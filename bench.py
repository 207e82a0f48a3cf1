"""Benchmark of the GB300 PetRBF solve path.

Workload: the 2D Lamb-Oseen interpolation at scale -- N = 4x10^6 points on a 2000 x 2000
lattice over [-1,1]^2 with seeded +/-0.25h jitter, sigma = h/0.8, cell edge 8 sigma,
cutoff 8 sigma past the cell edge (sigma_trunc 24), one-cell overlap buffer (24).

A step is one truncated Gaussian matvec (the operator GMRES applies every iteration,
mymatmult of 2d/matmult.cxx:6-51) over all 4x10^6 points in FP64; ``value`` is
Gpairs/s with the points resident in HBM and L2 flushed between steps; ``e2e`` is the
same metric through the C ABI (prbf_matvec) with pinned host vectors copied in and out
every step. The full solve to 1e-13 (plain FP64 and mixed precision) is timed once
after the steps and reported under ``solve``.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--skip-solve]
    python bench.py --workload vortex3d     # 3D mixed form, 128^3, three right-hand sides
    python bench.py --workload batch2d      # 256 problems of uneven N in one batch
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOPS_PER_PAIR = 15  # the reference's count per pair, exp counted as 1 (2d/matmult.cxx:44-45)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-solve", action="store_true")
    ap.add_argument("--m", type=int, default=2000, help="lattice edge (N = m^2)")
    ap.add_argument("--workload", default="matvec2d", choices=["matvec2d", "vortex3d", "batch2d"],
                    help="matvec2d: the headline line; vortex3d / batch2d: the 3D mixed and batched forms")
    ap.add_argument("--m3", type=int, default=128, help="3D lattice edge (vortex3d)")
    ap.add_argument("--nprob", type=int, default=256, help="problems (batch2d)")
    ap.add_argument("--batch-max-it", type=int, default=1000)
    ap.add_argument("--case", default=None, help="run one small kernel case (ncu captures) and exit")
    ap.add_argument("--sections", default="solve,cpu_solve,cpu_solve_4e6,vortex3d,batch2d,learned",
                    help="extra sections of the default line after the timed steps (comma list)")
    ap.add_argument("--cpu-solve-child", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--seed", type=int, default=12345, help=argparse.SUPPRESS)
    return ap.parse_args()


def dist_init(n):
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as td
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        td.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as td
        td.barrier()


def allmax(v, world):
    if world <= 1:
        return v
    import torch
    import torch.distributed as td
    t = torch.tensor([float(v)], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_step, steps, ms_local, world):
    """Whole-job throughput of N independent replicas: every rank processed the same units
    per step; the job's time is the slowest rank's (max over ranks). Returns (Gunits/s,
    max ms)."""
    ms = allmax(ms_local, world)
    return units_per_step * steps * world / (ms * 1e-3) / 1e9, ms


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev, self.rows, self.stop = dev, [], False
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        while not self.stop:
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([c.strip() for c in out.split(",")])
            except Exception:
                pass
            time.sleep(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop = True
        self.t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if len(r) > 2 + k and r[2 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.rows)}


def fp64_peak_tflops(torch):
    """FP64 peak measured in-run: cuBLAS DGEMM 8192^3 (2 N^3 flops), best of 5."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


def hbm_view(bytes_per_launch, ms_per_launch):
    """The matvec against the HBM roof: algorithmic bytes per launch (2D: x, y, g read and w
    written, 32 B per point) over the launch time, against the measured copy bandwidth of
    MEASURED_PEAKS.json (else the 6800 GB/s fallback). The sum is FP64-pipe bound; this
    shows how far from memory-bound it is."""
    peak, src = 6800.0, "fallback 6800 GB/s (no MEASURED_PEAKS.json)"
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peak, src = float(json.load(fh)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, TypeError, ValueError):
        pass
    gbs = bytes_per_launch / (ms_per_launch * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "peak_source": src, "bytes_per_launch": bytes_per_launch}


def profile_traffic(name):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def workload_name(m):
    return "2d_lamb_oseen_N4e6_jitter" if m == 2000 else "2d_lamb_oseen_m%d" % m


def _cpu_matvec_setup(p):
    """Cell list of the workload on the host (the oracle's cell sort) and its pair count."""
    import oracle as O
    g = O.grid_for(p.x, p.y, None, *p.params())
    perm, cs = O.cell_sort(g, p.x, p.y)
    xs, ys = p.x[perm], p.y[perm]
    pairs = int((np.diff(cs) * O.trunc_counts(g, xs, ys, None, cs)).sum())
    return g, xs, ys, cs, pairs


def cpu_baseline(p, seconds_target=10.0):
    """The oracle (C++ restatement of mymatmult, OpenMP over cells) on the workload itself,
    every point; the sample is the number of matvecs, bounded by seconds_target."""
    import oracle as O
    g, xs, ys, cs, pairs = _cpu_matvec_setup(p)
    v = np.random.default_rng(1).standard_normal(p.n)
    O.matvec(g, xs, ys, None, cs, v)  # warm
    t0 = time.perf_counter()
    reps = 0
    while True:
        O.matvec(g, xs, ys, None, cs, v)
        reps += 1
        if time.perf_counter() - t0 >= seconds_target or reps >= 50:
            break
    dt = time.perf_counter() - t0
    return {"value": pairs * reps / dt / 1e9, "unit": "Gpairs/s", "cores": O.num_threads(),
            "kind": "port",
            "sample": "%d FP64 matvecs of the full %d-point workload (%.3g pairs each), %.1f s" % (
                reps, p.n, pairs, dt)}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU matvec (the oracle port: the reference's compiled
    sources do not travel to an Arm host) on all host cores, over the same workload as the
    GPU arm -- every point, every step."""
    if rank != 0:
        return
    import oracle as O
    from petrbf_gb300 import workloads as W
    p = W.lamb_oseen_2d(args.m, jitter=0.25, seed=12345)
    g, xs, ys, cs, pairs = _cpu_matvec_setup(p)
    v = np.random.default_rng(1).standard_normal(p.n)
    for _ in range(args.warmup):
        O.matvec(g, xs, ys, None, cs, v)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.matvec(g, xs, ys, None, cs, v)
    dt = time.perf_counter() - t0
    val = pairs * args.steps / dt / 1e9
    sample = "%d FP64 matvecs of the full %d-point workload (%.3g pairs each)" % (args.steps, p.n, pairs)
    print(json.dumps({
        "impl": "reference", "metric": "Gaussian matvec Gpairs/s", "value": val, "unit": "Gpairs/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.m), "n_points": p.n, "sigma_over_h": 1.25,
                   "nsigma_box": 8, "sigma_buffer": 24, "sigma_trunc": 24, "pairs_per_matvec": pairs},
        "cpu_baseline": {"value": val, "unit": "Gpairs/s", "cores": O.num_threads(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": val, "unit": "Gpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def offgrid_error(ctx, p, g, torch_rng_seed=7, nt=1_000_000):
    """log10 relative error of the interpolant against the analytic field at nt random
    targets inside the lattice (off the collocation points), 2d/main.cxx:130-133."""
    from petrbf_gb300 import workloads as W
    rng = np.random.default_rng(torch_rng_seed)
    lo, hi = float(p.x.min()), float(p.x.max())
    xt, yt = rng.uniform(lo, hi, nt), rng.uniform(lo, hi, nt)
    w = ctx.evaluate(xt, yt, None, p.x, p.y, None, g)
    return W.log10_rel_error(w, W.lamb_oseen(xt, yt))


def run_ours(args, rank, world):
    import torch
    from petrbf_gb300 import workloads as W
    from petrbf_gb300.api import Context

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    p = W.lamb_oseen_2d(args.m, jitter=0.25, seed=12345 + rank)
    ctx = Context(dim=2, sigma=p.sigma, nsigma_box=8, sigma_buffer=24, sigma_trunc=24, device=dev)
    ctx.matvec_setup(p.x, p.y)
    info = ctx.matvec_info()
    pairs = info["pairs"]
    kernels_per_step, symmetric = ctx.matvec_kernels()
    n = p.n
    stream = torch.cuda.ExternalStream(ctx.stream)
    vin = torch.randn(n, dtype=torch.float64, device="cuda")
    vout = torch.empty_like(vin)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        ctx.matvec_dev(vin.data_ptr(), vout.data_ptr(), cell_order=True)
    ctx.synchronize()
    # ---- device-resident steps ------------------------------------------------------------
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    with Clocks(dev) as clk:
        barrier(world)
        torch.cuda.synchronize()
        t_wall0 = time.perf_counter()
        for e0, e1 in evs:
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            e0.record(stream)
            ctx.matvec_dev(vin.data_ptr(), vout.data_ptr(), cell_order=True)
            e1.record(stream)
        ctx.synchronize()
        torch.cuda.synchronize()
        barrier(world)
        t_wall = time.perf_counter() - t_wall0
    ms = sum(e0.elapsed_time(e1) for e0, e1 in evs)
    value, ms = replica_value(pairs, args.steps, ms, world)
    # ---- end to end through the C ABI with pinned host vectors ----------------------------------
    hin = torch.randn(n, dtype=torch.float64).pin_memory()
    hout = torch.empty(n, dtype=torch.float64).pin_memory()
    import ctypes
    from petrbf_gb300 import _native as N
    L = N.lib()
    pin = ctypes.cast(hin.data_ptr(), ctypes.POINTER(ctypes.c_double))
    pout = ctypes.cast(hout.data_ptr(), ctypes.POINTER(ctypes.c_double))
    for _ in range(max(1, args.warmup)):
        assert L.prbf_matvec(ctx.h, pin, pout) == 0
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        assert L.prbf_matvec(ctx.h, pin, pout) == 0
    e2e_s = allmax(time.perf_counter() - t0, world)
    e2e = pairs * args.steps * world / e2e_s / 1e9
    # FP32 pair arithmetic of the same operator (the mixed form's inner matvec)
    for _ in range(3):
        ctx.matvec_dev(vin.data_ptr(), vout.data_ptr(), cell_order=True, fp32=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(20):
        ctx.matvec_dev(vin.data_ptr(), vout.data_ptr(), cell_order=True, fp32=True)
    e1.record(stream)
    e1.synchronize()
    fp32_gpairs = pairs * 20 / (e0.elapsed_time(e1) * 1e-3) / 1e9
    ctx.close()
    del flush, vin, vout
    torch.cuda.empty_cache()

    peak = fp64_peak_tflops(torch) if rank == 0 else None
    achieved = FLOPS_PER_PAIR * pairs / (ms / args.steps * 1e-3) / 1e12
    result = {
        "metric": "Gaussian matvec Gpairs/s", "value": value, "unit": "Gpairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload_name(args.m),
                   "n_points": n, "sigma_over_h": 1.25, "nsigma_box": 8, "sigma_buffer": 24,
                   "sigma_trunc": 24, "pairs_per_matvec": pairs, "ncell": info["ncell"],
                   "l2": "flushed between steps (256 MiB write, outside the timed events)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": e2e, "unit": "Gpairs/s", "h2d_bytes_per_step": 8 * n,
                "d2h_bytes_per_step": 8 * n},
        "gpu_launches": args.steps * kernels_per_step,
        "clocks": clk.summary(),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None,
                     "peak_source": "in-run cuBLAS DGEMM 8192^3 (no FP64 figure in MEASURED_PEAKS)",
                     "flops_per_pair": FLOPS_PER_PAIR,
                     "symmetric": symmetric,
                     "note": ("achieved counts the reference's 15 flops per ordered pair; the symmetric sum "
                              "evaluates one exponential for both ordered pairs of a point pair") if symmetric else None,
                     "traffic": profile_traffic("gauss_fp64_2d_N4e6.txt"),
                     "hbm_view": hbm_view(32 * n, ms / args.steps)},
        "fp32_matvec_gpairs": fp32_gpairs,
        "wall_s_timed_region": t_wall,
    }
    if rank == 0 and world == 1:
        result["cpu_baseline"] = cpu_baseline(p)
    sections = set() if args.skip_solve else set(args.sections.split(","))
    if "solve" in sections:
        result["solve"], g64 = solve_section(p, dev, rank)
        if rank == 0 and world == 1 and "cpu_solve" in sections:
            result["cpu_solve"] = cpu_solve_section(dev)
            if "cpu_solve_4e6" in sections:
                result["cpu_solve"]["lamb_oseen_jitter_4e6"] = cpu_solve_full(p, args, g64, result["solve"]["fp64"])
    if rank == 0 and world == 1:
        if "vortex3d" in sections:
            result["vortex3d"] = vortex3d_section(args.m3)
        if "batch2d" in sections:
            result["batch2d"] = batch2d_section(args.nprob, args.batch_max_it)
        if "learned" in sections:
            result["learned_heldout"] = learned_heldout_section(dev)
    if rank == 0:
        print(json.dumps(result), flush=True)


def cpu_solve_section(dev):
    """The 10^4-point 100 x 100 lattice (config 1) solved to 1e-13 on the host cores by the
    oracle -- the C++ restatement of the reference's solve (cell list, dense Schwarz blocks
    with PETSc's LU, GMRES(30); OpenMP over cells), and the same with the GPU library's
    block arithmetic restated (Cholesky) -- and by the plain FP64 GPU form: times,
    iterations, and the weights' distance, beside the oracle's own rounding floor (the same
    solve with every matvec row summed in reverse order)."""
    import oracle as O
    from petrbf_gb300 import workloads as W
    from petrbf_gb300.api import Context
    p = W.lamb_oseen_lattice_1e4()
    prm = p.params()
    with Context(dim=2, sigma=p.sigma, nsigma_box=prm[1], sigma_buffer=prm[2], sigma_trunc=prm[3],
                 device=dev) as c:
        c.interpolate(p.x, p.y, None, p.f)  # first call: allocations and graph capture
        g_gpu, st = c.interpolate(p.x, p.y, None, p.f)
    gpu_s = (st.t_sort_ms + st.t_setup_ms + st.t_solve_ms) * 1e-3
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    out = {"cores": O.num_threads(), "kind": "port"}
    row = {"workload": p.name, "n_points": p.n, "gpu_time_s": gpu_s, "gpu_its": st.its,
           "gpu_pts_per_s": p.n / gpu_s}
    sols = {}
    for factor in ("lu", "chol"):
        t0 = time.perf_counter()
        g = O.grid_for(p.x, p.y, None, *prm)
        perm, cs = O.cell_sort(g, p.x, p.y)
        xs, ys = p.x[perm], p.y[perm]
        t1 = time.perf_counter()
        R = O.Rasm(g, xs, ys, None, cs, factor=factor)
        t2 = time.perf_counter()
        sol, its, reason, _ = O.gmres(g, xs, ys, None, cs, R, p.f[perm])
        t3 = time.perf_counter()
        R.close()
        gc = np.empty_like(sol)
        gc[perm] = sol
        sols[factor] = gc
        row["cpu_" + factor] = {"time_s": t3 - t0, "setup_s": t2 - t1, "gmres_s": t3 - t2, "its": its,
                                "reason": reason, "pts_per_s": p.n / (t3 - t0),
                                "weights_rel_diff_gpu_vs_cpu": rel(g_gpu, gc)}
    g_rev, its_rev, _ = O.rbf_interpolation(p.x, p.y, None, p.f, *prm, factor="chol", reverse_sums=True)
    row["oracle_rounding_floor"] = {"its": its_rev, "weights_rel_diff": rel(g_rev, sols["chol"]),
                                    "what": "the chol oracle against itself with every matvec row summed in "
                                            "reverse order (same operator, another rounding)"}
    row["note"] = ("cpu_lu is the reference's algorithm (PETSc LU blocks); cpu_chol restates the GPU library's "
                   "block arithmetic, so its Schwarz applies are bit-identical to the GPU's")
    out["lamb_oseen_lattice_1e4"] = row
    return out


def _meminfo_available():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def cpu_solve_child(args):
    """(child process) The 4x10^6-point problem solved to 1e-13 by the oracle on all host
    cores, with the GPU library's block arithmetic restated (packed FP64 Cholesky factors
    of the 40,000 blocks, ~127 GB). The address space is capped before the factors are
    allocated, so exhausting it fails this process, not the machine."""
    import resource
    import oracle as O
    from petrbf_gb300 import workloads as W
    p = W.lamb_oseen_2d(args.m, jitter=0.25, seed=args.seed)
    res = {"status": "ok"}
    t0 = time.perf_counter()
    g = O.grid_for(p.x, p.y, None, *p.params())
    perm, cs = O.cell_sort(g, p.x, p.y)
    xs, ys = p.x[perm], p.y[perm]
    nb = O.buffer_counts(g, xs, ys, None, cs).astype(np.float64)
    need = float(np.sum(nb * (nb + 1) / 2) * 8 + 31 * p.n * 8 * 2 + 4e9)
    avail = _meminfo_available()
    res.update(factor_bytes=float(np.sum(nb * (nb + 1) / 2) * 8), mem_available=avail, mem_needed=need)
    if need > 0.8 * avail:
        res["status"] = "skipped: the packed FP64 factors need %.0f GB, %.0f GB available" % (need / 1e9, avail / 1e9)
    else:
        lim = int(need + 24e9)
        resource.setrlimit(resource.RLIMIT_AS, (lim, lim))
        t1 = time.perf_counter()
        R = O.Rasm(g, xs, ys, None, cs, factor="chol")
        t2 = time.perf_counter()
        sol, its, reason, _ = O.gmres(g, xs, ys, None, cs, R, p.f[perm])
        t3 = time.perf_counter()
        R.close()
        gc = np.empty_like(sol)
        gc[perm] = sol
        res.update(time_s=t3 - t0, setup_s=t2 - t1, gmres_s=t3 - t2, its=its, reason=reason, cores=O.num_threads(),
                   setup_status=R.status)
        np.save(args.cpu_solve_child + ".g.npy", gc)
    with open(args.cpu_solve_child, "w") as fh:
        json.dump(res, fh)


def cpu_solve_full(p, args, g_gpu, gpu):
    """The config-2 problem (4x10^6 points) solved on the host cores in a child process
    (cpu_solve_child), measured, beside the plain FP64 GPU solve of the same points."""
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "cpu.json")
        cmd = [sys.executable, os.path.abspath(__file__), "--cpu-solve-child", out, "--m", str(args.m),
               "--seed", "12345"]
        t0 = time.perf_counter()
        r = subprocess.run(cmd, capture_output=True, text=True)
        wall = time.perf_counter() - t0
        if r.returncode != 0 or not os.path.exists(out):
            return {"status": "failed: rc %d %s" % (r.returncode, (r.stderr or "")[-300:]), "wall_s": wall}
        res = json.load(open(out))
        if res.get("status") == "ok":
            gc = np.load(out + ".g.npy")
            res["weights_rel_diff_gpu_vs_cpu"] = float(np.linalg.norm(g_gpu - gc) / np.linalg.norm(gc))
            res["gpu_its"] = gpu["its"]
            res["gpu_fp64_time_s"] = gpu["time_s"]
            res["cpu_pts_per_s"] = p.n / res["time_s"]
            res["kind"] = "port (block arithmetic of the GPU library restated: Cholesky)"
        res["wall_s"] = wall
        return res


def solve_section(p, dev, rank):
    """Time-to-1e-13 of the full interpolation (cell list, RASM set-up, Krylov): plain FP64
    (the reference's algorithm), mixed precision, and both with the learned initial guess
    (petrbf_gb300/data/guess_mlp.npz), each with the off-grid interpolation error."""
    from petrbf_gb300 import learned as L
    from petrbf_gb300.api import Context
    out = {}
    have_model = os.path.exists(L.MODEL_PATH)
    variants = [("fp64", "zero"), ("mixed", "zero")]
    if have_model:
        variants += [("mixed", "learned"), ("fp64", "learned")]
    g64 = None
    for prec, guess in variants:
        with Context(dim=2, sigma=p.sigma, nsigma_box=8, sigma_buffer=24, sigma_trunc=24,
                     precision=prec, guess=guess, device=dev) as c:
            if guess == "learned":
                L.install(c)
            t0 = time.perf_counter()
            g, st = c.interpolate(p.x, p.y, None, p.f)
            wall = time.perf_counter() - t0
            err = offgrid_error(c, p, g)
        if prec == "fp64" and guess == "zero":
            g64 = g
        dev_s = (st.t_sort_ms + st.t_setup_ms + st.t_solve_ms) * 1e-3
        key = prec if guess == "zero" else prec + "+learned"
        out[key] = {"time_s": dev_s, "wall_s_incl_copies": wall, "pts_per_s": p.n / dev_s,
                    "its": st.its, "outer_its": st.outer_its, "reason": st.reason,
                    "true_rel_resid": st.true_rel_resid, "log10_err_offgrid": err,
                    "t_sort_ms": st.t_sort_ms, "t_setup_ms": st.t_setup_ms,
                    "t_solve_ms": st.t_solve_ms, "t_guess_ms": st.t_guess_ms,
                    "guess_used": st.guess_used, "guess_rel_resid": st.guess_rel_resid,
                    "max_block": st.max_block, "blocks_shifted": st.nblocks_fallback}
    out["mixed_speedup_vs_fp64"] = out["fp64"]["time_s"] / out["mixed"]["time_s"]
    if have_model:
        out["learned_mixed_speedup_vs_fp64"] = out["fp64"]["time_s"] / out["mixed+learned"]["time_s"]
    out["metric"] = "pts/s to 1e-13 residual"
    return out, g64


def vortex3d_section(m3=128, m_oracle=32):
    """Config 3, the 3D mixed-precision form: an m3^3 jittered lattice (128^3 = 2.1x10^6),
    three vortex-ring right-hand sides, FP32 matvec + FP32 block Cholesky inside FP64
    refinement to 1e-12, against the plain FP64 GPU solve of the same problem; and at
    m_oracle^3 (a size the host cores solve in the run) every component's weights against
    the FP64 oracle (the reference's LU blocks, basic Schwarz, GMRES to 1e-12)."""
    import oracle as O
    from petrbf_gb300 import workloads as W
    from petrbf_gb300.api import Context

    def solve(p, prec):
        with Context(dim=3, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
                     sigma_trunc=p.sigma_trunc, precision=prec, rtol=1e-12, pc="asm") as c:
            t0 = time.perf_counter()
            g, st = c.interpolate(p.x, p.y, p.z, p.f)
            wall = time.perf_counter() - t0
        dev_s = (st.t_sort_ms + st.t_setup_ms + st.t_solve_ms) * 1e-3
        return g, {"time_s": dev_s, "wall_s_incl_copies": wall, "pts_per_s": p.n / dev_s, "its": st.its,
                   "outer_its": st.outer_its, "reason": st.reason, "true_rel_resid": st.true_rel_resid,
                   "t_sort_ms": st.t_sort_ms, "t_setup_ms": st.t_setup_ms, "t_solve_ms": st.t_solve_ms,
                   "max_block": st.max_block, "pairs_per_matvec": st.pairs_per_matvec}

    names = ("omega_x", "omega_y", "omega_z")
    p = W.vortex_ring_3d(m=m3)
    out = {"workload": p.name, "n_points": p.n, "nsigma_box": p.nsigma_box, "sigma_buffer": p.sigma_buffer,
           "sigma_trunc": p.sigma_trunc, "pc": "asm (basic additive Schwarz)", "rhs": 3}
    gm, out["mixed"] = solve(p, "mixed")
    gd, out["fp64"] = solve(p, "fp64")
    comp = {}
    for k, name in enumerate(names):
        dn = float(np.linalg.norm(gd[:, k]))
        diff = float(np.linalg.norm(gm[:, k] - gd[:, k]))
        comp[name] = {"weights_rel_diff_vs_fp64_gpu": diff / dn if dn > 0 else None, "weights_abs_diff": diff,
                      "fp64_weights_norm": dn}
    out["components_vs_fp64_gpu"] = comp
    out["mixed_speedup_vs_fp64"] = out["fp64"]["time_s"] / out["mixed"]["time_s"]
    # against the FP64 oracle at a size the host solves in the run
    q = W.vortex_ring_3d(m=m_oracle)
    gqm, rm = solve(q, "mixed")
    gqd, rd = solve(q, "fp64")
    t0 = time.perf_counter()
    g = O.grid_for(q.x, q.y, q.z, *q.params())
    perm, cs = O.cell_sort(g, q.x, q.y, q.z)
    R = O.Rasm(g, q.x[perm], q.y[perm], q.z[perm], cs, basic=True)
    orc = {"workload": q.name, "n_points": q.n, "gpu_mixed": rm, "gpu_fp64": rd}
    for k, name in enumerate(names):
        sol, its, reason, _ = O.gmres(g, q.x[perm], q.y[perm], q.z[perm], cs, R, q.f[perm, k], rtol=1e-12,
                                      max_it=1000)
        go = np.empty_like(sol)
        go[perm] = sol
        dn = float(np.linalg.norm(go))
        e = {"oracle_its": its, "oracle_reason": reason}
        for lab, gg in (("mixed", gqm), ("fp64", gqd)):
            diff = float(np.linalg.norm(gg[:, k] - go))
            # omega_z of a ring about the z axis is identically zero: absolute error
            e["weights_%s_vs_oracle" % lab] = diff / dn if dn > 0 else diff
        e["measure"] = "relative 2-norm" if dn > 0 else "absolute 2-norm (zero field)"
        orc[name] = e
    R.close()
    orc["oracle_time_s"] = time.perf_counter() - t0
    orc["oracle_cores"] = O.num_threads()
    out["components_vs_fp64_oracle"] = orc
    return out


def run_vortex3d(args, rank):
    out = vortex3d_section(args.m3)
    print(json.dumps({"metric": "pts/s to 1e-12, 3D mixed, 3 right-hand sides", "value": out["mixed"]["pts_per_s"],
                      "unit": "pts/s", "higher_is_better": True, "dtype": "f32/f64", "data": "synthetic",
                      "config": {"workload": out["workload"], "n_points": out["n_points"]}, "solve": out}),
          flush=True)


def batch2d_section(nprob=256, max_it=1000):
    """Config 4, the batched form: nprob problems of uneven N solved together (basic Schwarz,
    FP64 outer residual to 1e-13), on uniform-random (scattered) points and on jittered
    lattices of the same sizes, FP64 and mixed. The second call of each is reported (the
    autotuner's schedule then comes from its cache; the first call's tuning time is given);
    the batched sums' rates against the FP64 peak measured in the run."""
    import torch
    from petrbf_gb300 import workloads as W
    from petrbf_gb300.api import batch_interpolate
    peak = fp64_peak_tflops(torch)
    out = {}
    for kind, probs in (("scattered", W.batch_scattered(nprob=nprob)), ("lattice", W.batch_lattice(nprob=nprob))):
        for prec in ("fp64", "mixed"):
            res = {}
            for rep in range(2):
                t0 = time.perf_counter()
                g, its, reason, st = batch_interpolate(probs, rtol=1e-13, pc="asm", max_it=max_it, precision=prec)
                wall = time.perf_counter() - t0
                res[rep] = (st, wall, its, reason)
            st, wall, its, reason = res[1]
            dev_s = (st.t_sort_ms + st.t_setup_ms + st.t_tune_ms + st.t_solve_ms) * 1e-3
            gp = st.pairs_per_matvec / (st.t_matvec_ms * 1e-3) / 1e9
            row = dict(st.as_dict(), pts_per_s=st.points / dev_s, time_s=dev_s, wall_s=wall,
                       first_call_tune_ms=res[0][0].t_tune_ms, its_median=float(np.median(its)),
                       its_max=int(np.max(its)), unconverged=int(np.sum(reason <= 0)),
                       matvec_gpairs_per_s=gp,
                       matvec_roofline={"bound": "fp64", "achieved": FLOPS_PER_PAIR * gp / 1e3, "peak": peak,
                                        "unit": "TFLOP/s", "frac": FLOPS_PER_PAIR * gp / 1e3 / peak,
                                        "peak_source": "in-run cuBLAS DGEMM 8192^3"})
            if st.t_matvec32_ms > 0:
                row["matvec32_gpairs_per_s"] = st.pairs_per_matvec / (st.t_matvec32_ms * 1e-3) / 1e9
            out["%s_%s" % (kind, prec)] = row
    out["n_problems"] = nprob
    return out


def run_batch2d(args, rank):
    out = batch2d_section(args.nprob, args.batch_max_it)
    best = max(out["scattered_fp64"]["pts_per_s"], out["scattered_mixed"]["pts_per_s"])
    print(json.dumps({"metric": "pts/s to 1e-13, batched 2D", "value": best,
                      "unit": "pts/s", "higher_is_better": True, "dtype": "f64 outer residual", "data": "synthetic",
                      "config": {"workload": "batched_2d_%d_problems" % args.nprob,
                                 "n_points": out["scattered_fp64"]["points"], "pc": "asm (basic additive Schwarz)"},
                      "batch": out}), flush=True)


def learned_heldout_section(dev, seeds=(2001, 2002, 2003), m=2000):
    """Config 5 on held-out problems: Lamb-Oseen fields of the training distribution (G in
    [0.5, 2], core radius in [0.1, 0.3], centre in [-0.5, 0.5]^2) drawn with seeds outside
    the training set (1000-1007), on 4x10^6-point jittered lattices; GMRES iterations and
    time to 1e-13 with the learned initial guess against the zero guess, mixed and plain
    FP64, with the off-grid error of each."""
    from petrbf_gb300 import learned as L
    from petrbf_gb300.api import Context
    if not os.path.exists(L.MODEL_PATH):
        return {"status": "no trained model"}
    rows = []
    for sd in seeds:
        p = L.training_problem(sd, m=m)
        row = {"seed": sd, "n_points": p.n, "G": p.meta["G"], "core_radius": p.meta["rc"]}
        for prec in ("mixed", "fp64"):
            for guess in ("zero", "learned"):
                with Context(dim=2, sigma=p.sigma, nsigma_box=8, sigma_buffer=24, sigma_trunc=24, precision=prec,
                             guess=guess, device=dev) as c:
                    if guess == "learned":
                        L.install(c)
                    g, st = c.interpolate(p.x, p.y, None, p.f)
                dev_s = (st.t_sort_ms + st.t_setup_ms + st.t_solve_ms) * 1e-3  # t_solve includes the guess
                row["%s_%s" % (prec, guess)] = {"time_s": dev_s, "its": st.its, "outer_its": st.outer_its,
                                                "reason": st.reason, "true_rel_resid": st.true_rel_resid,
                                                "guess_used": st.guess_used, "guess_rel_resid": st.guess_rel_resid}
            z, l = row[prec + "_zero"], row[prec + "_learned"]
            row[prec + "_speedup_learned_vs_zero"] = z["time_s"] / l["time_s"]
        row["learned_mixed_vs_zero_fp64"] = row["fp64_zero"]["time_s"] / row["mixed_learned"]["time_s"]
        rows.append(row)
    return {"problems": rows, "seeds": list(seeds),
            "mean_speedup_learned_vs_zero": {prec: float(np.mean([r[prec + "_speedup_learned_vs_zero"] for r in rows]))
                                             for prec in ("mixed", "fp64")}}


def run_seam_case(steps=10):
    """Times prbf_gpumatmult_2d (host arrays in and out, copies included, as the reference's
    seam does) on the packed 10^6-point lattice."""
    from petrbf_gb300.api import gpumatmult
    from petrbf_gb300.workloads import pack_gpumatmult_2d
    tx, ty, sx, sy, sg, off, sigma, npts = pack_gpumatmult_2d()
    iblok = len(off) - 1
    for _ in range(3):
        gpumatmult(tx, ty, None, sx, sy, None, sg, off, sigma)
    t0 = time.perf_counter()
    for _ in range(steps):
        gpumatmult(tx, ty, None, sx, sy, None, sg, off, sigma)
    dt = (time.perf_counter() - t0) / steps
    slot_pairs = 128 * int(off[-1])
    h2d = 4 * (2 * len(tx) + 3 * int(off[-1]) + len(off))
    print(json.dumps({"case": "seam_2d", "points": npts, "blocks": iblok, "sources_packed": int(off[-1]),
                      "slot_pairs_per_call": slot_pairs, "ms_per_call": dt * 1e3,
                      "slot_gpairs_per_s_e2e": slot_pairs / dt / 1e9, "h2d_bytes": h2d, "d2h_bytes": 4 * len(tx)}),
          flush=True)


def run_case(name):
    """Small single-kernel cases for ncu captures (a few GB on the device at most)."""
    import torch
    from petrbf_gb300 import workloads as W
    from petrbf_gb300.api import Context, batch_interpolate
    if name in ("gauss32_2d", "gauss64_2d"):  # 10^6-point jittered lattice, 8-sigma-cell geometry
        x, y, h = W.lattice_2d(1000, jitter=0.25, seed=1)
        c = Context(dim=2, sigma=h / 0.8, nsigma_box=8, sigma_buffer=24, sigma_trunc=24)
        c.matvec_setup(x, y)
        v = torch.randn(len(x), dtype=torch.float64, device="cuda")
        o = torch.empty_like(v)
        torch.cuda.synchronize()
        for _ in range(3):
            c.matvec_dev(v.data_ptr(), o.data_ptr(), cell_order=True, fp32=(name == "gauss32_2d"))
        c.synchronize()
    elif name in ("gauss32_3d", "gauss64_3d"):  # 48^3 jittered lattice, 3D vortex-ring geometry
        x, y, z, h = W.lattice_3d(48, jitter=0.25, seed=1)
        c = Context(dim=3, sigma=h / 0.8, nsigma_box=3, sigma_buffer=7, sigma_trunc=17)
        c.matvec_setup(x, y, z)
        v = torch.randn(len(x), dtype=torch.float64, device="cuda")
        o = torch.empty_like(v)
        torch.cuda.synchronize()
        for _ in range(3):
            c.matvec_dev(v.data_ptr(), o.data_ptr(), cell_order=True, fp32=(name == "gauss32_3d"))
        c.synchronize()
    elif name == "asm32_3d":  # FP32 basic-Schwarz blocks of the 48^3 case
        x, y, z, h = W.lattice_3d(48, jitter=0.25, seed=1)
        c = Context(dim=3, sigma=h / 0.8, nsigma_box=3, sigma_buffer=7, sigma_trunc=17, pc="asm")
        c.matvec_setup(x, y, z)
        c.pc_setup("mixed")
        r = np.random.default_rng(1).standard_normal(len(x))
        for _ in range(3):
            c.pc_apply(r)
    elif name == "chol64_2d":  # FP64 block factorisation, 400^2 jittered lattice, 8-sigma-cell blocks
        x, y, h = W.lattice_2d(400, jitter=0.25, seed=1)
        c = Context(dim=2, sigma=h / 0.8, nsigma_box=8, sigma_buffer=24, sigma_trunc=24)
        c.matvec_setup(x, y)
        c.pc_setup("fp64")
        r = np.random.default_rng(1).standard_normal(len(x))
        for _ in range(3):
            c.pc_apply(r)
    elif name == "chol32_2d":  # FP32 restricted blocks (S_c form), 400^2 jittered lattice, 8-sigma-cell blocks
        x, y, h = W.lattice_2d(400, jitter=0.25, seed=1)
        c = Context(dim=2, sigma=h / 0.8, nsigma_box=8, sigma_buffer=24, sigma_trunc=24)
        c.matvec_setup(x, y)
        c.pc_setup("mixed")
        r = np.random.default_rng(1).standard_normal(len(x))
        for _ in range(3):
            c.pc_apply(r)
    elif name == "batch":  # 24 problems of the batched form (N up to 6x10^4)
        batch_interpolate(W.batch_scattered(nprob=24, nmax=60000), rtol=1e-13, pc="asm")
    elif name == "batch_mixed":  # 24 jittered-lattice problems of the batched form, mixed
        batch_interpolate(W.batch_lattice(nprob=24, nmax=60000), rtol=1e-13, pc="asm", precision="mixed")
    elif name == "mlp_guess":  # learned-guess inference on a 10^6-point lattice (tensor-core GEMMs)
        from petrbf_gb300 import learned as L
        p = L.training_problem(2001, m=1000)
        with Context(dim=2, sigma=p.sigma, guess="learned") as c:
            L.install(c)
            for _ in range(3):
                L.guess(c, p.x, p.y, p.f)
    elif name in ("mixed3d", "mixed3d_small"):  # the 3D mixed solve: vortex ring, 3 right-hand sides, to 1e-12
        p = W.vortex_ring_3d(m=128 if name == "mixed3d" else 48)  # 128^3 (2.1x10^6 points) or 48^3
        with Context(dim=3, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
                     sigma_trunc=p.sigma_trunc, precision="mixed", rtol=1e-12, pc="asm") as c:
            _, st = c.interpolate(p.x, p.y, p.z, p.f)
        print("its", st.its, "outer", st.outer_its, "solve_ms", st.t_solve_ms, "setup_ms", st.t_setup_ms,
              "reason", st.reason, "true_rel_resid", st.true_rel_resid)
    elif name == "mixed2d":  # the 2D mixed solve: 2000 x 2000 jittered lattice (4x10^6 points), to 1e-13
        p = W.lamb_oseen_2d(2000, jitter=0.25, seed=12345)
        with Context(dim=2, sigma=p.sigma, nsigma_box=8, sigma_buffer=24, sigma_trunc=24, precision="mixed",
                     rtol=1e-13) as c:
            _, st = c.interpolate(p.x, p.y, None, p.f)
        print("its", st.its, "outer", st.outer_its, "solve_ms", st.t_solve_ms, "setup_ms", st.t_setup_ms,
              "reason", st.reason, "true_rel_resid", st.true_rel_resid)
    elif name == "time3d":  # CUDA-event times of the 3D single-vector products, 128^3 vortex-ring lattice
        p = W.vortex_ring_3d(m=128)
        c = Context(dim=3, sigma=p.sigma, nsigma_box=p.nsigma_box, sigma_buffer=p.sigma_buffer,
                    sigma_trunc=p.sigma_trunc)
        c.matvec_setup(p.x, p.y, p.z)
        v = torch.randn(p.n, dtype=torch.float64, device="cuda")
        o = torch.empty_like(v)
        stream = torch.cuda.ExternalStream(c.stream)
        for fp32 in (False, True):
            for _ in range(3):
                c.matvec_dev(v.data_ptr(), o.data_ptr(), cell_order=True, fp32=fp32)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(5):
                c.matvec_dev(v.data_ptr(), o.data_ptr(), cell_order=True, fp32=fp32)
            e1.record(stream)
            c.synchronize()
            print("fp32" if fp32 else "fp64", "ms per product %.3f" % (e0.elapsed_time(e1) / 5),
                  "Gpairs/s %.1f" % (c.matvec_info()["pairs"] / (e0.elapsed_time(e1) / 5 * 1e-3) / 1e9))
        c.close()
    elif name == "seam_2d":  # the gpumatmult seam on the packed arrays of a 10^6-point lattice
        run_seam_case()
        return
    else:
        raise SystemExit("unknown case " + name)
    print("case", name, "done")


def main():
    args = parse()
    if args.cpu_solve_child:
        cpu_solve_child(args)
        return
    if args.case:
        run_case(args.case)
        return
    rank, world = dist_init(args.gpus)
    if args.workload == "vortex3d":
        if rank == 0:
            run_vortex3d(args, rank)
    elif args.workload == "batch2d":
        if rank == 0:
            run_batch2d(args, rank)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
