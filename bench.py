"""Benchmark of the stencil-apply path (one JSON line on rank 0).

Default workload (the headline configuration): 3-D 256^3 Float64 Laplacian,
the sum of CenteredDifference{1,2,3}(2, 4, h, 256), h = 1/257, with
RobinBC((1, .5, 0), (1, .5, 0), h, 1) on every face; u = a smooth random
Fourier field (8 modes per axis, amplitudes U(-1,1)) plus 1e-3 white noise.
A step is one fused apply du = (Dxx+Dyy+Dzz)*Q*u over the whole grid.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

`value` is device-resident throughput (grid points/s over all ranks, inputs
in HBM, 4 rotating input/output pairs = 1.07 GB so no step reads data another
step left in the 129 MB L2).  `e2e` is the same metric through the C ABI's
host-buffer entry point (deo_apply_host: pinned host input -> device ->
pinned host output, copies inside the timed region).  `--impl reference`
times the CPU restatement of the reference's loops (the oracle; the
reference itself is Julia, which is not installed) on all host cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
# optional folder for the clock samples and the autotuner cache (DEO_REPORT_DIR)
REPORT_DIR = os.environ.get("DEO_REPORT_DIR", "") or None
if REPORT_DIR and not os.path.isdir(REPORT_DIR):
    REPORT_DIR = None
sys.path.insert(0, os.path.join(ROOT, "diffeqoperators.jl_gb300"))

SEED = 20251203
L2_BYTES = 129 * 2 ** 20


# ---------------------------------------------------------------------------
# synthetic inputs
# ---------------------------------------------------------------------------
def fourier_field(n: int, modes: int = 8, seed: int = SEED, noise: float = 1e-3, dtype=np.float64):
    """Sum over axes of 8 sine/cosine modes with U(-1,1) amplitudes + white noise, Julia layout."""
    rng = np.random.default_rng(seed)
    x = np.arange(1, n + 1) / (n + 1)
    f = []
    for _ in range(3):
        a = rng.uniform(-1, 1, modes)
        b = rng.uniform(-1, 1, modes)
        k = np.arange(1, modes + 1)
        f.append((a[None, :] * np.sin(np.pi * k[None, :] * x[:, None]) +
                  b[None, :] * np.cos(np.pi * k[None, :] * x[:, None])).sum(1))
    u = (f[0][:, None, None] + f[1][None, :, None] + f[2][None, None, :])
    u = u + noise * rng.standard_normal(u.shape)
    return np.asfortranarray(u.astype(dtype))


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(name: str):
    """DRAM bytes per launch recorded from an ncu capture (profiles/<name>.md,
    line `traffic_bytes_per_launch: N`), or None."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = os.path.join(REPORT_DIR or tempfile.gettempdir(), f".clocks_{os.getpid()}.csv")

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# distributed plumbing (N>1: independent replicas, no data-path collective)
# ---------------------------------------------------------------------------
def dist_init():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def host_link_gbs(h_in, h_out, reps: int = 6) -> float:
    """GB/s each way of the host link with a host->device and a
    device->host copy of these pinned buffers in flight at once (two streams,
    the copy engines), as the pipelined host applies move them: the bound on
    the end-to-end throughput."""
    import torch
    d_in = torch.empty_like(h_in, device="cuda")
    d_out = torch.empty_like(h_out, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def both():
        with torch.cuda.stream(s1):
            d_in.copy_(h_in, non_blocking=True)
        with torch.cuda.stream(s2):
            h_out.copy_(d_out, non_blocking=True)

    for _ in range(2):
        both()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        both()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    del d_in, d_out
    return h_in.numel() * h_in.element_size() / dt / 1e9


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# FP64 issue rate of this part, measured with a throughput probe on the GPU
# machine (1216 CTAs x 256 threads, 8 independent DFMA chains per thread, best
# of 5): 1.68 DFMA per clock per SM.
FP64_PER_CLK_PER_SM = 1.68
NUM_SMS = 152


def fp64_order_bound(achieved_gbs: float, bytes_per_point: float, fp64_per_point: int = 17,
                     sm_mhz: float = 2070.0) -> dict:
    """The FP64 roofline of evaluating every point in the reference's tap order
    (17 FP64 instructions per point for the 4th-order 3-D Laplacian: 3 x 5 taps
    + 2 term sums), as algorithmic GB/s, beside the HBM one: `frac` > 1 means
    the kernel outruns what FP64 arithmetic could reach (the fixed-point
    interior issues no FP64 instruction for most points)."""
    pts = FP64_PER_CLK_PER_SM * NUM_SMS * sm_mhz * 1e6 / fp64_per_point
    gbs = pts * bytes_per_point / 1e9
    return {"gbs": gbs, "frac": achieved_gbs / gbs, "fp64_per_point": fp64_per_point,
            "basis": f"{FP64_PER_CLK_PER_SM} FP64 instructions per clock per SM (measured), {NUM_SMS} SMs, "
                     f"{sm_mhz:.0f} MHz"}


def shard(costs, rank: int, ws: int) -> list:
    """Indices of the instances (batched / served workloads) that `rank` owns,
    increasing.  Greedy by cost: instances in decreasing cost (ties by index)
    go to the least loaded rank (ties to the lower rank), so every rank
    computes the same partition without communicating.  Ranks run independent
    replicas of the path on their own instances; no collective touches the
    data."""
    n = len(costs)
    if ws == 1:
        return list(range(n))
    load, own = [0] * ws, [[] for _ in range(ws)]
    for i in sorted(range(n), key=lambda i: (-costs[i], i)):
        r = min(range(ws), key=lambda k: (load[k], k))
        load[r] += costs[i]
        own[r].append(i)
    return sorted(own[rank])


def gather_objects(x, ws: int) -> list:
    """Every rank's `x`, in rank order (host objects; the ranks' results
    and latencies, never device data)."""
    if ws == 1:
        return [x]
    import torch.distributed as dist
    out = [None] * ws
    dist.all_gather_object(out, x)
    return out


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def lap3d_setup(n: int, dtype_name: str):
    import torch

    import deo
    h = 1.0 / (n + 1)
    tdt = torch.float64 if dtype_name == "f64" else torch.float32
    A = deo.CenteredDifference(2, 4, h, n, axis=1) + deo.CenteredDifference(2, 4, h, n, axis=2) + \
        deo.CenteredDifference(2, 4, h, n, axis=3)
    Q = deo.compose(*deo.RobinBC((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), (h, h, h), 1, (n, n, n)))
    AQ = A * Q
    plan = deo.plan_for(AQ.terms(), (n, n, n), 0 if dtype_name == "f64" else 1)
    return AQ, plan, tdt


def cpu_oracle_lap3d(u: np.ndarray, n: int, nthreads: int, reps: int):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    h = 1.0 / (n + 1)
    q = O.robin((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), h, 1)
    terms = [(O.centered(2, 4, h, n, axis=k), q) for k in (1, 2, 3)]
    out = np.zeros(u.shape, order="F")
    O.apply(terms, u, out=out, nthreads=nthreads)  # warm-up
    t0 = time.perf_counter()
    for _ in range(reps):
        O.apply(terms, u, out=out, nthreads=nthreads)
    return (time.perf_counter() - t0) / reps


def run_ours(args, ws, rank):
    import torch

    import deo
    n = args.n
    dtype_name = "f32" if args.workload == "lap3d_f32" else "f64"
    AQ, plan, tdt = lap3d_setup(n, dtype_name)
    if getattr(args, "exact_sums", -1) >= 0:
        plan.set_option(deo.DEO_OPT_EXACT_SUMS, args.exact_sums)
    if getattr(args, "serial_shell", False):
        plan.set_option(deo.DEO_OPT_CONCURRENT_SHELL, 0)
    if getattr(args, "f32_scalar", False):
        plan.set_option(deo.DEO_OPT_F32_VECTOR, 0)
    esize = 8 if dtype_name == "f64" else 4
    npts = n ** 3
    u_host = fourier_field(n, seed=SEED + rank, dtype=np.float64 if esize == 8 else np.float32)
    nbuf = max(2, int(np.ceil(4 * L2_BYTES / (2 * npts * esize))))
    nbuf = min(nbuf, 4)
    us, dus = [], []
    for b in range(nbuf):
        t = deo.julia_array((n, n, n), tdt, "cuda")
        t.copy_(torch.from_numpy(u_host))
        us.append(t)
        dus.append(deo.julia_array((n, n, n), tdt, "cuda"))
    stream = torch.cuda.current_stream()
    # execution choices (tile shape, shell kernel, shell beside the interior or after it), all
    # bit-identical: timed on this workload by the library's autotuner before the warm-up
    tuned = None
    if not (getattr(args, "no_autotune", False) or getattr(args, "serial_shell", False) or
            getattr(args, "f32_scalar", False)):
        tuned = plan.autotune(us[0], dus[0], os.path.join(REPORT_DIR, "plan_autotune.cache") if REPORT_DIR else None)
    for i in range(args.warmup):
        plan.apply(us[i % nbuf], dus[i % nbuf])
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record(stream)
        for i in range(args.steps):
            plan.apply(us[i % nbuf], dus[i % nbuf])
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    barrier(ws)
    ms = max_over_ranks(ms, ws)
    ms_step = ms / args.steps
    value = ws * npts / (ms_step / 1e3)

    # e2e through the C ABI with host buffers (pinned)
    uh = torch.from_numpy(np.ascontiguousarray(u_host.ravel(order="F"))).pin_memory()
    dh = torch.empty_like(uh).pin_memory()
    lib = deo.lib()
    st = C.c_void_p(stream.cuda_stream)
    for _ in range(2):
        deo._lib.check(lib.deo_apply_host(plan.handle, C.c_void_p(uh.data_ptr()), C.c_void_p(dh.data_ptr()), st))
    # pipelined: the copy of step i+1's input, step i's apply and the copy of step i-1's result overlap
    for _ in range(2):
        plan.apply_host_async(uh, dh)
    plan.host_sync()
    barrier(ws)
    t0 = time.perf_counter()
    e2e_steps = max(3, min(args.steps, 50))
    for _ in range(e2e_steps):
        plan.apply_host_async(uh, dh)
    plan.host_sync()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s = max_over_ranks(e2e_s, ws)
    # check the e2e output against the device path once (same kernel)
    dev_out = dus[(args.steps - 1) % nbuf].permute(2, 1, 0).contiguous().view(-1).cpu()
    if not torch.equal(dev_out, dh):
        raise RuntimeError("host-buffer path disagrees with the device path")
    link = host_link_gbs(uh, dh)  # the copies alone, both directions at once (overwrites dh)

    hbm, peak_kind = peaks()
    alg_bytes = 2 * esize * npts
    step_achieved = alg_bytes / (ms_step / 1e3) / 1e9
    kernels = plan.kernels
    # the dominant kernel alone: CUDA events around each launch of an apply
    # (a separate loop over the same rotating buffers, one apply per sync)
    plan.set_option(deo.DEO_OPT_LAUNCH_TIMING, 1)
    per_launch = []
    for i in range(min(args.steps, 200)):
        plan.apply(us[i % nbuf], dus[i % nbuf])
        per_launch.append(plan.launch_times())
    plan.set_option(deo.DEO_OPT_LAUNCH_TIMING, 0)
    launch_ms = np.mean(np.asarray(per_launch), axis=0)
    H = 2                  # stencil radius of d2 a4
    box = n - 2 * max(1, H)  # interior box: rows clear of boundary stencils (1 per side) and ghosts
    if len(kernels) == 2:
        # interior kernel: reads the box and its H-deep halo on each face once, writes the box once
        k_bytes = esize * (box ** 3 + 6 * H * box ** 2 + box ** 3)
    else:
        k_bytes = alg_bytes
    achieved = k_bytes / (launch_ms[0] / 1e3) / 1e9
    path = " + ".join(kernels)
    traffic = profiled_traffic(f"{kernels[0]}_lap3d_{n}_{dtype_name}")
    line = {
        "metric": "grid-pts/s (3-D 256^3 Laplacian apply)",
        "value": value,
        "unit": "grid-pts/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": dtype_name,
        "data": "synthetic (seeded Fourier field + noise, same shape and distribution as the reference config)",
        "config": {"workload": f"laplacian3d_{n}^3_{dtype_name}_d2a4_robin_all_faces", "grid": [n, n, n],
                   "operator": "CenteredDifference{1,2,3}(2,4,1/257,256) summed",
                   "bc": "RobinBC((1,.5,0),(1,.5,0),h,1) composed on every face",
                   "l2_policy": f"{nbuf} rotating input/output pairs ({nbuf * 2 * npts * esize / 2**30:.2f} GiB) > L2",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU", "kernel_path": path,
                   "autotuned": tuned, "autotune_times_us": plan.autotune_times() if tuned else None},
        "e2e": {"value": ws * npts / e2e_s, "unit": "grid-pts/s", "h2d_bytes_per_step": npts * esize,
                "d2h_bytes_per_step": npts * esize,
                "path": "deo_apply_host_async + deo_plan_host_sync (C ABI, pinned host buffers, copies overlapped "
                        "with the applies of neighbouring steps)",
                # the host link with both copies in flight: each step moves npts * esize each way
                "host_link_gbs_each_way": link, "link_bound": ws * link * 1e9 / esize,
                "frac_of_link_bound": (npts / e2e_s) / (link * 1e9 / esize)},
        "gpu_launches": args.steps * len(kernels),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "kernel": kernels[0], "peak_source": f"{peak_kind} hbm_gbs (burst copy)",
                     "algorithmic_bytes_per_launch": k_bytes, "launch_ms": [float(x) for x in launch_ms],
                     "launch_share": [float(x / launch_ms.sum()) for x in launch_ms],
                     "step_achieved": step_achieved, "step_frac": step_achieved / hbm},
        "clocks": clk.summary(),
    }
    if dtype_name == "f64":
        # the min(HBM, FP64) view: the FP64 bound of evaluating in the reference's tap order
        fb = fp64_order_bound(achieved, k_bytes / box ** 3)
        line["roofline"]["fp64_order_bound"] = fb
        line["roofline"]["frac_of_min_hbm_fp64"] = achieved / min(hbm, fb["gbs"])
    if rank == 0 and not args.no_cpu:
        t_one = cpu_oracle_lap3d(np.asarray(u_host, dtype=np.float64), n, 1, 1)
        reps = int(max(1, min(30, 10.0 // max(t_one, 1e-3))))  # about 10 s of CPU work
        t_cpu = cpu_oracle_lap3d(np.asarray(u_host, dtype=np.float64), n, 1, reps)
        line["cpu_baseline"] = {"value": npts / t_cpu, "unit": "grid-pts/s", "cores": 1, "kind": "port",
                                "sample": f"{reps} full {n}^3 Float64 applies, 1 thread, C++ restatement "
                                          f"of the reference loops (oracle/deo_oracle.cpp)"}
    return line


# ---------------------------------------------------------------------------
# secondary workloads (each prints its own JSON line; the default stays lap3d)
# ---------------------------------------------------------------------------
def _event_time(fn, steps, warmup):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps / 1e3


def run_line1d(args):
    """1-D N=1024, CenteredDifference(2,2,1/1025,1024), Dirichlet0BC: launch-latency bound."""
    import torch

    import deo
    N = 1024
    h = 1.0 / (N + 1)
    rng = np.random.default_rng(SEED)
    u = np.sin(2 * np.pi * np.arange(1, N + 1) * h) + 0.01 * rng.standard_normal(N)
    AQ = deo.CenteredDifference(2, 2, h, N) * deo.Dirichlet0BC(np.float64)
    plan = deo.plan_for(AQ.terms(), (N,), 0)
    ud = torch.from_numpy(u).cuda()
    du = torch.empty_like(ud)
    s = _event_time(lambda: plan.apply(ud, du), args.steps, args.warmup)
    # CUDA-graph replay of 100 applies (how a solver loop would issue them)
    g = torch.cuda.CUDAGraph()
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(st):
        plan.apply(ud, du)
        torch.cuda.synchronize()
        with torch.cuda.graph(g, stream=st):
            for _ in range(100):
                plan.apply(ud, du)
    torch.cuda.current_stream().wait_stream(st)
    sg = _event_time(lambda: g.replay(), max(3, args.steps // 100), 2) / 100
    return {"metric": "grid-pts/s (1-D N=1024 apply)", "workload": "line1d_1024_f64_d2a2_dirichlet0",
            "value": N / s, "unit": "grid-pts/s", "us_per_apply": s * 1e6, "us_per_apply_graph": sg * 1e6,
            "value_graph": N / sg, "dtype": "f64"}


def nonuniform2d_ops(n, field_dev=None):
    import deo
    i = np.arange(n + 1)
    dx = 1.0 + 0.5 * np.sin(2 * np.pi * i / n)
    dx = dx / dx.sum()
    rng = np.random.default_rng(SEED + 7)
    al, ar = rng.uniform(-1, 1, 3), rng.uniform(-1, 1, 3)
    al[1] = abs(al[1]) + 0.5
    ar[1] = abs(ar[1]) + 0.5
    s = (n, n)
    q = {k: deo.MultiDimDirectionalBC(deo.GeneralBC(al, ar, dx, 1), k, s) for k in (1, 2)}
    ops = [deo.CenteredDifference(1, 6, dx, n, axis=1) * q[1], deo.CenteredDifference(1, 6, dx, n, axis=2) * q[2],
           deo.CenteredDifference(2, 6, dx, n, axis=1) * q[1], deo.CenteredDifference(2, 6, dx, n, axis=2) * q[2]]
    if field_dev is not None:
        ops.append(deo.with_field(deo.UpwindDifference(1, 3, dx, n, axis=1), field_dev) * q[1])
    return ops, (al, ar, dx)


def nonuniform2d_inputs(n, dx):
    """The coefficient field a(x, y) = cos(2 pi x) sin(2 pi y) on the grid's
    nodes and u ~ N(0, 1) smoothed by 5 Jacobi passes (seeded), Julia layout."""
    x = np.cumsum(dx)[:n]  # the grid's nodes
    a = np.asfortranarray(np.cos(2 * np.pi * x[:, None]) * np.sin(2 * np.pi * x[None, :]))
    rng = np.random.default_rng(SEED + 3)
    u = rng.standard_normal((n, n))
    for _ in range(5):  # Jacobi smoothing
        u[1:-1, 1:-1] = 0.25 * (u[:-2, 1:-1] + u[2:, 1:-1] + u[1:-1, :-2] + u[1:-1, 2:])
    return np.asfortranarray(u), a


def run_nonuniform2d(args):
    """2048^2 non-uniform grid: centred d1/d2 a6 on both axes + upwind d1 a3
    with the field a(x,y) = cos(2 pi x) sin(2 pi y), GeneralBC; per op and fused."""
    import torch

    import deo
    n = 2048
    ops, (_, _, dx) = nonuniform2d_ops(n)
    u, a = nonuniform2d_inputs(n, dx)
    fdev = deo.julia_array((n, n)); fdev.copy_(torch.from_numpy(a))
    ops, _ = nonuniform2d_ops(n, fdev)
    ud = deo.julia_array((n, n)); ud.copy_(torch.from_numpy(u))
    outs = [deo.julia_array((n, n)) for _ in range(2)]
    res = {"metric": "grid-pts/s (2-D 2048^2 non-uniform)", "workload": "nonuniform2d_2048_f64", "dtype": "f64",
           "per_op": {}}
    names = ["D1x", "D1y", "D2x", "D2y", "Upwind1x_field"]
    hbm, _ = peaks()
    for nm, g in zip(names, ops):
        p = deo.plan_for([g], (n, n), 0)
        t = _event_time(lambda: p.apply(ud, outs[0]), args.steps, args.warmup)
        b = (24 if g.field is not None else 16) * n * n
        res["per_op"][nm] = {"grid_pts_per_s": n * n / t, "ms": t * 1e3, "GBps": b / t / 1e9, "frac_hbm": b / t / 1e9 / hbm}
    p = deo.plan_for(ops, (n, n), 0)
    t = _event_time(lambda: p.apply(ud, outs[1]), args.steps, args.warmup)
    res["value"] = n * n / t
    res["unit"] = "grid-pts/s"
    res["fused_ms"] = t * 1e3
    res["fused_GBps"] = 24 * n * n / t / 1e9
    res["fused_frac_hbm"] = res["fused_GBps"] / hbm
    # DEO_PLAN_MERGE_TERMS: D1x + D2x and D1y + D2y each evaluated as one term (5 terms -> 3)
    pm = deo.plan_for(ops, (n, n), 0, merge_terms=True)
    om = deo.julia_array((n, n))
    tm = _event_time(lambda: pm.apply(ud, om), args.steps, args.warmup)
    torch.cuda.synchronize()
    res["fused_merged_ms"] = tm * 1e3
    res["fused_merged_terms"] = pm.evaluated_terms
    res["fused_merged_max_rel_diff"] = float((om - outs[1]).abs().max() / outs[1].abs().max())
    # and DEO_PLAN_FACTOR_FIELD: the upwind term as a(x, y) * (sum of its taps), one multiply per point
    pf = deo.plan_for(ops, (n, n), 0, merge_terms=True, factor_field=True)
    of = deo.julia_array((n, n))
    tf = _event_time(lambda: pf.apply(ud, of), args.steps, args.warmup)
    torch.cuda.synchronize()
    res["fused_merged_factored_ms"] = tf * 1e3
    res["fused_merged_factored_max_rel_diff"] = float((of - outs[1]).abs().max() / outs[1].abs().max())
    return res


def batch_specs(count=4096, seed=SEED, scale=1.0):
    """4096 instance specs (shape, d, a, graded, robin): 70% 1-D (N
    log-uniform [64, 65536]), 30% 2-D (sides log-uniform [32, 1024]); d in
    1..4, a in {2,4,6,8}; uniform or graded grid 50/50; Dirichlet or Robin."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        d, a = int(rng.integers(1, 5)), int(rng.choice([2, 4, 6, 8]))
        graded = rng.random() < 0.5
        robin = rng.random() < 0.5
        if rng.random() < 0.7:
            shape = (max(16, int(np.exp(rng.uniform(np.log(64), np.log(65536))) * scale)),)
        else:
            shape = tuple(max(16, int(np.exp(rng.uniform(np.log(32), np.log(1024))) * scale)) for _ in range(2))
        out.append((shape, d, a, graded, robin))
    return out


def batch_grid(n, graded):
    """dx of one axis: uniform 1/(n+1), or graded h(1 + 0.5 sin(2 pi i/(n+1))) normalised to 1."""
    if not graded:
        return 1.0 / (n + 1)
    i = np.arange(n + 1)
    dx = 1.0 + 0.5 * np.sin(2 * np.pi * i / (n + 1))
    return dx / dx.sum()


ROBIN_L, ROBIN_R, DIRICHLET_LR = (1.0, 0.5, 0.1), (1.0, 0.5, -0.1), (0.1, -0.2)


def batch_terms(spec):
    """The terms (L * Q per axis) of one instance spec."""
    import deo
    shape, d, a, graded, robin = spec
    terms = []
    for ax, n in enumerate(shape):
        dx = batch_grid(n, graded)
        bc = deo.RobinBC(ROBIN_L, ROBIN_R, dx, 1) if robin else deo.DirichletBC(*DIRICHLET_LR)
        L = deo.CenteredDifference(d, a, dx, n, axis=ax + 1)
        terms.append(L * (bc if len(shape) == 1 else deo.MultiDimDirectionalBC(bc, ax + 1, shape)))
    return terms


def batch_instances(count=4096, seed=SEED, scale=1.0):
    """(shape, terms) of the batched workload's instances (batch_specs)."""
    return [(spec[0], batch_terms(spec)) for spec in batch_specs(count, seed, scale)]


def run_batch(args, ws=1, rank=0):
    """Config 4.  Under torchrun each rank takes its share of the instances
    (shard, balanced by points) and runs the same batched passes on them;
    the times are the max over ranks and the solves/s count every rank's."""
    import torch

    import deo
    everything = batch_instances(scale=args.size_scale)
    mine = shard([int(np.prod(s)) for s, _ in everything], rank, ws)
    inst = [everything[i] for i in mine]
    plans, us, fw, bw, ones = [], [], [], [], []
    g = torch.Generator(device="cuda")
    total = sum(int(np.prod(s)) for s, _ in everything)
    for i, (shape, terms) in zip(mine, inst):
        p = deo.Plan(terms, shape, 0)
        u = deo.julia_array(shape)
        g.manual_seed(SEED + i)  # an instance's input does not depend on the sharding
        u.copy_(torch.randn(tuple(reversed(shape)), generator=g, device="cuda", dtype=torch.float64).permute(
            *reversed(range(len(shape)))))
        plans.append(p); us.append(u); fw.append(deo.julia_array(shape)); bw.append(deo.julia_array(shape))
        ones.append(deo.julia_array(shape))
    if args.batch_config:  # fixed tile / CTAs per SM (e.g. for profiling), no autotuning
        tile, ctas = (int(v) for v in args.batch_config.split(","))
        bf = deo.Batch(list(zip(plans, us, fw)), tile=tile, ctas_per_sm=ctas)
        ba = deo.Batch(list(zip(plans, fw, bw)), adjoint=True, tile=tile, ctas_per_sm=ctas)
        cfg_f, cfg_a = bf.config, ba.config
    else:
        bf = deo.Batch(list(zip(plans, us, fw)))
        ba = deo.Batch(list(zip(plans, fw, bw)), adjoint=True)
        cfg_f = bf.autotune(os.path.join(REPORT_DIR, "autotune.cache") if REPORT_DIR else None)
        cfg_a = ba.autotune()

    def batched():
        bf.run(True)
        ba.run(True)

    def one_by_one():
        for p, u, o, b in zip(plans, us, ones, bw):
            p.apply(u, o)
        for p, o, b in zip(plans, ones, bw):
            p.adjoint(o, b)

    bf1 = deo.Batch(list(zip(plans, us, ones)))
    ba1 = deo.Batch(list(zip(plans, ones, bw)), adjoint=True)

    def one_by_one_native():
        bf1.run_one_launch_each()
        ba1.run_one_launch_each()

    def timed(fn, steps, warmup):
        barrier(ws)
        return max_over_ranks(_event_time(fn, steps, warmup), ws)

    t_b = timed(batched, max(3, args.steps // 50), 2)
    t_1 = timed(one_by_one, max(2, args.steps // 200), 1)
    t_n = timed(one_by_one_native, max(2, args.steps // 100), 1)
    # the plain per-instance apply: the generic row-table kernel, one launch per instance
    for p in plans:
        p.set_option(deo.DEO_OPT_FAST_PATH, 0)
    t_p = timed(one_by_one_native, max(2, args.steps // 100), 1)
    for p in plans:
        p.set_option(deo.DEO_OPT_FAST_PATH, 1)
    # results agree bit for bit
    torch.cuda.synchronize()
    same = max([0.0] + [float(((a - b).abs().max() / b.abs().max().clamp_min(1e-300))) for a, b in zip(fw, ones)])
    same = max(gather_objects(same, ws))
    hbm, _ = peaks()
    byts = 2 * 16 * total
    return {"metric": "solves/s (4096 batched forward+adjoint applies)", "workload": "batched_4096_mixed_f64",
            "value": len(everything) / t_b, "unit": "solves/s", "dtype": "f64", "total_points": total,
            "n_gpus": ws, "scaling": "strong", "instances_per_rank": gather_objects(len(inst), ws),
            "ms_per_pass": t_b * 1e3,
            "one_launch_per_instance_plain_ms": t_p * 1e3,
            "speedup_vs_one_launch_per_instance_plain": t_p / t_b,
            "one_launch_per_instance_native_ms": t_n * 1e3,
            "speedup_vs_one_launch_per_instance_native": t_n / t_b,
            "one_launch_per_instance_python_ms": t_1 * 1e3,
            "speedup_vs_one_launch_per_instance_python": t_1 / t_b,
            "GBps": byts / t_b / 1e9, "frac_hbm": byts / t_b / 1e9 / hbm, "max_rel_diff_batched_vs_individual": same,
            "autotune_forward": cfg_f, "autotune_adjoint": cfg_a, "gpu_launches_per_pass": 2}


def _serve_cost(r):
    return r.npts * r.K * (2 if r.want_grad else 1)


def run_nld(args):
    """nonlinear_diffusion!(du, 2, 1, 4, p, q, h, N) on N = 2^24 points (Float64):
    six operator applications (orders 1-3 on q and 1-2 on p) and the products,
    one fused kernel."""
    import torch

    import deo
    N = 1 << 24
    h = 1.0 / (N + 1)
    g = torch.Generator(device="cuda").manual_seed(SEED)
    x = torch.linspace(0, 1, N + 2, device="cuda", dtype=torch.float64)
    q = torch.sin(6.283185307179586 * x) + 1e-3 * torch.randn(N + 2, generator=g, device="cuda", dtype=torch.float64)
    p = 1.0 + 0.5 * torch.cos(6.283185307179586 * x)
    du = torch.empty(N, device="cuda", dtype=torch.float64)
    t = _event_time(lambda: deo.nonlinear_diffusion_(du, 2, 1, 4, p, q, h, N), args.steps, args.warmup)
    hbm, _ = peaks()
    byts = 3 * 8 * N
    return {"metric": "grid-pts/s (nonlinear_diffusion!, n=2, m=1, a=4)", "workload": "nonlinear_diffusion_2^24_f64",
            "value": N / t, "unit": "grid-pts/s", "dtype": "f64", "us_per_apply": t * 1e6,
            "GBps": byts / t / 1e9, "frac_hbm": byts / t / 1e9 / hbm, "gpu_launches_per_apply": 1}


def run_serve(args, ws=1, rank=0):
    """Poisson arrivals (2000 req/s) of MOL advection-diffusion solves served
    by the native loop (deo_serve_*): solves/s, p50/p99 latency; against the
    same requests solved one at a time with one plain apply launch per stage
    (deo.serve.solve_one_launch_per_instance), the baseline the task names.
    Under torchrun each rank serves its share of the requests (shard,
    balanced by point-steps) with its own server; the makespan is the max
    over ranks and the latencies are pooled."""
    import torch

    import deo
    from deo.serve import Server, poisson_requests, solve_one_launch_per_instance
    everything = poisson_requests(args.requests, 2000.0, seed=SEED, size_scale=args.size_scale,
                                  k_range=(10, args.kmax))
    reqs = [everything[i] for i in shard([_serve_cost(r) for r in everything], rank, ws)]
    srv = Server(hbm_budget_bytes=120e9)
    barrier(ws)
    st = srv.run(reqs)
    lat = [x for part in gather_objects([r.latency for r in reqs if not r.rejected], ws) for x in part]
    makespan = max_over_ranks(st["makespan_s"], ws)
    completed = sum(gather_objects(st["completed"], ws))
    work = sum(_serve_cost(r) for r in everything)
    out = {"metric": "served solves/s (Poisson 2000 req/s, SSP-RK3 MOL)", "workload": "serve_mol_f64",
           "value": completed / makespan, "unit": "solves/s", "dtype": "f64",
           "p50_s": float(np.percentile(lat, 50)) if lat else None,
           "p99_s": float(np.percentile(lat, 99)) if lat else None, "requests": len(everything),
           "completed": completed, "makespan_s": makespan, "point_steps": work, "steps": st["ticks"],
           "rounds": st["rounds"], "launches": st["launches"], "rebuilds": st["rebuilds"],
           "device_busy_s": st["device_s"], "size_scale": args.size_scale, "kmax": args.kmax,
           "n_gpus": ws, "scaling": "strong"}
    if args.serve_baseline:
        reqs2 = poisson_requests(args.requests, 2000.0, seed=SEED, size_scale=args.size_scale,
                                 k_range=(10, args.kmax))
        reqs2 = [reqs2[i] for i in shard([_serve_cost(r) for r in reqs2], rank, ws)]
        barrier(ws)
        base = solve_one_launch_per_instance(reqs2)
        base["makespan_s"] = max_over_ranks(base["makespan_s"], ws)
        base["solves_per_s"] = len(everything) / base["makespan_s"]
        # the baseline rounds each stage's combination separately (torch
        # elementwise ops) where the server fuses it into the apply: compare
        # to the state's scale, not bitwise
        dev = 0.0
        for a, b in zip(sorted(reqs, key=lambda r: r.rid), sorted(reqs2, key=lambda r: r.rid)):
            if a.uT is not None and b.uT is not None:
                dev = max(dev, float(np.abs(a.uT - b.uT).max() / max(1e-300, np.abs(b.uT).max())))
        out["one_launch_per_instance"] = base
        out["speedup_vs_one_launch_per_instance"] = out["value"] / base["solves_per_s"]
        out["max_rel_diff_vs_baseline"] = max(gather_objects(dev, ws))
    return out


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    n = args.n
    u = fourier_field(n, seed=SEED)
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    for _ in range(args.warmup):
        cpu_oracle_lap3d(u, n, nthreads, 1)
    times = []
    for _ in range(args.steps):
        times.append(cpu_oracle_lap3d(u, n, nthreads, 1))
    t = float(np.mean(times))
    value = n ** 3 / t
    return {
        "impl": "reference",
        "metric": "grid-pts/s (3-D 256^3 Laplacian apply)",
        "value": value,
        "unit": "grid-pts/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded Fourier field + noise)",
        "config": {"workload": f"laplacian3d_{n}^3_f64_d2a4_robin_all_faces", "grid": [n, n, n]},
        "cpu_baseline": {"value": value, "unit": "grid-pts/s", "cores": nthreads, "kind": "port",
                         "sample": f"full {n}^3 apply per step, OpenMP over lines; the reference is Julia, "
                                   f"which is not installed, so its loops run as the C++ restatement"},
        "e2e": {"value": value, "unit": "grid-pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t0,
    }


def run_vector(args):
    """Gradient, Divergence and Curl (4th order, uniform grid) of 256^3 padded
    arrays, Float64 and Float32: device time per apply, grid points/s, the
    algorithmic bytes (padded input components once, output components once)
    against the measured HBM copy rate, and for Float64 the FP64 instructions
    per point (NK fused multiply-adds per derivative, the adds between terms)
    against the FP64 issue rate measured on this part (1.68 per clock per SM).
    cpu_baseline: the oracle (one thread) on a 64^3 sample of the same operator."""
    import time

    import torch

    import deo
    n = args.n
    hbm, _ = peaks()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    fp64_rate = 1.68 * sms * 2.07e9  # FP64 instructions/s at the maximum SM clock
    lines = []
    for kind, ctor, cin, cout, fp64 in (("gradient", deo.Gradient, 1, 3, 15), ("divergence", deo.Divergence, 3, 1, 17),
                                        ("curl", deo.Curl, 3, 3, 33)):
        for dt, es, name in ((torch.float64, 8, "f64"), (torch.float32, 4, "f32")):
            A = ctor(4, (1.0 / (n + 1),) * 3, (n, n, n))
            M = deo.julia_array(A.in_shape(), dt)
            M.normal_(generator=torch.Generator(device="cuda").manual_seed(SEED))
            out = deo.julia_array(A.out_shape(), dt)
            t = _event_time(lambda: A.mul_(out, M, overwrite=True), args.steps, max(args.warmup, 3))
            byts = es * ((n + 2) ** 3 * cin + n ** 3 * cout)
            rec = {"op": kind, "dtype": name, "us_per_apply": t * 1e6, "grid_pts_per_s": n ** 3 / t,
                   "GBps": byts / t / 1e9, "frac_hbm": byts / t / 1e9 / hbm}
            if name == "f64":
                rec["fp64_instr_per_pt"] = fp64
                rec["frac_fp64_issue"] = fp64 * n ** 3 / t / fp64_rate
            lines.append(rec)
    cpu = None
    if not args.no_cpu:
        import numpy as np
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        m = 64
        ops = [O.centered(1, 4, 1.0 / (m + 1), m, axis=a + 1) for a in range(3)]
        Mh = np.asfortranarray(np.random.default_rng(SEED).standard_normal((m + 2,) * 3))
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < 10.0:
            O.vector_calculus(O.GRADIENT, ops, Mh)
            reps += 1
        cpu = {"value": reps * m ** 3 / (time.perf_counter() - t0), "unit": "grid-pts/s", "cores": 1, "kind": "port",
               "sample": f"oracle Gradient on 64^3 Float64, {reps} applies in ~10 s"}
    return {"metric": "grid-pts/s (Gradient 256^3 f64, 4th order)", "workload": f"vector_calculus_{n}^3",
            "value": lines[0]["grid_pts_per_s"], "unit": "grid-pts/s", "dtype": "f64", "applies": lines,
            "cpu_baseline": cpu, "gpu_launches_per_apply": 1}


def run_solve(args):
    """A \\ u (ghost_derivative_operator.jl:39-58) on a 256^3 Float64 array along
    axis 3: CenteredDifference(2, a, h, 256) with RobinBC on that axis, a = 2
    (tridiagonal A_l) and a = 4 (4 sub- and super-diagonals after pivoting).
    Device time per solve (factors built once, in the plan), grid points/s, the
    algorithmic bytes (u read and x written once: 16 B/pt) and the bytes moved
    (the forward sweep's intermediate written and read back: 32 B/pt).
    cpu_baseline: LAPACK's banded solver (scipy.linalg.solve_banded, one thread)
    on a 4096-line sample of the same system."""
    import time

    import torch

    import deo
    n = args.n
    h = 1.0 / (n + 1)
    hbm, _ = peaks()
    out = []
    u = deo.julia_array((n, n, n), torch.float64)
    u.normal_(generator=torch.Generator(device="cuda").manual_seed(SEED))
    x = deo.julia_array((n, n, n), torch.float64)
    for a in (2, 4):
        L = deo.CenteredDifference(2, a, h, n, axis=3)
        A = L * deo.MultiDimBC(deo.RobinBC((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), h, a), (n, n, n), 3)
        bands = deo.solve_plan_for(A, (n, n, n), 0).bands()
        t = _event_time(lambda: deo.ldiv_(x, A, u), args.steps, max(args.warmup, 3))
        out.append({"approx_order": a, "bands": list(bands), "us_per_solve": t * 1e6, "grid_pts_per_s": n ** 3 / t,
                    "GBps_algorithmic": 16 * n ** 3 / t / 1e9, "frac_hbm": 16 * n ** 3 / t / 1e9 / hbm,
                    "GBps_moved": 32 * n ** 3 / t / 1e9})
    cpu = None
    if not args.no_cpu:
        import scipy.linalg as sl
        L = deo.CenteredDifference(2, 2, h, n)
        Al, Ab = (L * deo.RobinBC((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), h, 2)).array()
        kl = ku = 1
        band = np.zeros((kl + ku + 1, n))
        for i in range(n):
            for j in range(max(0, i - kl), min(n, i + ku + 1)):
                band[ku + i - j, j] = Al[i, j]
        rhs = np.random.default_rng(SEED).standard_normal((n, 4096)) - Ab[:, None]
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < 10.0:
            for c in range(0, 4096, 64):
                sl.solve_banded((kl, ku), band, rhs[:, c:c + 64], check_finite=False)
            reps += 1
        cpu = {"value": reps * 4096 * n / (time.perf_counter() - t0), "unit": "grid-pts/s", "cores": 1,
               "kind": "port", "sample": f"scipy.linalg.solve_banded (LAPACK gbsv), 4096 lines of {n}, {reps} passes"}
    return {"metric": "grid-pts/s (A \\ u, 256^3 f64 along axis 3, tridiagonal)", "workload": f"ghost_solve_{n}^3_f64",
            "value": out[0]["grid_pts_per_s"], "unit": "grid-pts/s", "dtype": "f64", "solves": out,
            "cpu_baseline": cpu, "gpu_launches_per_solve": 1}


def run_adjoint(args):
    """The transposed apply (deo_apply_adjoint, the rrule's pullback) of the
    256^3 Float64 Robin Laplacian, rotating buffers larger than L2."""
    import torch

    import deo
    n = args.n
    AQ, plan, tdt = lap3d_setup(n, "f64")
    g = torch.Generator(device="cuda").manual_seed(SEED)
    pairs = []
    for _ in range(3):
        v = deo.julia_array((n, n, n), tdt)
        v.copy_(torch.randn((n, n, n), generator=g, device="cuda", dtype=tdt))
        pairs.append((v, deo.julia_array((n, n, n), tdt)))
    k = [0]

    def step():
        v, ub = pairs[k[0] % 3]
        k[0] += 1
        plan.adjoint(v, ub)
    t = _event_time(step, args.steps, args.warmup)
    kernels = list(plan.kernels)
    plan.set_option(deo.DEO_OPT_FAST_PATH, 0)
    t_gen = _event_time(step, max(3, args.steps // 3), 2)
    plan.set_option(deo.DEO_OPT_FAST_PATH, 1)
    hbm, _ = peaks()
    return {"metric": "grid-pts/s (adjoint of the 256^3 Laplacian apply)", "workload": "adjoint_lap3d_256_f64",
            "value": n ** 3 / t, "unit": "grid-pts/s", "dtype": "f64", "ms": t * 1e3,
            "ms_generic_kernel": t_gen * 1e3,
            "GBps": 16 * n ** 3 / t / 1e9, "frac_hbm": 16 * n ** 3 / t / 1e9 / hbm, "kernels": kernels}


def run_secondary(args):
    """The other benchmark configurations, run after the headline and attached
    to its line (each bounded to a few seconds of timed work):
    the 256^3 Laplacian in Float32, the 1-D N=1024 apply (latency), the 2-D
    2048^2 non-uniform operators (per operator and fused), the 4096-instance
    batched pass against one launch per instance, and the served solves."""
    import copy
    import time
    out = {}

    def sub(name, fn, **over):
        a = copy.copy(args)
        for k, v in over.items():
            setattr(a, k, v)
        t0 = time.perf_counter()
        try:
            r = fn(a)
            r["wall_s"] = time.perf_counter() - t0
            out[name] = r
        except Exception as e:  # a failing sub-workload is reported, not fatal to the headline line
            out[name] = {"error": f"{type(e).__name__}: {e}"}

    sub("lap3d_f32", lambda a: run_ours(a, 1, 0), workload="lap3d_f32", steps=300, warmup=10, no_cpu=True)
    sub("line1d", run_line1d, steps=2000, warmup=50)
    sub("adjoint", run_adjoint, steps=30, warmup=3)
    sub("nonuniform2d", run_nonuniform2d, steps=50, warmup=5)
    sub("batch", run_batch, steps=150, warmup=3, size_scale=1.0, batch_config="")
    sub("serve", run_serve, requests=args.requests, size_scale=args.size_scale, kmax=args.kmax,
        serve_baseline=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="lap3d",
                    choices=["lap3d", "lap3d_f32", "line1d", "nonuniform2d", "batch", "serve", "nld", "vector", "solve",
                             "adjoint"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--size-scale", type=float, default=1.0)
    ap.add_argument("--kmax", type=int, default=1000)
    ap.add_argument("--serve-baseline", action="store_true")
    ap.add_argument("--batch-config", default="", help="tile,ctas_per_sm for the batch workload (skips autotuning)")
    ap.add_argument("--no-secondary", action="store_true", help="the headline line only")
    ap.add_argument("--exact-sums", type=int, default=-1,
                    help="plan option DEO_OPT_EXACT_SUMS for the 3-D workload (default: the library's)")
    ap.add_argument("--serial-shell", action="store_true", help="the boundary shell after the interior kernel")
    ap.add_argument("--no-autotune", action="store_true", help="the plan's default execution choices")
    ap.add_argument("--f32-scalar", action="store_true",
                    help="Float32: the one-column-per-thread interior (DEO_OPT_F32_VECTOR=0), no autotuning")
    args = ap.parse_args()
    if args.workload in ("batch", "serve"):
        ws, rank, _ = dist_init()
        line = (run_batch if args.workload == "batch" else run_serve)(args, ws, rank)
        if rank == 0:
            print(json.dumps(line), flush=True)
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.workload in ("line1d", "nonuniform2d", "nld", "vector", "solve", "adjoint"):
        import torch
        torch.cuda.set_device(0)
        fn = {"line1d": run_line1d, "nonuniform2d": run_nonuniform2d, "nld": run_nld, "vector": run_vector,
              "solve": run_solve, "adjoint": run_adjoint}[args.workload]
        print(json.dumps(fn(args)), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        ws = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        line = run_reference(args, ws, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    ws, rank, _ = dist_init()
    line = run_ours(args, ws, rank)
    if rank == 0 and not args.no_secondary and args.workload == "lap3d":
        line["secondary"] = run_secondary(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
