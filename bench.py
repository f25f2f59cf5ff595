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
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
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
        self.path = os.path.join(ROOT, "gpurun_out" if os.path.isdir(os.path.join(ROOT, "gpurun_out")) else "",
                                 f".clocks_{os.getpid()}.csv")

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


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


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
    barrier(ws)
    t0 = time.perf_counter()
    e2e_steps = max(3, min(args.steps, 20))
    for _ in range(e2e_steps):
        deo._lib.check(lib.deo_apply_host(plan.handle, C.c_void_p(uh.data_ptr()), C.c_void_p(dh.data_ptr()), st))
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s = max_over_ranks(e2e_s, ws)
    # check the e2e output against the device path once (same kernel)
    dev_out = dus[(args.steps - 1) % nbuf].permute(2, 1, 0).contiguous().view(-1).cpu()
    if not torch.equal(dev_out, dh):
        raise RuntimeError("host-buffer path disagrees with the device path")

    hbm, peak_kind = peaks()
    alg_bytes = 2 * esize * npts
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
    traffic = profiled_traffic(f"k_apply_lap3d_{n}_{dtype_name}")
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
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "e2e": {"value": ws * npts / e2e_s, "unit": "grid-pts/s", "h2d_bytes_per_step": npts * esize,
                "d2h_bytes_per_step": npts * esize, "path": "deo_apply_host (C ABI, pinned host buffers)"},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_launch": alg_bytes,
                     "traffic": traffic},
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu:
        reps = 1
        t_cpu = cpu_oracle_lap3d(np.asarray(u_host, dtype=np.float64), n, 1, reps)
        line["cpu_baseline"] = {"value": npts / t_cpu, "unit": "grid-pts/s", "cores": 1, "kind": "port",
                                "sample": f"one full {n}^3 apply, {reps} timed rep(s), 1 thread, C++ restatement "
                                          f"of the reference loops (oracle/deo_oracle.cpp)"}
    return line


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="lap3d", choices=["lap3d", "lap3d_f32"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
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
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
