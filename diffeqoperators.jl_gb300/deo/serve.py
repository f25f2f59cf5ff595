"""Continuous-batching server for method-of-lines solves.

Each request is an advection-diffusion solve
    du/dt = nu * Laplacian(u) - c * du/dx,   Dirichlet0 on every face,
built from the reference's operators (nu * CenteredDifference{k}(2, 2, h, n)
for every axis k, plus UpwindDifference{1}(1, a, h, n, -c)), advanced K
fixed SSP-RK3 steps (dt from CFL 0.4); optionally the gradient of
||u(T)||^2 with respect to u0 is computed by the transposed steps.

The state of every admitted request lives in device memory (three buffers
per request).  Each server tick advances EVERY active request by one step:
three batched stage launches (libdeo's persistent work-list kernel) cover all
requests at once -- forward and adjoint stages mixed -- replayed from a CUDA
graph while the set of active requests is unchanged.  Requests are admitted
FIFO whenever their memory fits under the HBM budget, so work that arrives
while others are on the GPU joins the next tick (continuous batching), and a
finished request frees its slot immediately.  Every request's arithmetic is
independent of the others (no cross-request reductions, fixed per-point
order), so its result is the same alone or in any mix.

No reference counterpart: the reference delegates time stepping to
OrdinaryDiffEq and has no serving layer.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .batch import StageBatch
from .operators import (CenteredDifference, DiffEqOperatorCombination, Dirichlet0BC, MultiDimDirectionalBC, Plan,
                        UpwindDifference, julia_array)


@dataclass
class Request:
    shape: tuple
    nu: float
    c: float
    K: int
    want_grad: bool = False
    u0: Optional[np.ndarray] = None      # host, Fortran order (generated from seed if None)
    seed: int = 0
    arrival: float = 0.0                 # seconds after the run starts
    rid: int = 0
    approx_order: int = 2
    # filled by the server
    uT: Optional[np.ndarray] = None
    grad: Optional[np.ndarray] = None
    t_admit: float = float("nan")
    t_done: float = float("nan")
    rejected: str = ""

    @property
    def npts(self) -> int:
        return int(np.prod(self.shape))

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival

    def bytes_needed(self, esize: int = 8) -> int:
        return 3 * self.npts * esize

    def dt(self) -> float:
        h = 1.0 / (self.shape[0] + 1)
        lim = []
        if self.c != 0:
            lim.append(h / abs(self.c))
        if self.nu > 0:
            lim.append(h * h / (2.0 * self.nu * len(self.shape)))
        return 0.4 * min(lim)

    def initial(self) -> np.ndarray:
        if self.u0 is not None:
            return np.asfortranarray(self.u0, dtype=np.float64)
        rng = np.random.default_rng(self.seed)
        return np.asfortranarray(rng.standard_normal(self.shape))


def advection_diffusion(shape, nu, c, approx_order=2):
    """nu * sum_k D2_k + UpwindDifference{1}(1, a, h, n, -c), Dirichlet0BC on every face."""
    ops = []
    for k, n in enumerate(shape):
        ops.append(nu * CenteredDifference(2, 2, 1.0 / (n + 1), n, axis=k + 1))
    ops.append(UpwindDifference(1, approx_order, 1.0 / (shape[0] + 1), shape[0], -c, axis=1))
    bc = Dirichlet0BC()
    if len(shape) == 1:
        return DiffEqOperatorCombination([P * bc for P in ops])
    return DiffEqOperatorCombination([P * MultiDimDirectionalBC(bc, P.axis, shape) for P in ops])


class _Slot:
    def __init__(self, req: Request, device):
        import torch
        self.req = req
        A = advection_diffusion(req.shape, req.nu, req.c, req.approx_order)
        self.A = A
        self.plan = Plan(A.terms(), req.shape, 0)
        self.u = julia_array(req.shape, torch.float64, device)
        self.u.copy_(torch.from_numpy(req.initial()))
        self.b1 = julia_array(req.shape, torch.float64, device)
        self.b2 = julia_array(req.shape, torch.float64, device)
        self.step = 0
        self.phase = "fwd"          # fwd -> (adj) -> done
        self.dt = req.dt()

    def stages(self):
        """(stage1, stage2, stage3) descriptors for this slot's next step."""
        p, dt = self.plan, self.dt
        if self.phase == "fwd":
            return (dict(plan=p, c=self.u, out=self.b1, gamma=1.0, dt=dt),
                    dict(plan=p, a=self.u, alpha=0.75, c=self.b1, out=self.b2, gamma=0.25, dt=dt),
                    dict(plan=p, a=self.u, alpha=1.0 / 3.0, c=self.b2, out=self.u, gamma=2.0 / 3.0, dt=dt))
        # transposed step on ub = self.u, g1 = b1, g2 = b2
        return (dict(plan=p, c=self.u, out=self.b2, gamma=2.0 / 3.0, dt=dt, adjoint=True),
                dict(plan=p, c=self.b2, out=self.b1, gamma=0.25, dt=dt, adjoint=True),
                dict(plan=p, a=self.u, alpha=1.0 / 3.0, b=self.b2, beta=0.75, c=self.b1, out=self.u, gamma=1.0,
                     dt=dt, adjoint=True))


class Server:
    def __init__(self, hbm_budget_bytes: float = 120e9, use_graph: bool = True, tile: int = 8192,
                 ctas_per_sm: int = 4, device="cuda", max_active: int = 1 << 30):
        self.budget = float(hbm_budget_bytes)
        self.use_graph = use_graph
        self.tile = tile
        self.ctas = ctas_per_sm
        self.device = device
        self.max_active = max_active
        self.queue: List[Request] = []
        self.active: List[_Slot] = []
        self.done: List[Request] = []
        self.in_use = 0.0
        self._batches = None
        self.ticks = 0
        self.rebuilds = 0
        self.launches = 0

    # -- admission ------------------------------------------------------------
    def submit(self, req: Request):
        if req.bytes_needed() > self.budget:
            req.rejected = "larger than the HBM budget"
            self.done.append(req)
            return False
        self.queue.append(req)
        return True

    def _admit(self, now: float):
        changed = False
        while self.queue and len(self.active) < self.max_active:
            r = self.queue[0]
            need = r.bytes_needed()
            if self.in_use + need > self.budget:
                break                      # FIFO: wait for memory to free up
            self.queue.pop(0)
            try:
                slot = _Slot(r, self.device)
            except Exception as e:         # allocation failure is reported, not fatal
                r.rejected = f"admission failed: {e}"
                self.done.append(r)
                continue
            r.t_admit = now
            self.in_use += need
            self.active.append(slot)
            changed = True
        return changed

    def _rebuild(self):
        sets = [s.stages() for s in self.active]
        self._batches = [StageBatch([st[k] for st in sets], tile=self.tile, ctas_per_sm=self.ctas) for k in range(3)]
        self.rebuilds += 1

    # -- one tick: one SSP-RK3 step (forward or transposed) for every active slot
    def tick(self):
        import torch
        for b in self._batches:
            b.run(self.use_graph)
        self.launches += 3
        self.ticks += 1
        torch.cuda.current_stream().synchronize()
        changed = False
        keep = []
        for s in self.active:
            s.step += 1
            if s.phase == "fwd" and s.step == s.req.K:
                s.req.uT = s.u.cpu().numpy()
                if s.req.want_grad:
                    s.u.mul_(2.0)          # ubar(T) = 2 u(T)
                    s.phase, s.step = "adj", 0
                    changed = True
                else:
                    s.phase = "done"
            elif s.phase == "adj" and s.step == s.req.K:
                s.req.grad = s.u.cpu().numpy()
                s.phase = "done"
            if s.phase == "done":
                changed = True
                self.in_use -= s.req.bytes_needed()
                self._finished.append(s.req)
            else:
                keep.append(s)
        self.active = keep
        return changed

    def run(self, requests: List[Request], realtime: bool = True, timeout_s: float = 600.0):
        """Serve `requests` (arrival times relative to the start).  Returns stats."""
        import torch
        pending = sorted(requests, key=lambda r: r.arrival)
        t0 = time.perf_counter()
        self._finished = []
        i = 0
        while (i < len(pending) or self.queue or self.active):
            now = time.perf_counter() - t0
            if now > timeout_s:
                raise TimeoutError("serving run exceeded its time limit")
            while i < len(pending) and (pending[i].arrival <= now or not realtime):
                self.submit(pending[i])
                i += 1
            changed = self._admit(now)
            if not self.active:
                if i < len(pending) and realtime:
                    time.sleep(max(0.0, min(pending[i].arrival - now, 0.001)))
                continue
            if changed or self._batches is None:
                self._rebuild()
            self._finished = []
            if self.tick():
                self._batches = None
            t = time.perf_counter() - t0
            for r in self._finished:
                r.t_done = t
                self.done.append(r)
        torch.cuda.synchronize()
        makespan = time.perf_counter() - t0
        ok = [r for r in self.done if not r.rejected]
        lat = np.array([r.latency for r in ok]) if ok else np.array([np.nan])
        return {"requests": len(requests), "completed": len(ok), "rejected": len(self.done) - len(ok),
                "makespan_s": makespan, "solves_per_s": len(ok) / makespan,
                "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "ticks": self.ticks, "launches": self.launches, "rebuilds": self.rebuilds}


def poisson_requests(n: int, rate: float, seed: int = 0, grad_frac: float = 0.2, size_scale: float = 1.0,
                     k_range=(10, 1000)) -> List[Request]:
    """Synthetic request stream: Poisson arrivals at `rate` req/s; sizes
    log-uniform per dimension class (1-D N in [1e3, 1e6], 2-D sides in
    [64, 2048], 3-D sides in [32, 256], each scaled by `size_scale`), nu in
    U(1e-3, 1e-1), c in U(-1, 1), K in U[k_range], 20% with a gradient."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        dim = int(rng.integers(1, 4))
        if dim == 1:
            lo, hi = 1e3, 1e6
        elif dim == 2:
            lo, hi = 64, 2048
        else:
            lo, hi = 32, 256
        lo, hi = max(8, lo * size_scale), max(9, hi * size_scale)
        side = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        shape = (side,) * dim
        out.append(Request(shape=shape, nu=float(rng.uniform(1e-3, 1e-1)), c=float(rng.uniform(-1, 1)),
                           K=int(rng.integers(k_range[0], k_range[1] + 1)), want_grad=bool(rng.random() < grad_frac),
                           seed=int(rng.integers(1 << 31)), arrival=t, rid=i))
    return out
