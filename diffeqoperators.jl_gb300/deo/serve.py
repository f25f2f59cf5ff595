"""Continuous-batching server for method-of-lines solves (libdeo's deo_serve_*).

Each request is an advection-diffusion solve
    du/dt = nu * Laplacian(u) - c * du/dx,   Dirichlet0 on every face,
built from the reference's operators (nu * CenteredDifference{k}(2, 2, h, n)
for every axis k, plus UpwindDifference{1}(1, a, h, n, -c)), advanced K
fixed SSP-RK3 steps (dt from CFL 0.4); optionally the gradient of
||u(T)||^2 with respect to u0 is computed by the transposed steps.

The serving loop is native (csrc/deo_serve.cpp): the state of every admitted
request lives in device memory; rounds of several steps that advance every
active request in three batched stage launches per step are enqueued back to
back without waiting for the device; results are copied out asynchronously;
requests that arrive while others run are admitted as memory frees up
(continuous batching) under a device-memory budget.  This module submits the
requests at their arrival times, drives deo_serve_pump and collects results.
Every request's arithmetic is independent of the others (no cross-request
reductions, fixed per-point order), so its result is the same alone or in any
mix.

No reference counterpart: the reference delegates time stepping to
OrdinaryDiffEq and has no serving layer.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import _lib as L
from ._lib import check
from .operators import (CenteredDifference, DiffEqOperatorCombination, Dirichlet0BC, MultiDimDirectionalBC, Plan,
                        UpwindDifference)


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
    t_done: float = float("nan")
    rejected: str = ""

    @property
    def npts(self) -> int:
        return int(np.prod(self.shape))

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival

    def bytes_needed(self, esize: int = 8) -> int:
        """The three state buffers (the server also counts the plan's device
        tables and the request's stage work-list entries)."""
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


class Server:
    def __init__(self, hbm_budget_bytes: float = 120e9, max_steps_per_round: int = 64,
                 inject_alloc_failures: int = 0, merge_terms: bool = True):
        """merge_terms: build each request's plan with DEO_PLAN_MERGE_TERMS
        (the diffusion and advection terms along axis 1 share the boundary
        condition, so they are evaluated as one tap set).  DEO_PLAN_STAR is
        not used: on the served mix it saved no time (3.11 against 3.04 s of
        device time)."""
        self.merge_terms = merge_terms
        h = C.c_void_p()
        check(L.lib().deo_serve_create(int(hbm_budget_bytes), 0, int(max_steps_per_round), C.byref(h)))
        self._h = h
        self.budget = float(hbm_budget_bytes)
        if inject_alloc_failures:
            check(L.lib().deo_serve_inject_alloc_failures(h, int(inject_alloc_failures)))
        self.done: List[Request] = []
        self._out = {}    # native id -> (request, plan, u0 buffer, uT buffer, grad buffer)
        self._native = {}  # id(request) -> native id

    def __del__(self):
        try:
            if self._h:
                L.lib().deo_serve_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def submit(self, req: Request, t0: float) -> bool:
        A = advection_diffusion(req.shape, req.nu, req.c, req.approx_order)
        plan = Plan(A.terms(), req.shape, 0, merge_terms=self.merge_terms)
        u0 = req.initial()
        q = L.Request(plan.handle, C.c_void_p(u0.ctypes.data), int(req.K), float(req.dt()), int(bool(req.want_grad)))
        rid = C.c_int64()
        st = L.lib().deo_serve_submit(self._h, C.byref(q), C.byref(rid))
        if st == 8:  # DEO_ERR_REJECTED
            req.rejected = "larger than the HBM budget"
            req.t_done = time.perf_counter() - t0
            L.lib().deo_serve_poll(self._h, rid.value, None, None, None)  # forget it
            self.done.append(req)
            return False
        check(st)
        uT = np.empty(req.shape, order="F")
        g = np.empty(req.shape, order="F") if req.want_grad else None
        self._out[rid.value] = (req, plan, u0, uT, g)
        self._native[id(req)] = rid.value
        return True

    def cancel(self, req: Request) -> None:
        check(L.lib().deo_serve_cancel(self._h, self._native[id(req)]))

    def _collect(self, t0: float) -> int:
        got = 0
        lib = L.lib()
        for rid in list(self._out):
            req, plan, u0, uT, g = self._out[rid]
            st = lib.deo_serve_poll(self._h, rid, C.c_void_p(uT.ctypes.data),
                                    C.c_void_p(g.ctypes.data) if g is not None else None, None)
            if st == 7:  # DEO_ERR_NOT_READY
                continue
            req.t_done = time.perf_counter() - t0
            if st == 0:
                req.uT, req.grad = uT, g
            elif st == 6:
                req.rejected = "admission failed: device memory for the state could not be allocated"
            elif st == 2:
                req.rejected = "cancelled"
            else:
                check(st)
            self.done.append(req)
            del self._out[rid]
            got += 1
        return got

    def stats(self) -> dict:
        s = L.ServeStats()
        check(L.lib().deo_serve_stats_get(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in L.ServeStats._fields_}

    def run(self, requests: List[Request], realtime: bool = True, timeout_s: float = 600.0, on_tick=None):
        """Serve `requests` (arrival times relative to the start).  on_tick(server,
        elapsed) is called once per loop iteration (tests cancel from it).
        Returns stats."""
        import torch
        lib = L.lib()
        pending = sorted(requests, key=lambda r: r.arrival)
        t0 = time.perf_counter()
        i = 0
        while i < len(pending) or self._out:
            now = time.perf_counter() - t0
            if now > timeout_s:
                raise TimeoutError("serving run exceeded its time limit")
            while i < len(pending) and (pending[i].arrival <= now or not realtime):
                self.submit(pending[i], t0)
                i += 1
            check(lib.deo_serve_pump(self._h))
            if on_tick is not None:
                on_tick(self, now)
            if not self._collect(t0) and i < len(pending) and not self._out and realtime:
                time.sleep(max(0.0, min(pending[i].arrival - now, 0.001)))
        torch.cuda.synchronize()
        makespan = time.perf_counter() - t0
        done = [r for r in self.done if r in requests]
        ok = [r for r in done if not r.rejected]
        lat = np.array([r.latency for r in ok]) if ok else np.array([np.nan])
        st = self.stats()
        return {"requests": len(requests), "completed": len(ok), "rejected": len(done) - len(ok),
                "makespan_s": makespan, "solves_per_s": len(ok) / makespan,
                "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "ticks": st["steps"], "rounds": st["rounds"], "launches": st["launches"],
                "rebuilds": st["rebuilds"], "failed": st["failed"], "cancelled": st["cancelled"],
                "device_s": st["device_us"] * 1e-6}


def solve_one_launch_per_instance(requests: List[Request]) -> dict:
    """The baseline the server is measured against: the same requests, one at a
    time in arrival order, each SSP-RK3 stage one plain apply of the request's
    plan (deo_apply) plus its own combination kernels, a host loop of launches
    per instance; the result of each request is copied to the host when it
    finishes (the gradient requests take their transposed steps the same way).
    Returns makespan and solves/s (arrivals ignored: the queue starts full)."""
    import torch
    from .operators import julia_array
    t0 = time.perf_counter()
    for r in requests:
        A = advection_diffusion(r.shape, r.nu, r.c, r.approx_order)
        p = Plan(A.terms(), r.shape, 0)
        u = julia_array(r.shape)
        u.copy_(torch.from_numpy(r.initial()))
        f = julia_array(r.shape)
        b1, b2 = julia_array(r.shape), julia_array(r.shape)
        dt = r.dt()
        for _ in range(r.K):
            p.apply(u, f)
            torch.add(u, f, alpha=dt, out=b1)
            p.apply(b1, f)
            b2.copy_(0.75 * u + 0.25 * (b1 + dt * f))
            p.apply(b2, f)
            u.copy_(u / 3.0 + (2.0 / 3.0) * (b2 + dt * f))
        r.uT = u.cpu().numpy()
        if r.want_grad:
            u.mul_(2.0)
            for _ in range(r.K):
                p.adjoint(u, f)
                b2.copy_((2.0 / 3.0) * (u + dt * f))
                p.adjoint(b2, f)
                b1.copy_(0.25 * (b2 + dt * f))
                p.adjoint(b1, f)
                u.copy_(u / 3.0 + 0.75 * b2 + (b1 + dt * f))
            r.grad = u.cpu().numpy()
    torch.cuda.synchronize()
    makespan = time.perf_counter() - t0
    return {"makespan_s": makespan, "solves_per_s": len(requests) / makespan}


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
