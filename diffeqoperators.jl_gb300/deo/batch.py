"""Batched applies and batched Runge-Kutta stages (one persistent launch each).

A Batch holds many independent (plan, u, du) instances -- different shapes,
operators and boundary conditions -- and runs them as ONE launch of a
persistent kernel that pulls fixed-size tiles from a work-list, optionally
replayed from a captured CUDA graph.  Tile size and CTAs per SM come from the
autotuner (cached per workload signature).  No reference counterpart: the
reference applies one operator per call.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

from . import _lib as L
from ._lib import Instance, Stage, check
from .operators import Plan, _stream_ptr


class Batch:
    def __init__(self, instances: Sequence[tuple], adjoint: bool = False, tile: int = 0, ctas_per_sm: int = 0):
        """instances: (Plan, u, du) with u/du device tensors in the plan's layout."""
        n = len(instances)
        arr = (Instance * max(n, 1))()
        self._keep = []
        for i, (p, u, du) in enumerate(instances):
            if not isinstance(p, Plan):
                raise TypeError("instances need a deo.Plan")
            p._check(u, du)
            arr[i].plan = p.handle
            arr[i].u = C.c_void_p(u.data_ptr())
            arr[i].du = C.c_void_p(du.data_ptr())
            self._keep.append((p, u, du))
        h = C.c_void_p()
        check(L.lib().deo_batch_create(n, arr, int(bool(adjoint)), int(tile), int(ctas_per_sm), C.byref(h)))
        self._h = h
        self.adjoint = adjoint
        self._arr, self._n = arr, n

    def run_one_launch_each(self, stream=None):
        """The same instances with one launch per instance (native host loop)."""
        check(L.lib().deo_apply_each(self._n, self._arr, int(bool(self.adjoint)),
                                     stream if stream is not None else _stream_ptr()))

    def __del__(self):
        try:
            if self._h:
                L.lib().deo_batch_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def run(self, use_graph: bool = True, stream=None):
        check(L.lib().deo_batch_run(self._h, int(bool(use_graph)), stream if stream is not None else _stream_ptr()))

    def autotune(self, cache_path: str | None = None, stream=None):
        check(L.lib().deo_batch_autotune(self._h, cache_path.encode() if cache_path else None,
                                         stream if stream is not None else _stream_ptr()))
        return self.config

    @property
    def config(self):
        t, c, n = C.c_int(), C.c_int(), C.c_int64()
        check(L.lib().deo_batch_config(self._h, C.byref(t), C.byref(c), C.byref(n)))
        return {"tile": t.value, "ctas_per_sm": c.value, "work_items": n.value}


class StageBatch(Batch):
    """One Runge-Kutta stage for many instances:
    out = alpha*a + beta*b + gamma*(c + dt*Op(c)), Op = plan or its adjoint."""

    def __init__(self, stages: Sequence[dict], tile: int = 0, ctas_per_sm: int = 0):
        n = len(stages)
        arr = (Stage * max(n, 1))()
        self._keep = []
        for i, s in enumerate(stages):
            p = s["plan"]
            arr[i].plan = p.handle
            for k in ("a", "b", "c", "out"):
                t = s.get(k)
                setattr(arr[i], k, C.c_void_p(t.data_ptr()) if t is not None else None)
            arr[i].alpha = float(s.get("alpha", 0.0))
            arr[i].beta = float(s.get("beta", 0.0))
            arr[i].gamma = float(s.get("gamma", 1.0))
            arr[i].dt = float(s["dt"])
            arr[i].adjoint = int(bool(s.get("adjoint", False)))
            self._keep.append(s)
        h = C.c_void_p()
        check(L.lib().deo_stage_batch_create(n, arr, int(tile), int(ctas_per_sm), C.byref(h)))
        self._h = h
        self.adjoint = None
