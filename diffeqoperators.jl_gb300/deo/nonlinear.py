"""nonlinear_diffusion / nonlinear_diffusion! on the GPU (derivative_operator.jl:34-77).

    du = (D_m q) .* (D_n p)          (q[2:nknots+1] .* (D_n p) when m == 0)
       + sum_{l=1}^{n-1} binomial(n, l) * (D_{l+m} q) .* (D_{n-l} p)
       + (D_{m+n} q) .* p[2:nknots+1]

with D_k = CenteredDifference(k, approx_order, dx, nknots) applied to the padded
vectors p, q (nknots + 2 entries) by the generic method, in the reference's
operation order; one fused kernel over the points.  The operators and their
tables are planned once per (orders, approx_order, dx, nknots, dtype).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import check
from .operators import _stream_ptr

_dp = C.POINTER(C.c_double)
_cache: dict = {}


class NonlinearDiffusionPlan:
    def __init__(self, second_order: int, first_order: int, approx_order: int, dx, nknots: int, dtype_code: int = 0):
        d = np.ascontiguousarray(np.atleast_1d(np.asarray(dx, dtype=np.float64)))
        h = C.c_void_p()
        check(L.lib().deo_nonlinear_diffusion_plan(int(second_order), int(first_order), int(approx_order),
                                                   d.ctypes.data_as(_dp), int(d.size), int(nknots), int(dtype_code),
                                                   C.byref(h)))
        self._h = h
        self.nknots = int(nknots)
        self.dtype_code = int(dtype_code)

    def __del__(self):
        try:
            if self._h:
                L.lib().deo_nonlinear_diffusion_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def apply(self, du, p, q):
        n = self.nknots
        for name, t, want in (("p", p, n + 2), ("q", q, n + 2), ("du", du, n)):
            if t.dim() != 1 or t.shape[0] != want or not t.is_cuda or not t.is_contiguous():
                raise ValueError(f"{name}: a contiguous CUDA vector of {want} entries is required")
        check(L.lib().deo_nonlinear_diffusion(self._h, C.c_void_p(p.data_ptr()), C.c_void_p(q.data_ptr()),
                                              C.c_void_p(du.data_ptr()), _stream_ptr()))
        return du


def _plan(n, m, approx, dx, nknots, dtype_code):
    dxa = np.atleast_1d(np.asarray(dx, dtype=np.float64))
    key = (n, m, approx, dxa.tobytes(), nknots, dtype_code)
    p = _cache.get(key)
    if p is None:
        p = _cache[key] = NonlinearDiffusionPlan(n, m, approx, dxa, nknots, dtype_code)
    return p


def nonlinear_diffusion_(du, second_order: int, first_order: int, approx_order: int, p, q, dx, nknots: int):
    """nonlinear_diffusion!(du, n, m, approx_order, p, q, dx, nknots) on CUDA vectors."""
    import torch
    code = 0 if q.dtype == torch.float64 else 1
    return _plan(second_order, first_order, approx_order, dx, nknots, code).apply(du, p, q)


def nonlinear_diffusion(second_order: int, first_order: int, approx_order: int, p, q, dx, nknots: int):
    """Out-of-place nonlinear_diffusion: a new vector of nknots entries."""
    du = q.new_empty(nknots)
    return nonlinear_diffusion_(du, second_order, first_order, approx_order, p, q, dx, nknots)
