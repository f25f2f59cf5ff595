"""The allocation-free batched entry point (deo_batch_apply_noalloc).

Callers that cannot allocate device memory -- plug-ins whose host application
owns every device allocation, servers that must not grow their footprint after
admission --
use this entry point: it keeps the batched kernel's instance table, work-list
and counter in a static device array instead of cudaMalloc'd buffers.  Its
results must equal the allocating entry point's (same kernel), call after
call, since every call reuses and re-clears the same array; and once the
set-up call (n = 0) has run on a device, later calls must leave the device's
free memory unchanged.  Kept in a file collected last so that a failure here
stops a `-x` run only after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

import deo
from deo import _lib
from cases import build, to_device
from test_gpu_parity import T

pytestmark = pytest.mark.gpu


def _instances(seed=17, n=24):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        if rng.random() < 0.6:
            N = int(np.exp(rng.uniform(np.log(64), np.log(20000))))
            case = dict(shape=(N,), terms=[T("centered", int(rng.integers(1, 5)), int(rng.choice([2, 4, 6])),
                                             grid="uniform" if rng.random() < 0.5 else "nonuniform",
                                             bc=("robin", (1.0, 0.5, 0.1), (1.0, 0.5, -0.1), 1))], seed=k)
        else:
            s = (int(rng.integers(20, 150)), int(rng.integers(20, 150)))
            case = dict(shape=s, terms=[T("centered", 2, 4, axis=1, bc=("dirichlet0",)),
                                        T("upwind", 1, 2, axis=2, coeff=-0.8, bc=("dirichlet", 0.5, -0.5))],
                        seed=k)
        out.append(case)
    return out


def _setup(adjoint):
    import torch
    plans, us, outs_ref, outs_new = [], [], [], []
    for c in _instances():
        A, _, u = build(c)
        shape = tuple(c["shape"])
        p = deo.Plan(A.terms(), shape, 0)
        plans.append(p)
        us.append(to_device(u))
        outs_ref.append(deo.julia_array(shape, fill=0.0))
        outs_new.append(deo.julia_array(shape, fill=np.nan))
    ref = deo.Batch(list(zip(plans, us, outs_ref)), adjoint=adjoint)
    ref.run(use_graph=False)
    torch.cuda.synchronize()
    arr = (_lib.Instance * len(plans))()
    for i, (p, u, o) in enumerate(zip(plans, us, outs_new)):
        arr[i].plan = p.handle
        arr[i].u = C.c_void_p(u.data_ptr())
        arr[i].du = C.c_void_p(o.data_ptr())
    return plans, us, outs_ref, outs_new, arr, ref


@pytest.mark.parametrize("adjoint", [0, 1])
def test_noalloc_matches_allocating_entry_point(cuda, adjoint):
    import torch
    plans, us, outs_ref, outs_new, arr, ref = _setup(adjoint)
    lib = deo.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):  # two calls in a row share (and re-clear) the static work-list
        for o in outs_new:
            o.fill_(np.nan)
        st = lib.deo_batch_apply_noalloc(len(plans), arr, adjoint, 1024 * (call + 1), stream)
        assert st == 0, lib.deo_last_error().decode()
        torch.cuda.synchronize()
        for a, b in zip(outs_new, outs_ref):
            assert torch.equal(a, b), f"call {call}"
    assert deo.device_status() == 0


def test_noalloc_rejects_batches_beyond_its_scratch(cuda):
    import torch
    plans, us, outs_ref, outs_new, arr, ref = _setup(0)
    lib = deo.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # one-point tiles need ~16 B per point of work-list: far beyond 1 MiB
    st = lib.deo_batch_apply_noalloc(len(plans), arr, 0, 1, stream)
    assert st == 3  # DEO_ERR_UNSUPPORTED
    assert b"static scratch" in lib.deo_last_error()
    # a rejected call leaves the entry point usable
    assert lib.deo_batch_apply_noalloc(len(plans), arr, 0, 0, stream) == 0
    torch.cuda.synchronize()
    for a, b in zip(outs_new, outs_ref):
        assert torch.equal(a, b)


def test_noalloc_calls_leave_free_device_memory_unchanged(cuda):
    """After the set-up call (n = 0), calls of several sizes, tiles and both
    directions allocate nothing: the driver's free-memory figure stays put."""
    import torch
    plans, us, outs_ref, outs_new, arr, ref = _setup(0)
    lib = deo.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.deo_batch_apply_noalloc(0, None, 0, 0, stream) == 0, lib.deo_last_error().decode()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for k, (count, tile, adj) in enumerate([(len(plans), 0, 0), (5, 512, 1), (len(plans), 4096, 0), (1, 0, 1)]):
        st = lib.deo_batch_apply_noalloc(count, arr, adj, tile, stream)
        assert st == 0, lib.deo_last_error().decode()
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, f"call {k}: free device memory changed by {free0 - free1} bytes"
    # the last forward call over every instance still matches the allocating entry point
    assert lib.deo_batch_apply_noalloc(len(plans), arr, 0, 0, stream) == 0
    torch.cuda.synchronize()
    for a, b in zip(outs_new, outs_ref):
        assert torch.equal(a, b)
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_refuses_stream_capture(cuda):
    """Under stream capture the call enqueues nothing and returns
    DEO_ERR_UNSUPPORTED; the capture stays valid and the entry point usable."""
    import torch
    plans, us, outs_ref, outs_new, arr, ref = _setup(0)
    lib = deo.lib()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st = lib.deo_batch_apply_noalloc(len(plans), arr, 0, 0, C.c_void_p(s.cuda_stream))
    assert st == 3  # DEO_ERR_UNSUPPORTED
    assert b"stream capture" in lib.deo_last_error()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.deo_batch_apply_noalloc(len(plans), arr, 0, 0, stream) == 0
    torch.cuda.synchronize()
    for a, b in zip(outs_new, outs_ref):
        assert torch.equal(a, b)
