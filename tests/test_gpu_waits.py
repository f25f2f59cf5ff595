"""GPU: a bounded device wait that runs out, without a fault.

Every mbarrier wait in the TMA kernels gives up after a bounded number of
polls, sets a device status bit, waits (bounded) for the kernel's other copies
still in flight and returns.  The plan option DEO_OPT_TEST_WITHHOLD makes that
happen on purpose: the kernels never issue one plane's copy (each CTA's first
shell box), so the wait for it runs out after 64 polls -- a flag that nothing
sets.  The host then reads DEO_ERR_TIMEOUT from deo_device_status, and the
same plan, with the hook off, applies correctly in the same process."""
import ctypes as C

import numpy as np
import pytest

import deo
import oracle as O
from cases import build, to_device, to_host
from test_gpu_parity import T

pytestmark = pytest.mark.gpu

CASE = dict(shape=(72, 40, 24), terms=[T("centered", 2, 4, axis=k, h=1 / 73,
                                         bc=("robin", (1.0, 0.5, 0.0), (1.0, 0.5, 0.0), 1)) for k in (1, 2, 3)],
            seed=41)
VARIANTS = [("f64", 1), ("f64", 5), ("f32", 1)]


@pytest.mark.parametrize("dtype,variant", VARIANTS)
def test_bounded_wait_runs_out_and_the_plan_recovers(cuda, dtype, variant):
    import torch
    A, oterms, u = build(CASE, dtype=dtype)
    shape = tuple(CASE["shape"])
    p = deo.Plan(A.terms(), shape, 0 if dtype == "f64" else 1)
    p.set_option(deo.DEO_OPT_EXACT_SUMS, variant)
    assert deo.device_status() == 0
    ud = to_device(u, dtype)
    out = deo.julia_array(shape, torch.float64 if dtype == "f64" else torch.float32)
    lib = deo.lib()
    for plane in (1, 3):
        p.set_option(deo.DEO_OPT_TEST_WITHHOLD, plane)
        assert p.get_option(deo.DEO_OPT_TEST_WITHHOLD) == plane
        p.apply(ud, out)
        assert p.kernels[0].startswith("k_lap_")
        assert p.kernels[1] == "k_face"  # the shell beside it withholds its first box too
        torch.cuda.synchronize()  # the kernels returned: nothing hangs
        v = C.c_uint(0)
        st = lib.deo_device_status(C.byref(v))
        assert st == 5, lib.deo_last_error().decode()  # DEO_ERR_TIMEOUT
        assert v.value & 1
        assert b"bounded device wait" in lib.deo_last_error()
        assert deo.device_status() == 0  # the flags were cleared by the read
    p.set_option(deo.DEO_OPT_TEST_WITHHOLD, 0)
    p.apply(ud, out)
    torch.cuda.synchronize()
    assert deo.device_status() == 0
    ref = O.apply(oterms, u)
    got = to_host(out)
    if dtype == "f64":
        assert (np.abs(got - ref) <= 4 * np.spacing(O.abs_scale(oterms, u))).all()
    else:
        assert (np.abs(got - ref) <= 64 * 2.0 ** -24 * O.abs_scale(oterms, u)).all()


def test_withhold_option_range(cuda):
    A, oterms, u = build(CASE)
    p = deo.Plan(A.terms(), tuple(CASE["shape"]), 0)
    with pytest.raises(deo.DeoArgError):
        p.set_option(deo.DEO_OPT_TEST_WITHHOLD, -1)
    with pytest.raises(deo.DeoArgError):
        p.set_option(deo.DEO_OPT_TEST_WITHHOLD, 65)
