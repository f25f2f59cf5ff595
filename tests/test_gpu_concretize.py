"""GPU: concretisation built on the device from the plan's row tables
(deo_plan_concretize, deo_plan_concretize_device, deo_plan_bandwidths,
deo_plan_concretize_banded) against the oracle's unit-vector probes of the
reference's loops (Array(L*Q), concretization.jl:914-958): 1-D to 3-D,
centred and upwind, uniform and non-uniform grids, every BC kind, coefficient
vectors and fields, per-line BCs, merged terms, Float32 plans; the banded
form equal to the dense one entry for entry; at a size no dense matrix fits
(1-D N = 10^6), the banded matrix times u equals the apply."""
import numpy as np
import pytest

import deo
import oracle as O
from cases import build, to_device, to_host
from test_gpu_parity import T

pytestmark = pytest.mark.gpu

ROBIN = ("robin", (1.0, 0.5, 0.2), (0.7, 0.3, -0.1), 1)
GEN = ("general", (-1.0, 1.0, 0.5), (0.5, 1.0, 0.25), 2)
CASES = {
    "1d-centred-robin": dict(shape=(41,), terms=[T("centered", 2, 4, bc=ROBIN, coeff="vector")], seed=1),
    "1d-nonuniform-general": dict(shape=(37,), terms=[T("centered", 1, 6, grid="nonuniform", bc=GEN)], seed=2),
    "1d-upwind-offside": dict(shape=(33,), terms=[T("upwind", 2, 2, offside=1, coeff=-1.5, bc=ROBIN)], seed=3),
    "1d-periodic": dict(shape=(30,), terms=[T("centered", 2, 4, bc=("periodic",))], seed=4),
    "1d-neumann-d4": dict(shape=(35,), terms=[T("centered", 4, 2, bc=("neumann", 0.3, -0.2, 1))], seed=5),
    "2d-mixed": dict(shape=(14, 11), terms=[T("centered", 2, 2, axis=1, bc=ROBIN),
                                            T("centered", 1, 4, axis=2, bc=("periodic",)),
                                            T("upwind", 1, 2, axis=1, coeff=0.7, bc=("dirichlet", 0.3, -1.2))],
                     seed=6),
    "2d-field": dict(shape=(13, 12), terms=[T("upwind", 1, 2, axis=1, coeff="field", bc=("dirichlet0",)),
                                            T("centered", 2, 2, axis=2, coeff="field", bc=ROBIN)], seed=7),
    "3d-lap": dict(shape=(9, 8, 7), terms=[T("centered", 2, 4, axis=k, bc=ROBIN) for k in (1, 2, 3)], seed=8),
}


def _check(Dl, Db, Al, Ab, rtol=1e-12):
    assert np.allclose(Dl, Al, rtol=rtol, atol=rtol * np.abs(Al).max())
    assert np.allclose(Db, Ab, rtol=rtol, atol=rtol * max(1.0, np.abs(Ab).max()))


def _banded_to_dense(lo, up, data, n):
    D = np.zeros((n, n))
    for j in range(n):
        for r in range(lo + up + 1):
            i = j + r - up
            if 0 <= i < n:
                D[i, j] = data[r, j]
    return D


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("merge", [False, True])
def test_dense_and_banded_against_oracle(cuda, name, merge):
    import torch
    case = CASES[name]
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    n = int(np.prod(shape))
    Al, Ab = O.concretize_probe(oterms, shape)
    p = deo.Plan(A.terms(), shape, 0, merge_terms=merge)
    Dl, Db = p.concretize()
    _check(Dl, Db, Al, Ab)
    # the structural bandwidths cover every nonzero; the band storage holds the dense matrix
    lo, up = p.bandwidths()
    nz = np.nonzero(Al)
    assert lo >= (nz[0] - nz[1]).max(initial=0) and up >= (nz[1] - nz[0]).max(initial=0)
    l2, u2, data, ab = p.concretize_banded()
    assert (l2, u2) == (lo, up)
    assert np.array_equal(_banded_to_dense(lo, up, data.cpu().numpy(), n), Dl)
    assert np.array_equal(ab.cpu().numpy(), Db)
    # on a stream of the caller's, into device buffers
    s = torch.cuda.Stream()
    dA = torch.empty((n, n), dtype=torch.float64, device="cuda")
    dB = torch.empty(n, dtype=torch.float64, device="cuda")
    with torch.cuda.stream(s):
        assert deo.lib().deo_plan_concretize_device(p.handle, __import__("ctypes").c_void_p(dA.data_ptr()),
                                                    __import__("ctypes").c_void_p(dB.data_ptr()),
                                                    __import__("ctypes").c_void_p(s.cuda_stream)) == 0
    s.synchronize()
    assert np.array_equal(dA.cpu().numpy().T, Dl)  # row-major view of the column-major matrix
    assert np.array_equal(dB.cpu().numpy(), Db)
    assert deo.device_status() == 0


def test_per_line_bcs_and_float32(cuda):
    from test_gpu_line_bcs import _problem
    shape = (12, 10)
    A, oterms = _problem(shape, {1, 2}, 2, 4, seed=3)
    Al, Ab = O.concretize_probe(oterms, shape)
    Dl, Db = deo.Plan(A.terms(), shape, 0).concretize()
    _check(Dl, Db, Al, Ab)
    # a Float32 plan: its float weights, widened
    case = CASES["3d-lap"]
    A, oterms, _ = build(case, dtype="f32")
    shape = tuple(case["shape"])
    Al, Ab = O.concretize_probe(oterms, shape)
    Dl, Db = deo.Plan(A.terms(), shape, 1).concretize()
    _check(Dl, Db, Al, Ab, rtol=1e-6)


def test_banded_times_u_equals_apply_at_one_million_points(cuda):
    import torch
    n = 1_000_000
    h = 1.0 / (n + 1)
    P = deo.CenteredDifference(2, 4, h, n)
    Q = deo.RobinBC((1.0, 0.5, 0.2), (0.7, 0.3, -0.1), h, 1)
    p = deo.Plan([P * Q], (n,), 0)
    lo, up, data, ab = p.concretize_banded()
    assert lo + up + 1 <= 16
    u = torch.randn(n, dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(3))
    du = torch.empty_like(u)
    p.apply(u, du)
    # (A_l u)_i = sum_r data[r, j] u_j over j = i + up - r
    mv = torch.zeros_like(u)
    for r in range(lo + up + 1):
        sh = up - r  # j = i + sh
        if sh >= 0:
            mv[:n - sh] += data[r, sh:] * u[sh:]
        else:
            mv[-sh:] += data[r, :n + sh] * u[:n + sh]
    mv += ab
    scale = torch.zeros_like(u)
    for r in range(lo + up + 1):
        sh = up - r
        if sh >= 0:
            scale[:n - sh] += (data[r, sh:] * u[sh:]).abs()
        else:
            scale[-sh:] += (data[r, :n + sh] * u[:n + sh]).abs()
    assert bool(((mv - du).abs() <= 64 * 2.0 ** -52 * (scale + ab.abs())).all())
    assert deo.device_status() == 0
