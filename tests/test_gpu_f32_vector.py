"""GPU: the vectorised Float32 interior kernel (k_lap_v, 4 consecutive x
points per thread) against the scalar one (k_lap_q) and the generic row-table
kernel, bit for bit, and against the oracle: band radii 1-3, 2-D and 3-D,
sizes that leave partial tiles and partial vectors at every edge, overwrite
and accumulate, Robin / Dirichlet / Neumann / periodic faces, every shell
kernel beside the interior and after it; an output that is not 16-byte
aligned falls back to k_lap_q."""
import numpy as np
import pytest

import deo
import oracle as O
from cases import build, to_device, to_host
from test_gpu_parity import T

pytestmark = pytest.mark.gpu

ROBIN = ("robin", (1.0, 0.5, 0.0), (1.0, 0.5, 0.0), 1)


def _lap(shape, d, a, bc, seed):
    return dict(shape=shape, terms=[T("centered", d, a, axis=k + 1, h=1.0 / (shape[0] + 1), bc=bc)
                                    for k in range(len(shape))], seed=seed)


CASES = [
    _lap((72, 45, 33), 2, 4, ROBIN, 1),               # H = 2, partial tiles along x, y, z
    _lap((68, 70, 19), 2, 2, ("dirichlet0",), 2),     # H = 1
    _lap((76, 34, 40), 2, 6, ("neumann", 0.3, -0.2, 1), 3),  # H = 3
    _lap((128, 96, 24), 1, 4, ("periodic",), 4),      # first derivative, H = 2, periodic faces
    _lap((260, 130), 2, 4, ROBIN, 5),                 # 2-D
    _lap((64, 64, 64), 4, 2, ("dirichlet", 0.3, -0.7), 6),  # d = 4
]
IDS = ["a4-robin", "a2-dirichlet0", "a6-neumann", "d1-periodic", "2d-a4", "d4-dirichlet"]


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_vector_interior_bitwise_equals_scalar_and_generic(cuda, case):
    import torch
    A, oterms, u = build(case, dtype="f32")
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 1)
    ud = to_device(u, "f32")
    base = to_device(np.asfortranarray(np.random.default_rng(9).standard_normal(shape)), "f32")
    outs = {}
    variants = {"vector": (1, 1, 1, 0, 0), "vector-after": (1, 1, 0, 0, 0), "vector-lines": (1, 1, 1, 2, 0),
                "vector-generic-shell": (1, 1, 0, 3, 0), "tile1": (1, 1, 1, 0, 1), "tile2": (1, 1, 1, 0, 2),
                "tile3": (1, 1, 1, 0, 3), "scalar": (1, 0, 1, 0, 0), "generic": (0, 1, 1, 0, 0)}
    for name, (fast, vec, conc, shell, tile) in variants.items():
        p.set_option(deo.DEO_OPT_FAST_PATH, fast)
        p.set_option(deo.DEO_OPT_F32_VECTOR, vec)
        p.set_option(deo.DEO_OPT_CONCURRENT_SHELL, conc)
        p.set_option(deo.DEO_OPT_SHELL_KERNEL, shell)
        p.set_option(deo.DEO_OPT_F32_TILE, tile)
        o = deo.julia_array(shape, torch.float32, fill=np.nan)
        p.apply(ud, o)
        acc = base.clone()
        p.apply(ud, acc, overwrite=False)
        outs[name] = (o, acc, p.kernels)
    assert p.get_option(deo.DEO_OPT_F32_VECTOR) == 1
    assert outs["vector"][2] == ("k_lap_v", "k_face")
    assert outs["vector-lines"][2] == ("k_lap_v", "k_shell_lines")
    assert outs["vector-generic-shell"][2] == ("k_lap_v", "k_shell_generic")
    assert outs["scalar"][2][0] == "k_lap_q"
    assert outs["generic"][2] == ("k_apply",)
    for name in variants:
        assert torch.equal(outs[name][0], outs["generic"][0]), name
        assert torch.equal(outs[name][1], outs["generic"][1]), name
    # Float32 against the FP64 oracle: within 64 * 2^-24 of sum |c_k u_k| per point
    ref = O.apply(oterms, u.astype(np.float64))
    scale = O.abs_scale(oterms, u.astype(np.float64))
    err = np.abs(to_host(outs["vector"][0]).astype(np.float64) - ref)
    assert (err <= 64 * 2.0 ** -24 * scale + 1e-30).all()
    assert deo.device_status() == 0


def test_unaligned_output_falls_back_to_scalar_kernel(cuda):
    import ctypes as C
    import torch
    case = CASES[0]
    A, oterms, u = build(case, dtype="f32")
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 1)
    ud = to_device(u, "f32")
    n = int(np.prod(shape))
    buf = torch.full((n + 1,), float("nan"), dtype=torch.float32, device="cuda")
    o_off = buf[1:]  # 4 bytes past a 16-byte boundary, the plan's (column-major) layout
    assert o_off.data_ptr() % 16 == 4
    st = torch.cuda.current_stream().cuda_stream
    assert deo.lib().deo_apply(p.handle, C.c_void_p(ud.data_ptr()), C.c_void_p(o_off.data_ptr()), 1,
                               C.c_void_p(st)) == 0
    assert p.kernels[0] == "k_lap_q" and p.kernels[1] == "k_face"  # the whole shell
    o = deo.julia_array(shape, torch.float32)
    p.apply(ud, o)
    assert p.kernels[0] == "k_lap_v"
    flat = o.permute(*reversed(range(len(shape)))).reshape(-1)  # memory order
    assert torch.equal(flat, o_off)
    assert deo.device_status() == 0


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_autotune_keeps_results_and_caches(cuda, dtype, tmp_path):
    """deo_plan_autotune chooses among bit-identical execution choices: after
    it the apply equals the generic kernel bit for bit; the choice is written
    to the cache file once and a second plan of the same signature takes it
    from there."""
    import torch
    case = CASES[0]
    A, oterms, u = build(case, dtype=dtype)
    shape = tuple(case["shape"])
    code = 0 if dtype == "f64" else 1
    tdt = torch.float64 if dtype == "f64" else torch.float32
    p = deo.Plan(A.terms(), shape, code)
    ud = to_device(u, dtype)
    scratch = deo.julia_array(shape, tdt)
    cache = str(tmp_path / "tune.cache")
    got = p.autotune(ud, scratch, cache)
    assert got["shell_kernel"] in (0, 1, 2) and got["concurrent_shell"] in (0, 1)  # 0: the plan's own choice kept
    if dtype == "f32":
        assert got["f32_vector"] in (0, 1) and got["f32_tile"] in (0, 1, 2, 3)
    o = deo.julia_array(shape, tdt)
    p.apply(ud, o)
    p.set_option(deo.DEO_OPT_FAST_PATH, 0)
    ref = deo.julia_array(shape, tdt)
    p.apply(ud, ref)
    if dtype == "f32":
        assert torch.equal(o, ref)
    else:  # the plan's Float64 interior (fixed point) is within 4 ulp of the reference order
        r, g = to_host(ref), to_host(o)
        assert (np.abs(r - g) <= 4 * np.spacing(O.abs_scale(oterms, u))).all()
    lines = open(cache).read().split("\n")
    assert len([x for x in lines if x.strip()]) == 1
    q = deo.Plan(A.terms(), shape, code)
    assert q.autotune(ud, scratch, cache) == got
    assert len([x for x in open(cache).read().split("\n") if x.strip()]) == 1  # taken from the cache
    assert deo.device_status() == 0
