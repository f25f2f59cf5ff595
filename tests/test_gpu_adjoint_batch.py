"""GPU: adjoint kernel, rrule, fast path vs generic path, batched launches,
SSP-RK3 stages and the time-integration adjoint."""
import numpy as np
import pytest

import deo
import oracle as O
from cases import build, to_device, to_host
from test_gpu_parity import ND, ONE_D, T

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _plan(A, shape):
    return deo.plan_for(A.terms(), shape, 0)


ADJ_CASES = [ONE_D[0], ONE_D[5], ONE_D[17], ONE_D[40], ONE_D[70], ONE_D[-1], ONE_D[-7],
             dict(ND[0], shape=(9, 8, 7)), dict(ND[1], shape=(6, 7, 8)), dict(ND[2], shape=(6, 5, 7)),
             dict(ND[3], shape=(14, 12)), dict(ND[4], shape=(7, 8, 9, 10)), ND[5], ND[6]]


@pytest.mark.parametrize("case", ADJ_CASES, ids=lambda c: "x".join(map(str, c["shape"])) + f"-s{c['seed']}")
def test_adjoint_matches_concretized_transpose(cuda, case):
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    Al, Ab = O.concretize_probe(oterms, shape)
    rng = np.random.default_rng(5)
    v = np.asfortranarray(rng.standard_normal(shape))
    p = _plan(A, shape)
    ub = deo.julia_array(shape)
    p.adjoint(to_device(v), ub)
    got = to_host(ub).ravel(order="F")
    ref = Al.T @ v.ravel(order="F")
    scale = np.abs(Al).T @ np.abs(v.ravel(order="F"))
    assert np.all(np.abs(got - ref) <= 64 * EPS * scale + 1e-300)
    # the device concretisation is the same matrix
    Dl, Db = p.concretize()
    assert np.allclose(Dl, Al, rtol=1e-12, atol=1e-12 * np.abs(Al).max())
    assert np.allclose(Db, Ab, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(Ab).max()))


@pytest.mark.parametrize("d,a,bc", [(2, 2, ("robin", (1.0, 0.5, 0.2), (0.7, 0.3, -0.1), 1)), (1, 4, ("dirichlet0",)),
                                    (2, 4, ("general", (-1.0, 1.0, 0.5), (0.5, 1.0, 0.25), 2)), (4, 2, ("periodic",))])
def test_adjoint_against_reference_concretization(cuda, d, a, bc):
    # transpose of Array(L*Q) = (Array(L)*Q_L, Array(L)*Q_b) (concretization.jl:914-918)
    case = dict(shape=(33,), terms=[T("centered", d, a, bc=bc)], seed=d + a)
    A, oterms, u = build(case)
    Lo, qo, _ = oterms[0]
    QL, Qb = qo.array(33)
    Al = Lo.array() @ QL
    v = np.random.default_rng(3).standard_normal(33)
    ub = deo.julia_array((33,))
    _plan(A, (33,)).adjoint(to_device(v), ub)
    assert np.allclose(to_host(ub), Al.T @ v, rtol=1e-11, atol=1e-11 * np.abs(Al).max() * np.abs(v).max())


def test_rrule_and_autograd_fd(cuda):
    import torch
    case = ND[3]
    A, oterms, u = build(case)
    ud = to_device(u)
    y, pb = deo.rrule(A, ud)
    w = to_device(np.asfortranarray(np.random.default_rng(1).standard_normal(u.shape)))
    _, _, ubar = pb(w)
    v = to_device(np.asfortranarray(np.random.default_rng(2).standard_normal(u.shape)))
    eps = 1e-3
    lp = float((w * (A * (ud + eps * v))).sum())
    lm = float((w * (A * (ud - eps * v))).sum())
    fd = (lp - lm) / (2 * eps)
    ad = float((ubar * v).sum())
    assert abs(fd - ad) <= 1e-8 * max(1.0, abs(ad)), (fd, ad)
    # torch autograd through the same kernels
    ut = ud.clone().requires_grad_(True)
    loss = (deo.autodiff.apply(A, ut) * w).sum()
    loss.backward()
    assert torch.equal(ut.grad, ubar)


def test_dot_product_identity_full_size(cuda):
    # <A_l u, v> = <u, A_l^T v> on the 256^3 Laplacian (size-independent check)
    import torch
    n = 256
    h = 1.0 / (n + 1)
    A = sum((deo.CenteredDifference(2, 4, h, n, axis=k) for k in (1, 2, 3)), deo.DiffEqOperatorCombination([]))
    Q = deo.compose(*deo.RobinBC((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), (h, h, h), 1, (n, n, n)))
    AQ = A * Q
    p = _plan(AQ, (n, n, n))
    g = torch.Generator(device="cuda").manual_seed(0)
    u = deo.julia_array((n, n, n)); u.copy_(torch.randn(n, n, n, generator=g, device="cuda", dtype=torch.float64))
    v = deo.julia_array((n, n, n)); v.copy_(torch.randn(n, n, n, generator=g, device="cuda", dtype=torch.float64))
    z = deo.julia_array((n, n, n), fill=0.0)
    Au, A0, Atv = deo.julia_array((n, n, n)), deo.julia_array((n, n, n)), deo.julia_array((n, n, n))
    p.apply(u, Au)
    p.apply(z, A0)  # affine part (zero for this BC)
    p.adjoint(v, Atv)
    lhs = float(((Au - A0) * v).sum())
    rhs = float((u * Atv).sum())
    assert abs(lhs - rhs) <= 1e-12 * float((Au.abs() * v.abs()).sum())


@pytest.mark.parametrize("case", [ND[0], ND[1], ND[2], dict(ND[0], shape=(70, 45, 33)),
                                  dict(shape=(64, 50), terms=[T("centered", 2, 6, axis=1, bc=("dirichlet0",)),
                                                              T("centered", 1, 8, axis=2, bc=("periodic",)),
                                                              T("upwind", 1, 2, axis=1, coeff=0.7,
                                                                bc=("dirichlet0",))], seed=31)],
                         ids=["lap3d", "d0", "periodic", "odd", "2d-mixed"])
def test_fast_path_bitwise_equals_generic(cuda, case):
    import torch
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 0)
    assert p.uses_fast_path
    ud = to_device(u)
    ref = O.apply(oterms, u)
    tol = 4 * np.spacing(O.abs_scale(oterms, u))
    outs = {}
    # (fast path, TMA ring, exact neighbour sums)
    for name, opts in {"tma-ens": (1, 1, 1), "tma-bfx": (1, 1, 5), "tma-ens-v2": (1, 1, 3), "tma-ens-v1": (1, 1, 2),
                       "tma-fma": (1, 1, 0),
                       "queue": (1, 0, 0), "generic": (0, 0, 0)}.items():
        p.set_option(deo.DEO_OPT_FAST_PATH, opts[0])
        p.set_option(deo.DEO_OPT_TMA, opts[1])
        p.set_option(deo.DEO_OPT_EXACT_SUMS, opts[2])
        o = deo.julia_array(shape)
        p.apply(ud, o)
        outs[name] = o
        assert (np.abs(to_host(o) - ref) <= tol).all(), name
    # the reference-order paths agree bit for bit
    assert torch.equal(outs["tma-fma"], outs["generic"])
    assert torch.equal(outs["queue"], outs["generic"])
    assert deo.device_status() == 0


def _mixed_instances(seed=0, n=40):
    rng = np.random.default_rng(seed)
    inst = []
    for k in range(n):
        if rng.random() < 0.7:
            N = int(np.exp(rng.uniform(np.log(64), np.log(4096))))
            case = dict(shape=(N,), terms=[T("centered", int(rng.integers(1, 5)), int(rng.choice([2, 4, 6, 8])),
                                             grid="uniform" if rng.random() < 0.5 else "nonuniform",
                                             bc=("robin", (1.0, 0.5, 0.1), (1.0, 0.5, -0.1), 1)
                                             if rng.random() < 0.5 else ("dirichlet0",))], seed=k)
        else:
            s = (int(np.exp(rng.uniform(np.log(32), np.log(200)))), int(np.exp(rng.uniform(np.log(32), np.log(200)))))
            d, a = int(rng.integers(1, 5)), int(rng.choice([2, 4, 6, 8]))
            g = "uniform" if rng.random() < 0.5 else "nonuniform"
            case = dict(shape=s, terms=[T("centered", d, a, axis=1, grid=g, bc=("dirichlet0",)),
                                        T("centered", d, a, axis=2, grid=g, bc=("dirichlet0",))], seed=k)
        inst.append(case)
    return inst


@pytest.mark.parametrize("adjoint", [False, True])
def test_batched_equals_individual(cuda, adjoint):
    import torch
    cases = _mixed_instances()
    plans, us, outs, refs = [], [], [], []
    for c in cases:
        A, oterms, u = build(c)
        shape = tuple(c["shape"])
        p = deo.Plan(A.terms(), shape, 0)
        p.set_option(deo.DEO_OPT_EXACT_SUMS, 0)  # the batched kernel keeps the reference's tap order
        ud = to_device(u)
        r = deo.julia_array(shape)
        (p.adjoint if adjoint else p.apply)(ud, r)
        plans.append(p); us.append(ud); refs.append(r); outs.append(deo.julia_array(shape))
    b = deo.Batch(list(zip(plans, us, outs)), adjoint=adjoint)
    b.run(use_graph=False)
    torch.cuda.synchronize()
    for o, r in zip(outs, refs):
        assert torch.equal(o, r)
    for o in outs:
        o.zero_()
    b.run(use_graph=True)
    b.run(use_graph=True)  # graph replay
    torch.cuda.synchronize()
    for o, r in zip(outs, refs):
        assert torch.equal(o, r)
    cfg = b.autotune()
    assert cfg["tile"] > 0 and cfg["work_items"] > 0
    for o in outs:
        o.zero_()
    b.run(use_graph=True)
    torch.cuda.synchronize()
    for o, r in zip(outs, refs):
        assert torch.equal(o, r)


def _advection_diffusion(shape, nu, c, a=2):
    """nu * sum_k D2_k + UpwindDifference(1, a, h, n, -c) along axis 1, Dirichlet0 on every face."""
    terms_p, terms_o = [], []
    for k, n in enumerate(shape):
        h = 1.0 / (n + 1)
        P = nu * deo.CenteredDifference(2, 2, h, n, axis=k + 1)
        Qo = O.centered(2, 2, h, n, axis=k + 1).scale(nu)
        terms_p.append(P)
        terms_o.append(Qo)
    h = 1.0 / (shape[0] + 1)
    terms_p.append(deo.UpwindDifference(1, a, h, shape[0], -c, axis=1))
    terms_o.append(O.upwind(1, a, h, shape[0], -c, axis=1))
    bc = deo.Dirichlet0BC()
    if len(shape) == 1:
        A = deo.DiffEqOperatorCombination([P * bc for P in terms_p])
    else:
        A = deo.DiffEqOperatorCombination([P * deo.MultiDimDirectionalBC(bc, P.axis, shape) for P in terms_p])
    oterms = [(Q, O.dirichlet0()) for Q in terms_o]
    return A, oterms


@pytest.mark.parametrize("shape", [(200,), (40, 30), (12, 11, 10)])
def test_ssprk3_matches_oracle(cuda, shape):
    A, oterms = _advection_diffusion(shape, 0.05, 0.6)
    rng = np.random.default_rng(8)
    u0 = np.asfortranarray(rng.standard_normal(shape))
    h = 1.0 / (shape[0] + 1)
    dt = 0.4 * min(h / 0.6, h * h / (2 * 0.05 * len(shape)))
    K = 25
    got = to_host(deo.autodiff.ssprk3_solve(A, to_device(u0), dt, K))
    ref = O.ssprk3(oterms, u0, dt, K)
    assert np.allclose(got, ref, rtol=0, atol=1e-12 * K * np.abs(ref).max())


def test_ssprk3_gradient_fd_and_checkpointing(cuda):
    import torch
    shape = (30, 20)
    A, oterms = _advection_diffusion(shape, 0.02, -0.4)
    rng = np.random.default_rng(9)
    u0 = to_device(np.asfortranarray(rng.standard_normal(shape)))
    h = 1.0 / 31
    dt = 0.4 * min(h / 0.4, h * h / (2 * 0.02 * 2))
    K = 17
    uT, g = deo.autodiff.ssprk3_grad_norm2(A, u0, dt, K)
    uT2, g2 = deo.autodiff.ssprk3_grad_norm2(A, u0, dt, K, checkpoint="sqrtK")
    assert torch.equal(uT, uT2) and torch.equal(g, g2)
    v = to_device(np.asfortranarray(rng.standard_normal(shape)))
    eps = 1e-4
    fp = float((deo.autodiff.ssprk3_solve(A, u0 + eps * v, dt, K) ** 2).sum())
    fm = float((deo.autodiff.ssprk3_solve(A, u0 - eps * v, dt, K) ** 2).sum())
    fd = (fp - fm) / (2 * eps)
    ad = float((g * v).sum())
    assert abs(fd - ad) <= 1e-7 * max(1.0, abs(ad)), (fd, ad)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_full_size_laplacian_against_oracle(cuda, dtype):
    """The 256^3 Robin Laplacian (the benchmark configuration) against the
    oracle at full size: Float64 within 4 ulp of sum|c_k u_k| in every mode;
    Float32 error against the Float64 oracle reported and bounded."""
    import json
    import os
    import torch
    import bench
    n = 256
    h = 1.0 / (n + 1)
    u = bench.fourier_field(n)
    q = O.robin((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), h, 1)
    terms = [(O.centered(2, 4, h, n, axis=k), q) for k in (1, 2, 3)]
    ref = O.apply(terms, u, nthreads=os.cpu_count() or 1)
    scale = O.abs_scale(terms, u)
    _, plan, tdt = bench.lap3d_setup(n, dtype)
    ud = deo.julia_array((n, n, n), tdt)
    ud.copy_(torch.from_numpy(u).to(tdt))
    report = {}
    modes = ({"exact-sums": 1, "block-fixed-point": 5, "exact-sums-v2": 3, "exact-sums-v1": 2, "reference-order": 0}
             if dtype == "f64" else {"default": 1})
    for name, ens in modes.items():
        plan.set_option(deo.DEO_OPT_EXACT_SUMS, ens)
        du = deo.julia_array((n, n, n), tdt)
        plan.apply(ud, du)
        report.setdefault("kernels", {})[name] = list(plan.kernels)
        got = du.to(torch.float64).cpu().numpy()
        ulps = np.abs(got - ref) / np.spacing(scale)
        report[name] = {"max_ulp_of_scale": float(ulps.max()), "mean_ulp_of_scale": float(ulps.mean()),
                        "max_rel_to_scale": float((np.abs(got - ref) / scale).max())}
        if dtype == "f64":
            assert ulps.max() <= 4.0, (name, report[name])
        else:
            assert report[name]["max_rel_to_scale"] < 64 * 2.0 ** -24
    if dtype == "f64":
        assert report["kernels"]["exact-sums"][0] == "k_lap_fx"
        assert report["kernels"]["block-fixed-point"][0] == "k_lap_bfx"
        assert report["kernels"]["exact-sums-v2"][0] == "k_lap_ens2"
    plan.set_option(deo.DEO_OPT_EXACT_SUMS, 1)
    assert deo.device_status() == 0
    out = os.environ.get("DEO_REPORT_DIR", "")  # optional folder for the parity report
    if out and os.path.isdir(out):
        with open(os.path.join(out, f"parity_256_{dtype}.json"), "w") as f:
            json.dump(report, f)


# ---- fixed-point interior kernel: bit-exact against its integer model ---------------
LAP_CASES = [ND[0], ND[1],
             dict(shape=(64, 50), terms=[T("centered", 2, 4, axis=k, h=1 / 65,
                                           bc=("robin", (1.0, 0.5, 0.0), (1.0, 0.5, 0.0), 1)) for k in (1, 2)],
                  seed=8)]


def _wide_range(shape, seed):
    rng = np.random.default_rng(seed)
    u = rng.standard_normal(shape) * np.exp2(rng.integers(-40, 41, size=shape).astype(np.float64))
    u[rng.random(shape) < 0.05] = 0.0
    return np.asfortranarray(u)


@pytest.mark.parametrize("rows", [0, 3, 8])
@pytest.mark.parametrize("field", ["normal", "wide", "special"])
@pytest.mark.parametrize("case", LAP_CASES, ids=["3d-a4-robin", "3d-a2-dirichlet0", "2d-a4-robin"])
def test_fixed_point_kernel_against_integer_model(cuda, case, field, rows):
    """Interior points: bit for bit the integer model (tests/fx_model.py) and
    within 2 ulp of sum|c_k u_k| of the exact rational value; shell points,
    Inf/NaN fallbacks and the tile rows evaluated on the FP64 pipe
    (DEO_OPT_FX_FP64_ROWS: ((y mod 8) - rows * (floor(y/8) + z)) mod 8 < rows,
    0-based y, z): bit for bit the reference's order."""
    import itertools
    from fractions import Fraction
    import fx_model as FX
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    nt = len(shape)
    if field != "normal":
        u = _wide_range(shape, 11)
    if field == "special":
        u[(3,) * nt] = np.inf
        u[(shape[0] // 2,) + (4,) * (nt - 1)] = np.nan
    p = deo.Plan(A.terms(), shape, 0)
    ud = to_device(u)
    got_t, gen_t = deo.julia_array(shape), deo.julia_array(shape)
    p.set_option(deo.DEO_OPT_EXACT_SUMS, 4)  # the per-point fixed-point kernel
    p.set_option(deo.DEO_OPT_FX_FP64_ROWS, rows)
    assert p.get_option(deo.DEO_OPT_FX_FP64_ROWS) == rows
    p.apply(ud, got_t)
    assert p.kernels[0] == "k_lap_fx"
    p.set_option(deo.DEO_OPT_FAST_PATH, 0)
    p.apply(ud, gen_t)
    assert p.kernels == ("k_apply",)
    got, gen = to_host(got_t), to_host(gen_t)
    Lo = oterms[0][0]
    w = Lo.tables()[0][0, 0, :]
    H = len(w) // 2
    lo = max(Lo.bpc, H)
    inner = [range(lo, n - lo) for n in shape]
    interior = np.zeros(shape, bool)
    interior[tuple(slice(lo, n - lo) for n in shape)] = True
    # shell: the reference's order, bit for bit (the generic row-table kernel)
    assert np.array_equal(got[~interior], gen[~interior], equal_nan=True)
    worst = 0.0
    fallbacks = 0
    for idx in itertools.product(*inner):
        if (idx[1] % 8 - rows * (idx[1] // 8 + (idx[2] if nt == 3 else 0))) % 8 < rows:
            assert np.array_equal(got[idx], gen[idx], equal_nan=True), idx
            continue
        m = FX.fx_point(u, idx, w, H, nt)
        if m is None:
            fallbacks += 1
            assert np.array_equal(got[idx], gen[idx], equal_nan=True), idx
            continue
        assert got[idx] == m and np.signbit(got[idx]) == np.signbit(m), (idx, got[idx], m)
        if field != "special":
            val, scale = FX.exact_point(u, idx, w, H, nt)
            if scale:
                err = abs(Fraction(float(got[idx])) - val)
                worst = max(worst, float(err / Fraction(float(np.spacing(float(scale))))))
    assert worst <= 2.0, worst
    if rows == 0:
        assert (fallbacks > 0) == (field == "special")
    elif field != "special":
        assert fallbacks == 0
    assert deo.device_status() == 0


def test_fixed_point_kernel_not_used_for_wide_weight_ratios(cuda):
    """A 6th-order Laplacian (outer weight 1/90 of the centre's scale) fails the
    per-point fixed-point kernel's error-bound rule (and the block kernel's
    weight-width rule): the plan runs the per-offset exact-sum kernel."""
    case = dict(shape=(24, 20, 18), terms=[T("centered", 2, 6, axis=k, h=0.05, bc=("dirichlet0",))
                                           for k in (1, 2, 3)], seed=9)
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 0)
    p.set_option(deo.DEO_OPT_EXACT_SUMS, 4)
    out = deo.julia_array(shape)
    p.apply(to_device(u), out)
    assert p.kernels[0] == "k_lap_ens2"
    tol = 4 * np.spacing(O.abs_scale(oterms, u))
    assert (np.abs(to_host(out) - O.apply(oterms, u)) <= tol).all()


def test_launch_timing(cuda):
    A, oterms, u = build(ND[0])
    shape = tuple(ND[0]["shape"])
    p = deo.Plan(A.terms(), shape, 0)
    p.set_option(deo.DEO_OPT_LAUNCH_TIMING, 1)
    out = deo.julia_array(shape)
    p.apply(to_device(u), out)
    ms = p.launch_times()
    assert len(ms) == 2 and ms[0] > 0 and ms[1] >= 0
    p.set_option(deo.DEO_OPT_FAST_PATH, 0)
    p.apply(to_device(u), out)
    assert p.kernels == ("k_apply",) and len(p.launch_times()) == 1
    with pytest.raises(deo.DeoArgError):
        p.set_option(deo.DEO_OPT_EXACT_SUMS, 6)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("case", LAP_CASES + [ND[2], dict(ND[0], shape=(70, 45, 33))],
                         ids=["3d-a4-robin", "3d-a2-dirichlet0", "2d-a4-robin", "3d-periodic", "3d-odd"])
def test_shell_kernels_bitwise_equal_generic(cuda, case, dtype):
    """Reference-order interior (k_lap_q) with every shell kernel: the shell on
    a side stream beside the interior, and after it (lines / faces), equal the
    generic row-table kernel bit for bit, overwrite and accumulate."""
    import torch
    A, oterms, u = build(case, dtype=dtype)
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 0 if dtype == "f64" else 1)
    ud = to_device(u, dtype)
    base = to_device(np.asfortranarray(np.random.default_rng(4).standard_normal(shape)), dtype)
    p.set_option(deo.DEO_OPT_FAST_PATH, 0)
    ref_ow, ref_acc = deo.julia_array(shape, ud.dtype), base.clone()
    p.apply(ud, ref_ow)
    p.apply(ud, ref_acc, overwrite=False)
    p.set_option(deo.DEO_OPT_FAST_PATH, 1)
    p.set_option(deo.DEO_OPT_EXACT_SUMS, 0)
    seen = set()
    for conc in (1, 0):
        p.set_option(deo.DEO_OPT_CONCURRENT_SHELL, conc)
        o = deo.julia_array(shape, ud.dtype)
        p.apply(ud, o)
        seen.add(p.kernels[-1])
        assert torch.equal(o, ref_ow), (conc, p.kernels)
        a = base.clone()
        p.apply(ud, a, overwrite=False)
        assert torch.equal(a, ref_acc), (conc, p.kernels)
    # rows of 16-byte multiples take the TMA path (interior + shell kernel); others one register-queue kernel
    assert bool(seen & {"k_shell_lines", "k_face"}) == ((shape[0] * (8 if dtype == "f64" else 4)) % 16 == 0)
    assert deo.device_status() == 0


def test_pipelined_host_applies(cuda):
    """deo_apply_host_async over a sequence of host inputs: every result equals
    the device apply of the same input, bit for bit (two staging slots in
    flight, copies on their own streams)."""
    import torch
    A, oterms, u = build(ND[0])
    shape = tuple(ND[0]["shape"])
    p = deo.Plan(A.terms(), shape, 0)
    rng = np.random.default_rng(21)
    ins = [torch.from_numpy(np.asfortranarray(rng.standard_normal(shape)).ravel(order="F")).pin_memory()
           for _ in range(5)]
    outs = [torch.empty_like(t).pin_memory() for t in ins]
    for a, b in zip(ins, outs):
        p.apply_host_async(a, b)
    p.host_sync()
    for a, b in zip(ins, outs):
        ud = to_device(a.numpy().reshape(shape, order="F"))
        d = deo.julia_array(shape)
        p.apply(ud, d)
        assert torch.equal(d.permute(*reversed(range(len(shape)))).contiguous().view(-1).cpu(), b)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_default_path_accumulate_equals_overwrite_plus_base(cuda, dtype):
    """Default options (fixed-point interior for Float64, concurrent shell):
    overwrite=false adds the same values the overwriting apply writes."""
    import torch
    A, oterms, u = build(ND[0], dtype=dtype)
    shape = tuple(ND[0]["shape"])
    p = deo.Plan(A.terms(), shape, 0 if dtype == "f64" else 1)
    assert p.get_option(deo.DEO_OPT_CONCURRENT_SHELL)
    ud = to_device(u, dtype)
    base = to_device(np.asfortranarray(np.random.default_rng(8).standard_normal(shape)), dtype)
    ow = deo.julia_array(shape, ud.dtype)
    p.apply(ud, ow)
    acc = base.clone()
    p.apply(ud, acc, overwrite=False)
    assert torch.equal(acc, base + ow)
    assert deo.device_status() == 0


@pytest.mark.parametrize("dtype,sums", [("f64", 0), ("f64", 1), ("f32", 0)])
@pytest.mark.parametrize("case", [dict(ND[0], shape=(72, 45, 33)), ND[1], dict(ND[2], shape=(24, 20, 18)),
                                  LAP_CASES[2],
                                  dict(shape=(64, 40, 30), terms=[T("centered", 2, 6, axis=k, h=0.02,
                                                                    bc=("neumann", 0.3, -0.2, 1)) for k in (1, 2, 3)],
                                       seed=12)],
                         ids=["a4-robin", "a2-dirichlet0", "a4-periodic", "2d-a4-robin", "a6-neumann"])
def test_transposed_fast_path(cuda, case, dtype, sums):
    """deo_apply_adjoint on the TMA path (the interior kernel on the columns
    read only by band rows, k_shell_adj on the rest) against the generic
    transposed kernel: bit for bit in the reference's order (EXACT_SUMS=0;
    Float32), within the 4-ulp bar for the fixed-point interior; overwrite and
    accumulate; the same result whatever DEO_OPT_CONCURRENT_SHELL says (the
    shell runs after the interior: beside it, one CTA per SM, the column
    evaluator outlasted the interior)."""
    import torch
    A, oterms, u = build(case, dtype=dtype)
    shape = tuple(case["shape"])
    p = deo.Plan(A.terms(), shape, 0 if dtype == "f64" else 1)
    p.set_option(deo.DEO_OPT_EXACT_SUMS, sums)
    v = to_device(np.asfortranarray(np.random.default_rng(8).standard_normal(shape)), dtype)
    base = to_device(np.asfortranarray(np.random.default_rng(9).standard_normal(shape)), dtype)
    tdt = v.dtype
    p.set_option(deo.DEO_OPT_FAST_PATH, 0)
    ref, ref_acc = deo.julia_array(shape, tdt), base.clone()
    p.adjoint(v, ref)
    p.adjoint(v, ref_acc, overwrite=False)
    assert p.kernels == ("k_apply",)
    p.set_option(deo.DEO_OPT_FAST_PATH, 1)
    outs = {}
    for conc in (1, 0):
        p.set_option(deo.DEO_OPT_CONCURRENT_SHELL, conc)
        o = deo.julia_array(shape, tdt, fill=np.nan)
        p.adjoint(v, o)
        assert p.kernels[1] == "k_shell_adj" and p.kernels[0].startswith("k_lap_"), p.kernels
        a = base.clone()
        p.adjoint(v, a, overwrite=False)
        outs[conc] = (o, a)
        if dtype == "f32" or sums == 0:
            assert torch.equal(o, ref), conc
            assert torch.equal(a, ref_acc), conc
        else:
            r, g = to_host(ref), to_host(o)
            vh = to_host(v)
            # the transposed sum's scale: sum_i |A[i, j] v_i|, from the forward operator's abs scale of |v|
            scale = O.abs_scale(oterms, np.abs(vh))
            assert (np.abs(g - r) <= 4 * np.spacing(np.maximum(scale, np.abs(r))) + 1e-300).all()
    torch.cuda.synchronize()
    assert torch.equal(outs[1][0], outs[0][0]) and torch.equal(outs[1][1], outs[0][1])
    assert deo.device_status() == 0
