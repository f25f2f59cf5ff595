"""GPU: the benchmark configurations against the oracle at their real sizes.

* 2-D non-uniform 2048^2 grid (centred d1/d2 a6 on both axes, upwind d1 a3
  with the field a(x,y) = cos(2 pi x) sin(2 pi y), GeneralBC): every operator
  alone and the fused 5-term sum, within 4 ulp of sum|c_k u_k|.
* Batched instances drawn as the batched workload draws them, plus instances
  at the top of each size range (1-D N = 65536, 2-D 1024 x 1024), graded and
  uniform grids, Robin and Dirichlet: the one-launch batched forward pass
  against the oracle; the batched adjoint pass against the per-instance
  adjoint (bit for bit) and by a finite-difference gradient check of
  f(u) = <v, A u> on a random cotangent v and direction w.
* Method-of-lines solves of the serving workload's real sizes (1-D 10^6,
  2-D 2048^2, 3-D 256^3, ...), served together: each against the oracle's
  SSP-RK3 and equal to the same request served alone.
"""
import json
import os

import numpy as np
import pytest

import bench
import deo
import oracle as O
from cases import to_device, to_host

pytestmark = pytest.mark.gpu
NTHREADS = os.cpu_count() or 1


def _report(name, data):
    """Writes the figures to DEO_REPORT_DIR/<name>.json when that folder exists."""
    out = os.environ.get("DEO_REPORT_DIR", "")
    if out and os.path.isdir(out):
        with open(os.path.join(out, name + ".json"), "w") as f:
            json.dump(data, f, indent=1)


def _ulps(got, ref, scale):
    return float((np.abs(got - ref) / np.spacing(scale)).max())


def test_nonuniform_2048_fused_and_per_operator_against_oracle(cuda):
    import torch
    n = 2048
    _, (al, ar, dx) = bench.nonuniform2d_ops(n)
    u, a = bench.nonuniform2d_inputs(n, dx)
    fdev = deo.julia_array((n, n))
    fdev.copy_(torch.from_numpy(a))
    ops, _ = bench.nonuniform2d_ops(n, fdev)
    q = O.general(al, ar, dx, 1)
    up = O.upwind(1, 3, dx, n, axis=1)
    up.set_coefficients(np.ones(n), 0)  # one operator per line, coefficient a(:, y_j)
    oterms = [(O.centered(1, 6, dx, n, axis=1), q), (O.centered(1, 6, dx, n, axis=2), q),
              (O.centered(2, 6, dx, n, axis=1), q), (O.centered(2, 6, dx, n, axis=2), q), (up, q, a)]
    ud = to_device(u)
    worst = {}
    for name, g, t in zip(["D1x", "D1y", "D2x", "D2y", "Upwind1x_field"], ops, oterms):
        p = deo.plan_for([g], (n, n), 0)
        out = deo.julia_array((n, n))
        p.apply(ud, out)
        ref = O.apply([t], u, nthreads=NTHREADS)
        worst[name] = _ulps(to_host(out), ref, O.abs_scale([t], u))
    p = deo.plan_for(ops, (n, n), 0)
    out = deo.julia_array((n, n))
    p.apply(ud, out)
    ref = O.apply(oterms, u, nthreads=NTHREADS)
    worst["fused"] = _ulps(to_host(out), ref, O.abs_scale(oterms, u))
    # the same terms with D1 + D2 merged per axis (DEO_PLAN_MERGE_TERMS): against the oracle's
    # term-by-term sums, same bar
    pm = deo.plan_for(ops, (n, n), 0, merge_terms=True)
    assert pm.evaluated_terms == 3
    pm.apply(ud, out)
    worst["fused_merged"] = _ulps(to_host(out), ref, O.abs_scale(oterms, u))
    # and the upwind term's field factored out of its tap sum (DEO_PLAN_FACTOR_FIELD)
    pf = deo.plan_for(ops, (n, n), 0, merge_terms=True, factor_field=True)
    pf.apply(ud, out)
    worst["fused_merged_factored"] = _ulps(to_host(out), ref, O.abs_scale(oterms, u))
    assert deo.device_status() == 0
    _report("parity_nonuniform2d_2048", {"max_ulp_of_scale": worst})
    assert max(worst.values()) <= 4.0, worst


def _oracle_terms(spec):
    shape, d, a, graded, robin = spec
    out = []
    for ax, n in enumerate(shape):
        dx = bench.batch_grid(n, graded)
        bc = O.robin(bench.ROBIN_L, bench.ROBIN_R, dx, 1) if robin else O.dirichlet(*bench.DIRICHLET_LR)
        out.append((O.centered(d, a, dx, n, axis=ax + 1), bc))
    return out


def _specs():
    specs = bench.batch_specs(4096)[:40]
    # the top of each size range, graded and uniform grids, Robin and Dirichlet
    specs += [((65536,), 4, 8, True, True), ((65536,), 1, 2, False, False), ((65536,), 3, 6, True, False),
              ((1024, 1024), 2, 6, True, True), ((1024, 1024), 4, 4, False, True), ((1024, 1000), 1, 8, True, False)]
    return specs


def test_batched_forward_adjoint_and_fd_gradient_full_range(cuda):
    import torch
    specs = _specs()
    rng = np.random.default_rng(12)
    plans, us, outs, vs, ubars, oterms, hosts = [], [], [], [], [], [], []
    for spec in specs:
        shape = spec[0]
        p = deo.Plan(bench.batch_terms(spec), shape, 0)
        u = np.asfortranarray(rng.standard_normal(shape))
        v = np.asfortranarray(rng.standard_normal(shape))
        plans.append(p); hosts.append((u, v)); oterms.append(_oracle_terms(spec))
        us.append(to_device(u)); vs.append(to_device(v))
        outs.append(deo.julia_array(shape, fill=np.nan)); ubars.append(deo.julia_array(shape, fill=np.nan))
    fwd = deo.Batch(list(zip(plans, us, outs)))
    adj = deo.Batch(list(zip(plans, vs, ubars)), adjoint=True)
    fwd.run(use_graph=True)
    adj.run(use_graph=True)
    torch.cuda.synchronize()
    assert deo.device_status() == 0
    worst = 0.0
    for (u, v), o, t, spec in zip(hosts, outs, oterms, specs):
        ref = O.apply(t, u, nthreads=NTHREADS)
        w = _ulps(to_host(o), ref, O.abs_scale(t, u))
        assert w <= 4.0, (spec, w)
        worst = max(worst, w)
    _report("parity_batched", {"instances": len(specs), "points": int(sum(np.prod(sp[0]) for sp in specs)),
                               "forward_max_ulp_of_scale": worst})
    # the batched adjoint equals the per-instance transposed apply in the reference's tap order bit for
    # bit (the batched kernel keeps that order; a Laplacian-type instance's own adjoint may take the
    # TMA path with the fixed-point interior, within the bar instead)
    for p, v, ub in zip(plans, vs, ubars):
        one = deo.julia_array(tuple(v.shape))
        p.set_option(deo.DEO_OPT_EXACT_SUMS, 0)
        p.adjoint(v, one)
        p.set_option(deo.DEO_OPT_EXACT_SUMS, 1)
        assert torch.equal(one, ub)
    # finite-difference gradient of f(u) = <v, A u> (A affine: the BC offsets cancel) on a random
    # direction w, through the batched forward pass, against <A^T v, w> from the batched adjoint
    ws = [to_device(np.asfortranarray(rng.standard_normal(tuple(u.shape)))) for u in us]
    eps = 0.5

    def shifted(u, w, s):
        t = deo.julia_array(tuple(u.shape))
        t.copy_(u + s * w)
        return t
    up = [shifted(u, w, eps) for u, w in zip(us, ws)]
    um = [shifted(u, w, -eps) for u, w in zip(us, ws)]
    op = [deo.julia_array(tuple(u.shape)) for u in us]
    om = [deo.julia_array(tuple(u.shape)) for u in us]
    deo.Batch(list(zip(plans, up, op))).run(use_graph=False)
    deo.Batch(list(zip(plans, um, om))).run(use_graph=False)
    torch.cuda.synchronize()
    for spec, v, w, a_p, a_m, ub in zip(specs, vs, ws, op, om, ubars):
        fd = float(((v * a_p).sum() - (v * a_m).sum()) / (2 * eps))
        ad = float((ub * w).sum())
        scale = float((v.abs() * (a_p.abs() + a_m.abs())).sum()) / (2 * eps)
        assert abs(fd - ad) <= 1e-12 * scale + 1e-300, (spec, fd, ad, scale)


def _serve_oracle(r):
    terms = []
    for k, n in enumerate(r.shape):
        terms.append((O.centered(2, 2, 1.0 / (n + 1), n, axis=k + 1).scale(r.nu), O.dirichlet0()))
    terms.append((O.upwind(1, r.approx_order, 1.0 / (r.shape[0] + 1), r.shape[0], -r.c, axis=1), O.dirichlet0()))
    return O.ssprk3(terms, r.initial(), r.dt(), r.K, nthreads=NTHREADS)


def test_served_solves_at_full_size_against_oracle(cuda):
    from deo.serve import Request, Server
    shapes = [(1_000_000,), (3000,), (2048, 2048), (64, 64), (256, 256, 256), (32, 32, 32), (97, 80, 71)]
    reqs = [Request(shape=s, nu=float(0.001 + 0.099 * (k / len(shapes))), c=float(-1 + 2 * k / len(shapes)),
                    K=10 + 3 * (k % 3), seed=100 + k, rid=k + 1, want_grad=(k % 3 == 1)) for k, s in enumerate(shapes)]
    mix = Server(hbm_budget_bytes=120e9)
    st = mix.run(reqs)
    assert st["completed"] == len(reqs)
    for r in reqs:
        ref = _serve_oracle(r)
        assert np.allclose(r.uT, ref, rtol=0, atol=1e-11 * r.K * max(1.0, np.abs(ref).max())), r.shape
    # alone equals the mix (a large and a small request)
    for k in (2, 3):
        r = reqs[k]
        alone = Request(shape=r.shape, nu=r.nu, c=r.c, K=r.K, seed=r.seed, rid=r.rid, want_grad=r.want_grad)
        Server(hbm_budget_bytes=120e9).run([alone])
        assert np.array_equal(alone.uT, r.uT)
        if r.want_grad:
            assert np.array_equal(alone.grad, r.grad)
