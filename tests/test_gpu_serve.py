"""GPU: continuous-batching MOL server -- results equal alone and in a mix,
match the oracle's SSP-RK3, admission respects the HBM budget."""
import numpy as np
import pytest

import oracle as O
from deo.serve import Request, Server, poisson_requests

pytestmark = pytest.mark.gpu


def _oracle_solve(r: Request):
    terms = []
    for k, n in enumerate(r.shape):
        terms.append((O.centered(2, 2, 1.0 / (n + 1), n, axis=k + 1).scale(r.nu), O.dirichlet0()))
    terms.append((O.upwind(1, r.approx_order, 1.0 / (r.shape[0] + 1), r.shape[0], -r.c, axis=1), O.dirichlet0()))
    return O.ssprk3(terms, r.initial(), r.dt(), r.K)


def _clone(reqs):
    return [Request(shape=r.shape, nu=r.nu, c=r.c, K=r.K, want_grad=r.want_grad, seed=r.seed, arrival=r.arrival,
                    rid=r.rid) for r in reqs]


def test_alone_equals_mix_and_oracle(cuda):
    reqs = poisson_requests(24, 2000.0, seed=3, size_scale=0.05, k_range=(5, 40), grad_frac=0.3)
    mix = Server(hbm_budget_bytes=4e9)
    st = mix.run(_clone(reqs))
    assert st["completed"] == len(reqs)
    by_id = {r.rid: r for r in mix.done}
    # each request alone
    for r in reqs[:8]:
        s = Server(hbm_budget_bytes=4e9)
        s.run(_clone([r]))
        alone = s.done[0]
        m = by_id[r.rid]
        assert np.array_equal(alone.uT, m.uT), r.rid
        if r.want_grad:
            assert np.array_equal(alone.grad, m.grad), r.rid
    # against the oracle (SSP-RK3 restated), a few requests
    for r in reqs[:6]:
        ref = _oracle_solve(r)
        got = by_id[r.rid].uT
        assert np.allclose(got, ref, rtol=0, atol=1e-11 * r.K * max(1.0, np.abs(ref).max())), r.rid


def test_admission_budget_and_rejection(cuda):
    big = Request(shape=(400, 400), nu=0.01, c=0.5, K=3, seed=1)
    small = [Request(shape=(200,), nu=0.01, c=0.5, K=3, seed=i, arrival=0.0, rid=i + 1) for i in range(5)]
    budget = big.bytes_needed() - 1
    s = Server(hbm_budget_bytes=budget)
    st = s.run([big] + small)
    assert st["rejected"] == 1 and st["completed"] == 5
    assert [r for r in s.done if r.rejected][0] is big
    # a budget that fits only two small requests at a time still serves all of them
    s2 = Server(hbm_budget_bytes=2 * small[0].bytes_needed())
    for r in small:
        r.uT = None
    st2 = s2.run(_clone(small))
    assert st2["completed"] == 5 and st2["rebuilds"] >= 3


def test_gradient_matches_single_solve_adjoint(cuda):
    import torch
    import deo
    from deo.serve import advection_diffusion
    r = Request(shape=(24, 20), nu=0.03, c=-0.7, K=15, want_grad=True, seed=5)
    s = Server()
    s.run([r])
    A = advection_diffusion(r.shape, r.nu, r.c)
    u0 = deo.julia_array(r.shape)
    u0.copy_(torch.from_numpy(r.initial()))
    uT, g = deo.autodiff.ssprk3_grad_norm2(A, u0, r.dt(), r.K)
    assert np.array_equal(uT.cpu().numpy(), r.uT)
    assert np.array_equal(g.cpu().numpy(), r.grad)
