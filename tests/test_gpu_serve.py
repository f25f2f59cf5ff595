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
    assert st2["rounds"] >= 3


def test_gradient_matches_single_solve_adjoint(cuda):
    import torch
    import deo
    from deo.serve import advection_diffusion
    r = Request(shape=(24, 20), nu=0.03, c=-0.7, K=15, want_grad=True, seed=5)
    s = Server(merge_terms=False)  # the plans of the single-solve path below
    s.run([r])
    A = advection_diffusion(r.shape, r.nu, r.c)
    u0 = deo.julia_array(r.shape)
    u0.copy_(torch.from_numpy(r.initial()))
    uT, g = deo.autodiff.ssprk3_grad_norm2(A, u0, r.dt(), r.K)
    assert np.array_equal(uT.cpu().numpy(), r.uT)
    assert np.array_equal(g.cpu().numpy(), r.grad)


def test_cancel_pending_and_running(cuda):
    """A request cancelled before admission and one cancelled while it runs
    leave; the others finish with the results they have alone."""
    reqs = [Request(shape=(300, 200), nu=0.02, c=0.3, K=400, seed=k, rid=k + 1) for k in range(3)]
    reqs.append(Request(shape=(5000,), nu=0.01, c=-0.5, K=50, seed=9, rid=9))
    budget = 2 * reqs[0].bytes_needed() + reqs[3].bytes_needed()  # the third 2-D request waits
    s = Server(hbm_budget_bytes=budget, max_steps_per_round=8)
    state = {"n": 0}

    def on_tick(srv, now):
        state["n"] += 1
        if state["n"] == 2:
            srv.cancel(reqs[2])   # still pending (no memory for it yet)
            srv.cancel(reqs[0])   # running
    st = s.run(reqs, on_tick=on_tick)
    assert st["cancelled"] == 2
    assert reqs[0].rejected == "cancelled" and reqs[2].rejected == "cancelled"
    for r in (reqs[1], reqs[3]):
        assert not r.rejected
        alone = _clone([r])[0]
        Server(hbm_budget_bytes=budget).run([alone])
        assert np.array_equal(alone.uT, r.uT)


def test_injected_allocation_failure(cuda):
    """An admission whose device allocation fails reports DEO_ERR_OOM for that
    request; the server goes on with the others."""
    reqs = [Request(shape=(64, 48), nu=0.02, c=0.3, K=12, seed=k, rid=k + 1) for k in range(4)]
    s = Server(hbm_budget_bytes=1e9, inject_alloc_failures=1)
    st = s.run(reqs)
    assert st["failed"] == 1 and st["completed"] == 3
    bad = [r for r in reqs if r.rejected]
    assert len(bad) == 1 and bad[0].rejected.startswith("admission failed")
    for r in reqs:
        if not r.rejected:
            assert np.allclose(r.uT, _oracle_solve(r), rtol=0, atol=1e-11 * r.K * max(1.0, np.abs(r.uT).max()))


def test_serve_c_abi_poll_states(cuda):
    """deo_serve_* through the C ABI: NOT_READY until pumped to completion,
    then the result once; unknown ids are refused; oversized requests are
    rejected at submission."""
    import ctypes as C
    import torch
    import deo
    from deo import _lib as L
    from deo.serve import advection_diffusion
    lib = deo.lib()
    srv = C.c_void_p()
    assert lib.deo_serve_create(1 << 28, 0, 4, C.byref(srv)) == 0  # 256 MiB
    r = Request(shape=(40, 30), nu=0.05, c=0.4, K=10, seed=3)
    A = advection_diffusion(r.shape, r.nu, r.c)
    p = deo.Plan(A.terms(), r.shape, 0)
    u0 = r.initial()
    q = L.Request(p.handle, C.c_void_p(u0.ctypes.data), r.K, r.dt(), 0)
    rid = C.c_int64()
    assert lib.deo_serve_submit(srv, C.byref(q), C.byref(rid)) == 0
    out = np.empty(r.shape, order="F")
    assert lib.deo_serve_poll(srv, rid.value, C.c_void_p(out.ctypes.data), None, None) == 7  # NOT_READY
    lat = C.c_double()
    for _ in range(100000):
        assert lib.deo_serve_pump(srv) == 0
        st = lib.deo_serve_poll(srv, rid.value, C.c_void_p(out.ctypes.data), None, C.byref(lat))
        if st != 7:
            break
    assert st == 0 and lat.value > 0
    assert np.allclose(out, _oracle_solve(r), rtol=0, atol=1e-11 * r.K * max(1.0, np.abs(out).max()))
    assert lib.deo_serve_poll(srv, rid.value, None, None, None) == 2  # forgotten after collection
    big = deo.Plan(advection_diffusion((4096, 4096), 0.01, 0.1).terms(), (4096, 4096), 0)
    zeros = np.zeros((4096, 4096), order="F")
    qb = L.Request(big.handle, C.c_void_p(zeros.ctypes.data), 3, 1e-6, 0)
    assert lib.deo_serve_submit(srv, C.byref(qb), C.byref(rid)) == 8  # REJECTED: larger than the budget
    torch.cuda.synchronize()
    lib.deo_serve_destroy(srv)
