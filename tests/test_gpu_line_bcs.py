"""GPU: boundary conditions that differ per line (MultiDimBC{dim}(BCs::Array),
multi_dim_bc_operators.jl:91-93) against the oracle: forward applies in
Float64 (4 ulp of sum|c_k u_k|) and Float32, the adjoint against the oracle's
concretisation, and the batched kernel against the per-instance apply."""
import numpy as np
import pytest

import deo
import oracle as O
from cases import to_device, to_host

pytestmark = pytest.mark.gpu
H = 0.1


def _pools():
    dev = [deo.RobinBC((1.0, 2.0, 3.0), (0.0, -1.0, 2.0), H, 4), deo.PeriodicBC(), deo.DirichletBC(0.5, -0.25),
           deo.GeneralBC([0.3, 1.0, 0.2], [-0.1, 0.7, 0.4], H, 2)]
    orc = [O.robin((1.0, 2.0, 3.0), (0.0, -1.0, 2.0), H, 4), O.periodic(), O.dirichlet(0.5, -0.25),
           O.general([0.3, 1.0, 0.2], [-0.1, 0.7, 0.4], H, 2)]
    return dev, orc


def _problem(shape, line_axes, d=2, a=2, seed=0, kinds=4):
    """One centred term per axis; axes in line_axes get a seeded per-line mix of BCs, the others Robin."""
    rng = np.random.default_rng(seed)
    dev, orc = _pools()
    gs, oterms = [], []
    for ax in range(1, len(shape) + 1):
        n = shape[ax - 1]
        L = deo.CenteredDifference(d, a, H, n, axis=ax)
        Lo = O.centered(d, a, H, n, axis=ax)
        if ax in line_axes:
            perp = tuple(m for k, m in enumerate(shape) if k != ax - 1)
            pick = rng.integers(0, kinds, int(np.prod(perp)))
            arr = np.empty(perp, dtype=object)
            flat = arr.reshape(-1, order="F")
            for j, k in enumerate(pick):
                flat[j] = dev[k]
            arr = flat.reshape(perp, order="F")
            gs.append(L * deo.MultiDimBC(arr, dim=ax))
            oterms.append((Lo, orc[pick[0]], None, [orc[k] for k in pick]))
        else:
            gs.append(L * deo.MultiDimBC(dev[0], shape, ax))
            oterms.append((Lo, orc[0]))
    return deo.DiffEqOperatorCombination(gs), oterms


CASES = [((17, 13), {1}), ((17, 13), {2}), ((17, 13), {1, 2}), ((12, 10, 9), {1}), ((12, 10, 9), {3}),
         ((12, 10, 9), {1, 2, 3}), ((64, 48, 40), {2})]


@pytest.mark.parametrize("shape,axes", CASES)
@pytest.mark.parametrize("d,a", [(2, 2), (2, 4), (1, 4)])
def test_per_line_bcs_against_oracle(cuda, shape, axes, d, a):
    A, oterms = _problem(shape, axes, d, a, seed=len(shape) + d)
    rng = np.random.default_rng(7)
    u = np.asfortranarray(rng.standard_normal(shape))
    p = deo.Plan(A.terms(), shape, 0)
    out = deo.julia_array(shape)
    p.apply(to_device(u), out)
    assert p.kernels == ("k_apply",)  # per-line ghost maps take the generic evaluator
    ref = O.apply(oterms, u)
    scale = O.abs_scale(oterms, u)
    assert (np.abs(to_host(out) - ref) <= 4 * np.spacing(scale)).all()
    # accumulate
    base = np.asfortranarray(rng.standard_normal(shape))
    acc = to_device(base)
    p.apply(to_device(u), acc, overwrite=False)
    ref2 = O.apply(oterms, u, out=base.copy(order="F"), overwrite=False)
    assert (np.abs(to_host(acc) - ref2) <= 4 * np.spacing(scale + np.abs(base))).all()
    # Float32 against the Float64 oracle
    pf = deo.Plan(A.terms(), shape, 1)
    import torch
    of = deo.julia_array(shape, torch.float32)
    pf.apply(to_device(u, "f32"), of)
    u32 = u.astype(np.float32).astype(np.float64)
    ref32 = O.apply(oterms, u32)
    assert (np.abs(to_host(of) - ref32) <= 64 * 2.0 ** -24 * O.abs_scale(oterms, u32) + 1e-30).all()
    assert deo.device_status() == 0


@pytest.mark.parametrize("shape,axes", [((9, 7), {1}), ((9, 7), {1, 2}), ((6, 5, 4), {2}), ((6, 5, 4), {1, 3})])
def test_per_line_bcs_adjoint_against_concretisation(cuda, shape, axes):
    A, oterms = _problem(shape, axes, 2, 4, seed=11)
    Al, Ab = O.concretize_probe(oterms, shape)
    rng = np.random.default_rng(5)
    v = np.asfortranarray(rng.standard_normal(shape))
    p = deo.Plan(A.terms(), shape, 0)
    ub = deo.julia_array(shape)
    p.adjoint(to_device(v), ub)
    got = to_host(ub).ravel(order="F")
    ref = Al.T @ v.ravel(order="F")
    tol = 64 * np.finfo(np.float64).eps * (np.abs(Al).T @ np.abs(v.ravel(order="F")))
    assert np.all(np.abs(got - ref) <= tol + 1e-300)
    Dl, Db = p.concretize()
    assert np.allclose(Dl, Al, rtol=1e-12, atol=1e-12 * np.abs(Al).max())
    assert np.allclose(Db, Ab, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(Ab).max()))


def test_per_line_bcs_in_the_batched_kernel(cuda):
    import torch
    probs = [_problem((40, 30), {1}, 2, 4, seed=1), _problem((20, 18, 16), {2, 3}, 2, 2, seed=2),
             _problem((33, 29), {1, 2}, 1, 4, seed=3)]
    rng = np.random.default_rng(9)
    plans, us, outs, refs = [], [], [], []
    for (A, oterms), shape in zip(probs, [(40, 30), (20, 18, 16), (33, 29)]):
        p = deo.Plan(A.terms(), shape, 0)
        u = to_device(np.asfortranarray(rng.standard_normal(shape)))
        r = deo.julia_array(shape)
        p.apply(u, r)
        plans.append(p); us.append(u); refs.append(r); outs.append(deo.julia_array(shape, fill=np.nan))
    b = deo.Batch(list(zip(plans, us, outs)))
    b.run(use_graph=True)
    torch.cuda.synchronize()
    for o, r in zip(outs, refs):
        assert torch.equal(o, r)


def test_uniform_array_takes_the_fast_path(cuda):
    """An array holding one BC for every line is that BC on every line: the
    plan keeps the tiled fast path and gives the atomic BC's result bit for bit."""
    import torch
    shape = (64, 40, 24)
    Q = deo.RobinBC((1.0, 0.5, 0.0), (1.0, 0.5, 0.0), H, 1)
    arrs = []
    for ax in (1, 2, 3):
        perp = tuple(m for k, m in enumerate(shape) if k != ax - 1)
        arr = np.empty(perp, dtype=object)
        arr.reshape(-1)[:] = [Q] * int(np.prod(perp))
        arrs.append(deo.MultiDimBC(arr, dim=ax))
    Ls = [deo.CenteredDifference(2, 4, H, n, axis=k + 1) for k, n in enumerate(shape)]
    A1 = deo.DiffEqOperatorCombination([L * q for L, q in zip(Ls, arrs)])
    A2 = deo.DiffEqOperatorCombination([L * deo.MultiDimBC(Q, shape, k + 1) for k, L in enumerate(Ls)])
    u = to_device(np.asfortranarray(np.random.default_rng(4).standard_normal(shape)))
    o1, o2 = deo.julia_array(shape), deo.julia_array(shape)
    p1, p2 = deo.Plan(A1.terms(), shape, 0), deo.Plan(A2.terms(), shape, 0)
    p1.apply(u, o1)
    p2.apply(u, o2)
    assert p1.kernels == p2.kernels and p1.kernels[0] != "k_apply"
    assert torch.equal(o1, o2)
