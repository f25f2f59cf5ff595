"""GPU parity on seeded random combinations of the path's parameters: 1-3
dimensions, 1-3 terms on random axes, centred and upwind operators (offside
included), uniform and non-uniform grids, scalar / vector / field
coefficients, every boundary condition kind, overwrite and accumulate, and
sizes down to the smallest the operators accept.  Each case against the
oracle at the 4-ulp-of-sum|c_k u_k| bar (the cases of test_gpu_parity.py, but
drawn at random to reach combinations the hand-written lists do not)."""
import numpy as np
import pytest

from test_gpu_parity import assert_parity, run_case

pytestmark = pytest.mark.gpu


def random_case(seed: int) -> dict:
    rng = np.random.default_rng(1000 + seed)
    nd = int(rng.choice([1, 1, 2, 2, 3]))
    nterms = int(rng.integers(1, 4)) if nd > 1 else int(rng.integers(1, 3))
    terms = []
    need = 0
    for _ in range(nterms):
        axis = int(rng.integers(1, nd + 1))
        if rng.random() < 0.6:
            d, a = int(rng.integers(1, 5)), int(rng.choice([2, 4, 6]))
            t = dict(kind="centered", d=d, a=a)
        else:
            d, a = int(rng.integers(1, 3)), int(rng.integers(1, 4))
            t = dict(kind="upwind", d=d, a=a, offside=int(rng.integers(0, (d + a - 1) // 2 + 1)))
        t["axis"] = axis
        t["grid"] = "nonuniform" if rng.random() < 0.35 else "uniform"
        r = rng.random()
        if r < 0.25:
            t["coeff"] = "vector"
        elif r < 0.4 and nd > 1:
            t["coeff"] = "field"
        elif r < 0.55:
            t["coeff"] = float(rng.uniform(-2.0, 2.0)) if t["kind"] == "upwind" else float(rng.uniform(0.3, 2.0))
        b = rng.random()
        al = (float(rng.uniform(0.5, 1.5)), float(rng.uniform(0.1, 1.0)), float(rng.uniform(-1, 1)))
        ar = (float(rng.uniform(0.5, 1.5)), float(rng.uniform(0.1, 1.0)), float(rng.uniform(-1, 1)))
        if b < 0.2:
            t["bc"] = ("dirichlet0",)
        elif b < 0.35:
            t["bc"] = ("dirichlet", al[2], ar[2])
        elif b < 0.5:
            t["bc"] = ("neumann", al[2], ar[2], int(rng.integers(1, 4)))
        elif b < 0.75:
            t["bc"] = ("robin", al, ar, int(rng.integers(1, 4)))
        elif b < 0.9:
            t["bc"] = ("general", (float(rng.uniform(-1, 1)), 1.0, float(rng.uniform(0.1, 1.0))),
                       (float(rng.uniform(-1, 1)), 1.0, float(rng.uniform(0.1, 1.0))), 2)
        else:
            t["bc"] = ("periodic",)
        need = max(need, 2 * (d + a) + 2)
        terms.append(t)
    lo = need
    hi = {1: 160, 2: 48, 3: 24}[nd]
    shape = tuple(int(rng.integers(lo, max(lo, hi) + 1)) for _ in range(nd))
    return dict(shape=shape, terms=terms, seed=seed)


NCASES = 400
CASES = [random_case(s) for s in range(NCASES)]


@pytest.mark.parametrize("case", CASES, ids=[f"fuzz{s}" for s in range(NCASES)])
def test_fuzz(cuda, case):
    assert_parity(case, overwrite=(case["seed"] % 3 != 0))


@pytest.mark.parametrize("case", CASES[::8], ids=[f"fuzz{s}" for s in range(0, NCASES, 8)])
def test_fuzz_float32(cuda, case):
    """Float32 applies against the Float64 oracle: a few units of 2^-24 of
    sum|c_k u_k| (Float32 tables and arithmetic)."""
    got, ref, scale = run_case(case, "f32")
    rel = np.abs(got - ref) / np.maximum(scale, 1e-300)
    assert rel.max() < 64 * 2.0 ** -24, rel.max()


def _small(case):
    """The case on a shape small enough for a dense concretisation (<= 4096 points)."""
    shape = list(case["shape"])
    while np.prod(shape) > 4096:
        k = int(np.argmax(shape))
        need = max(2 * (t["d"] + t["a"]) + 2 for t in case["terms"])
        if shape[k] - 1 < need:
            return None
        shape[k] -= 1
    return dict(case, shape=tuple(shape))


ADJ = [c for c in (_small(c) for c in CASES[1::5]) if c is not None]


@pytest.mark.parametrize("case", ADJ, ids=[f"adj{c['seed']}" for c in ADJ])
def test_fuzz_adjoint(cuda, case):
    """The adjoint kernel against the transpose of the oracle's concretisation
    (64 eps of |A_l|^T |v|), and the device concretisation against it."""
    import deo
    import oracle as O
    from cases import build, to_device, to_host
    A, oterms, u = build(case)
    shape = tuple(case["shape"])
    Al, Ab = O.concretize_probe(oterms, shape)
    v = np.asfortranarray(np.random.default_rng(case["seed"]).standard_normal(shape))
    p = deo.plan_for(A.terms(), shape, 0)
    ub = deo.julia_array(shape)
    p.adjoint(to_device(v), ub)
    got = to_host(ub).ravel(order="F")
    ref = Al.T @ v.ravel(order="F")
    scale = np.abs(Al).T @ np.abs(v.ravel(order="F"))
    assert np.all(np.abs(got - ref) <= 64 * np.finfo(float).eps * scale + 1e-300)
    Dl, Db = p.concretize()
    assert np.allclose(Dl, Al, rtol=1e-12, atol=1e-12 * np.abs(Al).max())
