"""Builds matching operator pairs: the product (deo, on the GPU) and the CPU
oracle, from one case spec, plus seeded inputs.  Shared by the parity tests."""
from __future__ import annotations

import numpy as np

import deo
import oracle as O


def nonuniform_dx(n: int, seed: int = 0, amp: float = 0.5) -> np.ndarray:
    """dx_i = h(1 + amp sin(2 pi i / N)) normalised to sum to 1 (len+1 entries)."""
    i = np.arange(n + 1)
    dx = (1.0 + amp * np.sin(2 * np.pi * i / (n + 1)))
    return dx / dx.sum()


def make_bc(spec, dx):
    kind = spec[0]
    if kind == "dirichlet0":
        return deo.Dirichlet0BC(), O.dirichlet0()
    if kind == "dirichlet":
        return deo.DirichletBC(spec[1], spec[2]), O.dirichlet(spec[1], spec[2])
    if kind == "neumann":
        return deo.NeumannBC((spec[1], spec[2]), dx, spec[3]), O.neumann((spec[1], spec[2]), dx, spec[3])
    if kind == "robin":
        return deo.RobinBC(spec[1], spec[2], dx, spec[3]), O.robin(spec[1], spec[2], dx, spec[3])
    if kind == "general":
        return deo.GeneralBC(spec[1], spec[2], dx, spec[3]), O.general(spec[1], spec[2], dx, spec[3])
    if kind == "periodic":
        return deo.PeriodicBC(), O.periodic()
    raise ValueError(kind)


def make_term(t, shape, rng):
    """t: dict(kind, d, a, axis, grid ('uniform'|'nonuniform'), h, coeff, offside, bc)."""
    ax = t.get("axis", 1)
    n = shape[ax - 1]
    if t.get("grid", "uniform") == "uniform":
        dx = t.get("h", 1.0 / (n + 1))
    else:
        dx = nonuniform_dx(n)
    coeff = t.get("coeff", None)
    field = None
    cvec = None
    if isinstance(coeff, str) and coeff == "vector":
        cvec = rng.uniform(-1.0, 1.0, n) if t["kind"] == "upwind" else rng.uniform(0.5, 1.5, n)
    elif isinstance(coeff, str) and coeff == "field":
        field = rng.uniform(-1.0, 1.0, shape) if t["kind"] == "upwind" else rng.uniform(0.5, 1.5, shape)
        field = np.asfortranarray(field)
    elif coeff is not None:
        cvec = coeff
    off = t.get("offside", 0)
    if t["kind"] == "centered":
        P = deo.CenteredDifference(t["d"], t["a"], dx, n, 1 if cvec is None else cvec, axis=ax)
        Q = O.centered(t["d"], t["a"], dx, n, cvec, axis=ax)
    else:
        P = deo.UpwindDifference(t["d"], t["a"], dx, n, 1 if cvec is None else cvec, offside=off, axis=ax)
        Q = O.upwind(t["d"], t["a"], dx, n, 1.0 if cvec is None else cvec, offside=off, axis=ax)
    if field is not None:
        # a field is one operator per line built from a coefficient Vector:
        # coeff_func is not a Number, so no coeff_func-sign branch applies
        Q.set_coefficients(np.ones(n), 0)
    bcp, bco = make_bc(t.get("bc", ("dirichlet0",)), dx)
    return P, Q, bcp, bco, field


def build(case, dtype="f64", device="cuda"):
    """Returns (A_gpu (combination of L*Q), oracle_terms, u numpy (Fortran), fields numpy)."""
    import torch
    rng = np.random.default_rng(case.get("seed", 0))
    shape = tuple(case["shape"])
    nd = len(shape)
    ghosts, oterms = [], []
    tdt = torch.float64 if dtype == "f64" else torch.float32
    for t in case["terms"]:
        P, Qo, bcp, bco, field = make_term(t, shape, rng)
        if nd == 1:
            qp = bcp
        else:
            qp = deo.MultiDimDirectionalBC(bcp, t.get("axis", 1), shape)
        if field is not None:
            ftens = deo.julia_array(shape, tdt, device)
            ftens.copy_(torch.from_numpy(np.asarray(field, dtype=np.float64)).to(device=device, dtype=tdt))
            g = deo.with_field(P, ftens) * qp
            g._field_host = field
        else:
            g = P * qp
        ghosts.append(g)
        oterms.append((Qo, bco, field))
    A = deo.DiffEqOperatorCombination(ghosts)
    u = np.asfortranarray(rng.standard_normal(shape))
    return A, oterms, u


def to_device(u: np.ndarray, dtype="f64"):
    import torch
    tdt = torch.float64 if dtype == "f64" else torch.float32
    t = deo.julia_array(u.shape, tdt, "cuda")
    t.copy_(torch.from_numpy(np.asarray(u, dtype=np.float64)).to("cuda", tdt))
    return t


def to_host(t) -> np.ndarray:
    return np.asfortranarray(t.detach().to("cpu", dtype=__import__("torch").float64).numpy())
