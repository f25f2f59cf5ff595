"""The reference's SimpleDifferentialOperators examples
(test/DerivativeOperators/BasicSDOExamples.jl): known-answer matrices of
`Array(L*Q)[1]` for upwind and centred operators with Neumann0BC and RobinBC,
scalar and per-point (state-dependent drift) coefficients, and the value
functions solved from them.

Each case is concretised three ways: the oracle's `Array(L) * Q_L`, the
library's host concretisation `(L*Q).array()`, and (GPU) the plan's device
concretisation by unit probes `deo.concretize`.  The reference compares with
`isapprox`: `norm(x - y) <= sqrt(eps) * max(norm(x), norm(y))`.
"""
import numpy as np
import pytest

import deo
import oracle as O

RTOL = np.sqrt(np.finfo(float).eps)
M = 3
XBAR = np.linspace(0.0, 1.0, M + 2)
X = XBAR[1:-1]
DX = X[1] - X[0]
SIGMA, RHO, S = 0.1, 0.05, 3.0


def _approx(x, y):
    x, y = np.asarray(x, float), np.asarray(y, float)
    return np.linalg.norm(x - y) <= RTOL * max(np.linalg.norm(x), np.linalg.norm(y))


def _oracle_LQ(op, bc):
    QL, Qb = bc.array(M)
    A = op.array()
    return A @ QL, A @ Qb


# Each case: terms as (kind, coeff, scale) -- UpwindDifference(1, 1, dx, M, coeff) or
# CenteredDifference(2, 2, dx, M), times the scalar `scale` (None: unscaled) -- summed
# after `* Q`; the BC; the expected Lx = sum Array(s*L*Q)[1], L_bc = rho*I - Lx and
# v = L_bc \ x.^2; and expected single-operator parts.
NEG, POS = -0.1, 0.1
CASES = {
    # BasicSDOExamples.jl:23-58, constant negative drift, reflecting barriers
    "negative_drift": dict(
        terms=[("upwind", 1.0, NEG), ("centered", None, SIGMA ** 2 / 2)], bc=("neumann0",),
        Lx=[[-0.08, 0.08, 0.0], [0.48, -0.56, 0.08], [0.0, 0.48, -0.48]],
        L_bc=[[0.13, -0.08, 0.0], [-0.48, 0.61, -0.08], [0.0, -0.48, 0.53]],
        v=[1.9182649086005406, 2.3359304764758773, 3.1768804315253277],
        parts={"L1m": ([("upwind", -1.0, None)], [[0.0, 0.0, 0.0], [-4.0, 4.0, 0.0], [0.0, -4.0, 4.0]]),
               "L2": ([("centered", None, None)], [[-16.0, 16.0, 0.0], [16.0, -32.0, 16.0], [0.0, 16.0, -16.0]])}),
    # :73-100, constant positive drift
    "positive_drift": dict(
        terms=[("upwind", 1.0, POS), ("centered", None, SIGMA ** 2 / 2)], bc=("neumann0",),
        Lx=[[-0.48, 0.48, 0.0], [0.08, -0.56, 0.48], [0.0, 0.08, -0.08]],
        L_bc=[[0.53, -0.48, 0.0], [-0.08, 0.61, -0.48], [0.0, -0.08, 0.13]],
        v=[8.855633802816902, 9.647887323943664, 10.264084507042257],
        parts={"L1p": ([("upwind", 1.0, None)], [[-4.0, 4.0, 0.0], [0.0, -4.0, 4.0], [0.0, 0.0, 0.0]])}),
    # :117-151, state-dependent drift mu(x) = -x; Lx = L1 - sigma^2/2 L2
    "state_dependent_drift": dict(
        terms=[("upwind", -X, None), ("centered", None, -SIGMA ** 2 / 2)], bc=("neumann0",),
        Lx=[[0.08, -0.08, 0.0], [1.92, -1.84, -0.08], [0.0, 2.92, -2.92]],
        L_bc=[[-0.03, 0.08, 0.0], [-1.92, 1.89, 0.08], [0.0, -2.92, 2.97]],
        v=[1.1027342984846056, 1.194775361931727, 1.3640552379934825],
        parts={"L1": ([("upwind", -X, None)], [[0.0, 0.0, 0.0], [2.0, -2.0, 0.0], [0.0, 3.0, -3.0]])}),
    # :174-209, absorbing lower barrier: RobinBC((1, 0, S), (0, 1, 0), dx, 1), drift mu = -0.1
    "absorbing_bc": dict(
        terms=[("upwind", NEG, None), ("centered", None, SIGMA ** 2 / 2)],
        bc=("robin", (1.0, 0.0, S), (0.0, 1.0, 0.0)),
        Lx=[[-0.56, 0.08, 0.0], [0.48, -0.56, 0.08], [0.0, 0.48, -0.48]],
        L_bc=[[0.61, -0.08, 0.0], [-0.48, 0.61, -0.08], [0.0, -0.48, 0.53]],
        v=[0.2085953844248779, 0.8092898062396943, 1.7942624660284021],
        parts={"L2": ([("centered", None, None)], [[-32.0, 16.0, 0.0], [16.0, -32.0, 16.0], [0.0, 16.0, -16.0]])}),
    # :235-277, the Kolmogorov forward equation with mixed (Robin) barriers
    "kfe": dict(
        terms=[("upwind", -NEG, None), ("centered", None, SIGMA ** 2 / 2)],
        bc=("robin", (-2 * NEG / SIGMA ** 2, 1.0, 0.0), (-2 * NEG / SIGMA ** 2, 1.0, 0.0)),
        Lx=[[-0.58, 0.48, 0.0], [0.08, -0.56, 0.48], [0.0, 0.08, -0.48]],
        L_bc=None, v=None,
        parts={"L2s": ([("centered", None, SIGMA ** 2 / 2)],
                       [[-0.18, 0.08, 0.0], [0.08, -0.16, 0.08], [0.0, 0.08, -0.1466666666666667]])}),
}


def _bcs(spec):
    if spec[0] == "neumann0":
        return O.neumann0(DX, 1), deo.Neumann0BC(DX, 1)
    return O.robin(spec[1], spec[2], DX, 1), deo.RobinBC(spec[1], spec[2], DX, 1)


def _ops(term):
    kind, coeff, scale = term
    if kind == "upwind":
        o = O.upwind(1, 1, DX, M, coeff)
        h = deo.UpwindDifference(1, 1, DX, M, coeff)
    else:
        o = O.centered(2, 2, DX, M)
        h = deo.CenteredDifference(2, 2, DX, M)
    if scale is not None:
        o.scale(scale)
        h = scale * h
    return o, h


def _sum_oracle(terms, bc):
    A = np.zeros((M, M))
    for t in terms:
        A = A + _oracle_LQ(_ops(t)[0], bc)[0]
    return A


def _sum_host(terms, bc):
    A = np.zeros((M, M))
    for t in terms:
        A = A + (_ops(t)[1] * bc).array()[0]
    return A


@pytest.mark.parametrize("name", list(CASES))
def test_sdo_example_concretisations(name):
    c = CASES[name]
    qo, qh = _bcs(c["bc"])
    for via in (_sum_oracle(c["terms"], qo), _sum_host(c["terms"], qh)):
        assert _approx(via, c["Lx"]), via
        if c["L_bc"] is not None:
            L_bc = RHO * np.eye(M) - via
            assert _approx(L_bc, c["L_bc"])
            v = np.linalg.solve(L_bc, X ** 2)
            assert _approx(v, c["v"])
    for part, (terms, expect) in c["parts"].items():
        got = _sum_oracle(terms, qo)
        if part == "L1m":  # L1_-bc = -1 .* Array(UpwindDifference(1, 1, dx, M, -1.0) * Q)[1]
            got = -got
        assert _approx(got, expect), (part, got)
        assert _approx(_sum_host(terms, qh) * (-1 if part == "L1m" else 1), expect)
    if name == "absorbing_bc":
        # L1_-bc = Array(L1 * Q)[1] ./ mu (:207)
        got = _sum_oracle([("upwind", NEG, None)], qo) / NEG
        assert _approx(got, [[4.0, 0.0, 0.0], [-4.0, 4.0, 0.0], [0.0, -4.0, 4.0]])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_sdo_example_device_concretisation(cuda, name):
    c = CASES[name]
    _, qh = _bcs(c["bc"])
    A = None
    for t in c["terms"]:
        g = _ops(t)[1] * qh
        A = g if A is None else A + g
    Al, Ab = deo.concretize(A, (M,))
    assert _approx(Al, c["Lx"]), Al
    assert not Ab.any() or c["bc"][0] == "robin"
    if c["L_bc"] is not None:
        assert _approx(np.linalg.solve(RHO * np.eye(M) - Al, X ** 2), c["v"])
