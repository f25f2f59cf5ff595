"""Golden fixtures transcribed from DiffEqOperators.jl's own test-suite.

Run ``python tests/golden/transcribe_reference.py`` to regenerate
``reference_fixtures.npz``.  Every matrix below is a hand-derived (analytic)
operator that the reference's tests compare its own operators against; the
source file and line of each is given beside it.  The reference is Julia and
cannot run here, so its known answers are carried over as data.

Matrices are dense ``len x (len+2)`` operators acting on a padded vector
``[ghost_l; u; ghost_r]``.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
IRR_DX = [0.08, 0.02, 0.05, 0.04, 0.07, 0.03]  # grid [0,.08,.1,.15,.19,.26,.29]


def fourth_deriv_approx_stencil(N):
    # test/DerivativeOperators/derivative_operators_interface.jl:8-21
    A = np.zeros((N, N + 2))
    r1 = [3.5, -56 / 3, 42.5, -54.0, 251 / 6, -20.0, 5.5, -2 / 3]
    r2 = [2 / 3, -11 / 6, 0.0, 31 / 6, -22 / 3, 4.5, -4 / 3, 1 / 6]
    A[0, 0:8] = r1
    A[1, 0:8] = r2
    A[N - 2, N - 6:] = r2[::-1]
    A[N - 1, N - 6:] = r1[::-1]
    for i in range(3, N - 1):
        A[i - 1, i - 3:i + 4] = [-1 / 6, 2.0, -13 / 2, 28 / 3, -13 / 2, 2.0, -1 / 6]
    return A


def second_deriv_fourth_approx_stencil(N):
    # derivative_operators_interface.jl:23-31
    A = np.zeros((N, N + 2))
    A[0, 0:6] = [5 / 6, -15 / 12, -1 / 3, 7 / 6, -6 / 12, 5 / 60]
    A[N - 1, N - 4:] = [1 / 12, -6 / 12, 14 / 12, -4 / 12, -15 / 12, 10 / 12]
    for i in range(2, N):
        A[i - 1, i - 2:i + 3] = [-1 / 12, 4 / 3, -5 / 2, 4 / 3, -1 / 12]
    return A


def second_derivative_stencil(N):
    # derivative_operators_interface.jl:33-40
    A = np.zeros((N, N + 2))
    for i in range(N):
        A[i, i] = 1
        A[i, i + 1] = -2
        A[i, i + 2] = 1
    return A


def _rows(shape, rows):
    A = np.zeros(shape)
    for (i, j0), vals in rows:
        A[i - 1, j0 - 1:j0 - 1 + len(vals)] = vals
    return A


def analytic_ctr_irr():
    # derivative_operators_interface.jl:47-100 (irregular grid, centred)
    out = {}
    out["ctr_1_2_irr"] = _rows((5, 7), [((1, 1), [-5.0 / 2.0, -75.0 / 2.0, 40.0]),
                                        ((2, 2), [-250.0 / 7.0, 30.0, 40.0 / 7.0]),
                                        ((3, 3), [-80.0 / 9.0, -5.0, 125.0 / 9.0]),
                                        ((4, 4), [-1225.0 / 77.0, 825.0 / 77.0, 400.0 / 77.0]),
                                        ((5, 5), [-30.0 / 7.0, -400.0 / 21.0, 70.0 / 3.0])])
    out["ctr_2_2_irr"] = _rows((5, 7), [((1, 1), [250.0, -1250.0, 1000.0]),
                                        ((2, 2), [10000.0 / 7.0, -2000.0, 4000.0 / 7.0]),
                                        ((3, 3), [4000.0 / 9.0, -1000.0, 5000.0 / 9.0]),
                                        ((4, 4), [454.0 + 42.0 / 77.0, -5000.0 / 7.0, 20000.0 / 77.0]),
                                        ((5, 5), [6000.0 / 21.0, -20000.0 / 21.0, 2000.0 / 3.0])])
    q = 13167.0
    out["ctr_2_4_irr"] = _rows((3, 7), [
        ((1, 1), [14.0 + 12012.0 / q, 1542.0 + 2736.0 / q, -2288.0 - 11704.0 / q, 838.0 + 1254.0 / q,
                  -106.0 - 4298.0 / q]),
        ((2, 2), [-223.0 - 461.0 / 693.0, 847.0 + 154.0 / 693.0, -1311.0 - 477.0 / 693.0,
                  699.0 + 593.0 / 693.0, -11.0 - 502.0 / 693.0]),
        ((3, 3), [2.0 + 12166.0 / q, 538.0 + 12654.0 / q, -912.0 - 9196.0 / q, 508.0 + 8664.0 / q,
                  -137.0 - 11121.0 / q])])
    out["ctr_4_2_irr"] = _rows((3, 7), [
        ((1, 1), [462000000.0 / 4389.0, -8550000000.0 / 4389.0, 11704000000.0 / 4389.0,
                  -5016000000.0 / 4389.0, 1400000000.0 / 4389.0]),
        ((2, 2), [200000000.0 / 231.0, -385000000.0 / 231.0, 360000000.0 / 231.0, -200000000.0 / 231.0,
                  25000000.0 / 231.0]),
        ((3, 3), [770000000.0 / 4389.0, -3420000000.0 / 4389.0, 4180000000.0 / 4389.0,
                  -2850000000.0 / 4389.0, 1320000000 / 4389.0])])
    return out


def analytic_upwind():
    # test/DerivativeOperators/upwind_operators_interface.jl:12-151
    out = {}
    A = np.zeros((5, 7))
    for i in range(1, 6):
        A[i - 1, i:i + 2] = [-1, 1]
    out["up_1_1_pos"] = A
    A = np.zeros((5, 7))
    for i in range(1, 6):
        A[i - 1, i - 1:i + 1] = [-1, 1]
    out["up_1_1_neg"] = A
    A = np.zeros((5, 7))
    for i in range(1, 5):
        A[i - 1, i:i + 3] = [-3 / 2, 2, -1 / 2]
    A[4, 4:7] = [-1 / 2, 0, 1 / 2]
    out["up_1_2_pos"] = A
    A = np.zeros((5, 7))
    A[0, 0:3] = [-1 / 2, 0, 1 / 2]
    for i in range(2, 6):
        A[i - 1, i - 2:i + 1] = [1 / 2, -2, 3 / 2]
    out["up_1_2_neg"] = A
    A = np.zeros((5, 7))
    for i in range(1, 4):
        A[i - 1, i:i + 4] = [2, -5, 4, -1]
    A[3, 3:7] = [1, -2, 1, 0]
    A[4, 3:7] = [0, 1, -2, 1]
    out["up_2_2_pos"] = A
    A = np.zeros((5, 7))
    A[0, 0:4] = [1, -2, 1, 0]
    A[1, 0:4] = [0, 1, -2, 1]
    for i in range(3, 6):
        A[i - 1, i - 3:i + 1] = [-1, 4, -5, 2]
    out["up_2_2_neg"] = A
    A = np.zeros((7, 9))
    for i in range(1, 5):
        A[i - 1, i:i + 5] = [35 / 12, -104 / 12, 114 / 12, -56 / 12, 11 / 12]
    A[4, 4:9] = [11 / 12, -20 / 12, 6 / 12, 4 / 12, -1 / 12]
    A[5, 4:9] = [-1 / 12, 16 / 12, -30 / 12, 16 / 12, -1 / 12]
    A[6, 4:9] = [-1 / 12, 4 / 12, 6 / 12, -20 / 12, 11 / 12]
    out["up_2_3_pos"] = A
    A = np.zeros((7, 9))
    A[0, 0:5] = [11 / 12, -20 / 12, 6 / 12, 4 / 12, -1 / 12]
    A[1, 0:5] = [-1 / 12, 16 / 12, -30 / 12, 16 / 12, -1 / 12]
    A[2, 0:5] = [-1 / 12, 4 / 12, 6 / 12, -20 / 12, 11 / 12]
    for i in range(4, 8):
        A[i - 1, i - 4:i + 1] = [11 / 12, -56 / 12, 114 / 12, -104 / 12, 35 / 12]
    out["up_2_3_neg"] = A
    out["up_1_1_pos_irr"] = _rows((5, 7), [((1, 2), [-50, 50]), ((2, 3), [-20, 20]), ((3, 4), [-25, 25]),
                                           ((4, 5), [-100 / 7, 100 / 7]), ((5, 6), [-100 / 3, 100 / 3])])
    out["up_1_1_neg_irr"] = _rows((5, 7), [((1, 1), [-25 / 2, 25 / 2]), ((2, 2), [-50, 50]),
                                           ((3, 3), [-20, 20]), ((4, 4), [-25, 25]),
                                           ((5, 5), [-100 / 7, 100 / 7])])
    out["up_1_2_pos_irr"] = _rows((5, 7), [((1, 2), [-450 / 7, 490 / 7, -40 / 7]),
                                           ((2, 3), [-280 / 9, 405 / 9, -125 / 9]),
                                           ((3, 4), [-2625 / 77, 3025 / 77, -400 / 77]),
                                           ((4, 5), [-510 / 21, 1000 / 21, -490 / 21]),
                                           ((5, 5), [-90 / 21, -400 / 21, 490 / 21])])
    out["up_1_2_neg_irr"] = _rows((5, 7), [((1, 1), [-5 / 2, -75 / 2, 80 / 2]),
                                           ((2, 1), [5 / 2, -125 / 2, 120 / 2]),
                                           ((3, 2), [250 / 7, -490 / 7, 240 / 7]),
                                           ((4, 3), [80 / 9, -405 / 9, 325 / 9]),
                                           ((5, 4), [1225 / 77, -3025 / 77, 1800 / 77])])
    out["up_2_2_pos_irr"] = _rows((5, 7), [
        ((1, 2), [200000 / 77, -308000 / 77, 143000 / 77, -35000 / 77]),
        ((2, 3), [27500 / 33, -75000 / 33, 55000 / 33, -7500 / 33]),
        ((3, 4), [72500 / 77, -137500 / 77, 120000 / 77, -55000 / 77]),
        ((4, 4), [42500 / 77, -71500 / 77, 40000 / 77, -11000 / 77]),
        ((5, 4), [-10000 / 77, 44000 / 77, -100000 / 77, 66000 / 77])])
    out["up_2_2_neg_irr"] = _rows((5, 7), [
        ((1, 1), [1050 / 7, -1250 / 7, -1400 / 7, 1600 / 7]),
        ((2, 1), [350 / 7, 6250 / 7, -9800 / 7, 3200 / 7]),
        ((3, 1), [-1400 / 7, 25000 / 7, -30800 / 7, 7200 / 7]),
        ((4, 2), [-390000 / 231, 770000 / 231, -660000 / 231, 280000 / 231]),
        ((5, 3), [-38500 / 77, 161000 / 77, -165000 / 77, 42500 / 77])])
    return out


# (name, d, a, dx ('irr' = IRR_DX), len, coefficient, fixture key, multiplier)
# upwind_operators_interface.jl:152-839
UPWIND_CASES = [
    ("1-1+", 1, 1, 1.0, 5, 1.0, "up_1_1_pos", 1.0),
    ("1-1-", 1, 1, 1.0, 5, -1.0, "up_1_1_neg", -1.0),
    ("1-2+", 1, 2, 1.0, 5, 1.0, "up_1_2_pos", 1.0),
    ("1-2-", 1, 2, 1.0, 5, -1.0, "up_1_2_neg", -1.0),
    ("2-2+", 2, 2, 1.0, 5, 1.0, "up_2_2_pos", 1.0),
    ("2-2-", 2, 2, 1.0, 5, -1.0, "up_2_2_neg", -1.0),
    ("2-3+", 2, 3, 1.0, 7, 1.0, "up_2_3_pos", 1.0),
    ("2-3-", 2, 3, 1.0, 7, -1.0, "up_2_3_neg", -1.0),
    ("1-1+irr", 1, 1, "irr", 5, 1.0, "up_1_1_pos_irr", 1.0),
    ("1-1-irr", 1, 1, "irr", 5, -1.0, "up_1_1_neg_irr", -1.0),
    ("1-2+irr", 1, 2, "irr", 5, 1.0, "up_1_2_pos_irr", 1.0),
    ("1-2-irr", 1, 2, "irr", 5, -1.0, "up_1_2_neg_irr", -1.0),
    ("2-2+irr", 2, 2, "irr", 5, 1.0, "up_2_2_pos_irr", 1.0),
    ("2-2-irr", 2, 2, "irr", 5, -1.0, "up_2_2_neg_irr", -1.0),
    ("1-2+h", 1, 2, 0.1, 5, 1.0, "up_1_2_pos", 10.0),
    ("1-2-h", 1, 2, 0.1, 5, -1.0, "up_1_2_neg", -10.0),
    ("2-2+h", 2, 2, 0.1, 5, 1.0, "up_2_2_pos", 100.0),
    ("2-2-h", 2, 2, 0.1, 5, -1.0, "up_2_2_neg", -100.0),
    ("2-2+c", 2, 2, 1.0, 5, 4.56, "up_2_2_pos", 4.56),
    ("2-2-c", 2, 2, 1.0, 5, -4.56, "up_2_2_neg", -4.56),
    ("2-2+hc", 2, 2, 0.1, 5, 4.56, "up_2_2_pos", 4.56 * 100.0),
    ("2-2-hc", 2, 2, 0.1, 5, -4.56, "up_2_2_neg", -4.56 * 100.0),
    ("2-2+irrc", 2, 2, "irr", 5, 4.56, "up_2_2_pos_irr", 4.56),
    ("2-2-irrc", 2, 2, "irr", 5, -4.56, "up_2_2_neg_irr", -4.56),
]

# (d, a, dx, len, fixture key, rows compared) derivative_operators_interface.jl:121-144,229-281
CENTRED_CASES = [
    (4, 4, 1.0, 20, "fourth_deriv_approx_stencil_20", None),
    (2, 4, 1.0, 20, "second_deriv_fourth_approx_stencil_20", None),
    (2, 2, 1.0, 10, "second_derivative_stencil_10", None),
    (1, 2, "irr", 5, "ctr_1_2_irr", None),
    (2, 2, "irr", 5, "ctr_2_2_irr", None),
    (2, 4, "irr", 5, "ctr_2_4_irr", (1, 4)),
    (4, 2, "irr", 5, "ctr_4_2_irr", (1, 4)),
]


def build() -> dict:
    fx = {}
    fx["fourth_deriv_approx_stencil_20"] = fourth_deriv_approx_stencil(20)
    fx["second_deriv_fourth_approx_stencil_20"] = second_deriv_fourth_approx_stencil(20)
    fx["second_derivative_stencil_10"] = second_derivative_stencil(10)
    fx.update(analytic_ctr_irr())
    fx.update(analytic_upwind())
    # derivative_operators_interface.jl:407-415: Array(3.3 * CenteredDifference(2,2,10.0,3))
    fx["scalar_mult_3p3"] = np.array([[0.033, -0.066, 0.033, 0.0, 0.0],
                                      [0.0, 0.033, -0.066, 0.033, 0.0],
                                      [0.0, 0.0, 0.033, -0.066, 0.033]])
    # robin.jl:92-110: 3rd-order Robin/General known answer for u = 1:10
    fx["robin3_u0"] = np.array([-4 / 10])
    fx["robin3_uend"] = np.array([125 / 12])
    # derivative_operators_interface.jl:148-151 (centred stencils, d = 1..3, a = 2, 4)
    fx["ctr_weights_a2"] = np.array([-0.5, 0, 0.5, 1.0, -2.0, 1.0, -1 / 2, 1.0, 0.0, -1.0, 1 / 2])
    fx["ctr_weights_a4"] = np.array([1 / 12, -2 / 3, 0, 2 / 3, -1 / 12, -1 / 12, 4 / 3, -5 / 2, 4 / 3, -1 / 12,
                                     1 / 8, -1.0, 13 / 8, 0.0, -13 / 8, 1.0, -1 / 8])
    return fx


if __name__ == "__main__":
    path = os.path.join(HERE, "reference_fixtures.npz")
    np.savez_compressed(path, **build())
    print("wrote", path)
