"""Integer model of the fixed-point interior kernel (k_lap_fx), for bit-exact
tests: the same decomposition, alignment, per-offset int64 sums, 128-bit
weighted accumulation and round-to-nearest-even, written with Python ints.
Also an exact rational evaluation of the interior stencil for error bounds."""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np


def fx_weights(w, H: int, nt: int):
    """(W, f) with w[k] = W[k] * 2^f exactly, or None where the kernel is not
    used (same acceptance rules as the library)."""
    S = 8 if nt == 3 else 9
    M, fk = [], []
    for x in w[:2 * H + 1]:
        x = float(x)
        if x == 0.0 or not math.isfinite(x) or abs(x) < 2.0 ** -1022:
            return None
        fr, ex = math.frexp(abs(x))
        M.append(int(fr * 2 ** 53))
        fk.append(ex - 53)
    bits = 53 + max(fk) - min(fk)
    lg = 0
    while (1 << lg) < (2 * H + 1) * nt:
        lg += 1
    if bits > 62 or bits + 53 + S + lg > 127:
        return None
    absw = [abs(float(x)) for x in w[:2 * H + 1]]
    if nt * sum(absw) / min(absw) > 256.0:
        return None
    f = min(fk)
    W = [(-1 if float(w[k]) < 0 else 1) * (M[k] << (fk[k] - f)) for k in range(2 * H + 1)]
    return W, f


def decompose(v: float, S: int):
    b = int(np.float64(v).view(np.uint64))
    ex = (b >> 52) & 0x7FF
    fr = b & ((1 << 52) - 1)
    mag = ((fr | (1 << 52)) if ex else fr) << S
    m = -mag if (b >> 63) else mag
    e = 4095 if ex == 0x7FF else (ex if ex else 1)
    return m, e


def fx_round(A: int, ebase: int):
    """A rounded to the nearest double (ties to even) with biased exponent
    ebase - lz for a 128-bit magnitude with lz leading zeros; None if the
    result would be subnormal or overflow."""
    if A == 0:
        return 0.0
    neg = A < 0
    mag = -A if neg else A
    lz = 128 - mag.bit_length()
    N = mag << lz
    mant = N >> 75
    rem = N & ((1 << 75) - 1)
    half = 1 << 74
    if rem > half or (rem == half and (mant & 1)):
        mant += 1
    be = ebase - lz
    if mant >> 53:
        mant >>= 1
        be += 1
    if be <= 0 or be >= 2047:
        return None
    bits = (int(neg) << 63) | (be << 52) | (mant & ((1 << 52) - 1))
    return float(np.uint64(bits).view(np.float64))


def _taps(u: np.ndarray, idx: tuple, H: int, nt: int):
    """Centre value and, for each offset k = -H..H (k != 0), the NT values at
    that offset (one per axis) of the point idx of a Fortran-ordered array."""
    c = u[idx]
    groups = {}
    for k in range(-H, H + 1):
        if k == 0:
            continue
        vals = []
        for a in range(nt):
            j = list(idx)
            j[a] += k
            vals.append(u[tuple(j)])
        groups[k] = vals
    return c, groups


def fx_point(u: np.ndarray, idx: tuple, w, H: int, nt: int):
    """The kernel's result at an interior point, or None where it falls back
    to the reference's tap order (Inf/NaN input, subnormal/overflowing result)."""
    Wf = fx_weights(w, H, nt)
    assert Wf is not None
    W, f = Wf
    S = 8 if nt == 3 else 9
    c, groups = _taps(u, idx, H, nt)
    m0, e0 = decompose(c, S)
    dec = {k: [decompose(v, S) for v in vals] for k, vals in groups.items()}
    E = max([e0] + [e for vals in dec.values() for _, e in vals])
    if E >= 2047:
        return None
    A = nt * (m0 >> min(E - e0, 63)) * W[H]
    for k, vals in dec.items():
        s = sum(m >> min(E - e, 63) for m, e in vals)
        A += s * W[H + k]
    return fx_round(A, 75 - S + f + E)


def exact_point(u: np.ndarray, idx: tuple, w, H: int, nt: int):
    """(exact value, sum|c_k u_k|) of the interior stencil as Fractions."""
    c, groups = _taps(u, idx, H, nt)
    wc = Fraction(float(w[H]))
    val = nt * wc * Fraction(float(c))
    scale = nt * abs(wc) * abs(Fraction(float(c)))
    for k, vals in groups.items():
        wk = Fraction(float(w[H + k]))
        for v in vals:
            val += wk * Fraction(float(v))
            scale += abs(wk) * abs(Fraction(float(v)))
    return val, scale
