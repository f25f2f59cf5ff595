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


# ---------------------------------------------------------------------------
# Block fixed point (k_lap_bfx): one exponent per (32 x 16 tile, z-plane)
# ---------------------------------------------------------------------------
BFX_TX, BFX_TY, BFX_G0 = 32, 16, 7


def bfx_weights(w, H: int):
    """(W, f, c0, tshift) as the library builds them (bfx_weights in
    deo_host.cpp), or None where the kernel is not used."""
    G0 = BFX_G0
    K = 2 * H + 1
    M, fk = [], []
    for x in w[:K]:
        x = float(x)
        if x == 0.0 or not math.isfinite(x) or abs(x) < 2.0 ** -1022:
            return None
        fr, ex = math.frexp(abs(x))
        M.append(int(fr * 2 ** 53))
        fk.append(ex - 53)
    if 53 + max(fk) - min(fk) > 58:
        return None
    f = min(fk)
    W = [(-1 if float(w[k]) < 0 else 1) * (M[k] << (fk[k] - f)) for k in range(K)]
    c0 = 3 * W[H]
    cneg = float(w[H]) < 0
    if any((float(w[k]) < 0) != (cneg != ((k - H) % 2 == 1)) for k in range(K)):
        return None  # the kernel needs signs alternating from the centre
    s0max = (1 << 31) - 1
    s1max = ((1 << 62) + (3 << 60)) >> 31
    cols = [0, 0, 0, 0]
    for k in range(K):
        aw = abs(c0 if k == H else W[k])
        w0, w1 = aw & ((1 << 29) - 1), aw >> 29
        cols[0] += s0max * w0
        cols[1] += s1max * w0
        cols[2] += s0max * w1
        cols[3] += s1max * w1
    if max(cols) >= 1 << 64:
        return None
    allw = sum(abs(float(w[k])) for k in range(K) if k != H)
    per = (4 / 3) * (allw / abs(float(w[H]))) * 2.0 ** (1 - G0)
    Tc = G0
    while Tc >= 0 and per * 2.0 ** Tc > 2.0:
        Tc -= 1
    if Tc < 0:
        return None
    return W, f, c0, 53 + G0 - 1 - Tc


def bfx_apply(u: np.ndarray, w, H: int, flo, fhi):
    """The kernel's result at every interior point of a 3-D Fortran-ordered
    array (flo/fhi: per axis, the 1-based rows evaluated from the band), as
    (values, use) arrays: use = False where the kernel leaves the point to the
    reference's tap order."""
    params = bfx_weights(w, H)
    assert params is not None
    W, f, c0, tshift = params
    G0 = BFX_G0
    nx, ny, nz = u.shape
    TX, TY = BFX_TX, BFX_TY
    tiles_x, tiles_y = -(-nx // TX), -(-ny // TY)
    # zero padding: H on every side, tiles rounded up (the copies fill zeros outside the array)
    up = np.zeros((tiles_x * TX + 2 * H, tiles_y * TY + 2 * H, nz + 2 * H))
    up[H:H + nx, H:H + ny, H:H + nz] = u
    bits = up.view(np.uint64)
    ex = ((bits >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    fr = bits & np.uint64((1 << 52) - 1)
    mant = np.where(ex > 0, fr | np.uint64(1 << 52), fr)
    neg = (bits >> np.uint64(63)) == 1
    nonzero = (bits << np.uint64(1)) != 0
    out = np.zeros(u.shape)
    use = np.zeros(u.shape, bool)
    # region a tile's conversion covers: its block and H-wide strips beside it (no corners)
    reg = np.zeros((TX + 2 * H, TY + 2 * H), bool)
    reg[H:H + TX, :] = True
    reg[:, H:H + TY] = True
    lo = [fl - 1 for fl in flo]  # 0-based interior range
    hi = [fh - 1 for fh in fhi]
    for ti in range(tiles_x):
        for tj in range(tiles_y):
            xs, ys = slice(ti * TX, ti * TX + TX + 2 * H), slice(tj * TY, tj * TY + TY + 2 * H)
            e1 = np.maximum(ex[xs, ys, :], 1)
            mn = mant[xs, ys, :]
            r3 = reg[:, :, None]
            E = np.where(r3, e1, 1).max(axis=(0, 1))  # per plane
            Emin = np.where(r3 & nonzero[xs, ys, :], e1, 4095).min(axis=(0, 1))
            exact_plane = (E - Emin) <= G0
            d = np.minimum(E[None, None, :] - e1, 63)
            mag = ((mn << np.uint64(G0)) >> d.astype(np.uint64)).astype(np.int64)
            m = np.where(neg[xs, ys, :], -mag, mag)
            for lx in range(TX):
                x = ti * TX + lx
                if not (x < nx and lo[0] <= x <= hi[0]):
                    continue
                for ly in range(TY):
                    y = tj * TY + ly
                    if not (y < ny and lo[1] <= y <= hi[1]):
                        continue
                    bx, by = lx + H, ly + H
                    for z in range(max(lo[2], 0), min(hi[2], nz - 1) + 1):
                        zc = z + H  # padded plane index of the centre
                        Es = [int(E[zc + o]) for o in range(-H, H + 1)]
                        Ept = max(Es)
                        same = all(x_ == Ept for x_ in Es)
                        exact = same and all(bool(exact_plane[zc + o]) for o in range(-H, H + 1))
                        dc = min(Ept - int(E[zc]), 63)
                        m0 = int(m[bx, by, zc]) >> dc
                        groups = {}
                        for o in range(1, H + 1):
                            for sgn in (-1, 1):
                                xy = int(m[bx + sgn * o, by, zc]) + int(m[bx, by + sgn * o, zc])
                                zz = int(m[bx, by, zc + sgn * o]) >> min(Ept - int(E[zc + sgn * o]), 63)
                                groups[sgn * o] = (xy >> dc) + zz
                        big = m0 >> tshift
                        if not (Ept < 2047 and (exact or big not in (0, -1))):
                            continue
                        A = c0 * m0
                        for o in range(1, H + 1):
                            A += W[H - o] * groups[-o] + W[H + o] * groups[o]
                        r = fx_round(A, Ept + f + 75 - G0)
                        if r is None:
                            continue
                        out[x, y, z] = r
                        use[x, y, z] = True
    return out, use
