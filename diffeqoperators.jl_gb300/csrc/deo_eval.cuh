// deo_eval.cuh -- device-side evaluators shared by the kernels: one output
// row of one term from its row table (forward), one column of the transposed
// operator (adjoint), the multi-term point sum, and small helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "deo_internal.h"

namespace deo {

template <typename T>
__device__ __forceinline__ T band_w(const RowTabDev& tb, int k);
template <>
__device__ __forceinline__ double band_w<double>(const RowTabDev& tb, int k) {
    return tb.wband[k];
}
template <>
__device__ __forceinline__ float band_w<float>(const RowTabDev& tb, int k) {
    return reinterpret_cast<const float*>(tb.wband)[k];
}

// The per-line BC record of the line starting at flat index `base`
// (multi_dim_bc_operators.jl:28-52: the BC at the line's index over the other axes).
__device__ __forceinline__ const double* line_bc(const TermDev& t, int64_t base) {
    const int64_t lo = base % t.stride, hi = base / (t.stride * (int64_t)t.len);
    return t.lbc + (lo + hi * t.stride) * (int64_t)t.lbc_stride;
}

// Ghosts from one line's own BC record: BCs[I, J] * u[I, :, J], the 1-D ghost
// fill (a periodic BC wraps around its line, bc_operators.jl:188-193).
template <typename T>
__device__ __noinline__ T ghost_line(const TermDev& t, const T* __restrict__ line, int64_t base, bool left) {
    const int64_t s = t.stride;
    const double* q = line_bc(t, base);
    if (q[0] != 0.0) return left ? line[(int64_t)(t.len - 1) * s] : line[0];
    const int m = (int)(left ? q[1] : q[2]);
    const double* a = q + 5 + (left ? 0 : t.lbc_mw);
    const int64_t o = left ? 0 : (int64_t)(t.len - m);
    T d = T(0);
    for (int j = 0; j < m; ++j) d = (j == 0) ? T(a[0]) * line[o * s] : fma(T(a[j]), line[(o + j) * s], d);
    return d + T(left ? q[3] : q[4]);
}

// LBC: the plan has per-line boundary conditions (PlanDev::has_lbc); the
// kernels are instantiated with and without that branch, so that plans
// without them carry no call to ghost_line.
template <typename T, bool LBC = false>
__device__ __forceinline__ T ghost_left(const TermDev& t, const T* __restrict__ line, int64_t base) {
    const int64_t s = t.stride;
    if (LBC && t.lbc) return ghost_line<T>(t, line, base, true);
    if (t.bc_kind == 1) return t.periodic_nd ? line[0] : line[(int64_t)(t.len - 1) * s];
    if (t.bc_kind == 2) return line[-s];  // padded input: the ghost is stored before the line
    T d = T(0);
    for (int j = 0; j < t.ml; ++j) d = (j == 0) ? T(t.al[0]) * line[0] : fma(T(t.al[j]), line[(int64_t)j * s], d);
    return d + T(t.bl);
}

template <typename T, bool LBC = false>
__device__ __forceinline__ T ghost_right(const TermDev& t, const T* __restrict__ line, int64_t base) {
    const int64_t s = t.stride;
    if (LBC && t.lbc) return ghost_line<T>(t, line, base, false);
    if (t.bc_kind == 1) return t.periodic_nd ? line[(int64_t)(t.len - 1) * s] : line[0];
    if (t.bc_kind == 2) return line[(int64_t)t.len * s];  // padded input: the ghost is stored after the line
    T d = T(0);
    const int64_t o = (int64_t)(t.len - t.mr);
    for (int j = 0; j < t.mr; ++j)
        d = (j == 0) ? T(t.ar[0]) * line[o * s] : fma(T(t.ar[j]), line[(o + j) * s], d);
    return d + T(t.br);
}

// The reference adds `!overwrite * x_temp[i]` (a strong zero) to every tap
// sum, which turns -0.0 into +0.0 and is otherwise exact.  Applied once to the
// final sum it has the same effect; done on the bits to spend no FP64 issue.
__device__ __forceinline__ double zero_fix(double x) {
    return __double_as_longlong(x) == (long long)0x8000000000000000ULL ? 0.0 : x;
}
__device__ __forceinline__ float zero_fix(float x) {
    return __float_as_uint(x) == 0x80000000u ? 0.0f : x;
}

struct RowInfo {
    int p0, nk, e;
    bool band;
};

__device__ __forceinline__ RowInfo row_info(const RowTabDev& tb, int i) {
    RowInfo r;
    r.band = (i >= tb.ilo) && (i <= tb.ihi);
    if (r.band) {
        r.p0 = i + tb.band_p0_off;
        r.nk = tb.band_nk;
        r.e = 0;
    } else {
        r.e = (i < tb.ilo) ? i - 1 : (tb.ilo - 1) + (i - tb.ihi - 1);
        r.p0 = __ldg(tb.p0 + r.e);
        r.nk = __ldg(tb.nk + r.e);
    }
    return r;
}

__device__ __forceinline__ int row_cidx(const RowTabDev& tb, int i) {
    if (i >= tb.ilo && i <= tb.ihi) return i + tb.band_cidx_off;
    const int e = (i < tb.ilo) ? i - 1 : (tb.ilo - 1) + (i - tb.ihi - 1);
    return __ldg(tb.cidx + e);
}

template <typename T>
__device__ __forceinline__ T row_w(const RowTabDev& tb, const RowInfo& r, int k) {
    return r.band ? band_w<T>(tb, k) : __ldg(reinterpret_cast<const T*>(tb.W) + (int64_t)k * tb.nexp + r.e);
}

// !(c >= 0) -- c negative (not -0) or NaN: the upwind operator's variant
// choice (convolutions.jl:134), tested on the bits so that it issues no FP64
// (Float32) comparison.
__device__ __forceinline__ bool not_nonneg(double c) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(c);
    return ((long long)b < 0 && (b << 1) != 0ULL) || (b << 1) > 0xFFE0000000000000ULL;
}
__device__ __forceinline__ bool not_nonneg(float c) {
    const unsigned b = __float_as_uint(c);
    return ((int)b < 0 && (b << 1) != 0u) || (b << 1) > 0xFF000000u;
}

// Coefficient and table variant of row i on the line starting at `base`.
template <typename T>
__device__ __forceinline__ const RowTabDev& row_variant(const TermDev& t, int64_t base, int i, T& c) {
    c = T(1);
    if (!t.has_field) return t.tab[0];
    const int ci = row_cidx(t.tab[0], i);
    c = __ldg(reinterpret_cast<const T*>(t.field) + base + (int64_t)(ci - 1) * t.stride);
    if (t.nvar == 2 && not_nonneg(c)) return t.tab[1];
    return t.tab[0];
}

// One term, one output row: the reference's per-point tap loop.
template <typename T, bool LBC = false>
__device__ __forceinline__ T eval_term(const TermDev& t, const T* __restrict__ u, int64_t idx, int i) {
    const int64_t s = t.stride;
    const int64_t base = idx - (int64_t)(i - 1) * s;
    const T* __restrict__ line = u + base;
    T c;
    const RowTabDev& tb = row_variant<T>(t, base, i, c);
    const RowInfo r = row_info(tb, i);
    const int L2 = t.len + 2;
    // (the field and no-field loops are separate so that the common no-field
    // rows issue no c * w multiply: a speculated one would double the FP64 work)
    if (r.band && r.p0 >= 2 && r.p0 + r.nk <= L2) {
        // band row away from the ghosts: straight tap loop (same order and rounding)
        const T* __restrict__ xp = line + (int64_t)(r.p0 - 2) * s;
        T acc = T(0);
        if (t.has_field == 2) {  // DEO_PLAN_FACTOR_FIELD: c * (sum_k w_k x_k)
            for (int k = 0; k < r.nk; ++k) acc = fma(band_w<T>(tb, k), __ldg(xp + (int64_t)k * s), acc);
            acc = c * acc;
        } else if (t.has_field) {
            for (int k = 0; k < r.nk; ++k) acc = fma(c * band_w<T>(tb, k), __ldg(xp + (int64_t)k * s), acc);
        } else {
            for (int k = 0; k < r.nk; ++k) acc = fma(band_w<T>(tb, k), __ldg(xp + (int64_t)k * s), acc);
        }
        return acc;
    }
    T gl = T(0), gr = T(0);
    if (r.p0 == 1) gl = ghost_left<T, LBC>(t, line, base);
    if (r.p0 + r.nk - 1 == L2) gr = ghost_right<T, LBC>(t, line, base);
    auto tap = [&](int k) {
        const int p = r.p0 + k;
        return (p == 1) ? gl : (p == L2 ? gr : __ldg(line + (int64_t)(p - 2) * s));
    };
    T acc = T(0);
    if (t.has_field == 2) {
        for (int k = 0; k < r.nk; ++k) acc = fma(row_w<T>(tb, r, k), tap(k), acc);
        acc = c * acc;
    } else if (t.has_field) {
        for (int k = 0; k < r.nk; ++k) acc = fma(c * row_w<T>(tb, r, k), tap(k), acc);
    } else {
        for (int k = 0; k < r.nk; ++k) acc = fma(row_w<T>(tb, r, k), tap(k), acc);
    }
    return acc;
}

// One row of a term's table over a padded line whose ghosts are stored around
// it (bc_kind 2), so every tap is a plain load: line position p (1-based) is
// x0[(p - 1) * s], x0 pointing at the left ghost.  Same products and order as
// eval_term; no field coefficient.
template <typename T>
__device__ __forceinline__ T eval_row_padded(const RowTabDev& tb, const T* __restrict__ x0, int64_t s, int i) {
    const RowInfo r = row_info(tb, i);
    const T* __restrict__ xp = x0 + (int64_t)(r.p0 - 1) * s;
    T acc = T(0);
    for (int k = 0; k < r.nk; ++k) acc = fma(row_w<T>(tb, r, k), __ldg(xp + (int64_t)k * s), acc);
    return acc;
}

// Column p of one term's L (padded space) dotted with dbar along the line.
template <typename T>
__device__ __forceinline__ T adj_column(const TermDev& t, const T* __restrict__ d, int64_t base, int p) {
    const int64_t s = t.stride;
    const int lo = __ldg(t.rlo + (p - 1)), hi = __ldg(t.rhi + (p - 1));
    T acc = T(0);
    if (!t.has_field) {
        // column inside the band: the touching rows are exactly the band rows
        // p - off - nk + 1 .. p - off; same row order as the general loop below
        const RowTabDev& tb = t.tab[0];
        const int blo = p - tb.band_p0_off - tb.band_nk + 1, bhi = p - tb.band_p0_off;
        if (lo == blo && hi == bhi && blo >= tb.ilo && bhi <= tb.ihi) {
            for (int i = lo; i <= hi; ++i)
                acc = fma(band_w<T>(tb, p - i - tb.band_p0_off), __ldg(d + base + (int64_t)(i - 1) * s), acc);
            return acc;
        }
    }
    if (!t.has_field) {  // (no c * w multiply issued, see eval_term)
        const RowTabDev& tb = t.tab[0];
        for (int i = lo; i <= hi; ++i) {
            const RowInfo r = row_info(tb, i);
            const int k = p - r.p0;
            if (k < 0 || k >= r.nk) continue;
            acc = fma(row_w<T>(tb, r, k), __ldg(d + base + (int64_t)(i - 1) * s), acc);
        }
        return acc;
    }
    for (int i = lo; i <= hi; ++i) {
        T c;
        const RowTabDev& tb = row_variant<T>(t, base, i, c);
        const RowInfo r = row_info(tb, i);
        const int k = p - r.p0;
        if (k < 0 || k >= r.nk) continue;
        acc = fma(c * row_w<T>(tb, r, k), __ldg(d + base + (int64_t)(i - 1) * s), acc);
    }
    return acc;
}

template <typename T, bool LBC = false>
__device__ __forceinline__ T adj_term(const TermDev& t, const T* __restrict__ d, int64_t idx, int j) {
    const int64_t base = idx - (int64_t)(j - 1) * t.stride;
    const int L = t.len;
    T w = adj_column<T>(t, d, base, j + 1);
    if (LBC && t.lbc) {  // this line's own BC
        const double* q = line_bc(t, base);
        if (q[0] != 0.0) {  // periodic line: the left ghost is u[len], the right u[1]
            if (j == L) w += adj_column<T>(t, d, base, 1);
            if (j == 1) w += adj_column<T>(t, d, base, L + 2);
        } else {
            const int ml = (int)q[1], mr = (int)q[2];
            if (j <= ml) w = fma(T(q[5 + j - 1]), adj_column<T>(t, d, base, 1), w);
            if (j > L - mr) w = fma(T(q[5 + t.lbc_mw + j - 1 - (L - mr)]), adj_column<T>(t, d, base, L + 2), w);
        }
        return w;
    }
    if (t.bc_kind == 0) {
        if (j <= t.ml) w = fma(T(t.al[j - 1]), adj_column<T>(t, d, base, 1), w);
        if (j > L - t.mr) w = fma(T(t.ar[j - 1 - (L - t.mr)]), adj_column<T>(t, d, base, L + 2), w);
    } else {
        const int jl = t.periodic_nd ? 1 : L;  // column receiving the left ghost
        const int jr = t.periodic_nd ? L : 1;
        if (j == jl) w += adj_column<T>(t, d, base, 1);
        if (j == jr) w += adj_column<T>(t, d, base, L + 2);
    }
    return w;
}

__device__ __forceinline__ uint32_t fast_div(uint32_t n, const FastDiv& d) {
    return (__umulhi(n, d.mul) + n) >> d.shr;
}

// 1-based row of flat index idx along term t's axis
__device__ __forceinline__ int term_row(const PlanDev& P, const TermDev& t, int64_t idx) {
    if (P.fastdiv) {
        const uint32_t q = fast_div((uint32_t)idx, t.div_stride);
        return (int)(q - fast_div(q, t.div_len) * (uint32_t)t.len) + 1;
    }
    return (int)((idx / t.stride) % t.len) + 1;
}

template <typename T, bool ADJ, bool LBC = false>
__device__ __forceinline__ T eval_point(const PlanDev& P, const T* __restrict__ u, int64_t idx) {
    if (!ADJ && P.star.n) {  // the merged star at points whose rows read no ghost along any axis
        bool in = true;
        for (int tt = 0; tt < P.nterms; ++tt) {
            const int i = term_row(P, P.t[tt], idx);
            in = in && i >= P.star.lo[tt] && i <= P.star.hi[tt];
        }
        if (in) {
            T acc = T(0);
            for (int k = 0; k < P.star.n; ++k) acc = fma(T(P.star.w[k]), __ldg(u + idx + P.star.off[k]), acc);
            return zero_fix(acc);
        }
    }
    auto term = [&](int tt) {
        const TermDev& t = P.t[tt];
        const int i = term_row(P, t, idx);
        return ADJ ? adj_term<T, LBC>(t, u, idx, i) : eval_term<T, LBC>(t, u, idx, i);
    };
    T acc = term(0);  // the first term as is, then the others added left to right
    for (int tt = 1; tt < P.nterms; ++tt) acc = acc + term(tt);
    return ADJ ? acc : zero_fix(acc);
}

// Out-of-line copy of the generic column evaluator (the transposed shell's
// boundary columns).
template <typename T>
__device__ __noinline__ T adj_term_cold(const TermDev& t, const T* __restrict__ d, int64_t idx, int j) {
    return adj_term<T>(t, d, idx, j);
}

// Out-of-line copy for a kernel that evaluates a few boundary points with
// the generic evaluator (the shell fallback).
template <typename T>
__device__ __noinline__ T eval_term_cold(const TermDev& t, const T* __restrict__ u, int64_t idx, int i) {
    return eval_term<T>(t, u, idx, i);
}

template <typename T>
__device__ __forceinline__ T uni_w(const UniTerm& t, int k);
template <>
__device__ __forceinline__ double uni_w<double>(const UniTerm& t, int k) { return t.w[k]; }
template <>
__device__ __forceinline__ float uni_w<float>(const UniTerm& t, int k) {
    return reinterpret_cast<const float*>(t.w)[k];
}

}  // namespace deo
