// deo_rows.cuh -- boundary rows of Laplacian-type plans evaluated from a
// ShellTerm (weights, ghost maps) in the generic evaluator's arithmetic, on a
// line in global memory or in a shared-memory box (the shell kernels of
// deo_shell.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "deo_eval.cuh"

namespace deo {

// Plain load: the row helpers read global memory or a shared-memory box.
template <typename T>
__device__ __forceinline__ T ldv(const T* p) {
    return *p;
}

// Element k of a packed weight array (doubles, or floats packed from the start).
template <typename T>
__device__ __forceinline__ T sw(const double* a, int k);
template <>
__device__ __forceinline__ double sw<double>(const double* a, int k) {
    return a[k];
}
template <>
__device__ __forceinline__ float sw<float>(const double* a, int k) {
    return reinterpret_cast<const float*>(a)[k];
}

// Ghost value of one end of a line with its m taps unrolled (M = m): the
// arithmetic of ghost_left / ghost_right.  The dispatchers below take MAXW, the
// widest ghost map / row they must handle (8 or 16), to keep registers low.
template <typename T, int M>
__device__ __forceinline__ T ghost_m(const double* a, const double* b, const T* __restrict__ p, int64_t s) {
    T d = sw<T>(a, 0) * ldv(p);
#pragma unroll
    for (int j = 1; j < M; ++j) d = fma(sw<T>(a, j), ldv(p + j * s), d);
    return d + sw<T>(b, 0);
}

template <typename T, int MAXW = 16>
__device__ __forceinline__ T shell_ghost(const ShellTerm& S, const T* __restrict__ line, int64_t s, bool left) {
    if (S.bc_kind == 1) return (S.periodic_nd == left) ? ldv(line) : ldv(line + (int64_t)(S.len - 1) * s);
    const int m = left ? S.ml : S.mr;
    const T* p = left ? line : line + (int64_t)(S.len - S.mr) * s;
    const double* a = left ? S.al : S.ar;
    const double* b = left ? &S.bl : &S.br;
    switch (m) {
        case 0: return T(0) + sw<T>(b, 0);
        case 1: return ghost_m<T, 1>(a, b, p, s);
        case 2: return ghost_m<T, 2>(a, b, p, s);
        case 3: return ghost_m<T, 3>(a, b, p, s);
        case 4: return ghost_m<T, 4>(a, b, p, s);
        case 5: return ghost_m<T, 5>(a, b, p, s);
        case 6: return ghost_m<T, 6>(a, b, p, s);
        case 7: return ghost_m<T, 7>(a, b, p, s);
        case 8: return ghost_m<T, 8>(a, b, p, s);
        case 9: if constexpr (9 <= MAXW) return ghost_m<T, 9>(a, b, p, s); break;
        case 10: if constexpr (10 <= MAXW) return ghost_m<T, 10>(a, b, p, s); break;
        case 11: if constexpr (11 <= MAXW) return ghost_m<T, 11>(a, b, p, s); break;
        case 12: if constexpr (12 <= MAXW) return ghost_m<T, 12>(a, b, p, s); break;
        case 13: if constexpr (13 <= MAXW) return ghost_m<T, 13>(a, b, p, s); break;
        case 14: if constexpr (14 <= MAXW) return ghost_m<T, 14>(a, b, p, s); break;
        case 15: if constexpr (15 <= MAXW) return ghost_m<T, 15>(a, b, p, s); break;
        case 16: if constexpr (16 <= MAXW) return ghost_m<T, 16>(a, b, p, s); break;
    }
    return T(0);
}

// One boundary row with its NK taps unrolled: the taps of eval_term in its
// order; a tap at padded index 1 or len+2 is the ghost of that end.
template <typename T, int NK>
__device__ __forceinline__ T row_nk(const double* w, int p0, const T* __restrict__ line, int64_t s, int L2, T gl,
                                    T gr) {
    const T* p = line + (int64_t)(p0 - 2) * s;
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < NK; ++k) {
        T x;
        if (k == 0 && p0 == 1) x = gl;
        else if (k == NK - 1 && p0 + NK - 1 == L2) x = gr;
        else x = ldv(p + k * s);
        acc = fma(sw<T>(w, k), x, acc);
    }
    return acc;
}

template <typename T, int MAXW = 16>
__device__ __forceinline__ T row_eval(const ShellRow& R, const T* __restrict__ line, int64_t s, int L2, T gl, T gr) {
    switch (R.nk) {
        case 1: return row_nk<T, 1>(R.w, R.p0, line, s, L2, gl, gr);
        case 2: return row_nk<T, 2>(R.w, R.p0, line, s, L2, gl, gr);
        case 3: return row_nk<T, 3>(R.w, R.p0, line, s, L2, gl, gr);
        case 4: return row_nk<T, 4>(R.w, R.p0, line, s, L2, gl, gr);
        case 5: return row_nk<T, 5>(R.w, R.p0, line, s, L2, gl, gr);
        case 6: return row_nk<T, 6>(R.w, R.p0, line, s, L2, gl, gr);
        case 7: return row_nk<T, 7>(R.w, R.p0, line, s, L2, gl, gr);
        case 8: return row_nk<T, 8>(R.w, R.p0, line, s, L2, gl, gr);
        case 9: if constexpr (9 <= MAXW) return row_nk<T, 9>(R.w, R.p0, line, s, L2, gl, gr); break;
        case 10: if constexpr (10 <= MAXW) return row_nk<T, 10>(R.w, R.p0, line, s, L2, gl, gr); break;
        case 11: if constexpr (11 <= MAXW) return row_nk<T, 11>(R.w, R.p0, line, s, L2, gl, gr); break;
        case 12: if constexpr (12 <= MAXW) return row_nk<T, 12>(R.w, R.p0, line, s, L2, gl, gr); break;
        case 13: if constexpr (13 <= MAXW) return row_nk<T, 13>(R.w, R.p0, line, s, L2, gl, gr); break;
        case 14: if constexpr (14 <= MAXW) return row_nk<T, 14>(R.w, R.p0, line, s, L2, gl, gr); break;
        case 15: if constexpr (15 <= MAXW) return row_nk<T, 15>(R.w, R.p0, line, s, L2, gl, gr); break;
        case 16: if constexpr (16 <= MAXW) return row_nk<T, 16>(R.w, R.p0, line, s, L2, gl, gr); break;
    }
    return T(0);
}

// Boundary row i (1-based) of a term on the line starting at `line`, with
// its own ghosts (edges and corners of the shell).
template <typename T, int MAXW = 16>
__device__ __forceinline__ T shell_row(const ShellTerm& S, const T* __restrict__ line, int64_t s, int i) {
    const int r = i <= S.nlo ? i - 1 : S.nlo + (i - (S.len - S.nhi + 1));
    const ShellRow& R = S.row[r];
    const int L2 = S.len + 2;
    const T gl = R.p0 == 1 ? shell_ghost<T, MAXW>(S, line, s, true) : T(0);
    const T gr = R.p0 + R.nk - 1 == L2 ? shell_ghost<T, MAXW>(S, line, s, false) : T(0);
    return row_eval<T, MAXW>(R, line, s, L2, gl, gr);
}

// Out of line, for the rarely taken rows (edges and corners of the shell).
template <typename T, int MAXW = 16>
__device__ __noinline__ T shell_row_cold(const ShellTerm& S, const T* __restrict__ line, int64_t s, int i) {
    return shell_row<T, MAXW>(S, line, s, i);
}

// Band taps of axis a at idx (interior row along a), as eval_term's band
// path; H = the band's radius (<= 4).
template <typename T>
__device__ __forceinline__ T shell_band(const UniTerm& ut, int H, const T* __restrict__ u, int64_t idx, int64_t s) {
    const T* p = u + idx - H * s;
    T x[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) x[k] = k <= 2 * H ? ldv(p + k * s) : T(0);
    T r = T(0);
#pragma unroll
    for (int k = 0; k < 9; ++k)
        if (k <= 2 * H) r = fma(uni_w<T>(ut, k), x[k], r);
    return r;
}

// The same with the radius known at compile time: exactly 2H + 1 taps.
template <typename T, int H>
__device__ __forceinline__ T shell_band_h(const UniTerm& ut, const T* __restrict__ p, int64_t s) {
    const T* q = p - H * s;
    T r = T(0);
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) r = fma(uni_w<T>(ut, k), ldv(q + k * s), r);
    return r;
}

}  // namespace deo
