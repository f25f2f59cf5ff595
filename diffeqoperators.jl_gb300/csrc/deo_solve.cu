// deo_solve.cu -- A \ u for A = L*Q along one axis: every line of u along the
// operator's axis is solved with the same banded LU factors (partial pivoting,
// band storage as LAPACK's gbtrf leaves it), one thread per line.
//   b = u - A_b;  b <- P, L^-1 b (forward, with the row interchanges);  x = U^-1 b.
// Lines along axis 1 are contiguous, so consecutive threads own lines n
// elements apart; along the other axes consecutive threads own adjacent
// lines and every step is a coalesced access.  The lines are solved in
// Float64 (in x itself, or in a plan-owned Float64 workspace for Float32).
#include <cuda_runtime.h>
#include <stdint.h>

#include "deo_internal.h"

namespace deo {
namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_band_solve(int n, int kl, int ku, const double* __restrict__ ab,
                                                    const int* __restrict__ ipiv, const double* __restrict__ Ab,
                                                    int64_t stride, int64_t nlines, const T* u, T* x,
                                                    double* work) {
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= nlines) return;
    const int64_t base = line % stride + (line / stride) * stride * n;
    double* w = work ? work + base : reinterpret_cast<double*>(x) + base;  // Float64: x itself
    const int kv = kl + ku;
    for (int i = 0; i < n; ++i) w[(int64_t)i * stride] = (double)u[base + (int64_t)i * stride] - __ldg(Ab + i);
    // forward: row interchanges and the unit lower factor
    for (int j = 0; j < n - 1; ++j) {
        const int l = __ldg(ipiv + j);
        double bj = w[(int64_t)j * stride];
        if (l != j) {
            const double t = w[(int64_t)l * stride];
            w[(int64_t)l * stride] = bj;
            bj = t;
            w[(int64_t)j * stride] = bj;
        }
        const int km = min(kl, n - 1 - j);
        for (int r = 1; r <= km; ++r) {
            double& wr = w[(int64_t)(j + r) * stride];
            wr = fma(-__ldg(ab + (int64_t)(kv + r) * n + j), bj, wr);
        }
    }
    // backward: the upper factor (kv super-diagonals)
    for (int j = n - 1; j >= 0; --j) {
        const double xj = w[(int64_t)j * stride] / __ldg(ab + (int64_t)kv * n + j);
        w[(int64_t)j * stride] = xj;
        const int i0 = max(0, j - kv);
        for (int i = i0; i < j; ++i) {
            double& wi = w[(int64_t)i * stride];
            wi = fma(-__ldg(ab + (int64_t)(kv + i - j) * n + j), xj, wi);
        }
        if (work) x[base + (int64_t)j * stride] = (T)xj;
    }
}

// The same solve with the rows in flight held in registers: the forward sweep
// keeps rows j .. j+kl (the pivot search window and the rows the current
// column updates), the backward sweep rows j-kv .. j, so every element of the
// line is read once and written once per sweep (y between the sweeps lives in
// x for Float64, in the workspace for Float32).  The pivots U[j][j] enter as
// their reciprocals rdiag (the GPU has no fast FP64 divide).  W >= max(kl, kl + ku).
template <typename T, int W, int PF = 8>
__global__ void __launch_bounds__(256) k_band_solve_w(int n, int kl, int ku, const double* __restrict__ ab,
                                                      const int* __restrict__ ipiv, const double* __restrict__ Ab,
                                                      const double* __restrict__ rdiag, int64_t stride,
                                                      int64_t nlines, const T* u, T* x, double* work) {
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= nlines) return;
    const int64_t base = line % stride + (line / stride) * stride * n;
    double* y = work ? work + base : reinterpret_cast<double*>(x) + base;
    const T* ul = u + base;
    const int kv = kl + ku;
    double f[W + 1];
#pragma unroll
    for (int r = 0; r <= W; ++r) f[r] = (r <= kl && r < n) ? (double)ul[(int64_t)r * stride] - __ldg(Ab + r) : 0.0;
    // the next PF new rows' values are loaded one block of PF steps ahead
    double cur[PF], nxt[PF];
#pragma unroll
    for (int k = 0; k < PF; ++k) {
        const int jn = k + 1 + kl;
        cur[k] = jn < n ? (double)ul[(int64_t)jn * stride] - __ldg(Ab + jn) : 0.0;
    }
    for (int jb = 0; jb < n; jb += PF) {
#pragma unroll
        for (int k = 0; k < PF; ++k) {
            const int jn = jb + PF + k + 1 + kl;
            nxt[k] = jn < n ? (double)ul[(int64_t)jn * stride] - __ldg(Ab + jn) : 0.0;
        }
#pragma unroll
        for (int k = 0; k < PF; ++k) {
            const int j = jb + k;
            if (j < n) {
                const int p = __ldg(ipiv + j) - j;  // 0 .. kl
#pragma unroll
                for (int r = 1; r <= W; ++r)
                    if (r == p) {
                        const double t = f[0];
                        f[0] = f[r];
                        f[r] = t;
                    }
                const double bj = f[0];
                const int km = min(kl, n - 1 - j);
#pragma unroll
                for (int r = 1; r <= W; ++r)
                    if (r <= km) f[r] = fma(-__ldg(ab + (int64_t)(kv + r) * n + j), bj, f[r]);
                y[(int64_t)j * stride] = bj;
                const double nv = cur[k];
#pragma unroll
                for (int r = 0; r < W; ++r) f[r] = (r == kl) ? nv : f[r + 1];
                if (kl == W) f[W] = nv;
            }
        }
#pragma unroll
        for (int k = 0; k < PF; ++k) cur[k] = nxt[k];
    }
    // backward: g[r] = y[j - r]
    double g[W + 1];
#pragma unroll
    for (int r = 0; r <= W; ++r) g[r] = (r <= kv && n - 1 - r >= 0) ? y[(int64_t)(n - 1 - r) * stride] : 0.0;
#pragma unroll
    for (int k = 0; k < PF; ++k) {
        const int jn = n - 2 - kv - k;
        cur[k] = jn >= 0 ? y[(int64_t)jn * stride] : 0.0;
    }
    for (int jb = n - 1; jb >= 0; jb -= PF) {
#pragma unroll
        for (int k = 0; k < PF; ++k) {
            const int jn = jb - PF - 1 - kv - k;
            nxt[k] = jn >= 0 ? y[(int64_t)jn * stride] : 0.0;
        }
#pragma unroll
        for (int k = 0; k < PF; ++k) {
            const int j = jb - k;
            if (j >= 0) {
                const double xj = g[0] * __ldg(rdiag + j);  // one rounding more than a division, no FP64 divide
                if (work) x[base + (int64_t)j * stride] = (T)xj;
                else y[(int64_t)j * stride] = xj;
#pragma unroll
                for (int r = 1; r <= W; ++r)
                    if (r <= kv && j - r >= 0) g[r] = fma(-__ldg(ab + (int64_t)(kv - r) * n + j), xj, g[r]);
                const double nv = cur[k];
#pragma unroll
                for (int r = 0; r < W; ++r) g[r] = (r == kv) ? nv : g[r + 1];
                if (kv == W) g[W] = nv;
            }
        }
#pragma unroll
        for (int k = 0; k < PF; ++k) cur[k] = nxt[k];
    }
}

}  // namespace
}  // namespace deo

extern "C" int deo_k_band_solve(int n, int kl, int ku, const double* ab, const int* ipiv, const double* Ab,
                                const double* rdiag, int64_t stride, int64_t nlines, int dtype, const void* u, void* x,
                                double* work, void* stream) {
    if (nlines <= 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((nlines + 255) / 256);
    const int kv = kl + ku, wmax = kv > kl ? kv : kl;
#define DEO_BAND_W(W)                                                                                          \
    if (wmax <= W) {                                                                                           \
        if (dtype == 0)                                                                                        \
            deo::k_band_solve_w<double, W><<<blocks, 256, 0, st>>>(n, kl, ku, ab, ipiv, Ab, rdiag, stride,     \
                                                                   nlines, (const double*)u, (double*)x, nullptr);     \
        else                                                                                                   \
            deo::k_band_solve_w<float, W><<<blocks, 256, 0, st>>>(n, kl, ku, ab, ipiv, Ab, rdiag, stride,      \
                                                                  nlines, (const float*)u, (float*)x, work);           \
        return (int)cudaGetLastError();                                                                        \
    }
    DEO_BAND_W(2)
    DEO_BAND_W(4)
    DEO_BAND_W(8)
    DEO_BAND_W(16)
#undef DEO_BAND_W
    if (dtype == 0)
        deo::k_band_solve<double><<<blocks, 256, 0, st>>>(n, kl, ku, ab, ipiv, Ab, stride, nlines, (const double*)u,
                                                          (double*)x, nullptr);
    else
        deo::k_band_solve<float><<<blocks, 256, 0, st>>>(n, kl, ku, ab, ipiv, Ab, stride, nlines, (const float*)u,
                                                         (float*)x, work);
    return (int)cudaGetLastError();
}
