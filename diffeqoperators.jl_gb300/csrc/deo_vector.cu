// deo_vector.cu -- Gradient / Divergence / Curl of a padded array
// (vector_calculus_operators.jl, vector_calculus_convolutions.jl) and the
// pointwise vector algebra (vector_algebraic_operations.jl).
//
// One thread per output point.  Every derivative is one row of an axis
// operator's row table over the padded input (ghosts are the input's own
// first/last planes, bc_kind 2), so boundary rows, non-uniform stencils and
// coefficient vectors follow the same tables as the stencil-apply path; rows
// of a uniform operator's interior band take an unrolled loop with the same
// fused multiply-adds in the same order.  The reference's per-point additions
// into the output are replayed in its order (see VcDev).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>

#include "deo_eval.cuh"

namespace deo {
namespace {

// 0: a BC_left row, 1: an interior row, 2: a BC_right row (0-based position o)
__device__ __forceinline__ int vc_phase(int64_t o, int64_t len, int bpc) {
    return o < bpc ? 0 : (o < len - bpc ? 1 : 2);
}

// One derivative along axis a at the point whose axis-a line passes through
// flat padded index ia (the row's centre), 0-based row oa along the axis.
// NK > 0: the row is an interior row of a uniform operator, whose NK band
// weights are the term's wband.  NK == 0: the row table gives the row (its
// first tap p0, tap count and weights: boundary rows, non-uniform stencils);
// every tap is a plain load because the input holds its own ghosts.
template <typename T, int NK>
__device__ __forceinline__ T vc_deriv(const TermDev& t, const T* __restrict__ M, int64_t ia, int64_t oa) {
    const int64_t s = t.stride;
    T acc = T(0);
    if (NK > 0) {
        const T* __restrict__ xp = M + ia - (int64_t)(NK / 2) * s;
#pragma unroll
        for (int k = 0; k < NK; ++k) acc = fma(band_w<T>(t.tab[0], k), __ldg(xp + (int64_t)k * s), acc);
        return acc;
    }
    return eval_row_padded<T>(t.tab[0], M + ia - (oa + 1) * s, s, (int)oa + 1);  // the line's left ghost
}

// The 2-D / 3-D methods (vector_calculus_convolutions.jl:174-838, curl :844-1067).
// Blocks of 32 x 8 points of one (x, y) plane; blockIdx.z walks the planes.
// Used for Float64, for operators without a uniform interior band, and where
// the marching kernel's grid would not fit; launched with NK = 0 (every row
// from the row tables).  NK > 0 would give a derivative along an axis on which
// the point is an interior row the unrolled band loop.
template <typename T, int KIND, int ND, int NK>
__global__ void __launch_bounds__(256) k_vc(const VcDev V, const T* __restrict__ M, T* __restrict__ out,
                                            int overwrite) {
    const int64_t n0 = V.len[0], n1 = V.len[1], n2 = ND == 3 ? V.len[2] : 1;
    const int64_t o0 = (int64_t)blockIdx.x * 32 + threadIdx.x % 32;
    if (o0 >= n0) return;
    for (int64_t o1 = (int64_t)blockIdx.y * 8 + threadIdx.x / 32; o1 < n1; o1 += (int64_t)gridDim.y * 8) {
        for (int64_t o2 = blockIdx.z; o2 < n2; o2 += gridDim.z) {
            const int64_t o[3] = {o0, o1, o2};
            const int64_t n = o0 + n0 * (o1 + n1 * o2);
            // other axes at the padded index equal to the output index; +1 along the differentiated axis
            int64_t q = 0;
#pragma unroll
            for (int b = 0; b < ND; ++b) q += o[b] * V.pstride[b];
            int ph[ND];
#pragma unroll
            for (int a = 0; a < ND; ++a) ph[a] = vc_phase(o[a], V.len[a], V.bpc);
            auto D = [&](const TermDev& t, const T* x, int a) {
                return (NK > 0 && ph[a] == 1) ? vc_deriv<T, NK>(t, x, q + V.pstride[a], o[a])
                                              : vc_deriv<T, 0>(t, x, q + V.pstride[a], o[a]);
            };
            if (KIND == DEO_VC_GRADIENT) {
#pragma unroll
                for (int a = 0; a < ND; ++a) {
                    const T d = D(V.t[a], M, a);
                    T* y = out + n + a * V.ovol;
                    *y = overwrite ? zero_fix(d) : *y + d;
                }
            } else if (KIND == DEO_VC_DIVERGENCE) {
                T d[ND];
#pragma unroll
                for (int a = 0; a < ND; ++a) d[a] = D(V.t[a], M + a * V.pvol, a);
                T acc = overwrite ? T(0) : out[n];
                bool first = overwrite != 0;  // 0 + x is x up to the sign of zero
#pragma unroll
                for (int p = 0; p < 3; ++p)
#pragma unroll
                    for (int a = 0; a < ND; ++a)
                        if (ph[a] == p) {
                            acc = first ? zero_fix(d[a]) : acc + d[a];
                            first = false;
                        }
                out[n] = acc;
            } else {
                // curl component c = (D_{a1} u[c1]) sign1 + (D_{a2} u[c2]) sign2, a1 < a2:
                //   x1: +D2 u3, -D3 u2;  x2: -D1 u3, +D3 u1;  x3: +D1 u2, -D2 u1
                constexpr int A1[3] = {1, 0, 0}, A2[3] = {2, 2, 1};
                constexpr int C1[3] = {2, 2, 1}, C2[3] = {1, 0, 0};
                constexpr bool N1[3] = {false, true, false}, N2[3] = {true, false, true};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const int a1 = A1[c], a2 = A2[c];
                    const T e1 = D(N1[c] ? V.tn[a1] : V.t[a1], M + C1[c] * V.pvol, a1);
                    const T e2 = D(N2[c] ? V.tn[a2] : V.t[a2], M + C2[c] * V.pvol, a2);
                    T* y = out + n + c * V.ovol;
                    const T f = ph[a1] <= ph[a2] ? e1 : e2, g = ph[a1] <= ph[a2] ? e2 : e1;
                    *y = (overwrite ? zero_fix(f) : *y + f) + g;
                }
            }
        }
    }
}

// The same methods for operators with a uniform interior band of NK taps.
// Each thread owns one column across the axes other than the last and marches
// along the last axis (axis ND) over zb positions, keeping the taps along
// that axis in a register queue (one new load per step); taps along x are
// contiguous (compile-time offsets) and taps along y use offsets computed once
// per thread, so an interior point costs its loads and fused multiply-adds.
// A derivative along an axis on which the point is an interior row takes the
// unrolled band loop; on a boundary row, the row table.  ND = 3: blocks of
// 32 x 8 columns, blockIdx.z = the march chunk; ND = 2: 256 columns,
// blockIdx.y = the chunk.  Same fused multiply-adds in the same order as k_vc.
template <typename T, int KIND, int ND, int NK>
__global__ void __launch_bounds__(256) k_vc_march(const VcDev V, const T* __restrict__ M, T* __restrict__ out,
                                                  int overwrite, int zb) {
    constexpr int MA = ND - 1;                           // marching axis
    constexpr int NQ = KIND == DEO_VC_CURL ? 2 : 1;      // queued input components
    constexpr int MID = NK / 2;
    int64_t o[3] = {0, 0, 0};
    if (ND == 3) {
        o[0] = (int64_t)blockIdx.x * 32 + threadIdx.x % 32;
        o[1] = (int64_t)blockIdx.y * 8 + threadIdx.x / 32;
    } else {
        o[0] = (int64_t)blockIdx.x * 256 + threadIdx.x;
    }
#pragma unroll
    for (int b = 0; b < MA; ++b)
        if (o[b] >= V.len[b]) return;
    const int64_t chunk = ND == 3 ? blockIdx.z : blockIdx.y;
    const int64_t mlo = chunk * zb, mhi = min(mlo + zb, V.len[MA]);
    int ph[ND];
#pragma unroll
    for (int b = 0; b < MA; ++b) ph[b] = vc_phase(o[b], V.len[b], V.bpc);
    int64_t col = 0;  // other axes at the padded index equal to the output index
#pragma unroll
    for (int b = 0; b < MA; ++b) col += o[b] * V.pstride[b];
    const int64_t ocol = o[0] + (ND == 3 ? V.len[0] * o[1] : 0);
    const int64_t ms = V.pstride[MA], oms = ND == 3 ? V.len[0] * V.len[1] : V.len[0];
    const int64_t ys = V.pstride[1];
    // queued components: gradient M; divergence u[ND]; curl u2 (for x1 -= D3 u2) and u1 (for x2 += D3 u1)
    int64_t qoff[NQ];
    qoff[0] = KIND == DEO_VC_GRADIENT ? 0 : (KIND == DEO_VC_DIVERGENCE ? MA * V.pvol : V.pvol);
    if (NQ == 2) qoff[NQ - 1] = 0;
    T Q[NQ][NK];
    bool qvalid = false;
    for (int64_t om = mlo; om < mhi; ++om) {
        o[MA] = om;
        ph[MA] = vc_phase(om, V.len[MA], V.bpc);
        const bool mid_row = ph[MA] == 1;  // uniform over the block
        const int64_t q = col + om * ms;
        const int64_t n = ocol + om * oms;
        if (mid_row) {
            if (!qvalid) {
#pragma unroll
                for (int c = 0; c < NQ; ++c)
#pragma unroll
                    for (int k = 0; k < NK; ++k) Q[c][k] = __ldg(M + qoff[c] + q + (int64_t)(k + 1 - MID) * ms);
            } else {
#pragma unroll
                for (int c = 0; c < NQ; ++c) {
#pragma unroll
                    for (int k = 0; k < NK - 1; ++k) Q[c][k] = Q[c][k + 1];
                    Q[c][NK - 1] = __ldg(M + qoff[c] + q + (int64_t)(MID + 1) * ms);
                }
            }
        }
        qvalid = mid_row;
        // derivative along axis a of the input at component offset coff (queue qi along the marching axis)
        auto D = [&](const TermDev& t, int64_t coff, int a, int qi) -> T {
            if (ph[a] != 1) return vc_deriv<T, 0>(t, M + coff, q + V.pstride[a], o[a]);
            T acc = T(0);
            if (a == MA) {
#pragma unroll
                for (int k = 0; k < NK; ++k) acc = fma(band_w<T>(t.tab[0], k), Q[qi][k], acc);
            } else if (a == 0) {  // pstride[0] == 1
                const T* __restrict__ xp = M + coff + q + (1 - MID);
#pragma unroll
                for (int k = 0; k < NK; ++k) acc = fma(band_w<T>(t.tab[0], k), __ldg(xp + k), acc);
            } else {
                const T* __restrict__ yp = M + coff + q + (1 - MID) * ys;
#pragma unroll
                for (int k = 0; k < NK; ++k) acc = fma(band_w<T>(t.tab[0], k), __ldg(yp + k * ys), acc);
            }
            return acc;
        };
        if (KIND == DEO_VC_GRADIENT) {
#pragma unroll
            for (int a = 0; a < ND; ++a) {
                const T d = D(V.t[a], 0, a, 0);
                T* y = out + n + a * V.ovol;
                *y = overwrite ? zero_fix(d) : *y + d;
            }
        } else if (KIND == DEO_VC_DIVERGENCE) {
            T d[ND];
#pragma unroll
            for (int a = 0; a < ND; ++a) d[a] = D(V.t[a], a * V.pvol, a, 0);
            T acc = overwrite ? T(0) : out[n];
            bool first = overwrite != 0;  // 0 + x is x up to the sign of zero
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int a = 0; a < ND; ++a)
                    if (ph[a] == p) {
                        acc = first ? zero_fix(d[a]) : acc + d[a];
                        first = false;
                    }
            out[n] = acc;
        } else {
            // x1: +D2 u3, -D3 u2 (queue 0);  x2: -D1 u3, +D3 u1 (queue 1);  x3: +D1 u2, -D2 u1
            const T x1a = D(V.t[1], 2 * V.pvol, 1, 0), x1b = D(V.tn[2], V.pvol, 2, 0);
            const T x2a = D(V.tn[0], 2 * V.pvol, 0, 0), x2b = D(V.t[2], 0, 2, NQ - 1);
            const T x3a = D(V.t[0], V.pvol, 0, 0), x3b = D(V.tn[1], 0, 1, 0);
            const T e1[3] = {x1a, x2a, x3a}, e2[3] = {x1b, x2b, x3b};
            constexpr int A1[3] = {1, 0, 0}, A2[3] = {2, 2, 1};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                T* y = out + n + c * V.ovol;
                const bool in_order = ph[A1[c]] <= ph[A2[c]];
                const T f = in_order ? e1[c] : e2[c], g = in_order ? e2[c] : e1[c];
                *y = (overwrite ? zero_fix(f) : *y + f) + g;
            }
        }
    }
}

// The generic per-line methods (vector_calculus_convolutions.jl:1-170): any N,
// other axes read at index + 1, operators added in axis order.
template <typename T, int KIND>
__global__ void __launch_bounds__(256) k_vc_lines(const VcDev V, const T* __restrict__ M, T* __restrict__ out,
                                                  int overwrite) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= V.ovol) return;
    int64_t o[8];
    int64_t r = n, q = 0;
    for (int b = 0; b < V.nd; ++b) {
        o[b] = (b == V.nd - 1) ? r : r % V.len[b];
        r = (b == V.nd - 1) ? 0 : r / V.len[b];
        q += (o[b] + 1) * V.pstride[b];
    }
    if (KIND == DEO_VC_GRADIENT) {
        for (int a = 0; a < V.nd; ++a) {
            const T d = eval_term<T>(V.t[a], M, q, (int)o[a] + 1);
            T* y = out + n + a * V.ovol;
            *y = overwrite ? zero_fix(d) : *y + d;
        }
    } else {
        T acc = overwrite ? T(0) : out[n];
        for (int a = 0; a < V.nd; ++a) {
            const T d = eval_term<T>(V.t[a], M + a * V.pvol, q, (int)o[a] + 1);
            acc = (a == 0 && overwrite) ? zero_fix(d) : acc + d;
        }
        out[n] = acc;
    }
}

// L*M / mul!(x_temp, L, M; overwrite) on an already padded array M
// (derivative_operator_functions.jl:17-69, 150-163; convolutions.jl:17-22 for
// vectors): one thread per output point; its line along `axis` starts at the
// left ghost, other axes at the output index + off (1 where M is padded on that
// axis, so its edge planes are skipped; `coff` = sum of those offsets times the
// strides); the row from the operator's table (generic methods).
template <typename T>
__global__ void __launch_bounds__(256) k_padded(const VcDev V, int axis, int64_t coff, const T* __restrict__ M,
                                                T* __restrict__ out, int overwrite) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= V.ovol) return;
    int64_t r = n, ls = coff, oa = 0;
    for (int b = 0; b < V.nd; ++b) {
        const int64_t o = (b == V.nd - 1) ? r : r % V.len[b];
        r = (b == V.nd - 1) ? 0 : r / V.len[b];
        if (b == axis) oa = o;
        else ls += o * V.pstride[b];
    }
    const T d = eval_row_padded<T>(V.t[0].tab[0], M + ls, V.pstride[axis], (int)oa + 1);
    out[n] = overwrite ? zero_fix(d) : d + out[n];
}

// Products rounded before the sums (no contraction), as plain Julia code does.
template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b);
template <>
__device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <>
__device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b);
template <>
__device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <>
__device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }
template <typename T>
__device__ __forceinline__ T sub_rn(T a, T b);
template <>
__device__ __forceinline__ double sub_rn<double>(double a, double b) { return __dsub_rn(a, b); }
template <>
__device__ __forceinline__ float sub_rn<float>(float a, float b) { return __fsub_rn(a, b); }

// dot_product! / square_norm! (vector_algebraic_operations.jl:11-28, :54-62)
template <typename T, bool NORM>
__global__ void __launch_bounds__(256) k_dot(int64_t npts, int ncomp, const T* __restrict__ A, const T* __restrict__ B,
                                             T* __restrict__ u) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npts) return;
    T acc = T(0);
    for (int i = 0; i < ncomp; ++i) {
        const T a = A[n + i * npts];
        acc = add_rn(acc, mul_rn(a, NORM ? a : B[n + i * npts]));
    }
    u[n] = NORM ? sqrt(acc) : acc;
}

// cross_product! (vector_algebraic_operations.jl:39-52)
template <typename T>
__global__ void __launch_bounds__(256) k_cross(int64_t npts, const T* __restrict__ A, const T* __restrict__ B,
                                               T* __restrict__ u) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= npts) return;
    const T a1 = A[n], a2 = A[n + npts], a3 = A[n + 2 * npts];
    const T b1 = B[n], b2 = B[n + npts], b3 = B[n + 2 * npts];
    u[n] = sub_rn(mul_rn(a2, b3), mul_rn(a3, b2));
    u[n + npts] = sub_rn(mul_rn(a3, b1), mul_rn(a1, b3));
    u[n + 2 * npts] = sub_rn(mul_rn(a1, b2), mul_rn(a2, b1));
}

template <typename T, int KIND, int ND>
void launch_tiled(const VcDev& V, const T* M, T* out, int ow, cudaStream_t st) {
    // marching kernel: columns x chunks of the last axis within the grid limits
    const int64_t nm = V.len[ND - 1];
    const int64_t ncol1 = ND == 3 ? (V.len[1] + 7) / 8 : 1;
    const int64_t ncols = (ND == 3 ? (V.len[0] + 31) / 32 : (V.len[0] + 255) / 256) * ncol1;
    // chunks of the march: short enough for many waves of blocks (the last wave's
    // idle SMs are the tail), long enough to amortise the queue's first fill
    int64_t zb = 4;
    while (zb < 32 && ncols * ((nm + 2 * zb - 1) / (2 * zb)) >= 8192) zb *= 2;
    while ((nm + zb - 1) / zb > 65535) zb *= 2;
    // Float64 is FP64-bound either way and the per-point row-table kernel keeps
    // the FP64 pipe busier (gradient 548 us against 624 us at 256^3), so the
    // marching kernel serves Float32 only
    if (V.band_nk > 0 && ncol1 <= 65535 && !std::is_same<T, double>::value) {
        const unsigned chunks = (unsigned)((nm + zb - 1) / zb);
        const dim3 grid = ND == 3 ? dim3((unsigned)((V.len[0] + 31) / 32), (unsigned)ncol1, chunks)
                                  : dim3((unsigned)((V.len[0] + 255) / 256), chunks, 1);
        const int z = (int)zb;
        switch (V.band_nk) {
            case 3: k_vc_march<T, KIND, ND, 3><<<grid, 256, 0, st>>>(V, M, out, ow, z); return;
            case 5: k_vc_march<T, KIND, ND, 5><<<grid, 256, 0, st>>>(V, M, out, ow, z); return;
            case 7: k_vc_march<T, KIND, ND, 7><<<grid, 256, 0, st>>>(V, M, out, ow, z); return;
            case 9: k_vc_march<T, KIND, ND, 9><<<grid, 256, 0, st>>>(V, M, out, ow, z); return;
            default: break;
        }
    }
    const int64_t n2 = ND == 3 ? V.len[2] : 1;
    dim3 grid((unsigned)((V.len[0] + 31) / 32), (unsigned)std::min<int64_t>((V.len[1] + 7) / 8, 65535),
              (unsigned)std::min<int64_t>(n2, 65535));
    k_vc<T, KIND, ND, 0><<<grid, 256, 0, st>>>(V, M, out, ow);
}

template <typename T>
int launch_vc(const VcDev& V, const void* Mv, void* outv, int ow, cudaStream_t st) {
    const T* M = static_cast<const T*>(Mv);
    T* out = static_cast<T*>(outv);
    if (V.quirk && V.nd == 2) {
        if (V.kind == DEO_VC_GRADIENT) launch_tiled<T, DEO_VC_GRADIENT, 2>(V, M, out, ow, st);
        else launch_tiled<T, DEO_VC_DIVERGENCE, 2>(V, M, out, ow, st);
    } else if (V.quirk && V.nd == 3) {
        if (V.kind == DEO_VC_GRADIENT) launch_tiled<T, DEO_VC_GRADIENT, 3>(V, M, out, ow, st);
        else if (V.kind == DEO_VC_DIVERGENCE) launch_tiled<T, DEO_VC_DIVERGENCE, 3>(V, M, out, ow, st);
        else launch_tiled<T, DEO_VC_CURL, 3>(V, M, out, ow, st);
    } else {
        const unsigned blocks = (unsigned)((V.ovol + 255) / 256);
        if (V.kind == DEO_VC_GRADIENT) k_vc_lines<T, DEO_VC_GRADIENT><<<blocks, 256, 0, st>>>(V, M, out, ow);
        else k_vc_lines<T, DEO_VC_DIVERGENCE><<<blocks, 256, 0, st>>>(V, M, out, ow);
    }
    return (int)cudaGetLastError();
}

}  // namespace
}  // namespace deo

extern "C" int deo_k_vector_calculus(const deo::VcDev* V, int dtype, const void* M, void* out, int overwrite,
                                     void* stream) {
    if (V->ovol <= 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return dtype == 0 ? deo::launch_vc<double>(*V, M, out, overwrite, st)
                      : deo::launch_vc<float>(*V, M, out, overwrite, st);
}

extern "C" int deo_k_padded_apply(const deo::VcDev* V, int axis, int64_t coff, int dtype, const void* M, void* out,
                                  int overwrite, void* stream) {
    if (V->ovol <= 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((V->ovol + 255) / 256);
    if (dtype == 0)
        deo::k_padded<double><<<blocks, 256, 0, st>>>(*V, axis, coff, (const double*)M, (double*)out, overwrite);
    else
        deo::k_padded<float><<<blocks, 256, 0, st>>>(*V, axis, coff, (const float*)M, (float*)out, overwrite);
    return (int)cudaGetLastError();
}

extern "C" int deo_k_vector_algebra(int op, int dtype, int64_t npts, int ncomp, const void* A, const void* B, void* u,
                                    void* stream) {
    if (npts <= 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((npts + 255) / 256);
    if (dtype == 0) {
        const double *a = (const double*)A, *b = (const double*)B;
        if (op == 0) deo::k_dot<double, false><<<blocks, 256, 0, st>>>(npts, ncomp, a, b, (double*)u);
        else if (op == 1) deo::k_cross<double><<<blocks, 256, 0, st>>>(npts, a, b, (double*)u);
        else deo::k_dot<double, true><<<blocks, 256, 0, st>>>(npts, ncomp, a, a, (double*)u);
    } else {
        const float *a = (const float*)A, *b = (const float*)B;
        if (op == 0) deo::k_dot<float, false><<<blocks, 256, 0, st>>>(npts, ncomp, a, b, (float*)u);
        else if (op == 1) deo::k_cross<float><<<blocks, 256, 0, st>>>(npts, a, b, (float*)u);
        else deo::k_dot<float, true><<<blocks, 256, 0, st>>>(npts, ncomp, a, a, (float*)u);
    }
    return (int)cudaGetLastError();
}
