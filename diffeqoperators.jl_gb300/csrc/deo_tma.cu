// deo_tma.cu -- TMA-fed fused apply for plans whose terms are centred bands on
// axes 1..NT of a 2-D/3-D array (the Laplacian-type plans, UniPlan::lap).
//
// Each CTA owns a TX x TY column of the grid and walks a chunk of z.  One
// elected thread streams z-planes of the (TX + 2HR) x (TY + 2H) tile (HR = H
// rounded up to 16 bytes, the TMA alignment of the innermost coordinate) into a
// shared-memory ring of P slots with cp.async.bulk.tensor, each slot guarded by
// an mbarrier; the ring keeps P - (2H+1) planes in flight ahead of the plane
// being evaluated.  Planes outside the array arrive zero-filled (TMA OOB fill),
// so loads need no bounds checks.  A slot is refilled only after a barrier
// that follows every thread's last read of it (its values are in registers by
// then), so the copy needs no cross-proxy fence: nothing written by the
// threads is read by the copy.  Every mbarrier wait is bounded: on timeout
// the CTA records bit 0 of g_deo_status, waits (bounded) for its own copies
// still in flight and returns.
//
// Interior points (band rows along every axis) are evaluated from the ring:
//   * FMA mode: the reference's per-term tap order, bit-identical to the
//     generic row-table evaluator;
//   * ENS mode (Float64, all terms share one band): the NT neighbours at
//     offset o (one per axis) have the same weight w[o], so
//       r = c0 * u0 + sum_{o != 0} w[o] * S_o,
//     where S_o is their sum computed exactly in 64-bit integer arithmetic
//     (aligned to the largest of the NT exponents; bits below 2^-59 of that
//     value are dropped) and rounded once.  This takes 2H + 1 FP64
//     instructions per point instead of NT*(2H+1) + NT - 1, which is what
//     bounds a Float64 stencil on this part (1.68 DFMA/clk/SM).
// Points on boundary rows (the boundary shell) are left to deo_shell.cu.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "deo_eval.cuh"
#include "deo_fx.cuh"
#include "deo_lap.cuh"
#include "deo_ptx.cuh"

namespace deo {

__device__ unsigned int g_deo_status;  // bit 0: a bounded mbarrier wait gave up

// Sum of N doubles, exact up to bits below 2^-59 of the largest, rounded
// once to nearest.  ok = false for Inf/NaN inputs or a result that is
// subnormal or overflows (the caller then uses the FMA chain).
template <int N>
__device__ __forceinline__ double ens_sum(const double (&v)[N], bool& ok) {
    int e[N];
    unsigned long long m[N];
    int emax = 1;
    bool special = false;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(v[j]);
        const int ex = (int)((b >> 52) & 0x7ffULL);
        special |= (ex == 0x7ff);
        const unsigned long long fr = b & 0xFFFFFFFFFFFFFULL;
        m[j] = ex ? (fr | (1ULL << 52)) : fr;
        e[j] = ex ? ex : 1;
        emax = max(emax, e[j]);
    }
    long long acc = 0;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const int d = emax - e[j];
        const unsigned long long t = d < 64 ? ((m[j] << 7) >> d) : 0ULL;
        acc += (__double_as_longlong(v[j]) < 0) ? -(long long)t : (long long)t;
    }
    if (special) {
        ok = false;
        return 0.0;
    }
    if (acc == 0) {
        ok = true;
        return 0.0;
    }
    unsigned long long a = acc < 0 ? 0ULL - (unsigned long long)acc : (unsigned long long)acc;
    const int lz = __clzll((long long)a);
    a <<= lz;
    unsigned long long mant = a >> 11;
    const unsigned long long rb = a & 0x7FFULL;
    int bexp = emax + 4 - lz;  // value = acc * 2^(emax - 1082)
    if (rb > 0x400ULL || (rb == 0x400ULL && (mant & 1ULL))) mant += 1ULL;
    if (mant == (1ULL << 53)) {
        mant >>= 1;
        bexp += 1;
    }
    if (bexp <= 0 || bexp >= 2047) {
        ok = false;
        return 0.0;
    }
    unsigned long long bits = ((unsigned long long)bexp << 52) | (mant & 0xFFFFFFFFFFFFFULL);
    if (acc < 0) bits |= 0x8000000000000000ULL;
    ok = true;
    return __longlong_as_double((long long)bits);
}

template <typename T, int H>
struct TmaCfg {
    static constexpr int TX = 32, TY = 8;
    static constexpr int ES = (int)sizeof(T);
    static constexpr int HR = ((H * ES + 15) / 16) * 16 / ES;  // x halo rounded up to 16 bytes
    static constexpr int BX = TX + 2 * HR, BY = TY + 2 * H;
    static constexpr int PLANE = BX * BY;
    static constexpr int PLANE_BYTES = PLANE * ES;
    static constexpr int SLOT = ((PLANE_BYTES + 127) / 128) * 128;
    static constexpr int PMIN = 2 * H + 2;
    static constexpr int PBASE = ES == 8 ? 8 : 16;
    static constexpr int P = PMIN <= PBASE ? PBASE : 16;  // power of two >= 2H+2
    static constexpr int SMEM = P * SLOT;
};

}  // namespace deo

#include "deo_bfx.cuh"

namespace deo {

template <typename T, int H, int NT, bool ENS>
__global__ void __launch_bounds__(256) k_lap_tma(const __grid_constant__ CUtensorMap tmap,
                                                 const __grid_constant__ UniPlan U, const LapGrid g,
                                                 const PlanDev* __restrict__ Pd, const T* __restrict__ u,
                                                 T* __restrict__ du, int overwrite) {
    using C = TmaCfg<T, H>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[C::P];
    constexpr int HZ = NT == 3 ? H : 0;  // z halo (2-D plans stream one plane)
    const int nx = (int)U.n[0], ny = (int)U.n[1], nz = (int)U.n[2];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * C::TX + tx;
    const int64_t sxy = (int64_t)nx * ny;
    const int cc = (ty + H) * C::BX + tx + C::HR;  // this thread's point inside a plane slot
    if (tid == 0) {
        for (int s = 0; s < C::P; ++s) mbar_init(&mbar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto slot = [&](int gj) -> const T* {
        return reinterpret_cast<const T*>(smem + (gj & (C::P - 1)) * C::SLOT);
    };
    int base = 0;        // running plane count of this CTA (ring position of the unit's plane 0)
    int issued = 0;      // planes issued in the current unit (thread 0)
    int waited = 0;      // planes of the current unit known complete
    bool aborted = false;
    for (int k = blockIdx.x; k < g.units && !aborted; k += gridDim.x) {
        const int unit = (int)(((long long)k * g.perm) % g.units);
        const int txi = unit % g.tiles_x;
        const int rest = unit / g.tiles_x;
        const int tyi = rest % g.tiles_y;
        const int ci = rest / g.tiles_y;
        const int x0 = txi * C::TX, y0 = tyi * C::TY;
        const int x = x0 + tx, y = y0 + ty;
        const int z0 = ci * g.zc;
        const int z1 = min(z0 + g.zc, nz);
        const int npl = (z1 - z0) + 2 * HZ;
        const bool inxy = x < nx && y < ny;
        const int64_t col = (int64_t)y * nx + x;
        // rows of this thread along x and y, and whether they are band rows without ghosts
        const bool bx = x + 1 >= U.t[0].flo && x + 1 <= U.t[0].fhi;
        const bool by = y + 1 >= U.t[1].flo && y + 1 <= U.t[1].fhi;
        if (tid == 0) {
            const int pre = min(C::P, npl);
            for (int j = 0; j < pre; ++j) {
                const int s = (base + j) & (C::P - 1);
                mbar_expect_tx(&mbar[s], C::PLANE_BYTES);
                tma_load_3d(smem + s * C::SLOT, &tmap, &mbar[s], x0 - C::HR, y0 - H, z0 - HZ + j);
            }
            issued = pre;
        }
        waited = 0;
        for (int z = z0; z < z1; ++z) {
            const int jc = z - z0 + HZ;
            bool timeout = false;
            while (waited <= jc + HZ) {
                const int gj = base + waited;
                const uint32_t par = (uint32_t)((gj / C::P) & 1);
                uint32_t it = 0;
                while (!mbar_try_wait(&mbar[gj & (C::P - 1)], par)) {
                    if (++it > (1u << 22)) {
                        timeout = true;
                        break;
                    }
                }
                if (timeout) break;
                ++waited;
            }
            const bool bz = (NT < 3) || (z + 1 >= U.t[NT - 1].flo && z + 1 <= U.t[NT - 1].fhi);
            if (inxy && !timeout && bx && by && bz) {
                // interior point: every term reads band rows only (boundary shell: k_shell)
                const int64_t idx = (int64_t)z * sxy + col;
                const T* pc = slot(base + jc);
                T total;
                bool done = false;
                if constexpr (ENS) {
                    double r = U.ens_c0[(1 << NT) - 1] * (double)pc[cc];
                    bool ok = true;
#pragma unroll
                    for (int k = 1; k <= H; ++k) {
                        double vm[NT], vp[NT];
                        vm[0] = (double)pc[cc - k];
                        vp[0] = (double)pc[cc + k];
                        vm[1] = (double)pc[cc - k * C::BX];
                        vp[1] = (double)pc[cc + k * C::BX];
                        if constexpr (NT == 3) {
                            vm[2] = (double)slot(base + jc - k)[cc];
                            vp[2] = (double)slot(base + jc + k)[cc];
                        }
                        bool okm, okp;
                        const double sm = ens_sum<NT>(vm, okm);
                        const double sp = ens_sum<NT>(vp, okp);
                        ok = ok && okm && okp;
                        r = fma(U.ens_w[H - k], sm, r);
                        r = fma(U.ens_w[H + k], sp, r);
                    }
                    if (ok) {
                        total = (T)zero_fix(r);
                        done = true;
                    }
                }
                if (!done) {
                    // the reference's per-term tap order (also the fallback for Inf/NaN or extreme exponents)
#pragma unroll
                    for (int t = 0; t < NT; ++t) {
                        T acc = T(0);
#pragma unroll
                        for (int k = 0; k < 2 * H + 1; ++k) {
                            const int o = k - H;
                            const T v = t == 0 ? pc[cc + o] : (t == 1 ? pc[cc + o * C::BX] : slot(base + jc + o)[cc]);
                            acc = fma(uni_w<T>(U.t[t], k), v, acc);
                        }
                        total = (t == 0) ? acc : total + acc;
                    }
                    total = zero_fix(total);
                }
                du[idx] = overwrite ? total : total + du[idx];
            }
            if (__syncthreads_or(timeout)) {
                aborted = true;
                break;
            }
            // plane jc - HZ has left the window: refill its slot
            if (tid == 0) {
                const int jn = (jc - HZ) + C::P;
                if (jn < npl) {
                    const int s = (base + jn) & (C::P - 1);
                    mbar_expect_tx(&mbar[s], C::PLANE_BYTES);
                    tma_load_3d(smem + s * C::SLOT, &tmap, &mbar[s], x0 - C::HR, y0 - H, z0 - HZ + jn);
                    issued = jn + 1;
                }
            }
        }
        if (!aborted) base += npl;
    }
    if (aborted && tid == 0) {
        atomicOr(&g_deo_status, 1u);
        // wait (bounded) for this CTA's copies still in flight before its shared memory is released
        for (int j = waited; j < issued; ++j) {
            const int gj = base + j;
            const uint32_t par = (uint32_t)((gj / C::P) & 1);
            for (uint32_t it = 0; it < (1u << 22); ++it)
                if (mbar_try_wait(&mbar[gj & (C::P - 1)], par)) break;
        }
    }
}

// ---------------------------------------------------------------------------
// Exact-sum kernel, v2 (Float64): each value is decomposed ONCE, when its
// plane lands, into (e, m) with value = m * 2^(e - 1082) and m = +-mantissa
// << 7, kept in a second shared-memory ring.  A group of NT equal-weight
// neighbours then costs: max of NT exponents, NT arithmetic shifts, NT-1
// 64-bit adds, one int64 -> double conversion (I2F, rounds once) and one FMA
// with the weight scaled by 2^(emax - 1082) through its exponent bits.
// Interior points only; every other point takes the raw-ring paths.
// ---------------------------------------------------------------------------
template <int H>
struct Ens2Cfg {
    using R = TmaCfg<double, H>;
    static constexpr int DP = 8;                     // decomposed planes kept (>= 2H+1)
    static constexpr int DSLOT_M = R::PLANE * 8;     // bytes of mantissas per slot
    static constexpr int DSLOT_E = R::PLANE * 4;     // bytes of exponents per slot
    static constexpr int DSLOT = ((DSLOT_M + DSLOT_E + 127) / 128) * 128;
    static constexpr int SMEM = R::SMEM + DP * DSLOT;
};

__device__ __forceinline__ void decompose(double v, long long& m, int& e) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int ex = (int)((b >> 52) & 0x7ffULL);
    const unsigned long long fr = b & 0xFFFFFFFFFFFFFULL;
    const long long mag = (long long)((ex ? (fr | (1ULL << 52)) : fr) << 7);
    m = ((long long)b < 0) ? -mag : mag;
    e = ex == 0x7ff ? 4095 : (ex ? ex : 1);  // 4095 marks Inf/NaN: forces the fallback
}

template <int NT>
__device__ __forceinline__ bool ens2_group(const long long (&m)[NT], const int (&e)[NT], double w, double& r) {
    int emax = e[0];
#pragma unroll
    for (int j = 1; j < NT; ++j) emax = max(emax, e[j]);
    long long acc = 0;
#pragma unroll
    for (int j = 0; j < NT; ++j) acc += m[j] >> min(emax - e[j], 63);
    if (emax >= 2047) return false;  // an Inf/NaN input
    if (acc == 0) return true;       // the group contributes exactly zero
    // weight * 2^(emax - 1082) by its exponent field (weights are nonzero normals, checked on the host)
    const long long wb = __double_as_longlong(w);
    const int ew = (int)((wb >> 52) & 0x7ff) + emax - 1082;
    if (ew < 1 || ew > 2046) return false;
    const double ws = __longlong_as_double(wb + ((long long)(emax - 1082) << 52));
    r = fma(ws, __ll2double_rn(acc), r);
    return true;
}

template <int H, int NT>
__global__ void __launch_bounds__(256) k_lap_ens2(const __grid_constant__ CUtensorMap tmap,
                                                  const __grid_constant__ UniPlan U, const LapGrid g,
                                                  const PlanDev* __restrict__ Pd, const double* __restrict__ u,
                                                  double* __restrict__ du, int overwrite) {
    using C = TmaCfg<double, H>;
    using E = Ens2Cfg<H>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[C::P];
    constexpr int HZ = NT == 3 ? H : 0;
    unsigned char* dsm = smem + C::SMEM;
    const int nx = (int)U.n[0], ny = (int)U.n[1], nz = (int)U.n[2];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * C::TX + tx;
    const int64_t sxy = (int64_t)nx * ny;
    const int cc = (ty + H) * C::BX + tx + C::HR;
    if (tid == 0) {
        for (int s = 0; s < C::P; ++s) mbar_init(&mbar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto raw = [&](int gj) -> const double* {
        return reinterpret_cast<const double*>(smem + (gj & (C::P - 1)) * C::SLOT);
    };
    auto dm = [&](int gj) -> long long* {
        return reinterpret_cast<long long*>(dsm + (gj & (E::DP - 1)) * E::DSLOT);
    };
    auto de = [&](int gj) -> int* {
        return reinterpret_cast<int*>(dsm + (gj & (E::DP - 1)) * E::DSLOT + E::DSLOT_M);
    };
    int base = 0, issued = 0, waited = 0, converted = 0;
    bool aborted = false;
    for (int k = blockIdx.x; k < g.units && !aborted; k += gridDim.x) {
        const int unit = (int)(((long long)k * g.perm) % g.units);
        const int txi = unit % g.tiles_x;
        const int rest = unit / g.tiles_x;
        const int tyi = rest % g.tiles_y;
        const int ci = rest / g.tiles_y;
        const int x0 = txi * C::TX, y0 = tyi * C::TY;
        const int x = x0 + tx, y = y0 + ty;
        const int z0 = ci * g.zc;
        const int z1 = min(z0 + g.zc, nz);
        const int npl = (z1 - z0) + 2 * HZ;
        const bool inxy = x < nx && y < ny;
        const int64_t col = (int64_t)y * nx + x;
        const bool bx = x + 1 >= U.t[0].flo && x + 1 <= U.t[0].fhi;
        const bool by = y + 1 >= U.t[1].flo && y + 1 <= U.t[1].fhi;
        if (tid == 0) {
            const int pre = min(C::P, npl);
            for (int j = 0; j < pre; ++j) {
                const int s = (base + j) & (C::P - 1);
                mbar_expect_tx(&mbar[s], C::PLANE_BYTES);
                tma_load_3d(smem + s * C::SLOT, &tmap, &mbar[s], x0 - C::HR, y0 - H, z0 - HZ + j);
            }
            issued = pre;
        }
        waited = 0;
        converted = 0;
        for (int z = z0; z < z1; ++z) {
            const int jc = z - z0 + HZ;
            bool timeout = false;
            while (waited <= jc + HZ) {
                const int gj = base + waited;
                const uint32_t par = (uint32_t)((gj / C::P) & 1);
                uint32_t it = 0;
                while (!mbar_try_wait(&mbar[gj & (C::P - 1)], par)) {
                    if (++it > (1u << 22)) {
                        timeout = true;
                        break;
                    }
                }
                if (timeout) break;
                ++waited;
            }
            // decompose the planes that arrived (shared by the whole CTA)
            if (!timeout) {
                for (; converted < waited; ++converted) {
                    const int gj = base + converted;
                    const double* rp = raw(gj);
                    long long* mp = dm(gj);
                    int* ep = de(gj);
                    for (int q = tid; q < C::PLANE; q += C::TX * C::TY) decompose(rp[q], mp[q], ep[q]);
                }
            }
            if (__syncthreads_or(timeout)) {
                aborted = true;
                break;
            }
            const bool bz = (NT < 3) || (z + 1 >= U.t[NT - 1].flo && z + 1 <= U.t[NT - 1].fhi);
            if (inxy && bx && by && bz) {
                const int64_t idx = (int64_t)z * sxy + col;
                const double* pc = raw(base + jc);
                double total = 0.0;
                double r = U.ens_c0[(1 << NT) - 1] * pc[cc];
                bool ok = true;
                const long long* mc = dm(base + jc);
                const int* ec = de(base + jc);
#pragma unroll
                for (int kk = 1; kk <= H; ++kk) {
                    long long mm[NT], mp[NT];
                    int em[NT], ep[NT];
                    mm[0] = mc[cc - kk];
                    em[0] = ec[cc - kk];
                    mp[0] = mc[cc + kk];
                    ep[0] = ec[cc + kk];
                    mm[1] = mc[cc - kk * C::BX];
                    em[1] = ec[cc - kk * C::BX];
                    mp[1] = mc[cc + kk * C::BX];
                    ep[1] = ec[cc + kk * C::BX];
                    if constexpr (NT == 3) {
                        mm[2] = dm(base + jc - kk)[cc];
                        em[2] = de(base + jc - kk)[cc];
                        mp[2] = dm(base + jc + kk)[cc];
                        ep[2] = de(base + jc + kk)[cc];
                    }
                    ok = ok && ens2_group<NT>(mm, em, U.ens_w[H - kk], r);
                    ok = ok && ens2_group<NT>(mp, ep, U.ens_w[H + kk], r);
                }
                if (ok) {
                    total = zero_fix(r);
                } else {
                    // Inf/NaN or extreme exponents: the reference's per-term tap order
#pragma unroll
                    for (int t = 0; t < NT; ++t) {
                        double acc = 0.0;
#pragma unroll
                        for (int kk = 0; kk < 2 * H + 1; ++kk) {
                            const int o = kk - H;
                            const double v = t == 0 ? pc[cc + o] : (t == 1 ? pc[cc + o * C::BX] : raw(base + jc + o)[cc]);
                            acc = fma(U.t[t].w[kk], v, acc);
                        }
                        total = (t == 0) ? acc : total + acc;
                    }
                    total = zero_fix(total);
                }
                du[idx] = overwrite ? total : total + du[idx];
            }
            __syncthreads();
            if (tid == 0) {
                const int jn = (jc - HZ) + C::P;
                if (jn < npl) {
                    const int s = (base + jn) & (C::P - 1);
                    mbar_expect_tx(&mbar[s], C::PLANE_BYTES);
                    tma_load_3d(smem + s * C::SLOT, &tmap, &mbar[s], x0 - C::HR, y0 - H, z0 - HZ + jn);
                    issued = jn + 1;
                }
            }
        }
        if (!aborted) base += npl;
    }
    if (aborted && tid == 0) {
        atomicOr(&g_deo_status, 1u);
        for (int j = waited; j < issued; ++j) {
            const int gj = base + j;
            const uint32_t par = (uint32_t)((gj / C::P) & 1);
            for (uint32_t it = 0; it < (1u << 22); ++it)
                if (mbar_try_wait(&mbar[gj & (C::P - 1)], par)) break;
        }
    }
}

// ---------------------------------------------------------------------------
// Fixed-point kernel (Float64): an interior point with no FP64 instruction.
// Each value is decomposed once, when its plane lands, into (e, m) with
// value = m * 2^(e - 1075 - S) and m = +-mantissa << S (S = 8 for three axes,
// 9 for two, so that the NT taps of one offset add in int64 without
// overflow).  For a point, the 1 + 2H*NT taps are aligned to their largest
// exponent E by arithmetic shifts (bits below 2^(E - 1075 - S) are dropped,
// rounding toward -inf), the NT taps of each offset are added in int64, each
// offset's sum is multiplied by its weight's exact integer image fx_w (common
// exponent fx_f) into a 128-bit accumulator, and the total is rounded once to
// nearest even.  The dropped bits cost at most sum|w| * 2^(E - 1075 - S),
// less than ratio * 2^(1 - S) ulp of sum|c_k u_k| with ratio = NT*sum|w| /
// min|w|; the host enables the kernel only for ratio <= 256 and for weights
// whose products cannot overflow the accumulator.  Inf/NaN inputs and results
// that would be subnormal or overflow take the reference's tap order from
// global memory.
// The raw ring only receives planes (P slots); the decomposed ring (DP >= 2H+2
// slots) holds the planes a point reads, so one barrier per plane orders the
// decomposition before its use, and a slot is rewritten only after every
// thread has left the points that read it.
// ---------------------------------------------------------------------------
template <int H>
struct FxCfg {
    using R = TmaCfg<double, H>;
    static constexpr int P = 4;                                              // raw landing slots
    static constexpr int DP = (2 * H + 2) <= 4 ? 4 : ((2 * H + 2) <= 8 ? 8 : 16);  // power of two >= 2H+2
    static constexpr int DSLOT_M = R::PLANE * 8;                             // int64 mantissas
    static constexpr int DSLOT = ((DSLOT_M + R::PLANE * 2 + 127) / 128) * 128;  // + int16 exponents
    static constexpr int SMEM = P * R::SLOT + DP * DSLOT;
};

template <int H, int NT>
__global__ void __launch_bounds__(256) k_lap_fx(const __grid_constant__ CUtensorMap tmap,
                                                const __grid_constant__ UniPlan U, const LapGrid g,
                                                const double* __restrict__ u, double* __restrict__ du,
                                                int overwrite) {
    using C = TmaCfg<double, H>;
    using F = FxCfg<H>;
    constexpr int S = NT == 3 ? 8 : 9;
    constexpr int HZ = NT == 3 ? H : 0;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[F::P];
    unsigned char* dsm = smem + F::P * C::SLOT;
    const int nx = (int)U.n[0], ny = (int)U.n[1], nz = (int)U.n[2];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * C::TX + tx;
    const int64_t sxy = (int64_t)nx * ny;
    const int cc = (ty + H) * C::BX + tx + C::HR;
    // result exponent: A * 2^(E - 1075 - S + fx_f) with |A| = N * 2^-lz, mantissa = N >> 75
    const int ebase0 = 75 - S + U.fx_f;
    const unsigned int polls = U.wait_polls ? U.wait_polls : (1u << 22);
    if (tid == 0) {
        for (int s = 0; s < F::P; ++s) mbar_init(&mbar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto raw = [&](int gj) -> const double* {
        return reinterpret_cast<const double*>(smem + (gj & (F::P - 1)) * C::SLOT);
    };
    auto dm = [&](int gj) -> long long* {
        return reinterpret_cast<long long*>(dsm + (gj & (F::DP - 1)) * F::DSLOT);
    };
    auto de = [&](int gj) -> short* {
        return reinterpret_cast<short*>(dsm + (gj & (F::DP - 1)) * F::DSLOT + F::DSLOT_M);
    };
    int base = 0, issued = 0, waited = 0;
    bool aborted = false;
    __shared__ int s_next;
    for (int k = claim_unit(g, s_next, blockIdx.x); k < g.units && !aborted;
         k = claim_unit(g, s_next, k + gridDim.x)) {
        const int unit = (int)(((long long)k * g.perm) % g.units);
        const int txi = unit % g.tiles_x;
        const int rest = unit / g.tiles_x;
        const int tyi = rest % g.tiles_y;
        const int ci = rest / g.tiles_y;
        const int x0 = txi * C::TX, y0 = tyi * C::TY;
        const int x = x0 + tx, y = y0 + ty;
        const int z0 = ci * g.zc;
        const int z1 = min(z0 + g.zc, nz);
        const int npl = (z1 - z0) + 2 * HZ;
        const bool live = x < nx && y < ny && x + 1 >= U.t[0].flo && x + 1 <= U.t[0].fhi &&
                          y + 1 >= U.t[1].flo && y + 1 <= U.t[1].fhi;
        const int64_t col = (int64_t)y * nx + x;
        if (tid == 0) {
            const int pre = min(F::P, npl);
            for (int j = 0; j < pre; ++j) {
                if (base == 0 && U.test_withhold > 0 && j == U.test_withhold) continue;  // test hook
                const int s = (base + j) & (F::P - 1);
                mbar_expect_tx(&mbar[s], C::PLANE_BYTES);
                tma_load_3d(smem + s * C::SLOT, &tmap, &mbar[s], x0 - C::HR, y0 - H, z0 - HZ + j);
            }
            issued = pre;
        }
        waited = 0;
        for (int p = 0; p < npl; ++p) {
            const int gj = base + p;
            bool timeout = false;
            {
                const uint32_t par = (uint32_t)((gj / F::P) & 1);
                uint32_t it = 0;
                while (!mbar_try_wait(&mbar[gj & (F::P - 1)], par)) {
                    if (++it > polls) {
                        timeout = true;
                        break;
                    }
                }
            }
            if (!timeout) {
                waited = p + 1;
                const double* rp = raw(gj);
                long long* mp = dm(gj);
                short* ep = de(gj);
                for (int q = tid; q < C::PLANE; q += C::TX * C::TY) decompose_fx<S>(rp[q], mp[q], ep[q]);
            }
            if (__syncthreads_or(timeout)) {
                aborted = true;
                break;
            }
            // every thread has decomposed plane p: its raw slot takes plane p + P
            if (tid == 0 && p + F::P < npl &&
                !(base == 0 && U.test_withhold > 0 && p + F::P == U.test_withhold)) {
                const int s = gj & (F::P - 1);
                mbar_expect_tx(&mbar[s], C::PLANE_BYTES);
                tma_load_3d(smem + s * C::SLOT, &tmap, &mbar[s], x0 - C::HR, y0 - H, z0 - HZ + p + F::P);
                issued = p + F::P + 1;
            }
            if (p < 2 * HZ) continue;
            const int z = z0 + p - 2 * HZ;  // the point whose last plane is p
            const bool bz = (NT < 3) || (z + 1 >= U.t[NT - 1].flo && z + 1 <= U.t[NT - 1].fhi);
            if (!(live && bz)) continue;
            const int jg = gj - HZ;  // its centre plane
            const int64_t idx = (int64_t)z * sxy + col;
            double total = 0.0;
            bool ok = false;
            // fx_rows of the tile's 8 rows (whole warps) take the reference's FP64 tap order below, on
            // the FP64 pipe, while the other warps fill the integer pipes; the rows rotate with the
            // tile row and the plane, (ty - fx_rows * (tyi + z)) mod 8 < fx_rows, so that the FP64
            // warps take turns on the SM's four sub-partitions (warp ty runs on sub-partition ty mod 4)
            if (((ty - U.fx_rows * (tyi + z)) & 7) >= U.fx_rows) {
                const long long* mc = dm(jg);
                const short* ec = de(jg);
                long long mt[2 * H][NT];  // [side * H + k - 1][axis]
                int et[2 * H][NT];
                const long long m0 = mc[cc];
                const int e0 = ec[cc];
#pragma unroll
                for (int kk = 1; kk <= H; ++kk) {
                    mt[kk - 1][0] = mc[cc - kk];
                    et[kk - 1][0] = ec[cc - kk];
                    mt[H + kk - 1][0] = mc[cc + kk];
                    et[H + kk - 1][0] = ec[cc + kk];
                    mt[kk - 1][1] = mc[cc - kk * C::BX];
                    et[kk - 1][1] = ec[cc - kk * C::BX];
                    mt[H + kk - 1][1] = mc[cc + kk * C::BX];
                    et[H + kk - 1][1] = ec[cc + kk * C::BX];
                    if constexpr (NT == 3) {
                        mt[kk - 1][2] = dm(jg - kk)[cc];
                        et[kk - 1][2] = de(jg - kk)[cc];
                        mt[H + kk - 1][2] = dm(jg + kk)[cc];
                        et[H + kk - 1][2] = de(jg + kk)[cc];
                    }
                }
                int E = e0;
#pragma unroll
                for (int j = 0; j < 2 * H; ++j)
#pragma unroll
                    for (int a = 0; a < NT; ++a) E = max(E, et[j][a]);
                ok = E < 2047;
                if (ok) {
                    Acc128 A{0ULL, 0LL};
                    mad128(A, (long long)NT * sar64(m0, E - e0), U.fx_w[H]);
#pragma unroll
                    for (int kk = 1; kk <= H; ++kk) {
                        long long sm = 0, sp = 0;
#pragma unroll
                        for (int a = 0; a < NT; ++a) {
                            sm += sar64(mt[kk - 1][a], E - et[kk - 1][a]);
                            sp += sar64(mt[H + kk - 1][a], E - et[H + kk - 1][a]);
                        }
                        mad128(A, sm, U.fx_w[H - kk]);
                        mad128(A, sp, U.fx_w[H + kk]);
                    }
                    total = fx_round(A.hi, A.lo, ebase0 + E, ok);
                }
            }
            if (!ok) {
                // FP64 rows, Inf/NaN or an extreme exponent: the reference's per-term tap order, from global
                // memory (L2-resident: the ring has just loaded these planes)
                const int64_t st[3] = {1, (int64_t)nx, sxy};
#pragma unroll
                for (int t = 0; t < NT; ++t) {
                    double acc = 0.0;
#pragma unroll
                    for (int kk = 0; kk < 2 * H + 1; ++kk) acc = fma(U.t[t].w[kk], u[idx + (kk - H) * st[t]], acc);
                    total = (t == 0) ? acc : total + acc;
                }
                total = zero_fix(total);
            }
            du[idx] = overwrite ? total : total + du[idx];
        }
        if (!aborted) base += npl;
    }
    if (aborted && tid == 0) {
        atomicOr(&g_deo_status, 1u);
        // wait (bounded) for this CTA's copies still in flight before its shared memory is released
        for (int j = waited; j < issued; ++j) {
            if (base == 0 && U.test_withhold > 0 && j == U.test_withhold) continue;  // never issued
            const int gj = base + j;
            const uint32_t par = (uint32_t)((gj / F::P) & 1);
            for (uint32_t it = 0; it < (1u << 22); ++it)
                if (mbar_try_wait(&mbar[gj & (F::P - 1)], par)) break;
        }
    }
}

// ---------------------------------------------------------------------------
// Reference-order kernel with a register queue (Float32 and Float64).
// CTA = 32 x 8 threads over a 32 x (8 RY) tile; each thread owns RY
// consecutive rows of one column.  Planes stream through a TMA ring as in
// k_lap_tma.  Each thread keeps its rows' values at z-H..z+H in registers (one
// shared-memory load per row and plane; the plane loop is unrolled by 2H+1 so
// the queue rotates by register naming, without moves), reads the
// y-neighbours beyond its own rows (2H loads) and the x-neighbours (2H per
// row) from the centre plane, and evaluates each term's taps in the
// reference's order, bit for bit the generic evaluator.  One barrier per plane
// releases the centre plane's slot, which then takes the plane P further on.
// ---------------------------------------------------------------------------
template <typename T, int H>
struct QCfg {
    static constexpr int ES = (int)sizeof(T);
    static constexpr int TX = 32, TYT = 8, RY = ES == 4 ? 8 : 4, TY = TYT * RY;
    static constexpr int HR = ((H * ES + 15) / 16) * 16 / ES;  // x halo rounded up to 16 bytes
    static constexpr int BX = TX + 2 * HR, BY = TY + 2 * H;
    static constexpr int PLANE = BX * BY;
    static constexpr int PLANE_BYTES = PLANE * ES;
    static constexpr int SLOT = ((PLANE_BYTES + 127) / 128) * 128;
    // ring slots (>= H + 2, a power of two): 4 for Float32 at H <= 2 (more CTAs per SM), else 8
    static constexpr int P = (ES == 4 && H + 2 <= 4) ? 4 : 8;
    static constexpr int SMEM = P * SLOT;
};

// -0 -> +0 (see zero_fix); for Float32 one add of +0, which is exact otherwise.
template <typename T>
__device__ __forceinline__ T zero_fix_q(T x) {
    return zero_fix(x);
}
template <>
__device__ __forceinline__ float zero_fix_q<float>(float x) {
    return __fadd_rn(x, 0.0f);
}

template <typename T, int H, int NT, bool OW>
__global__ void __launch_bounds__(256) k_lap_q(const __grid_constant__ CUtensorMap tmap,
                                               const __grid_constant__ UniPlan U, const LapGrid g,
                                               T* __restrict__ du) {
    using C = QCfg<T, H>;
    constexpr int HZ = NT == 3 ? H : 0;
    constexpr int NQ = 2 * HZ + 1;  // queue length = unroll factor of the plane loop
    constexpr int RY = C::RY;
    constexpr int K = 2 * H + 1;
    static_assert(C::P >= H + 2, "ring too short");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[C::P];
    const int nx = (int)U.n[0], ny = (int)U.n[1], nz = (int)U.n[2];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * C::TX + tx;
    const int64_t sxy = (int64_t)nx * ny;
    const int c0 = (ty * RY + H) * C::BX + tx + C::HR;  // the first own row's point inside a slot
    const unsigned int polls = U.wait_polls ? U.wait_polls : (1u << 22);
    T w[NT][K];
#pragma unroll
    for (int t = 0; t < NT; ++t)
#pragma unroll
        for (int k = 0; k < K; ++k) w[t][k] = uni_w<T>(U.t[t], k);
    if (tid == 0) {
        for (int s = 0; s < C::P; ++s) mbar_init(&mbar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto slot = [&](int gj) -> const T* {
        return reinterpret_cast<const T*>(smem + (gj & (C::P - 1)) * C::SLOT);
    };
    int base = 0, issued = 0, waited = 0;
    bool aborted = false;
    __shared__ int s_next;
    for (int kk = claim_unit(g, s_next, blockIdx.x); kk < g.units && !aborted;
         kk = claim_unit(g, s_next, kk + gridDim.x)) {
        const int unit = (int)(((long long)kk * g.perm) % g.units);
        const int txi = unit % g.tiles_x;
        const int rest = unit / g.tiles_x;
        const int tyi = rest % g.tiles_y;
        const int ci = rest / g.tiles_y;
        const int x0 = txi * C::TX, y0 = tyi * C::TY;
        const int x = x0 + tx, yr = y0 + ty * RY;
        const int z0 = ci * g.zc;
        const int z1 = min(z0 + g.zc, nz);
        const int npl = (z1 - z0) + 2 * HZ;
        const bool bx = x < nx && x + 1 >= U.t[0].flo && x + 1 <= U.t[0].fhi;
        unsigned vmask = 0;  // own rows that are interior rows along y
#pragma unroll
        for (int j = 0; j < RY; ++j)
            if (bx && yr + j < ny && yr + j + 1 >= U.t[1].flo && yr + j + 1 <= U.t[1].fhi) vmask |= 1u << j;
        T* dcol = du + (int64_t)yr * nx + x;
        if (tid == 0) {
            const int pre = min(C::P, npl);
            for (int j = 0; j < pre; ++j) {
                if (base == 0 && U.test_withhold > 0 && j == U.test_withhold) continue;  // test hook
                const int s = (base + j) & (C::P - 1);
                mbar_expect_tx(&mbar[s], C::PLANE_BYTES);
                tma_load_3d(smem + s * C::SLOT, &tmap, &mbar[s], x0 - C::HR, y0 - H, z0 - HZ + j);
            }
            issued = pre;
        }
        waited = 0;
        T q[RY][NQ];  // own rows; plane p lands in q[.][p % NQ]
        for (int p0 = 0; p0 < npl && !aborted; p0 += NQ) {
#pragma unroll
            for (int ph = 0; ph < NQ; ++ph) {
                const int p = p0 + ph;
                if (p >= npl) break;
                const int gj = base + p;
                bool timeout = false;
                {
                    const uint32_t par = (uint32_t)((gj / C::P) & 1);
                    uint32_t it = 0;
                    while (!mbar_try_wait(&mbar[gj & (C::P - 1)], par)) {
                        if (++it > polls) {
                            timeout = true;
                            break;
                        }
                    }
                }
                if (!timeout) {
                    waited = p + 1;
                    const T* pn = slot(gj);
#pragma unroll
                    for (int j = 0; j < RY; ++j) q[j][ph] = pn[c0 + j * C::BX];
                    const int z = z0 + p - 2 * HZ;  // the point whose last plane is p
                    const bool bz = (NT < 3) || (z + 1 >= U.t[NT - 1].flo && z + 1 <= U.t[NT - 1].fhi);
                    if (p >= 2 * HZ && vmask && bz) {
                        const T* pc = slot(gj - HZ);  // its centre plane
                        T col[RY + 2 * H];            // this column at rows yr - H .. yr + RY - 1 + H
#pragma unroll
                        for (int m = 0; m < H; ++m) {
                            col[m] = pc[c0 + (m - H) * C::BX];
                            col[RY + H + m] = pc[c0 + (RY + m) * C::BX];
                        }
#pragma unroll
                        for (int j = 0; j < RY; ++j) col[H + j] = q[j][(ph + 1 + HZ) % NQ];
                        T* dz = dcol + (int64_t)z * sxy;
#pragma unroll
                        for (int j = 0; j < RY; ++j) {
                            // every row is evaluated (the tile in shared memory covers it: no branch
                            // around the loads, so they schedule across rows); only interior rows are stored
                            const int cc = c0 + j * C::BX;
                            T ax = T(0), ay = T(0);
#pragma unroll
                            for (int k = 0; k < K; ++k)
                                ax = fma(w[0][k], k == H ? col[H + j] : pc[cc + k - H], ax);
#pragma unroll
                            for (int k = 0; k < K; ++k) ay = fma(w[1][k], col[j + k], ay);
                            T tot = ax + ay;
                            if constexpr (NT == 3) {
                                T az = T(0);
#pragma unroll
                                for (int k = 0; k < K; ++k) az = fma(w[2][k], q[j][(ph + 1 + k) % NQ], az);
                                tot = tot + az;
                            }
                            tot = zero_fix_q(tot);
                            if (vmask & (1u << j)) {
                                T* d = dz + (int64_t)j * nx;
                                if constexpr (OW) *d = tot;
                                else *d = tot + *d;
                            }
                        }
                    }
                }
                if (__syncthreads_or(timeout)) {
                    aborted = true;
                    break;
                }
                // every thread is done with plane p - HZ: its slot takes plane p - HZ + P
                if (tid == 0 && p >= HZ && p - HZ + C::P < npl &&
                    !(base == 0 && U.test_withhold > 0 && p - HZ + C::P == U.test_withhold)) {
                    const int jn = p - HZ + C::P;
                    const int s = (base + jn) & (C::P - 1);
                    mbar_expect_tx(&mbar[s], C::PLANE_BYTES);
                    tma_load_3d(smem + s * C::SLOT, &tmap, &mbar[s], x0 - C::HR, y0 - H, z0 - HZ + jn);
                    issued = jn + 1;
                }
            }
        }
        if (!aborted) base += npl;
    }
    if (aborted && tid == 0) {
        atomicOr(&g_deo_status, 1u);
        // wait (bounded) for this CTA's copies still in flight before its shared memory is released
        for (int j = waited; j < issued; ++j) {
            if (base == 0 && U.test_withhold > 0 && j == U.test_withhold) continue;  // never issued
            const int gj = base + j;
            const uint32_t par = (uint32_t)((gj / C::P) & 1);
            for (uint32_t it = 0; it < (1u << 22); ++it)
                if (mbar_try_wait(&mbar[gj & (C::P - 1)], par)) break;
        }
    }
}

}  // namespace deo

using namespace deo;

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

static bool make_map3(CUtensorMap& map, const void* u, int es, int64_t nx, int64_t ny, int64_t nz, int bx, int by,
                      int bz) {
    if (((uintptr_t)u & 15) || ((nx * es) & 15) || ((bx * es) & 15) || nx > (1 << 30) || ny > (1 << 30) ||
        nz > (1 << 30) || bx < 1 || bx > 256 || by < 1 || by > 256 || bz < 1 || bz > 256)
        return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t gdim[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t gstride[2] = {(cuuint64_t)(nx * es), (cuuint64_t)(nx * ny * es)};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(&map, es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(u),
               gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static bool make_map(CUtensorMap& map, const void* u, int es, int64_t nx, int64_t ny, int64_t nz, int bx, int by) {
    return make_map3(map, u, es, nx, ny, nz, bx, by, 1);
}

// 1 if the TMA path can run on u (the tensor-map rules: 16-byte aligned base,
// rows of a 16-byte multiple, sizes below 2^30).
extern "C" int deo_k_tma_ok(const UniPlan* up, int dtype, const void* u) {
    const int64_t es = dtype == 0 ? 8 : 4;
    return up->lap && !((uintptr_t)u & 15) && !((up->n[0] * es) & 15) && up->n[0] <= (1 << 30) &&
           up->n[1] <= (1 << 30) && up->n[2] <= (1 << 30);
}

extern "C" int deo_k_encode_map3(void* map, const void* u, int es, int64_t nx, int64_t ny, int64_t nz, int bx, int by,
                                 int bz) {
    return make_map3(*reinterpret_cast<CUtensorMap*>(map), u, es, nx, ny, nz, bx, by, bz) ? 0
                                                                                          : (int)cudaErrorNotSupported;
}

template <typename T, int H, int NT, bool ENS>
static int launch_tma(const UniPlan* up, const PlanDev* dp, const void* u, void* du, int ow, cudaStream_t st) {
    using C = TmaCfg<T, H>;
    CUtensorMap map;
    if (!make_map(map, u, C::ES, up->n[0], up->n[1], up->n[2], C::BX, C::BY)) return (int)cudaErrorNotSupported;
    static int64_t G = 0;
    if (!G) {
        const int e = occupancy_grid(k_lap_tma<T, H, NT, ENS>, C::TX * C::TY, C::SMEM, G);
        if (e) return e;
    }
    const LapGrid g = make_grid(up, C::TX, C::TY, H, NT, G);
    const int grid = (int)std::min<int64_t>(G, g.units);
    k_lap_tma<T, H, NT, ENS><<<grid, dim3(C::TX, C::TY), C::SMEM, st>>>(map, *up, g, dp, (const T*)u, (T*)du, ow);
    return (int)cudaGetLastError();
}

template <int H, int NT>
static int launch_ens2(const UniPlan* up, const PlanDev* dp, const void* u, void* du, int ow, cudaStream_t st) {
    using C = TmaCfg<double, H>;
    using E = Ens2Cfg<H>;
    CUtensorMap map;
    if (!make_map(map, u, 8, up->n[0], up->n[1], up->n[2], C::BX, C::BY)) return (int)cudaErrorNotSupported;
    static int64_t G = 0;
    if (!G) {
        const int e = occupancy_grid(k_lap_ens2<H, NT>, C::TX * C::TY, E::SMEM, G);
        if (e) return e;
    }
    const LapGrid g = make_grid(up, C::TX, C::TY, H, NT, G);
    const int grid = (int)std::min<int64_t>(G, g.units);
    k_lap_ens2<H, NT><<<grid, dim3(C::TX, C::TY), E::SMEM, st>>>(map, *up, g, dp, (const double*)u, (double*)du, ow);
    return (int)cudaGetLastError();
}

template <typename T, int H, int NT>
static int launch_q(const UniPlan* up, unsigned int* sched, const void* u, void* du, int ow, cudaStream_t st) {
    using C = QCfg<T, H>;
    CUtensorMap map;
    if (!make_map(map, u, C::ES, up->n[0], up->n[1], up->n[2], C::BX, C::BY)) return (int)cudaErrorNotSupported;
    static int64_t G = 0;
    if (!G) {
        int e = occupancy_grid(k_lap_q<T, H, NT, true>, C::TX * C::TYT, C::SMEM, G);
        if (!e) e = occupancy_grid(k_lap_q<T, H, NT, false>, C::TX * C::TYT, C::SMEM, G);
        if (e) return e;
    }
    const LapGrid g = make_grid(up, C::TX, C::TY, H, NT, G);
    LapGrid g2 = g;
    g2.sched = sched;
    if (sched) {
        const cudaError_t e = cudaMemsetAsync(sched, 0, sizeof(unsigned int), st);
        if (e != cudaSuccess) return (int)e;
    }
    const int grid = (int)std::min<int64_t>(G, g.units);
    if (ow)
        k_lap_q<T, H, NT, true><<<grid, dim3(C::TX, C::TYT), C::SMEM, st>>>(map, *up, g2, (T*)du);
    else
        k_lap_q<T, H, NT, false><<<grid, dim3(C::TX, C::TYT), C::SMEM, st>>>(map, *up, g2, (T*)du);
    return (int)cudaGetLastError();
}

template <typename T>
static int launch_q_h(const UniPlan* up, unsigned int* sched, const void* u, void* du, int ow, cudaStream_t st) {
    const int H = up->radius;
    if (up->nterms == 3) {
        switch (H) {
            case 1: return launch_q<T, 1, 3>(up, sched, u, du, ow, st);
            case 2: return launch_q<T, 2, 3>(up, sched, u, du, ow, st);
            case 3: return launch_q<T, 3, 3>(up, sched, u, du, ow, st);
            case 4: return launch_q<T, 4, 3>(up, sched, u, du, ow, st);
        }
    } else if (up->nterms == 2) {
        switch (H) {
            case 1: return launch_q<T, 1, 2>(up, sched, u, du, ow, st);
            case 2: return launch_q<T, 2, 2>(up, sched, u, du, ow, st);
            case 3: return launch_q<T, 3, 2>(up, sched, u, du, ow, st);
            case 4: return launch_q<T, 4, 2>(up, sched, u, du, ow, st);
        }
    }
    return (int)cudaErrorNotSupported;
}

template <typename T, bool ENS>
static int launch_tma_h(const UniPlan* up, const PlanDev* dp, const void* u, void* du, int ow, cudaStream_t st) {
    const int H = up->radius;
    if (up->nterms == 3) {
        switch (H) {
            case 1: return launch_tma<T, 1, 3, ENS>(up, dp, u, du, ow, st);
            case 2: return launch_tma<T, 2, 3, ENS>(up, dp, u, du, ow, st);
            case 3: return launch_tma<T, 3, 3, ENS>(up, dp, u, du, ow, st);
            case 4: return launch_tma<T, 4, 3, ENS>(up, dp, u, du, ow, st);
        }
    } else if (up->nterms == 2) {
        switch (H) {
            case 1: return launch_tma<T, 1, 2, ENS>(up, dp, u, du, ow, st);
            case 2: return launch_tma<T, 2, 2, ENS>(up, dp, u, du, ow, st);
            case 3: return launch_tma<T, 3, 2, ENS>(up, dp, u, du, ow, st);
            case 4: return launch_tma<T, 4, 2, ENS>(up, dp, u, du, ow, st);
        }
    }
    return (int)cudaErrorNotSupported;
}

template <int H, int NT>
static int launch_fx(const UniPlan* up, unsigned int* sched, const void* u, void* du, int ow, cudaStream_t st) {
    using C = TmaCfg<double, H>;
    using F = FxCfg<H>;
    CUtensorMap map;
    if (!make_map(map, u, 8, up->n[0], up->n[1], up->n[2], C::BX, C::BY)) return (int)cudaErrorNotSupported;
    static int64_t G = 0;
    if (!G) {
        const int e = occupancy_grid(k_lap_fx<H, NT>, C::TX * C::TY, F::SMEM, G);
        if (e) return e;
    }
    const LapGrid g = make_grid(up, C::TX, C::TY, H, NT, G);
    LapGrid g2 = g;
    g2.sched = sched;
    if (sched) {
        const cudaError_t e = cudaMemsetAsync(sched, 0, sizeof(unsigned int), st);
        if (e != cudaSuccess) return (int)e;
    }
    const int grid = (int)std::min<int64_t>(G, g.units);
    k_lap_fx<H, NT><<<grid, dim3(C::TX, C::TY), F::SMEM, st>>>(map, *up, g2, (const double*)u, (double*)du, ow);
    return (int)cudaGetLastError();
}

template <int H, bool CNEG>
static int launch_bfx(const UniPlan* up, unsigned int* sched, const void* u, void* du, int ow, cudaStream_t st) {
    using C = BfxCfg<H>;
    CUtensorMap map;
    if (!make_map(map, u, 8, up->n[0], up->n[1], up->n[2], C::BX, C::BY)) return (int)cudaErrorNotSupported;
    static int64_t G = 0;
    if (!G) {
        const int e = occupancy_grid(k_lap_bfx<H, CNEG>, C::NTHR, C::SMEM, G);
        if (e) return e;
    }
    const LapGrid g = make_grid(up, C::TX, C::TY, H, 3, G);
    LapGrid g2 = g;
    g2.sched = sched;
    if (sched) {
        const cudaError_t e = cudaMemsetAsync(sched, 0, sizeof(unsigned int), st);
        if (e != cudaSuccess) return (int)e;
    }
    const int grid = (int)std::min<int64_t>(G, g.units);
    k_lap_bfx<H, CNEG><<<grid, dim3(C::TXT, C::TYT), C::SMEM, st>>>(map, *up, g2, (const double*)u, (double*)du, ow);
    return (int)cudaGetLastError();
}

#define DEO_TRY_KERNEL(call, name)                            \
    do {                                                      \
        const int e_ = (call);                                \
        if (e_ != (int)cudaErrorNotSupported) {               \
            if (!e_) *kernel = (name);                        \
            return e_;                                        \
        }                                                     \
    } while (0)

extern "C" int deo_k_apply_tma(const UniPlan* up, const PlanDev* dp, int dtype, const void* u, void* du,
                               int overwrite, int use_ens, void* stream, const char** kernel, unsigned int* sched) {
    static const char* none = "";
    if (!kernel) kernel = &none;
    if (!up->lap || up->nterms < 2 || up->nterms > 3) return (int)cudaErrorNotSupported;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int H = up->radius, NT = up->nterms;
    if (dtype == 0 && use_ens == 5 && up->bfx && NT == 3) {
        const bool cn = up->bfx_cneg != 0;
        if (H == 1) DEO_TRY_KERNEL((cn ? launch_bfx<1, true>(up, sched, u, du, overwrite, st)
                                       : launch_bfx<1, false>(up, sched, u, du, overwrite, st)), "k_lap_bfx");
        if (H == 2) DEO_TRY_KERNEL((cn ? launch_bfx<2, true>(up, sched, u, du, overwrite, st)
                                       : launch_bfx<2, false>(up, sched, u, du, overwrite, st)), "k_lap_bfx");
        if (H == 3) DEO_TRY_KERNEL((cn ? launch_bfx<3, true>(up, sched, u, du, overwrite, st)
                                       : launch_bfx<3, false>(up, sched, u, du, overwrite, st)), "k_lap_bfx");
    }
    if (dtype == 0 && (use_ens == 1 || use_ens == 4 || use_ens == 5) && up->fx) {
        if (NT == 3 && H == 1) DEO_TRY_KERNEL((launch_fx<1, 3>(up, sched, u, du, overwrite, st)), "k_lap_fx");
        if (NT == 3 && H == 2) DEO_TRY_KERNEL((launch_fx<2, 3>(up, sched, u, du, overwrite, st)), "k_lap_fx");
        if (NT == 3 && H == 3) DEO_TRY_KERNEL((launch_fx<3, 3>(up, sched, u, du, overwrite, st)), "k_lap_fx");
        if (NT == 2 && H == 1) DEO_TRY_KERNEL((launch_fx<1, 2>(up, sched, u, du, overwrite, st)), "k_lap_fx");
        if (NT == 2 && H == 2) DEO_TRY_KERNEL((launch_fx<2, 2>(up, sched, u, du, overwrite, st)), "k_lap_fx");
        if (NT == 2 && H == 3) DEO_TRY_KERNEL((launch_fx<3, 2>(up, sched, u, du, overwrite, st)), "k_lap_fx");
    }
    if (dtype == 0 && (use_ens == 1 || use_ens == 3 || use_ens == 4 || use_ens == 5) && up->ens) {
        if (NT == 3 && H == 1) DEO_TRY_KERNEL((launch_ens2<1, 3>(up, dp, u, du, overwrite, st)), "k_lap_ens2");
        if (NT == 3 && H == 2) DEO_TRY_KERNEL((launch_ens2<2, 3>(up, dp, u, du, overwrite, st)), "k_lap_ens2");
        if (NT == 3 && H == 3) DEO_TRY_KERNEL((launch_ens2<3, 3>(up, dp, u, du, overwrite, st)), "k_lap_ens2");
        if (NT == 2 && H == 1) DEO_TRY_KERNEL((launch_ens2<1, 2>(up, dp, u, du, overwrite, st)), "k_lap_ens2");
        if (NT == 2 && H == 2) DEO_TRY_KERNEL((launch_ens2<2, 2>(up, dp, u, du, overwrite, st)), "k_lap_ens2");
        if (NT == 2 && H == 3) DEO_TRY_KERNEL((launch_ens2<3, 2>(up, dp, u, du, overwrite, st)), "k_lap_ens2");
    }
    if (dtype == 0) {
        if (use_ens && up->ens)
            DEO_TRY_KERNEL((launch_tma_h<double, true>(up, dp, u, du, overwrite, st)), "k_lap_tma(exact sums v1)");
        DEO_TRY_KERNEL((launch_q_h<double>(up, sched, u, du, overwrite, st)), "k_lap_q");
    } else {
        if (up->f32_vec) DEO_TRY_KERNEL((deo_k_apply_vec(up, sched, u, du, overwrite, st)), "k_lap_v");
        DEO_TRY_KERNEL((launch_q_h<float>(up, sched, u, du, overwrite, st)), "k_lap_q");
    }
    return (int)cudaErrorNotSupported;
}


extern "C" int deo_k_read_status(unsigned int* status) {
    unsigned int v = 0, zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_deo_status, sizeof v);
    if (e != cudaSuccess) return (int)e;
    e = cudaMemcpyToSymbol(g_deo_status, &zero, sizeof zero);
    if (e != cudaSuccess) return (int)e;
    *status = v;
    return 0;
}
