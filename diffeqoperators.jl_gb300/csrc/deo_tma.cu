// deo_tma.cu -- TMA-fed fused apply for plans whose terms are centred bands on
// axes 1..NT of a 2-D/3-D array (the Laplacian-type plans, UniPlan::lap).
//
// Each CTA owns a TX x TY column of the grid and walks a chunk of z.  One
// elected thread streams z-planes of the (TX + 2HR) x (TY + 2H) tile (HR = H
// rounded up to 16 bytes, the TMA alignment of the innermost coordinate) into a
// shared-memory ring of P slots with cp.async.bulk.tensor, each slot guarded by
// an mbarrier; the ring keeps P - (2H+1) planes in flight ahead of the plane
// being evaluated.  Planes outside the array arrive zero-filled (TMA OOB fill),
// so loads need no bounds checks.  Every mbarrier wait is bounded: on timeout
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
// Points on boundary rows use the generic evaluator for the affected terms.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "deo_eval.cuh"

namespace deo {

__device__ unsigned int g_deo_status;  // bit 0: a bounded mbarrier wait gave up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* m, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* m, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(m)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* m, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(m))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

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

// Work unit u = (tile x, tile y, z chunk); a persistent grid of G CTAs takes
// units b, b + G, b + 2G, ... (static, so one plan may run on several streams
// at once).  Planes stream through the ring with a running count, so slot and
// mbarrier phase carry over from one unit to the next.
struct LapGrid {
    int tiles_x, tiles_y, chunks, zc;
    int units;
    int perm;  // coprime with units: unit k of the round-robin is (k * perm) % units,
               // so one CTA's units are spread over tile columns and z chunks
};

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
                fence_proxy_async();
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
                    fence_proxy_async();
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
                fence_proxy_async();
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
                    fence_proxy_async();
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

// The boundary shell of a Laplacian-type plan: every point with a non-band
// row along some axis (it reads a ghost or uses a boundary stencil).  The
// tiled kernels compute the interior box [flo, fhi]^NT; this kernel computes
// the rest with the generic row-table evaluator (the reference's order).
// Index space: z outside the box (full planes), then z inside & y outside
// (full rows), then z, y inside & x outside.
struct ShellBox {
    int lo[3], hi[3];      // interior box, 0-based inclusive (empty if lo > hi)
    int64_t n[3];
    int64_t cz, cy, cx;    // points in each part
};

template <typename T>
__global__ void __launch_bounds__(256) k_shell(const __grid_constant__ ShellBox B, const PlanDev* __restrict__ P,
                                               const T* __restrict__ u, T* __restrict__ du, int overwrite) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nx = B.n[0], ny = B.n[1];
    int64_t x, y, z;
    if (t < B.cz) {
        const int64_t nzo = B.n[2] - (B.hi[2] - B.lo[2] + 1);  // planes outside
        const int64_t pl = t / (nx * ny), r = t - pl * nx * ny;
        const int64_t below = B.lo[2];
        z = pl < below ? pl : pl - below + B.hi[2] + 1;
        (void)nzo;
        y = r / nx;
        x = r - y * nx;
    } else if (t < B.cz + B.cy) {
        const int64_t q = t - B.cz;
        const int64_t nyo = ny - (B.hi[1] - B.lo[1] + 1);
        const int64_t pl = q / (nyo * nx), r = q - pl * nyo * nx;
        z = B.lo[2] + pl;
        const int64_t row = r / nx;
        x = r - row * nx;
        y = row < B.lo[1] ? row : row - B.lo[1] + B.hi[1] + 1;
    } else if (t < B.cz + B.cy + B.cx) {
        const int64_t q = t - B.cz - B.cy;
        const int64_t nxo = nx - (B.hi[0] - B.lo[0] + 1);
        const int64_t line = q / nxo, c = q - line * nxo;
        const int64_t niy = B.hi[1] - B.lo[1] + 1;
        z = B.lo[2] + line / niy;
        y = B.lo[1] + line % niy;
        x = c < B.lo[0] ? c : c - B.lo[0] + B.hi[0] + 1;
    } else {
        return;
    }
    const int64_t idx = (z * ny + y) * nx + x;
    const T r = eval_point<T, false>(*P, u, idx);
    du[idx] = overwrite ? r : r + du[idx];
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

static bool make_map(CUtensorMap& map, const void* u, int es, int64_t nx, int64_t ny, int64_t nz, int bx, int by) {
    if (((uintptr_t)u & 15) || ((nx * es) & 15) || nx > (1 << 30) || ny > (1 << 30) || nz > (1 << 30)) return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t gdim[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t gstride[2] = {(cuuint64_t)(nx * es), (cuuint64_t)(nx * ny * es)};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(&map, es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(u),
               gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Units and z chunk for a persistent grid of G CTAs (see LapGrid).
static LapGrid make_grid(const UniPlan* up, int tx, int ty, int H, int nt, int64_t G) {
    const int64_t nx = up->n[0], ny = up->n[1], nz = up->n[2];
    LapGrid g;
    g.tiles_x = (int)((nx + tx - 1) / tx);
    g.tiles_y = (int)((ny + ty - 1) / ty);
    const int64_t tiles = (int64_t)g.tiles_x * g.tiles_y;
    g.zc = (int)nz;
    if (nt == 3) {
        double best = -1.0;
        const int zmin = (int)std::min<int64_t>(nz, 12);
        for (int zc = zmin; zc <= nz; ++zc) {
            const int64_t chunks = (nz + zc - 1) / zc;
            const int64_t units = tiles * chunks;
            const int64_t rounds = (units + G - 1) / G;
            const double eff = (double)units / (double)(rounds * G) * (double)zc / (double)(zc + 2 * H) *
                               ((double)nz / (double)(chunks * zc));
            if (eff > best + 1e-9) {
                best = eff;
                g.zc = zc;
            }
        }
    }
    g.chunks = (int)((nz + g.zc - 1) / g.zc);
    g.units = (int)(tiles * g.chunks);
    g.perm = 1;
    for (int cand : {7919, 6007, 4099, 2053, 1031, 521, 263, 131, 67, 37, 17}) {
        int a = cand, b = g.units;
        while (b) {
            const int t = a % b;
            a = b;
            b = t;
        }
        if (a == 1 && cand < g.units) {
            g.perm = cand;
            break;
        }
    }
    return g;
}

template <typename K>
static int occupancy_grid(K kernel, int threads, int smem, int64_t& G) {
    static thread_local int dummy = 0;
    (void)dummy;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return (int)e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (e != cudaSuccess || per_sm < 1) per_sm = 1;
    G = (int64_t)sms * per_sm;
    return 0;
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

template <typename T>
static int launch_shell(const UniPlan* up, const PlanDev* dp, const void* u, void* du, int ow, cudaStream_t st) {
    ShellBox B;
    for (int k = 0; k < 3; ++k) {
        B.n[k] = up->n[k];
        if (k < up->nterms) {
            B.lo[k] = up->t[k].flo - 1;
            B.hi[k] = up->t[k].fhi - 1;
        } else {
            B.lo[k] = 0;
            B.hi[k] = (int)up->n[k] - 1;
        }
        if (B.lo[k] > B.hi[k]) {  // no interior along k: everything is shell
            B.lo[k] = (int)up->n[k];
            B.hi[k] = (int)up->n[k] - 1;
        }
    }
    const int64_t ix = B.hi[0] - B.lo[0] + 1, iy = B.hi[1] - B.lo[1] + 1, iz = B.hi[2] - B.lo[2] + 1;
    const int64_t nx = B.n[0], ny = B.n[1], nz = B.n[2];
    B.cz = (nz - iz) * nx * ny;
    B.cy = iz * (ny - iy) * nx;
    B.cx = iz * iy * (nx - ix);
    const int64_t total = B.cz + B.cy + B.cx;
    if (total == 0) return 0;
    const int64_t blocks = (total + 255) / 256;
    k_shell<T><<<(unsigned)blocks, 256, 0, st>>>(B, dp, (const T*)u, (T*)du, ow);
    return (int)cudaGetLastError();
}

static int launch_tma_any(const UniPlan* up, const PlanDev* dp, int dtype, const void* u, void* du, int overwrite,
                          int use_ens, cudaStream_t st);

extern "C" int deo_k_apply_tma(const UniPlan* up, const PlanDev* dp, int dtype, const void* u, void* du,
                               int overwrite, int use_ens, void* stream) {
    if (!up->lap) return (int)cudaErrorNotSupported;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int e = launch_tma_any(up, dp, dtype, u, du, overwrite, use_ens, st);
    if (e) return e;
    return dtype == 0 ? launch_shell<double>(up, dp, u, du, overwrite, st)
                      : launch_shell<float>(up, dp, u, du, overwrite, st);
}

static int launch_tma_any(const UniPlan* up, const PlanDev* dp, int dtype, const void* u, void* du, int overwrite,
                          int use_ens, cudaStream_t st) {
    if (dtype == 0 && use_ens && up->ens && use_ens != 2) {
        int e = (int)cudaErrorNotSupported;
        if (up->nterms == 3 && up->radius == 1) e = launch_ens2<1, 3>(up, dp, u, du, overwrite, st);
        if (up->nterms == 3 && up->radius == 2) e = launch_ens2<2, 3>(up, dp, u, du, overwrite, st);
        if (up->nterms == 3 && up->radius == 3) e = launch_ens2<3, 3>(up, dp, u, du, overwrite, st);
        if (up->nterms == 2 && up->radius == 1) e = launch_ens2<1, 2>(up, dp, u, du, overwrite, st);
        if (up->nterms == 2 && up->radius == 2) e = launch_ens2<2, 2>(up, dp, u, du, overwrite, st);
        if (up->nterms == 2 && up->radius == 3) e = launch_ens2<3, 2>(up, dp, u, du, overwrite, st);
        if (e != (int)cudaErrorNotSupported) return e;
    }
    if (dtype == 0)
        return (use_ens && up->ens) ? launch_tma_h<double, true>(up, dp, u, du, overwrite, st)
                                    : launch_tma_h<double, false>(up, dp, u, du, overwrite, st);
    return launch_tma_h<float, false>(up, dp, u, du, overwrite, st);
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
