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
            if (inxy && !timeout) {
                const int64_t idx = (int64_t)z * sxy + col;
                const T* pc = slot(base + jc);
                const bool bz = (NT < 3) || (z + 1 >= U.t[NT - 1].flo && z + 1 <= U.t[NT - 1].fhi);
                const bool band[3] = {bx, by, bz};
                T total;
                bool done = false;
                if constexpr (ENS) {
                    // exact sums over the axes whose row is a band row; other axes by their row tables
                    const int mask = (bx ? 1 : 0) | (by ? 2 : 0) | ((NT == 3 && bz) ? 4 : 0);
                    if (mask) {
                        double r = U.ens_c0[mask] * (double)pc[cc];
                        bool ok = true;
#pragma unroll
                        for (int k = 1; k <= H; ++k) {
                            double vm[NT], vp[NT];
                            vm[0] = bx ? (double)pc[cc - k] : 0.0;
                            vp[0] = bx ? (double)pc[cc + k] : 0.0;
                            vm[1] = by ? (double)pc[cc - k * C::BX] : 0.0;
                            vp[1] = by ? (double)pc[cc + k * C::BX] : 0.0;
                            if constexpr (NT == 3) {
                                vm[2] = bz ? (double)slot(base + jc - k)[cc] : 0.0;
                                vp[2] = bz ? (double)slot(base + jc + k)[cc] : 0.0;
                            }
                            bool okm, okp;
                            const double sm = ens_sum<NT>(vm, okm);
                            const double sp = ens_sum<NT>(vp, okp);
                            ok = ok && okm && okp;
                            r = fma(U.ens_w[H - k], sm, r);
                            r = fma(U.ens_w[H + k], sp, r);
                        }
                        if (ok) {
#pragma unroll
                            for (int t = 0; t < NT; ++t)
                                if (!band[t]) r = r + (double)eval_term<T>(Pd->t[t], u, idx, (t == 0 ? x : (t == 1 ? y : z)) + 1);
                            total = (T)zero_fix(r);
                            done = true;
                        }
                    }
                }
                if (!done) {
                    // the reference's per-term tap order: band rows from the ring, others by row tables
#pragma unroll
                    for (int t = 0; t < NT; ++t) {
                        T acc;
                        if (band[t]) {
                            acc = T(0);
#pragma unroll
                            for (int k = 0; k < 2 * H + 1; ++k) {
                                const int o = k - H;
                                const T v = t == 0 ? pc[cc + o]
                                                   : (t == 1 ? pc[cc + o * C::BX] : slot(base + jc + o)[cc]);
                                acc = fma(uni_w<T>(U.t[t], k), v, acc);
                            }
                        } else {
                            acc = eval_term<T>(Pd->t[t], u, idx, (t == 0 ? x : (t == 1 ? y : z)) + 1);
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

template <typename T, int H, int NT, bool ENS>
static int launch_tma(const UniPlan* up, const PlanDev* dp, const void* u, void* du, int ow, cudaStream_t st) {
    using C = TmaCfg<T, H>;
    const int64_t nx = up->n[0], ny = up->n[1], nz = up->n[2];
    if (((uintptr_t)u & 15) || ((nx * C::ES) & 15) || nx > (1 << 30) || ny > (1 << 30) || nz > (1 << 30))
        return (int)cudaErrorNotSupported;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return (int)cudaErrorNotSupported;
    CUtensorMap map;
    const cuuint64_t gdim[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t gstride[2] = {(cuuint64_t)(nx * C::ES), (cuuint64_t)(nx * ny * C::ES)};
    const cuuint32_t box[3] = {(cuuint32_t)C::BX, (cuuint32_t)C::BY, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(&map, C::ES == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                           const_cast<void*>(u), gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return (int)cudaErrorNotSupported;
    static int per_sm = 0, sms = 0;
    if (!per_sm) {
        cudaError_t e = cudaFuncSetAttribute(k_lap_tma<T, H, NT, ENS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             C::SMEM);
        if (e != cudaSuccess) return (int)e;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lap_tma<T, H, NT, ENS>, C::TX * C::TY, C::SMEM);
        if (e != cudaSuccess || per_sm < 1) per_sm = 1;
    }
    LapGrid g;
    g.tiles_x = (int)((nx + C::TX - 1) / C::TX);
    g.tiles_y = (int)((ny + C::TY - 1) / C::TY);
    const int64_t G = (int64_t)sms * per_sm;
    const int64_t tiles = (int64_t)g.tiles_x * g.tiles_y;
    // z chunk: at least 12 planes (halo overhead 2H/zc), chosen so the units
    // fill the persistent grid's rounds as evenly as possible
    g.zc = (int)nz;
    if (NT == 3) {
        double best = -1.0;
        const int zmin = (int)std::min<int64_t>(nz, 12);
        for (int zc = zmin; zc <= nz; ++zc) {
            const int64_t units = tiles * ((nz + zc - 1) / zc);
            const int64_t rounds = (units + G - 1) / G;
            const double eff = (double)units / (double)(rounds * G) * (double)zc / (double)(zc + 2 * H) *
                               ((double)nz / (double)(((nz + zc - 1) / zc) * zc));
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
        while (b) { const int t = a % b; a = b; b = t; }
        if (a == 1 && cand < g.units) { g.perm = cand; break; }
    }
    const int grid = (int)std::min<int64_t>(G, g.units);
    k_lap_tma<T, H, NT, ENS><<<grid, dim3(C::TX, C::TY), C::SMEM, st>>>(map, *up, g, dp, (const T*)u, (T*)du, ow);
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

extern "C" int deo_k_apply_tma(const UniPlan* up, const PlanDev* dp, int dtype, const void* u, void* du,
                               int overwrite, int use_ens, void* stream) {
    if (!up->lap) return (int)cudaErrorNotSupported;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
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
