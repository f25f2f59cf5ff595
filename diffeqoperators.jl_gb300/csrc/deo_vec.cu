// deo_vec.cu -- Float32 interior of a Laplacian-type plan, vectorised along x.
//
// CTA = 16 x TYT threads over a 64 x (TYT * RY) tile; each thread owns a
// 4-wide x vector (one float4) on RY consecutive rows (the register-block
// depth).  Planes stream through a TMA ring of P slots as in k_lap_q
// (deo_tma.cu), and the z neighbours of the thread's 4 RY points wait in a
// register queue of float4s (the plane loop unrolled by 2H + 1, so the queue
// rotates by register naming).  The tile shape (TYT, RY) is a plan option,
// chosen by deo_plan_autotune among the instantiated variants.  Per plane a thread reads
// from shared memory, all as 16-byte loads: its own vectors of the newest
// plane (into the queue), the 2H vectors above and below its rows and the
// vectors left and right of its own on the centre plane (the x taps of all 4
// lanes come from those three vectors).  That is 3 RY + 2H loads for 4 RY
// points, against about 6 scalar loads per point in k_lap_q, and the results
// leave as one 16-byte store per row.
//
// Arithmetic: each lane evaluates each term's taps in the reference's order
// (fma from 0 over the taps, terms added left to right, -0 made +0), the
// same operations as k_lap_q and the generic evaluator, so the three agree
// bit for bit.
// Points on boundary rows are left to the shell kernels.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "deo_lap.cuh"
#include "deo_ptx.cuh"

namespace deo {

__device__ unsigned int g_deo_vec_status;  // bit 0: a bounded mbarrier wait gave up

template <int H, int TYT_, int RY_>
struct VCfg {
    static constexpr int TXT = 16, TYT = TYT_, VW = 4, RY = RY_;
    static constexpr int NTHR = TXT * TYT;
    static constexpr int TX = TXT * VW, TY = TYT * RY;  // 64 x TY points
    static constexpr int HR = 4;                        // x halo: one float4 (so H <= 4)
    static constexpr int BX = TX + 2 * HR, BY = TY + 2 * H;
    static constexpr int PLANE = BX * BY;
    static constexpr int PLANE_BYTES = PLANE * 4;
    static constexpr int SLOT = ((PLANE_BYTES + 127) / 128) * 128;
    static constexpr int P = 8;  // ring slots: H + 1 resident, the rest in flight
    static constexpr int SMEM = P * SLOT;
    static_assert(H >= 1 && H <= 4, "x halo is one float4");
    static_assert((BX * 4) % 16 == 0, "rows of 16-byte multiples (TMA box, float4 loads)");
};

__device__ __forceinline__ float lane(const float4& v, int l) {
    return l == 0 ? v.x : (l == 1 ? v.y : (l == 2 ? v.z : v.w));
}
__device__ __forceinline__ float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }

template <int H, int NT, bool OW, int TYT, int RYB>
__global__ void __launch_bounds__(16 * TYT, 512 / (16 * TYT)) k_lap_v(const __grid_constant__ CUtensorMap tmap,
                                                                      const __grid_constant__ UniPlan U,
                                                                      const LapGrid g, float* __restrict__ du) {
    using C = VCfg<H, TYT, RYB>;
    constexpr int HZ = NT == 3 ? H : 0;
    constexpr int NQ = 2 * HZ + 1;  // queue length = unroll factor of the plane loop
    constexpr int RY = C::RY;
    constexpr int K = 2 * H + 1;
    static_assert(C::P >= H + 2, "ring too short");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[C::P];
    const int nx = (int)U.n[0], ny = (int)U.n[1], nz = (int)U.n[2];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * C::TXT + tx;
    const int64_t sxy = (int64_t)nx * ny;
    const int c0 = (ty * RY + H) * C::BX + C::HR + 4 * tx;  // the first own row's vector inside a slot
    const unsigned int polls = U.wait_polls ? U.wait_polls : (1u << 22);
    if (tid == 0) {
        for (int s = 0; s < C::P; ++s) mbar_init(&mbar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto slot = [&](int gj) -> const float* {
        return reinterpret_cast<const float*>(smem + (gj & (C::P - 1)) * C::SLOT);
    };
    auto w = [&](int t, int k) -> float { return reinterpret_cast<const float*>(U.t[t].w)[k]; };
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
        const int x = x0 + 4 * tx, yr = y0 + ty * RY;
        const int z0 = ci * g.zc;
        const int z1 = min(z0 + g.zc, nz);
        const int npl = (z1 - z0) + 2 * HZ;
        unsigned lmask = 0;  // lanes that are interior rows along x
#pragma unroll
        for (int l = 0; l < 4; ++l)
            if (x + l < nx && x + l + 1 >= U.t[0].flo && x + l + 1 <= U.t[0].fhi) lmask |= 1u << l;
        unsigned vmask = 0;  // own rows that are interior rows along y
#pragma unroll
        for (int j = 0; j < RY; ++j)
            if (lmask && yr + j < ny && yr + j + 1 >= U.t[1].flo && yr + j + 1 <= U.t[1].fhi) vmask |= 1u << j;
        float* dcol = du + (int64_t)yr * nx + x;
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
        float4 q[RY][NQ];  // own vectors; plane p lands in q[.][p % NQ]
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
                    const float* pn = slot(gj);
#pragma unroll
                    for (int j = 0; j < RY; ++j) q[j][ph] = lds4(pn + c0 + j * C::BX);
                    const int z = z0 + p - 2 * HZ;  // the plane whose last z neighbour is plane p
                    const bool bz = (NT < 3) || (z + 1 >= U.t[NT - 1].flo && z + 1 <= U.t[NT - 1].fhi);
                    if (p >= 2 * HZ && vmask && bz) {
                        const float* pc = slot(gj - HZ);  // its centre plane
                        float4 col[RY + 2 * H];           // this vector column at rows yr - H .. yr + RY - 1 + H
#pragma unroll
                        for (int m = 0; m < H; ++m) {
                            col[m] = lds4(pc + c0 + (m - H) * C::BX);
                            col[RY + H + m] = lds4(pc + c0 + (RY + m) * C::BX);
                        }
#pragma unroll
                        for (int j = 0; j < RY; ++j) col[H + j] = q[j][(ph + 1 + HZ) % NQ];
                        float* dz = dcol + (int64_t)z * sxy;
#pragma unroll
                        for (int j = 0; j < RY; ++j) {
                            const float4 L = lds4(pc + c0 + j * C::BX - 4), R = lds4(pc + c0 + j * C::BX + 4);
                            const float4& M = col[H + j];
                            const float v[12] = {L.x, L.y, L.z, L.w, M.x, M.y, M.z, M.w, R.x, R.y, R.z, R.w};
                            float o[4];
#pragma unroll
                            for (int l = 0; l < 4; ++l) {
                                float ax = 0.0f, ay = 0.0f;
#pragma unroll
                                for (int k = 0; k < K; ++k) ax = fmaf(w(0, k), v[4 + l + k - H], ax);
#pragma unroll
                                for (int k = 0; k < K; ++k) ay = fmaf(w(1, k), lane(col[j + k], l), ay);
                                float tot = ax + ay;
                                if constexpr (NT == 3) {
                                    float az = 0.0f;
#pragma unroll
                                    for (int k = 0; k < K; ++k) az = fmaf(w(2, k), lane(q[j][(ph + 1 + k) % NQ], l), az);
                                    tot = tot + az;
                                }
                                o[l] = __fadd_rn(tot, 0.0f);  // -0 -> +0
                            }
                            if (vmask & (1u << j)) {
                                float* d = dz + (int64_t)j * nx;
                                if (lmask == 0xFu) {
                                    float4 r = make_float4(o[0], o[1], o[2], o[3]);
                                    if constexpr (!OW) {
                                        const float4 a = *reinterpret_cast<const float4*>(d);
                                        r = make_float4(o[0] + a.x, o[1] + a.y, o[2] + a.z, o[3] + a.w);
                                    }
                                    *reinterpret_cast<float4*>(d) = r;
                                } else {
#pragma unroll
                                    for (int l = 0; l < 4; ++l)
                                        if (lmask & (1u << l)) {
                                            if constexpr (OW) d[l] = o[l];
                                            else d[l] = o[l] + d[l];
                                        }
                                }
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
        atomicOr(&g_deo_vec_status, 1u);
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

namespace {

template <int H, int NT, int TYT, int RYB>
int launch_v(const UniPlan* up, unsigned int* sched, const void* u, void* du, int ow, cudaStream_t st) {
    using C = VCfg<H, TYT, RYB>;
    if ((uintptr_t)du & 15) return (int)cudaErrorNotSupported;  // 16-byte stores
    alignas(64) CUtensorMap map;
    if (deo_k_encode_map3(&map, u, 4, up->n[0], up->n[1], up->n[2], C::BX, C::BY, 1))
        return (int)cudaErrorNotSupported;
    static int64_t G = 0;
    if (!G) {
        int e = occupancy_grid(k_lap_v<H, NT, true, TYT, RYB>, C::NTHR, C::SMEM, G);
        if (!e) e = occupancy_grid(k_lap_v<H, NT, false, TYT, RYB>, C::NTHR, C::SMEM, G);
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
        k_lap_v<H, NT, true, TYT, RYB><<<grid, dim3(C::TXT, C::TYT), C::SMEM, st>>>(map, *up, g2, (float*)du);
    else
        k_lap_v<H, NT, false, TYT, RYB><<<grid, dim3(C::TXT, C::TYT), C::SMEM, st>>>(map, *up, g2, (float*)du);
    return (int)cudaGetLastError();
}

// Tile variants (threads along y, rows per thread): 0 16 x 2 (64 x 32
// points, 256 threads), 1 8 x 2 (64 x 16, 128 threads), 2 16 x 1 (64 x 16,
// 256 threads), 3 8 x 4 (64 x 32, 128 threads).  Two-axis plans run variant 0.
template <int H, int NT>
int launch_v_cfg(const UniPlan* up, unsigned int* sched, const void* u, void* du, int ow, cudaStream_t st) {
    if constexpr (NT == 3) {
        switch (up->vcfg) {
            case 1: return launch_v<H, NT, 8, 2>(up, sched, u, du, ow, st);
            case 2: return launch_v<H, NT, 16, 1>(up, sched, u, du, ow, st);
            case 3:  // (4 rows of a 2H + 1 deep queue: registers spill beyond H = 2)
                if constexpr (H <= 2) return launch_v<H, NT, 8, 4>(up, sched, u, du, ow, st);
                break;
        }
    }
    return launch_v<H, NT, 16, 2>(up, sched, u, du, ow, st);
}

}  // namespace

extern "C" int deo_k_apply_vec(const UniPlan* up, unsigned int* sched, const void* u, void* du, int ow,
                               void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int H = up->radius;
    if (up->nterms == 3) {
        switch (H) {
            case 1: return launch_v_cfg<1, 3>(up, sched, u, du, ow, st);
            case 2: return launch_v_cfg<2, 3>(up, sched, u, du, ow, st);
            case 3: return launch_v_cfg<3, 3>(up, sched, u, du, ow, st);
        }
    } else if (up->nterms == 2) {
        switch (H) {
            case 1: return launch_v_cfg<1, 2>(up, sched, u, du, ow, st);
            case 2: return launch_v_cfg<2, 2>(up, sched, u, du, ow, st);
            case 3: return launch_v_cfg<3, 2>(up, sched, u, du, ow, st);
        }
    }
    return (int)cudaErrorNotSupported;
}

extern "C" int deo_k_read_vec_status(unsigned int* status) {
    unsigned int v = 0, zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_deo_vec_status, sizeof v);
    if (e != cudaSuccess) return (int)e;
    e = cudaMemcpyToSymbol(g_deo_vec_status, &zero, sizeof zero);
    if (e != cudaSuccess) return (int)e;
    *status = v;
    return 0;
}
