// deo_lap.cuh -- the work units of the TMA-fed Laplacian-type kernels
// (deo_tma.cu, deo_vec.cu): a persistent grid walks units of (tile x, tile y,
// z chunk), claimed from a device counter; the host picks the z chunk and
// the grid size.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "deo_internal.h"

namespace deo {

// Work unit u = (tile x, tile y, z chunk); a persistent grid of G CTAs takes
// units b, b + G, b + 2G, ... (static, so one plan may run on several streams
// at once).  Planes stream through the ring with a running count, so slot and
// mbarrier phase carry over from one unit to the next.
struct LapGrid {
    int tiles_x, tiles_y, chunks, zc;
    int units;
    int perm;  // coprime with units: unit k of the round-robin is (k * perm) % units,
               // so one CTA's units are spread over tile columns and z chunks
    unsigned int* sched;  // null: static round-robin; else a zeroed device counter the CTAs claim units from
};

// The next unit of a CTA: with g.sched claimed from the counter (dynamic, so
// CTAs that share their SM with other work take fewer units), else k_static.
// Every thread of the CTA calls it (it contains a barrier).
__device__ __forceinline__ int claim_unit(const LapGrid& g, int& s_next, int k_static) {
    if (!g.sched) return k_static;
    if (threadIdx.x == 0 && threadIdx.y == 0) s_next = (int)atomicAdd(g.sched, 1u);
    __syncthreads();
    return s_next;
}


// Units and z chunk for a persistent grid of G CTAs (see LapGrid).
static inline LapGrid make_grid(const UniPlan* up, int tx, int ty, int H, int nt, int64_t G) {
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
    g.sched = nullptr;
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
static inline int occupancy_grid(K kernel, int threads, int smem, int64_t& G) {
    static thread_local int dummy = 0;
    (void)dummy;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    // the largest shared-memory carveout: an SM configured for the interior's CTAs alone would leave
    // no room for the boundary-shell CTAs that run beside them
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return (int)e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (e != cudaSuccess || per_sm < 1) per_sm = 1;
    G = (int64_t)sms * per_sm;
    return 0;
}


}  // namespace deo
