// deo_shell.cu -- the boundary shell of a Laplacian-type plan: the points
// the interior kernels of deo_tma.cu leave out (a boundary row along some
// axis), in the reference's order.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "deo_ptx.cuh"
#include "deo_rows.cuh"

namespace deo {

// The boundary shell of a Laplacian-type plan: every point with a non-band
// row along some axis (it reads a ghost or uses a boundary stencil).  The
// tiled kernels compute the interior box [flo, fhi]^NT; this kernel computes
// the rest in the reference's order (the generic evaluator's arithmetic, tap
// for tap): along an axis where the point's row is an interior row, the
// band's taps; along the others, the boundary row's taps with the ghost
// values of the boundary condition.  With ROWS the boundary rows, weights and
// ghost maps are staged once per CTA from the plan's ShellPlan into shared
// memory and every load of a point is independent of the others; without it,
// they come from the plan's row tables (the generic evaluator itself).
// Index space, ordered so that the 32 points of a warp share their boundary
// row: z outside the box (full planes, x fastest), then z inside & y outside
// (full rows, x fastest), then z, y inside & x outside (y fastest).  The grid
// strides over it.
struct ShellBox {
    int lo[3], hi[3];      // interior box, 0-based inclusive (empty if lo > hi)
    int64_t n[3];
    int64_t cz, cy, cx;    // points in each part
    int small;             // cz + cy + cx < 2^31: index arithmetic by the FastDiv constants below
    FastDiv d_nxny, d_nx, d_nyonx, d_niy, d_nxo;
};

// Coordinates of shell point t (see the index-space order above).
__device__ __forceinline__ void shell_coords(const ShellBox& B, int64_t t, int64_t& x, int64_t& y, int64_t& z) {
    const int64_t nx = B.n[0], ny = B.n[1];
    const int64_t nyo = ny - (B.hi[1] - B.lo[1] + 1);
    const int64_t nxo = nx - (B.hi[0] - B.lo[0] + 1);
    const int64_t niy = B.hi[1] - B.lo[1] + 1;
    if (t < B.cz) {
        int64_t pl, r;
        if (B.small) {
            pl = fast_div((uint32_t)t, B.d_nxny);
            r = t - pl * nx * ny;
            y = fast_div((uint32_t)r, B.d_nx);
        } else {
            pl = t / (nx * ny);
            r = t - pl * nx * ny;
            y = r / nx;
        }
        x = r - y * nx;
        z = pl < B.lo[2] ? pl : pl - B.lo[2] + B.hi[2] + 1;
    } else if (t < B.cz + B.cy) {
        const int64_t q = t - B.cz;
        int64_t pl, r, row;
        if (B.small) {
            pl = fast_div((uint32_t)q, B.d_nyonx);
            r = q - pl * nyo * nx;
            row = fast_div((uint32_t)r, B.d_nx);
        } else {
            pl = q / (nyo * nx);
            r = q - pl * nyo * nx;
            row = r / nx;
        }
        z = B.lo[2] + pl;
        x = r - row * nx;
        y = row < B.lo[1] ? row : row - B.lo[1] + B.hi[1] + 1;
    } else {
        const int64_t q = t - B.cz - B.cy;
        int64_t line, zz;
        if (B.small) {
            line = fast_div((uint32_t)q, B.d_niy);  // (z, x column) pairs, y fastest
            zz = fast_div((uint32_t)line, B.d_nxo);
        } else {
            line = q / niy;
            zz = line / nxo;
        }
        y = B.lo[1] + (q - line * niy);
        z = B.lo[2] + zz;
        const int64_t c = line - zz * nxo;
        x = c < B.lo[0] ? c : c - B.lo[0] + B.hi[0] + 1;
    }
}

__device__ unsigned int g_deo_shell_status;  // bit 0: a bounded mbarrier wait gave up

// Face kernel: the shell as faces, each CTA evaluating one tile of one face
// from a shared-memory box filled by one TMA copy.  Face A (the axis of its
// boundary rows), end e (low / high): the boundary rows of that end along A
// times a tile of the two other axes b1 < b2.  Parts: A = 3 (all of axes 1, 2),
// A = 2 (axis 3 interior only), A = 1 (axes 2, 3 interior only), so every
// shell point is evaluated once.  The box covers the points the rows read
// along A (with the ghost), the tile plus the band halo along b1, b2; a term
// whose boundary row (at an edge or corner of the shell) reads outside the box
// reads global memory instead.  The arithmetic is the generic evaluator's.
struct FaceGrid {
    int n[3];
    int cta0[4];      // first CTA of face A = 3, 2, 1 (axis index 2, 1, 0); cta0[3] = all
    int tiles1[3], tiles2[3];  // tiles along b1, b2 of face A (index = axis index of A)
    int tw1[3], tw2[3];        // tile extents along b1, b2
    int r1[3], r2[3];          // tiled range along b1, b2: [r, e)
    int e1[3], e2[3];
    int halo[3];               // box halo along each axis when it is an in-face axis
    int orgA[3][2];            // box origin along A for the low / high end
    int box[3][3];             // box dims (x, y, z) of face A
    int box_bytes[3];
    int nbuf;                  // box buffers: 2 = the next tile's copy in flight while a tile is computed
    int slot;                  // bytes per buffer (a multiple of 128)
};

// Tile blk of the face grid: face axis A, end e, its first coordinates
// (c1, c2) along the two other axes b1 < b2, and its box's origin.
struct FaceTile {
    int A, e, c1, c2, o0, o1, o2;
};
__device__ __forceinline__ FaceTile face_tile_at(const FaceGrid& G, int blk) {
    FaceTile f;
    const int A = blk < G.cta0[1] ? 2 : (blk < G.cta0[2] ? 1 : 0);
    const int local = blk - G.cta0[2 - A];
    const int per_end = G.tiles1[A] * G.tiles2[A];
    const int e = local / per_end;
    const int rem = local - e * per_end;
    const int tt2 = rem / G.tiles1[A], tt1 = rem - tt2 * G.tiles1[A];
    f.A = A;
    f.e = e;
    f.c1 = G.r1[A] + tt1 * G.tw1[A];
    f.c2 = G.r2[A] + tt2 * G.tw2[A];
    // box origin: along A the end's origin; along b1 < b2 the tile less the halo
    const int oA = G.orgA[A][e];
    f.o0 = A == 0 ? oA : f.c1 - G.halo[0];
    f.o1 = A == 1 ? oA : (A == 0 ? f.c1 - G.halo[1] : f.c2 - G.halo[1]);
    f.o2 = A == 2 ? oA : f.c2 - G.halo[2];
    return f;
}

// The terms of a face point other than the face's own axis A, added into
// acc in axis order around the A term `va` (the generic evaluator's order):
// a band from the box, or (at edges and corners of the shell) the other
// axis's boundary row, from the box when its points lie in it.  HB: the
// band radius when known at compile time (0: U.radius).  A is a template
// parameter so that every coordinate array is indexed by constants and
// stays in registers.
template <typename T, int NT, int MAXW, int HB, int A>
__device__ __forceinline__ T face_sum(const ShellTerm* S, const UniPlan& U, const T* __restrict__ pc, T va,
                                      const int (&c)[3], const int (&org)[3], const int (&bd)[3],
                                      const int64_t (&sb)[3], const T* __restrict__ u, int64_t gidx,
                                      const int64_t (&gst)[3]) {
    T acc = T(0);
#pragma unroll
    for (int b = 0; b < NT; ++b) {
        T v;
        if (b == A) {
            v = va;
        } else {
            const int ib = c[b] + 1;
            if (ib >= U.t[b].flo && ib <= U.t[b].fhi) {
                if constexpr (HB > 0) v = shell_band_h<T, HB>(U.t[b], pc, sb[b]);
                else v = shell_band<T>(U.t[b], U.radius, pc, 0, sb[b]);
            } else {
                const ShellTerm& SB = S[b];
                const bool low = ib <= SB.nlo;
                const int w0 = low ? 0 : SB.len - SB.whi;
                const int w1 = low ? SB.wlo : SB.len;
                if (w0 >= org[b] && w1 <= org[b] + bd[b])
                    v = shell_row_cold<T, MAXW>(SB, pc - c[b] * sb[b], sb[b], ib);
                else
                    v = shell_row_cold<T, MAXW>(SB, u + gidx - c[b] * gst[b], gst[b], ib);
            }
        }
        acc = (b == 0) ? v : acc + v;
    }
    return zero_fix(acc);
}

// One face tile from its landed box: one thread per line of the tile along
// A, the line's ghosts once (the boundary condition's map of its end points,
// from the box), then its boundary rows at end e, each with the other axes'
// terms.  (c1, c2): the tile's first coordinates along b1 < b2; org: the
// box's origin.
template <typename T, int NT, int MAXW, int HB, int A>
__device__ __forceinline__ void face_tile(const ShellTerm* S, const UniPlan& U, const FaceGrid& G,
                                          const T* __restrict__ box, const T* __restrict__ u, T* __restrict__ du,
                                          int ow, int e, int c1, int c2, int o0, int o1, int o2) {
    if constexpr (A < NT) {
        constexpr int b1 = A == 0 ? 1 : 0, b2 = A == 2 ? 1 : 2;
        const int org[3] = {o0, o1, o2};
        const int bd[3] = {G.box[A][0], G.box[A][1], G.box[A][2]};
        const int64_t nx = G.n[0], sxy = (int64_t)G.n[0] * G.n[1];
        const int64_t gst[3] = {1, nx, sxy};
        const int64_t sb[3] = {1, bd[0], (int64_t)bd[0] * bd[1]};
        const ShellTerm& SA = S[A];
        const int nrows = e ? SA.nhi : SA.nlo;
        const int cA0 = e ? SA.len - SA.nhi : 0;
        const int tw1 = G.tw1[A], tw2 = G.tw2[A];
        const int e1 = G.e1[A], e2 = G.e2[A];
        const int L2 = SA.len + 2;
        const int row0 = e ? SA.nlo : 0;
        bool need_l = false, need_r = false;
        for (int r = 0; r < nrows; ++r) {
            const ShellRow& R = SA.row[row0 + r];
            need_l |= R.p0 == 1;
            need_r |= R.p0 + R.nk - 1 == L2;
        }
        const bool line_in_box = (e ? SA.len - SA.whi : 0) >= org[A] && (e ? SA.len : SA.wlo) <= org[A] + bd[A];
        for (int q = threadIdx.x; q < tw1 * tw2; q += blockDim.x) {
            const int p2 = q / tw1, p1 = q - p2 * tw1;
            int c[3];
            c[A] = 0;
            c[b1] = c1 + p1;
            c[b2] = c2 + p2;
            if (c[b1] >= e1 || c[b2] >= e2) continue;
            const int64_t g0 = c[0] + c[1] * nx + (int64_t)c[2] * sxy;  // the line's first point
            const T* box0 = box + (int64_t)(c[2] - org[2]) * sb[2] + (int64_t)(c[1] - org[1]) * sb[1] + (c[0] - org[0]);
            const T* line = line_in_box ? box0 : u + g0;  // position 0 of the line along A
            const int64_t ls = line_in_box ? sb[A] : gst[A];
            const T gl = need_l ? shell_ghost<T, MAXW>(SA, line, ls, true) : T(0);
            const T gr = need_r ? shell_ghost<T, MAXW>(SA, line, ls, false) : T(0);
            for (int r = 0; r < nrows; ++r) {
                c[A] = cA0 + r;
                const ShellRow& R = SA.row[row0 + r];
                const T va = row_eval<T, MAXW>(R, line, ls, L2, gl, gr);
                const int64_t gidx = g0 + (int64_t)c[A] * gst[A];
                const T* pc = box0 + (int64_t)c[A] * sb[A];
                const T tot = face_sum<T, NT, MAXW, HB, A>(S, U, pc, va, c, org, bd, sb, u, gidx, gst);
                du[gidx] = ow ? tot : tot + du[gidx];
            }
        }
    }
}

// A persistent grid over the face tiles (tiles blockIdx.x, + gridDim.x, ...),
// 128 threads per CTA.  With two buffers the next tile's box copy is issued
// before the current tile is computed; buffer b's mbarrier completes once per
// use, so its phase is the parity of its use count.
template <typename T, int NT, int MAXW, int HB>
__global__ void __launch_bounds__(128, 4) k_face(const __grid_constant__ CUtensorMap m0,
                                                 const __grid_constant__ CUtensorMap m1,
                                                 const __grid_constant__ CUtensorMap m2,
                                                 const __grid_constant__ FaceGrid G, const __grid_constant__ UniPlan U,
                                                 const ShellPlan* __restrict__ SPg, const T* __restrict__ u,
                                                 T* __restrict__ du, int ow) {
    static_assert(sizeof(ShellTerm) % 8 == 0, "ShellTerm copied in 8-byte words");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(16) ShellTerm S[NT];
    __shared__ __align__(8) uint64_t mbar[2];
    const int nb = G.nbuf, total = G.cta0[3], stride = (int)gridDim.x;
    auto issue = [&](int blk, int buf) {
        const FaceTile f = face_tile_at(G, blk);
        mbar_expect_tx(&mbar[buf], (uint32_t)G.box_bytes[f.A]);
        tma_load_3d(smem + buf * G.slot, f.A == 0 ? &m0 : (f.A == 1 ? &m1 : &m2), &mbar[buf], f.o0, f.o1, f.o2);
    };
    // test hook: each CTA's first box copy withheld, so that its wait runs out
    const bool hold0 = U.test_withhold > 0;
    if (threadIdx.x == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        fence_mbar_init();
        if ((int)blockIdx.x < total && !hold0) issue(blockIdx.x, 0);  // in flight while the terms are staged
    }
    {
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(SPg->t);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(S);
        for (int q = threadIdx.x; q < (int)(NT * sizeof(ShellTerm) / 8); q += blockDim.x) dst[q] = __ldg(src + q);
    }
    __syncthreads();
    int i = 0;
    for (int blk = blockIdx.x; blk < total; blk += stride, ++i) {
        const int buf = nb == 2 ? (i & 1) : 0;
        const uint32_t ph = nb == 2 ? ((uint32_t)(i >> 1) & 1u) : ((uint32_t)i & 1u);
        const int nxt = blk + stride;
        // the other buffer's last reader (tile i - 1) finished at the barrier closing its iteration
        if (threadIdx.x == 0) {
            if (nb == 2) {
                if (nxt < total) issue(nxt, buf ^ 1);
            } else if (i > 0) {
                issue(blk, 0);
            }
        }
        bool timeout = false;
        {
            const unsigned int polls = U.wait_polls ? U.wait_polls : (1u << 22);
            uint32_t it = 0;
            while (!mbar_try_wait(&mbar[buf], ph)) {
                if (++it > polls) {
                    timeout = true;
                    break;
                }
            }
        }
        if (__syncthreads_or(timeout)) {
            if (threadIdx.x == 0) {
                atomicOr(&g_deo_shell_status, 1u);
                // the copies that may still be in flight: this tile's (unless withheld), the next tile's
                if (!(hold0 && i == 0))
                    for (uint32_t it = 0; it < (1u << 22); ++it)
                        if (mbar_try_wait(&mbar[buf], ph)) break;
                if (nb == 2 && nxt < total)
                    for (uint32_t it = 0; it < (1u << 22); ++it)
                        if (mbar_try_wait(&mbar[buf ^ 1], (uint32_t)((i + 1) >> 1) & 1u)) break;
            }
            return;
        }
        const FaceTile f = face_tile_at(G, blk);
        const T* box = reinterpret_cast<const T*>(smem + buf * G.slot);
        if (f.A == 0) face_tile<T, NT, MAXW, HB, 0>(S, U, G, box, u, du, ow, f.e, f.c1, f.c2, f.o0, f.o1, f.o2);
        else if (f.A == 1) face_tile<T, NT, MAXW, HB, 1>(S, U, G, box, u, du, ow, f.e, f.c1, f.c2, f.o0, f.o1, f.o2);
        else face_tile<T, NT, MAXW, HB, 2>(S, U, G, box, u, du, ow, f.e, f.c1, f.c2, f.o0, f.o1, f.o2);
        __syncthreads();  // every thread is done with the box before a later copy overwrites it
    }
}

// Line-oriented shell kernel: one thread per (line along axis A, end of the
// line) computing the nlo (or nhi) boundary rows of that end from global
// memory; the ghost of that end once for all of them, the band taps (or, at
// edges and corners, the boundary rows) of the other axes per point.  Lines:
// axis 3 (all x, y), axis 2 (z interior, all x), axis 1 (y, z interior), the
// end the slowest index so that a warp shares its boundary rows.  Small in
// shared memory and registers, so that one CTA per SM can run beside the
// interior kernel and overlap its FP64 work with the interior's integer work.
struct ShellLines {
    int64_t l2, l1, l0;  // lines of each part (each counted twice: low and high end)
    FastDiv d_nx, d_iy;
    int small;           // 2 * (l2 + l1 + l0) < 2^31
};

template <typename T, int NT, int A, int MAXW>
__device__ __forceinline__ void shell_line(const ShellTerm* S, const UniPlan& U, const T* __restrict__ u,
                                           T* __restrict__ du, int ow, int e, int64_t c0, int64_t c1, int64_t c2,
                                           int64_t nx, int64_t sxy) {
    const ShellTerm& SA = S[A];
    const int nrows = e ? SA.nhi : SA.nlo;
    const int ifirst = e ? SA.len - SA.nhi + 1 : 1;
    const int L2 = SA.len + 2;
    const int64_t st[3] = {1, nx, sxy};
    int64_t c[3] = {c0, c1, c2};
    c[A] = 0;
    const T* line = u + c[0] + c[1] * nx + (NT == 3 ? c[2] * sxy : 0);
    bool need_l = false, need_r = false;
    for (int r = 0; r < nrows; ++r) {
        const ShellRow& R = SA.row[(e ? SA.nlo : 0) + r];
        need_l |= R.p0 == 1;
        need_r |= R.p0 + R.nk - 1 == L2;
    }
    const T gl = need_l ? shell_ghost<T, MAXW>(SA, line, st[A], true) : T(0);
    const T gr = need_r ? shell_ghost<T, MAXW>(SA, line, st[A], false) : T(0);
#pragma unroll 1
    for (int r = 0; r < nrows; ++r) {
        const ShellRow& R = SA.row[(e ? SA.nlo : 0) + r];
        c[A] = ifirst + r - 1;
        const int64_t idx = c[0] + c[1] * nx + (NT == 3 ? c[2] * sxy : 0);
        T acc = T(0);
#pragma unroll
        for (int b = 0; b < NT; ++b) {
            T v;
            if (b == A) {
                v = row_eval<T, MAXW>(R, line, st[A], L2, gl, gr);
            } else {
                const int ib = (int)c[b] + 1;
                v = (ib >= U.t[b].flo && ib <= U.t[b].fhi)
                        ? shell_band<T>(U.t[b], U.radius, u, idx, st[b])
                        : shell_row_cold<T, MAXW>(S[b], u + idx - c[b] * st[b], st[b], ib);
            }
            acc = (b == 0) ? v : acc + v;
        }
        const T tot = zero_fix(acc);
        du[idx] = ow ? tot : tot + du[idx];
    }
}

template <typename T, int NT, int MAXW>
__global__ void __launch_bounds__(256) k_shell_lines(const __grid_constant__ ShellBox B,
                                                     const __grid_constant__ ShellLines SL,
                                                     const __grid_constant__ UniPlan U,
                                                     const ShellPlan* __restrict__ SPg, const T* __restrict__ u,
                                                     T* __restrict__ du, int ow) {
    static_assert(sizeof(ShellTerm) % 8 == 0, "ShellTerm copied in 8-byte words");
    __shared__ __align__(16) ShellTerm S[NT];
    {
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(SPg->t);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(S);
        for (int q = threadIdx.x; q < (int)(NT * sizeof(ShellTerm) / 8); q += blockDim.x) dst[q] = __ldg(src + q);
        __syncthreads();
    }
    const int64_t nx = B.n[0], ny = B.n[1];
    const int64_t iy = B.hi[1] - B.lo[1] + 1;
    const int64_t sxy = nx * ny;
    const int64_t total = 2 * (SL.l2 + SL.l1 + SL.l0);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t q = t;
        if (q < 2 * SL.l2) {
            const int e = q >= SL.l2;
            q -= e * SL.l2;
            const int64_t yy = SL.small ? (int64_t)fast_div((uint32_t)q, SL.d_nx) : q / nx;
            if constexpr (NT == 3) shell_line<T, NT, 2, MAXW>(S, U, u, du, ow, e, q - yy * nx, yy, 0, nx, sxy);
        } else if ((q -= 2 * SL.l2) < 2 * SL.l1) {
            const int e = q >= SL.l1;
            q -= e * SL.l1;
            const int64_t zi = SL.small ? (int64_t)fast_div((uint32_t)q, SL.d_nx) : q / nx;
            shell_line<T, NT, 1, MAXW>(S, U, u, du, ow, e, q - zi * nx, 0, B.lo[2] + zi, nx, sxy);
        } else {
            q -= 2 * SL.l1;
            const int e = q >= SL.l0;
            q -= e * SL.l0;
            const int64_t zi = SL.small ? (int64_t)fast_div((uint32_t)q, SL.d_iy) : q / iy;
            shell_line<T, NT, 0, MAXW>(S, U, u, du, ow, e, 0, B.lo[1] + (q - zi * iy), B.lo[2] + zi, nx, sxy);
        }
    }
}

// The same shell with the boundary rows from the plan's row tables (plans
// whose boundary rows do not fit a ShellPlan).
template <typename T, int NT>
__global__ void __launch_bounds__(256) k_shell_generic(const __grid_constant__ ShellBox B,
                                                       const __grid_constant__ UniPlan U,
                                                       const PlanDev* __restrict__ P, const T* __restrict__ u,
                                                       T* __restrict__ du, int overwrite) {
    const int64_t nx = B.n[0], ny = B.n[1];
    const int64_t total = B.cz + B.cy + B.cx;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x, y, z;
        shell_coords(B, t, x, y, z);
        const int64_t idx = (z * ny + y) * nx + x;
        const int64_t crd[3] = {x, y, z};
        const int64_t st[3] = {1, nx, nx * ny};
        T acc = T(0);
#pragma unroll
        for (int a = 0; a < NT; ++a) {
            const int i = (int)crd[a] + 1;
            const T r = (i >= U.t[a].flo && i <= U.t[a].fhi) ? shell_band<T>(U.t[a], U.radius, u, idx, st[a])
                                                             : eval_term_cold<T>(P->t[a], u, idx, i);
            acc = (a == 0) ? r : acc + r;
        }
        const T tot = zero_fix(acc);
        du[idx] = overwrite ? tot : tot + du[idx];
    }
}

// The transposed operator on the points outside the box of the interior
// kernels' transposed applies, one thread per point.  Along an axis where the
// point's column is read only by band rows (inside that axis's [flo, fhi] of
// U, whose bands carry their taps reversed) the term is the reversed band,
// summed as the generic column evaluator sums its rows; along the others the
// generic column evaluator (adj_term: every row touching the column, the
// ghost columns folded back through the BC map).  Terms added in axis order.
template <typename T, int NT>
__global__ void __launch_bounds__(256) k_shell_adj(const __grid_constant__ ShellBox B, const __grid_constant__ UniPlan U,
                                                   const PlanDev* __restrict__ P, const T* __restrict__ d,
                                                   T* __restrict__ ub, int overwrite) {
    const int64_t nx = B.n[0], ny = B.n[1];
    const int64_t total = B.cz + B.cy + B.cx;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t x, y, z;
        shell_coords(B, t, x, y, z);
        const int64_t idx = (z * ny + y) * nx + x;
        const int64_t crd[3] = {x, y, z};
        const int64_t st[3] = {1, nx, nx * ny};
        T acc = T(0);
#pragma unroll
        for (int a = 0; a < NT; ++a) {
            const int j = (int)crd[a] + 1;
            const T r = (j >= U.t[a].flo && j <= U.t[a].fhi) ? shell_band<T>(U.t[a], U.radius, d, idx, st[a])
                                                             : adj_term_cold<T>(P->t[a], d, idx, j);
            acc = (a == 0) ? r : acc + r;
        }
        ub[idx] = overwrite ? acc : acc + ub[idx];
    }
}

}  // namespace deo

using namespace deo;

template <typename K>
static int64_t shell_grid(K kernel, int64_t total) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0);
    if (per_sm < 1) per_sm = 1;
    return std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, (int64_t)deo_k_num_sms() * per_sm));
}

// Face grid and the three tensor maps; returns cudaErrorNotSupported when a
// box would exceed the TMA / shared-memory limits (the caller falls back).
// small: one persistent CTA per SM over 32 x 8 tiles (16 x 8 on the x faces),
// one box buffer, small enough to run beside the Float64 interior kernel's
// CTAs; else 32 x 8 tiles, two box buffers and as many persistent CTAs as fit
// on the device.  128 threads per CTA either way.
template <typename T, int NT>
static int face_launch(const UniPlan* up, const ShellPlan* sp, const ShellPlan* sp_dev, const void* u, void* du, int ow,
                       cudaStream_t st, bool small) {
    const int ES = (int)sizeof(T);
    const int al = 16 / ES;  // TMA: x coordinates and x extents in multiples of 16 bytes
    FaceGrid G{};
    int lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        G.n[k] = (int)up->n[k];
        lo[k] = k < NT ? up->t[k].flo - 1 : 0;
        hi[k] = k < NT ? up->t[k].fhi - 1 : G.n[k] - 1;
        if (lo[k] > hi[k]) return (int)cudaErrorNotSupported;  // no interior along k: generic shell
    }
    const int H = up->radius;
    const int HR = ((H * ES + 15) / 16) * 16 / ES;
    G.halo[0] = HR;
    G.halo[1] = NT >= 2 ? H : 0;
    G.halo[2] = NT >= 3 ? H : 0;
    int cta = 0;
    size_t smem_max = 0;
    for (int A = 2; A >= 0; --A) {
        G.cta0[2 - A] = cta;
        if (A >= NT) continue;
        const ShellTerm& SA = sp->t[A];
        const int b1 = A == 0 ? 1 : 0, b2 = A == 2 ? 1 : 2;
        // tiled ranges: parts as in the kernel comment
        auto range = [&](int b, int& r, int& e) {
            const bool interior_only = (A == 1 && b == 2) || (A == 0);
            r = interior_only ? lo[b] : 0;
            e = interior_only ? hi[b] + 1 : G.n[b];
        };
        range(b1, G.r1[A], G.e1[A]);
        range(b2, G.r2[A], G.e2[A]);
        G.tw1[A] = std::min(small && b1 == 1 ? 16 : 32, G.e1[A] - G.r1[A]);
        G.tw2[A] = (b2 < NT) ? std::min(8, G.e2[A] - G.r2[A]) : 1;
        G.tiles1[A] = (G.e1[A] - G.r1[A] + G.tw1[A] - 1) / G.tw1[A];
        G.tiles2[A] = (G.e2[A] - G.r2[A] + G.tw2[A] - 1) / G.tw2[A];
        // box along A: the points both ends' rows read
        int extA;
        if (A == 0) {
            const int olo = 0, ohi = ((G.n[0] - SA.whi) / al) * al;
            extA = std::max(((SA.wlo + al - 1) / al) * al, ((G.n[0] - ohi + al - 1) / al) * al);
            G.orgA[0][0] = olo;
            G.orgA[0][1] = ohi;
        } else {
            extA = std::max(SA.wlo, SA.whi);
            G.orgA[A][0] = 0;
            G.orgA[A][1] = G.n[A] - SA.whi;
        }
        int bdim[3];
        bdim[A] = extA;
        bdim[b1] = G.tw1[A] + 2 * G.halo[b1];
        bdim[b2] = G.tw2[A] + 2 * G.halo[b2];
        if (b1 == 0 && (bdim[0] % al)) bdim[0] += al - bdim[0] % al;
        for (int k = 0; k < 3; ++k) {
            if (bdim[k] < 1 || bdim[k] > 256) return (int)cudaErrorNotSupported;
            G.box[A][k] = bdim[k];
        }
        G.box_bytes[A] = bdim[0] * bdim[1] * bdim[2] * ES;
        smem_max = std::max(smem_max, (size_t)G.box_bytes[A]);
        cta += 2 * G.tiles1[A] * G.tiles2[A];
    }
    G.cta0[3] = cta;
    if (cta == 0) return 0;
    G.nbuf = small ? 1 : 2;
    G.slot = (int)((smem_max + 127) / 128 * 128);
    const size_t dyn = (size_t)G.nbuf * G.slot;
    if (dyn > 200 * 1024) return (int)cudaErrorNotSupported;
    alignas(64) CUtensorMap maps[3];
    for (int A = 0; A < 3; ++A) {
        if (A >= NT) {
            maps[A] = maps[0];
            continue;
        }
        const int e = deo_k_encode_map3(&maps[A], u, ES, G.n[0], G.n[1], G.n[2], G.box[A][0], G.box[A][1],
                                        G.box[A][2]);
        if (e) return e;
    }
    if (NT < 3) maps[2] = maps[0];
    auto go = [&](auto kernel) -> int {
        // per instantiation (told apart by address: they share one function type) the dynamic shared
        // memory it was last allowed, and its resident CTAs per SM for a given dynamic size
        static std::mutex mu;
        static std::map<const void*, size_t> smem_set;
        static std::map<std::pair<const void*, size_t>, int> per_sm;
        std::lock_guard<std::mutex> lk(mu);
        const void* key = reinterpret_cast<const void*>(kernel);
        size_t& set = smem_set[key];
        if (dyn > set) {
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
            // the interior kernels run with the largest shared-memory carveout; asking for the same lets
            // this kernel's CTAs share their SMs
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
            if (e != cudaSuccess) return (int)e;
            set = dyn;
        }
        int& occ = per_sm[{key, dyn}];
        if (occ == 0) {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 128, dyn) != cudaSuccess || occ < 1)
                occ = 1;
        }
        const unsigned grid = (unsigned)std::min(cta, (small ? 1 : occ) * deo_k_num_sms());
        kernel<<<grid, 128, dyn, st>>>(maps[0], maps[1], maps[2], G, *up, sp_dev, (const T*)u, (T*)du, ow);
        return (int)cudaGetLastError();
    };
    // rows and ghost maps of at most 8 points with the band radius known at compile time; else general
    if (sp->maxw <= 8) {
        switch (up->radius) {
            case 1: return go(k_face<T, NT, 8, 1>);
            case 2: return go(k_face<T, NT, 8, 2>);
            case 3: return go(k_face<T, NT, 8, 3>);
            case 4: return go(k_face<T, NT, 8, 4>);
        }
    }
    return go(k_face<T, NT, 16, 0>);
}

// The shell's index space: the points of the array outside the box
// [flo, fhi] of every term's axis (UniTerm; 0-based below).
static ShellBox shell_box(const UniPlan* up) {
    ShellBox B{};
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
    B.small = total < (1LL << 31) && nx * ny < (1LL << 31);
    if (B.small) {
        auto fd = [](int64_t d) { return make_fastdiv((uint32_t)std::max<int64_t>(d, 1)); };
        B.d_nxny = fd(nx * ny);
        B.d_nx = fd(nx);
        B.d_nyonx = fd((ny - iy) * nx);
        B.d_niy = fd(iy);
        B.d_nxo = fd(nx - ix);
    }
    return B;
}

template <typename T, int NT>
static int launch_shell_t(const UniPlan* up, const ShellPlan* sp, const ShellPlan* sp_dev, int mode,
                          const PlanDev* dp, const void* u, void* du, int ow, cudaStream_t st, const char** kernel) {
    ShellBox B = shell_box(up);
    const int64_t ix = B.hi[0] - B.lo[0] + 1, iy = B.hi[1] - B.lo[1] + 1, iz = B.hi[2] - B.lo[2] + 1;
    const int64_t nx = B.n[0], ny = B.n[1];
    (void)ny;
    const int64_t total = B.cz + B.cy + B.cx;
    if (total == 0) return 0;
    const bool have_lines = sp && sp_dev && B.lo[0] <= B.hi[0] && B.lo[1] <= B.hi[1] && B.lo[2] <= B.hi[2];
    // Float64 alone: the line kernel (FP64-bound, full grid).  Otherwise the face kernel: a shared-memory
    // box per tile; beside a Float64 interior kernel in small CTAs that fit next to its CTAs, so that the
    // shell's FP64 work overlaps the interior's integer work.
    const int pick = up->shell_kernel;
    if (have_lines && (pick == 2 || (pick == 0 && sizeof(T) == 8 && mode == DEO_SHELL_ALONE))) {
        ShellLines SL{};
        const int64_t niz = NT == 3 ? iz : 1;
        SL.l2 = NT == 3 ? nx * ny : 0;
        SL.l1 = nx * niz;
        SL.l0 = iy * niz;
        SL.small = 2 * (SL.l2 + SL.l1 + SL.l0) < (1LL << 31);
        SL.d_nx = make_fastdiv((uint32_t)std::max<int64_t>(nx, 1));
        SL.d_iy = make_fastdiv((uint32_t)std::max<int64_t>(iy, 1));
        const int64_t lines = 2 * (SL.l2 + SL.l1 + SL.l0);
        auto go = [&](auto kernel) {
            static int64_t g = 0;
            if (!g) g = shell_grid(kernel, 1LL << 40);
            // beside the interior kernel: one CTA per SM (fits next to its CTAs); alone: a full grid
            const int64_t grid =
                std::min<int64_t>(mode == DEO_SHELL_CONCURRENT ? deo_k_num_sms() : g, (lines + 255) / 256);
            kernel<<<(unsigned)std::max<int64_t>(grid, 1), 256, 0, st>>>(B, SL, *up, sp_dev, (const T*)u, (T*)du, ow);
        };
        if (sp->maxw <= 8) go(k_shell_lines<T, NT, 8>);
        else go(k_shell_lines<T, NT, 16>);
        *kernel = "k_shell_lines";
        return (int)cudaGetLastError();
    }
    if (sp && sp_dev && pick != 3) {
        // Float64 interiors are long: a small persistent shell beside them; Float32 interiors are short: a full grid
        const int e = face_launch<T, NT>(up, sp, sp_dev, u, du, ow, st, mode == DEO_SHELL_CONCURRENT && sizeof(T) == 8);
        if (e != (int)cudaErrorNotSupported) {
            *kernel = "k_face";
            return e;
        }
    }
    *kernel = "k_shell_generic";
    static int64_t g = 0;
    if (!g) g = shell_grid(k_shell_generic<T, NT>, 1LL << 40);
    k_shell_generic<T, NT><<<(unsigned)std::min(g, (total + 255) / 256), 256, 0, st>>>(B, *up, dp, (const T*)u,
                                                                                      (T*)du, ow);
    return (int)cudaGetLastError();
}

template <typename T>
static int launch_shell(const UniPlan* up, const ShellPlan* sp, const ShellPlan* sp_dev, int mode, const PlanDev* dp,
                        const void* u, void* du, int ow, cudaStream_t st, const char** kernel) {
    if (up->radius < 1 || up->radius > 4) return (int)cudaErrorNotSupported;
    if (up->nterms == 3) return launch_shell_t<T, 3>(up, sp, sp_dev, mode, dp, u, du, ow, st, kernel);
    if (up->nterms == 2) return launch_shell_t<T, 2>(up, sp, sp_dev, mode, dp, u, du, ow, st, kernel);
    return (int)cudaErrorNotSupported;
}

extern "C" int deo_k_apply_shell(const UniPlan* up, const ShellPlan* sp, const ShellPlan* sp_dev, int mode,
                                 const PlanDev* dp, int dtype, const void* u, void* du, int overwrite, void* stream,
                                 const char** kernel) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    static const char* none = "";
    if (!kernel) kernel = &none;
    return dtype == 0 ? launch_shell<double>(up, sp, sp_dev, mode, dp, u, du, overwrite, st, kernel)
                      : launch_shell<float>(up, sp, sp_dev, mode, dp, u, du, overwrite, st, kernel);
}

extern "C" int deo_k_apply_shell_adj(const UniPlan* up, const PlanDev* dp, int dtype, const void* d, void* ub,
                                     int overwrite, int concurrent, void* stream) {
    if (up->nterms < 2 || up->nterms > 3) return (int)cudaErrorNotSupported;
    const ShellBox B = shell_box(up);
    const int64_t total = B.cz + B.cy + B.cx;
    if (total == 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto go = [&](auto kernel, const auto* in, auto* out) {
        static int64_t g = 0;
        if (!g) g = shell_grid(kernel, 1LL << 40);
        // beside the interior kernel: one CTA per SM (fits next to its CTAs); alone: a full grid
        const int64_t grid = std::min<int64_t>(concurrent ? deo_k_num_sms() : g, (total + 255) / 256);
        kernel<<<(unsigned)std::max<int64_t>(grid, 1), 256, 0, st>>>(B, *up, dp, in, out, overwrite);
    };
    if (up->nterms == 3) {
        if (dtype == 0) go(k_shell_adj<double, 3>, (const double*)d, (double*)ub);
        else go(k_shell_adj<float, 3>, (const float*)d, (float*)ub);
    } else {
        if (dtype == 0) go(k_shell_adj<double, 2>, (const double*)d, (double*)ub);
        else go(k_shell_adj<float, 2>, (const float*)d, (float*)ub);
    }
    return (int)cudaGetLastError();
}

extern "C" int deo_k_read_shell_status(unsigned int* status) {
    unsigned int v = 0, zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_deo_shell_status, sizeof v);
    if (e != cudaSuccess) return (int)e;
    e = cudaMemcpyToSymbol(g_deo_shell_status, &zero, sizeof zero);
    if (e != cudaSuccess) return (int)e;
    *status = v;
    return 0;
}
