// deo_bfx.cuh -- block fixed-point interior kernel for Float64 three-axis
// Laplacian-type plans (included by deo_tma.cu, which provides the TMA ring
// helpers, LapGrid and claim_unit).
//
// The reference sums each axis term tap by tap in Float64.  Evaluated that
// way a 13-point 4th-order Laplacian takes 17 FP64 instructions per point,
// which the GB300's FP64 rate (1.68 per clock per SM) caps far below the HBM
// bound.  This kernel evaluates a point with integer instructions only:
//
//  * A CTA owns a 32 x 16 tile of (x, y) and streams z-planes of the tile plus
//    its halo through a ring of P shared-memory slots with TMA.
//  * When plane p lands, the CTA takes the largest biased exponent E_p over
//    the plane tile (its own points and the x/y halo strips the stencil reads)
//    and rewrites the slot in place as int64 fixed point on that one scale:
//        m = sign * ((mantissa << G0) >> (E_p - e)),  value ~ m * 2^(E_p - 1075 - G0),
//    G0 = 7: |m| < 2^60, so the 3 neighbours at one offset (one per axis) add
//    in int64 without overflow.  Values within G0 binades of E_p are exact.
//  * Each thread owns a 2 x 2 block of points.  The ring keeps the 2H + 1
//    planes a point reads (z neighbours from their own slots) plus the planes
//    in flight, so one barrier per plane orders everything.
//  * A point's planes may have different scales: they are aligned to the
//    largest, E = max(E_{z-H} .. E_{z+H}), by arithmetic shifts (a CTA-wide
//    branch: most planes share E).  Group sums S_o of the neighbours at each
//    offset o are exact int64 additions; the total
//        A = bfx_c0 * m_0 + sum_o bfx_w[o] * S_o
//    is an exact signed 128-bit integer (the weights' integer images on one
//    exponent bfx_f), accumulated as four uint64 columns of unsigned 32 x
//    32-bit products (signs folded into the sums, which are biased to be
//    non-negative; operands split at bits 31 and 29, so no column overflows:
//    the host checks the bounds), and rounded once to the nearest double,
//    ties to even: the 128-bit total is normalised to 64 bits with a sticky
//    bit and converted by one correctly rounded int64 -> double conversion.
//
// Error: each group sum carries less than 4 units of truncation, so the error
// is bounded through the centre term: when the centre's magnitude is at least
// 2^bfx_tshift units, the error is below the bound the host chose bfx_tshift
// for (2 ulp of sum|c_k u_k|), plus the final rounding's 0.5 ulp.  Points whose
// centre is smaller (near a zero of u), whose planes hold Inf/NaN, or whose
// result would be subnormal or overflow, are appended to a per-CTA queue and
// evaluated, a plane later, in the reference's per-term tap order from global
// memory (L2-resident by then) by all threads of the CTA together, so the FP64
// fallback costs per point, not per warp.  If every nonzero value of a point's
// planes lies within G0 binades of their common scale, the sum is exact and no
// centre test applies.
#pragma once

namespace deo {

template <int H>
struct BfxCfg {
    static constexpr int TXT = 16, TYT = 8, NTHR = TXT * TYT;
    static constexpr int RX = 2, RY = 2;
    static constexpr int TX = TXT * RX, TY = TYT * RY;          // 32 x 16 points per tile
    static constexpr int HR = H <= 2 ? 2 : 4;                    // x halo in doubles: >= H, a 16-byte multiple
    static constexpr int BX = TX + 2 * HR, BY = TY + 2 * H;
    static constexpr int PLANE = BX * BY;
    static constexpr int PLANE_BYTES = PLANE * 8;
    static constexpr int SLOT = ((PLANE_BYTES + 127) / 128) * 128;
    static constexpr int LOOK = 1;                               // planes in flight beyond the next one
    // 128 threads, 7 slots of 5.6 KB and at most 96 registers: five CTAs per SM
    static constexpr int P = 2 * H + 2 + LOOK;                   // ring slots
    static constexpr int NHX = 2 * H * TY, NHY = 2 * H * TX;     // halo strips (no corners: a star stencil)
    static constexpr int NHALO = NHX + NHY;
    static constexpr int HPT = (NHALO + NTHR - 1) / NTHR;        // halo values per thread
    static constexpr int QCAP = 128;                             // fallback queue entries per buffer
    static constexpr int SMEM = P * SLOT;
    static constexpr int G0 = 7;
};

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Biased exponent field of the double with bits b (0 for zero and subnormals).
__device__ __forceinline__ int bfx_exp(unsigned long long b) { return (int)((b >> 52) & 0x7ffULL); }

// Fixed point of the double with bits b on the scale of biased exponent E
// (E >= every exponent of the block): sign * ((mantissa << G0) >> (E - e)).
template <int G0>
__device__ __forceinline__ long long bfx_conv(unsigned long long b, int E) {
    const int ex = bfx_exp(b);
    const unsigned long long fr = b & 0xFFFFFFFFFFFFFULL;
    const unsigned long long mant = ex ? (fr | (1ULL << 52)) : fr;
    const int d = min(E - max(ex, 1), 63);
    const long long mag = (long long)((mant << G0) >> d);
    return ((long long)b < 0) ? -mag : mag;
}

// The reference's per-term tap order for one point, from global memory
// (bit-identical to the generic evaluator).
template <int H>
__device__ __forceinline__ double bfx_reference(const UniPlan& U, const double* __restrict__ u, int64_t idx,
                                                int64_t nx, int64_t sxy) {
    const int64_t st[3] = {1, nx, sxy};
    double total = 0.0;
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < 2 * H + 1; ++k) acc = fma(U.t[t].w[k], u[idx + (k - H) * st[t]], acc);
        total = (t == 0) ? acc : total + acc;
    }
    return zero_fix(total);
}

// 128-bit product sum in four uint64 columns.  Every group sum enters with
// its weight's sign folded in and a bias of 2^62 added, S' = sgn(W) S + 2^62
// (0 <= S' < 2^63), and every weight as |W|, so that each partial product is
// one unsigned 32 x 32 -> 64-bit multiply-add: for S' = s1 2^31 + s0 (s0 in
// [0, 2^31)) and |W| = w1 2^29 + w0 (w0 in [0, 2^29)),
//     S' |W| = s0 w0 + s1 w0 2^31 + s0 w1 2^29 + s1 w1 2^60.
// The total is sum_g |W_g| S'_g = A + K with K = 2^62 sum_g |W_g| (the host
// checks that no column can overflow).
struct BfxCols {
    unsigned long long c0, c31, c29, c60;
};
__device__ __forceinline__ void bfx_mac(BfxCols& A, unsigned long long S, unsigned w0, unsigned w1) {
    const unsigned s0 = (unsigned)S & 0x7FFFFFFFu;
    const unsigned s1 = (unsigned)(S >> 31);
    A.c0 += (unsigned long long)s0 * w0;
    A.c31 += (unsigned long long)s1 * w0;
    A.c29 += (unsigned long long)s0 * w1;
    A.c60 += (unsigned long long)s1 * w1;
}

// The columns summed into one signed 128-bit integer (hi, lo), minus K.
__device__ __forceinline__ void bfx_combine(const BfxCols& A, unsigned long long k_lo, unsigned long long k_hi,
                                            long long& hi, unsigned long long& lo) {
    unsigned long long l = A.c0, h = 0ULL;
    const unsigned long long a = A.c31 << 31, b = A.c29 << 29, c = A.c60 << 60;
    const unsigned long long ah = A.c31 >> 33, bh = A.c29 >> 35, ch = A.c60 >> 4;
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(l), "+l"(h) : "l"(a), "l"(ah));
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(l), "+l"(h) : "l"(b), "l"(bh));
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(l), "+l"(h) : "l"(c), "l"(ch));
    asm("sub.cc.u64 %0, %0, %2;\n\tsubc.u64 %1, %1, %3;" : "+l"(l), "+l"(h) : "l"(k_lo), "l"(k_hi));
    hi = (long long)h;
    lo = l;
}

// (hi, lo) * 2^sc rounded to the nearest double, ties to even.  The integer
// is shifted left until bit 126 holds its leading magnitude bit (bit 127 the
// sign); the top 64 bits, with the bits below folded into a sticky bit 0, go
// through one int64 -> double conversion (round to nearest even), whose
// exponent then takes the scale.  False if the result is not a normal double.
__device__ __forceinline__ bool bfx_round(long long hi, unsigned long long lo, int sc, double& out) {
    // fast path: the top 32-bit word is more than the sign (|A| >= 2^95), so the
    // normalising shift is below 32 and two funnel shifts give the top 64 bits
    const int a3 = (int)(hi >> 32);
    const unsigned x3 = (unsigned)(a3 ^ (a3 >> 31));
    if (x3) {
        const int sh = __clz(x3) - 1;  // 0 .. 30
        const unsigned a2 = (unsigned)hi, a1 = (unsigned)(lo >> 32), a0 = (unsigned)lo;
        const unsigned t1 = __funnelshift_l(a2, (unsigned)a3, sh);
        unsigned t0 = __funnelshift_l(a1, a2, sh);
        t0 |= ((a1 << sh) | a0) ? 1u : 0u;
        const double d = __ll2double_rn((long long)(((unsigned long long)t1 << 32) | t0));
        const long long b = __double_as_longlong(d);
        const int k = 64 - sh + sc;
        const int be = (int)((b >> 52) & 0x7ff) + k;
        if (be <= 0 || be >= 2047) return false;
        out = __longlong_as_double(b + ((long long)k << 52));
        return true;
    }
    const unsigned long long s = (unsigned long long)(hi >> 63);
    const unsigned long long xh = (unsigned long long)hi ^ s, xl = lo ^ s;
    if ((xh | xl) == 0ULL && s == 0ULL) {  // zero
        out = 0.0;
        return true;
    }
    unsigned long long top, rest;
    int sh;
    if (xh) {
        sh = __clzll((long long)xh) - 1;  // 0 .. 62
        top = ((unsigned long long)hi << sh) | ((lo >> 1) >> (63 - sh));
        rest = lo << sh;
    } else {
        sh = 63 + __clzll((long long)xl);  // 63 .. 127
        top = (sh == 63) ? (((unsigned long long)hi << 63) | (lo >> 1)) : (lo << (sh - 64));
        rest = (sh == 63) ? (lo << 63) : 0ULL;
    }
    top |= rest ? 1ULL : 0ULL;
    const double d = __ll2double_rn((long long)top);
    const long long b = __double_as_longlong(d);
    const int k = 64 - sh + sc;
    const int be = (int)((b >> 52) & 0x7ff) + k;
    if (be <= 0 || be >= 2047) return false;
    out = __longlong_as_double(b + ((long long)k << 52));
    return true;
}

template <int H, bool CNEG>
__global__ void __launch_bounds__(128, 5) k_lap_bfx(const __grid_constant__ CUtensorMap tmap,
                                                    const __grid_constant__ UniPlan U, const LapGrid g,
                                                    const double* __restrict__ u, double* __restrict__ du,
                                                    int overwrite) {
    using C = BfxCfg<H>;
    constexpr int G0 = C::G0;
    constexpr int P = C::P, RY = C::RY, RX = C::RX, BX = C::BX;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[P];
    __shared__ int s_emax[P], s_emin[P];  // per slot: exponent range of the landing plane (pass 1)
    __shared__ int s_E[P], s_X[P];        // per slot: the converted plane's scale, all values exact
    __shared__ long long s_fq[3][C::QCAP];
    __shared__ int s_fqn[3];
    __shared__ int s_next;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * C::TXT + tx;
    const int nx = (int)U.n[0], ny = (int)U.n[1], nz = (int)U.n[2];
    const int64_t sxy = (int64_t)nx * ny;
    const int own0 = (H + RY * ty) * BX + C::HR + RX * tx;  // own point (row 0, column 0) inside a slot
    const unsigned int polls = U.wait_polls ? U.wait_polls : (1u << 22);
    const int withhold = U.test_withhold;  // test hook: copy never issued (0: none)
    // halo values this thread converts: x strips (H columns beside the tile), then y strips (H rows)
    int hoff[C::HPT];
#pragma unroll
    for (int h = 0; h < C::HPT; ++h) {
        const int q = tid + h * C::NTHR;
        int off = -1;
        if (q < C::NHX) {
            const int side = q / (H * C::TY), rem = q - side * (H * C::TY);
            const int row = rem / H, col = rem - row * H;
            off = (H + row) * BX + (side ? C::HR + C::TX + col : C::HR - H + col);
        } else if (q < C::NHALO) {
            const int q2 = q - C::NHX;
            const int side = q2 / (H * C::TX), rem = q2 - side * (H * C::TX);
            const int row = rem / C::TX, col = rem - row * C::TX;
            off = (side ? H + C::TY + row : row) * BX + C::HR + col;
        }
        hoff[h] = off;
    }
    // |weights| split for the column products: |W| = w1 2^29 + w0.  The signs
    // alternate from the centre's (CNEG: negative centre), as the host checked.
    unsigned wlo[2 * H + 1], whi[2 * H + 1];
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) {
        const long long W = k == H ? U.bfx_c0 : U.bfx_w[k];
        const unsigned long long aw = (unsigned long long)(W < 0 ? -W : W);
        wlo[k] = (unsigned)(aw & 0x1FFFFFFFULL);
        whi[k] = (unsigned)(aw >> 29);
    }
    // a group sum with its weight's sign folded in and the bias 2^62 (offset o from the centre)
    auto biased = [](long long v, int o) -> unsigned long long {
        const bool neg = CNEG != ((o & 1) != 0);
        return (unsigned long long)(neg ? -v : v) + (1ULL << 62);
    };
    if (tid < P) {
        s_emax[tid] = 1;
        s_emin[tid] = 4095;
    }
    if (tid == 0) {
        for (int s = 0; s < P; ++s) mbar_init(&mbar[s], 1);
        fence_mbar_init();
        s_fqn[0] = s_fqn[1] = s_fqn[2] = 0;
    }
    __syncthreads();
    auto slot_ptr = [&](int gj) -> unsigned char* { return smem + (gj % P) * C::SLOT; };
    int gbase = 0;  // running plane count of this CTA at the current unit's plane 0
    int issued = 0, waited = 0;
    bool aborted = false;
    bool first_unit = true;

    // thread 0: copy plane j of the unit (x0, y0, z0 - H + j) into its slot
    auto issue = [&](int j, int x0, int y0, int z0) {
        if (first_unit && withhold > 0 && j == withhold) return;
        const int gj = gbase + j;
        mbar_expect_tx(&mbar[gj % P], C::PLANE_BYTES);
        tma_load_3d(slot_ptr(gj), &tmap, &mbar[gj % P], x0 - C::HR, y0 - H, z0 - H + j);
    };
    auto wait_plane = [&](int j) -> bool {
        const int gj = gbase + j;
        const uint32_t par = (uint32_t)((gj / P) & 1);
        uint32_t it = 0;
        while (!mbar_try_wait(&mbar[gj % P], par))
            if (++it > polls) return false;
        return true;
    };
    // pass 1: exponent range of a landed plane over the values this thread converts
    // (zeros excluded from the minimum); warp maxima / minima into s_emax / s_emin
    auto plane_range = [&](int gj) {
        const unsigned long long* pr = reinterpret_cast<const unsigned long long*>(slot_ptr(gj));
        int emax = 1, emin = 4095;
        auto take = [&](unsigned long long b) {
            const int e = max(bfx_exp(b), 1);
            emax = max(emax, e);
            if (b << 1) emin = min(emin, e);
        };
#pragma unroll
        for (int r = 0; r < RY; ++r) {
            const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(pr + own0 + r * BX);
            take(v.x);
            take(v.y);
        }
#pragma unroll
        for (int h = 0; h < C::HPT; ++h)
            if (hoff[h] >= 0) take(pr[hoff[h]]);
        emax = (int)__reduce_max_sync(0xffffffffu, (unsigned)emax);
        emin = (int)__reduce_min_sync(0xffffffffu, (unsigned)emin);
        if (tx == 0) {
            atomicMax(&s_emax[gj % P], emax);
            atomicMin(&s_emin[gj % P], emin);
        }
    };
    auto drain_queue = [&](int b) {
        const int n = min(s_fqn[b], C::QCAP);
        for (int e = tid; e < n; e += C::NTHR) {
            const int64_t idx = s_fq[b][e];
            const double r = bfx_reference<H>(U, u, idx, nx, sxy);
            du[idx] = overwrite ? r : r + du[idx];
        }
    };

    for (int k = claim_unit(g, s_next, blockIdx.x); k < g.units && !aborted;
         k = claim_unit(g, s_next, k + gridDim.x)) {
        const int unit = (int)(((long long)k * g.perm) % g.units);
        const int txi = unit % g.tiles_x;
        const int rest = unit / g.tiles_x;
        const int tyi = rest % g.tiles_y;
        const int ci = rest / g.tiles_y;
        const int x0 = txi * C::TX, y0 = tyi * C::TY;
        const int z0 = ci * g.zc;
        const int z1 = min(z0 + g.zc, nz);
        const int npl = (z1 - z0) + 2 * H;
        const int x = x0 + RX * tx, y = y0 + RY * ty;
        // own points that are interior along x and y (bit r * 2 + c)
        unsigned live = 0;
#pragma unroll
        for (int r = 0; r < RY; ++r)
#pragma unroll
            for (int c = 0; c < RX; ++c)
                if (x + c < nx && y + r < ny && x + c + 1 >= U.t[0].flo && x + c + 1 <= U.t[0].fhi &&
                    y + r + 1 >= U.t[1].flo && y + r + 1 <= U.t[1].fhi)
                    live |= 1u << (r * RX + c);
        const bool pair_ok = !(((uintptr_t)du) & 15) && !(nx & 1);
        if (tid == 0) {
            const int pre = min(P, npl);
            for (int j = 0; j < pre; ++j) issue(j, x0, y0, z0);
            issued = pre;
        }
        waited = 0;
        {
            const bool ok = wait_plane(0);
            if (ok) {
                waited = 1;
                plane_range(gbase);
            }
            if (__syncthreads_or(!ok)) {
                aborted = true;
                break;
            }
        }
#pragma unroll 1
        for (int j = 0; j < npl; ++j) {
            const int gj = gbase + j;
            const int sj = gj % P;
            // pass 1 on plane j + 1
            bool ok = true;
            if (j + 1 < npl) {
                ok = wait_plane(j + 1);
                if (ok) {
                    waited = j + 2;
                    plane_range(gj + 1);
                }
            }
            // pass 2 on plane j: in-place conversion to its scale
            {
                const int E = s_emax[sj];
                const int En = s_emin[sj];
                long long* pm = reinterpret_cast<long long*>(slot_ptr(gj));
                const unsigned long long* pr = reinterpret_cast<const unsigned long long*>(pm);
                unsigned long long hv[C::HPT];
#pragma unroll
                for (int h = 0; h < C::HPT; ++h) hv[h] = hoff[h] >= 0 ? pr[hoff[h]] : 0ULL;
#pragma unroll
                for (int r = 0; r < RY; ++r) {
                    const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(pr + own0 + r * BX);
                    *reinterpret_cast<longlong2*>(pm + own0 + r * BX) =
                        make_longlong2(bfx_conv<G0>(v.x, E), bfx_conv<G0>(v.y, E));
                }
#pragma unroll
                for (int h = 0; h < C::HPT; ++h)
                    if (hoff[h] >= 0) pm[hoff[h]] = bfx_conv<G0>(hv[h], E);
                if (tid == 0) {
                    s_E[sj] = E;
                    s_X[sj] = (E - En <= G0) ? 1 : 0;
                }
            }
            fence_proxy_async_smem();  // these writes precede the copy that later refills the slot
            if (__syncthreads_or(!ok)) {
                aborted = true;
                break;
            }
            if (tid == 0) {
                s_emax[sj] = 1;  // ready for the pass 1 of plane j + P
                s_emin[sj] = 4095;
                // plane j - 2H - 1 has left every point's window: its slot takes plane j - 2H - 1 + P
                const int jn = j - 2 * H - 1 + P;
                if (j - 2 * H - 1 >= 0 && jn < npl) {
                    issue(jn, x0, y0, z0);
                    issued = jn + 1;
                }
            }
            // fallback points queued while evaluating plane j - 1; then clear the buffer of j - 2
            drain_queue((gj + 2) % 3);
            if (tid == 0) s_fqn[(gj + 1) % 3] = 0;
            if (j < 2 * H) continue;
            // evaluate the points of plane z = z0 + j - 2H (centre plane j - H)
            const int z = z0 + j - 2 * H;
            if (!live || z + 1 < U.t[2].flo || z + 1 > U.t[2].fhi) continue;
            int Ept = 1, Emin = 4095;
            bool exact = true;
#pragma unroll
            for (int o = 0; o <= 2 * H; ++o) {
                const int s = (gj - 2 * H + o) % P;
                Ept = max(Ept, s_E[s]);
                Emin = min(Emin, s_E[s]);
                exact = exact && s_X[s];
            }
            const bool same = Ept == Emin;
            exact = exact && same;
            int dz[2 * H + 1];
#pragma unroll
            for (int o = 0; o <= 2 * H; ++o) dz[o] = Ept - s_E[(gj - 2 * H + o) % P];
            const int bq = gj % 3;
            const long long* pz[2 * H + 1];
#pragma unroll
            for (int o = 0; o <= 2 * H; ++o) pz[o] = reinterpret_cast<const long long*>(slot_ptr(gj - 2 * H + o));
            const long long* pc = pz[H];
            // the own column pair at rows -H .. RY - 1 + H of the centre plane
            long long col[RY + 2 * H][RX];
#pragma unroll
            for (int m = 0; m < RY + 2 * H; ++m) {
                const longlong2 a = *reinterpret_cast<const longlong2*>(pc + own0 + (m - H) * BX);
                col[m][0] = a.x;
                col[m][1] = a.y;
            }
            const int64_t zrow = (int64_t)z * sxy;
#pragma unroll
            for (int r = 0; r < RY; ++r) {
                // x neighbours beside the own pair: positions -HR .. -1 and 2 .. 1 + HR
                long long xl[C::HR], xr[C::HR];
#pragma unroll
                for (int m = 0; m < C::HR; m += 2) {
                    const longlong2 a = *reinterpret_cast<const longlong2*>(pc + own0 + r * BX - C::HR + m);
                    const longlong2 b = *reinterpret_cast<const longlong2*>(pc + own0 + r * BX + 2 + m);
                    xl[m] = a.x;
                    xl[m + 1] = a.y;
                    xr[m] = b.x;
                    xr[m + 1] = b.y;
                }
                // z neighbours of the own pair in this row
                long long zm[H][RX], zp[H][RX];
#pragma unroll
                for (int o = 1; o <= H; ++o) {
                    const longlong2 a = *reinterpret_cast<const longlong2*>(pz[H - o] + own0 + r * BX);
                    const longlong2 b = *reinterpret_cast<const longlong2*>(pz[H + o] + own0 + r * BX);
                    zm[o - 1][0] = a.x;
                    zm[o - 1][1] = a.y;
                    zp[o - 1][0] = b.x;
                    zp[o - 1][1] = b.y;
                }
                double res[RX];
                bool fb[RX];
#pragma unroll
                for (int c = 0; c < RX; ++c) {
                    auto xv = [&](int o) -> long long {  // centre plane, x offset o
                        const int p = c + o;
                        return p < 0 ? xl[C::HR + p] : (p < RX ? col[H + r][p] : xr[p - RX]);
                    };
                    auto yv = [&](int o) -> long long { return col[H + r + o][c]; };
                    long long m0 = col[H + r][c];
                    long long sm[H], sp[H];
                    if (same) {
#pragma unroll
                        for (int o = 1; o <= H; ++o) {
                            sm[o - 1] = xv(-o) + yv(-o) + zm[o - 1][c];
                            sp[o - 1] = xv(o) + yv(o) + zp[o - 1][c];
                        }
                    } else {
                        m0 = sar64(m0, dz[H]);
#pragma unroll
                        for (int o = 1; o <= H; ++o) {
                            sm[o - 1] = sar64(xv(-o) + yv(-o), dz[H]) + sar64(zm[o - 1][c], dz[H - o]);
                            sp[o - 1] = sar64(xv(o) + yv(o), dz[H]) + sar64(zp[o - 1][c], dz[H + o]);
                        }
                    }
                    // the error bound needs the centre (unless every value was exact)
                    const long long big = m0 >> U.bfx_tshift;
                    bool use = Ept < 2047 && (exact || (big != 0LL && big != -1LL));
                    double tot = 0.0;
                    if (use) {
                        BfxCols A{0ULL, 0ULL, 0ULL, 0ULL};
                        bfx_mac(A, biased(m0, 0), wlo[H], whi[H]);
#pragma unroll
                        for (int o = 1; o <= H; ++o) {
                            bfx_mac(A, biased(sm[o - 1], o), wlo[H - o], whi[H - o]);
                            bfx_mac(A, biased(sp[o - 1], o), wlo[H + o], whi[H + o]);
                        }
                        long long hi;
                        unsigned long long lo;
                        bfx_combine(A, U.bfx_k_lo, U.bfx_k_hi, hi, lo);
                        // value = A * 2^(bfx_f + Ept - 1075 - G0)
                        use = bfx_round(hi, lo, U.bfx_f + Ept - 1075 - G0, tot);
                    }
                    res[c] = tot;
                    fb[c] = !use;
                }
                const int64_t row = zrow + (int64_t)(y + r) * nx + x;
                const unsigned lr = (live >> (r * RX)) & 3u;
                if (pair_ok && lr == 3u && !fb[0] && !fb[1]) {
                    double2* d2 = reinterpret_cast<double2*>(du + row);
                    if (overwrite) {
                        *d2 = make_double2(res[0], res[1]);
                    } else {
                        const double2 o2 = *d2;
                        *d2 = make_double2(res[0] + o2.x, res[1] + o2.y);
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < RX; ++c) {
                        if (!(lr & (1u << c))) continue;
                        const int64_t idx = row + c;
                        if (fb[c]) {
                            // the reference's order: queued for the whole CTA (inline if the queue is full)
                            const int slot = atomicAdd(&s_fqn[bq], 1);
                            if (slot < C::QCAP) {
                                s_fq[bq][slot] = idx;
                            } else {
                                const double rr = bfx_reference<H>(U, u, idx, nx, sxy);
                                du[idx] = overwrite ? rr : rr + du[idx];
                            }
                        } else {
                            du[idx] = overwrite ? res[c] : res[c] + du[idx];
                        }
                    }
                }
            }
        }
        // the unit's last fallback points; then every buffer is clear for the next unit
        if (__syncthreads_or(aborted)) {
            aborted = true;
            break;
        }
        drain_queue((gbase + npl - 1) % 3);
        __syncthreads();
        if (tid == 0) s_fqn[0] = s_fqn[1] = s_fqn[2] = 0;
        gbase += npl;
        first_unit = false;
    }
    if (aborted && tid == 0) {
        atomicOr(&g_deo_status, 1u);
        // wait (bounded, full limit) for this CTA's copies still in flight before its shared memory is released
        for (int j = waited; j < issued; ++j) {
            if (first_unit && withhold > 0 && j == withhold) continue;  // never issued
            const int gj = gbase + j;
            const uint32_t par = (uint32_t)((gj / P) & 1);
            for (uint32_t it = 0; it < (1u << 22); ++it)
                if (mbar_try_wait(&mbar[gj % P], par)) break;
        }
    }
}

}  // namespace deo
