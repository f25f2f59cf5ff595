// deo_concretize.cu -- the affine map du = A_l u + A_b of a plan, built on
// the device from the plan's own row tables (concretization.jl:914-958:
// Array(L*Q) = (Array(L) * Q_l, Array(L) * Q_b), summed over the terms of a
// combination; BandedMatrix(L*Q) likewise).
//
// One thread per output point i.  For each term, the row of point i along
// the term's axis (band or explicit row, the coefficient field's value and
// upwind variant as the apply reads them) contributes weight w_k at padded
// position p = p0 + k: to column base + (p - 2) stride for p inside the line;
// for a ghost position, w_k times the boundary condition's map: a_j to
// column base + j stride (left; the last m_r points for the right) and w_k b
// to A_b, or the periodic end point.  Contributions to one entry are added in
// the terms' order and, within a term, in increasing p: the order of the
// matrix product L * Q_l.  Each thread writes only its own row, so there are
// no races.  Entries are computed in Float64 from the plan's weights (Float32
// plans: their float weights, widened).
#include <cuda_runtime.h>
#include <stdint.h>

#include "deo_eval.cuh"

namespace deo {

// MODE 0: dense A_l (n x n, column-major, zeroed by the caller);
// MODE 1: band storage (l + u + 1) x n, column-major, entry (i, j) at row
//         u + i - j of column j (BandedMatrices' layout, zeroed by the caller);
//         an entry outside the band sets *flag;
// MODE 2: the bandwidths: atomicMax of i - j into lu[0], of j - i into lu[1].
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_concretize(const __grid_constant__ PlanDev P, double* __restrict__ A,
                                                    double* __restrict__ Ab, int64_t l, int64_t u,
                                                    unsigned long long* __restrict__ lu, int* __restrict__ flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.total) return;
    const int64_t n = P.total;
    long long lo_off = 0, hi_off = 0;  // MODE 2: i - j and j - i maxima
    auto put = [&](int64_t j, double v) {
        if constexpr (MODE == 0) {
            A[j * n + i] += v;
        } else if constexpr (MODE == 1) {
            const int64_t r = u + i - j;
            if (r < 0 || r > l + u) {
                atomicOr(flag, 1);
                return;
            }
            A[j * (l + u + 1) + r] += v;
        } else {
            lo_off = max(lo_off, (long long)(i - j));
            hi_off = max(hi_off, (long long)(j - i));
        }
    };
    double b_acc = 0.0;
    for (int tt = 0; tt < P.nterms; ++tt) {
        const TermDev& t = P.t[tt];
        const int64_t s = t.stride;
        const int r1 = term_row(P, t, i);
        const int64_t base = i - (int64_t)(r1 - 1) * s;
        T c;
        const RowTabDev& tb = row_variant<T>(t, base, r1, c);
        const RowInfo ri = row_info(tb, r1);
        const int L2 = t.len + 2;
        // this line's boundary condition
        int kind = t.bc_kind, ml = t.ml, mr = t.mr;
        const double *al = t.al, *ar = t.ar;
        double bl = t.bl, br = t.br;
        bool pnd = t.periodic_nd != 0;
        if (t.lbc) {
            const double* q = line_bc(t, base);
            kind = q[0] != 0.0 ? 1 : 0;
            pnd = false;  // a periodic BC among per-line BCs wraps around its line
            ml = (int)q[1];
            mr = (int)q[2];
            bl = q[3];
            br = q[4];
            al = q + 5;
            ar = q + 5 + t.lbc_mw;
        }
        for (int k = 0; k < ri.nk; ++k) {
            const double w = (double)(t.has_field ? c * row_w<T>(tb, ri, k) : row_w<T>(tb, ri, k));
            const int p = ri.p0 + k;
            if (p == 1 || p == L2) {
                const bool left = p == 1;
                if (kind == 1) {  // the periodic end point (edge plane for N-D PeriodicBC)
                    put(base + (int64_t)((left != pnd) ? t.len - 1 : 0) * s, w);
                } else {
                    const int m = left ? ml : mr;
                    const double* a = left ? al : ar;
                    const int64_t o = left ? 0 : t.len - mr;
                    for (int j = 0; j < m; ++j) put(base + (o + j) * s, w * a[j]);
                    b_acc += w * (left ? bl : br);
                }
            } else {
                put(base + (int64_t)(p - 2) * s, w);
            }
        }
    }
    if constexpr (MODE == 2) {
        atomicMax(&lu[0], (unsigned long long)lo_off);
        atomicMax(&lu[1], (unsigned long long)hi_off);
    } else {
        if (Ab) Ab[i] = b_acc;
    }
}

}  // namespace deo

using namespace deo;

// mode 0 dense, 1 banded, 2 bandwidths (see k_concretize); the plan must not
// read ghosts stored around its lines (padded-input plans).
extern "C" int deo_k_concretize(const PlanDev* p, int mode, double* A, double* Ab, int64_t l, int64_t u,
                                unsigned long long* lu, int* flag, void* stream) {
    for (int t = 0; t < p->nterms; ++t)
        if (p->t[t].bc_kind == 2) return (int)cudaErrorNotSupported;
    const int64_t blocks = (p->total + 255) / 256;
    if (blocks == 0) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto go = [&](auto kernel) { kernel<<<(unsigned)blocks, 256, 0, st>>>(*p, A, Ab, l, u, lu, flag); };
    if (p->dtype == 0) {
        if (mode == 0) go(k_concretize<double, 0>);
        else if (mode == 1) go(k_concretize<double, 1>);
        else go(k_concretize<double, 2>);
    } else {
        if (mode == 0) go(k_concretize<float, 0>);
        else if (mode == 1) go(k_concretize<float, 1>);
        else go(k_concretize<float, 2>);
    }
    return (int)cudaGetLastError();
}
