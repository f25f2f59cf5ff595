// deo_internal.h -- structures shared by the host compiler (deo_host.cpp)
// and the CUDA kernels (deo_kernels.cu).
//
// Every operator term is lowered on the host to a *row table*: for output row
// i (1-based position along the differentiated axis) the reference computes
//     out[i] = sum_k  W_i[k] * x[p0_i + k],   k = 0 .. nk_i-1,
// where x is the ghost-padded line (x[1] = left ghost, x[len+2] = right ghost)
// and W_i[k] = coefficient * stencil weight, rounded exactly as the
// reference's `cur_coeff * cur_stencil[idx]`.  All of the reference's branch
// logic (boundary rows, upwind direction by coefficient sign, offside,
// the coefficient-index conventions of the padded and generic methods) is
// resolved when the table is built, so one device evaluator serves every
// operator kind.  Rows whose (p0 - i, nk, W) repeat form a "band" stored once.
#pragma once
#include <stdint.h>

#define DEO_MAX_NW 16      // widest row (max(stencil_length, boundary_stencil_length))
#define DEO_MAX_BCW 16

namespace deo {

struct RowTabDev {
    int ilo, ihi;        // band rows [ilo, ihi] (1-based, inclusive); empty if ilo > ihi
    int band_p0_off;     // p0 = i + band_p0_off
    int band_cidx_off;   // coefficient position = i + band_cidx_off
    int band_nk;
    int nexp;            // explicit rows: all rows outside the band
    int nw;              // row stride of W (max nk)
    int pad_;
    double wband[DEO_MAX_NW];
    const int* p0;       // [nexp]
    const int* nk;       // [nexp]
    const int* cidx;     // [nexp]
    const void* W;       // [nw][nexp], element type = plan dtype (k-major: coalesced along rows)
};

// Division by a runtime constant for 31-bit dividends (Granlund-Montgomery):
// q = (umulhi(n, mul) + n) >> shr.  Built on the host by make_fastdiv.
struct FastDiv {
    uint32_t mul;
    uint32_t shr;
};

// Granlund-Montgomery constants for n / d with n < 2^31: l = ceil(log2 d),
// mul = floor(2^32 (2^l - d) / d) + 1, q = (umulhi(n, mul) + n) >> l.
inline FastDiv make_fastdiv(uint32_t d) {
    uint32_t l = 0;
    while (l < 32 && (1ULL << l) < d) ++l;
    const unsigned long long m = ((1ULL << 32) * ((1ULL << l) - d)) / d + 1;
    return FastDiv{(uint32_t)m, l};
}

struct TermDev {
    int64_t stride;      // elements between neighbours along the axis
    int len;             // points along the axis
    int axis;            // 0-based
    FastDiv div_stride;  // valid when PlanDev::fastdiv
    FastDiv div_len;
    int nvar;            // 1, or 2 for an upwind operator with a coefficient field (c>=0 / c<0)
    int has_field;       // 0: none; 1: row i = sum_k (c_i w_k) u_k; 2: c_i * sum_k w_k u_k (forward)
    const void* field;   // coefficient field (same shape/dtype as u) or null
    RowTabDev tab[2];
    // adjoint: rows touching padded column p (1..len+2) lie in [rlo[p-1], rhi[p-1]]
    const int* rlo;
    const int* rhi;
    // boundary condition (ghost map)
    int bc_kind;         // 0 affine, 1 periodic, 2 padded input (ghosts stored around the line)
    int periodic_nd;     // N-D PeriodicBC pads with the edge planes (multi_dim_bc_operators.jl:221-228)
    int ml, mr;
    double al[DEO_MAX_BCW];
    double ar[DEO_MAX_BCW];
    double bl, br;
    // Boundary conditions that differ per line (MultiDimBC{dim}(BCs::Array)):
    // null, or one record of lbc_stride doubles per line, lines numbered in
    // the column-major order of the other axes:
    //   [kind (0 affine, 1 periodic: the line wraps), m_l, m_r, b_l, b_r,
    //    a_l[0 .. lbc_mw-1], a_r[0 .. lbc_mw-1]]
    const double* lbc;
    int lbc_stride;
    int lbc_mw;
};

#define DEO_KMAX_TERMS 8
#define DEO_STAR_MAX 32
// A plan built with DEO_PLAN_STAR whose terms are all constant bands: at a
// point whose row along every term's axis is in [lo, hi] of that term (band
// rows that read no ghost), the forward apply is one sum over n taps at flat
// offsets `off` with weights `w` -- every term's taps, the centre taps of the
// terms merged into one (weights of the plan's dtype, held as doubles).
struct StarDev {
    int n;
    int lo[DEO_KMAX_TERMS], hi[DEO_KMAX_TERMS];
    int64_t off[DEO_STAR_MAX];
    double w[DEO_STAR_MAX];
};

struct PlanDev {
    int ndims;
    int nterms;
    int dtype;           // 0 f64, 1 f32
    int fastdiv;         // total < 2^31: row indices by FastDiv instead of 64-bit division
    int has_lbc;         // some term has per-line boundary conditions (TermDev::lbc)
    int64_t sizes[8];
    int64_t total;
    TermDev t[DEO_KMAX_TERMS];
    StarDev star;
};

// The band rows of a plan whose terms all have constant interior rows (uniform
// grid, constant coefficient along the axis) on a 2-D/3-D array.  Laplacian-
// type plans (lap) take the TMA path: interior points, whose rows along every
// term's axis lie in [flo, fhi] (no ghosts, no boundary rows), from staged
// planes with the band weights; the rest of the points (the shell) from the
// boundary rows.  Other plans run the generic evaluator.
struct UniTerm {
    int axis;        // 0, 1, 2
    int nk;          // taps
    int off0;        // offset of tap 0 from the point along the axis
    int flo, fhi;    // rows (1-based) evaluated from the band without ghosts
    int pad_;
    double w[DEO_MAX_NW];  // band weights (float-packed for Float32 plans)
};
struct UniPlan {
    int enabled;
    int radius;      // H = max |offset| over terms
    int nterms;
    int lap;         // 1: term t acts on axis t with a centred band of 2H+1 taps (the TMA path)
    int64_t n[3];    // sizes along axes 1..3 (1 for absent axes)
    UniTerm t[DEO_KMAX_TERMS];
    // Exact-neighbour-sum evaluation (Float64, all terms share one band):
    // r = c0[mask]*u0 + sum_{o != 0} w[o] * S_o, where S_o = the exact sum of
    // the |mask| neighbours at offset o (one per axis), rounded once.
    int ens;
    int fx_rows;  // fixed-point kernel: fx_rows of each 32 x 8 tile's rows (rotating) use the FP64 order
    double ens_c0[8];             // merged centre weight for each mask of axes
    double ens_w[DEO_MAX_NW];     // band weight at offset k - H (index k)
    // Fixed-point evaluation (Float64, one shared band of nonzero normal
    // weights whose integer images fit the 128-bit accumulator): band weight
    // at offset k - H = fx_w[k] * 2^fx_f exactly.
    int fx;
    int fx_f;
    long long fx_w[DEO_MAX_NW];
    // Block fixed point (Float64, three axes, k_lap_bfx): values aligned once
    // per plane to one exponent per plane tile.  Band weight at offset k - H =
    // bfx_w[k] * 2^bfx_f exactly; bfx_c0 = 3 * bfx_w[H] (the merged centre).
    // A point whose centre has magnitude below 2^bfx_tshift units of its
    // scale (and whose planes were not all aligned exactly) is evaluated in
    // the reference's tap order instead (the error bound needs it).
    int bfx;
    int bfx_tshift;
    int bfx_f;
    int bfx_cneg;  // the centre weight is negative (the band's signs alternate from the centre)
    long long bfx_c0;
    long long bfx_w[DEO_MAX_NW];
    unsigned long long bfx_k_lo, bfx_k_hi;  // 2^62 * (|bfx_c0| + sum_{k != H} |bfx_w[k]|), a 128-bit constant
    // Bounded waits: mbarrier polls before a wait in a TMA kernel gives up
    // (0: the default 2^22), and, for the tests of that path only, the index
    // (>= 1) of the plane (box, for the shell) of each CTA's first unit whose
    // copy the kernels withhold, so that its wait runs out (0: none).
    unsigned int wait_polls;
    int test_withhold;
    // Float32: 1 the vectorised interior kernel (k_lap_v) where the output
    // allows 16-byte stores, 0 the scalar one (k_lap_q); vcfg its tile
    // variant (0..3, deo_vec.cu)
    int f32_vec;
    int vcfg;
    // boundary shell kernel: 0 automatic, 1 faces (k_face), 2 lines
    // (k_shell_lines), 3 one thread per point (k_shell_generic)
    int shell_kernel;
};

// Boundary rows of the terms of a Laplacian-type plan (the rows outside each
// term's interior range [flo, fhi]) with their weights and ghost maps; the
// plan keeps a device copy that the boundary-shell kernel stages into shared
// memory.  Weights (w, al, ar, bl, br) are the plan dtype's values: doubles,
// or for Float32 plans floats packed from the start of each double array
// (bl and br: a float in the first half of the double).
#define DEO_SHELL_ROWS 8  // per end
struct ShellRow {
    int p0, nk;
    double w[DEO_MAX_NW];
};
struct ShellTerm {
    int nlo, nhi;  // rows 1..nlo and len-nhi+1..len
    int len, bc_kind, periodic_nd, ml, mr;
    int wlo, whi;  // points of the line the low / high rows read (with the ghost): [0, wlo), [len-whi, len)
    int pad_;
    double al[DEO_MAX_BCW], ar[DEO_MAX_BCW];
    double bl, br;
    ShellRow row[2 * DEO_SHELL_ROWS];  // the nlo low rows, then the nhi high rows
};
struct ShellPlan {
    int ok;    // every term's boundary rows fit
    int maxw;  // widest boundary row or ghost map over the terms
    ShellTerm t[3];
};

// Work item of the batched persistent kernel: `count` points starting at
// flat index `start` of instance `inst`.
struct WorkItem {
    int inst;
    int count;
    int64_t start;
};

struct InstDev {
    const PlanDev* plan;   // device copy of the instance's plan
    const void* u;
    void* du;
};

// One Runge-Kutta stage of one instance:
//   out = alpha*a + beta*b + gamma*(c + dt*Op(c)),  Op = plan (or its adjoint)
// a / b may be null (their term is then absent).  Applied point-wise, out may
// alias a (each point reads a[idx] before writing out[idx]) but not c.
struct StageDev {
    const PlanDev* plan;
    const void* a;
    const void* b;
    const void* c;
    void* out;
    double alpha, beta, gamma, dt;
    int adjoint;
    int pad_;
};

// Gradient / Divergence / Curl on a padded array (vector_calculus_*.jl).
// t[a]: the row table of axis a's operator over the padded input (bc_kind 2,
// stride = the padded stride); tn[a]: the same rows with negated weights
// (the curl's `-cur_coeff * ...` terms).  quirk = 1 for the 2-D / 3-D
// methods: the axes other than the differentiated one are read at the padded
// index equal to the output index, and each output adds its terms in the order
// (BC_left, interior, BC_right) x (axis 1, 2, 3); quirk = 0 for the generic
// per-line methods (other axes at index + 1, terms in axis order).
#define DEO_VC_GRADIENT 0
#define DEO_VC_DIVERGENCE 1
#define DEO_VC_CURL 2
struct VcDev {
    int kind;
    int nd;
    int quirk;
    int bpc;             // boundary_point_count shared by the operators
    int band_nk;         // > 0: every operator's interior rows (bpc+1 .. len-bpc) are one
                         // band of band_nk taps centred on the point (uniform grid)
    int pad_;
    int64_t len[8];      // output size per axis (the operators' len)
    int64_t pstride[8];  // strides of the padded input
    int64_t pvol;        // points of one padded component
    int64_t ovol;        // points of one output component
    TermDev t[8];
    TermDev tn[3];
};

}  // namespace deo

// Launchers implemented in deo_vector.cu.  kind/nd/quirk come from V; out may
// not overlap M.  overwrite = 1 writes A*M, 0 adds it to out (mul!).
extern "C" int deo_k_vector_calculus(const deo::VcDev* V, int dtype, const void* M, void* out, int overwrite,
                                     void* stream);
// L*M on a padded array: V.t[0] is the operator's table (generic methods),
// V.len the output size, V.pstride M's strides; coff the offset of the
// stripped edge planes of M's other axes.
extern "C" int deo_k_padded_apply(const deo::VcDev* V, int axis, int64_t coff, int dtype, const void* M, void* out,
                                  int overwrite, void* stream);
// op 0: u = dot(A, B) over ncomp components; 1: u = cross(A, B) (ncomp 3);
// 2: u = sqrt(dot(A, A)).  npts points per component, component-major.
extern "C" int deo_k_vector_algebra(int op, int dtype, int64_t npts, int ncomp, const void* A, const void* B, void* u,
                                    void* stream);

// Launcher implemented in deo_solve.cu: every line along an axis (stride, n
// points) of u solved with the banded LU factors ab ([kl+ku+kl+1][n]), pivots
// ipiv, reciprocal pivots rdiag and offset Ab: x = A_l^-1 (u - A_b).  x may be
// u.  work: null for Float64 (x is the workspace), else total doubles.
extern "C" int deo_k_band_solve(int n, int kl, int ku, const double* ab, const int* ipiv, const double* Ab,
                                const double* rdiag, int64_t stride, int64_t nlines, int dtype, const void* u, void* x,
                                double* work, void* stream);

// Launchers implemented in deo_kernels.cu (return cudaError_t as int).
extern "C" int deo_k_apply(const deo::PlanDev* p, const void* u, void* du, int overwrite, int adjoint,
                           void* stream);
// x *= f over n points (dtype 0 f64, 1 f32), stream-ordered.
extern "C" int deo_k_scale(void* x, int64_t n, int dtype, double f, void* stream);
// Commits k_batch's module image and launch resources on the current device
// (one empty launch of each instantiation; *counter is bumped, nothing else).
extern "C" int deo_k_batch_prepare(unsigned int* counter, void* stream);
// lbc: some instance's plan has per-line boundary conditions (the kernel
// instantiation with that branch)
extern "C" int deo_k_batch(const deo::InstDev* inst, const deo::WorkItem* items, int64_t n_items,
                           unsigned int* counter, int dtype, int adjoint, int lbc, int ctas_per_sm, int threads,
                           void* stream);
extern "C" int deo_k_num_sms(void);
// nonlinear_diffusion! on padded vectors p, q (length len+2): term k-1 of the
// plan (host copy, passed by value) is CenteredDifference of order k.
extern "C" int deo_k_nonlinear_diffusion(const deo::PlanDev* plan, int len, int n, int m, int dtype, const void* p,
                                         const void* q, void* du, void* stream);
// TMA-fed fast path (deo_tma.cu): the interior box of a Laplacian-type plan;
// returns cudaErrorNotSupported when the array does not meet the tensor-map
// alignment rules (caller falls back).  use_ens: 0 the reference's tap order,
// 1 the best exact-sum kernel that applies, 2 exact sums v1, 3 exact sums v2.
// *kernel receives the name of the kernel launched.  sched: null, or a device
// counter the persistent CTAs claim their units from (zeroed here on the
// stream before the launch), so that they balance around other work sharing
// the SMs (the concurrent shell).
extern "C" int deo_k_apply_tma(const deo::UniPlan* up, const deo::PlanDev* d_plan, int dtype, const void* u,
                               void* du, int overwrite, int use_ens, void* stream, const char** kernel,
                               unsigned int* sched);
// The boundary shell around that interior box (boundary rows in the reference's
// order); sp / sp_dev are the host and device copies of the plan's ShellPlan,
// or null to evaluate the boundary rows from the row tables.  mode: run alone
// after the interior kernel (the faster kernel for the dtype) or concurrently
// with it on another stream (a small grid that fits beside it).  *kernel
// receives the name of the kernel that runs (it may fall back to another).
#define DEO_SHELL_ALONE 0
#define DEO_SHELL_CONCURRENT 1
extern "C" int deo_k_apply_shell(const deo::UniPlan* up, const deo::ShellPlan* sp, const deo::ShellPlan* sp_dev,
                                 int mode, const deo::PlanDev* d_plan, int dtype, const void* u, void* du,
                                 int overwrite, void* stream, const char** kernel);
extern "C" int deo_k_read_status(unsigned int* status);
// Encodes a CUtensorMap (written to map, 128 bytes) of a 3-D array nx x ny x nz
// of es-byte elements for box loads of bx x by x bz; cudaErrorNotSupported if
// the tensor-map alignment rules are not met.
extern "C" int deo_k_encode_map3(void* map, const void* u, int es, int64_t nx, int64_t ny, int64_t nz, int bx, int by,
                                 int bz);
extern "C" int deo_k_read_shell_status(unsigned int* status);
// The transposed operator outside the box of up's [flo, fhi] (the generic
// column evaluator, one thread per point); concurrent: one CTA per SM
extern "C" int deo_k_apply_shell_adj(const deo::UniPlan* up, const deo::PlanDev* dp, int dtype, const void* d,
                                     void* ub, int overwrite, int concurrent, void* stream);
// Float32 vectorised interior (deo_vec.cu): cudaErrorNotSupported when the
// plan or the buffers do not fit it (the caller then runs k_lap_q)
extern "C" int deo_k_apply_vec(const deo::UniPlan* up, unsigned int* sched, const void* u, void* du, int ow,
                               void* stream);
extern "C" int deo_k_read_vec_status(unsigned int* status);
// Device concretisation from the plan's tables (deo_concretize.cu): mode 0
// dense, 1 banded (l, u; *flag set for an entry outside), 2 bandwidths into lu
extern "C" int deo_k_concretize(const deo::PlanDev* p, int mode, double* A, double* Ab, int64_t l, int64_t u,
                                unsigned long long* lu, int* flag, void* stream);
// 1 if deo_k_apply_tma can run on u (tensor-map alignment rules).
extern "C" int deo_k_tma_ok(const deo::UniPlan* up, int dtype, const void* u);
extern "C" int deo_k_stage_batch(const deo::StageDev* st, const deo::WorkItem* items, int64_t n_items,
                                 unsigned int* counter, int lbc, int dtype, int ctas_per_sm, int threads,
                                 void* stream);
