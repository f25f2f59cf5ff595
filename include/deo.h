/*
 * deo.h -- C ABI of libdeo, a GB300 (sm_103a) implementation of the
 * stencil-apply path of DiffEqOperators.jl (`L*Q*u`, `mul!`).
 *
 * Conventions
 *   - Arrays are column-major with axis 1 contiguous, exactly as Julia lays
 *     out an Array/CuArray.  `sizes[k]` is Julia's `size(u, k+1)`.
 *   - Device buffers are plain device pointers (CuArray's pointer, a torch
 *     tensor's data_ptr).  Streams are passed as `void*` (a cudaStream_t;
 *     NULL = legacy default stream).
 *   - Every entry point returns a deo_status; no exception or device trap
 *     crosses the ABI.  deo_last_error() gives a per-thread message.
 *   - Operators (deo_operator) and boundary conditions (deo_bc) are host
 *     objects built either by the constructors below (which restate the
 *     reference's constructors) or from the tables a Julia DerivativeOperator
 *     already holds (deo_operator_from_tables).
 *   - A plan binds terms (operator, axis, boundary condition) to an array
 *     shape and dtype, uploads its tables once, and is immutable afterwards:
 *     it may be shared by host threads and used on any stream.  deo_apply
 *     allocates nothing and does not synchronise.
 */
#ifndef DEO_H
#define DEO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DEO_ABI_VERSION 2
#define DEO_MAX_BC 16      /* longest ghost stencil a_l / a_r */
#define DEO_MAX_TERMS 8    /* terms in one plan */
#define DEO_MAX_DIMS 8

typedef enum {
    DEO_OK = 0,
    DEO_ERR_BAD_SHAPE = 1,   /* reference: AssertionError / DimensionMismatch */
    DEO_ERR_BAD_ARG = 2,     /* reference: AssertionError / ArgumentError */
    DEO_ERR_UNSUPPORTED = 3,
    DEO_ERR_CUDA = 4,
    DEO_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
    DEO_ERR_OOM = 6,
    DEO_ERR_NOT_READY = 7,   /* serving: result not finished yet */
    DEO_ERR_REJECTED = 8     /* serving: admission refused */
} deo_status;

typedef enum { DEO_F64 = 0, DEO_F32 = 1 } deo_dtype;

typedef struct deo_operator deo_operator;
typedef struct deo_plan deo_plan;

/* Per-thread message of the last failing call ("" if none). */
const char* deo_last_error(void);
int deo_abi_version(void);

/* ------------------------------------------------------------------------
 * Finite-difference weights.
 * Replaces calculate_weights(order, x0, x), src/derivative_operators/fornberg.jl:7-62
 * (Fornberg's recurrence with the centre row-sum correction).
 * ---------------------------------------------------------------------- */
deo_status deo_calculate_weights(int order, double x0, const double* x, int n, double* out);

/* ------------------------------------------------------------------------
 * Operators.  dx has ndx = 1 entry (uniform grid) or at least len+1 entries
 * (non-uniform: the reference's upwind operators read dx[1:len+1], its
 * centred ones dx[1:len+1] and the last d+a entries for the high boundary
 * rows, so centred operators also need ndx >= d+a).  Grids too short for
 * the stencil give DEO_ERR_BAD_SHAPE where the reference throws BoundsError.
 * ---------------------------------------------------------------------- */
/* CenteredDifference{N}(d, a, dx, len), derivative_operator.jl:81-135 (uniform), :150-205 (non-uniform) */
deo_status deo_centered_difference(int derivative_order, int approximation_order, const double* dx,
                                   int ndx, int len, deo_operator** out);
/* UpwindDifference{N}(d, a, dx, len; offside), derivative_operator.jl:454-512 (uniform), :515-639 (non-uniform) */
deo_status deo_upwind_difference(int derivative_order, int approximation_order, const double* dx, int ndx,
                                 int len, int offside, deo_operator** out);

/* The fields of a DerivativeOperator (derivative_operator.jl:14-29), flattened.
 * Tables are row-major [halves][rows][width]; halves = 2 only for a
 * non-uniform UpwindDifference (row 1 upwind, row 2 downwind, as its
 * SMatrix stencils are stored), else 1. */
typedef struct {
    int derivative_order;
    int approximation_order;
    int len;
    int stencil_length;
    int boundary_stencil_length;
    int boundary_point_count;
    int offside;
    int winding;          /* 0 CenteredDifference, 1 UpwindDifference */
    int uniform;          /* 1: dx::Number (one stencil row), 0: dx::Vector */
    int coeff_func_sign;  /* +1 coeff_func is a Number >= 0, -1 a Number < 0, 0 otherwise */
    int n_stencil_rows;   /* rows per half */
    int n_low_rows;
    int n_high_rows;
    const double* stencil_coefs;
    const double* low_boundary_coefs;
    const double* high_boundary_coefs;
    const double* coefficients; /* [len] */
} deo_operator_desc;

/* Build an operator from a DerivativeOperator's own tables (the Julia shim
 * passes L.stencil_coefs etc.); the tables are copied. */
deo_status deo_operator_from_tables(const deo_operator_desc* desc, deo_operator** out);
/* Pointers in *desc stay valid until the operator is modified or destroyed. */
deo_status deo_operator_describe(const deo_operator* op, deo_operator_desc* desc);
/* coefficients = 0 .+ c  (compute_coeffs!, coefficient_functions.jl:7-15); n = 1 or len */
deo_status deo_operator_set_coefficients(deo_operator* op, const double* c, int n, int coeff_func_sign);
/* coefficients = c .* coefficients  (c*L, derivative_operator_functions.jl:165-197); n = 1 or len */
deo_status deo_operator_scale_coefficients(deo_operator* op, const double* c, int n);
deo_status deo_operator_clone(const deo_operator* op, deo_operator** out);
void deo_operator_destroy(deo_operator* op);
/* Array(L) (concretization.jl:8-52 centred, :556-671 upwind): len x (len+2), column-major. */
deo_status deo_operator_array(const deo_operator* op, double* out);
/* BandedMatrix(L) (concretization.jl:123-128 centred, :794-890 upwind): *l, *u receive the
 * reference's bandwidths ((bstl-3, bstl-1) centred, (stl-2, stl) upwind); data (may be null)
 * receives the (l+u+1) x (len+2) band storage, column-major, with entry (i, j) of Array(L)
 * (1-based) at row u+i-j of column j -- BandedMatrices.jl's `bandeddata` layout.
 * DEO_ERR_BAD_SHAPE if a nonzero of Array(L) lies outside those bands. */
deo_status deo_operator_banded(const deo_operator* op, int* l, int* u, double* data);

/* ------------------------------------------------------------------------
 * Boundary conditions: the affine ghost map of an AffineBC
 * (ghost_l = a_l . u[1:m_l] + b_l, ghost_r = a_r . u[end-m_r+1:end] + b_r),
 * or PeriodicBC.  bc_operators.jl:1-196.
 * ---------------------------------------------------------------------- */
#define DEO_BC_AFFINE 0
#define DEO_BC_PERIODIC 1
typedef struct {
    int kind;
    int m_l, m_r;
    double a_l[DEO_MAX_BC];
    double a_r[DEO_MAX_BC];
    double b_l, b_r;
} deo_bc;

/* RobinBC(l, r, dx, order), bc_operators.jl:26-60.  l = (α, β, γ). */
deo_status deo_robin_bc(const double* l, const double* r, const double* dx, int ndx, int order, deo_bc* out);
/* GeneralBC(αl, αr, dx, order), bc_operators.jl:90-169. */
deo_status deo_general_bc(const double* alpha_l, int nl, const double* alpha_r, int nr, const double* dx,
                          int ndx, int order, deo_bc* out);
/* DirichletBC(l, r) = RobinBC((1,0,l),(1,0,r),1,2), bc_operators.jl:175-177; Dirichlet0BC: l = r = 0. */
deo_status deo_dirichlet_bc(double l, double r, deo_bc* out);
/* NeumannBC((l, r), dx, order) = RobinBC((0,1,l),(0,1,r),dx,order), bc_operators.jl:173-174. */
deo_status deo_neumann_bc(double l, double r, const double* dx, int ndx, int order, deo_bc* out);
/* PeriodicBC(T), bc_operators.jl:17-19. */
deo_status deo_periodic_bc(deo_bc* out);
/* Array(Q, N) -> (Q_L (N+2) x N column-major, Q_b[N+2]), concretization.jl:187-192, :227-230. */
deo_status deo_bc_array(const deo_bc* bc, int n, double* QL, double* Qb);

/* ------------------------------------------------------------------------
 * Plans: sum_t (L_t * Q_t) * u over an N-D array.
 *   ndims == 1 follows the reference's BoundaryPaddedVector methods
 *   (convolutions.jl:367-730, reached by `L*Q*u` on a Vector); ndims > 1
 *   follows the per-line generic methods reached through MultiDimBC padding
 *   (derivative_operator_functions.jl:27-69, convolutions.jl:27-362,
 *   multi_dim_bc_operators.jl:212-252).  Terms are summed left to right as
 *   `sum(op -> op*u, ops)` does (composite_operators.jl:64-65).
 *   coeff_field (device pointer, same shape and dtype as u, or NULL) makes
 *   term t act on every line with coefficients = the field along that line:
 *   the reference's one-operator-per-line construction of a field coefficient.
 * ---------------------------------------------------------------------- */
#define DEO_PATH_AUTO 0      /* padded-vector methods if ndims == 1, else generic */
#define DEO_PATH_PADDED 1    /* BoundaryPaddedVector methods (convolutions.jl:367-730) */
#define DEO_PATH_GENERIC 2   /* AbstractVector methods (convolutions.jl:27-362), e.g. `L*x` on a padded Vector */
typedef struct {
    const deo_operator* op;
    int axis;                 /* 1-based, Julia's N in CenteredDifference{N} */
    const deo_bc* bc;         /* applied along `axis` to every line (ignored when line_bcs is set) */
    const void* coeff_field;  /* device pointer or NULL */
    int path;                 /* DEO_PATH_* */
    /* NULL, or one BC per line along `axis` (host array of prod(sizes)/sizes[axis]
     * entries, column-major over the other axes): MultiDimBC{dim}(BCs::Array),
     * multi_dim_bc_operators.jl:91-93, whose lines get BCs[I, J] * u[I, :, J]
     * (:28-52).  A periodic BC among others wraps around its line; an array
     * of periodic BCs only pads with the edge planes, as PeriodicBC does. */
    const deo_bc* line_bcs;
} deo_term;

deo_status deo_plan_create(int ndims, const int64_t* sizes, deo_dtype dtype, int nterms, const deo_term* terms,
                           deo_plan** out);
/* deo_plan_create with flags:
 *   DEO_PLAN_MERGE_TERMS: terms on one axis with the same boundary condition
 *     and path, without coefficient fields or per-line BCs, are evaluated as
 *     one term whose row i has the union of their windows and, at each padded
 *     position, the sum of their weights (added in the terms' order, rounded
 *     once; row widths up to 16).  Each merged row then takes one tap per
 *     position instead of one per term and position, and the result differs
 *     from the reference's term-by-term sums by rounding only: within the
 *     same 4 ulp of sum |c_k u_k| (the weights' rounding adds at most half an
 *     ulp of each merged weight times its value).  No reference counterpart. */
#define DEO_PLAN_MERGE_TERMS 1
/*   DEO_PLAN_STAR: when every term is a constant band (no coefficient field,
 *     no per-line BCs), points whose rows read no ghost along any axis are
 *     evaluated as one sum over all the terms' taps, the terms' centre
 *     weights added into one (in Float64, rounded once): one FP64 (Float32)
 *     instruction per tap instead of per tap and per term sum, for the
 *     generic, batched and Runge-Kutta stage kernels (Laplacian-type plans on
 *     the TMA path keep their interior kernels).  Rounding differs from the
 *     reference's term-by-term sums, within the same bar. */
#define DEO_PLAN_STAR 2
/*   DEO_PLAN_FACTOR_FIELD: a term with a coefficient field c(x) evaluates
 *     row i as c_i * (sum_k w_k u_k) -- the taps summed first, one multiply
 *     by the field value after -- instead of the reference's
 *     sum_k (c_i w_k) u_k (convolutions.jl:47, :140): one FP64 (Float32)
 *     multiply per point instead of one per tap.  Forward applies of the
 *     generic, batched and Runge-Kutta stage kernels; the adjoint and the
 *     concretisation keep c_i w_k.  Rounding differs from the reference's
 *     order, within the same 4 ulp of sum |c_k u_k|. */
#define DEO_PLAN_FACTOR_FIELD 4
deo_status deo_plan_create_opts(int ndims, const int64_t* sizes, deo_dtype dtype, int nterms, const deo_term* terms,
                                int flags, deo_plan** out);
/* Frees the plan's device tables, streams and events (cudaFree waits for the device). */
void deo_plan_destroy(deo_plan* plan);
/* Device bytes held by the plan's tables. */
size_t deo_plan_table_bytes(const deo_plan* plan);
/* Terms the plan evaluates per point (fewer than it was given when
 * DEO_PLAN_MERGE_TERMS joined some); -1 for a null plan. */
int deo_plan_terms(const deo_plan* plan);
/* Taps of the plan's merged star (DEO_PLAN_STAR; 0 when it has none); -1 for a null plan. */
int deo_plan_star_taps(const deo_plan* plan);
/* Plan options (defaults 1 unless stated):
 *   DEO_OPT_FAST_PATH: Laplacian-type 2-D/3-D plans (term t a centred band on
 *     axis t) use the tiled TMA kernels below for interior points; 0 forces
 *     the generic row-table kernel (which every other plan runs).
 *   DEO_OPT_TMA: those plans stream planes with TMA into a shared-memory ring;
 *     0 uses the generic kernel as well.
 *   DEO_OPT_EXACT_SUMS: Float64 Laplacian-type plans whose terms share one
 *     band evaluate interior points in integer arithmetic and round once
 *     (result within a few ulp of sum|c_k u_k| of the reference's order):
 *       1 the best variant that applies (default): the per-point
 *         fixed-point kernel (variant 4) when the band's weights allow it,
 *         else variant 3;
 *       5 for three axes the block fixed-point kernel (values aligned once
 *         per plane to one exponent per plane tile, no FP64 instruction per
 *         point; points near a zero of u, where that alignment cannot bound
 *         the error, in the reference's order; as fast as variant 4 at 256^3,
 *         kept for comparison), else as 1;
 *       2 exact sums of the equal-weight neighbours, decomposing values at
 *         every use (kept for comparison);
 *       3 the same sums from values decomposed once per plane, one int64 ->
 *         double conversion and one FMA per offset;
 *       4 the per-point fixed-point kernel when the band's weights allow it,
 *         else variant 3;
 *       0 the reference's per-term tap order, bit-identical to the generic
 *         kernel.
 *   DEO_OPT_LAUNCH_TIMING: 1 records CUDA events around every kernel launch
 *     of each forward apply (read with deo_plan_launch_times); default 0.
 *   DEO_OPT_CONCURRENT_SHELL: 1 evaluates the boundary shell of a
 *     Laplacian-type plan on the TMA path on a plan-owned side stream at the
 *     same time as the interior (forked from and joined back into the
 *     caller's stream, so the apply stays stream-ordered; the shell's CTAs
 *     are sized to fit beside the interior kernel's).  It applies to Float32
 *     plans and to the fixed-point Float64 interior (whose FP64 pipe is free
 *     for the shell); other Float64 interiors are FP64-bound and run the
 *     shell after them.  0 runs the shell after the interior always.
 *   DEO_OPT_FX_FP64_ROWS: 0..8 (default 2): in the fixed-point Float64
 *     interior kernel, the points with ((y mod 8) - value * (floor(y/8) + z))
 *     mod 8 < value (y, z the 0-based indices along axes 2 and 3, z = 0 in
 *     2-D: `value` of every 8 rows of a 32 x 8 tile, rotating from plane to
 *     plane; whole warps) are evaluated in the reference's per-term tap order
 *     on the FP64 pipe, bit-identical to the generic kernel, while the others
 *     use the integer pipes; 0 evaluates every interior point in fixed point.
 *     deo_plan_get_option returns the value when the fixed-point kernel
 *     applies, else 0.
 *   DEO_OPT_TEST_WITHHOLD: 0 (default) or k in 1..64, for tests of the
 *     bounded waits only: the TMA kernels (interior and shell) withhold the
 *     copy of plane k of each CTA's first unit (the shell: each CTA's first
 *     box) and give up on a wait after 64 polls instead of 2^22, so the wait
 *     for that copy runs out: the kernel sets its device status bit, waits for
 *     its other copies in flight and returns, leaving its points unwritten.
 *     deo_device_status then reports DEO_ERR_TIMEOUT.  Nothing faults.
 *   DEO_OPT_F32_VECTOR: Float32 Laplacian-type plans on the TMA path with
 *     band radius <= 3: 1 (default) evaluates the interior with each thread
 *     on 4 consecutive x points (16-byte shared-memory loads and stores, when
 *     du is 16-byte aligned), 0 one point per thread; the two are
 *     bit-identical to each other and to the generic kernel.
 *   DEO_OPT_F32_TILE: 0..3, the vectorised kernel's tile (threads along y x
 *     rows per thread): 0 (default) 16 x 2, 1 8 x 2, 2 16 x 1, 3 8 x 4 (band
 *     radius <= 2; else as 0); two-axis plans use 0.
 *   DEO_OPT_SHELL_KERNEL: the boundary-shell kernel of those plans: 0
 *     (default) automatic, 1 face tiles staged by TMA, 2 one thread per
 *     (line, end), 3 one thread per point; all in the reference's order
 *     (bit-identical to the generic kernel).
 * No reference counterpart (execution choices only). */
#define DEO_OPT_FAST_PATH 1
#define DEO_OPT_TMA 2
#define DEO_OPT_EXACT_SUMS 3
#define DEO_OPT_LAUNCH_TIMING 4
#define DEO_OPT_CONCURRENT_SHELL 5
#define DEO_OPT_FX_FP64_ROWS 6
#define DEO_OPT_TEST_WITHHOLD 7
#define DEO_OPT_F32_VECTOR 8
#define DEO_OPT_SHELL_KERNEL 9
#define DEO_OPT_F32_TILE 10
deo_status deo_plan_set_option(deo_plan* plan, int option, int value);
/* 1 if the option is set AND applies to this plan, 0 if not, -1 on error. */
int deo_plan_get_option(const deo_plan* plan, int option);
/* Name of the kernel the last forward apply launched first (which = 0) and
 * second (which = 1; "" if it launched one), e.g. "k_lap_fx" and "k_face".
 * Static strings; "" before the first apply.  No reference counterpart. */
const char* deo_plan_kernels(const deo_plan* plan, int which);
/* Device time in ms of each launch of the last forward apply (DEO_OPT_LAUNCH_TIMING
 * must be on); ms needs room for 2 entries, *n receives the count.  With a
 * concurrent shell, ms[0] is the interior kernel and ms[1] the time the apply
 * then still waits for the shell.  Waits for that apply to finish.  No
 * reference counterpart. */
deo_status deo_plan_launch_times(const deo_plan* plan, float* ms, int* n);
/* Device-side error flags raised since the last call (bit 0: a bounded wait
 * in a kernel gave up; the kernel returned without finishing).  Synchronises.
 * Returns DEO_ERR_TIMEOUT if any flag was set. */
deo_status deo_device_status(unsigned int* status);

/* mul!(du, A*Q, u): du = sum_t L_t Q_t u  (overwrite = 1), or du += ... (overwrite = 0,
 * the reference's `mul!(x, L, M; overwrite=false)`, convolutions.jl:17-22).
 * Replaces LinearAlgebra.mul!(out, A::GhostDerivativeOperator, u)
 * (ghost_derivative_operator.jl:15-24) and `(A*Q)*u` (ghost_derivative_operator.jl:26-37,
 * composite_operators.jl:64-65).  u and du must not overlap.  A plan may be applied
 * from several host threads and streams at once (up to 1024 applies of one plan in
 * flight at the same time). */
deo_status deo_apply(const deo_plan* plan, const void* u, void* du, int overwrite, void* stream);

/* Same, reading u from host memory and writing du to host memory (copies
 * through the plan's staging buffers on `stream`; synchronises before return). */
deo_status deo_apply_host(deo_plan* plan, const void* u_host, void* du_host, void* stream);
/* The same for a sequence of host arrays, pipelined and not synchronising: the
 * copy of call i+1's input, call i's apply and the copy of call i-1's result
 * overlap (two plan-owned staging slots, plan-owned copy streams; the apply
 * itself runs on `stream`).  u_host and du_host (pinned memory for overlap)
 * must stay valid, and du_host unread, until deo_plan_host_sync returns.
 * No reference counterpart (the reference applies to host arrays only). */
deo_status deo_apply_host_async(deo_plan* plan, const void* u_host, void* du_host, void* stream);
/* Waits for every deo_apply_host_async of the plan issued so far. */
deo_status deo_plan_host_sync(deo_plan* plan);

/* Adjoint of the linear part: ubar = A_l^T dbar, where (A_l, A_b) = Array(L*Q)
 * (concretization.jl:914-918) of the map deo_apply computes.  No reference
 * counterpart (the reference's adjoint(L) returns L, abstract_operator_functions.jl:130-135). */
deo_status deo_apply_adjoint(const deo_plan* plan, const void* dbar, void* ubar, int overwrite, void* stream);

/* nonlinear_diffusion!{N}(du, n, m, approx_order, p, q, dx, nknots)
 * (derivative_operator.jl:34-66):
 *   du = (D_m q) .* (D_n p)   (q[2:nknots+1] .* (D_n p) when m == 0)
 *      + sum_{l=1}^{n-1} binomial(n, l) * (D_{l+m} q) .* (D_{n-l} p)
 *      + (D_{m+n} q) .* p[2:nknots+1]
 * with D_k = CenteredDifference(k, approx_order, dx, nknots) applied to the
 * padded vectors p, q (nknots + 2 entries, ghosts first and last) by the
 * generic method, in the reference's operation order.  Planned once
 * (operators and tables), applied on device vectors p, q -> du (nknots). */
typedef struct deo_nld deo_nld;
deo_status deo_nonlinear_diffusion_plan(int second_order, int first_order, int approx_order, const double* dx,
                                        int dx_len, int nknots, deo_dtype dtype, deo_nld** out);
deo_status deo_nonlinear_diffusion(const deo_nld* plan, const void* p, const void* q, void* du, void* stream);
void deo_nonlinear_diffusion_destroy(deo_nld* plan);

/* ------------------------------------------------------------------------
 * A DerivativeOperator on an already padded array (no boundary condition):
 * x_temp = L*M or mul!(x_temp, L, M; overwrite) with L acting along `axis`
 * (derivative_operator_functions.jl:17-69, 150-163; convolutions.jl:17-22 for
 * vectors), every line by the generic AbstractVector methods.  M's size along
 * `axis` is len+2 (the ghosts are its first and last entries); along every
 * other axis it equals x_temp's or is 2 longer, in which case its first and
 * last planes are skipped (:47-56).  overwrite = 0 adds into x_temp.  The plan
 * holds the row table for (operator, sizes, dtype); x_temp must not overlap M.
 * ---------------------------------------------------------------------- */
typedef struct deo_padded deo_padded;
deo_status deo_padded_plan(const deo_operator* op, int axis, int ndims, const int64_t* out_sizes,
                           const int64_t* in_sizes, deo_dtype dtype, deo_padded** out);
deo_status deo_padded_apply(const deo_padded* plan, const void* M, void* x_temp, int overwrite, void* stream);
void deo_padded_destroy(deo_padded* plan);
/* The same on a view of M: M has sizes in_sizes and the operator reads the
 * block that starts at 0-based index starts[b] along axis b and has x_temp's
 * size there (starts[axis-1] = 0: the first len+2 entries along the
 * differentiated axis).  Replaces the `view(M, 1:x_temp_1, ..., 1:(x_temp_k+2),
 * ...)` calls of mul!(x_temp, A::DiffEqOperatorCombination, M) for 2-D and
 * 3-D arrays (derivative_operator_functions.jl:380-463, 742-800), which begin
 * at index 1 along the other axes even where M is padded there. */
deo_status deo_padded_plan_view(const deo_operator* op, int axis, int ndims, const int64_t* out_sizes,
                                const int64_t* in_sizes, const int64_t* starts, deo_dtype dtype, deo_padded** out);

/* ------------------------------------------------------------------------
 * Implicit solves: x = A \ u for A = L*Q (ghost_derivative_operator.jl:39-58).
 * The reference concretises (A_l, A_b) = sparse(A) (concretization.jl:938-958:
 * sparse(L) * sparse(Q), Array(PeriodicBC) wrapping around) and solves
 * A_l x = u - A_b with a sparse LU.  Here A_l, the same n x n band for every
 * line of u along `axis` (n = the operator's len), is factored once on the
 * host with partial pivoting (DEO_ERR_BAD_ARG if singular), and the device
 * solves all lines.  sizes: u's Julia size.  x may be u itself (in place) but
 * may not otherwise overlap it.  Float32 lines are solved in Float64 in a
 * plan-owned workspace and rounded once, so the Float32 applies of one plan
 * must be ordered on one stream (Float64 solves work in x and may run
 * concurrently). 
 * ---------------------------------------------------------------------- */
typedef struct deo_solve deo_solve;
deo_status deo_solve_plan(const deo_operator* op, const deo_bc* bc, int ndims, const int64_t* sizes, int axis,
                          deo_dtype dtype, deo_solve** out);
/* Sub- and super-diagonals of A_l. */
deo_status deo_solve_bands(const deo_solve* plan, int* kl, int* ku);
deo_status deo_solve_apply(const deo_solve* plan, const void* u, void* x, void* stream);
void deo_solve_destroy(deo_solve* plan);

/* ------------------------------------------------------------------------
 * Vector calculus on padded arrays.
 * Replaces `A * M` and `mul!(x_temp, .., A, M)` for A = Gradient / Divergence /
 * Curl(approx_order, dx, len; coeff_func) (vector_calculus_operators.jl:7-73,
 * vector_calculus_convolutions.jl).  ops[a] is the operator of axis a+1, i.e.
 * the reference's A.ops[a+1] = CenteredDifference{a+1}(1, approx_order, dx[a+1],
 * len[a+1], coeff_func) (its `c * A` scales each op's coefficients).
 *   DEO_VC_GRADIENT:   M (len1+2, .., lenN+2)    -> out (len1, .., lenN, N)
 *   DEO_VC_DIVERGENCE: M (len1+2, .., lenN+2, N) -> out (len1, .., lenN)
 *   DEO_VC_CURL:       M (len+2, len+2, len+2, 3) -> out (len, len, len, 3)
 * N = 2 and 3 follow the reference's specialised methods, including their
 * indexing: along the differentiated axis the taps read the padded line, on
 * the other axes the point at the padded index equal to the output index
 * (x[i + idx - mid, j] for output (i, j)); each output adds its terms as the
 * reference's BC_left / interior / BC_right passes do.  Other N follow the
 * generic per-line methods (other axes at index + 1).  Column-major arrays.
 * overwrite = 1 gives `A * M` (from zeros); 0 adds into out, as the
 * reference's mul! always does.  out must not overlap M.
 * ---------------------------------------------------------------------- */
#define DEO_VC_GRADIENT 0
#define DEO_VC_DIVERGENCE 1
#define DEO_VC_CURL 2
typedef struct deo_vc deo_vc;
deo_status deo_vector_calculus_plan(int kind, int ndims, const deo_operator* const* ops, deo_dtype dtype,
                                    deo_vc** out);
/* Elements of M and of out (all components). */
deo_status deo_vector_calculus_sizes(const deo_vc* plan, int64_t* in_elems, int64_t* out_elems);
/* Execution choice (no reference counterpart): *band_nk > 0 when every
 * operator's interior rows are one centred band of that many taps (the
 * unrolled marching kernel), 0 when every row goes through the row tables. */
deo_status deo_vector_calculus_info(const deo_vc* plan, int* band_nk);
deo_status deo_vector_calculus_apply(const deo_vc* plan, const void* M, void* out, int overwrite, void* stream);
void deo_vector_calculus_destroy(deo_vc* plan);

/* Pointwise vector algebra over npts points of ncomp components stored
 * component after component (an (s..., ncomp) column-major array).
 * dot_product!(u, A, B) (vector_algebraic_operations.jl:11-28),
 * cross_product!(u, A, B) (:39-52; ncomp = 3, u has 3 components),
 * square_norm!(u, A) (:54-62).  Products are rounded before the sums.  u must
 * not overlap the inputs. */
deo_status deo_dot_product(deo_dtype dtype, int64_t npts, int ncomp, const void* A, const void* B, void* u,
                           void* stream);
deo_status deo_cross_product(deo_dtype dtype, int64_t npts, const void* A, const void* B, void* u, void* stream);
deo_status deo_square_norm(deo_dtype dtype, int64_t npts, int ncomp, const void* A, void* u, void* stream);

/* Concretisation: the affine map du = A_l u + A_b of the plan, built on the
 * device from its row tables (Array(L*Q) = (Array(L) * Q_l, Array(L) * Q_b),
 * concretization.jl:914-958, summed over the terms of a combination): one
 * thread per row, each entry the sum of its contributions in the order of
 * the product L * Q_l, in Float64 (Float32 plans: their weights widened).
 * n = prod(sizes).  Plans of padded inputs are DEO_ERR_UNSUPPORTED.
 *   deo_plan_concretize: dense A_l (n x n, column-major) and A_b (n) into
 *     host memory; device scratch from the stream-ordered allocator on a
 *     private stream; DEO_ERR_OOM when n x n does not fit the device.
 *   deo_plan_concretize_device: the same into device buffers, on `stream`,
 *     without waiting (A_l is zeroed first).
 *   deo_plan_bandwidths: the lower / upper bandwidths l, u of A_l (largest
 *     i - j and j - i over its structural entries); waits for `stream`.
 *   deo_plan_concretize_banded: BandedMatrix(L*Q): A_l in band storage,
 *     (l + u + 1) x n column-major with entry (i, j) at row u + i - j of
 *     column j (BandedMatrices' bandeddata layout), and A_b, device buffers,
 *     on `stream`; DEO_ERR_BAD_SHAPE if an entry lies outside (l, u).  Waits
 *     for `stream` (to read that check). */
deo_status deo_plan_concretize(const deo_plan* plan, double* A_l_host, double* A_b_host);
deo_status deo_plan_concretize_device(const deo_plan* plan, double* A_l_dev, double* A_b_dev, void* stream);
deo_status deo_plan_bandwidths(const deo_plan* plan, int64_t* l, int64_t* u, void* stream);
deo_status deo_plan_concretize_banded(const deo_plan* plan, int64_t l, int64_t u, double* data_dev, double* A_b_dev,
                                      void* stream);

/* ------------------------------------------------------------------------
 * Batched applies: many independent (plan, u, du) instances in ONE launch of
 * a persistent kernel that pulls tiles from a work-list.  No reference
 * counterpart (the reference applies one operator per call).
 * ---------------------------------------------------------------------- */
typedef struct deo_batch deo_batch;
typedef struct {
    const deo_plan* plan;
    const void* u;
    void* du;
} deo_instance;
/* tile = points per work item (0 = autotuned), ctas_per_sm (0 = autotuned). */
deo_status deo_batch_create(int n, const deo_instance* inst, int adjoint, int tile, int ctas_per_sm,
                            deo_batch** out);
/* The same instances with one launch each, issued from a host loop: the
 * baseline the batched launch is measured against. */
deo_status deo_apply_each(int n, const deo_instance* inst, int adjoint, void* stream);
/* Runs the batch; with use_graph = 1 the launch is captured once into a CUDA
 * graph and replayed. */
deo_status deo_batch_run(deo_batch* b, int use_graph, void* stream);
/* Re-point instance i at new buffers (same plan); invalidates the graph. */
deo_status deo_batch_set_buffers(deo_batch* b, int i, const void* u, void* du);
deo_status deo_batch_config(const deo_batch* b, int* tile, int* ctas_per_sm, int64_t* n_items);
void deo_batch_destroy(deo_batch* b);
/* Batched Runge-Kutta stage over many instances in one persistent launch:
 *   out = alpha*a + beta*b + gamma*(c + dt*Op(c))
 * with Op the instance's plan (adjoint = 0) or its adjoint (adjoint = 1);
 * a or b may be NULL (term absent); out may alias a, not c.  Three of these
 * make one SSP-RK3 step for every active instance.  No reference counterpart
 * (the reference leaves time stepping to OrdinaryDiffEq). */
typedef struct {
    const deo_plan* plan;
    const void* a;
    const void* b;
    const void* c;
    void* out;
    double alpha, beta, gamma, dt;
    int adjoint;
} deo_stage;
deo_status deo_stage_batch_create(int n, const deo_stage* stages, int tile, int ctas_per_sm, deo_batch** out);

/* Batched apply that allocates no device memory.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc -- a plug-in whose host
 * application owns every device allocation through its own pool, a server
 * that must not grow its device footprint after admitting a request -- this
 * runs the same persistent kernel as
 * deo_batch_run with its instance table, work-list and counter in one static
 * device array of DEO_NOALLOC_SCRATCH_BYTES (1 MiB).  The plans (created
 * earlier, where allocation was possible) and the instances' buffers are the
 * caller's.  Limit: 256 + 24*n (rounded up to 256) + 16*ceil(points_i / tile)
 * summed over instances bytes; larger batches return DEO_ERR_UNSUPPORTED.
 * tile = 0 means 8192 points per work item.
 * Footprint: CUDA loads modules lazily, so the array and the kernel's image
 * take device memory at the FIRST call on a device (it looks up the array's
 * address with cudaGetSymbolAddress and launches the kernel once over an empty
 * work-list), not when the library is loaded; they stay until the process
 * exits.  A call with n = 0 does only this set-up: make it where the footprint
 * may still grow (before admitting requests).  No call may be made under
 * stream capture (its copy from a reused host image cannot be captured):
 * on a capturing stream it returns DEO_ERR_UNSUPPORTED and enqueues nothing.
 * After a device reset the next call repeats the set-up.
 * Each call copies its work-list from host memory on `stream`; calls on one
 * stream are ordered by that stream.  Every call reuses the same array (the
 * counter is cleared each time), so calls that overlap on the GPU -- on
 * different streams or host threads -- race and must be serialised by the
 * caller. */
#define DEO_NOALLOC_SCRATCH_BYTES (1 << 20)
deo_status deo_batch_apply_noalloc(int n, const deo_instance* inst, int adjoint, int tile, void* stream);

/* ------------------------------------------------------------------------
 * Serving: a device-resident loop of method-of-lines solves.  No reference
 * counterpart (the reference leaves time stepping to OrdinaryDiffEq and has
 * no serving layer); each solve's right-hand side is a plan, the reference's
 * (L)(du, u, p, t) = mul!(du, L, u) (DiffEqOperators.jl:67-76).
 * A request is nsteps fixed SSP-RK3 steps (Shu-Osher) of du/dt = A u from u0,
 * and with want_grad also the gradient of ||u(T)||^2 with respect to u0 (the
 * transposed steps from 2 u(T)).  Its state (three device arrays of the
 * plan's size and dtype) comes from the stream-ordered allocator at
 * admission; admission is FIFO under the byte budget.  deo_serve_pump never
 * waits for the device: it collects finished results, admits what fits, and
 * enqueues rounds (at most two in flight) of S steps, S the fewest steps any
 * active request has left, in which three batched stage launches per step
 * advance every active request.  A request's result does not depend on the
 * others served with it.  All functions are thread-safe on one server.
 * ---------------------------------------------------------------------- */
typedef struct deo_server deo_server;
typedef struct {
    const deo_plan* plan;  /* right-hand side A; its size and dtype are the state's; kept alive by the caller */
    const void* u0;        /* host memory, Julia layout, the server's dtype; copied by deo_serve_submit */
    int nsteps;            /* K >= 1 */
    double dt;             /* > 0 */
    int want_grad;         /* also d ||u(T)||^2 / d u0 */
} deo_request;
typedef struct {
    int64_t submitted, admitted, completed, rejected, failed, cancelled;
    int64_t rounds, steps, launches, rebuilds;
    int64_t in_use_bytes, active, pending;
    int64_t device_us;  /* device time of the retired rounds, first launch to last */
} deo_serve_stats;
/* budget_bytes: device memory the admitted requests may take: each one's
 * three state buffers, its plan's device tables and its stage work-list
 * entries;
 * max_steps_per_round caps S (0 = 64). */
deo_status deo_serve_create(size_t budget_bytes, deo_dtype dtype, int max_steps_per_round, deo_server** out);
/* *rid receives the request id.  DEO_ERR_REJECTED (with *rid set) if its state
 * is larger than the whole budget. */
deo_status deo_serve_submit(deo_server* s, const deo_request* r, int64_t* rid);
/* One round of bookkeeping (see above); call it in the caller's loop. */
deo_status deo_serve_pump(deo_server* s);
/* DEO_ERR_NOT_READY while the request runs; DEO_OK once finished: u(T) (and
 * with want_grad the gradient) copied to uT / grad (host, may be NULL), the
 * time from submission to completion to *latency_s (may be NULL), and the
 * request forgotten.  A rejected, cancelled or failed request reports
 * DEO_ERR_REJECTED, DEO_ERR_BAD_ARG or DEO_ERR_OOM (device memory for its
 * state could not be allocated) once, and is forgotten too. */
deo_status deo_serve_poll(deo_server* s, int64_t rid, void* uT, void* grad, double* latency_s);
/* Withdraws a pending or running request (its memory returns after the rounds
 * already enqueued); DEO_ERR_BAD_ARG if it has finished. */
deo_status deo_serve_cancel(deo_server* s, int64_t rid);
deo_status deo_serve_stats_get(deo_server* s, deo_serve_stats* out);
/* Test hook: the next n admissions fail as if the device allocation had
 * failed (the request reports DEO_ERR_OOM; the server goes on). */
deo_status deo_serve_inject_alloc_failures(deo_server* s, int n);
/* Waits for the server's work, frees its memory. */
void deo_serve_destroy(deo_server* s);

/* Plan autotuner for Laplacian-type plans on the TMA path: times the
 * bit-identical execution choices (Float32: scalar or vectorised interior and
 * its tile; the boundary-shell kernel; the shell beside the interior or after
 * it) with overwriting applies u -> du on `stream`, keeps the fastest in the
 * plan's options (DEO_OPT_F32_VECTOR, DEO_OPT_F32_TILE, DEO_OPT_SHELL_KERNEL,
 * DEO_OPT_CONCURRENT_SHELL), and caches it per (sizes, dtype, terms, band
 * radius, exact-sums variant, boundary kinds) in the file `cache_path`
 * (NULL = in-process only).  Other plans: nothing to choose, DEO_OK.
 * Writes du.  No reference counterpart. */
deo_status deo_plan_autotune(deo_plan* plan, const void* u, void* du, const char* cache_path, void* stream);
/* What the last deo_plan_autotune on this plan timed (nothing when it took
 * its choice from the cache): *n candidates, the first the plan's choice
 * before it; candidate i is cands[4i .. 4i+3] = (DEO_OPT_F32_VECTOR,
 * DEO_OPT_F32_TILE, DEO_OPT_SHELL_KERNEL, DEO_OPT_CONCURRENT_SHELL) and
 * ms[i] its best time per apply; at most cap are written. */
deo_status deo_plan_autotune_times(const deo_plan* plan, int* cands, float* ms, int cap, int* n);
/* Autotuner: times candidate (tile, ctas_per_sm) pairs on this batch and
 * keeps the fastest; results are cached per workload signature in the file
 * `cache_path` (NULL = in-process cache only). */
deo_status deo_batch_autotune(deo_batch* b, const char* cache_path, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DEO_H */
