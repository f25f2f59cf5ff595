// deo_host.cpp -- host side of libdeo: operator and boundary-condition
// constructors, the row-table compiler, plans and the C ABI (include/deo.h).
//
// The constructors restate DiffEqOperators.jl's (cited per function) so a
// caller without Julia gets the same tables; a Julia caller passes its own
// DerivativeOperator tables through deo_operator_from_tables instead.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/deo.h"
#include "deo_internal.h"

using deo::PlanDev;
using deo::RowTabDev;
using deo::TermDev;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_err;

static deo_status fail(deo_status s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
static deo_status fail(deo_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return s;
}

static deo_status cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? DEO_ERR_OOM : DEO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CUDA_TRY(expr, what)                         \
    do {                                             \
        cudaError_t e_ = (expr);                     \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

extern "C" const char* deo_last_error(void) { return g_err.c_str(); }
extern "C" int deo_abi_version(void) { return DEO_ABI_VERSION; }

// ---------------------------------------------------------------------------
// Float64 ^ Int as Julia computes it (Base.pow_body, compensated squaring):
// the operators scale their weights by 1/dx^d with this.
// ---------------------------------------------------------------------------
static double pow_int(double x, long n) {
    if (n == 0) return 1.0;
    if (n == 3) return x * x * x;
    double y = 1.0, xnlo = 0.0, ynlo = 0.0;
    if (n < 0) {
        const double rx = 1.0 / x;
        if (n == -2) return rx * rx;
        if (std::isfinite(x)) xnlo = -std::fma(x, rx, -1.0) * rx;
        x = rx;
        n = -n;
    }
    while (n > 1) {
        if (n & 1) {
            const double err = std::fma(y, xnlo, x * ynlo);
            const double hi = x * y;
            ynlo = std::fma(x, y, -hi) + err;
            y = hi;
        }
        const double err = x * 2 * xnlo;
        const double hi = x * x;
        xnlo = std::fma(x, x, -hi) + err;
        x = hi;
        n >>= 1;
    }
    const double err = std::fma(y, xnlo, x * ynlo);
    return (std::isfinite(x) && std::isfinite(err)) ? std::fma(x, y, err) : x * y;
}

// ---------------------------------------------------------------------------
// Fornberg weights (fornberg.jl:7-62): recurrence over the points, then the
// centre entry absorbs the rounding residue of the weight sum.
// ---------------------------------------------------------------------------
static std::vector<double> fd_weights(int m, double x0, const std::vector<double>& x) {
    const int n = (int)x.size();
    const int w = m + 1;
    std::vector<double> C((size_t)n * w, 0.0);  // C[row*w + order]
    C[0] = 1.0;
    double c1 = 1.0, c4 = x[0] - x0;
    for (int i = 1; i < n; ++i) {
        const int mn = std::min(i, m);
        double c2 = 1.0;
        const double c5 = c4;
        c4 = x[i] - x0;
        for (int j = 0; j < i; ++j) {
            const double c3 = x[i] - x[j];
            c2 *= c3;
            if (j == i - 1) {
                for (int s = mn; s >= 1; --s)
                    C[(size_t)i * w + s] = c1 * ((double)s * C[(size_t)(i - 1) * w + s - 1] - c5 * C[(size_t)(i - 1) * w + s]) / c2;
                C[(size_t)i * w] = -c1 * c5 * C[(size_t)(i - 1) * w] / c2;
            }
            for (int s = mn; s >= 1; --s)
                C[(size_t)j * w + s] = (c4 * C[(size_t)j * w + s] - (double)s * C[(size_t)j * w + s - 1]) / c3;
            C[(size_t)j * w] = c4 * C[(size_t)j * w] / c3;
        }
        c1 = c2;
    }
    std::vector<double> out(n);
    for (int i = 0; i < n; ++i) out[i] = C[(size_t)i * w + m];
    if (m != 0) {
        double s = out[0];
        for (int i = 1; i < n; ++i) s = s + out[i];
        out[n / 2] -= s;
    }
    return out;
}

// ---------------------------------------------------------------------------
// operators
// ---------------------------------------------------------------------------
struct deo_operator {
    int d = 0, a = 0, len = 0, stl = 0, bstl = 0, bpc = 0, off = 0;
    int wind = 0, uniform = 1, cfs = 1;
    int n_st = 0, n_low = 0, n_high = 0;
    std::vector<double> st, lo, hi, coeff;
    int halves() const { return (wind && !uniform) ? 2 : 1; }
    const double* S(int row, int h = 0) const { return &st[((size_t)h * n_st + row) * stl]; }
    const double* Lo(int row, int h = 0) const { return &lo[((size_t)h * n_low + row) * bstl]; }
    const double* Hi(int row, int h = 0) const { return &hi[((size_t)h * n_high + row) * bstl]; }
};

static void append(std::vector<double>& dst, const std::vector<double>& r) { dst.insert(dst.end(), r.begin(), r.end()); }
static std::vector<double> iota_d(int lo, int hi, int step = 1) {
    std::vector<double> v;
    for (int k = lo; step > 0 ? k <= hi : k >= hi; k += step) v.push_back((double)k);
    return v;
}
static std::vector<double> times(double s, std::vector<double> v) {
    for (auto& e : v) e = s * e;
    return v;
}

extern "C" deo_status deo_calculate_weights(int order, double x0, const double* x, int n, double* out) {
    if (!x || !out || n <= 0) return fail(DEO_ERR_BAD_ARG, "null or empty point set");
    if (order < 0 || order >= n) return fail(DEO_ERR_BAD_ARG, "Not enough points for the requested order.");
    std::vector<double> w = fd_weights(order, x0, std::vector<double>(x, x + n));
    std::copy(w.begin(), w.end(), out);
    return DEO_OK;
}

extern "C" deo_status deo_centered_difference(int d, int a, const double* dx, int ndx, int len, deo_operator** out) {
    if (!out || !dx) return fail(DEO_ERR_BAD_ARG, "null argument");
    if (a <= 1) return fail(DEO_ERR_BAD_ARG, "approximation_order must be greater than 1.");
    if (d < 0 || len < 1) return fail(DEO_ERR_BAD_ARG, "invalid derivative order or length");
    // The reference reads dx[1 : len+1] for the interior and dx[end-bstl+1 : end]
    // for the high boundary rows (derivative_operator.jl:150-170), so a longer
    // dx is accepted as it is there; a shorter one is its BoundsError.
    if (ndx != 1 && (ndx < len + 1 || ndx < d + a))
        return fail(DEO_ERR_BAD_SHAPE, "dx must have 1 entry or at least max(len+1, d+a) entries");
    auto op = std::make_unique<deo_operator>();
    op->d = d; op->a = a; op->len = len;
    op->stl = d + a - 1 + (d + a) % 2;
    op->bstl = d + a;
    op->bpc = op->stl / 2 - 1;
    if (std::max(op->stl, op->bstl) > DEO_MAX_NW) return fail(DEO_ERR_UNSUPPORTED, "stencil wider than %d", DEO_MAX_NW);
    const int stl = op->stl, bstl = op->bstl, bpc = op->bpc;
    if (ndx == 1) {
        op->uniform = 1;
        const double s = 1.0 / pow_int(dx[0], d);
        append(op->st, times(s, fd_weights(d, 0.0, iota_d(-(stl / 2), stl / 2))));
        op->n_st = 1;
        std::vector<std::vector<double>> low;
        const std::vector<double> lx = iota_d(0, bstl - 1);
        for (int x0 = 1; x0 <= stl / 2 - 1; ++x0) low.push_back(times(s, fd_weights(d, (double)x0, lx)));
        for (auto& r : low) append(op->lo, r);
        // high = reverse(map(reverse, low * (-1)^d))  (derivative_operator.jl:114-116)
        const double sg = (d % 2 == 0) ? 1.0 : -1.0;
        for (int i = bpc - 1; i >= 0; --i)
            for (int k = 0; k < bstl; ++k) op->hi.push_back(low[i][bstl - 1 - k] * sg);
    } else {
        op->uniform = 0;
        if (len + 1 - bpc < bpc + 2 && len - 2 * bpc < 0) return fail(DEO_ERR_BAD_SHAPE, "grid too short for stencil");
        std::vector<double> sx(stl, 0.0);
        const int c = stl / 2;
        for (int i = bpc + 2; i <= len + 1 - bpc; ++i) {  // generate_coordinates, :137-148
            for (auto& e : sx) e = e * 0.0;
            for (int k = 1; k <= stl / 2; ++k) {
                sx[c + k] = sx[c + k - 1] + dx[i + k - 2];
                sx[c - k] = sx[c - k + 1] - dx[i - k - 1];
            }
            append(op->st, fd_weights(d, 0.0, sx));
        }
        op->n_st = std::max(0, len - 2 * bpc);
        std::vector<double> lx(bstl), hx(bstl);
        lx[0] = 0.0;
        for (int k = 1; k < bstl; ++k) lx[k] = lx[k - 1] + dx[k - 1];
        for (int k = 0; k < bstl; ++k) hx[k] = (k == 0) ? dx[ndx - bstl] : hx[k - 1] + dx[ndx - bstl + k];
        for (int i = 1; i <= bpc; ++i) append(op->lo, fd_weights(d, lx[i], lx));
        for (int i = bpc; i >= 1; --i) append(op->hi, fd_weights(d, hx[bstl - 1 - i], hx));
    }
    op->n_low = op->n_high = bpc;
    op->coeff.assign(len, 0.0 + 1.0);
    op->cfs = 1;
    *out = op.release();
    return DEO_OK;
}

extern "C" deo_status deo_upwind_difference(int d, int a, const double* dx, int ndx, int len, int off,
                                            deo_operator** out) {
    if (!out || !dx) return fail(DEO_ERR_BAD_ARG, "null argument");
    if (off < 0) return fail(DEO_ERR_BAD_ARG, "Number of offside points should be non-negative");
    if (off > (d + a - 1) / 2) return fail(DEO_ERR_BAD_ARG, "Number of offside points should not exceed the primary wind points");
    if (d < 0 || a < 1 || len < 1) return fail(DEO_ERR_BAD_ARG, "invalid derivative order or length");
    // The reference builds its grid x = [0; cumsum(dx)] and reads x[1 : len+2]
    // (derivative_operator.jl:515-639): a longer dx is accepted, a shorter one
    // is its BoundsError.
    if (ndx != 1 && ndx < len + 1) return fail(DEO_ERR_BAD_SHAPE, "dx must have 1 entry or at least len+1 entries");
    auto op = std::make_unique<deo_operator>();
    op->d = d; op->a = a; op->len = len; op->wind = 1; op->off = off;
    op->stl = op->bstl = d + a;
    op->bpc = op->bstl - 2 - off;
    if (op->stl > DEO_MAX_NW) return fail(DEO_ERR_UNSUPPORTED, "stencil wider than %d", DEO_MAX_NW);
    const int stl = op->stl, bstl = op->bstl, bpc = op->bpc;
    if (ndx == 1) {
        op->uniform = 1;
        const double h = dx[0];
        const double s = 1.0 / pow_int(h, d);
        append(op->st, times(s, fd_weights(d, 0.0, iota_d(-off, stl - 1 - off))));
        op->n_st = 1;
        const std::vector<double> lx = iota_d(0, bstl - 1);
        for (int x0 = 1; x0 <= bstl - 2 - off; ++x0) append(op->lo, times(s, fd_weights(d, (double)x0, lx)));
        op->n_low = bpc;
        const std::vector<double> hx = iota_d(0, -(bstl - 1), -1);
        const double sh = pow_int(-1.0 / h, d);
        int nh = 0;
        for (int x0 = -1; x0 >= -(bstl - 2); --x0, ++nh) append(op->hi, times(sh, fd_weights(d, (double)x0, hx)));
        op->n_high = nh;
    } else {
        op->uniform = 0;
        if (len - 2 * bpc < 0) return fail(DEO_ERR_BAD_SHAPE, "grid too short for stencil");
        std::vector<double> x(len + 2);
        x[0] = 0.0;
        for (int k = 1; k <= len + 1; ++k) x[k] = x[k - 1] + dx[k - 1];
        auto X = [&](int j) { return x[j - 1]; };
        // x[lo:hi] (1-based, inclusive); a window outside x is the reference's
        // BoundsError for a grid too short for the stencil
        bool outside = false;
        auto sub = [&](int lo, int hi) {
            if (lo < 1 || hi > len + 2 || hi - lo + 1 != bstl) {
                outside = true;
                return iota_d(0, bstl - 1);
            }
            return std::vector<double>(x.begin() + (lo - 1), x.begin() + hi);
        };
        std::vector<double> up, dn;
        if (off == 0) {
            for (int i = 1; i <= bpc; ++i) append(up, fd_weights(d, X(i + 1), sub(i + 1, i + bstl)));
        } else {
            for (int i = 1; i <= off - 1; ++i) append(up, fd_weights(d, X(i + 1), sub(1, bstl)));
            for (int i = off; i <= bpc; ++i) append(up, fd_weights(d, X(i + 1), sub(i + 1 - off, i + bstl - off)));
        }
        for (int i = 1; i <= bpc; ++i) append(dn, fd_weights(d, X(i + 1), sub(1, bstl)));
        op->lo = up;
        append(op->lo, dn);
        op->n_low = bpc;
        up.clear(); dn.clear();
        for (int i = bpc + 1; i <= len - bpc; ++i) append(up, fd_weights(d, X(i + 1), sub(i + 1 - off, i + stl - off)));
        for (int i = bpc + 1; i <= len - bpc; ++i)
            append(dn, fd_weights(d, X(i + 1), sub(i - stl + 2 + off, i + 1 + off)));
        op->st = up;
        append(op->st, dn);
        op->n_st = std::max(0, len - 2 * bpc);
        up.clear(); dn.clear();
        for (int i = len - bpc + 1 - off; i <= len; ++i) append(up, fd_weights(d, X(i + 1), sub(len - bstl + 3, len + 2)));
        if (off == 0) {
            for (int i = len - bpc + 1; i <= len; ++i) append(dn, fd_weights(d, X(i + 1), sub(i - stl + 2, i + 1)));
        } else {
            for (int i = len - bpc + 1 - off; i <= len - off + 1; ++i)
                append(dn, fd_weights(d, X(i + 1), sub(i - stl + 2 + off, i + 1 + off)));
            for (int i = len - off + 2; i <= len; ++i) append(dn, fd_weights(d, X(i + 1), sub(len - stl + 3, len + 2)));
        }
        op->hi = up;
        append(op->hi, dn);
        op->n_high = bpc + off;
        if (outside) return fail(DEO_ERR_BAD_SHAPE, "grid too short for stencil");
    }
    op->coeff.assign(len, 0.0 + 1.0);
    op->cfs = 1;
    *out = op.release();
    return DEO_OK;
}

extern "C" deo_status deo_operator_from_tables(const deo_operator_desc* ds, deo_operator** out) {
    if (!ds || !out) return fail(DEO_ERR_BAD_ARG, "null argument");
    auto op = std::make_unique<deo_operator>();
    op->d = ds->derivative_order; op->a = ds->approximation_order; op->len = ds->len;
    op->stl = ds->stencil_length; op->bstl = ds->boundary_stencil_length; op->bpc = ds->boundary_point_count;
    op->off = ds->offside; op->wind = ds->winding != 0; op->uniform = ds->uniform != 0; op->cfs = ds->coeff_func_sign;
    op->n_st = ds->n_stencil_rows; op->n_low = ds->n_low_rows; op->n_high = ds->n_high_rows;
    if (op->len < 1 || op->stl < 1 || op->bstl < 1 || op->bpc < 0 || op->off < 0)
        return fail(DEO_ERR_BAD_ARG, "invalid operator sizes");
    if (std::max(op->stl, op->bstl) > DEO_MAX_NW) return fail(DEO_ERR_UNSUPPORTED, "stencil wider than %d", DEO_MAX_NW);
    const int h = op->halves();
    if (op->uniform ? op->n_st != 1 : op->n_st != std::max(0, op->len - 2 * op->bpc))
        return fail(DEO_ERR_BAD_SHAPE, "stencil row count does not match len and boundary_point_count");
    if (!ds->stencil_coefs || !ds->coefficients) return fail(DEO_ERR_BAD_ARG, "null table");
    op->st.assign(ds->stencil_coefs, ds->stencil_coefs + (size_t)h * op->n_st * op->stl);
    if (op->n_low) {
        if (!ds->low_boundary_coefs) return fail(DEO_ERR_BAD_ARG, "null low boundary table");
        op->lo.assign(ds->low_boundary_coefs, ds->low_boundary_coefs + (size_t)h * op->n_low * op->bstl);
    }
    if (op->n_high) {
        if (!ds->high_boundary_coefs) return fail(DEO_ERR_BAD_ARG, "null high boundary table");
        op->hi.assign(ds->high_boundary_coefs, ds->high_boundary_coefs + (size_t)h * op->n_high * op->bstl);
    }
    op->coeff.assign(ds->coefficients, ds->coefficients + op->len);
    *out = op.release();
    return DEO_OK;
}

extern "C" deo_status deo_operator_describe(const deo_operator* op, deo_operator_desc* ds) {
    if (!op || !ds) return fail(DEO_ERR_BAD_ARG, "null argument");
    ds->derivative_order = op->d; ds->approximation_order = op->a; ds->len = op->len;
    ds->stencil_length = op->stl; ds->boundary_stencil_length = op->bstl; ds->boundary_point_count = op->bpc;
    ds->offside = op->off; ds->winding = op->wind; ds->uniform = op->uniform; ds->coeff_func_sign = op->cfs;
    ds->n_stencil_rows = op->n_st; ds->n_low_rows = op->n_low; ds->n_high_rows = op->n_high;
    ds->stencil_coefs = op->st.data(); ds->low_boundary_coefs = op->lo.data();
    ds->high_boundary_coefs = op->hi.data(); ds->coefficients = op->coeff.data();
    return DEO_OK;
}

extern "C" deo_status deo_operator_set_coefficients(deo_operator* op, const double* c, int n, int cfs) {
    if (!op || !c) return fail(DEO_ERR_BAD_ARG, "null argument");
    if (n != 1 && n != op->len)
        return fail(DEO_ERR_BAD_SHAPE, "length of c (%d) must match length of A (%d)", n, op->len);
    for (int i = 0; i < op->len; ++i) op->coeff[i] = 0.0 + (n == 1 ? c[0] : c[i]);
    op->cfs = cfs;
    return DEO_OK;
}

extern "C" deo_status deo_operator_scale_coefficients(deo_operator* op, const double* c, int n) {
    if (!op || !c) return fail(DEO_ERR_BAD_ARG, "null argument");
    if (n != 1 && n != op->len)
        return fail(DEO_ERR_BAD_SHAPE, "length of c (%d) must match length of A (%d)", n, op->len);
    for (int i = 0; i < op->len; ++i) op->coeff[i] = (n == 1 ? c[0] : c[i]) * op->coeff[i];
    return DEO_OK;
}

extern "C" deo_status deo_operator_clone(const deo_operator* op, deo_operator** out) {
    if (!op || !out) return fail(DEO_ERR_BAD_ARG, "null argument");
    *out = new deo_operator(*op);
    return DEO_OK;
}

extern "C" void deo_operator_destroy(deo_operator* op) { delete op; }

// ---------------------------------------------------------------------------
// boundary conditions
// ---------------------------------------------------------------------------
static std::vector<double> one_to(int n) { return iota_d(1, n); }

extern "C" deo_status deo_robin_bc(const double* l, const double* r, const double* dx, int ndx, int order, deo_bc* q) {
    if (!l || !r || !dx || !q) return fail(DEO_ERR_BAD_ARG, "null argument");
    if (order < 1 || order > DEO_MAX_BC) return fail(DEO_ERR_UNSUPPORTED, "Robin order must be in 1..%d", DEO_MAX_BC);
    std::memset(q, 0, sizeof *q);
    const std::vector<double> s = fd_weights(1, 1.0, one_to(order + 1));
    const int m = order;
    if (ndx == 1) {  // bc_operators.jl:26-39
        const double h = dx[0];
        const double dl = l[0] * h / l[1] + s[0], dr = r[0] * h / r[1] - s[0];
        for (int k = 0; k < m; ++k) q->a_l[k] = -s[1 + k] / dl;
        for (int k = 0; k < m; ++k) q->a_r[k] = s[m - k] / dr;
        q->b_l = l[2] / (l[0] + l[1] * s[0] / h);
        q->b_r = r[2] / (r[0] - r[1] * s[0] / h);
    } else {  // bc_operators.jl:40-60
        const int ns = order + 1;
        if (ndx < ns) return fail(DEO_ERR_BAD_SHAPE, "dx shorter than the Robin stencil");
        const double* xl = dx;
        const double* xr = dx + (ndx - ns);
        const double dl = l[0] + l[1] * s[0] / xl[0];
        const double dr = r[0] - r[1] * s[0] / xr[ns - 1];
        for (int k = 0; k < m; ++k) q->a_l[k] = -l[1] * s[1 + k] / (dl * xl[1 + k]);
        for (int k = 0; k < m; ++k) q->a_r[k] = r[1] * s[m - k] / (dr * xr[k]);
        q->b_l = l[2] / dl;
        q->b_r = r[2] / dr;
    }
    q->m_l = q->m_r = m;
    q->kind = DEO_BC_AFFINE;
    return DEO_OK;
}

extern "C" deo_status deo_general_bc(const double* al, int nl, const double* ar, int nr, const double* dx, int ndx,
                                     int order, deo_bc* q) {
    if (!al || !ar || !dx || !q) return fail(DEO_ERR_BAD_ARG, "null argument");
    if (nl < 3 || nr < 3) return fail(DEO_ERR_BAD_ARG, "GeneralBC needs at least 3 coefficients per side");
    const int wl = order + nl - 2, wr = order + nr - 2;
    if (order < 1 || wl - 1 > DEO_MAX_BC || wr - 1 > DEO_MAX_BC) return fail(DEO_ERR_UNSUPPORTED, "GeneralBC stencil too long");
    if (ndx != 1 && (ndx < wl || ndx < wr)) return fail(DEO_ERR_BAD_SHAPE, "dx shorter than the GeneralBC stencil");
    std::memset(q, 0, sizeof *q);
    // S rows: weights of derivative i at the boundary, divided by dx^i
    // (per point dx_l[k]^i on a non-uniform grid, bc_operators.jl:139-144).
    std::vector<std::vector<double>> Sl(nl - 2, std::vector<double>(wl, 0.0)), Sr(nr - 2, std::vector<double>(wr, 0.0));
    for (int i = 1; i <= nl - 2; ++i) {
        const std::vector<double> w = fd_weights(i, 1.0, one_to(order + i));
        for (int k = 0; k < wl; ++k)
            Sl[i - 1][k] = (k < (int)w.size() ? w[k] : 0.0) / pow_int(ndx == 1 ? dx[0] : dx[k], i);
    }
    for (int i = 1; i <= nr - 2; ++i) {
        const std::vector<double> w = fd_weights(i, (double)(order + i), one_to(order + i));
        for (int k = 0; k < wr; ++k)
            Sr[i - 1][k] = (k < (int)w.size() ? w[k] : 0.0) / pow_int(ndx == 1 ? dx[0] : dx[ndx - 1 - k], i);
    }
    double sl = 0.0, sr = 0.0;
    for (int i = 0; i < nl - 2; ++i) sl = (i == 0) ? al[2] * Sl[0][0] : sl + al[2 + i] * Sl[i][0];
    for (int i = 0; i < nr - 2; ++i) sr = (i == 0) ? ar[2] * Sr[0][wr - 1] : sr + ar[2 + i] * Sr[i][wr - 1];
    const double denl = al[1] + sl, denr = ar[1] + sr;
    q->m_l = wl - 1;
    for (int k = 0; k < wl - 1; ++k) {
        double acc = 0.0;
        for (int i = 0; i < nl - 2; ++i) acc = (i == 0) ? al[2] * Sl[0][1 + k] : acc + al[2 + i] * Sl[i][1 + k];
        q->a_l[k] = -acc / denl;
    }
    q->m_r = wr - 1;
    for (int k = 0; k < wr - 1; ++k) {
        // column k of Sr = S_r[:, end-1-k]; a_r is the reversal
        double acc = 0.0;
        for (int i = 0; i < nr - 2; ++i) acc = (i == 0) ? ar[2] * Sr[0][wr - 2 - k] : acc + ar[2 + i] * Sr[i][wr - 2 - k];
        q->a_r[wr - 2 - k] = -acc / denr;
    }
    q->b_l = -al[0] / denl;
    q->b_r = -ar[0] / denr;
    q->kind = DEO_BC_AFFINE;
    return DEO_OK;
}

extern "C" deo_status deo_dirichlet_bc(double l, double r, deo_bc* q) {
    const double L[3] = {1.0, 0.0, l}, R[3] = {1.0, 0.0, r}, one = 1.0;
    return deo_robin_bc(L, R, &one, 1, 2, q);
}

extern "C" deo_status deo_neumann_bc(double l, double r, const double* dx, int ndx, int order, deo_bc* q) {
    const double L[3] = {0.0, 1.0, l}, R[3] = {0.0, 1.0, r};
    return deo_robin_bc(L, R, dx, ndx, order, q);
}

extern "C" deo_status deo_periodic_bc(deo_bc* q) {
    if (!q) return fail(DEO_ERR_BAD_ARG, "null argument");
    std::memset(q, 0, sizeof *q);
    q->kind = DEO_BC_PERIODIC;
    return DEO_OK;
}

extern "C" deo_status deo_bc_array(const deo_bc* b, int N, double* QL, double* Qb) {
    if (!b || !QL || !Qb || N < 1) return fail(DEO_ERR_BAD_ARG, "bad argument");
    const long R = N + 2;
    std::fill(QL, QL + R * N, 0.0);
    std::fill(Qb, Qb + R, 0.0);
    for (long i = 0; i < N; ++i) QL[i * R + i + 1] = 1.0;
    if (b->kind == DEO_BC_PERIODIC) {
        QL[(N - 1) * R] = 1.0;
        QL[N + 1] = 1.0;
        return DEO_OK;
    }
    if (b->m_l > N || b->m_r > N) return fail(DEO_ERR_BAD_SHAPE, "BC stencil longer than N");
    for (int j = 0; j < b->m_l; ++j) QL[j * R] = b->a_l[j];
    for (int j = 0; j < b->m_r; ++j) QL[(N - b->m_r + j) * R + N + 1] = b->a_r[j];
    Qb[0] = b->b_l;
    Qb[N + 1] = b->b_r;
    return DEO_OK;
}

// ---------------------------------------------------------------------------
// Array(L): concretization.jl:8-52 (centred) and :556-671 (upwind)
// ---------------------------------------------------------------------------
// The entries of Array(L) in the reference's assignment order: set(i, j, v)
// for row i (1..len) and padded column j (1..len+2); later calls overwrite.
template <class Set>
static void array_entries(const deo_operator* op, Set set_any) {
    const long N = op->len;
    auto set = [&](long i, long j, double v) {
        if (i >= 1 && i <= N && j >= 1 && j <= N + 2) set_any(i, j, v);
    };
    const int bl = op->bpc, stl = op->stl, bstl = op->bstl, off = op->off;
    auto c = [&](long i) { return op->coeff[i - 1]; };
    if (!op->wind) {
        const int pivot = stl / 2;
        for (int i = 1; i <= bl; ++i)
            for (int k = 0; k < bstl; ++k) set(i, 1 + k, c(i) * op->Lo(i - 1)[k]);
        for (long i = bl + 1; i <= N - bl; ++i) {
            const double* s = op->uniform ? op->S(0) : op->S((int)(i - bl - 1));
            for (int k = 0; k < stl; ++k) set(i, i + 1 - pivot + k, c(i) * s[k]);
        }
        for (long i = N - bl + 1; i <= N; ++i)
            for (int k = 0; k < bstl; ++k) set(i, N - bstl + 3 + k, c(i) * op->Hi((int)(i - N + bl - 1))[k]);
        return;
    }
    const double sg = (op->d % 2 == 0) ? 1.0 : -1.0;
    if (op->uniform) {
        const double* S = op->S(0);
        for (int i = 1; i <= bl; ++i) {
            if (c(i) >= 0 && i + stl <= N + 2 && i >= off)
                for (int k = 0; k < stl; ++k) set(i, i + 1 - off + k, c(i) * S[k]);
            else
                for (int k = 0; k < bstl; ++k) set(i, 1 + k, c(i) * op->Lo(i - 1)[k]);
        }
        for (long i = bl + 1; i <= N - bl - off; ++i) {
            if (c(i) >= 0)
                for (int k = 0; k < stl; ++k) set(i, i + 1 - off + k, c(i) * S[k]);
            else
                for (int k = 0; k < stl; ++k) set(i, i - stl + 2 + off + k, c(i) * (sg * S[stl - 1 - k]));
        }
        for (int r = 1; r <= bl + off; ++r) {
            const long i = N - bl + r - off;
            const double ci = c(i);
            if (ci < 0 && N + 2 - stl - bl + r >= 1 && r <= bl + 1)
                for (int k = 0; k < stl; ++k) set(i, r + N - stl - bl + 2 + k, ci * (sg * S[stl - 1 - k]));
            else if (ci < 0 && N + 2 - stl - bl + r >= 1 && r > bl + 1) {
                const double* h = op->Hi(bl + off + 1 - r - 1);
                for (int k = 0; k < bstl; ++k) set(i, N - bstl + 3 + k, ci * (sg * h[bstl - 1 - k]));
            } else if (ci >= 0 && r < off + 1)
                for (int k = 0; k < stl; ++k) set(i, N - stl + r - off + 3 + k, ci * S[k]);
            else
                for (int k = 0; k < bstl; ++k) set(i, N - bstl + 3 + k, ci * op->Hi(r - 1)[k]);
        }
        return;
    }
    for (int i = 1; i <= bl; ++i) {
        if (c(i) >= 0 && off == 0)
            for (int k = 0; k < stl; ++k) set(i, i + 1 + k, c(i) * op->Lo(i - 1, 0)[k]);
        else if (c(i) >= 0 && i < off)
            for (int k = 0; k < stl; ++k) set(i, 1 + k, c(i) * op->Lo(i - 1, 0)[k]);
        else if (c(i) >= 0 && i >= off)
            for (int k = 0; k < stl; ++k) set(i, i + 1 - off + k, c(i) * op->Lo(i - 1, 0)[k]);
        else
            for (int k = 0; k < bstl; ++k) set(i, 1 + k, c(i) * op->Lo(i - 1, 1)[k]);
    }
    for (long i = bl + 1; i <= N - bl - off; ++i) {
        if (c(i) >= 0)
            for (int k = 0; k < stl; ++k) set(i, i + 1 - off + k, c(i) * op->S((int)(i - bl - 1), 0)[k]);
        else
            for (int k = 0; k < stl; ++k) set(i, i - stl + 2 + off + k, c(i) * op->S((int)(i - bl - 1), 1)[k]);
    }
    for (long i = N - bl + 1 - off; i <= N; ++i) {
        const int hr = (int)(i - N + bl + off - 1);
        if (c(i) < 0 && i <= N - off)
            for (int k = 0; k < stl; ++k) set(i, i - stl + 2 + off + k, c(i) * op->Hi(hr, 1)[k]);
        else if (c(i) < 0)
            for (int k = 0; k < stl; ++k) set(i, N - stl + 3 + k, c(i) * op->Hi(hr, 1)[k]);
        else if (i <= N - bl)
            for (int k = 0; k < stl; ++k) set(i, i - bstl + 2 + off + k, c(i) * op->S((int)(i - bl - 1), 0)[k]);
        else
            for (int k = 0; k < bstl; ++k) set(i, N - bstl + 3 + k, c(i) * op->Hi(hr, 0)[k]);
    }
    return;
}

extern "C" deo_status deo_operator_array(const deo_operator* op, double* M) {
    if (!op || !M) return fail(DEO_ERR_BAD_ARG, "null argument");
    const long N = op->len;
    std::fill(M, M + N * (N + 2), 0.0);
    array_entries(op, [&](long i, long j, double v) { M[(j - 1) * N + (i - 1)] = v; });
    return DEO_OK;
}

// BandedMatrix(L): the reference's bandwidths (concretization.jl:123-128 centred,
// :794-890 upwind) and the entries of Array(L) in band storage.
extern "C" deo_status deo_operator_banded(const deo_operator* op, int* l, int* u, double* data) {
    if (!op || !l || !u) return fail(DEO_ERR_BAD_ARG, "null argument");
    *l = op->wind ? op->stl - 2 : op->bstl - 3;
    *u = op->wind ? op->stl : op->bstl - 1;
    if (!data) return DEO_OK;
    const long N = op->len, rows = *l + *u + 1;
    std::vector<double> M((size_t)N * (N + 2));
    deo_status s = deo_operator_array(op, M.data());
    if (s != DEO_OK) return s;
    std::fill(data, data + rows * (N + 2), 0.0);
    for (long j = 1; j <= N + 2; ++j)
        for (long i = 1; i <= N; ++i) {
            const double v = M[(size_t)(j - 1) * N + (i - 1)];
            const long b = *u + i - j;  // band row of entry (i, j)
            if (b >= 0 && b < rows) data[(size_t)(j - 1) * rows + b] = v;
            else if (v != 0.0)
                return fail(DEO_ERR_BAD_SHAPE, "entry (%ld, %ld) of Array(L) lies outside the bands (%d, %d)", i, j,
                            *l, *u);
        }
    return DEO_OK;
}

// ---------------------------------------------------------------------------
// Row-table compiler.  build_row() resolves, for output row i, which branch
// of the reference's convolve_* loops runs and returns its window and
// weights W[k] = coefficient * stencil[k] (the reference's first product).
//   mode 1: BoundaryPaddedVector methods (convolutions.jl:367-730)
//   mode 0: generic AbstractVector methods (convolutions.jl:27-362)
//   scaled: W = c*s with the operator's own coefficients; otherwise the
//           weights are left unscaled (a coefficient field multiplies them on
//           the device) and `sgn` (+1 / -1) stands in for the coefficient in
//           the sign tests.
// ---------------------------------------------------------------------------
struct RowSpec {
    int p0, nk, cidx;
    double w[DEO_MAX_NW];
};

static void row_fill(RowSpec& r, int p0, int nk, int cidx, double c, const double* s, double sg = 1.0,
                     bool reversed = false) {
    r.p0 = p0; r.nk = nk; r.cidx = cidx;
    for (int k = 0; k < nk; ++k) {
        double sk = reversed ? sg * s[nk - 1 - k] : s[k];
        r.w[k] = c * sk;
    }
}

// Row i of operator A as a (p0, nk, cidx, weights) record.  mode 1: the
// BoundaryPaddedVector methods; 0: the generic AbstractVector methods; 2: the
// vector-calculus methods (centred: coefficients[i] on every row).
static RowSpec build_row(const deo_operator& A, int mode, bool scaled, double sgn, long i) {
    RowSpec r;
    const long len = A.len;
    const int stl = A.stl, bstl = A.bstl, bpc = A.bpc, off = A.off;
    auto coef = [&](long pos) { return scaled ? A.coeff[pos - 1] : sgn; };
    auto mult = [&](long pos) { return scaled ? A.coeff[pos - 1] : 1.0; };
    if (!A.wind) {
        if (i <= bpc) {
            row_fill(r, 1, bstl, (int)i, mult(i), A.Lo((int)i - 1));
        } else if (i <= len - bpc) {
            const long ci = (mode == 1) ? i - bpc : i;
            const double* s = A.uniform ? A.S(0) : A.S((int)(i - bpc - 1));
            row_fill(r, (int)(i + 1 - stl / 2), stl, (int)ci, mult(ci), s);
        } else {
            const long rr = i - (len - bpc);
            // generic right rows read coeff[1:bpc] (convolutions.jl:109); the padded
            // methods and the vector-calculus methods (mode 2) read coeff[i]
            const long ci = (mode == 0) ? rr : i;
            row_fill(r, (int)(len + 3 - bstl), bstl, (int)ci, mult(ci), A.Hi((int)rr - 1));
        }
        return r;
    }
    const double sg = (A.d % 2 == 0) ? 1.0 : -1.0;
    const double c = coef(i), m = mult(i);
    if (A.uniform) {
        const double* S = A.S(0);
        if (i <= bpc) {
            if (c >= 0 && i + stl <= len + 2 && i >= off) row_fill(r, (int)(i + 1 - off), stl, (int)i, m, S);
            else row_fill(r, 1, bstl, (int)i, m, A.Lo((int)i - 1));
        } else if (i <= len - bpc - off) {
            if (c >= 0) row_fill(r, (int)(i + 1 - off), stl, (int)i, m, S);
            else row_fill(r, (int)(i - stl + 2 + off), stl, (int)i, m, S, sg, true);
        } else {
            const long q = i - (len - bpc - off);
            if (c < 0 && len + 2 - stl - bpc + q >= 1 && q <= bpc + 1)
                row_fill(r, (int)(len + 2 - stl - bpc + q), stl, (int)i, m, S, sg, true);
            else if (c < 0 && len + 2 - stl - bpc + q >= 1 && q > bpc + 1)
                row_fill(r, (int)(len + 3 - bstl), bstl, (int)i, m, A.Hi((int)(bpc + off + 1 - q - 1)), sg, true);
            else if (c >= 0 && q < off + 1)
                row_fill(r, (int)(len + 3 - stl + q - off), stl, (int)i, m, S);
            else
                row_fill(r, (int)(len + 3 - bstl), bstl, (int)i, m, A.Hi((int)q - 1));
        }
        return r;
    }
    // non-uniform upwind
    if (i <= bpc) {
        if (c >= 0 && off == 0) row_fill(r, (int)(i + 1), stl, (int)i, m, A.Lo((int)i - 1, 0));
        else if (c >= 0 && i < off) row_fill(r, 1, stl, (int)i, m, A.Lo((int)i - 1, 0));
        else if (c >= 0 && i >= off) row_fill(r, (int)(i + 1 - off), stl, (int)i, m, A.Lo((int)i - 1, 0));
        else row_fill(r, 1, bstl, (int)i, m, A.Lo((int)i - 1, 1));
    } else if (i <= len - bpc - off) {
        int half;
        if (mode == 0 && scaled && A.cfs > 0) half = 0;        // convolutions.jl:234-243
        else if (mode == 0 && scaled && A.cfs < 0) half = 1;   // convolutions.jl:244-253
        else half = (c >= 0) ? 0 : 1;
        if (half == 0) row_fill(r, (int)(i + 1 - off), stl, (int)i, m, A.S((int)(i - bpc - 1), 0));
        else row_fill(r, (int)(i - stl + 2 + off), stl, (int)i, m, A.S((int)(i - bpc - 1), 1));
    } else {
        const int hr = (int)(i - len + bpc + off);
        if (c < 0) {
            const int p0 = (i <= len - off) ? (int)(i - stl + 2 + off) : (int)(len - stl + 3);
            row_fill(r, p0, stl, (int)i, m, A.Hi(hr - 1, 1));
        } else if (i <= len - bpc) {
            row_fill(r, (int)(i - stl + 2 + off), stl, (int)i, m, A.S((int)(i - bpc - 1), 0));
        } else {
            row_fill(r, (int)(len - bstl + 3), bstl, (int)i, m, A.Hi(hr - 1, 0));
        }
    }
    return r;
}

static bool same_shape(const RowSpec& a, long ia, const RowSpec& b, long ib) {
    if (a.nk != b.nk || a.p0 - ia != b.p0 - ib || a.cidx - ia != b.cidx - ib) return false;
    for (int k = 0; k < a.nk; ++k)
        if (std::memcmp(&a.w[k], &b.w[k], sizeof(double)) != 0) return false;
    return true;
}

struct HostTab {
    RowTabDev dev{};
    std::vector<int> p0, nk, cidx;
    std::vector<double> W;  // [nw][nexp]
};

// The table of rows i = 1..len given by `row(i)`.
template <typename Row>
static deo_status compile_rows(long len, Row row, HostTab& T, std::vector<int>& rlo, std::vector<int>& rhi) {
    // pass 1: longest run of identical rows -> band
    long best_lo = 1, best_len = 0, run_lo = 1;
    RowSpec prev = row(1);
    for (long i = 1; i <= len; ++i) {
        RowSpec cur = (i == 1) ? prev : row(i);
        if (cur.p0 < 1 || cur.p0 + cur.nk - 1 > len + 2 || cur.nk < 1)
            return fail(DEO_ERR_BAD_SHAPE, "row %ld of the operator reads outside the padded line (len %ld too short)",
                        i, len);
        for (int p = cur.p0; p < cur.p0 + cur.nk; ++p) {
            rlo[p - 1] = std::min(rlo[p - 1], (int)i);
            rhi[p - 1] = std::max(rhi[p - 1], (int)i);
        }
        if (i > 1 && !same_shape(prev, i - 1, cur, i)) run_lo = i;
        if (i - run_lo + 1 > best_len) {
            best_len = i - run_lo + 1;
            best_lo = run_lo;
        }
        prev = cur;
    }
    RowTabDev& d = T.dev;
    if (best_len >= 2) {
        d.ilo = (int)best_lo;
        d.ihi = (int)(best_lo + best_len - 1);
        RowSpec b = row(best_lo);
        d.band_p0_off = (int)(b.p0 - best_lo);
        d.band_cidx_off = (int)(b.cidx - best_lo);
        d.band_nk = b.nk;
        for (int k = 0; k < b.nk; ++k) d.wband[k] = b.w[k];
    } else {
        d.ilo = (int)len + 1;
        d.ihi = (int)len;
    }
    // pass 2: explicit rows
    int nw = 1;
    std::vector<RowSpec> ex;
    for (long i = 1; i <= len; ++i) {
        if (i >= d.ilo && i <= d.ihi) continue;
        ex.push_back(row(i));
        nw = std::max(nw, ex.back().nk);
    }
    d.nexp = (int)ex.size();
    d.nw = nw;
    T.p0.resize(ex.size()); T.nk.resize(ex.size()); T.cidx.resize(ex.size());
    T.W.assign((size_t)nw * ex.size(), 0.0);
    for (size_t e = 0; e < ex.size(); ++e) {
        T.p0[e] = ex[e].p0; T.nk[e] = ex[e].nk; T.cidx[e] = ex[e].cidx;
        for (int k = 0; k < ex[e].nk; ++k) T.W[(size_t)k * ex.size() + e] = ex[e].w[k];
    }
    return DEO_OK;
}

static deo_status compile_table(const deo_operator& A, int mode, bool scaled, double sgn, HostTab& T,
                                std::vector<int>& rlo, std::vector<int>& rhi) {
    return compile_rows(A.len, [&](long i) { return build_row(A, mode, scaled, sgn, i); }, T, rlo, rhi);
}

// Row i of a sum of terms on one axis with one boundary condition: the
// union of their windows, the weights of each padded position added in the
// terms' order (a position a term does not read contributes nothing).
// nk = 0 when the union is wider than DEO_MAX_NW.
static RowSpec merge_row(const RowSpec& a, const RowSpec& b) {
    RowSpec r;
    r.p0 = std::min(a.p0, b.p0);
    const int end = std::max(a.p0 + a.nk, b.p0 + b.nk);
    r.nk = end - r.p0;
    r.cidx = a.cidx;
    if (r.nk > DEO_MAX_NW) {
        r.nk = 0;
        return r;
    }
    for (int k = 0; k < r.nk; ++k) {
        const int p = r.p0 + k;
        const bool ia = p >= a.p0 && p < a.p0 + a.nk, ib = p >= b.p0 && p < b.p0 + b.nk;
        r.w[k] = ia && ib ? a.w[p - a.p0] + b.w[p - b.p0] : (ia ? a.w[p - a.p0] : b.w[p - b.p0]);
    }
    return r;
}

// ---------------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------------
using deo::make_fastdiv;

extern "C" int deo_fastdiv_probe(uint32_t n, uint32_t d) {  // host check of the constants (tests)
    const deo::FastDiv f = make_fastdiv(d);
    const uint32_t t = (uint32_t)(((unsigned long long)n * f.mul) >> 32);
    return (int)((t + n) >> f.shr);
}
// Unit counters of the dynamically scheduled interior kernels, used in
// rotation: applies of one plan in flight at the same time on different
// streams each need their own (up to kSchedSlots of them).
constexpr unsigned int kSchedSlots = 1024;
// DEO_OPT_FX_FP64_ROWS default: rows of each 32 x 8 tile of the fixed-point
// kernel evaluated in the reference's FP64 order (FP64 pipe) beside the
// integer-pipe rows
constexpr int kFxFp64Rows = 2;

struct deo_plan {
    PlanDev dev{};
    deo::UniPlan uni{};
    deo::ShellPlan shell{};
    int fast_path = 1;   // DEO_OPT_FAST_PATH
    int use_tma = 1;     // DEO_OPT_TMA
    int exact_sums = 1;  // DEO_OPT_EXACT_SUMS
    int timing = 0;      // DEO_OPT_LAUNCH_TIMING
    int concurrent = 1;  // DEO_OPT_CONCURRENT_SHELL
    // the last deo_plan_autotune: per candidate (f32_vec, vcfg, shell kernel, concurrent) its best ms
    std::vector<int> tune_cands;
    std::vector<float> tune_ms;
    PlanDev* d_plan = nullptr;  // device copy (batched kernel)
    deo::ShellPlan* d_shell = nullptr;  // device copy of `shell` when shell.ok
    // concurrent shell: a side stream, fork/join events and the interior kernel's unit counter
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    unsigned int* d_sched = nullptr;  // kSchedSlots unit counters, one per apply in rotation
    mutable std::atomic<unsigned int> sched_slot{0};
    mutable std::mutex apply_mu;  // one fork/join sequence at a time per plan
    std::vector<void*> allocs;
    size_t table_bytes = 0;
    void* stage_u = nullptr;
    void* stage_du = nullptr;
    // pipelined host applies: two staging slots, copy-in / copy-out streams and their events
    struct HostPipe {
        void* u[2] = {nullptr, nullptr};
        void* du[2] = {nullptr, nullptr};
        cudaStream_t in = nullptr, out = nullptr;
        cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_comp[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr};
        unsigned next = 0;
    } pipe;
    std::mutex pipe_mu;
    // kernels launched by the last forward apply (diagnostics; last writer wins)
    // transposed applies on the TMA path: the box of columns read only by band rows of every axis
    // (1-based, per term), where the transpose is the band itself (symmetric bands)
    int adj_ok = 0;
    int adj_lo[3] = {0, 0, 0}, adj_hi[3] = {0, 0, 0};  // (the transpose there: the band, taps reversed)
    mutable std::atomic<const char*> last_kernel{""};
    mutable std::atomic<const char*> last_kernel2{""};
    // launch timing: events around each launch of the last forward apply
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    mutable int ev_launches = 0;
    ~deo_plan() {
        for (void* p : allocs) cudaFree(p);
        if (d_plan) cudaFree(d_plan);
        if (d_shell) cudaFree(d_shell);
        if (d_sched) cudaFree(d_sched);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (side) cudaStreamDestroy(side);
        if (stage_u) cudaFree(stage_u);
        if (stage_du) cudaFree(stage_du);
        for (int k = 0; k < 2; ++k) {
            if (pipe.u[k]) cudaFree(pipe.u[k]);
            if (pipe.du[k]) cudaFree(pipe.du[k]);
            for (cudaEvent_t e : {pipe.ev_in[k], pipe.ev_comp[k], pipe.ev_out[k]})
                if (e) cudaEventDestroy(e);
        }
        if (pipe.in) cudaStreamDestroy(pipe.in);
        if (pipe.out) cudaStreamDestroy(pipe.out);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
};

template <class V>
static deo_status upload(deo_plan& P, const V& v, const void** dst) {
    if (v.empty()) {
        *dst = nullptr;
        return DEO_OK;
    }
    void* p = nullptr;
    const size_t bytes = v.size() * sizeof(v[0]);
    CUDA_TRY(cudaMalloc(&p, bytes), "cudaMalloc(plan table)");
    P.allocs.push_back(p);
    CUDA_TRY(cudaMemcpy(p, v.data(), bytes, cudaMemcpyHostToDevice), "cudaMemcpy(plan table)");
    P.table_bytes += bytes;
    *dst = p;
    return DEO_OK;
}

static deo_status upload_tab(deo_plan& P, HostTab& T, int dtype, RowTabDev& out) {
    out = T.dev;
    deo_status s;
    if ((s = upload(P, T.p0, reinterpret_cast<const void**>(&out.p0))) != DEO_OK) return s;
    if ((s = upload(P, T.nk, reinterpret_cast<const void**>(&out.nk))) != DEO_OK) return s;
    if ((s = upload(P, T.cidx, reinterpret_cast<const void**>(&out.cidx))) != DEO_OK) return s;
    if (dtype == DEO_F64) {
        if ((s = upload(P, T.W, &out.W)) != DEO_OK) return s;
    } else {
        std::vector<float> wf(T.W.begin(), T.W.end());
        if ((s = upload(P, wf, &out.W)) != DEO_OK) return s;
        float* fb = reinterpret_cast<float*>(out.wband);
        double tmp[DEO_MAX_NW];
        std::memcpy(tmp, T.dev.wband, sizeof tmp);
        std::memset(out.wband, 0, sizeof out.wband);
        for (int k = 0; k < DEO_MAX_NW; ++k) fb[k] = (float)tmp[k];
    }
    return DEO_OK;
}

// The rows of term t outside its interior range [flo, fhi] (the range the
// tiled kernels evaluate; same formulas as the UniPlan setup), copied from its
// row table for the shell kernel.  Marks sp.ok = -1 if they do not fit.
// n values into dst as the plan dtype's values: doubles, or floats packed
// from the start of dst (the layout the shell kernel reads).
static void pack_values(const double* src, double* dst, int n, int dtype) {
    double tmp[DEO_MAX_NW > DEO_MAX_BCW ? DEO_MAX_NW : DEO_MAX_BCW];
    std::memcpy(tmp, src, sizeof(double) * n);
    std::memset(dst, 0, sizeof(double) * n);
    for (int k = 0; k < n; ++k) {
        if (dtype == DEO_F64) dst[k] = tmp[k];
        else reinterpret_cast<float*>(dst)[k] = (float)tmp[k];
    }
}

static void shell_rows(const HostTab& H, int len, int dtype, int t, deo::ShellPlan& sp) {
    if (t >= 3) return;
    const RowTabDev& d = H.dev;
    int flo = std::max(d.ilo, 2 - d.band_p0_off);
    int fhi = std::min(d.ihi, len + 2 - d.band_nk - d.band_p0_off);
    if (d.ilo > d.ihi || flo > fhi) { flo = 1; fhi = 0; }
    deo::ShellTerm& S = sp.t[t];
    S.len = len;
    S.nlo = flo > fhi ? len : flo - 1;
    S.nhi = flo > fhi ? 0 : len - fhi;
    if (S.nlo > DEO_SHELL_ROWS || S.nhi > DEO_SHELL_ROWS) {
        sp.ok = -1;
        return;
    }
    auto put = [&](int slot, int i) {
        deo::ShellRow& R = S.row[slot];
        const bool band = i >= d.ilo && i <= d.ihi;
        const int e = band ? 0 : (i < d.ilo ? i - 1 : (d.ilo - 1) + (i - d.ihi - 1));
        R.p0 = band ? i + d.band_p0_off : H.p0[e];
        R.nk = band ? d.band_nk : H.nk[e];
        double w[DEO_MAX_NW];
        for (int k = 0; k < DEO_MAX_NW; ++k)
            w[k] = k >= R.nk ? 0.0 : (band ? d.wband[k] : H.W[(size_t)k * d.nexp + e]);
        pack_values(w, R.w, DEO_MAX_NW, dtype);
        sp.maxw = std::max(sp.maxw, R.nk);
    };
    for (int r = 0; r < S.nlo; ++r) put(r, r + 1);
    for (int r = 0; r < S.nhi; ++r) put(S.nlo + r, len - S.nhi + 1 + r);
    // the points of the line each end's rows read (ghost maps added with the BC)
    S.wlo = S.whi = 0;
    for (int r = 0; r < S.nlo; ++r) S.wlo = std::max(S.wlo, S.row[r].p0 + S.row[r].nk - 2);
    for (int r = 0; r < S.nhi; ++r) S.whi = std::max(S.whi, len + 2 - S.row[S.nlo + r].p0);
    S.wlo = std::min(S.wlo, len);
    S.whi = std::min(S.whi, len);
}

// The fixed-point kernel's weights: the shared band w[0..2H] as integers on
// one exponent f (w[k] = W[k] * 2^f exactly).  Accepted only if (a) every
// integer image fits 62 bits and the 2H+1 products with NT-tap sums (each
// below NT * 2^(53+S)) cannot overflow a signed 128-bit accumulator, and (b)
// ratio = NT * sum|w| / min|w| <= 256, which bounds the alignment error of the
// kernel by ratio * 2^(1-S) <= 2 ulp of sum|c_k u_k|.
static bool fx_weights(const double* w, int H, int nt, long long* W, int& f) {
    const int S = nt == 3 ? 8 : 9;
    long long M[DEO_MAX_NW];
    int fk[DEO_MAX_NW];
    int fmin = INT_MAX, fmax = INT_MIN;
    double sum = 0.0, wmin = INFINITY;
    for (int k = 0; k < 2 * H + 1; ++k) {
        if (std::fpclassify(w[k]) != FP_NORMAL) return false;
        int ex = 0;
        const double fr = std::frexp(std::fabs(w[k]), &ex);  // |w| = fr * 2^ex, fr in [0.5, 1)
        M[k] = (long long)std::ldexp(fr, 53);                  // exact 53-bit integer
        fk[k] = ex - 53;
        fmin = std::min(fmin, fk[k]);
        fmax = std::max(fmax, fk[k]);
        sum += std::fabs(w[k]);
        wmin = std::min(wmin, std::fabs(w[k]));
    }
    const int bits = 53 + (fmax - fmin);
    int lg = 0;
    while ((1 << lg) < (2 * H + 1) * nt) ++lg;
    if (bits > 62 || bits + 53 + S + lg > 127) return false;
    if (nt * sum / wmin > 256.0) return false;
    for (int k = 0; k < 2 * H + 1; ++k) W[k] = (w[k] < 0 ? -1 : 1) * (M[k] << (fk[k] - fmin));
    f = fmin;
    return true;
}

// Block fixed point (k_lap_bfx, three axes sharing the band w[0..2H]): the
// weights' exact integer images W[k] on one exponent f (w[k] = W[k] * 2^f),
// the merged centre 3 W[H], and the centre threshold.  Values carry G0 = 7
// bits below their 53-bit mantissas; each group of the 3 neighbours at one
// offset then carries less than 4 units of truncation, so the kernel's error
// is below (4/3) r 2^(Tc - G0 + 1) ulp of sum|c_k u_k| (r = sum_{k != H} |w_k|
// / |w_H|) when the centre value is at least 2^-Tc of the plane tile's largest
// binade; Tc is the largest value keeping that bound at 2 ulp (at most G0, so
// that the centre itself is exact).  The centre test is |m_0| >= 2^tshift
// units, tshift = 53 + G0 - 1 - Tc.  The kernel folds each weight's sign into
// its group sum S (|S| < 3 * 2^60), adds 2^62, splits that at bit 31 and |W|
// at bit 29, and accumulates the four unsigned 32 x 32-bit partial products
// in uint64 columns: false when one could overflow, when the band's signs do
// not alternate from the centre, when a weight is zero or not normal, or when
// the images need more than 58 bits.
static bool bfx_weights(const double* w, int H, deo::UniPlan& U) {
    constexpr int G0 = 7;
    const int K = 2 * H + 1;
    long long M[DEO_MAX_NW];
    int fk[DEO_MAX_NW];
    int fmin = INT_MAX, fmax = INT_MIN;
    for (int k = 0; k < K; ++k) {
        if (std::fpclassify(w[k]) != FP_NORMAL) return false;
        int ex = 0;
        const double fr = std::frexp(std::fabs(w[k]), &ex);
        M[k] = (long long)std::ldexp(fr, 53);
        fk[k] = ex - 53;
        fmin = std::min(fmin, fk[k]);
        fmax = std::max(fmax, fk[k]);
    }
    if (53 + (fmax - fmin) > 58) return false;  // 3 W[H] < 2^60 as well
    long double all = 0.0L;
    for (int k = 0; k < K; ++k) {
        U.bfx_w[k] = (w[k] < 0 ? -1 : 1) * (M[k] << (fk[k] - fmin));
        if (k != H) all += std::fabs((long double)w[k]);
    }
    U.bfx_c0 = 3 * U.bfx_w[H];
    // signs alternating from the centre (every centred even-derivative band)
    const bool cneg = w[H] < 0;
    for (int k = 0; k < K; ++k)
        if ((w[k] < 0) != (cneg != (((k - H) & 1) != 0))) return false;
    // column bounds: S' = sgn(W) S + 2^62 = s1 2^31 + s0 (|S| < 3 2^60), |W| = w1 2^29 + w0
    unsigned __int128 c0 = 0, c31 = 0, c29 = 0, c60 = 0, ksum = 0;
    const unsigned __int128 s0max = (1u << 31) - 1;
    const unsigned __int128 s1max = (((unsigned __int128)1 << 62) + 3 * ((unsigned __int128)1 << 60)) >> 31;
    for (int k = 0; k < K; ++k) {
        const long long W = k == H ? U.bfx_c0 : U.bfx_w[k];
        const unsigned __int128 aw = (unsigned __int128)(W < 0 ? -W : W);
        const unsigned __int128 w0 = aw & 0x1FFFFFFFu, w1 = aw >> 29;
        c0 += s0max * w0;
        c31 += s1max * w0;
        c29 += s0max * w1;
        c60 += s1max * w1;
        ksum += aw;
    }
    const unsigned __int128 lim = ~(unsigned __int128)0 >> 64;  // 2^64 - 1
    if (c0 > lim || c31 > lim || c29 > lim || c60 > lim) return false;
    const long double per = (4.0L / 3.0L) * (all / std::fabs((long double)w[H])) * std::ldexp(1.0L, 1 - G0);
    int Tc = G0;
    while (Tc >= 0 && per * std::ldexp(1.0L, Tc) > 2.0L) --Tc;
    if (Tc < 0) return false;
    const unsigned __int128 kk = ksum << 62;
    U.bfx_k_lo = (unsigned long long)kk;
    U.bfx_k_hi = (unsigned long long)(kk >> 64);
    U.bfx_cneg = cneg ? 1 : 0;
    U.bfx_f = fmin;
    U.bfx_tshift = 53 + G0 - 1 - Tc;
    return true;
}

static bool same_bc(const deo_bc& a, const deo_bc& b) {
    if (a.kind != b.kind) return false;
    if (a.kind == DEO_BC_PERIODIC) return true;
    if (a.m_l != b.m_l || a.m_r != b.m_r || a.b_l != b.b_l || a.b_r != b.b_r) return false;
    for (int j = 0; j < a.m_l; ++j)
        if (a.a_l[j] != b.a_l[j]) return false;
    for (int j = 0; j < a.m_r; ++j)
        if (a.a_r[j] != b.a_r[j]) return false;
    return true;
}

extern "C" deo_status deo_plan_create(int ndims, const int64_t* sizes, deo_dtype dtype, int nterms,
                                      const deo_term* terms, deo_plan** out) {
    return deo_plan_create_opts(ndims, sizes, dtype, nterms, terms, 0, out);
}

extern "C" deo_status deo_plan_create_opts(int ndims, const int64_t* sizes, deo_dtype dtype, int nterms,
                                           const deo_term* terms, int flags, deo_plan** out) {
    if (!out || !sizes || !terms) return fail(DEO_ERR_BAD_ARG, "null argument");
    *out = nullptr;
    if (ndims < 1 || ndims > DEO_MAX_DIMS) return fail(DEO_ERR_BAD_SHAPE, "ndims must be 1..%d", DEO_MAX_DIMS);
    if (nterms < 1 || nterms > DEO_MAX_TERMS) return fail(DEO_ERR_BAD_ARG, "nterms must be 1..%d", DEO_MAX_TERMS);
    if (dtype != DEO_F64 && dtype != DEO_F32) return fail(DEO_ERR_BAD_ARG, "unknown dtype");
    auto P = std::make_unique<deo_plan>();
    PlanDev& D = P->dev;
    D.ndims = ndims;
    D.nterms = nterms;
    D.dtype = dtype;
    int64_t total = 1;
    for (int k = 0; k < ndims; ++k) {
        if (sizes[k] < 1) return fail(DEO_ERR_BAD_SHAPE, "size(u, %d) = %lld", k + 1, (long long)sizes[k]);
        D.sizes[k] = sizes[k];
        total *= sizes[k];
    }
    D.total = total;
    D.fastdiv = total < (1LL << 31) ? 1 : 0;
    // DEO_PLAN_MERGE_TERMS: a term on the same axis as an earlier one, with the same boundary condition
    // and path, no coefficient field and no per-line BCs, joins it (lead[t] = that term) when every
    // row's union window fits DEO_MAX_NW taps; the plan then has fewer terms
    std::vector<int> lead(nterms, -1), eff(nterms, 0);
    if (flags & DEO_PLAN_MERGE_TERMS) {
        auto joinable = [&](const deo_term& a, const deo_term& b) {
            if (!a.op || !b.op || !a.bc || !b.bc || a.line_bcs || b.line_bcs || a.coeff_field || b.coeff_field)
                return false;
            if (a.axis != b.axis || a.path != b.path || a.op->len != b.op->len || !same_bc(*a.bc, *b.bc)) return false;
            const int md = a.path == DEO_PATH_PADDED ? 1 : a.path == DEO_PATH_GENERIC ? 0 : (ndims == 1 ? 1 : 0);
            for (long i = 1; i <= a.op->len; ++i) {
                const RowSpec ra = build_row(*a.op, md, true, 1.0, i), rb = build_row(*b.op, md, true, 1.0, i);
                if (ra.nk < 1 || rb.nk < 1 || merge_row(ra, rb).nk < 1) return false;
            }
            return true;
        };
        for (int t = 1; t < nterms; ++t)
            for (int s = 0; s < t; ++s) {
                if (lead[s] >= 0) continue;
                // the union of every member so far must stay within DEO_MAX_NW: check against each
                bool ok = joinable(terms[s], terms[t]);
                for (int m = s + 1; m < t && ok; ++m)
                    if (lead[m] == s) ok = joinable(terms[m], terms[t]);
                if (ok) {
                    lead[t] = s;
                    break;
                }
            }
    }
    {
        int ne = 0;
        for (int t = 0; t < nterms; ++t) eff[t] = lead[t] < 0 ? ne++ : eff[lead[t]];
        D.nterms = ne;
    }
    for (int t = 0; t < nterms; ++t) {
        const deo_term& tm = terms[t];
        if (tm.path < DEO_PATH_AUTO || tm.path > DEO_PATH_GENERIC)
            return fail(DEO_ERR_BAD_ARG, "term %d: unknown path %d", t + 1, tm.path);
        const int mode = tm.path == DEO_PATH_PADDED ? 1 : tm.path == DEO_PATH_GENERIC ? 0 : (ndims == 1 ? 1 : 0);
        if (!tm.op || (!tm.bc && !tm.line_bcs))
            return fail(DEO_ERR_BAD_ARG, "term %d: null operator or boundary condition", t + 1);
        const deo_operator& A = *tm.op;
        const int ax = tm.axis - 1;
        if (ax < 0 || ax >= ndims) return fail(DEO_ERR_BAD_SHAPE, "term %d: axis %d outside 1..%d", t + 1, tm.axis, ndims);
        if (sizes[ax] != A.len)
            return fail(DEO_ERR_BAD_SHAPE, "term %d: size(u, %d) = %lld but the operator has len %d", t + 1, tm.axis,
                        (long long)sizes[ax], A.len);
        auto bad_bc = [&](const deo_bc& b) {
            if (b.kind != DEO_BC_AFFINE && b.kind != DEO_BC_PERIODIC) return true;
            return b.kind == DEO_BC_AFFINE && (b.m_l < 0 || b.m_r < 0 || b.m_l > DEO_MAX_BC || b.m_r > DEO_MAX_BC ||
                                               b.m_l > A.len || b.m_r > A.len);
        };
        // one BC per line (MultiDimBC{dim}(BCs::Array)): an array of periodic BCs pads with the edge
        // planes like PeriodicBC; an array of one affine map is that map on every line; otherwise
        // every line reads its own ghost map (no fast path)
        const deo_bc* qp = tm.bc;
        std::vector<double> lrec;
        int lmw = 0;
        if (tm.line_bcs) {
            const deo_bc* lb = tm.line_bcs;
            const int64_t nlines = total / A.len;
            bool all_per = true, all_same = true;
            auto same_map = [](const deo_bc& a, const deo_bc& b) {
                if (a.kind != b.kind) return false;
                if (a.kind == DEO_BC_PERIODIC) return true;
                if (a.m_l != b.m_l || a.m_r != b.m_r || a.b_l != b.b_l || a.b_r != b.b_r) return false;
                for (int j = 0; j < a.m_l; ++j) if (a.a_l[j] != b.a_l[j]) return false;
                for (int j = 0; j < a.m_r; ++j) if (a.a_r[j] != b.a_r[j]) return false;
                return true;
            };
            for (int64_t l = 0; l < nlines; ++l) {
                if (bad_bc(lb[l]))
                    return fail(DEO_ERR_BAD_SHAPE, "term %d: line %lld: unknown BC or boundary stencil longer than the line",
                                t + 1, (long long)l + 1);
                all_per = all_per && lb[l].kind == DEO_BC_PERIODIC;
                all_same = all_same && same_map(lb[0], lb[l]);
                if (lb[l].kind == DEO_BC_AFFINE) lmw = std::max(lmw, std::max(lb[l].m_l, lb[l].m_r));
            }
            if (all_per || all_same || ndims == 1) {
                qp = &lb[0];
            } else {
                qp = nullptr;
                lmw = std::max(lmw, 1);
                const int rs = 5 + 2 * lmw;
                lrec.assign((size_t)(nlines * rs), 0.0);
                for (int64_t l = 0; l < nlines; ++l) {
                    double* r = lrec.data() + l * rs;
                    const deo_bc& b = lb[l];
                    r[0] = b.kind == DEO_BC_PERIODIC ? 1.0 : 0.0;
                    if (b.kind == DEO_BC_AFFINE) {
                        r[1] = b.m_l;
                        r[2] = b.m_r;
                        r[3] = b.b_l;
                        r[4] = b.b_r;
                        for (int j = 0; j < b.m_l; ++j) r[5 + j] = b.a_l[j];
                        for (int j = 0; j < b.m_r; ++j) r[5 + lmw + j] = b.a_r[j];
                    }
                }
            }
        }
        static const deo_bc kNoBC{};
        const deo_bc& q = qp ? *qp : kNoBC;
        if (qp && bad_bc(q)) return fail(DEO_ERR_BAD_SHAPE, "term %d: boundary stencil longer than the line", t + 1);
        if (!A.wind && A.len < 2 * A.bpc + 1)
            return fail(DEO_ERR_BAD_SHAPE, "term %d: len %d < 2*boundary_point_count+1", t + 1, A.len);
        if (A.wind && A.len < 2 * A.bpc + A.off)
            return fail(DEO_ERR_BAD_SHAPE, "term %d: len %d too short for the upwind boundary rows", t + 1, A.len);
        if (lead[t] >= 0) continue;  // joined an earlier term (its rows are in that term's table)
        TermDev& T = D.t[eff[t]];
        T.axis = ax;
        T.len = A.len;
        int64_t stride = 1;
        for (int k = 0; k < ax; ++k) stride *= sizes[k];
        T.stride = stride;
        if (total < (1LL << 31)) {
            T.div_stride = make_fastdiv((uint32_t)stride);
            T.div_len = make_fastdiv((uint32_t)A.len);
        }
        T.has_field = tm.coeff_field != nullptr ? ((flags & DEO_PLAN_FACTOR_FIELD) ? 2 : 1) : 0;
        T.field = tm.coeff_field;
        T.nvar = (T.has_field && A.wind) ? 2 : 1;
        std::vector<int> rlo(A.len + 2, A.len + 1), rhi(A.len + 2, 0);
        std::vector<const deo_operator*> members{&A};
        for (int m = t + 1; m < nterms; ++m)
            if (lead[m] == t) members.push_back(terms[m].op);
        for (int v = 0; v < T.nvar; ++v) {
            HostTab H;
            deo_status s;
            if (members.size() == 1) {
                s = compile_table(A, mode, !T.has_field, v == 0 ? 1.0 : -1.0, H, rlo, rhi);
            } else {
                s = compile_rows(A.len, [&](long i) {
                    RowSpec r = build_row(*members[0], mode, true, 1.0, i);
                    for (size_t m = 1; m < members.size(); ++m) r = merge_row(r, build_row(*members[m], mode, true, 1.0, i));
                    return r;
                }, H, rlo, rhi);
            }
            if (s != DEO_OK) return s;
            if (v == 0) shell_rows(H, A.len, dtype, eff[t], P->shell);
            if ((s = upload_tab(*P, H, dtype, T.tab[v])) != DEO_OK) return s;
        }
        for (int p = 0; p < A.len + 2; ++p)
            if (rhi[p] < rlo[p]) { rlo[p] = 1; rhi[p] = 0; }
        deo_status s;
        if ((s = upload(*P, rlo, reinterpret_cast<const void**>(&T.rlo))) != DEO_OK) return s;
        if ((s = upload(*P, rhi, reinterpret_cast<const void**>(&T.rhi))) != DEO_OK) return s;
        T.bc_kind = q.kind;
        T.periodic_nd = (q.kind == DEO_BC_PERIODIC && ndims > 1) ? 1 : 0;
        T.ml = q.kind == DEO_BC_AFFINE ? q.m_l : 0;
        T.mr = q.kind == DEO_BC_AFFINE ? q.m_r : 0;
        for (int k = 0; k < DEO_MAX_BC; ++k) { T.al[k] = q.a_l[k]; T.ar[k] = q.a_r[k]; }
        T.bl = q.b_l;
        T.br = q.b_r;
        T.lbc = nullptr;
        T.lbc_stride = 0;
        T.lbc_mw = 0;
        if (!lrec.empty()) {
            deo_status ls;
            if ((ls = upload(*P, lrec, reinterpret_cast<const void**>(&T.lbc))) != DEO_OK) return ls;
            T.lbc_stride = 5 + 2 * lmw;
            T.lbc_mw = lmw;
            D.has_lbc = 1;
        }
        if (eff[t] < 3) {
            deo::ShellTerm& S = P->shell.t[eff[t]];
            S.bc_kind = T.bc_kind;
            S.periodic_nd = T.periodic_nd;
            S.ml = T.ml;
            S.mr = T.mr;
            pack_values(T.al, S.al, DEO_MAX_BCW, dtype);
            pack_values(T.ar, S.ar, DEO_MAX_BCW, dtype);
            pack_values(&T.bl, &S.bl, 1, dtype);
            pack_values(&T.br, &S.br, 1, dtype);
            P->shell.maxw = std::max(P->shell.maxw, std::max(S.ml, S.mr));
            if (S.bc_kind == 1) {  // periodic: the ghost is an end point, of this end (N-D) or the other (1-D)
                S.wlo = std::max(S.wlo, S.periodic_nd ? 1 : S.len);
                S.whi = std::max(S.whi, S.periodic_nd ? 1 : S.len);
            } else {
                S.wlo = std::max(S.wlo, S.ml);
                S.whi = std::max(S.whi, S.mr);
            }
        }
    }
    P->shell.ok = P->shell.ok >= 0 && D.nterms <= 3 ? 1 : 0;
    // DEO_PLAN_STAR: every term a constant band (no coefficient field, no per-line BCs): one star of
    // taps for the points whose rows read no ghost along any axis, the centre taps merged (added in
    // the terms' order in Float64, rounded once to the plan's dtype)
    if (flags & DEO_PLAN_STAR) {
        deo::StarDev S{};
        bool ok = true;
        double centre = 0.0;
        bool have_centre = false;
        std::vector<std::pair<int64_t, double>> taps;
        for (int t = 0; t < D.nterms && ok; ++t) {
            const TermDev& T = D.t[t];
            const RowTabDev& tb = T.tab[0];
            ok = !T.has_field && T.nvar == 1 && !T.lbc && tb.ilo <= tb.ihi;
            if (!ok) break;
            const int flo = std::max(tb.ilo, 2 - tb.band_p0_off);
            const int fhi = std::min(tb.ihi, T.len + 2 - tb.band_nk - tb.band_p0_off);
            ok = flo <= fhi;
            S.lo[t] = flo;
            S.hi[t] = fhi;
            for (int k = 0; k < tb.band_nk && ok; ++k) {
                const double w = dtype == DEO_F64 ? tb.wband[k] : (double)reinterpret_cast<const float*>(tb.wband)[k];
                const int rel = tb.band_p0_off + k - 1;  // line position of tap k minus the point's
                if (rel == 0) {
                    centre = have_centre ? centre + w : w;
                    have_centre = true;
                } else {
                    taps.emplace_back((int64_t)rel * T.stride, w);
                }
            }
        }
        if (ok && (int)taps.size() + (have_centre ? 1 : 0) <= DEO_STAR_MAX) {
            if (have_centre) {
                S.off[S.n] = 0;
                S.w[S.n++] = dtype == DEO_F64 ? centre : (double)(float)centre;
            }
            for (const auto& tw : taps) {
                S.off[S.n] = tw.first;
                S.w[S.n++] = tw.second;
            }
            D.star = S;
        }
    }
    // fast path for 2-D/3-D plans whose terms all have constant interior rows
    {
        deo::UniPlan& U = P->uni;
        bool ok = (ndims == 2 || ndims == 3) && sizes[0] < (1LL << 30) && sizes[1] < (1LL << 30) &&
                  (ndims < 3 || sizes[2] < (1LL << 30));
        int H = 0;
        for (int t = 0; t < D.nterms && ok; ++t) {
            const TermDev& T = D.t[t];
            const RowTabDev& tb = T.tab[0];
            if (T.has_field || T.nvar != 1 || tb.ilo > tb.ihi || T.axis > 2 || T.lbc) {
                ok = false;
                break;
            }
            deo::UniTerm& u = U.t[t];
            u.axis = T.axis;
            u.nk = tb.band_nk;
            u.off0 = tb.band_p0_off - 1;
            u.flo = std::max(tb.ilo, 2 - tb.band_p0_off);
            u.fhi = std::min(tb.ihi, T.len + 2 - tb.band_nk - tb.band_p0_off);
            if (u.flo > u.fhi) { u.flo = 1; u.fhi = 0; }
            std::memcpy(u.w, tb.wband, sizeof u.w);  // already float-packed for Float32 plans
            H = std::max(H, std::max(std::abs(u.off0), std::abs(u.off0 + u.nk - 1)));
        }
        if (ok && H >= 1 && H <= 4) {
            U.enabled = 1;
            U.radius = H;
            U.nterms = D.nterms;
            // centred-band specialisation: term t on axis t, 2H+1 taps from -H
            U.lap = (D.nterms == ndims);
            for (int t = 0; t < D.nterms && U.lap; ++t)
                U.lap = U.t[t].axis == t && U.t[t].nk == 2 * H + 1 && U.t[t].off0 == -H;
            // exact neighbour sums: Float64, one band shared by every term
            U.ens = U.lap && dtype == DEO_F64;
            for (int t = 0; t < D.nterms && U.ens; ++t)
                U.ens = std::memcmp(U.t[t].w, U.t[0].w, sizeof(double) * (2 * H + 1)) == 0;
            for (int k = 0; k < 2 * H + 1 && U.ens; ++k)
                U.ens = k == H || std::fpclassify(U.t[0].w[k]) == FP_NORMAL;  // scaled through their exponents
            if (U.ens) {
                const double w0 = U.t[0].w[H];
                for (int mask = 0; mask < 8; ++mask) {
                    double c = 0.0;
                    for (int t = 0; t < 3; ++t)
                        if (mask & (1 << t)) c = c + w0;  // 2*w0 is exact, so 3*w0 rounds once
                    U.ens_c0[mask] = c;
                }
                for (int k = 0; k < 2 * H + 1; ++k) U.ens_w[k] = U.t[0].w[k];  // weight at offset k - H
            }
            // fixed-point evaluation: the same shared band, as exact integers on one exponent
            U.fx = U.lap && dtype == DEO_F64 && H <= 3 && (D.nterms == 2 || D.nterms == 3);
            for (int t = 0; t < D.nterms && U.fx; ++t)
                U.fx = std::memcmp(U.t[t].w, U.t[0].w, sizeof(double) * (2 * H + 1)) == 0;
            if (U.fx) U.fx = fx_weights(U.t[0].w, H, D.nterms, U.fx_w, U.fx_f);
            U.fx_rows = kFxFp64Rows;
            U.f32_vec = 1;
            // block fixed point: three axes sharing one band
            U.bfx = U.lap && dtype == DEO_F64 && H <= 3 && D.nterms == 3;
            for (int t = 0; t < D.nterms && U.bfx; ++t)
                U.bfx = std::memcmp(U.t[t].w, U.t[0].w, sizeof(double) * (2 * H + 1)) == 0;
            if (U.bfx) U.bfx = bfx_weights(U.t[0].w, H, U);
            for (int k = 0; k < 3; ++k) U.n[k] = k < ndims ? sizes[k] : 1;
        } else {
            U.enabled = 0;
        }
    }
    CUDA_TRY(cudaMalloc(&P->d_plan, sizeof(PlanDev)), "cudaMalloc(plan)");
    CUDA_TRY(cudaMemcpy(P->d_plan, &P->dev, sizeof(PlanDev), cudaMemcpyHostToDevice), "cudaMemcpy(plan)");
    if (P->shell.ok && P->uni.enabled && P->uni.lap) {
        CUDA_TRY(cudaMalloc(&P->d_shell, sizeof(deo::ShellPlan)), "cudaMalloc(shell rows)");
        CUDA_TRY(cudaMemcpy(P->d_shell, &P->shell, sizeof(deo::ShellPlan), cudaMemcpyHostToDevice),
                 "cudaMemcpy(shell rows)");

        CUDA_TRY(cudaMalloc(&P->d_sched, kSchedSlots * sizeof(unsigned int)), "cudaMalloc(unit counters)");
        CUDA_TRY(cudaStreamCreateWithFlags(&P->side, cudaStreamNonBlocking), "cudaStreamCreate");
        // the transposed fast path: the box of columns along each axis read only by band rows:
        // [flo + H, fhi - H], clear of the points the boundary rows and the ghost maps read
        // (ShellTerm::wlo, whi; a boundary row may be wider than the band)
        {
            const deo::UniPlan& U = P->uni;
            const int H = U.radius;
            bool ok = U.nterms >= 2 && U.nterms <= 3;
            for (int a = 0; a < U.nterms && ok; ++a) {
                const deo::UniTerm& t = U.t[a];
                ok = t.nk == 2 * H + 1 && t.off0 == -H && t.axis == a;
                const TermDev& T = D.t[a];
                const deo::ShellTerm& S = P->shell.t[a];
                const int lo = std::max(t.flo + H, S.wlo + 1), hi = std::min(t.fhi - H, S.len - S.whi);
                ok = ok && lo <= hi && !T.lbc && S.len == T.len;
                P->adj_lo[a] = lo;
                P->adj_hi[a] = hi;
            }
            P->adj_ok = ok ? 1 : 0;
        }
        CUDA_TRY(cudaEventCreateWithFlags(&P->ev_fork, cudaEventDisableTiming), "cudaEventCreate");
        CUDA_TRY(cudaEventCreateWithFlags(&P->ev_join, cudaEventDisableTiming), "cudaEventCreate");
    }
    *out = P.release();
    return DEO_OK;
}

extern "C" void deo_plan_destroy(deo_plan* p) { delete p; }

// internal accessors used by deo_static.cu
extern "C" const PlanDev* deo_plan_device_copy(const deo_plan* p) { return p->d_plan; }
extern "C" int64_t deo_plan_points(const deo_plan* p) { return p->dev.total; }
extern "C" int deo_plan_dtype_code(const deo_plan* p) { return p->dev.dtype; }
extern "C" int deo_plan_has_lbc(const deo_plan* p) { return p->dev.has_lbc; }
extern "C" int deo_plan_terms(const deo_plan* p) { return p ? p->dev.nterms : -1; }
extern "C" int deo_plan_star_taps(const deo_plan* p) { return p ? p->dev.star.n : -1; }
extern "C" deo_status deo_set_error(deo_status s, const char* msg) { return fail(s, "%s", msg); }
extern "C" size_t deo_plan_table_bytes(const deo_plan* p) { return p ? p->table_bytes : 0; }

static deo_status check_ptrs(const deo_plan* p, const void* a, const void* b) {
    if (!p) return fail(DEO_ERR_BAD_ARG, "null plan");
    if (!a || !b) return fail(DEO_ERR_BAD_ARG, "null array");
    if (a == b) return fail(DEO_ERR_BAD_ARG, "input and output must not alias");
    return DEO_OK;
}

static void mark(const deo_plan* p, int k, void* stream) {
    if (p->timing) cudaEventRecord(p->ev[k], static_cast<cudaStream_t>(stream));
}

// Laplacian-type plans: interior kernel on the caller's stream and the
// boundary shell either after it on the same stream, or (DEO_OPT_CONCURRENT_SHELL,
// default) on the plan's side stream at the same time, forked from and joined
// back into the caller's stream.  The interior kernels claim their units from
// a device counter (zeroed on the stream before each launch), so they balance
// around the shell's CTAs.  Launch timing with a concurrent shell: ms[0] =
// fork to the end of the interior kernel, ms[1] = the wait for the shell after it.
static int launch_forward(const deo_plan* p, const void* u, void* du, int overwrite, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    mark(p, 0, stream);
    if (p->uni.enabled && p->fast_path) {
        if (p->uni.lap && p->use_tma && deo_k_tma_ok(&p->uni, p->dev.dtype, u)) {
            // overlap only pays beside an interior kernel that leaves the FP64 pipe free: the fixed-point
            // kernel (Float64) or any Float32 kernel; the FP64-bound interiors run the shell after them
            const bool fx = p->dev.dtype == DEO_F64 &&
                            ((p->exact_sums == 5 && (p->uni.fx || p->uni.bfx)) ||
                             ((p->exact_sums == 1 || p->exact_sums == 4) && p->uni.fx)) &&
                            p->uni.radius <= 3;
            const bool conc = p->concurrent && p->side && p->d_shell && (p->dev.dtype == DEO_F32 || fx);
            const deo::UniPlan* up = &p->uni;
            const char* k = "";
            const char* k2 = "";
            // a counter of its own for this launch (applies of one plan may run on several streams at once)
            unsigned int* sched = p->d_sched ? p->d_sched + (p->sched_slot.fetch_add(1) % kSchedSlots) : nullptr;
            if (conc) {
                // the interior first, on the caller's stream: its persistent grid takes its CTAs' places
                // on every SM at once; then the shell on the side stream, whose CTAs fill the place left
                // beside them (both kernels ask for the largest shared-memory carveout so that this
                // place exists: with the interior's SMs configured for its CTAs alone the shell ran
                // after it, 420 against 303 us at 256^3); the caller's stream waits for the shell
                std::lock_guard<std::mutex> lk(p->apply_mu);
                cudaError_t c = cudaEventRecord(p->ev_fork, st);
                if (c != cudaSuccess) return (int)c;
                const int e = deo_k_apply_tma(up, p->d_plan, p->dev.dtype, u, du, overwrite, p->exact_sums,
                                              stream, &k, sched);
                if (e) return e;  // (cudaErrorNotSupported cannot occur: the tensor-map rules were checked)
                mark(p, 1, stream);
                c = cudaStreamWaitEvent(p->side, p->ev_fork, 0);
                if (c != cudaSuccess) return (int)c;
                int e2 = deo_k_apply_shell(up, &p->shell, p->d_shell, DEO_SHELL_CONCURRENT, p->d_plan,
                                           p->dev.dtype, u, du, overwrite, p->side, &k2);
                if (e2) return e2;
                c = cudaEventRecord(p->ev_join, p->side);
                if (c == cudaSuccess) c = cudaStreamWaitEvent(st, p->ev_join, 0);
                if (c != cudaSuccess) return (int)c;
            } else {
                const int e = deo_k_apply_tma(up, p->d_plan, p->dev.dtype, u, du, overwrite, p->exact_sums,
                                              stream, &k, sched);
                if (e) return e;
                mark(p, 1, stream);
                const int e2 = deo_k_apply_shell(up, p->d_shell ? &p->shell : nullptr, p->d_shell,
                                                 DEO_SHELL_ALONE, p->d_plan, p->dev.dtype, u, du, overwrite,
                                                 stream, &k2);
                if (e2) return e2;
            }
            p->last_kernel = k;
            p->last_kernel2 = k2;
            p->ev_launches = 2;
            mark(p, 2, stream);
            return 0;
        }
        // without the TMA path the generic kernel is the fastest (it outran the register-queue and
        // rolling-window tiles it replaced by 1.1-2.9x once it stopped issuing field multiplies)
    }
    p->last_kernel = "k_apply";
    p->last_kernel2 = "";
    p->ev_launches = 1;
    const int e = deo_k_apply(&p->dev, u, du, overwrite, 0, stream);
    mark(p, 1, stream);
    return e;
}

extern "C" deo_status deo_plan_set_option(deo_plan* p, int option, int value) {
    if (!p) return fail(DEO_ERR_BAD_ARG, "null plan");
    switch (option) {
        case DEO_OPT_FAST_PATH: p->fast_path = value ? 1 : 0; return DEO_OK;
        case DEO_OPT_TMA: p->use_tma = value ? 1 : 0; return DEO_OK;
        case DEO_OPT_EXACT_SUMS:
            if (value < 0 || value > 5) return fail(DEO_ERR_BAD_ARG, "exact-sums variant %d not in 0..5", value);
            p->exact_sums = value;
            return DEO_OK;
        case DEO_OPT_CONCURRENT_SHELL: p->concurrent = value ? 1 : 0; return DEO_OK;
        case DEO_OPT_FX_FP64_ROWS:
            if (value < 0 || value > 8) return fail(DEO_ERR_BAD_ARG, "FP64 rows %d not in 0..8", value);
            p->uni.fx_rows = value;
            return DEO_OK;
        case DEO_OPT_F32_VECTOR: p->uni.f32_vec = value ? 1 : 0; return DEO_OK;
        case DEO_OPT_F32_TILE:
            if (value < 0 || value > 3) return fail(DEO_ERR_BAD_ARG, "tile variant %d not in 0..3", value);
            p->uni.vcfg = value;
            return DEO_OK;
        case DEO_OPT_SHELL_KERNEL:
            if (value < 0 || value > 3) return fail(DEO_ERR_BAD_ARG, "shell kernel %d not in 0..3", value);
            p->uni.shell_kernel = value;
            return DEO_OK;
        case DEO_OPT_TEST_WITHHOLD:
            if (value < 0 || value > 64) return fail(DEO_ERR_BAD_ARG, "withheld plane %d not in 0..64", value);
            p->uni.test_withhold = value;
            p->uni.wait_polls = value ? 64u : 0u;
            return DEO_OK;
        case DEO_OPT_LAUNCH_TIMING:
            if (value && !p->ev[0])
                for (cudaEvent_t& e : p->ev) CUDA_TRY(cudaEventCreate(&e), "cudaEventCreate");
            p->timing = value ? 1 : 0;
            return DEO_OK;
    }
    return fail(DEO_ERR_BAD_ARG, "unknown plan option %d", option);
}

extern "C" int deo_plan_get_option(const deo_plan* p, int option) {
    if (!p) return -1;
    switch (option) {
        case DEO_OPT_FAST_PATH: return p->fast_path && p->uni.enabled;
        case DEO_OPT_TMA: return p->use_tma && p->uni.enabled && p->uni.lap;
        case DEO_OPT_EXACT_SUMS:
            return p->exact_sums && p->uni.enabled && p->uni.lap && (p->uni.ens || p->uni.fx || p->uni.bfx);
        case DEO_OPT_LAUNCH_TIMING: return p->timing;
        case DEO_OPT_TEST_WITHHOLD: return p->uni.test_withhold;
        case DEO_OPT_SHELL_KERNEL: return p->uni.shell_kernel;
        case DEO_OPT_F32_TILE: return p->uni.vcfg;
        case DEO_OPT_F32_VECTOR:
            return p->dev.dtype == DEO_F32 && p->uni.enabled && p->uni.lap && p->uni.f32_vec && p->uni.radius <= 3;
        case DEO_OPT_FX_FP64_ROWS:
            return (p->dev.dtype == DEO_F64 && p->uni.enabled && p->uni.lap &&
                    (p->exact_sums == 1 || p->exact_sums == 4 || (p->exact_sums == 5 && !p->uni.bfx)) &&
                    p->uni.fx &&
                    p->uni.radius <= 3)
                       ? p->uni.fx_rows
                       : 0;
        case DEO_OPT_CONCURRENT_SHELL:
            return p->concurrent && p->side && p->d_shell && p->uni.enabled && p->uni.lap &&
                   (p->dev.dtype == DEO_F32 ||
                    (((p->exact_sums == 5 && (p->uni.fx || p->uni.bfx)) ||
                      ((p->exact_sums == 1 || p->exact_sums == 4) && p->uni.fx)) &&
                     p->uni.radius <= 3));
    }
    return -1;
}

extern "C" const char* deo_plan_kernels(const deo_plan* p, int which) {
    if (!p) return "";
    return which == 0 ? p->last_kernel.load() : (which == 1 ? p->last_kernel2.load() : "");
}

extern "C" deo_status deo_plan_launch_times(const deo_plan* p, float* ms, int* n) {
    if (!p || !ms || !n) return fail(DEO_ERR_BAD_ARG, "null argument");
    if (!p->timing || !p->ev_launches) return fail(DEO_ERR_BAD_ARG, "launch timing is off or nothing was applied");
    const int k = p->ev_launches;
    CUDA_TRY(cudaEventSynchronize(p->ev[k]), "cudaEventSynchronize");
    for (int j = 0; j < k; ++j) CUDA_TRY(cudaEventElapsedTime(&ms[j], p->ev[j], p->ev[j + 1]), "cudaEventElapsedTime");
    *n = k;
    return DEO_OK;
}

extern "C" deo_status deo_device_status(unsigned int* status) {
    if (!status) return fail(DEO_ERR_BAD_ARG, "null argument");
    int e = deo_k_read_status(status);
    unsigned int s2 = 0, s3 = 0;
    if (!e) e = deo_k_read_shell_status(&s2);
    if (!e) e = deo_k_read_vec_status(&s3);
    if (e) return cuda_fail((cudaError_t)e, "deo_device_status");
    *status |= s2 | s3;
    return *status ? fail(DEO_ERR_TIMEOUT, "a bounded device wait gave up (status 0x%x)", *status) : DEO_OK;
}

extern "C" deo_status deo_apply(const deo_plan* p, const void* u, void* du, int overwrite, void* stream) {
    deo_status s = check_ptrs(p, u, du);
    if (s != DEO_OK) return s;
    const int e = launch_forward(p, u, du, overwrite, stream);
    if (e) return cuda_fail((cudaError_t)e, "deo_apply launch");
    return DEO_OK;
}

// Transposed applies.  Laplacian-type plans on the TMA path: the interior
// kernel of the forward apply, with every band's taps reversed, on the box
// of columns read only by band rows (there column j of the transpose is
// sum_k w[2H - k] d[j + k - H], the order in which the generic column
// evaluator adds the rows), then the generic column evaluator on the rest
// (k_shell_adj, a full grid; beside the interior, in the one CTA per SM that
// fits there, it took longer than the interior: 0.52 against 0.37 ms at
// 256^3).  Other plans: the generic transposed kernel.
template <typename E>
static void reverse_taps(E* w, int n) {
    for (int k = 0; k < n / 2; ++k) std::swap(w[k], w[n - 1 - k]);
}

static int launch_adjoint(const deo_plan* p, const void* d, void* ub, int overwrite, void* stream) {
    if (p->adj_ok && p->uni.enabled && p->uni.lap && p->fast_path && p->use_tma &&
        deo_k_tma_ok(&p->uni, p->dev.dtype, d)) {
        deo::UniPlan ua = p->uni;
        const int K = 2 * ua.radius + 1;
        for (int a = 0; a < ua.nterms; ++a) {
            ua.t[a].flo = p->adj_lo[a];
            ua.t[a].fhi = p->adj_hi[a];
            if (p->dev.dtype == DEO_F64) reverse_taps(ua.t[a].w, K);
            else reverse_taps(reinterpret_cast<float*>(ua.t[a].w), K);
        }
        // the same reversal of the integer and exact-sum images of the shared band (their centre
        // weight and scale are unchanged)
        reverse_taps(ua.ens_w, K);
        reverse_taps(ua.fx_w, K);
        reverse_taps(ua.bfx_w, K);
        unsigned int* sched = p->d_sched ? p->d_sched + (p->sched_slot.fetch_add(1) % kSchedSlots) : nullptr;
        const char* k = "";
        const int e = deo_k_apply_tma(&ua, p->d_plan, p->dev.dtype, d, ub, overwrite, p->exact_sums, stream, &k,
                                      sched);
        if (e) return e;
        const int e2 = deo_k_apply_shell_adj(&ua, p->d_plan, p->dev.dtype, d, ub, overwrite, 0, stream);
        if (e2) return e2;
        p->last_kernel = k;
        p->last_kernel2 = "k_shell_adj";
        return 0;
    }
    p->last_kernel = "k_apply";
    p->last_kernel2 = "";
    return deo_k_apply(&p->dev, d, ub, overwrite, 1, stream);
}

extern "C" deo_status deo_apply_adjoint(const deo_plan* p, const void* d, void* ub, int overwrite, void* stream) {
    deo_status s = check_ptrs(p, d, ub);
    if (s != DEO_OK) return s;
    const int e = launch_adjoint(p, d, ub, overwrite, stream);
    if (e) return cuda_fail((cudaError_t)e, "deo_apply_adjoint launch");
    return DEO_OK;
}

extern "C" deo_status deo_apply_host(deo_plan* p, const void* uh, void* duh, void* stream) {
    deo_status s = check_ptrs(p, uh, duh);
    if (s != DEO_OK) return s;
    const size_t bytes = (size_t)p->dev.total * (p->dev.dtype == DEO_F64 ? 8 : 4);
    if (!p->stage_u) {
        CUDA_TRY(cudaMalloc(&p->stage_u, bytes), "cudaMalloc(staging)");
        CUDA_TRY(cudaMalloc(&p->stage_du, bytes), "cudaMalloc(staging)");
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CUDA_TRY(cudaMemcpyAsync(p->stage_u, uh, bytes, cudaMemcpyHostToDevice, st), "H2D");
    const int e = launch_forward(p, p->stage_u, p->stage_du, 1, stream);
    if (e) return cuda_fail((cudaError_t)e, "deo_apply_host launch");
    CUDA_TRY(cudaMemcpyAsync(duh, p->stage_du, bytes, cudaMemcpyDeviceToHost, st), "D2H");
    CUDA_TRY(cudaStreamSynchronize(st), "synchronize");
    return DEO_OK;
}

// Pipelined host applies: call i uses staging slot i % 2.  Its copy-in runs
// on the plan's copy-in stream once apply i-2 has finished reading the slot;
// the apply runs on the caller's stream once the copy-in has landed and copy-out
// i-2 has drained the slot; the copy-out runs on the plan's copy-out stream.
// So copy-in i+1, apply i and copy-out i-1 overlap (H2D and D2H run in both
// directions at once).
extern "C" deo_status deo_apply_host_async(deo_plan* p, const void* uh, void* duh, void* stream) {
    deo_status s = check_ptrs(p, uh, duh);
    if (s != DEO_OK) return s;
    const size_t bytes = (size_t)p->dev.total * (p->dev.dtype == DEO_F64 ? 8 : 4);
    std::lock_guard<std::mutex> lk(p->pipe_mu);
    auto& P = p->pipe;
    if (!P.in) {
        for (int k = 0; k < 2; ++k) {
            CUDA_TRY(cudaMalloc(&P.u[k], bytes), "cudaMalloc(staging)");
            CUDA_TRY(cudaMalloc(&P.du[k], bytes), "cudaMalloc(staging)");
            for (cudaEvent_t* e : {&P.ev_in[k], &P.ev_comp[k], &P.ev_out[k]})
                CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
        }
        CUDA_TRY(cudaStreamCreateWithFlags(&P.out, cudaStreamNonBlocking), "cudaStreamCreate");
        CUDA_TRY(cudaStreamCreateWithFlags(&P.in, cudaStreamNonBlocking), "cudaStreamCreate");
    }
    const int k = (int)(P.next++ & 1u);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CUDA_TRY(cudaStreamWaitEvent(P.in, P.ev_comp[k], 0), "cudaStreamWaitEvent");
    CUDA_TRY(cudaMemcpyAsync(P.u[k], uh, bytes, cudaMemcpyHostToDevice, P.in), "H2D");
    CUDA_TRY(cudaEventRecord(P.ev_in[k], P.in), "cudaEventRecord");
    CUDA_TRY(cudaStreamWaitEvent(st, P.ev_in[k], 0), "cudaStreamWaitEvent");
    CUDA_TRY(cudaStreamWaitEvent(st, P.ev_out[k], 0), "cudaStreamWaitEvent");
    const int e = launch_forward(p, P.u[k], P.du[k], 1, stream);
    if (e) return cuda_fail((cudaError_t)e, "deo_apply_host_async launch");
    CUDA_TRY(cudaEventRecord(P.ev_comp[k], st), "cudaEventRecord");
    CUDA_TRY(cudaStreamWaitEvent(P.out, P.ev_comp[k], 0), "cudaStreamWaitEvent");
    CUDA_TRY(cudaMemcpyAsync(duh, P.du[k], bytes, cudaMemcpyDeviceToHost, P.out), "D2H");
    CUDA_TRY(cudaEventRecord(P.ev_out[k], P.out), "cudaEventRecord");
    return DEO_OK;
}

extern "C" deo_status deo_plan_host_sync(deo_plan* p) {
    if (!p) return fail(DEO_ERR_BAD_ARG, "null plan");
    std::lock_guard<std::mutex> lk(p->pipe_mu);
    for (int k = 0; k < 2; ++k)
        if (p->pipe.ev_out[k]) CUDA_TRY(cudaEventSynchronize(p->pipe.ev_out[k]), "cudaEventSynchronize");
    return DEO_OK;
}

// nonlinear_diffusion!: a plan over the order-1 .. (m+n) CenteredDifference
// operators of the grid (term k-1 has order k), whose ghosts are read from the
// padded inputs themselves (bc_kind 2), evaluated by the generic method.
struct deo_nld {
    deo_plan* plan = nullptr;
    int n = 0, m = 0, len = 0;
    ~deo_nld() { deo_plan_destroy(plan); }
};

extern "C" deo_status deo_nonlinear_diffusion_plan(int second_order, int first_order, int approx_order,
                                                   const double* dx, int dx_len, int nknots, deo_dtype dtype,
                                                   deo_nld** out) {
    if (!out || !dx) return fail(DEO_ERR_BAD_ARG, "null argument");
    *out = nullptr;
    if (approx_order <= 1) return fail(DEO_ERR_BAD_ARG, "approximation_order must be greater than 1.");
    if (second_order < 1 || first_order < 0 || first_order + second_order > DEO_MAX_TERMS)
        return fail(DEO_ERR_BAD_ARG, "differential orders must satisfy n >= 1, m >= 0, m + n <= %d", DEO_MAX_TERMS);
    const int K = first_order + second_order;
    std::vector<deo_operator*> ops(K, nullptr);
    auto free_ops = [&] {
        for (deo_operator* o : ops) deo_operator_destroy(o);
    };
    deo_bc bc;
    deo_status s = deo_dirichlet_bc(0.0, 0.0, &bc);  // placeholder: the ghosts come from the padded inputs
    std::vector<deo_term> terms(K);
    for (int k = 1; k <= K && s == DEO_OK; ++k) {
        s = deo_centered_difference(k, approx_order, dx, dx_len, nknots, &ops[k - 1]);
        terms[k - 1] = deo_term{ops[k - 1], 1, &bc, nullptr, DEO_PATH_GENERIC};
    }
    auto N = std::make_unique<deo_nld>();
    const int64_t size = nknots;
    if (s == DEO_OK) s = deo_plan_create(1, &size, dtype, K, terms.data(), &N->plan);
    free_ops();
    if (s != DEO_OK) return s;
    for (int k = 0; k < K; ++k) N->plan->dev.t[k].bc_kind = 2;
    CUDA_TRY(cudaMemcpy(N->plan->d_plan, &N->plan->dev, sizeof(PlanDev), cudaMemcpyHostToDevice), "cudaMemcpy(plan)");
    N->n = second_order;
    N->m = first_order;
    N->len = nknots;
    *out = N.release();
    return DEO_OK;
}

extern "C" deo_status deo_nonlinear_diffusion(const deo_nld* nl, const void* p, const void* q, void* du,
                                              void* stream) {
    if (!nl || !p || !q || !du) return fail(DEO_ERR_BAD_ARG, "null argument");
    if (du == p || du == q) return fail(DEO_ERR_BAD_ARG, "du must not alias p or q");
    const int e = deo_k_nonlinear_diffusion(&nl->plan->dev, nl->len, nl->n, nl->m, nl->plan->dev.dtype, p, q, du,
                                            stream);
    if (e) return cuda_fail((cudaError_t)e, "deo_nonlinear_diffusion launch");
    return DEO_OK;
}

extern "C" void deo_nonlinear_diffusion_destroy(deo_nld* nl) { delete nl; }

// Gradient / Divergence / Curl: one row table per axis operator over the padded
// input (ghosts = the input's own edge planes), plus negated copies for the
// curl's subtracted terms; evaluated by the vector-calculus kernels.
struct deo_vc {
    deo_plan tabs;  // owns the uploaded tables (no kernels of its own)
    deo::VcDev dev{};
    int dtype = 0;
    int ncomp_in = 1, ncomp_out = 1;
};

extern "C" deo_status deo_vector_calculus_plan(int kind, int ndims, const deo_operator* const* ops, deo_dtype dtype,
                                               deo_vc** out) {
    if (!out || !ops) return fail(DEO_ERR_BAD_ARG, "null argument");
    *out = nullptr;
    if (kind < DEO_VC_GRADIENT || kind > DEO_VC_CURL) return fail(DEO_ERR_BAD_ARG, "unknown operator kind %d", kind);
    if (ndims < 1 || ndims > DEO_MAX_DIMS) return fail(DEO_ERR_BAD_SHAPE, "ndims must be 1..%d", DEO_MAX_DIMS);
    if (dtype != DEO_F64 && dtype != DEO_F32) return fail(DEO_ERR_BAD_ARG, "unknown dtype");
    if (kind == DEO_VC_CURL && ndims != 3) return fail(DEO_ERR_BAD_SHAPE, "Curl acts on 3-dimensional vectors");
    for (int a = 0; a < ndims; ++a) {
        if (!ops[a]) return fail(DEO_ERR_BAD_ARG, "null operator for axis %d", a + 1);
        const deo_operator& A = *ops[a];
        if (A.wind) return fail(DEO_ERR_UNSUPPORTED, "axis %d: vector-calculus operators are CenteredDifference", a + 1);
        if (A.stl != ops[0]->stl || A.bstl != ops[0]->bstl || A.bpc != ops[0]->bpc)
            return fail(DEO_ERR_BAD_ARG,
                        "axis %d: the axis operators must share stencil_length, boundary_stencil_length and "
                        "boundary_point_count (the methods take them from the first)", a + 1);
        if (A.len < 2 * A.bpc + 1) return fail(DEO_ERR_BAD_SHAPE, "axis %d: len %d < 2*boundary_point_count+1", a + 1, A.len);
        if (kind == DEO_VC_CURL && A.len != ops[0]->len)
            return fail(DEO_ERR_BAD_SHAPE, "All dimensions must have equal no. of grid points");
    }
    auto V = std::make_unique<deo_vc>();
    deo::VcDev& D = V->dev;
    D.kind = kind;
    D.nd = ndims;
    D.quirk = (ndims == 2 || ndims == 3) ? 1 : 0;
    D.bpc = ops[0]->bpc;
    int64_t pv = 1, ov = 1;
    for (int a = 0; a < ndims; ++a) {
        D.len[a] = ops[a]->len;
        D.pstride[a] = pv;
        pv *= ops[a]->len + 2;
        ov *= ops[a]->len;
    }
    D.pvol = pv;
    D.ovol = ov;
    const int mode = D.quirk ? 2 : 0;
    for (int a = 0; a < ndims; ++a) {
        const deo_operator& A = *ops[a];
        for (int neg = 0; neg < (kind == DEO_VC_CURL ? 2 : 1); ++neg) {
            TermDev& T = neg ? D.tn[a] : D.t[a];
            T.axis = a;
            T.len = A.len;
            T.stride = D.pstride[a];
            T.nvar = 1;
            T.bc_kind = 2;
            std::vector<int> rlo(A.len + 2, A.len + 1), rhi(A.len + 2, 0);
            HostTab H;
            deo_status s = compile_table(A, mode, true, 1.0, H, rlo, rhi);
            if (s != DEO_OK) return s;
            if (neg) {  // (-c) * s = -(c * s) exactly
                for (double& w : H.dev.wband) w = -w;
                for (double& w : H.W) w = -w;
            }
            if ((s = upload_tab(V->tabs, H, dtype, T.tab[0])) != DEO_OK) return s;
        }
    }
    // unrolled interior loop: every operator's rows bpc+1 .. len-bpc are one centred band
    int bnk = ops[0]->stl;
    for (int a = 0; a < ndims; ++a) {
        const RowTabDev& tb = D.t[a].tab[0];
        if (!(tb.ilo <= D.bpc + 1 && tb.ihi >= D.len[a] - D.bpc && tb.band_nk == bnk && tb.band_p0_off == 1 - bnk / 2))
            bnk = 0;
    }
    D.band_nk = (bnk == 3 || bnk == 5 || bnk == 7 || bnk == 9) ? bnk : 0;
    V->dtype = dtype;
    V->ncomp_in = kind == DEO_VC_GRADIENT ? 1 : (kind == DEO_VC_CURL ? 3 : ndims);
    V->ncomp_out = kind == DEO_VC_DIVERGENCE ? 1 : (kind == DEO_VC_CURL ? 3 : ndims);
    *out = V.release();
    return DEO_OK;
}

static bool overlaps(const void* a, size_t na, const void* b, size_t nb) {
    const char *pa = static_cast<const char*>(a), *pb = static_cast<const char*>(b);
    return pa < pb + nb && pb < pa + na;
}

extern "C" deo_status deo_vector_calculus_sizes(const deo_vc* vc, int64_t* in_elems, int64_t* out_elems) {
    if (!vc) return fail(DEO_ERR_BAD_ARG, "null plan");
    if (in_elems) *in_elems = vc->dev.pvol * vc->ncomp_in;
    if (out_elems) *out_elems = vc->dev.ovol * vc->ncomp_out;
    return DEO_OK;
}

extern "C" deo_status deo_vector_calculus_info(const deo_vc* vc, int* band_nk) {
    if (!vc || !band_nk) return fail(DEO_ERR_BAD_ARG, "null argument");
    *band_nk = vc->dev.band_nk;
    return DEO_OK;
}

extern "C" deo_status deo_vector_calculus_apply(const deo_vc* vc, const void* M, void* out, int overwrite,
                                                void* stream) {
    if (!vc || !M || !out) return fail(DEO_ERR_BAD_ARG, "null argument");
    const size_t es = vc->dtype == DEO_F64 ? 8 : 4;
    if (overlaps(M, (size_t)(vc->dev.pvol * vc->ncomp_in) * es, out, (size_t)(vc->dev.ovol * vc->ncomp_out) * es))
        return fail(DEO_ERR_BAD_ARG, "the output must not overlap the input");
    const int e = deo_k_vector_calculus(&vc->dev, vc->dtype, M, out, overwrite ? 1 : 0, stream);
    if (e) return cuda_fail((cudaError_t)e, "deo_vector_calculus_apply launch");
    return DEO_OK;
}

extern "C" void deo_vector_calculus_destroy(deo_vc* vc) { delete vc; }

// L*M / mul!(x_temp, L, M) on an already padded array (derivative_operator_functions.jl:17-69).
struct deo_padded {
    deo_plan tabs;  // owns the uploaded row table
    deo::VcDev dev{};
    int axis = 0;
    int64_t coff = 0, in_elems = 0;
    int dtype = 0;
};

// starts = null: M's size along every axis but `axis` equals x_temp's or is 2
// longer (then its edge planes are skipped, the stripping of
// derivative_operator_functions.jl:47-56); else M is the view of the array
// with sizes in_sizes that begins at 0-based index starts[b] along axis b.
static deo_status padded_plan(const deo_operator* op, int axis, int ndims, const int64_t* out_sizes,
                              const int64_t* in_sizes, const int64_t* starts, deo_dtype dtype, deo_padded** out) {
    if (!op || !out_sizes || !in_sizes || !out) return fail(DEO_ERR_BAD_ARG, "null argument");
    *out = nullptr;
    if (ndims < 1 || ndims > DEO_MAX_DIMS) return fail(DEO_ERR_BAD_SHAPE, "ndims must be 1..%d", DEO_MAX_DIMS);
    if (axis < 1 || axis > ndims) return fail(DEO_ERR_BAD_SHAPE, "axis %d outside 1..%d", axis, ndims);
    if (dtype != DEO_F64 && dtype != DEO_F32) return fail(DEO_ERR_BAD_ARG, "unknown dtype");
    const int a = axis - 1;
    int64_t start[DEO_MAX_DIMS];
    for (int b = 0; b < ndims; ++b) {
        if (out_sizes[b] < 1) return fail(DEO_ERR_BAD_SHAPE, "size(x_temp, %d) = %lld", b + 1, (long long)out_sizes[b]);
        if (starts) {
            start[b] = starts[b];
            const bool ok = b == a ? (start[b] == 0 && in_sizes[b] >= out_sizes[b] + 2)
                                   : (start[b] >= 0 && start[b] + out_sizes[b] <= in_sizes[b]);
            if (!ok)
                return fail(DEO_ERR_BAD_SHAPE, "view of M along %d (start %lld, size(M) %lld) does not hold x_temp's %lld%s",
                            b + 1, (long long)start[b], (long long)in_sizes[b], (long long)out_sizes[b],
                            b == a ? " + 2 from index 0 (the differentiated dimension)" : "");
            continue;
        }
        const bool ok = b == a ? in_sizes[b] == out_sizes[b] + 2
                               : (in_sizes[b] == out_sizes[b] || in_sizes[b] == out_sizes[b] + 2);
        if (!ok)
            return fail(DEO_ERR_BAD_SHAPE, "size(M, %d) = %lld does not fit size(x_temp, %d) = %lld%s", b + 1,
                        (long long)in_sizes[b], b + 1, (long long)out_sizes[b],
                        b == a ? " + 2 (the differentiated dimension must be padded)" : " (or + 2)");
        start[b] = (b != a && in_sizes[b] == out_sizes[b] + 2) ? 1 : 0;
    }
    if (out_sizes[a] != op->len)
        return fail(DEO_ERR_BAD_SHAPE, "size(x_temp, %d) = %lld but the operator has len %d", axis,
                    (long long)out_sizes[a], op->len);
    if (!op->wind && op->len < 2 * op->bpc + 1)
        return fail(DEO_ERR_BAD_SHAPE, "len %d < 2*boundary_point_count+1", op->len);
    auto P = std::make_unique<deo_padded>();
    deo::VcDev& D = P->dev;
    D.nd = ndims;
    int64_t pv = 1, ov = 1, coff = 0;
    for (int b = 0; b < ndims; ++b) {
        D.len[b] = out_sizes[b];
        D.pstride[b] = pv;
        coff += start[b] * pv;
        pv *= in_sizes[b];
        ov *= out_sizes[b];
    }
    D.pvol = pv;
    D.ovol = ov;
    TermDev& T = D.t[0];
    T.axis = a;
    T.len = op->len;
    T.stride = D.pstride[a];
    T.nvar = 1;
    T.bc_kind = 2;
    std::vector<int> rlo(op->len + 2, op->len + 1), rhi(op->len + 2, 0);
    HostTab H;
    deo_status s = compile_table(*op, 0, true, 1.0, H, rlo, rhi);
    if (s != DEO_OK) return s;
    if ((s = upload_tab(P->tabs, H, dtype, T.tab[0])) != DEO_OK) return s;
    P->axis = a;
    P->coff = coff;
    P->in_elems = pv;
    P->dtype = dtype;
    *out = P.release();
    return DEO_OK;
}

extern "C" deo_status deo_padded_plan(const deo_operator* op, int axis, int ndims, const int64_t* out_sizes,
                                      const int64_t* in_sizes, deo_dtype dtype, deo_padded** out) {
    return padded_plan(op, axis, ndims, out_sizes, in_sizes, nullptr, dtype, out);
}

extern "C" deo_status deo_padded_plan_view(const deo_operator* op, int axis, int ndims, const int64_t* out_sizes,
                                           const int64_t* in_sizes, const int64_t* starts, deo_dtype dtype,
                                           deo_padded** out) {
    if (!starts) return fail(DEO_ERR_BAD_ARG, "null starts");
    return padded_plan(op, axis, ndims, out_sizes, in_sizes, starts, dtype, out);
}

extern "C" deo_status deo_padded_apply(const deo_padded* p, const void* M, void* x_temp, int overwrite,
                                       void* stream) {
    if (!p || !M || !x_temp) return fail(DEO_ERR_BAD_ARG, "null argument");
    const size_t es = p->dtype == DEO_F64 ? 8 : 4;
    if (overlaps(M, (size_t)p->in_elems * es, x_temp, (size_t)p->dev.ovol * es))
        return fail(DEO_ERR_BAD_ARG, "x_temp must not overlap M");
    const int e = deo_k_padded_apply(&p->dev, p->axis, p->coff, p->dtype, M, x_temp, overwrite ? 1 : 0, stream);
    if (e) return cuda_fail((cudaError_t)e, "deo_padded_apply launch");
    return DEO_OK;
}

extern "C" void deo_padded_destroy(deo_padded* p) { delete p; }

static deo_status vector_algebra(int op, deo_dtype dtype, int64_t npts, int ncomp, const void* A, const void* B,
                                 void* u, void* stream) {
    if (!A || !u || (op != 2 && !B)) return fail(DEO_ERR_BAD_ARG, "null argument");
    if (dtype != DEO_F64 && dtype != DEO_F32) return fail(DEO_ERR_BAD_ARG, "unknown dtype");
    if (npts < 0 || ncomp < 1) return fail(DEO_ERR_BAD_SHAPE, "npts must be >= 0 and ncomp >= 1");
    const size_t es = dtype == DEO_F64 ? 8 : 4;
    const size_t nin = (size_t)npts * ncomp * es, nout = (size_t)npts * (op == 1 ? 3 : 1) * es;
    if (overlaps(A, nin, u, nout) || (B && op != 2 && overlaps(B, nin, u, nout)))
        return fail(DEO_ERR_BAD_ARG, "the output must not overlap the inputs");
    const int e = deo_k_vector_algebra(op, dtype, npts, ncomp, A, B, u, stream);
    if (e) return cuda_fail((cudaError_t)e, "vector algebra launch");
    return DEO_OK;
}

extern "C" deo_status deo_dot_product(deo_dtype dtype, int64_t npts, int ncomp, const void* A, const void* B, void* u,
                                      void* stream) {
    return vector_algebra(0, dtype, npts, ncomp, A, B, u, stream);
}

extern "C" deo_status deo_cross_product(deo_dtype dtype, int64_t npts, const void* A, const void* B, void* u,
                                        void* stream) {
    return vector_algebra(1, dtype, npts, 3, A, B, u, stream);
}

extern "C" deo_status deo_square_norm(deo_dtype dtype, int64_t npts, int ncomp, const void* A, void* u,
                                      void* stream) {
    return vector_algebra(2, dtype, npts, ncomp, A, nullptr, u, stream);
}

// ---------------------------------------------------------------------------
// A \ u for A = L*Q (ghost_derivative_operator.jl:39-58): the reference
// concretises (A_l, A_b) = sparse(A) (concretization.jl:938-958: sparse(L) *
// sparse(Q)) and solves A_l x = u - A_b with a sparse LU.  Here A_l is the
// same len x len band on every line along the operator's axis, factored once
// on the host (partial pivoting), and every line is solved on the device.
// ---------------------------------------------------------------------------
struct deo_solve {
    int n = 0, kl = 0, ku = 0, ldab = 0, dtype = 0;
    int64_t stride = 1, nlines = 0, total = 0;
    double* d_ab = nullptr;   // LU factors, band storage [ldab][n] (row r holds diagonal kl+ku-r)
    int* d_ipiv = nullptr;
    double* d_b = nullptr;    // A_b
    double* d_rdiag = nullptr; // 1 / U[j][j]
    double* d_work = nullptr; // Float32 plans: the lines in Float64 while they are solved
    ~deo_solve() {
        if (d_rdiag) cudaFree(d_rdiag);
        if (d_ab) cudaFree(d_ab);
        if (d_ipiv) cudaFree(d_ipiv);
        if (d_b) cudaFree(d_b);
        if (d_work) cudaFree(d_work);
    }
};

// (A_l, A_b) of L*Q as sparse rows: A_l[i] = {column (1..n) -> value}, the
// products L[i,j] * Q[j,c] summed in increasing j as the sparse product does.
static deo_status ghost_rows(const deo_operator& op, const deo_bc& q, std::vector<std::vector<std::pair<long, double>>>& A,
                             std::vector<double>& Ab) {
    const long N = op.len;
    std::vector<std::vector<std::pair<long, double>>> Lr(N);
    array_entries(&op, [&](long i, long j, double v) {
        auto& r = Lr[i - 1];
        for (auto& e : r)
            if (e.first == j) {
                e.second = v;
                return;
            }
        r.emplace_back(j, v);
    });
    if (q.kind == DEO_BC_AFFINE && (q.m_l > N || q.m_r > N)) return fail(DEO_ERR_BAD_SHAPE, "BC stencil longer than N");
    A.assign(N, {});
    Ab.assign(N, 0.0);
    for (long i = 0; i < N; ++i) {
        auto& r = Lr[i];
        std::sort(r.begin(), r.end());
        auto add = [&](long c, double v) {
            for (auto& e : A[i])
                if (e.first == c) {
                    e.second = e.second + v;
                    return;
                }
            A[i].emplace_back(c, v);
        };
        bool have_b = false;
        for (const auto& e : r) {
            const long j = e.first;
            const double v = e.second;
            if (j == 1 || j == N + 2) {  // a ghost: its row of Q
                if (q.kind == DEO_BC_PERIODIC) {  // Array(PeriodicBC, N): ghost_l = u[N], ghost_r = u[1]
                    add(j == 1 ? N : 1, v);
                } else {
                    const int m = j == 1 ? q.m_l : q.m_r;
                    const double* a = j == 1 ? q.a_l : q.a_r;
                    const long c0 = j == 1 ? 1 : N - q.m_r + 1;
                    for (int k = 0; k < m; ++k) add(c0 + k, v * a[k]);
                    const double bv = v * (j == 1 ? q.b_l : q.b_r);
                    Ab[i] = have_b ? Ab[i] + bv : bv;
                    have_b = true;
                }
            } else {
                add(j - 1, v);
            }
        }
    }
    // columns in increasing order within each row, with the sums above done in
    // increasing j: re-sort only for the band placement below
    for (auto& r : A) std::sort(r.begin(), r.end());
    return DEO_OK;
}

// Banded LU with partial pivoting (the unblocked LAPACK gbtf2 scheme) of the
// n x n band with kl sub- and ku super-diagonals in AB[(kl+ku+r)...]: row r of
// AB holds diagonal (kl + ku - r) -- entry (i, j) at AB[(kl + ku + i - j) * n + j];
// rows 0..kl-1 receive the fill-in.
static bool band_lu(int n, int kl, int ku, std::vector<double>& AB, std::vector<int>& ipiv) {
    const int kv = kl + ku;
    auto at = [&](long i, long j) -> double& { return AB[(size_t)(kv + i - j) * n + j]; };
    ipiv.assign(n, 0);
    long ju = 0;
    for (long j = 0; j < n; ++j) {
        const long km = std::min<long>(kl, n - 1 - j);
        long jp = 0;
        double best = std::fabs(at(j, j));
        for (long r = 1; r <= km; ++r)
            if (std::fabs(at(j + r, j)) > best) {
                best = std::fabs(at(j + r, j));
                jp = r;
            }
        ipiv[j] = (int)(j + jp);
        if (at(j + jp, j) == 0.0) return false;
        ju = std::max(ju, std::min<long>(j + ku + jp, n - 1));
        if (jp != 0)
            for (long c = j; c <= ju; ++c) std::swap(at(j, c), at(j + jp, c));
        const double piv = at(j, j);
        for (long r = 1; r <= km; ++r) at(j + r, j) = at(j + r, j) / piv;
        for (long c = j + 1; c <= ju; ++c) {
            const double u = at(j, c);
            if (u == 0.0) continue;
            for (long r = 1; r <= km; ++r) at(j + r, c) = at(j + r, c) - at(j + r, j) * u;
        }
    }
    return true;
}

extern "C" deo_status deo_solve_plan(const deo_operator* op, const deo_bc* bc, int ndims, const int64_t* sizes, int axis,
                                     deo_dtype dtype, deo_solve** out) {
    if (!op || !bc || !sizes || !out) return fail(DEO_ERR_BAD_ARG, "null argument");
    *out = nullptr;
    if (ndims < 1 || ndims > DEO_MAX_DIMS) return fail(DEO_ERR_BAD_SHAPE, "ndims must be 1..%d", DEO_MAX_DIMS);
    if (axis < 1 || axis > ndims) return fail(DEO_ERR_BAD_SHAPE, "axis %d outside 1..%d", axis, ndims);
    if (dtype != DEO_F64 && dtype != DEO_F32) return fail(DEO_ERR_BAD_ARG, "unknown dtype");
    if (sizes[axis - 1] != op->len)
        return fail(DEO_ERR_BAD_SHAPE, "size(u, %d) = %lld but the operator has len %d", axis,
                    (long long)sizes[axis - 1], op->len);
    const long N = op->len;
    std::vector<std::vector<std::pair<long, double>>> A;
    std::vector<double> Ab;
    deo_status st = ghost_rows(*op, *bc, A, Ab);
    if (st != DEO_OK) return st;
    int kl = 0, ku = 0;
    for (long i = 0; i < N; ++i)
        for (const auto& e : A[i]) {
            const long c = e.first - 1;
            kl = std::max<int>(kl, (int)(i - c));
            ku = std::max<int>(ku, (int)(c - i));
        }
    const int ldab = 2 * kl + ku + 1;
    if ((double)ldab * (double)N > 6.4e7)
        return fail(DEO_ERR_UNSUPPORTED, "the band of A_l (%d sub-, %d super-diagonals, n = %ld) is too wide to factor",
                    kl, ku, N);
    std::vector<double> AB((size_t)ldab * N, 0.0);
    for (long i = 0; i < N; ++i)
        for (const auto& e : A[i]) {
            const long j = e.first - 1;
            AB[(size_t)(kl + ku + i - j) * N + j] = e.second;
        }
    std::vector<int> ipiv;
    if (!band_lu((int)N, kl, ku, AB, ipiv))
        return fail(DEO_ERR_BAD_ARG, "A_l is singular (the operator with this boundary condition has no inverse)");
    auto S = std::make_unique<deo_solve>();
    S->n = (int)N;
    S->kl = kl;
    S->ku = ku;
    S->ldab = ldab;
    S->dtype = dtype;
    int64_t stride = 1, total = 1;
    for (int k = 0; k < ndims; ++k) {
        if (sizes[k] < 1) return fail(DEO_ERR_BAD_SHAPE, "size(u, %d) = %lld", k + 1, (long long)sizes[k]);
        if (k < axis - 1) stride *= sizes[k];
        total *= sizes[k];
    }
    S->stride = stride;
    S->total = total;
    S->nlines = total / N;
    CUDA_TRY(cudaMalloc(&S->d_ab, AB.size() * sizeof(double)), "cudaMalloc(LU factors)");
    CUDA_TRY(cudaMemcpy(S->d_ab, AB.data(), AB.size() * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy");
    CUDA_TRY(cudaMalloc(&S->d_ipiv, ipiv.size() * sizeof(int)), "cudaMalloc(pivots)");
    CUDA_TRY(cudaMemcpy(S->d_ipiv, ipiv.data(), ipiv.size() * sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
    CUDA_TRY(cudaMalloc(&S->d_b, Ab.size() * sizeof(double)), "cudaMalloc(A_b)");
    CUDA_TRY(cudaMemcpy(S->d_b, Ab.data(), Ab.size() * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy");
    std::vector<double> rdiag(N);
    for (long j = 0; j < N; ++j) rdiag[j] = 1.0 / AB[(size_t)(kl + ku) * N + j];
    CUDA_TRY(cudaMalloc(&S->d_rdiag, rdiag.size() * sizeof(double)), "cudaMalloc(pivots)");
    CUDA_TRY(cudaMemcpy(S->d_rdiag, rdiag.data(), rdiag.size() * sizeof(double), cudaMemcpyHostToDevice), "cudaMemcpy");
    if (dtype == DEO_F32) CUDA_TRY(cudaMalloc(&S->d_work, (size_t)total * sizeof(double)), "cudaMalloc(workspace)");
    *out = S.release();
    return DEO_OK;
}

extern "C" deo_status deo_solve_bands(const deo_solve* s, int* kl, int* ku) {
    if (!s) return fail(DEO_ERR_BAD_ARG, "null plan");
    if (kl) *kl = s->kl;
    if (ku) *ku = s->ku;
    return DEO_OK;
}

extern "C" deo_status deo_solve_apply(const deo_solve* s, const void* u, void* x, void* stream) {
    if (!s || !u || !x) return fail(DEO_ERR_BAD_ARG, "null argument");
    const size_t es = s->dtype == DEO_F64 ? 8 : 4, bytes = (size_t)s->total * es;
    if (u != x && overlaps(u, bytes, x, bytes)) return fail(DEO_ERR_BAD_ARG, "x must be u itself or not overlap it");
    const int e = deo_k_band_solve(s->n, s->kl, s->ku, s->d_ab, s->d_ipiv, s->d_b, s->d_rdiag, s->stride, s->nlines,
                                   s->dtype, u, x, s->d_work, stream);
    if (e) return cuda_fail((cudaError_t)e, "deo_solve_apply launch");
    return DEO_OK;
}

extern "C" void deo_solve_destroy(deo_solve* s) { delete s; }

extern "C" deo_status deo_plan_concretize_device(const deo_plan* p, double* Al, double* Ab, void* stream) {
    if (!p || !Al || !Ab) return fail(DEO_ERR_BAD_ARG, "null argument");
    const int64_t n = p->dev.total;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CUDA_TRY(cudaMemsetAsync(Al, 0, (size_t)n * (size_t)n * sizeof(double), st), "cudaMemsetAsync");
    const int e = deo_k_concretize(&p->dev, 0, Al, Ab, 0, 0, nullptr, nullptr, stream);
    if (e == (int)cudaErrorNotSupported) return fail(DEO_ERR_UNSUPPORTED, "plan reads ghosts stored around its lines");
    if (e) return cuda_fail((cudaError_t)e, "concretize");
    return DEO_OK;
}

extern "C" deo_status deo_plan_concretize(const deo_plan* p, double* Al, double* Ab) {
    if (!p || !Al || !Ab) return fail(DEO_ERR_BAD_ARG, "null argument");
    const int64_t n = p->dev.total;
    if (n > (1LL << 31) / 8) return fail(DEO_ERR_UNSUPPORTED, "n x n too large for a dense matrix; use the banded form");
    const size_t bytes = (size_t)n * (size_t)n * sizeof(double);
    size_t fr = 0, tot = 0;
    CUDA_TRY(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
    if (bytes + (size_t)n * 8 > fr / 10 * 9) return fail(DEO_ERR_OOM, "dense A_l needs %zu bytes of device memory", bytes);
    cudaStream_t st = nullptr;
    CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    double *dA = nullptr, *dB = nullptr;
    deo_status s = DEO_OK;
    if (cudaMallocAsync(&dA, bytes, st) != cudaSuccess || cudaMallocAsync(&dB, (size_t)n * 8, st) != cudaSuccess) {
        s = fail(DEO_ERR_OOM, "cudaMallocAsync");
    } else {
        s = deo_plan_concretize_device(p, dA, dB, st);
        if (s == DEO_OK && (cudaMemcpyAsync(Al, dA, bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                            cudaMemcpyAsync(Ab, dB, (size_t)n * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess))
            s = fail(DEO_ERR_CUDA, "D2H");
    }
    if (dA) cudaFreeAsync(dA, st);
    if (dB) cudaFreeAsync(dB, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (s == DEO_OK && e != cudaSuccess) s = cuda_fail(e, "concretize");
    return s;
}

extern "C" deo_status deo_plan_bandwidths(const deo_plan* p, int64_t* l, int64_t* u, void* stream) {
    if (!p || !l || !u) return fail(DEO_ERR_BAD_ARG, "null argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned long long* d = nullptr;
    CUDA_TRY(cudaMallocAsync(&d, 2 * sizeof(unsigned long long), st), "cudaMallocAsync");
    unsigned long long h[2] = {0, 0};
    cudaError_t c = cudaMemsetAsync(d, 0, sizeof h, st);
    int e = c == cudaSuccess ? deo_k_concretize(&p->dev, 2, nullptr, nullptr, 0, 0, d, nullptr, stream) : (int)c;
    if (!e) e = (int)cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (!e) e = (int)cudaStreamSynchronize(st);
    if (e == (int)cudaErrorNotSupported) return fail(DEO_ERR_UNSUPPORTED, "plan reads ghosts stored around its lines");
    if (e) return cuda_fail((cudaError_t)e, "bandwidths");
    *l = (int64_t)h[0];
    *u = (int64_t)h[1];
    return DEO_OK;
}

extern "C" deo_status deo_plan_concretize_banded(const deo_plan* p, int64_t l, int64_t u, double* data, double* Ab,
                                                 void* stream) {
    if (!p || !data || !Ab || l < 0 || u < 0) return fail(DEO_ERR_BAD_ARG, "null argument or negative bandwidth");
    const int64_t n = p->dev.total;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int* flag = nullptr;
    CUDA_TRY(cudaMallocAsync(&flag, sizeof(int), st), "cudaMallocAsync");
    cudaError_t c = cudaMemsetAsync(flag, 0, sizeof(int), st);
    if (c == cudaSuccess) c = cudaMemsetAsync(data, 0, (size_t)(l + u + 1) * (size_t)n * sizeof(double), st);
    int e = c == cudaSuccess ? deo_k_concretize(&p->dev, 1, data, Ab, l, u, nullptr, flag, stream) : (int)c;
    int hf = 0;
    if (!e) e = (int)cudaMemcpyAsync(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(flag, st);
    if (!e) e = (int)cudaStreamSynchronize(st);
    if (e == (int)cudaErrorNotSupported) return fail(DEO_ERR_UNSUPPORTED, "plan reads ghosts stored around its lines");
    if (e) return cuda_fail((cudaError_t)e, "concretize (banded)");
    if (hf) return fail(DEO_ERR_BAD_SHAPE, "an entry of A_l lies outside the bands (%lld, %lld)", (long long)l,
                        (long long)u);
    return DEO_OK;
}

// ---------------------------------------------------------------------------
// batched applies: one persistent launch over a work-list of tiles
// ---------------------------------------------------------------------------
struct deo_batch {
    int kind = 0;  // 0 apply/adjoint batch, 1 Runge-Kutta stage batch
    std::vector<deo::StageDev> stages;
    deo::StageDev* d_stages = nullptr;
    std::vector<deo::InstDev> inst;
    std::vector<const deo_plan*> plans;
    int adjoint = 0, dtype = 0;
    int lbc = 0;  // some plan has per-line boundary conditions
    int tile = 0, ctas = 0;
    int64_t n_items = 0;
    deo::InstDev* d_inst = nullptr;
    deo::WorkItem* d_items = nullptr;
    unsigned int* d_counter = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;
    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
    ~deo_batch() {
        drop_graph();
        if (cap) cudaStreamDestroy(cap);
        cudaFree(d_inst);
        cudaFree(d_stages);
        cudaFree(d_items);
        cudaFree(d_counter);
    }
};

static deo_status batch_items(deo_batch& b, int tile) {
    std::vector<deo::WorkItem> items;
    for (size_t i = 0; i < b.plans.size(); ++i) {
        const int64_t n = b.plans[i]->dev.total;
        for (int64_t s = 0; s < n; s += tile)
            items.push_back(deo::WorkItem{(int)i, (int)std::min<int64_t>(tile, n - s), s});
    }
    // largest tiles first keeps the tail of the persistent launch short
    std::stable_sort(items.begin(), items.end(),
                     [](const deo::WorkItem& x, const deo::WorkItem& y) { return x.count > y.count; });
    cudaFree(b.d_items);
    b.d_items = nullptr;
    b.n_items = (int64_t)items.size();
    if (items.empty()) return DEO_OK;
    CUDA_TRY(cudaMalloc(&b.d_items, items.size() * sizeof(deo::WorkItem)), "cudaMalloc(work-list)");
    CUDA_TRY(cudaMemcpy(b.d_items, items.data(), items.size() * sizeof(deo::WorkItem), cudaMemcpyHostToDevice),
             "cudaMemcpy(work-list)");
    b.tile = tile;
    b.drop_graph();
    return DEO_OK;
}

extern "C" deo_status deo_batch_create(int n, const deo_instance* in, int adjoint, int tile, int ctas,
                                       deo_batch** out) {
    if (!out || (n > 0 && !in)) return fail(DEO_ERR_BAD_ARG, "null argument");
    *out = nullptr;
    auto b = std::make_unique<deo_batch>();
    b->adjoint = adjoint ? 1 : 0;
    for (int i = 0; i < n; ++i) {
        if (!in[i].plan || !in[i].u || !in[i].du) return fail(DEO_ERR_BAD_ARG, "instance %d: null plan or buffer", i);
        if (in[i].u == in[i].du) return fail(DEO_ERR_BAD_ARG, "instance %d: input and output alias", i);
        if (i > 0 && in[i].plan->dev.dtype != in[0].plan->dev.dtype)
            return fail(DEO_ERR_BAD_ARG, "all instances of a batch must share one dtype");
        b->plans.push_back(in[i].plan);
        b->inst.push_back(deo::InstDev{in[i].plan->d_plan, in[i].u, in[i].du});
        b->lbc |= in[i].plan->dev.has_lbc;
    }
    b->dtype = n > 0 ? in[0].plan->dev.dtype : 0;
    if (n > 0) {
        CUDA_TRY(cudaMalloc(&b->d_inst, n * sizeof(deo::InstDev)), "cudaMalloc(instances)");
        CUDA_TRY(cudaMemcpy(b->d_inst, b->inst.data(), n * sizeof(deo::InstDev), cudaMemcpyHostToDevice),
                 "cudaMemcpy(instances)");
    }
    CUDA_TRY(cudaMalloc(&b->d_counter, sizeof(unsigned int)), "cudaMalloc(counter)");
    b->ctas = ctas > 0 ? ctas : 4;
    deo_status s = batch_items(*b, tile > 0 ? tile : 8192);
    if (s != DEO_OK) return s;
    *out = b.release();
    return DEO_OK;
}

extern "C" deo_status deo_apply_each(int n, const deo_instance* in, int adjoint, void* stream) {
    if (n > 0 && !in) return fail(DEO_ERR_BAD_ARG, "null argument");
    for (int i = 0; i < n; ++i) {
        deo_status s = adjoint ? deo_apply_adjoint(in[i].plan, in[i].u, in[i].du, 1, stream)
                               : deo_apply(in[i].plan, in[i].u, in[i].du, 1, stream);
        if (s != DEO_OK) return s;
    }
    return DEO_OK;
}

static deo_status batch_launch(deo_batch& b, cudaStream_t st) {
    const int e = b.kind == 1
                      ? deo_k_stage_batch(b.d_stages, b.d_items, b.n_items, b.d_counter, b.lbc, b.dtype, b.ctas, 256,
                                          st)
                      : deo_k_batch(b.d_inst, b.d_items, b.n_items, b.d_counter, b.dtype, b.adjoint, b.lbc, b.ctas,
                                    256, st);
    if (e) return cuda_fail((cudaError_t)e, "batched launch");
    return DEO_OK;
}

extern "C" deo_status deo_stage_batch_create(int n, const deo_stage* in, int tile, int ctas, deo_batch** out) {
    if (!out || (n > 0 && !in)) return fail(DEO_ERR_BAD_ARG, "null argument");
    *out = nullptr;
    auto b = std::make_unique<deo_batch>();
    b->kind = 1;
    for (int i = 0; i < n; ++i) {
        const deo_stage& s = in[i];
        if (!s.plan || !s.c || !s.out) return fail(DEO_ERR_BAD_ARG, "stage %d: null plan, input or output", i);
        if (s.c == s.out) return fail(DEO_ERR_BAD_ARG, "stage %d: output must not alias the operator input", i);
        if ((s.a == nullptr) != (s.alpha == 0.0) && s.a == nullptr)
            return fail(DEO_ERR_BAD_ARG, "stage %d: alpha != 0 needs a", i);
        if (s.b == nullptr && s.beta != 0.0) return fail(DEO_ERR_BAD_ARG, "stage %d: beta != 0 needs b", i);
        if (i > 0 && s.plan->dev.dtype != in[0].plan->dev.dtype)
            return fail(DEO_ERR_BAD_ARG, "all instances of a batch must share one dtype");
        b->plans.push_back(s.plan);
        b->stages.push_back(deo::StageDev{s.plan->d_plan, s.a, s.b, s.c, s.out, s.alpha, s.beta, s.gamma, s.dt,
                                          s.adjoint ? 1 : 0, 0});
        b->lbc |= s.plan->dev.has_lbc;
    }
    b->dtype = n > 0 ? in[0].plan->dev.dtype : 0;
    if (n > 0) {
        CUDA_TRY(cudaMalloc(&b->d_stages, n * sizeof(deo::StageDev)), "cudaMalloc(stages)");
        CUDA_TRY(cudaMemcpy(b->d_stages, b->stages.data(), n * sizeof(deo::StageDev), cudaMemcpyHostToDevice),
                 "cudaMemcpy(stages)");
    }
    CUDA_TRY(cudaMalloc(&b->d_counter, sizeof(unsigned int)), "cudaMalloc(counter)");
    b->ctas = ctas > 0 ? ctas : 4;
    deo_status s = batch_items(*b, tile > 0 ? tile : 8192);
    if (s != DEO_OK) return s;
    *out = b.release();
    return DEO_OK;
}

extern "C" deo_status deo_batch_run(deo_batch* b, int use_graph, void* stream) {
    if (!b) return fail(DEO_ERR_BAD_ARG, "null batch");
    if (b->n_items == 0) return DEO_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!use_graph) return batch_launch(*b, st);
    if (!b->exec) {
        if (!b->cap) CUDA_TRY(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking), "cudaStreamCreate");
        CUDA_TRY(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        deo_status s = batch_launch(*b, b->cap);
        cudaGraph_t g = nullptr;
        cudaError_t ec = cudaStreamEndCapture(b->cap, &g);
        if (s != DEO_OK) {
            if (g) cudaGraphDestroy(g);
            return s;
        }
        if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture");
        b->graph = g;
        CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0), "cudaGraphInstantiate");
    }
    CUDA_TRY(cudaGraphLaunch(b->exec, st), "cudaGraphLaunch");
    return DEO_OK;
}

extern "C" deo_status deo_batch_set_buffers(deo_batch* b, int i, const void* u, void* du) {
    if (!b || b->kind != 0 || i < 0 || i >= (int)b->inst.size() || !u || !du || u == du)
        return fail(DEO_ERR_BAD_ARG, "bad argument");
    b->inst[i].u = u;
    b->inst[i].du = du;
    CUDA_TRY(cudaMemcpy(b->d_inst + i, &b->inst[i], sizeof(deo::InstDev), cudaMemcpyHostToDevice), "cudaMemcpy");
    return DEO_OK;
}

extern "C" deo_status deo_batch_config(const deo_batch* b, int* tile, int* ctas, int64_t* n_items) {
    if (!b) return fail(DEO_ERR_BAD_ARG, "null batch");
    if (tile) *tile = b->tile;
    if (ctas) *ctas = b->ctas;
    if (n_items) *n_items = b->n_items;
    return DEO_OK;
}

extern "C" void deo_batch_destroy(deo_batch* b) { delete b; }

// Workload signature for the autotuner cache: dtype, direction, instance
// count and a log2-size histogram of the instances' point counts.
static std::string batch_signature(const deo_batch& b) {
    int hist[48] = {0};
    int64_t total = 0;
    int maxw = 0;
    for (const deo_plan* p : b.plans) {
        int lg = 0;
        while ((int64_t(1) << (lg + 1)) <= p->dev.total && lg < 47) ++lg;
        hist[lg]++;
        total += p->dev.total;
        for (int t = 0; t < p->dev.nterms; ++t) maxw = std::max(maxw, p->dev.t[t].tab[0].nw);
    }
    char buf[64];
    std::string s;
    snprintf(buf, sizeof buf, "v1:d%d:a%d:n%zu:w%d:t%lld", b.dtype, b.adjoint, b.plans.size(), maxw, (long long)total);
    s += buf;
    for (int i = 0; i < 48; ++i)
        if (hist[i]) {
            snprintf(buf, sizeof buf, ":%d=%d", i, hist[i]);
            s += buf;
        }
    return s;
}

static std::mutex g_tune_mu;
static std::map<std::string, std::pair<int, int>> g_tune_cache;

// ---- plan autotuner: execution choices of the Laplacian-type TMA path --------
// The candidates are bit-identical to each other (they differ in tiling,
// which kernel evaluates the boundary shell and whether it runs beside the
// interior); the numerical variant (DEO_OPT_EXACT_SUMS) is the caller's.
struct PlanTune {
    int f32_vec, vcfg, shell, conc;
};
static std::map<std::string, PlanTune> g_plan_tune;

static std::string plan_signature(const deo_plan& p) {
    const deo::UniPlan& U = p.uni;
    char buf[256];
    std::snprintf(buf, sizeof buf, "lap/%s/%lldx%lldx%lld/t%d/H%d/es%d/bc%d%d%d", p.dev.dtype == DEO_F64 ? "f64" : "f32",
                  (long long)U.n[0], (long long)U.n[1], (long long)U.n[2], U.nterms, U.radius, p.exact_sums,
                  p.shell.t[0].bc_kind, p.shell.t[1].bc_kind, p.shell.t[2].bc_kind);
    return buf;
}

static void plan_tune_set(deo_plan* p, const PlanTune& c) {
    p->uni.f32_vec = c.f32_vec;
    p->uni.vcfg = c.vcfg;
    p->uni.shell_kernel = c.shell;
    p->concurrent = c.conc;
}

extern "C" deo_status deo_plan_autotune(deo_plan* p, const void* u, void* du, const char* cache_path, void* stream) {
    deo_status s = check_ptrs(p, u, du);
    if (s != DEO_OK) return s;
    if (!(p->uni.enabled && p->uni.lap && p->fast_path && p->use_tma && p->d_shell &&
          deo_k_tma_ok(&p->uni, p->dev.dtype, u)))
        return DEO_OK;  // nothing to choose: the plan runs one kernel
    const std::string key = plan_signature(*p);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (cache_path && g_plan_tune.find(key) == g_plan_tune.end()) {
            if (FILE* f = fopen(cache_path, "r")) {
                char k[512];
                PlanTune c;
                while (fscanf(f, "%511s %d %d %d %d", k, &c.f32_vec, &c.vcfg, &c.shell, &c.conc) == 5)
                    if (std::strncmp(k, "lap/", 4) == 0) g_plan_tune[k] = c;
                fclose(f);
            }
        }
        auto it = g_plan_tune.find(key);
        if (it != g_plan_tune.end()) {
            plan_tune_set(p, it->second);
            return DEO_OK;
        }
    }
    std::vector<PlanTune> cand;
    const bool f32 = p->dev.dtype == DEO_F32;
    const int nv = f32 ? (p->uni.nterms == 3 ? (p->uni.radius <= 2 ? 4 : 3) : 1) : 0;
    for (int shell = 1; shell <= 2; ++shell)
        for (int conc = 1; conc >= 0; --conc) {
            for (int v = 0; v < nv; ++v) cand.push_back(PlanTune{1, v, shell, conc});
            cand.push_back(PlanTune{0, 0, shell, conc});  // Float32: the scalar interior; Float64: the plan's kernel
        }
    const PlanTune keep{p->uni.f32_vec, p->uni.vcfg, p->uni.shell_kernel, p->concurrent};
    cand.insert(cand.begin(), keep);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0), "cudaEventCreate");
    CUDA_TRY(cudaEventCreate(&e1), "cudaEventCreate");
    // The clocks up first: the current choice applied for about 50 ms.  Then three rounds over the
    // candidates (forward, reverse, forward), each timing about 3 ms of applies; a candidate's time is
    // its best round, and it replaces the current choice only if faster by more than 2 %.
    int e = 0;
    float t_one = 0.0f;
    {
        cudaEventRecord(e0, st);
        for (int r = 0; r < 5 && !e; ++r) e = launch_forward(p, u, du, 1, stream);
        cudaEventRecord(e1, st);
        if (!e && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&t_one, e0, e1);
        t_one = std::max(t_one / 5.0f, 1e-3f);
    }
    for (int r = 0, nw = (int)std::min(2000.0f, 50.0f / t_one); r < nw && !e; ++r)
        e = launch_forward(p, u, du, 1, stream);
    const int reps = std::max(5, std::min(200, (int)(3.0f / t_one)));
    std::vector<float> t(cand.size(), 1e30f);
    for (int round = 0; round < 3 && !e && s == DEO_OK; ++round)
        for (size_t i0 = 0; i0 < cand.size() && !e; ++i0) {
            const size_t i = round == 1 ? cand.size() - 1 - i0 : i0;
            plan_tune_set(p, cand[i]);
            for (int r = 0; r < 2 && !e; ++r) e = launch_forward(p, u, du, 1, stream);  // warm-up
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps && !e; ++r) e = launch_forward(p, u, du, 1, stream);
            cudaEventRecord(e1, st);
            if (e) break;
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                s = fail(DEO_ERR_CUDA, "autotune timing failed");
                break;
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            t[i] = std::min(t[i], ms / reps);
        }
    if (e && s == DEO_OK) s = cuda_fail((cudaError_t)e, "autotune apply");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    p->tune_cands.clear();
    p->tune_ms.clear();
    for (size_t i = 0; i < cand.size(); ++i) {
        p->tune_cands.insert(p->tune_cands.end(), {cand[i].f32_vec, cand[i].vcfg, cand[i].shell, cand[i].conc});
        p->tune_ms.push_back(t[i]);
    }
    PlanTune pick = keep;
    float best = t[0] * 0.98f;
    for (size_t i = 1; i < cand.size(); ++i)
        if (t[i] < best) {
            best = t[i];
            pick = cand[i];
        }
    plan_tune_set(p, s == DEO_OK ? pick : keep);
    if (s != DEO_OK) return s;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_plan_tune[key] = pick;
    if (cache_path) {
        if (FILE* f = fopen(cache_path, "a")) {
            fprintf(f, "%s %d %d %d %d\n", key.c_str(), pick.f32_vec, pick.vcfg, pick.shell, pick.conc);
            fclose(f);
        }
    }
    return DEO_OK;
}

extern "C" deo_status deo_plan_autotune_times(const deo_plan* p, int* cands, float* ms, int cap, int* n) {
    if (!p || !n) return fail(DEO_ERR_BAD_ARG, "null argument");
    *n = (int)p->tune_ms.size();
    for (int i = 0; i < *n && i < cap; ++i) {
        if (ms) ms[i] = p->tune_ms[i];
        if (cands)
            for (int k = 0; k < 4; ++k) cands[4 * i + k] = p->tune_cands[4 * i + k];
    }
    return DEO_OK;
}

extern "C" deo_status deo_batch_autotune(deo_batch* b, const char* cache_path, void* stream) {
    if (!b) return fail(DEO_ERR_BAD_ARG, "null batch");
    const std::string key = batch_signature(*b);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (cache_path && g_tune_cache.find(key) == g_tune_cache.end()) {
            if (FILE* f = fopen(cache_path, "r")) {
                char k[4096];
                int t, c;
                while (fscanf(f, "%4095s %d %d", k, &t, &c) == 3) g_tune_cache[k] = {t, c};
                fclose(f);
            }
        }
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            b->ctas = it->second.second;
            return batch_items(*b, it->second.first);
        }
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0), "cudaEventCreate");
    CUDA_TRY(cudaEventCreate(&e1), "cudaEventCreate");
    const int tiles[] = {1024, 2048, 4096, 8192, 16384, 32768, 65536};
    const int ctas[] = {2, 4, 6, 8};
    float best = 1e30f;
    int bt = 8192, bc = 4;
    deo_status s = DEO_OK;
    for (int tile : tiles) {
        if ((s = batch_items(*b, tile)) != DEO_OK) break;
        for (int c : ctas) {
            b->ctas = c;
            if ((s = batch_launch(*b, st)) != DEO_OK) break;  // warm-up
            cudaEventRecord(e0, st);
            for (int r = 0; r < 3 && s == DEO_OK; ++r) s = batch_launch(*b, st);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                s = fail(DEO_ERR_CUDA, "autotune timing failed");
                break;
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                bt = tile;
                bc = c;
            }
        }
        if (s != DEO_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != DEO_OK) return s;
    b->ctas = bc;
    s = batch_items(*b, bt);
    if (s != DEO_OK) return s;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = {bt, bc};
    if (cache_path) {
        if (FILE* f = fopen(cache_path, "a")) {
            fprintf(f, "%s %d %d\n", key.c_str(), bt, bc);
            fclose(f);
        }
    }
    return DEO_OK;
}
