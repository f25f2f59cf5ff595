// deo_oracle.cpp -- CPU restatement of DiffEqOperators.jl's stencil-apply path.
//
// TEST INFRASTRUCTURE ONLY. This file is the oracle: the parity tests, the
// smoke check and the bench's CPU-baseline leg call it; the product library
// never links or calls it.
//
// Every function restates one reference function (paths are relative to the
// DiffEqOperators.jl source tree) in the reference's own operation order.
// Build flags disable FMA contraction (-ffp-contract=off) so each `a*b + c`
// rounds twice, as plain Julia code does; the reference's @turbo loops may
// contract to FMA and reorder, which is why parity is checked with a tolerance
// of 4 ulp of sum|c_k*u_k| per point rather than bit-exactly.
//
// Known-unreproducible details (documented, absorbed by the tolerance):
//   * LoopVectorization.@turbo may fuse/reassociate the tap sums
//     (src/derivative_operators/convolutions.jl:42,52,86,107,381,391,412,430,456,460);
//   * LinearAlgebra.dot in the BC ghost fill goes to BLAS ddot
//     (src/derivative_operators/bc_operators.jl:188-192); restated here as a
//     sequential sum;
//   * Float64^Int follows Julia >= 1.9 Base.pow_body (compensated squaring);
//     for exponents 1..3 it equals plain repeated multiplication.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

#if defined(_OPENMP)
#include <omp.h>
#endif

namespace {

typedef std::vector<double> vec;

// When set, every tap contributes |c*w|*|x| and ghosts are |a|.|u| + |b|:
// applying the operator then yields sum_k |c_k u_k| per point (ghost terms
// expanded), the scale of the parity tolerance.  Row selection still follows
// the real coefficient signs.
static thread_local bool g_abs = false;
static inline double T3(double c, double w, double x) {
    return g_abs ? std::fabs(c * w) * std::fabs(x) : c * w * x;
}

// ---------------------------------------------------------------------------
// Julia Base: Float64 ^ Int (base/math.jl pow_body, Julia >= 1.9)
// ---------------------------------------------------------------------------
static inline void two_mul(double a, double b, double& hi, double& lo) {
    hi = a * b;
    lo = std::fma(a, b, -hi);
}

double julia_powi(double x, long n) {
    if (n == 0) return 1.0;
    double y = 1.0, xnlo = 0.0, ynlo = 0.0;
    if (n == 3) return x * x * x;
    if (n < 0) {
        double rx = 1.0 / x;
        if (n == -2) return rx * rx;
        if (std::isfinite(x)) xnlo = -std::fma(x, rx, -1.0) * rx;
        x = rx;
        n = -n;
    }
    while (n > 1) {
        if (n & 1) {
            double err = std::fma(y, xnlo, x * ynlo);
            double h, l;
            two_mul(x, y, h, l);
            y = h;
            ynlo = l + err;
        }
        double err = x * 2 * xnlo;
        double h, l;
        two_mul(x, x, h, l);
        x = h;
        xnlo = l + err;
        n >>= 1;
    }
    double err = std::fma(y, xnlo, x * ynlo);
    return (std::isfinite(x) && std::isfinite(err)) ? std::fma(x, y, err) : x * y;
}

// ---------------------------------------------------------------------------
// src/derivative_operators/fornberg.jl:7-62  calculate_weights
// ---------------------------------------------------------------------------
vec calculate_weights(int order, double x0, const vec& x) {
    const int N = (int)x.size();
    const int M = order;
    const int W = M + 1;
    double c1 = 1.0;
    double c4 = x[0] - x0;
    vec C((size_t)N * W, 0.0);
    auto at = [&](int i1, int s1) -> double& {  // Julia 1-based C[i1, s1]
        return C[(size_t)(i1 - 1) * W + (s1 - 1)];
    };
    at(1, 1) = 1;
    for (int i = 1; i <= N - 1; ++i) {
        const int i1 = i + 1;
        const int mn = std::min(i, M);
        double c2 = 1.0;
        const double c5 = c4;
        c4 = x[i1 - 1] - x0;
        for (int j = 0; j <= i - 1; ++j) {
            const int j1 = j + 1;
            const double c3 = x[i1 - 1] - x[j1 - 1];
            c2 *= c3;
            if (j == i - 1) {
                for (int s = mn; s >= 1; --s) {
                    const int s1 = s + 1;
                    at(i1, s1) = c1 * ((double)s * at(i, s) - c5 * at(i, s1)) / c2;
                }
                at(i1, 1) = -c1 * c5 * at(i, 1) / c2;
            }
            for (int s = mn; s >= 1; --s) {
                const int s1 = s + 1;
                at(j1, s1) = (c4 * at(j1, s1) - (double)s * at(j1, s)) / c3;
            }
            at(j1, 1) = c4 * at(j1, 1) / c3;
        }
        c1 = c2;
    }
    vec out(N);
    for (int i = 1; i <= N; ++i) out[i - 1] = at(i, M + 1);
    if (order != 0) {
        // Julia `sum` of a Vector with fewer than 16 entries: sequential.
        double s = out[0];
        for (int i = 1; i < N; ++i) s = s + out[i];
        out[N / 2] -= s;
    }
    return out;
}

// ---------------------------------------------------------------------------
// src/derivative_operators/derivative_operator.jl:14-29  DerivativeOperator
// ---------------------------------------------------------------------------
struct Op {
    int d = 0, a = 0, len = 0, stl = 0, bstl = 0, bpc = 0, off = 0;
    bool wind = false, uniform = true;
    // 0 = coeff_func is not a Number, +1 = Number >= 0, -1 = Number < 0
    // (only consulted by the non-uniform upwind generic interior,
    //  convolutions.jl:234-253)
    int coeff_func_sign = 1;
    // Tables, row-major [rows][width]:
    //  centred uniform:      stencil[1][stl],  low[bpc][bstl], high[bpc][bstl]
    //  centred non-uniform:  stencil[len-2bpc][stl], low/high as above
    //  upwind uniform:       stencil[1][stl],  low[bpc][bstl], high[bpc+off][bstl]
    //  upwind non-uniform:   stencil[2][len-2bpc][stl], low[2][bpc][bstl],
    //                        high[2][bpc+off][bstl]
    vec stencil, low, high;
    int n_st = 0, n_low = 0, n_high = 0;  // rows per (wind) half
    vec coeff;                            // coefficients[len]

    const double* st(int row, int half = 0) const {
        return &stencil[((size_t)half * n_st + row) * stl];
    }
    const double* lo(int row, int half = 0) const {
        return &low[((size_t)half * n_low + row) * bstl];
    }
    const double* hi(int row, int half = 0) const {
        return &high[((size_t)half * n_high + row) * bstl];
    }
};

static void push_rows(vec& dst, const vec& row) { dst.insert(dst.end(), row.begin(), row.end()); }

static vec range_vec(double lo, double hi, double step = 1.0) {
    vec v;
    if (step > 0) for (double t = lo; t <= hi + 1e-12; t += step) v.push_back(t);
    else for (double t = lo; t >= hi - 1e-12; t += step) v.push_back(t);
    return v;
}

static vec scaled(double s, const vec& w) {
    vec o(w.size());
    for (size_t k = 0; k < w.size(); ++k) o[k] = s * w[k];
    return o;
}

// derivative_operator.jl:81-135 (uniform) and :150-205 (non-uniform)
Op* centered(int d, int a, const double* dx, int ndx, int len) {
    Op* op = new Op();
    op->d = d; op->a = a; op->len = len; op->wind = false; op->off = 0;
    op->stl = d + a - 1 + (d + a) % 2;
    op->bstl = d + a;
    op->bpc = op->stl / 2 - 1;
    const int stl = op->stl, bstl = op->bstl, bpc = op->bpc;
    if (ndx == 1) {
        op->uniform = true;
        const double h = dx[0];
        const double s = 1.0 / julia_powi(h, d);
        vec dummy_x = range_vec(-(stl / 2), stl / 2);
        push_rows(op->stencil, scaled(s, calculate_weights(d, 0.0, dummy_x)));
        op->n_st = 1;
        vec left_x = range_vec(0, bstl - 1);
        std::vector<vec> lowrows;
        for (int x0 = 1; x0 <= stl / 2 - 1; ++x0)
            lowrows.push_back(scaled(s, calculate_weights(d, (double)x0, left_x)));
        for (auto& r : lowrows) push_rows(op->low, r);
        op->n_low = bpc;
        // high = reverse(map(reverse, low * (-1)^d))
        const double sgn = (d % 2 == 0) ? 1.0 : -1.0;
        for (int i = bpc - 1; i >= 0; --i) {
            vec r(bstl);
            for (int k = 0; k < bstl; ++k) r[k] = lowrows[i][bstl - 1 - k] * sgn;
            push_rows(op->high, r);
        }
        op->n_high = bpc;
    } else {
        op->uniform = false;
        // generate_coordinates, derivative_operator.jl:137-148
        vec stencil_x(stl, 0.0);
        const int c = stl / 2;  // 0-based centre (Julia index(0,len) - 1)
        op->n_st = std::max(0, len - 2 * bpc);
        for (int i = bpc + 2; i <= len + 1 - bpc; ++i) {
            for (int k = 0; k < stl; ++k) stencil_x[k] = stencil_x[k] * 0.0;
            for (int idx = 1; idx <= stl / 2; ++idx) {
                stencil_x[c + idx] = stencil_x[c + idx - 1] + dx[i + idx - 1 - 1];
                stencil_x[c - idx] = stencil_x[c - idx + 1] - dx[i - idx - 1];
            }
            push_rows(op->stencil, calculate_weights(d, 0.0, stencil_x));
        }
        vec low_x(bstl);
        low_x[0] = 0.0;
        for (int k = 1; k < bstl; ++k) low_x[k] = low_x[k - 1] + dx[k - 1];
        vec high_x(bstl);
        {
            double acc = 0.0;
            for (int k = 0; k < bstl; ++k) {
                double v = dx[ndx - bstl + k];
                acc = (k == 0) ? v : acc + v;
                high_x[k] = acc;
            }
        }
        for (int i = 1; i <= bpc; ++i) push_rows(op->low, calculate_weights(d, low_x[i], low_x));
        op->n_low = bpc;
        for (int i = bpc; i >= 1; --i)
            push_rows(op->high, calculate_weights(d, high_x[bstl - 1 - i], high_x));
        op->n_high = bpc;
    }
    op->coeff.assign(len, 1.0);  // compute_coeffs!(1, zeros) -> 0 + 1
    op->coeff_func_sign = 1;
    return op;
}

// derivative_operator.jl:454-512 (uniform) and :515-639 (non-uniform)
Op* upwind(int d, int a, const double* dx, int ndx, int len, int off) {
    Op* op = new Op();
    op->d = d; op->a = a; op->len = len; op->wind = true; op->off = off;
    op->stl = d + a;
    op->bstl = d + a;
    op->bpc = op->bstl - 2 - off;
    const int stl = op->stl, bstl = op->bstl, bpc = op->bpc;
    if (ndx == 1) {
        op->uniform = true;
        const double h = dx[0];
        const double s = 1.0 / julia_powi(h, d);
        vec dummy_x = range_vec(0.0 - off, stl - 1.0 - off);
        push_rows(op->stencil, scaled(s, calculate_weights(d, 0.0, dummy_x)));
        op->n_st = 1;
        vec low_x = range_vec(0.0, bstl - 1);
        for (int x0 = 1; x0 <= bstl - 2 - off; ++x0)
            push_rows(op->low, scaled(s, calculate_weights(d, (double)x0, low_x)));
        op->n_low = bpc;
        vec high_x = range_vec(0.0, -(bstl - 1.0), -1.0);
        const double sh = julia_powi(-1.0 / h, d);
        int nh = 0;
        for (int x0 = -1; x0 >= -(bstl - 2); --x0, ++nh)
            push_rows(op->high, scaled(sh, calculate_weights(d, (double)x0, high_x)));
        op->n_high = nh;  // = bpc + off
    } else {
        op->uniform = false;
        vec x(len + 2);
        x[0] = 0.0;
        for (int k = 1; k <= len + 1; ++k) x[k] = x[k - 1] + dx[k - 1];
        auto X = [&](int j) { return x[j - 1]; };  // Julia 1-based
        // x[lo:hi]; a window outside x is the reference's BoundsError (grid
        // too short for the stencil): flagged, and the operator is rejected
        bool outside = false;
        auto sub = [&](int lo, int hi) {
            if (lo < 1 || hi > len + 2 || hi < lo) {
                outside = true;
                return range_vec(0.0, bstl - 1.0);
            }
            return vec(x.begin() + (lo - 1), x.begin() + hi);
        };
        // low: [upwind; downwind], each bpc rows
        vec up, dn;
        if (off == 0) {
            for (int i = 1; i <= bpc; ++i) push_rows(up, calculate_weights(d, X(i + 1), sub(i + 1, i + bstl)));
        } else {
            for (int i = 1; i <= off - 1; ++i) push_rows(up, calculate_weights(d, X(i + 1), sub(1, bstl)));
            for (int i = off; i <= bpc; ++i)
                push_rows(up, calculate_weights(d, X(i + 1), sub(i + 1 - off, i + bstl - off)));
        }
        for (int i = 1; i <= bpc; ++i) push_rows(dn, calculate_weights(d, X(i + 1), sub(1, bstl)));
        op->low = up; op->low.insert(op->low.end(), dn.begin(), dn.end());
        op->n_low = bpc;
        // interior: [upwind; downwind], len-2bpc rows each
        up.clear(); dn.clear();
        for (int i = bpc + 1; i <= len - bpc; ++i)
            push_rows(up, calculate_weights(d, X(i + 1), sub(i + 1 - off, i + stl - off)));
        for (int i = bpc + 1; i <= len - bpc; ++i)
            push_rows(dn, calculate_weights(d, X(i + 1), sub(i - stl + 2 + off, i + 1 + off)));
        op->stencil = up; op->stencil.insert(op->stencil.end(), dn.begin(), dn.end());
        op->n_st = std::max(0, len - 2 * bpc);
        // high: [upwind; downwind], bpc+off rows each
        up.clear(); dn.clear();
        for (int i = len - bpc + 1 - off; i <= len; ++i)
            push_rows(up, calculate_weights(d, X(i + 1), sub(len - bstl + 3, len + 2)));
        if (off == 0) {
            for (int i = len - bpc + 1; i <= len; ++i)
                push_rows(dn, calculate_weights(d, X(i + 1), sub(i - stl + 2, i + 1)));
        } else {
            for (int i = len - bpc + 1 - off; i <= len - off + 1; ++i)
                push_rows(dn, calculate_weights(d, X(i + 1), sub(i - stl + 2 + off, i + 1 + off)));
            if (off >= 2)
                for (int i = len - off + 2; i <= len; ++i)
                    push_rows(dn, calculate_weights(d, X(i + 1), sub(len - stl + 3, len + 2)));
        }
        op->high = up; op->high.insert(op->high.end(), dn.begin(), dn.end());
        op->n_high = bpc + off;
        if (outside) {
            delete op;
            return nullptr;
        }
    }
    op->coeff.assign(len, 1.0);
    op->coeff_func_sign = 1;
    return op;
}

// ---------------------------------------------------------------------------
// Boundary conditions: src/derivative_operators/bc_operators.jl
// ---------------------------------------------------------------------------
struct BC {
    int kind;  // 0 affine, 1 periodic
    int ml, mr;
    double al[32], ar[32];
    double bl, br;
};

static vec ones_to(int order_plus_1) {
    vec v;
    for (int k = 1; k <= order_plus_1; ++k) v.push_back((double)k);
    return v;
}

// bc_operators.jl:26-60 RobinBC
int robin(const double* l, const double* r, const double* dx, int ndx, int order, BC* out) {
    const double al = l[0], bl = l[1], gl = l[2];
    const double ar = r[0], br = r[1], gr = r[2];
    std::memset(out, 0, sizeof(BC));
    out->kind = 0;
    vec s_index = ones_to(order + 1);
    vec s = calculate_weights(1, 1.0, s_index);
    const int m = order;
    if (m > 32) return -1;
    if (ndx == 1) {
        const double h = dx[0];
        const double denl = al * h / bl + s[0];
        const double denr = ar * h / br - s[0];
        for (int k = 0; k < m; ++k) out->al[k] = -s[1 + k] / denl;
        for (int k = 0; k < m; ++k) out->ar[k] = s[m - k] / denr;  // s[end:-1:2]
        out->bl = gl / (al + bl * s[0] / h);
        out->br = gr / (ar - br * s[0] / h);
    } else {
        const int ns = order + 1;
        if (ndx < ns) return -1;                // the reference's BoundsError
        const double* dxl = dx;                 // dx[1:ns]
        const double* dxr = dx + (ndx - ns);    // dx[end-ns+1:end]
        const double denom_l = al + bl * s[0] / dxl[0];
        const double denom_r = ar - br * s[0] / dxr[ns - 1];
        for (int k = 0; k < m; ++k) out->al[k] = -bl * s[1 + k] / (denom_l * dxl[1 + k]);
        for (int k = 0; k < m; ++k) out->ar[k] = br * s[m - k] / (denom_r * dxr[k]);
        out->bl = gl / denom_l;
        out->br = gr / denom_r;
    }
    out->ml = m;
    out->mr = m;
    return 0;
}

// bc_operators.jl:90-169 GeneralBC
int general(const double* alpha_l, int nl, const double* alpha_r, int nr, const double* dx, int ndx,
            int order, BC* out) {
    std::memset(out, 0, sizeof(BC));
    out->kind = 0;
    const int wl = order + nl - 2, wr = order + nr - 2;
    if (wl - 1 > 32 || wr - 1 > 32) return -1;
    if (ndx != 1 && (ndx < wl || ndx < wr)) return -1;  // the reference's BoundsError
    std::vector<vec> Sl(nl - 2, vec(wl, 0.0)), Sr(nr - 2, vec(wr, 0.0));
    vec dx_l, dx_r;
    if (ndx != 1) {
        for (int k = 0; k < order + nl - 2; ++k) dx_l.push_back(dx[k]);
        // reverse(dx[(end - order - nr + 3):end])
        for (int k = ndx - 1; k >= ndx - (order + nr - 2); --k) dx_r.push_back(dx[k]);
    }
    for (int i = 1; i <= nl - 2; ++i) {
        vec w = calculate_weights(i, 1.0, ones_to(order + i));
        for (int k = 0; k < wl; ++k) {
            double v = k < (int)w.size() ? w[k] : 0.0;
            double den = (ndx == 1) ? julia_powi(dx[0], i) : julia_powi(dx_l[k], i);
            Sl[i - 1][k] = v / den;
        }
    }
    for (int i = 1; i <= nr - 2; ++i) {
        vec w = calculate_weights(i, (double)(order + i), ones_to(order + i));
        for (int k = 0; k < wr; ++k) {
            double v = k < (int)w.size() ? w[k] : 0.0;
            double den = (ndx == 1) ? julia_powi(dx[0], i) : julia_powi(dx_r[k], i);
            Sr[i - 1][k] = v / den;
        }
    }
    // s0_l = S_l[:,1], Sl = S_l[:, 2:end]; s0_r = S_r[:, end], Sr = S_r[:, end-1:-1:1]
    // denoml = αl[2] .+ αl[3:end] ⋅ s0_l  (dot: sequential)
    double dl = 0.0;
    for (int i = 0; i < nl - 2; ++i) dl = (i == 0) ? alpha_l[2 + i] * Sl[i][0] : dl + alpha_l[2 + i] * Sl[i][0];
    if (nl - 2 == 0) dl = 0.0;
    const double denoml = alpha_l[1] + dl;
    double dr = 0.0;
    for (int i = 0; i < nr - 2; ++i)
        dr = (i == 0) ? alpha_r[2 + i] * Sr[i][wr - 1] : dr + alpha_r[2 + i] * Sr[i][wr - 1];
    if (nr - 2 == 0) dr = 0.0;
    const double denomr = alpha_r[1] + dr;
    // a_l = -(αl[3:end]ᵀ Sl) ./ denoml  (row-vector times matrix: column sums)
    out->ml = wl - 1;
    for (int k = 0; k < wl - 1; ++k) {
        double acc = 0.0;
        for (int i = 0; i < nl - 2; ++i) acc = (i == 0) ? alpha_l[2 + i] * Sl[i][1 + k] : acc + alpha_l[2 + i] * Sl[i][1 + k];
        out->al[k] = -acc / denoml;
    }
    out->mr = wr - 1;
    vec tmp(wr - 1);
    for (int k = 0; k < wr - 1; ++k) {
        // Sr column k = S_r[:, end-1-k]
        double acc = 0.0;
        for (int i = 0; i < nr - 2; ++i)
            acc = (i == 0) ? alpha_r[2 + i] * Sr[i][wr - 2 - k] : acc + alpha_r[2 + i] * Sr[i][wr - 2 - k];
        tmp[k] = -acc / denomr;
    }
    for (int k = 0; k < wr - 1; ++k) out->ar[k] = tmp[wr - 2 - k];  // reverse
    out->bl = -alpha_l[0] / denoml;
    out->br = -alpha_r[0] / denomr;
    return 0;
}

// bc_operators.jl:188-192  Q*u  (1-D ghost fill)
static inline void ghosts_1d(const BC& q, const double* u, long n, long stride, double& l, double& r) {
    if (q.kind == 1) {  // PeriodicBC: BoundaryPaddedVector(u[end], u[1], u)
        l = u[(n - 1) * stride];
        r = u[0];
        if (g_abs) { l = std::fabs(l); r = std::fabs(r); }
        return;
    }
    double dl = 0.0;
    for (int j = 0; j < q.ml; ++j) {
        const double t = g_abs ? std::fabs(q.al[j]) * std::fabs(u[j * stride]) : q.al[j] * u[j * stride];
        dl = (j == 0) ? t : dl + t;
    }
    l = dl + (g_abs ? std::fabs(q.bl) : q.bl);
    double dr = 0.0;
    for (int j = 0; j < q.mr; ++j) {
        const double uu = u[(n - q.mr + j) * stride];
        const double t = g_abs ? std::fabs(q.ar[j]) * std::fabs(uu) : q.ar[j] * uu;
        dr = (j == 0) ? t : dr + t;
    }
    r = dr + (g_abs ? std::fabs(q.br) : q.br);
}

// multi_dim_bc_operators.jl:221-228 (N-D PeriodicBC): lower = selectdim(u,D,1),
// upper = selectdim(u,D,end) -- the N-D periodic padding copies the edge planes.
static inline void ghosts_nd(const BC& q, const double* u, long n, long stride, double& l, double& r) {
    if (q.kind == 1) {
        l = u[0];
        r = u[(n - 1) * stride];
        if (g_abs) { l = std::fabs(l); r = std::fabs(r); }
        return;
    }
    ghosts_1d(q, u, n, stride, l, r);
}

// ---------------------------------------------------------------------------
// convolutions.jl -- the apply loops.  x is 1-based, x(1) = left ghost,
// x(len+2) = right ghost.  `tail` implements `+ !overwrite * x_temp[i]`.
// ---------------------------------------------------------------------------
struct Line {
    const double* u;  // interior values, stride
    long stride;
    double l, r;
    long len;
    double operator()(long p) const {  // padded index, 1-based
        if (p == 1) return l;
        if (p == len + 2) return r;
        return u[(p - 2) * stride];
    }
};

static inline double tail(double acc, double old, bool overwrite) {
    return acc + (overwrite ? 0.0 : old);
}

// convolutions.jl:27-118 generic centred (AbstractVector x)
template <class X, class C>
void centred_generic(const Op& A, const X& x, double* out, long ostride, const C& coeff, bool ow) {
    const long len = A.len;
    const int bpc = A.bpc, stl = A.stl, bstl = A.bstl;
    // convolve_BC_left!  :76-95
    for (int i = 1; i <= bpc; ++i) {
        const double* cs = A.lo(i - 1);
        const double cc = coeff(i);
        double acc = 0.0;
        for (int idx = 1; idx <= bstl; ++idx) acc += T3(cc, cs[idx - 1], x(idx));
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    // convolve_interior!  :27-74
    const int mid = stl / 2;
    for (long i = 1 + bpc; i <= len - bpc; ++i) {
        const double* cs = A.uniform ? A.st(0) : A.st((int)(i - bpc - 1));
        const double cc = coeff(i);
        double acc = 0.0;
        for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], x(i - mid + idx));
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    // convolve_BC_right!  :97-118  (coefficient quirk: coeff[i], i in 1:bpc)
    const long L2 = len + 2;
    for (int i = 1; i <= bpc; ++i) {
        const double* cs = A.hi(i - 1);
        const double cc = coeff(i);
        double acc = 0.0;
        for (int idx = bstl - 1; idx >= 0; --idx) acc += T3(cc, cs[bstl - 1 - idx], x(L2 - idx));
        double& o = out[(len - bpc + i - 1) * ostride];
        o = tail(acc, o, ow);
    }
}

// convolutions.jl:367-469 centred on a BoundaryPaddedVector
template <class C>
void centred_padded(const Op& A, const Line& L, double* out, long ostride, const C& coeff, bool ow) {
    const long len = A.len;
    const int bpc = A.bpc, stl = A.stl, bstl = A.bstl;
    auto u = [&](long k) { return L.u[(k - 1) * L.stride]; };  // _x.u[k]
    const int mid = stl / 2 + 1;
    // convolve_BC_left! :402-434
    for (int i = 1; i <= bpc; ++i) {
        const double* cs = A.lo(i - 1);
        const double cc = coeff(i);
        double acc = T3(cc, cs[0], L.l);
        for (int idx = 2; idx <= bstl; ++idx) acc += T3(cc, cs[idx - 1], u(idx - 1));
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    {
        const long i = 1 + bpc;
        const double* cs = A.uniform ? A.st(0) : A.st((int)(i - bpc - 1));
        const double cc = coeff(i - bpc);
        double acc = T3(cc, cs[0], L.l);
        for (int idx = 2; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], u((i - 1) - (mid - idx) + 1));
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    // convolve_interior! :367-400  (coefficient quirk: coeff[i - bpc])
    for (long i = 2 + bpc; i <= (len - bpc) - 1; ++i) {
        const double* cs = A.uniform ? A.st(0) : A.st((int)(i - bpc - 1));
        const double cc = coeff(i - bpc);
        double acc = 0.0;
        for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], u((i - 1) - (mid - idx) + 1));
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    // convolve_BC_right! :436-469
    {
        const long i = len - bpc;
        const double* cs = A.uniform ? A.st(0) : A.st((int)(i - bpc - 1));
        const double cc = coeff(i - bpc);
        double acc = T3(cc, cs[stl - 1], L.r);
        for (int idx = 1; idx <= stl - 1; ++idx) acc += T3(cc, cs[idx - 1], u((i - 1) - (mid - idx) + 1));
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    const long bc_start = len - bpc;
    for (int i = 1; i <= bpc; ++i) {
        const double* cs = A.hi(i - 1);
        const double cc = coeff(bc_start + i);
        double acc = T3(cc, cs[bstl - 1], L.r);
        for (int idx = bstl - 1; idx >= 1; --idx) acc += T3(cc, cs[bstl - 1 - idx], u(len - idx + 1));
        double& o = out[(bc_start + i - 1) * ostride];
        o = tail(acc, o, ow);
    }
}

// convolutions.jl:123-215 (generic) and :479-591 (padded) -- uniform upwind.
template <class X, class C>
void upwind_uniform(const Op& A, const X& x, double* out, long ostride, const C& coeff, bool ow) {
    const long len = A.len, xl = len + 2;
    const int bpc = A.bpc, stl = A.stl, bstl = A.bstl, off = A.off, d = A.d;
    const double* S = A.st(0);
    // convolve_BC_left!
    for (int i = 1; i <= bpc; ++i) {
        const double cc = coeff(i);
        double acc = 0.0;
        if (cc >= 0 && i + stl <= xl && i >= off) {
            for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, S[idx - 1], x(i + idx - off));
        } else {
            const double* cs = A.lo(i - 1);
            for (int idx = 1; idx <= bstl; ++idx) acc += T3(cc, cs[idx - 1], x(idx));
        }
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    // convolve_interior!
    double rev[64];
    for (long i = 1 + bpc; i <= len - bpc - off; ++i) {
        const double cc = coeff(i);
        const double* cs = S;
        if (!(cc >= 0)) {
            const double sg = (d % 2 == 0) ? 1.0 : -1.0;
            for (int k = 0; k < stl; ++k) rev[k] = (d % 2 == 0) ? S[stl - 1 - k] : sg * S[stl - 1 - k];
            cs = rev;
        }
        double acc = 0.0;
        for (int idx = 1; idx <= stl; ++idx) {
            const double xv = cc < 0 ? x(i - stl + 1 + idx + off) : x(i + idx - off);
            acc += T3(cc, cs[idx - 1], xv);
        }
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    // convolve_BC_right!
    const double sgd = (d % 2 == 0) ? 1.0 : -1.0;  // (-1)^d
    for (int i = 1; i <= bpc + off; ++i) {
        const double cc = coeff(len - bpc + i - off);
        double acc = 0.0;
        if (cc < 0 && xl - stl - bpc + i >= 1 && i <= bpc + 1) {
            for (int k = 0; k < stl; ++k) rev[k] = sgd * S[stl - 1 - k];
            for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, rev[idx - 1], x(xl - stl + idx - bpc + i - 1));
        } else if (cc < 0 && xl - stl - bpc + i >= 1 && i > bpc + 1) {
            const double* hs = A.hi(bpc + off + 1 - i - 1);
            for (int k = 0; k < bstl; ++k) rev[k] = sgd * hs[bstl - 1 - k];
            for (int idx = 1; idx <= bstl; ++idx) acc += T3(cc, rev[idx - 1], x(xl - bstl + idx));
        } else if (cc >= 0 && i < off + 1) {
            for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, S[idx - 1], x(xl - stl + i + idx - off));
        } else {
            const double* hs = A.hi(i - 1);
            for (int idx = 1; idx <= bstl; ++idx) acc += T3(cc, hs[idx - 1], x(xl - bstl + idx));
        }
        double& o = out[(len - bpc + i - off - 1) * ostride];
        o = tail(acc, o, ow);
    }
}

// convolutions.jl:221-362 (generic) and :597-730 (padded) -- non-uniform upwind.
// `generic` selects the coeff_func branch of :234-253 (absent from the padded path).
template <class X, class C>
void upwind_nonuniform(const Op& A, const X& x, double* out, long ostride, const C& coeff, bool ow,
                       bool generic) {
    const long len = A.len;
    const int bpc = A.bpc, stl = A.stl, bstl = A.bstl, off = A.off;
    // convolve_interior!
    for (long i = bpc + 1; i <= len - bpc - off; ++i) {
        const double cc = coeff(i);
        int half;
        if (generic && A.coeff_func_sign > 0) half = 0;
        else if (generic && A.coeff_func_sign < 0) half = 1;
        else half = (cc >= 0) ? 0 : 1;
        const double* cs = A.st((int)(i - bpc - 1), half);
        double acc = 0.0;
        if (half == 0)
            for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], x(i + idx - off));
        else
            for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], x(i - stl + 1 + idx + off));
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    // convolve_BC_left!
    for (int i = 1; i <= bpc; ++i) {
        const double cc = coeff(i);
        double acc = 0.0;
        if (cc >= 0 && off == 0) {
            const double* cs = A.lo(i - 1, 0);
            for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], x(i + idx));
        } else if (cc >= 0 && i < off) {
            const double* cs = A.lo(i - 1, 0);
            for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], x(idx));
        } else if (cc >= 0 && i >= off) {
            const double* cs = A.lo(i - 1, 0);
            for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], x(i + idx - off));
        } else {
            const double* cs = A.lo(i - 1, 1);
            for (int idx = 1; idx <= bstl; ++idx) acc += T3(cc, cs[idx - 1], x(idx));
        }
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
    // convolve_BC_right!
    for (long i = len - bpc + 1 - off; i <= len; ++i) {
        const double cc = coeff(i);
        double acc = 0.0;
        if (cc < 0) {
            const double* cs = A.hi((int)(i - len + bpc + off - 1), 1);
            if (i <= len - off)
                for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], x(i - stl + 1 + idx + off));
            else
                for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], x(len - stl + 2 + idx));
        } else {
            if (i <= len - bpc) {
                const double* cs = A.st((int)(i - bpc - 1), 0);
                for (int idx = 1; idx <= stl; ++idx) acc += T3(cc, cs[idx - 1], x(i - stl + 1 + idx + off));
            } else {
                const double* cs = A.hi((int)(i - len + bpc + off - 1), 0);
                for (int idx = 1; idx <= bstl; ++idx) acc += T3(cc, cs[idx - 1], x(len - bstl + 2 + idx));
            }
        }
        double& o = out[(i - 1) * ostride];
        o = tail(acc, o, ow);
    }
}

struct VecCoeff {
    const double* c;
    long stride;
    double operator()(long i) const { return c[(i - 1) * stride]; }
};

// One operator applied to one line.  mode 1 = BoundaryPaddedVector methods
// (1-D `L*Q*u`), mode 0 = generic AbstractVector methods (N-D per-line
// `_mul!`, derivative_operator_functions.jl:27-69, and `L*x` on a plain
// padded vector).
template <class C>
void apply_line(const Op& A, const Line& L, double* out, long ostride, const C& coeff, bool ow, int mode) {
    if (!A.wind) {
        if (mode == 1) centred_padded(A, L, out, ostride, coeff, ow);
        else centred_generic(A, L, out, ostride, coeff, ow);
    } else if (A.uniform) {
        upwind_uniform(A, L, out, ostride, coeff, ow);
    } else {
        upwind_nonuniform(A, L, out, ostride, coeff, ow, mode == 0);
    }
}

}  // namespace

// ===========================================================================
// C ABI for the Python test harness
// ===========================================================================
extern "C" {

double orc_julia_powi(double x, long n) { return julia_powi(x, n); }

int orc_calculate_weights(int order, double x0, const double* x, int n, double* out) {
    if (order >= n || n <= 0) return -1;
    vec xv(x, x + n);
    vec w = calculate_weights(order, x0, xv);
    std::copy(w.begin(), w.end(), out);
    return 0;
}

void* orc_centered(int d, int a, const double* dx, int ndx, int len) {
    if (a < 2 || d < 0 || len < 1) return nullptr;
    // dx[1:len+1] and dx[end-bstl+1:end] are read (derivative_operator.jl:150-170)
    if (ndx != 1 && (ndx < len + 1 || ndx < d + a)) return nullptr;
    return centered(d, a, dx, ndx, len);
}

void* orc_upwind(int d, int a, const double* dx, int ndx, int len, int off) {
    if (off < 0 || off > (d + a - 1) / 2 || len < 1) return nullptr;
    // x = [0; cumsum(dx)] is read at x[1:len+2] (derivative_operator.jl:515-639)
    if (ndx != 1 && ndx < len + 1) return nullptr;
    return upwind(d, a, dx, ndx, len, off);
}

void orc_op_free(void* p) { delete static_cast<Op*>(p); }

// info: d,a,len,stl,bstl,bpc,off,wind,uniform,n_st,n_low,n_high,coeff_func_sign
void orc_op_info(const void* p, int* info) {
    const Op& A = *static_cast<const Op*>(p);
    int v[13] = {A.d, A.a, A.len, A.stl, A.bstl, A.bpc, A.off, A.wind, A.uniform,
                 A.n_st, A.n_low, A.n_high, A.coeff_func_sign};
    std::memcpy(info, v, sizeof(v));
}

void orc_op_tables(const void* p, double* stencil, double* low, double* high, double* coeff) {
    const Op& A = *static_cast<const Op*>(p);
    if (stencil) std::copy(A.stencil.begin(), A.stencil.end(), stencil);
    if (low) std::copy(A.low.begin(), A.low.end(), low);
    if (high) std::copy(A.high.begin(), A.high.end(), high);
    if (coeff) std::copy(A.coeff.begin(), A.coeff.end(), coeff);
}

// compute_coeffs!(coeff_func, zeros) for a Number or a Vector coeff_func
// (coefficient_functions.jl:7-15): coefficients = 0 + c.
void orc_op_set_coeff(void* p, const double* c, int nc, int coeff_func_sign) {
    Op& A = *static_cast<Op*>(p);
    for (int i = 0; i < A.len; ++i) A.coeff[i] = 0.0 + (nc == 1 ? c[0] : c[i]);
    A.coeff_func_sign = coeff_func_sign;
}

// c * L (derivative_operator_functions.jl:165-197): coefficients = c .* coefficients
void orc_op_scale_coeff(void* p, const double* c, int nc) {
    Op& A = *static_cast<Op*>(p);
    for (int i = 0; i < A.len; ++i) A.coeff[i] = (nc == 1 ? c[0] : c[i]) * A.coeff[i];
}

// Tolerance helper: the same operator with every table entry and coefficient
// replaced by its absolute value, so that applying it (with |BC| and |u|)
// gives sum_k |c_k * u_k| per point, ghost terms expanded.
void* orc_op_abs(const void* p) {
    Op* o = new Op(*static_cast<const Op*>(p));
    for (auto& v : o->stencil) v = std::fabs(v);
    for (auto& v : o->low) v = std::fabs(v);
    for (auto& v : o->high) v = std::fabs(v);
    for (auto& v : o->coeff) v = std::fabs(v);
    return o;
}

int orc_robin(const double* l, const double* r, const double* dx, int ndx, int order, void* out) {
    return robin(l, r, dx, ndx, order, static_cast<BC*>(out));
}

int orc_general(const double* al, int nl, const double* ar, int nr, const double* dx, int ndx, int order,
                void* out) {
    return general(al, nl, ar, nr, dx, ndx, order, static_cast<BC*>(out));
}

int orc_bc_size(void) { return (int)sizeof(BC); }

void orc_bc_ghosts(const void* q, const double* u, long n, double* l, double* r) {
    ghosts_1d(*static_cast<const BC*>(q), u, n, 1, *l, *r);
}

// 1-D `L*x` on a plain vector x of length len+2 (generic methods).
void orc_mul_generic(const void* p, const double* x, double* out, int overwrite) {
    const Op& A = *static_cast<const Op*>(p);
    Line L{x + 1, 1, x[0], x[A.len + 1], A.len};
    VecCoeff c{A.coeff.data(), 1};
    apply_line(A, L, out, 1, c, overwrite != 0, 0);
}

// 1-D `L * (l, u, r)` on a BoundaryPaddedVector (padded methods).
void orc_mul_padded(const void* p, double l, double r, const double* u, double* out, int overwrite) {
    const Op& A = *static_cast<const Op*>(p);
    Line L{u, 1, l, r, A.len};
    VecCoeff c{A.coeff.data(), 1};
    apply_line(A, L, out, 1, c, overwrite != 0, 1);
}

// Sum of terms  sum_t (L_t * Q_t) * u  on a column-major array of `ndims`
// dimensions.  ndims == 1 follows the BoundaryPaddedVector path; ndims > 1 the
// per-line generic path with ghosts from MultiDimDirectionalBC/ComposedMultiDimBC
// (multi_dim_bc_operators.jl:4-52, 212-252).  fields[t] (may be NULL) gives a
// full coefficient field: term t then acts on each line with coefficients =
// the field restricted to that line, i.e. one reference operator per line.
// The terms are summed left to right, as `sum(op -> op*u, ops)` does
// (composite_operators.jl:64-65).  `overwrite=0` adds the result to `out`.
int orc_apply_nd(int nterms, void* const* ops, const int* axes, const void* bcs, const double* const* fields,
                 int ndims, const long* sizes, const double* u, double* out, int overwrite, int nthreads);

// sum_k |c_k u_k| per point for the same terms (tolerance scale).
int orc_abs_scale_nd(int nterms, void* const* ops, const int* axes, const void* bcs, const double* const* fields,
                     int ndims, const long* sizes, const double* u, double* out) {
    g_abs = true;
    const int rc = orc_apply_nd(nterms, ops, axes, bcs, fields, ndims, sizes, u, out, 1, 1);
    g_abs = false;
    return rc;
}

// MultiDimBC{dim}(BCs::Array) (multi_dim_bc_operators.jl:91-93): line_bcs[t]
// (may be NULL) holds one BC per line of term t, in the column-major order of
// the other axes (the BCs array's own order); each line's ghosts are
// BCs[I, J] * u[I, :, J] (slice_rmul, :28-52), the 1-D ghost fill -- so a
// periodic BC among others wraps around its line -- except when every BC of
// the array is periodic, where the array's element type selects the N-D
// periodic padding with the edge planes (:221-228).
static int apply_nd_impl(int nterms, void* const* ops, const int* axes, const void* bcs, const double* const* fields,
                         const void* const* line_bcs, int ndims, const long* sizes, const double* u, double* out,
                         int overwrite, int nthreads);

int orc_apply_nd(int nterms, void* const* ops, const int* axes, const void* bcs, const double* const* fields,
                 int ndims, const long* sizes, const double* u, double* out, int overwrite, int nthreads) {
    return apply_nd_impl(nterms, ops, axes, bcs, fields, nullptr, ndims, sizes, u, out, overwrite, nthreads);
}

int orc_apply_nd_lines(int nterms, void* const* ops, const int* axes, const void* bcs, const double* const* fields,
                       const void* const* line_bcs, int ndims, const long* sizes, const double* u, double* out,
                       int overwrite, int nthreads) {
    return apply_nd_impl(nterms, ops, axes, bcs, fields, line_bcs, ndims, sizes, u, out, overwrite, nthreads);
}

int orc_abs_scale_nd_lines(int nterms, void* const* ops, const int* axes, const void* bcs,
                           const double* const* fields, const void* const* line_bcs, int ndims, const long* sizes,
                           const double* u, double* out) {
    g_abs = true;
    const int rc = apply_nd_impl(nterms, ops, axes, bcs, fields, line_bcs, ndims, sizes, u, out, 1, 1);
    g_abs = false;
    return rc;
}

static int apply_nd_impl(int nterms, void* const* ops, const int* axes, const void* bcs, const double* const* fields,
                         const void* const* line_bcs, int ndims, const long* sizes, const double* u, double* out,
                         int overwrite, int nthreads) {
    long total = 1;
    for (int k = 0; k < ndims; ++k) total *= sizes[k];
    const BC* bc = static_cast<const BC*>(bcs);
    vec acc(total, 0.0), term(total, 0.0);
    for (int t = 0; t < nterms; ++t) {
        const Op& A = *static_cast<const Op*>(ops[t]);
        const int ax = axes[t] - 1;
        if (ax < 0 || ax >= ndims || sizes[ax] != A.len) return -1;
        long stride = 1;
        for (int k = 0; k < ax; ++k) stride *= sizes[k];
        const long n = sizes[ax];
        const long nlines = total / n;
        const long inner = stride;
        const int mode = (ndims == 1) ? 1 : 0;
        double* dst = (t == 0) ? acc.data() : term.data();
        const BC* lb = (line_bcs && line_bcs[t]) ? static_cast<const BC*>(line_bcs[t]) : nullptr;
        bool all_periodic = lb != nullptr;
        for (long line = 0; lb && line < nlines && all_periodic; ++line) all_periodic = lb[line].kind == 1;
#if defined(_OPENMP)
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
        for (long line = 0; line < nlines; ++line) {
            const long lo = line % inner, hi = line / inner;
            const long base = lo + hi * inner * n;
            Line L;
            L.u = u + base;
            L.stride = stride;
            L.len = n;
            if (lb && !all_periodic) ghosts_1d(lb[line], L.u, n, stride, L.l, L.r);
            else if (lb) ghosts_nd(lb[line], L.u, n, stride, L.l, L.r);
            else if (ndims == 1) ghosts_1d(bc[t], L.u, n, stride, L.l, L.r);
            else ghosts_nd(bc[t], L.u, n, stride, L.l, L.r);
            if (fields && fields[t]) {
                VecCoeff c{fields[t] + base, stride};
                apply_line(A, L, dst + base, stride, c, true, mode);
            } else {
                VecCoeff c{A.coeff.data(), 1};
                apply_line(A, L, dst + base, stride, c, true, mode);
            }
        }
        if (t > 0)
            for (long i = 0; i < total; ++i) acc[i] = acc[i] + term[i];
    }
    for (long i = 0; i < total; ++i) out[i] = overwrite ? acc[i] : acc[i] + out[i];
    (void)nthreads;
    return 0;
}

// Array(L) (concretization.jl:8-52 centred; :556-671 upwind), column-major
// len x (len+2).
void orc_array_op(const void* p, double* M) {
    const Op& A = *static_cast<const Op*>(p);
    const long N = A.len, R = N;
    auto set = [&](long i, long j, double v) { M[(j - 1) * R + (i - 1)] = v; };
    std::fill(M, M + N * (N + 2), 0.0);
    const int bl = A.bpc, stl = A.stl, bstl = A.bstl, off = A.off;
    auto coeff = [&](long i) { return A.coeff[i - 1]; };
    if (!A.wind) {
        const int pivot = stl / 2;
        for (int i = 1; i <= bl; ++i)
            for (int k = 0; k < bstl; ++k) set(i, 1 + k, coeff(i) * A.lo(i - 1)[k]);
        for (long i = bl + 1; i <= N - bl; ++i) {
            const double* s = A.uniform ? A.st(0) : A.st((int)(i - bl - 1));
            for (int k = 0; k < stl; ++k) set(i, i + 1 - pivot + k, coeff(i) * s[k]);
        }
        for (long i = N - bl + 1; i <= N; ++i)
            for (int k = 0; k < bstl; ++k) set(i, N - bstl + 3 + k, coeff(i) * A.hi((int)(i - N + bl - 1))[k]);
        return;
    }
    const int d = A.d;
    const double sgd = (d % 2 == 0) ? 1.0 : -1.0;
    if (A.uniform) {
        const double* S = A.st(0);
        for (int i = 1; i <= bl; ++i) {
            const double c = coeff(i);
            if (c >= 0 && i + stl <= N + 2 && i >= off)
                for (int k = 0; k < stl; ++k) set(i, i + 1 - off + k, c * S[k]);
            else
                for (int k = 0; k < bstl; ++k) set(i, 1 + k, c * A.lo(i - 1)[k]);
        }
        for (long i = bl + 1; i <= N - bl - off; ++i) {
            const double c = coeff(i);
            if (c >= 0)
                for (int k = 0; k < stl; ++k) set(i, i + 1 - off + k, c * S[k]);
            else
                for (int k = 0; k < stl; ++k) set(i, i - stl + 2 + off + k, c * (sgd * S[stl - 1 - k]));
        }
        for (int i = 1; i <= bl + off; ++i) {
            const long row = N - bl + i - off;
            const double c = coeff(row);
            if (c < 0 && N + 2 - stl - bl + i >= 1 && i <= bl + 1) {
                for (int k = 0; k < stl; ++k) set(row, i + N - stl - bl + 2 + k, c * (sgd * S[stl - 1 - k]));
            } else if (c < 0 && N + 2 - stl - bl + i >= 1 && i > bl + 1) {
                const double* h = A.hi(bl + off + 1 - i - 1);
                for (int k = 0; k < bstl; ++k) set(row, N - bstl + 3 + k, c * (sgd * h[bstl - 1 - k]));
            } else if (c >= 0 && i < off + 1) {
                for (int k = 0; k < stl; ++k) set(row, N - stl + i - off + 3 + k, c * S[k]);
            } else {
                const double* h = A.hi(i - 1);
                for (int k = 0; k < bstl; ++k) set(row, N - bstl + 3 + k, c * h[k]);
            }
        }
        return;
    }
    for (int i = 1; i <= bl; ++i) {
        const double c = coeff(i);
        if (c >= 0 && off == 0)
            for (int k = 0; k < stl; ++k) set(i, i + 1 + k, c * A.lo(i - 1, 0)[k]);
        else if (c >= 0 && i < off)
            for (int k = 0; k < stl; ++k) set(i, 1 + k, c * A.lo(i - 1, 0)[k]);
        else if (c >= 0 && i >= off)
            for (int k = 0; k < stl; ++k) set(i, i + 1 - off + k, c * A.lo(i - 1, 0)[k]);
        else
            for (int k = 0; k < bstl; ++k) set(i, 1 + k, c * A.lo(i - 1, 1)[k]);
    }
    for (long i = bl + 1; i <= N - bl - off; ++i) {
        const double c = coeff(i);
        if (c >= 0)
            for (int k = 0; k < stl; ++k) set(i, i + 1 - off + k, c * A.st((int)(i - bl - 1), 0)[k]);
        else
            for (int k = 0; k < stl; ++k) set(i, i - stl + 2 + off + k, c * A.st((int)(i - bl - 1), 1)[k]);
    }
    for (long i = N - bl + 1 - off; i <= N; ++i) {
        const double c = coeff(i);
        const int hr = (int)(i - N + bl + off - 1);
        if (c < 0 && i <= N - off)
            for (int k = 0; k < stl; ++k) set(i, i - stl + 2 + off + k, c * A.hi(hr, 1)[k]);
        else if (c < 0)
            for (int k = 0; k < stl; ++k) set(i, N - stl + 3 + k, c * A.hi(hr, 1)[k]);
        else if (c >= 0 && i <= N - bl)
            for (int k = 0; k < stl; ++k) set(i, i - bstl + 2 + off + k, c * A.st((int)(i - bl - 1), 0)[k]);
        else
            for (int k = 0; k < bstl; ++k) set(i, N - bstl + 3 + k, c * A.hi(hr, 0)[k]);
    }
}

// Array(Q, N) (concretization.jl:187-192 affine, :227-230 periodic):
// Q_L (N+2) x N column-major, Q_b (N+2).
void orc_array_bc(const void* q, long N, double* QL, double* Qb) {
    const BC& b = *static_cast<const BC*>(q);
    const long R = N + 2;
    std::fill(QL, QL + R * N, 0.0);
    std::fill(Qb, Qb + R, 0.0);
    for (long i = 0; i < N; ++i) QL[i * R + (i + 1)] = 1.0;
    if (b.kind == 1) {
        QL[(N - 1) * R + 0] = 1.0;
        QL[0 * R + (N + 1)] = 1.0;
        return;
    }
    for (int j = 0; j < b.ml; ++j) QL[j * R + 0] = b.al[j];
    for (int j = 0; j < b.mr; ++j) QL[(N - b.mr + j) * R + (N + 1)] = b.ar[j];
    Qb[0] = b.bl;
    Qb[N + 1] = b.br;
}

// Shu-Osher SSP-RK3 on the RHS f(u) = sum_t (L_t Q_t) u (restated scheme;
// the reference leaves time stepping to OrdinaryDiffEq):
//   u1 = u + dt*f(u)
//   u2 = 0.75*u + 0.25*(u1 + dt*f(u1))
//   u  = (1/3)*u + (2/3)*(u2 + dt*f(u2))
int orc_ssprk3(int nterms, void* const* ops, const int* axes, const void* bcs, const double* const* fields,
               int ndims, const long* sizes, double* u, double dt, int nsteps, int nthreads) {
    long total = 1;
    for (int k = 0; k < ndims; ++k) total *= sizes[k];
    vec f(total), u1(total), u2(total);
    const double third = 1.0 / 3.0, two_third = 2.0 / 3.0;
    for (int s = 0; s < nsteps; ++s) {
        if (orc_apply_nd(nterms, ops, axes, bcs, fields, ndims, sizes, u, f.data(), 1, nthreads)) return -1;
        for (long i = 0; i < total; ++i) u1[i] = u[i] + dt * f[i];
        orc_apply_nd(nterms, ops, axes, bcs, fields, ndims, sizes, u1.data(), f.data(), 1, nthreads);
        for (long i = 0; i < total; ++i) u2[i] = 0.75 * u[i] + 0.25 * (u1[i] + dt * f[i]);
        orc_apply_nd(nterms, ops, axes, bcs, fields, ndims, sizes, u2.data(), f.data(), 1, nthreads);
        for (long i = 0; i < total; ++i) u[i] = third * u[i] + two_third * (u2[i] + dt * f[i]);
    }
    return 0;
}

// ---------------------------------------------------------------------------
// mul!(x_temp, L, M; overwrite) and L*M for L = DerivativeOperator{T,N} on an
// already padded array M (derivative_operator_functions.jl:17-69, 150-163):
// size(M, N) = size(x_temp, N) + 2, every other axis of M equal to x_temp's or
// 2 longer (then its first and last planes are stripped, :47-56); each line
// along N by the generic AbstractVector methods (convolutions.jl:17-22, 27-118).
// ---------------------------------------------------------------------------
int orc_mul_nd(const void* op_, int axis, int nd, const long* out_sizes, const long* in_sizes, const double* M,
               double* out, int overwrite, int absolute) {
    const Op& A = *static_cast<const Op*>(op_);
    const int a = axis - 1;
    if (a < 0 || a >= nd || nd > 8) return -1;
    long ps[8], os[8], ovol = 1, pvol = 1;
    for (int b = 0; b < nd; ++b) {
        if (b == a ? in_sizes[b] != out_sizes[b] + 2 : (in_sizes[b] != out_sizes[b] && in_sizes[b] != out_sizes[b] + 2))
            return -1;
        ps[b] = pvol;
        os[b] = ovol;
        pvol *= in_sizes[b];
        ovol *= out_sizes[b];
    }
    if (out_sizes[a] != A.len) return -1;
    const long L = out_sizes[a], nlines = ovol / L;
    g_abs = absolute != 0;  // sum |c_k u_k| with the real rows (tolerance scale)
    for (long line = 0; line < nlines; ++line) {
        long r = line, q = 0, ob = 0;
        for (int b = 0; b < nd; ++b) {
            if (b == a) continue;
            const long c = r % out_sizes[b];
            r /= out_sizes[b];
            q += (c + (in_sizes[b] == out_sizes[b] + 2 ? 1 : 0)) * ps[b];
            ob += c * os[b];
        }
        const double* x = M + q;
        Line Ln{x + ps[a], ps[a], x[0], x[(L + 1) * ps[a]], L};
        apply_line(A, Ln, out + ob, os[a], VecCoeff{A.coeff.data(), 1}, overwrite != 0, 0);
    }
    g_abs = false;
    return 0;
}

// ---------------------------------------------------------------------------
// Gradient / Divergence / Curl on padded arrays
// (vector_calculus_operators.jl:47-73, vector_calculus_convolutions.jl).
// kind 0 Gradient: M (s1+2, .., sN+2) -> out (s1, .., sN, N);
// kind 1 Divergence: M (s1+2, .., sN+2, N) -> out (s1, .., sN);
// kind 2 Curl: M (s+2, s+2, s+2, 3) -> out (s, s, s, 3).
// ops[a] is the operator of axis a+1 (CenteredDifference{a+1}(1, ...)).
// N = 2, 3 follow the specialised methods (:186-838 and the curl's :844-1067):
// each pass adds to out (`x_temp[...] += ...`) in the order BC_left, interior,
// BC_right, axes in order within each; the axes other than the differentiated
// one are read at the padded array's index equal to the output index
// (x[i + idx - mid, j], not x[i + idx - mid, j + 1]); the right boundary rows
// use coefficients[i].  Other N follow the generic per-line methods (:1-170),
// one operator after the other, on the minimally padded views (other axes at
// index + 1), whose right boundary rows read coefficients[1:bpc].
// overwrite = 1 starts from zeros (the `*` methods), 0 adds to out (mul!).
// absolute = 1 (with |tables| operators and |M|) gives sum_k |c_k u_k|.
// ---------------------------------------------------------------------------
namespace {
struct VcTerm {
    int in, out;  // component read (-1: scalar M) and written (-1: scalar out)
    double sg;    // -1 where the reference negates the coefficient (`-cur_coeff * ...`)
};
int vc_terms(int kind, int a, VcTerm* t) {
    if (kind == 0) {
        t[0] = VcTerm{-1, a, 1.0};
        return 1;
    }
    if (kind == 1) {
        t[0] = VcTerm{a, -1, 1.0};
        return 1;
    }
    // Curl, vector_calculus_convolutions.jl:871-907: along axis 1 x2 -= D u3, x3 += D u2;
    // axis 2: x1 += D u3, x3 -= D u1; axis 3: x1 -= D u2, x2 += D u1.
    static const VcTerm curl[3][2] = {{{2, 1, -1.0}, {1, 2, 1.0}},
                                      {{2, 0, 1.0}, {0, 2, -1.0}},
                                      {{1, 0, -1.0}, {0, 1, 1.0}}};
    t[0] = curl[a][0];
    t[1] = curl[a][1];
    return 2;
}
}  // namespace

int orc_vector_calculus(int kind, int nd, void* const* ops_, const double* M, double* out, int overwrite,
                        int absolute) {
    if (kind < 0 || kind > 2 || nd < 1 || nd > 8 || (kind == 2 && nd != 3)) return -1;
    const Op* ops[8];
    long s[8], ps[8], os[8], pvol = 1, ovol = 1;
    for (int a = 0; a < nd; ++a) {
        ops[a] = static_cast<const Op*>(ops_[a]);
        s[a] = ops[a]->len;
        ps[a] = pvol;
        os[a] = ovol;
        pvol *= s[a] + 2;
        ovol *= s[a];
    }
    const int ncomp = kind == 1 ? 1 : (kind == 0 ? nd : 3);
    if (overwrite)
        for (long n = 0; n < ovol * ncomp; ++n) out[n] = 0.0;
    g_abs = absolute != 0;
    if (nd == 2 || nd == 3) {
        const int bpc = ops[0]->bpc, stl = ops[0]->stl, bstl = ops[0]->bstl, mid = stl / 2;
        for (int ph = 0; ph < 3; ++ph) {  // convolve_BC_left!, convolve_interior!, convolve_BC_right!
            for (int a = 0; a < nd; ++a) {
                const Op& A = *ops[a];
                VcTerm tt[2];
                const int nt = vc_terms(kind, a, tt);
                for (long n = 0; n < ovol; ++n) {
                    long o[3], r = n;
                    for (int b = 0; b < nd; ++b) {
                        o[b] = r % s[b];
                        r /= s[b];
                    }
                    const long i = o[a] + 1, L = s[a];
                    const int phase = i <= bpc ? 0 : (i <= L - bpc ? 1 : 2);
                    if (phase != ph) continue;
                    long q = 0;  // other axes at the padded index equal to the output index
                    for (int b = 0; b < nd; ++b)
                        if (b != a) q += o[b] * ps[b];
                    const double* cs;
                    int nk;
                    long p0;  // first tap, 1-based padded position along axis a
                    if (phase == 0) {
                        cs = A.lo((int)i - 1);
                        nk = bstl;
                        p0 = 1;
                    } else if (phase == 1) {
                        cs = A.uniform ? A.st(0) : A.st((int)(i - bpc - 1));
                        nk = stl;
                        p0 = i - mid + 1;
                    } else {
                        cs = A.hi((int)(i - (L - bpc) - 1));
                        nk = bstl;
                        p0 = L - bstl + 3;
                    }
                    const double cc = A.coeff[i - 1];
                    for (int k = 0; k < nt; ++k) {
                        const double* x = M + (tt[k].in < 0 ? 0 : tt[k].in * pvol) + q;
                        double acc = 0.0;
                        for (int idx = 0; idx < nk; ++idx) acc += T3(tt[k].sg * cc, cs[idx], x[(p0 + idx - 1) * ps[a]]);
                        double& y = out[n + (tt[k].out < 0 ? 0 : tt[k].out * ovol)];
                        y = y + acc;
                    }
                }
            }
        }
    } else {
        if (kind == 2) {
            g_abs = false;
            return -1;
        }
        for (int a = 0; a < nd; ++a) {  // `for L in A.ops  mul!(x_temp, has_vector, L, M)`
            const Op& A = *ops[a];
            const long L = s[a], nlines = ovol / L;
            for (long line = 0; line < nlines; ++line) {
                long r = line, q = 0, ob = 0;
                for (int b = 0; b < nd; ++b) {
                    if (b == a) continue;
                    const long c = r % s[b];
                    r /= s[b];
                    q += (c + 1) * ps[b];
                    ob += c * os[b];
                }
                const double* x = M + (kind == 1 ? a * pvol : 0) + q;
                Line Ln{x + ps[a], ps[a], x[0], x[(L + 1) * ps[a]], L};
                double* y = out + ob + (kind == 0 ? a * ovol : 0);
                apply_line(A, Ln, y, os[a], VecCoeff{A.coeff.data(), 1}, false, 0);
            }
        }
    }
    g_abs = false;
    return 0;
}

}  // extern "C"
