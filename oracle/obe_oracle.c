/*
 * obe_oracle.c -- CPU FP64 restatement of the reference's Lindblad `expanded_sparse` path.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline); see obe_oracle.h.
 * Compile with -ffp-contract=off: the reference is Rust, which never fuses a*b+c, and the
 * oracle must round like it on every host (the GPU machine is aarch64, where gcc contracts by
 * default).
 *
 * Complex arithmetic follows crate num-complex 0.4.6 (rust/Cargo.lock:108-109), whose
 * published formulas are restated in the cx_* helpers below: naive product and quotient,
 * exp/sin/cos/tan via real exp/sin/cos/sinh/cosh, ln via hypot/atan2, powc as exp(y*ln x)
 * with x^0 = 1.
 */
#include "obe_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------------ */
/* errors                                                                                      */

typedef struct {
    char msg[512];
    int set;
} errbuf;

static int fail(errbuf* e, const char* fmt, ...) {
    if (!e->set) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(e->msg, sizeof e->msg, fmt, ap);
        va_end(ap);
        e->set = 1;
    }
    return 1;
}

static void copy_err(const errbuf* e, char* err, size_t err_len) {
    if (err && err_len) {
        snprintf(err, err_len, "%s", e->msg);
    }
}

/* Rust's Display for f64 (used in the reference's messages): shortest round-trip digits,
   always positional (no exponent), integers without a fraction. */
static void fmt_f64(double v, char* out, size_t len) {
    if (isnan(v)) { snprintf(out, len, "NaN"); return; }
    if (isinf(v)) { snprintf(out, len, v > 0 ? "inf" : "-inf"); return; }
    if (v == 0.0) { snprintf(out, len, signbit(v) ? "-0" : "0"); return; }
    char buf[64];
    int prec;
    for (prec = 1; prec <= 17; ++prec) {
        snprintf(buf, sizeof buf, "%.*e", prec - 1, v);
        if (strtod(buf, NULL) == v) break;
    }
    /* buf = [-]d.ddddde[+-]XX */
    char digits[32];
    int nd = 0, neg = 0;
    const char* p = buf;
    if (*p == '-') { neg = 1; ++p; }
    for (; *p && *p != 'e'; ++p) if (*p != '.') digits[nd++] = *p;
    int exp10 = atoi(p + 1);
    while (nd > 1 && digits[nd - 1] == '0') --nd;
    char res[400];
    int k = 0;
    if (neg) res[k++] = '-';
    if (exp10 >= 0) {
        for (int i = 0; i <= exp10 || i < nd; ++i) {
            if (i == exp10 + 1) res[k++] = '.';
            res[k++] = i < nd ? digits[i] : '0';
            if (i >= exp10 && i >= nd - 1) break;
        }
    } else {
        res[k++] = '0';
        res[k++] = '.';
        for (int i = 0; i < -exp10 - 1; ++i) res[k++] = '0';
        for (int i = 0; i < nd; ++i) res[k++] = digits[i];
    }
    res[k] = 0;
    snprintf(out, len, "%s", res);
}

/* ------------------------------------------------------------------------------------------ */
/* complex arithmetic (num-complex 0.4.6)                                                      */

typedef struct { double re, im; } cx;

static inline cx C(double re, double im) { cx z = {re, im}; return z; }
static inline cx cx_add(cx a, cx b) { return C(a.re + b.re, a.im + b.im); }
static inline cx cx_sub(cx a, cx b) { return C(a.re - b.re, a.im - b.im); }
static inline cx cx_mul(cx a, cx b) { return C(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cx cx_div(cx a, cx b) {
    double ns = b.re * b.re + b.im * b.im;
    double re = a.re * b.re + a.im * b.im;
    double im = a.im * b.re - a.re * b.im;
    return C(re / ns, im / ns);
}
static inline cx cx_neg(cx a) { return C(-a.re, -a.im); }
static inline cx cx_conj(cx a) { return C(a.re, -a.im); }
static inline double cx_norm(cx a) { return hypot(a.re, a.im); }
static inline cx cx_from_polar(double r, double th) { return C(r * cos(th), r * sin(th)); }
static cx cx_exp(cx z) {
    double re = z.re, im = z.im;
    if (isinf(re)) {
        if (re < 0.0) {
            if (!isfinite(im)) return C(0.0, 0.0);
        } else if (im == 0.0 || !isfinite(im)) {
            if (isinf(im)) im = NAN;
            return C(re, im);
        }
    } else if (isnan(re) && im == 0.0) {
        return z;
    }
    return cx_from_polar(exp(re), im);
}
static inline cx cx_ln(cx z) { return C(log(cx_norm(z)), atan2(z.im, z.re)); }
static cx cx_powc(cx x, cx y) {
    if (y.re == 0.0 && y.im == 0.0) return C(1.0, 0.0);
    return cx_exp(cx_mul(y, cx_ln(x)));
}
static inline cx cx_sin(cx z) { return C(sin(z.re) * cosh(z.im), cos(z.re) * sinh(z.im)); }
static inline cx cx_cos(cx z) { return C(cos(z.re) * cosh(z.im), -sin(z.re) * sinh(z.im)); }
static cx cx_tan(cx z) {
    double tr = z.re + z.re, ti = z.im + z.im;
    double d = cos(tr) + cosh(ti);
    return C(sin(tr) / d, sinh(ti) / d);
}

/* ------------------------------------------------------------------------------------------ */
/* runtime values and the expression VM (eval.rs)                                              */

enum {
    OP_CONST = 1, OP_SLOT = 2, OP_TEMP = 3, OP_TIME = 4, OP_ADD = 5, OP_SUB = 6, OP_MUL = 7,
    OP_DIV = 8, OP_POW = 9, OP_NEG = 10, OP_CONJ = 11, OP_BUILTIN = 12, OP_HELPER = 13,
    OP_GT = 14, OP_GE = 15, OP_LT = 16, OP_LE = 17, OP_EQ = 18, OP_NE = 19
};

typedef struct {
    int is_tuple;
    cx s;
    const cx* items;
    int64_t len;
} rv;

typedef struct {
    int64_t n;
    int32_t* op;
    int64_t* index;
    int32_t* argc;
    int32_t* function;
    cx* value;
    int scalar_only;
    int output_is_tuple;
    int uses_time;
} expr_t;

/* arena for the tuple temporaries of one evaluation: a list of blocks that never move, so
   tuple pointers already on the VM stack stay valid while later tuples are allocated */
typedef struct {
    cx** blocks;
    int64_t n_blocks, cap_blocks;
    int64_t used, cap;      /* of the last block */
} arena;

static void arena_reset(arena* a) {
    for (int64_t i = 0; i < a->n_blocks; ++i) free(a->blocks[i]);
    a->n_blocks = 0;
    a->used = a->cap = 0;
}

static void arena_free(arena* a) {
    arena_reset(a);
    free(a->blocks);
    a->blocks = NULL;
    a->cap_blocks = 0;
}

static cx* arena_alloc(arena* a, int64_t n) {
    if (n <= 0) n = 1;
    if (a->n_blocks == 0 || a->used + n > a->cap) {
        int64_t cap = n > 64 ? n : 64;
        if (a->n_blocks == a->cap_blocks) {
            a->cap_blocks = a->cap_blocks ? 2 * a->cap_blocks : 8;
            a->blocks = (cx**)realloc(a->blocks, sizeof(cx*) * (size_t)a->cap_blocks);
        }
        a->blocks[a->n_blocks++] = (cx*)malloc(sizeof(cx) * (size_t)cap);
        a->used = 0;
        a->cap = cap;
    }
    cx* q = a->blocks[a->n_blocks - 1] + a->used;
    a->used += n;
    return q;
}

typedef struct {
    int64_t n;          /* grid length */
    double* grid;
    double* coef;       /* [4*(n-1)] */
} pchip_table;

/* PchipTable::from_grid_values (plan.rs:34-80) */
static int pchip_build(pchip_table* tb, const double* grid, const double* values, int64_t n, errbuf* e) {
    tb->n = n;
    tb->grid = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    memcpy(tb->grid, grid, sizeof(double) * (size_t)n);
    tb->coef = NULL;
    if (n < 2) return 0;
    double* h = (double*)malloc(sizeof(double) * (size_t)(n - 1));
    double* delta = (double*)malloc(sizeof(double) * (size_t)(n - 1));
    double* d = (double*)malloc(sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n - 1; ++i) {
        h[i] = grid[i + 1] - grid[i];
        if (h[i] <= 0.0) {
            free(h); free(delta); free(d);
            return fail(e, "pchip grid must be strictly increasing");
        }
        delta[i] = (values[i + 1] - values[i]) / h[i];
    }
    d[0] = delta[0];
    d[n - 1] = delta[n - 2];
    for (int64_t i = 1; i < n - 1; ++i) {
        double s0 = delta[i - 1] > 0 ? 1.0 : (delta[i - 1] < 0 ? -1.0 : (signbit(delta[i - 1]) ? -1.0 : 1.0));
        double s1 = delta[i] > 0 ? 1.0 : (delta[i] < 0 ? -1.0 : (signbit(delta[i]) ? -1.0 : 1.0));
        if (s0 != s1 || delta[i - 1] == 0.0 || delta[i] == 0.0) {
            d[i] = 0.0;
        } else {
            double w1 = 2.0 * h[i] + h[i - 1];
            double w2 = h[i] + 2.0 * h[i - 1];
            d[i] = (w1 + w2) / (w1 / delta[i - 1] + w2 / delta[i]);
        }
    }
    tb->coef = (double*)malloc(sizeof(double) * 4 * (size_t)(n - 1));
    for (int64_t i = 0; i < n - 1; ++i) {
        tb->coef[4 * i + 0] = values[i];
        tb->coef[4 * i + 1] = d[i];
        tb->coef[4 * i + 2] = (3.0 * delta[i] - 2.0 * d[i] - d[i + 1]) / h[i];
        tb->coef[4 * i + 3] = (d[i] + d[i + 1] - 2.0 * delta[i]) / (h[i] * h[i]);
    }
    free(h); free(delta); free(d);
    return 0;
}

/* PchipTable::evaluate (plan.rs:82-115) */
static double pchip_eval(const pchip_table* tb, double x, int64_t* hint) {
    int64_t n = tb->n;
    if (n < 2) return 0.0; /* a 1-point table has no coefficients: evaluates to 0 */
    if (x <= tb->grid[0]) { *hint = 0; return tb->coef[0]; }
    if (x >= tb->grid[n - 1]) {
        int64_t last = n - 2;
        *hint = last;
        double dx = tb->grid[n - 1] - tb->grid[last];
        const double* c = tb->coef + 4 * last;
        return c[0] + dx * (c[1] + dx * (c[2] + dx * c[3]));
    }
    int64_t i;
    if (*hint < n - 1 && tb->grid[*hint] <= x && x <= tb->grid[*hint + 1]) {
        i = *hint;
    } else {
        /* partition_point(|g| g <= x) - 1, clamped */
        int64_t lo = 0, hi = n;
        while (lo < hi) {
            int64_t mid = lo + (hi - lo) / 2;
            if (tb->grid[mid] <= x) lo = mid + 1; else hi = mid;
        }
        i = lo > 0 ? lo - 1 : 0;
        if (i > n - 2) i = n - 2;
        *hint = i;
    }
    double dx = x - tb->grid[i];
    const double* c = tb->coef + 4 * i;
    return c[0] + dx * (c[1] + dx * (c[2] + dx * c[3]));
}

static int as_scalar(const rv* v, cx* out, errbuf* e) {
    if (v->is_tuple) return fail(e, "sequence value used where scalar was required");
    *out = v->s;
    return 0;
}

static int as_real(const rv* v, double* out, errbuf* e) {
    cx s = {0.0, 0.0};
    if (as_scalar(v, &s, e)) return 1;
    if (fabs(s.im) > 1e-12) return fail(e, "complex value used where real scalar was required");
    *out = s.re;
    return 0;
}

static double rem_euclid(double a, double b) {
    double r = fmod(a, b);
    return r < 0.0 ? r + fabs(b) : r;
}

static const double PI_ = 3.14159265358979323846;
static const double ED_XTB = 0.315 * 1.602176634e-19 * 5.29177210544e-11;

static double gaussian_2d(double x, double y, double a, double mx, double my, double sx, double sy) {
    double dx = x - mx, dy = y - my;
    return a * exp(-((dx * dx) / (2.0 * sx * sx) + (dy * dy) / (2.0 * sy * sy)));
}

static double gaussian_2d_rotated(double x, double y, double amp, double mx, double my, double sx,
                                  double sy, double th) {
    double ct = cos(th), st = sin(th);
    double a = ct * ct / (2.0 * sx * sx) + st * st / (2.0 * sy * sy);
    double b = sin(2.0 * th) / (2.0 * sx * sx) - sin(2.0 * th) / (2.0 * sy * sy);
    double c = st * st / (2.0 * sx * sx) + ct * ct / (2.0 * sy * sy);
    double dx = x - mx, dy = y - my;
    return amp * exp(-(a * dx * dx + b * dx * dy + c * dy * dy));
}

static double rabi_from_intensity(double intensity, double coupling, double dipole) {
    const double hbar = 1.0545718176461565e-34, c = 299792458.0, eps0 = 8.8541878128e-12;
    double field = sqrt(intensity * 2.0 / (c * eps0));
    return field * coupling * dipole / hbar;
}

static int multipass_intensity(double x, double y, const rv* amps, const rv* xl, const rv* yl,
                               double sx, double sy, double* out, errbuf* e) {
    if (!amps->is_tuple || !xl->is_tuple || !yl->is_tuple) return fail(e, "helper expected tuple argument");
    if (amps->len != xl->len || amps->len != yl->len) return fail(e, "multipass helper tuple lengths do not match");
    double acc = 0.0;
    for (int64_t i = 0; i < amps->len; ++i) {
        rv a = {0, amps->items[i], NULL, 0}, bx = {0, xl->items[i], NULL, 0}, by = {0, yl->items[i], NULL, 0};
        double av, xv, yv;
        if (as_real(&a, &av, e) || as_real(&bx, &xv, e) || as_real(&by, &yv, e)) return 1;
        acc += gaussian_2d(x, y, av, xv, yv, sx, sy);
    }
    *out = acc;
    return 0;
}

/* pchip_interp (eval.rs:305-351): direct evaluation from tuples */
static int pchip_interp_direct(double x, const rv* grid, const rv* vals, double* out, errbuf* e) {
    if (!grid->is_tuple || !vals->is_tuple) return fail(e, "helper expected tuple argument");
    if (grid->len != vals->len) return fail(e, "pchip_interp grid and values must have the same length");
    int64_t n = grid->len;
    if (n < 2) {
        if (n == 1) {
            rv v = {0, vals->items[0], NULL, 0};
            return as_real(&v, out, e);
        }
        return fail(e, "pchip_interp grid must contain at least one point");
    }
    double* g = (double*)malloc(sizeof(double) * (size_t)n);
    double* v = (double*)malloc(sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) { g[i] = grid->items[i].re; v[i] = vals->items[i].re; }
    int rc = 0;
    if (x <= g[0]) { *out = v[0]; goto done; }
    if (x >= g[n - 1]) { *out = v[n - 1]; goto done; }
    {
        double* h = (double*)malloc(sizeof(double) * (size_t)(n - 1));
        double* delta = (double*)malloc(sizeof(double) * (size_t)(n - 1));
        double* d = (double*)malloc(sizeof(double) * (size_t)n);
        for (int64_t i = 0; i < n - 1; ++i) {
            h[i] = g[i + 1] - g[i];
            if (h[i] <= 0.0) {
                free(h); free(delta); free(d);
                rc = fail(e, "pchip_interp grid must be strictly increasing");
                goto done;
            }
            delta[i] = (v[i + 1] - v[i]) / h[i];
        }
        d[0] = delta[0];
        d[n - 1] = delta[n - 2];
        for (int64_t i = 1; i < n - 1; ++i) {
            double s0 = signbit(delta[i - 1]) ? -1.0 : 1.0, s1 = signbit(delta[i]) ? -1.0 : 1.0;
            if (s0 != s1 || delta[i - 1] == 0.0 || delta[i] == 0.0) d[i] = 0.0;
            else {
                double w1 = 2.0 * h[i] + h[i - 1], w2 = h[i] + 2.0 * h[i - 1];
                d[i] = (w1 + w2) / (w1 / delta[i - 1] + w2 / delta[i]);
            }
        }
        int64_t idx = 0;
        for (int64_t i = 0; i < n - 1; ++i) {
            if (x < g[i + 1] || i == n - 2) { idx = i; break; }
        }
        double t = (x - g[idx]) / h[idx], t2 = t * t, t3 = t2 * t;
        double h00 = 2.0 * t3 - 3.0 * t2 + 1.0, h10 = t3 - 2.0 * t2 + t, h01 = -2.0 * t3 + 3.0 * t2, h11 = t3 - t2;
        *out = h00 * v[idx] + h10 * h[idx] * d[idx] + h01 * v[idx + 1] + h11 * h[idx] * d[idx + 1];
        free(h); free(delta); free(d);
    }
done:
    free(g); free(v);
    return rc;
}

/* linear_interp (eval.rs:359-386) */
static int linear_interp(double x, const rv* grid, const rv* vals, double* out, errbuf* e) {
    if (!grid->is_tuple || !vals->is_tuple) return fail(e, "helper expected tuple argument");
    if (grid->len != vals->len) return fail(e, "linear_interp grid and values must have the same length");
    if (grid->len == 0) return fail(e, "linear_interp grid must contain at least one point");
    rv v0 = {0, vals->items[0], NULL, 0};
    if (grid->len == 1) return as_real(&v0, out, e);
    rv g0 = {0, grid->items[0], NULL, 0};
    double first;
    if (as_real(&g0, &first, e)) return 1;
    if (x <= first) return as_real(&v0, out, e);
    for (int64_t i = 0; i < grid->len - 1; ++i) {
        rv l = {0, grid->items[i], NULL, 0}, r = {0, grid->items[i + 1], NULL, 0};
        double left, right;
        if (as_real(&l, &left, e) || as_real(&r, &right, e)) return 1;
        if (right <= left) return fail(e, "linear_interp grid must be strictly increasing");
        if (x <= right) {
            rv yl = {0, vals->items[i], NULL, 0}, yr = {0, vals->items[i + 1], NULL, 0};
            double a, b;
            if (as_real(&yl, &a, e) || as_real(&yr, &b, e)) return 1;
            double frac = (x - left) / (right - left);
            *out = a + frac * (b - a);
            return 0;
        }
    }
    rv vl = {0, vals->items[vals->len - 1], NULL, 0};
    return as_real(&vl, out, e);
}

/* apply_helper_scalar (eval.rs:664-789); args are scalars, scalar_arg takes the real part */
static int helper_scalar(int32_t fid, const cx* a, int64_t argc, cx* out, errbuf* e) {
#define SA(i) ((i) < argc ? a[i].re : 0.0)
    switch (fid) {
    case 1: *out = C(gaussian_2d(SA(0), SA(1), SA(2), SA(3), SA(4), SA(5), SA(6)), 0.0); return 0;
    case 2: *out = C(gaussian_2d_rotated(SA(0), SA(1), SA(2), SA(3), SA(4), SA(5), SA(6), SA(7)), 0.0); return 0;
    case 3: {
        double phi = SA(1) * sin(SA(2) * SA(0));
        *out = C(cos(phi), sin(phi));
        return 0;
    }
    case 4: *out = C(0.5 * (1.0 + (sin(SA(1) * SA(0) + SA(2)) >= 0.0 ? 1.0 : -1.0)), 0.0); return 0;
    case 5: {
        double theta = 0.5 * SA(1) * sin(SA(2) * SA(0));
        double v = 0.5 * (cos(theta) + sin(theta));
        *out = C(v, v);
        return 0;
    }
    case 6: *out = C(rem_euclid((SA(1) * SA(0) + SA(2)) / (2.0 * PI_), 1.0), 0.0); return 0;
    case 7: {
        double period = SA(1) + SA(2);
        double duty = SA(1) / period;
        double frac = rem_euclid(2.0 * PI_ * SA(0) / period + SA(3), 2.0 * PI_) / (2.0 * PI_);
        *out = C(frac < duty ? 1.0 : 0.0, 0.0);
        return 0;
    }
    case 8: case 10: case 14: case 16:
        return fail(e, "tuple-valued helper used in scalar evaluator");
    case 15: {
        double dx = SA(0) - SA(1);
        *out = C(exp(-dx * dx / (2.0 * SA(2) * SA(2))), 0.0);
        return 0;
    }
    case 9: *out = C(rabi_from_intensity(SA(0), SA(1), argc > 2 ? SA(2) : ED_XTB), 0.0); return 0;
    case 11: {
        double inten = gaussian_2d(SA(0), SA(1), SA(2), SA(3), SA(4), SA(5), SA(6));
        *out = C(rabi_from_intensity(inten, SA(7), argc > 8 ? SA(8) : ED_XTB), 0.0);
        return 0;
    }
    case 12: {
        double frac = rem_euclid(SA(0) * SA(2) + SA(3) / (2.0 * PI_), 1.0);
        if (frac <= 0.0) frac += 1.0;
        *out = C(frac < SA(1) ? 1.0 : 0.0, 0.0);
        return 0;
    }
    case 13: {
        double q = floor((SA(0) - SA(1)) / SA(2));
        long long nq;
        if (isnan(q)) nq = 0;
        else if (q >= 9.2e18) nq = 9223372036854775807LL;
        else if (q <= -9.2e18) nq = (-9223372036854775807LL - 1);
        else nq = (long long)q;
        *out = C(nq % 2 == 0 ? 1.0 : -1.0, 0.0);
        return 0;
    }
    default: {
        return fail(e, "unknown helper function id %d", fid);
    }
    }
#undef SA
}

static int builtin_scalar(int32_t fid, cx v, cx* out, errbuf* e) {
    switch (fid) {
    case 1: *out = cx_sin(v); return 0;
    case 2: *out = cx_cos(v); return 0;
    case 3: *out = cx_tan(v); return 0;
    case 4: *out = cx_exp(v); return 0;
    case 5: *out = C(cx_norm(v), 0.0); return 0;
    case 6: *out = C(v.re, 0.0); return 0;
    case 7: *out = C(v.im, 0.0); return 0;
    default: return fail(e, "unknown builtin function id %d", fid);
    }
}

/* eval_scalar_expression_into (eval.rs:791-911) */
static int eval_scalar(const expr_t* x, const rv* slots, double t, cx* stack, cx* out, errbuf* e) {
    int64_t sp = 0;
    for (int64_t k = 0; k < x->n; ++k) {
        int32_t op = x->op[k];
        switch (op) {
        case OP_CONST: stack[sp++] = x->value[k]; break;
        case OP_SLOT:
            if (as_scalar(&slots[x->index[k]], &stack[sp], e)) return 1;
            ++sp;
            break;
        case OP_TEMP: return fail(e, "sequence value used where scalar was required");
        case OP_TIME: stack[sp++] = C(t, 0.0); break;
        case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_POW: {
            if (sp < 2) {
                const char* nm = op == OP_ADD ? "ADD" : op == OP_SUB ? "SUB" : op == OP_MUL ? "MUL" : op == OP_DIV ? "DIV" : "POW";
                return fail(e, "stack underflow on %s", nm);
            }
            cx r = stack[--sp], l = stack[--sp], v;
            if (op == OP_ADD) v = cx_add(l, r);
            else if (op == OP_SUB) v = cx_sub(l, r);
            else if (op == OP_MUL) v = cx_mul(l, r);
            else if (op == OP_DIV) v = cx_div(l, r);
            else v = cx_powc(l, r);
            stack[sp++] = v;
            break;
        }
        case OP_NEG:
            if (sp < 1) return fail(e, "stack underflow on NEG");
            stack[sp - 1] = cx_neg(stack[sp - 1]);
            break;
        case OP_CONJ:
            if (sp < 1) return fail(e, "stack underflow on CONJ");
            stack[sp - 1] = cx_conj(stack[sp - 1]);
            break;
        case OP_BUILTIN: {
            int64_t argc = x->argc[k];
            if (sp < argc) return fail(e, "stack underflow on BUILTIN_FUNC");
            int64_t start = sp - argc;
            cx r;
            if (builtin_scalar(x->function[k], stack[start], &r, e)) return 1;
            sp = start;
            stack[sp++] = r;
            break;
        }
        case OP_HELPER: {
            int64_t argc = x->argc[k];
            if (sp < argc) return fail(e, "stack underflow on HELPER_FUNC");
            int64_t start = sp - argc;
            cx r;
            if (helper_scalar(x->function[k], stack + start, argc, &r, e)) return 1;
            sp = start;
            stack[sp++] = r;
            break;
        }
        case OP_GT: case OP_GE: case OP_LT: case OP_LE: case OP_EQ: case OP_NE: {
            if (sp < 2) return fail(e, "stack underflow on comparison");
            double r = stack[sp - 1].re, l = stack[sp - 2].re;
            sp -= 2;
            int res = op == OP_GT ? l > r : op == OP_GE ? l >= r : op == OP_LT ? l < r : op == OP_LE ? l <= r : op == OP_EQ ? l == r : l != r;
            stack[sp++] = C(res ? 1.0 : 0.0, 0.0);
            break;
        }
        default: return fail(e, "unknown instruction op %d", op);
        }
    }
    if (sp != 1) return fail(e, "expression evaluation did not end with a single stack value");
    *out = stack[0];
    return 0;
}

typedef struct {
    const pchip_table* tables;
    int64_t n_tables;
    int64_t* hints;
} pchip_ctx;

static int elementwise(const rv* l, const rv* r, int op, arena* ar, rv* out, errbuf* e) {
    cx (*f)(cx, cx) = op == OP_ADD ? cx_add : op == OP_SUB ? cx_sub : op == OP_MUL ? cx_mul : op == OP_DIV ? cx_div : cx_powc;
    if (!l->is_tuple && !r->is_tuple) { out->is_tuple = 0; out->s = f(l->s, r->s); return 0; }
    int64_t n;
    if (l->is_tuple && r->is_tuple) {
        if (l->len != r->len) return fail(e, "tuple lengths do not match for elementwise operation");
        n = l->len;
    } else {
        n = l->is_tuple ? l->len : r->len;
    }
    cx* items = arena_alloc(ar, n);
    for (int64_t i = 0; i < n; ++i) {
        cx a = l->is_tuple ? l->items[i] : l->s;
        cx b = r->is_tuple ? r->items[i] : r->s;
        items[i] = f(a, b);
    }
    out->is_tuple = 1;
    out->items = items;
    out->len = n;
    return 0;
}

/* apply_helper (eval.rs:388-451) on general runtime values */
static int helper_general(int32_t fid, const rv* a, int64_t argc, rv* out, errbuf* e) {
    double v0, v1, v5, v6, v7, v8, res;
    switch (fid) {
    case 8:
        if (argc < 7) return fail(e, "helper expected tuple argument");
        if (as_real(&a[0], &v0, e) || as_real(&a[1], &v1, e) || as_real(&a[5], &v5, e) || as_real(&a[6], &v6, e)) return 1;
        if (multipass_intensity(v0, v1, &a[2], &a[3], &a[4], v5, v6, &res, e)) return 1;
        out->is_tuple = 0; out->s = C(res, 0.0);
        return 0;
    case 10:
        if (argc < 8) return fail(e, "helper expected tuple argument");
        if (as_real(&a[0], &v0, e) || as_real(&a[1], &v1, e) || as_real(&a[5], &v5, e) || as_real(&a[6], &v6, e)) return 1;
        if (multipass_intensity(v0, v1, &a[2], &a[3], &a[4], v5, v6, &res, e)) return 1;
        if (as_real(&a[7], &v7, e)) return 1;
        v8 = ED_XTB;
        if (argc > 8 && as_real(&a[8], &v8, e)) return 1;
        out->is_tuple = 0; out->s = C(rabi_from_intensity(res, v7, v8), 0.0);
        return 0;
    case 14:
        if (argc < 3) return fail(e, "helper expected tuple argument");
        if (as_real(&a[0], &v0, e) || linear_interp(v0, &a[1], &a[2], &res, e)) return 1;
        out->is_tuple = 0; out->s = C(res, 0.0);
        return 0;
    case 16:
        if (argc < 3) return fail(e, "helper expected tuple argument");
        if (as_real(&a[0], &v0, e) || pchip_interp_direct(v0, &a[1], &a[2], &res, e)) return 1;
        out->is_tuple = 0; out->s = C(res, 0.0);
        return 0;
    default: {
        cx sa[32];
        if (argc > 32) return fail(e, "too many helper arguments");
        for (int64_t i = 0; i < argc; ++i)
            if (as_scalar(&a[i], &sa[i], e)) return 1;
        cx r;
        if (helper_scalar(fid, sa, argc, &r, e)) return 1;
        out->is_tuple = 0; out->s = r;
        return 0;
    }
    }
}

/* eval_expression_into_with_pchip (eval.rs:478-657) */
static int eval_general(const expr_t* x, const rv* slots, double t, rv* stack, arena* ar,
                        const pchip_ctx* pc, rv* out, errbuf* e) {
    int64_t sp = 0;
    arena_reset(ar);
    for (int64_t k = 0; k < x->n; ++k) {
        int32_t op = x->op[k];
        switch (op) {
        case OP_CONST: stack[sp].is_tuple = 0; stack[sp].s = x->value[k]; ++sp; break;
        case OP_SLOT: stack[sp++] = slots[x->index[k]]; break;
        case OP_TEMP: return fail(e, "temporary values are not part of a decomposed plan");
        case OP_TIME: stack[sp].is_tuple = 0; stack[sp].s = C(t, 0.0); ++sp; break;
        case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_POW: {
            if (sp < 2) {
                const char* nm = op == OP_ADD ? "ADD" : op == OP_SUB ? "SUB" : op == OP_MUL ? "MUL" : op == OP_DIV ? "DIV" : "POW";
                return fail(e, "stack underflow on %s", nm);
            }
            rv r = stack[--sp], l = stack[--sp], v;
            if (elementwise(&l, &r, op, ar, &v, e)) return 1;
            stack[sp++] = v;
            break;
        }
        case OP_NEG: case OP_CONJ: {
            if (sp < 1) return fail(e, op == OP_NEG ? "stack underflow on NEG" : "stack underflow on CONJ");
            rv v = stack[sp - 1];
            if (!v.is_tuple) {
                stack[sp - 1].s = op == OP_NEG ? cx_neg(v.s) : cx_conj(v.s);
            } else {
                cx* items = arena_alloc(ar, v.len);
                for (int64_t i = 0; i < v.len; ++i) items[i] = op == OP_NEG ? cx_neg(v.items[i]) : cx_conj(v.items[i]);
                stack[sp - 1].items = items;
            }
            break;
        }
        case OP_BUILTIN: {
            int64_t argc = x->argc[k];
            if (sp < argc) return fail(e, "stack underflow on BUILTIN_FUNC");
            int64_t start = sp - argc;
            cx s, r;
            if (as_scalar(&stack[start], &s, e)) return 1;
            if (builtin_scalar(x->function[k], s, &r, e)) return 1;
            sp = start;
            stack[sp].is_tuple = 0; stack[sp].s = r; ++sp;
            break;
        }
        case OP_HELPER: {
            int64_t argc = x->argc[k];
            if (sp < argc) return fail(e, "stack underflow on HELPER_FUNC");
            int64_t start = sp - argc;
            rv r;
            int done = 0;
            if (x->function[k] == 16 && pc && pc->n_tables > 0) {
                double xv;
                if (as_real(&stack[start], &xv, e)) return 1;
                if (!stack[start + 1].is_tuple || !stack[start + 2].is_tuple) return fail(e, "helper expected tuple argument");
                const rv* grid = &stack[start + 1];
                for (int64_t ti = 0; ti < pc->n_tables; ++ti) {
                    const pchip_table* tb = &pc->tables[ti];
                    if (tb->n != grid->len) continue;
                    int match = 1;
                    for (int64_t i = 0; i < tb->n; ++i)
                        if (!(fabs(tb->grid[i] - grid->items[i].re) < 1e-15)) { match = 0; break; }
                    if (match) {
                        r.is_tuple = 0;
                        r.s = C(pchip_eval(tb, xv, &pc->hints[ti]), 0.0);
                        done = 1;
                        break;
                    }
                }
            }
            if (!done && helper_general(x->function[k], stack + start, argc, &r, e)) return 1;
            sp = start;
            stack[sp++] = r;
            break;
        }
        case OP_GT: case OP_GE: case OP_LT: case OP_LE: case OP_EQ: case OP_NE: {
            if (sp < 2) return fail(e, "stack underflow on comparison");
            double r, l;
            if (as_real(&stack[sp - 2], &l, e) || as_real(&stack[sp - 1], &r, e)) return 1;
            sp -= 2;
            int res = op == OP_GT ? l > r : op == OP_GE ? l >= r : op == OP_LT ? l < r : op == OP_LE ? l <= r : op == OP_EQ ? l == r : l != r;
            stack[sp].is_tuple = 0; stack[sp].s = C(res ? 1.0 : 0.0, 0.0); ++sp;
            break;
        }
        default: return fail(e, "unknown instruction op %d", op);
        }
    }
    if (sp != 1) return fail(e, "expression evaluation did not end with a single stack value");
    *out = stack[0];
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* plan                                                                                        */

#define NO_IM (-1)

typedef struct { int64_t re, im; } pidx;

typedef struct {
    int64_t* src;      /* source term indices */
    int64_t n_src;
    int64_t re, im;
    double sign;
} static_term;

typedef struct {
    int64_t term;
    int64_t re, im;
    double sign;
} dyn_term;

struct orc_plan {
    int32_t n;
    int64_t N, U;
    /* parameter graph */
    int32_t n_slots, n_base;
    rv* base;               /* base values (tuples point into tuple_items) */
    cx* tuple_items;
    int32_t n_comp;
    int32_t* comp_slot;
    expr_t* comp_expr;
    int64_t n_pchip;
    pchip_table* pchip;
    /* coefficients */
    int32_t decomposed;
    int32_t n_coeff;
    expr_t* coeff_expr;
    uint8_t* coeff_dynamic;
    int32_t time_dependent;
    int64_t max_stack;
    /* expanded plan */
    int32_t has_expanded;
    int64_t T;
    int64_t* out_ptr;
    int64_t* in_idx;
    int64_t* c_idx;
    uint8_t* c_conj;
    uint8_t* in_conj;
    cx* factor;
    pidx* u2p;              /* upper index -> packed (re, im) */
    /* partitioned layout (n <= 40) */
    int64_t *sr_ptr, *sc_ptr, *dr_ptr, *dc_ptr;
    static_term *sr, *sc;
    dyn_term *dr, *dc;
    int64_t n_sr, n_sc, n_dr, n_dc;
    /* grouped split-input layout (n > 40) */
    int64_t *gr_ptr, *gc_ptr;
    dyn_term *gr, *gc;
    /* populations are y[i * pop_stride]: 1 in the packed layout, n + 1 in the split-real one */
    int64_t pop_stride;
    /* interpolated effective-Hamiltonian plans (effective_lindblad/plan.rs, rhs.rs) */
    int32_t eff;
    int32_t eff_ngrid;
    double* eff_grid;
    int64_t* eff_rows[3];
    int64_t* eff_cols[3];
    double* eff_coef[3];
    int64_t eff_nnz[3];
    int32_t eff_field, eff_rabi, eff_det;
    int32_t eff_rabi_const, eff_det_const;
    double eff_rabi_val, eff_det_val;
};

#define PARTITIONED_MAX_STATES 40

static int expr_from_desc(expr_t* x, const obe_expr* d) {
    x->n = d->n_instr;
    size_t n = (size_t)(d->n_instr > 0 ? d->n_instr : 1);
    x->op = (int32_t*)malloc(n * sizeof(int32_t));
    x->index = (int64_t*)malloc(n * sizeof(int64_t));
    x->argc = (int32_t*)malloc(n * sizeof(int32_t));
    x->function = (int32_t*)malloc(n * sizeof(int32_t));
    x->value = (cx*)malloc(n * sizeof(cx));
    x->uses_time = 0;
    for (int64_t k = 0; k < d->n_instr; ++k) {
        x->op[k] = d->op[k];
        x->index[k] = d->index ? d->index[k] : 0;
        x->argc[k] = d->argc ? d->argc[k] : 0;
        x->function[k] = d->function ? d->function[k] : 0;
        x->value[k] = d->value ? C(d->value[2 * k], d->value[2 * k + 1]) : C(0.0, 0.0);
        if (x->op[k] == OP_TIME) x->uses_time = 1;
    }
    x->scalar_only = d->scalar_only;
    x->output_is_tuple = d->output_is_tuple;
    return 0;
}

static void expr_free(expr_t* x) {
    free(x->op); free(x->index); free(x->argc); free(x->function); free(x->value);
}

static int expr_uses_dynamic_slot(const expr_t* x, const uint8_t* dyn_slot, int32_t n_slots) {
    for (int64_t k = 0; k < x->n; ++k)
        if (x->op[k] == OP_SLOT && x->index[k] >= 0 && x->index[k] < n_slots && dyn_slot[x->index[k]]) return 1;
    return 0;
}

static int validate_expr(const expr_t* x, int32_t n_slots, errbuf* e) {
    for (int64_t k = 0; k < x->n; ++k) {
        if (x->op[k] < 1 || x->op[k] > 19) return fail(e, "unknown instruction op %d", x->op[k]);
        if (x->op[k] == OP_SLOT && (x->index[k] < 0 || x->index[k] >= n_slots))
            return fail(e, "slot index %lld out of bounds for %d slots", (long long)x->index[k], n_slots);
    }
    return 0;
}

static int cmp_i64(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return x < y ? -1 : x > y;
}

typedef struct { int64_t re, im; int sign; int64_t term; } key_rec;

static int cmp_key_real(const void* a, const void* b) {
    const key_rec* x = (const key_rec*)a; const key_rec* y = (const key_rec*)b;
    if (x->re != y->re) return x->re < y->re ? -1 : 1;
    return x->term < y->term ? -1 : x->term > y->term;
}

static int cmp_key_complex(const void* a, const void* b) {
    const key_rec* x = (const key_rec*)a; const key_rec* y = (const key_rec*)b;
    if (x->re != y->re) return x->re < y->re ? -1 : 1;
    if (x->im != y->im) return x->im < y->im ? -1 : 1;
    if (x->sign != y->sign) return x->sign < y->sign ? -1 : 1;
    return x->term < y->term ? -1 : x->term > y->term;
}

static void plan_free(orc_plan* p) {
    if (!p) return;
    free(p->base); free(p->tuple_items);
    for (int32_t i = 0; i < p->n_comp; ++i) expr_free(&p->comp_expr[i]);
    free(p->comp_slot); free(p->comp_expr);
    for (int64_t i = 0; i < p->n_pchip; ++i) { free(p->pchip[i].grid); free(p->pchip[i].coef); }
    free(p->pchip);
    for (int32_t i = 0; i < p->n_coeff; ++i) expr_free(&p->coeff_expr[i]);
    free(p->coeff_expr); free(p->coeff_dynamic);
    free(p->out_ptr); free(p->in_idx); free(p->c_idx); free(p->c_conj); free(p->in_conj); free(p->factor);
    free(p->u2p);
    free(p->sr_ptr); free(p->sc_ptr); free(p->dr_ptr); free(p->dc_ptr);
    for (int64_t i = 0; i < p->n_sr; ++i) free(p->sr[i].src);
    for (int64_t i = 0; i < p->n_sc; ++i) free(p->sc[i].src);
    free(p->sr); free(p->sc); free(p->dr); free(p->dc);
    free(p->gr_ptr); free(p->gc_ptr); free(p->gr); free(p->gc);
    free(p);
}

void orc_plan_destroy(orc_plan* plan) {
    if (plan && plan->eff) {
        free(plan->eff_grid);
        for (int k = 0; k < 3; ++k) { free(plan->eff_rows[k]); free(plan->eff_cols[k]); free(plan->eff_coef[k]); }
    }
    plan_free(plan);
}

/* detect_constant_slot (effective_lindblad/plan.rs:205-277): a base scalar, or a compound whose
   program neither reads the time nor a slot whose (first) compound reads it, evaluated at t = 0
   from the base values with the compounds before it (no interpolation tables) */
static int eff_constant_slot(const orc_plan* p, int32_t slot, double* out) {
    if (slot < p->n_base && !p->base[slot].is_tuple) { *out = p->base[slot].s.re; return 1; }
    for (int32_t i = 0; i < p->n_comp; ++i) {
        if (p->comp_slot[i] != slot) continue;
        const expr_t* x = &p->comp_expr[i];
        if (x->uses_time) return 0;
        for (int64_t k = 0; k < x->n; ++k) {
            if (x->op[k] != OP_SLOT) continue;
            for (int32_t j = 0; j < p->n_comp; ++j)
                if (p->comp_slot[j] == x->index[k]) {
                    if (p->comp_expr[j].uses_time) return 0;
                    break;
                }
        }
        int32_t ns = p->n_slots > 0 ? p->n_slots : 1;
        rv* slots = (rv*)calloc((size_t)ns, sizeof(rv));
        for (int32_t b = 0; b < p->n_base; ++b) slots[b] = p->base[b];
        int64_t ms = p->max_stack + 4;
        rv* stack = (rv*)malloc(sizeof(rv) * (size_t)ms);
        arena ar;
        memset(&ar, 0, sizeof ar);
        errbuf e = {{0}, 0};
        pchip_ctx none = {NULL, 0, NULL};
        for (int32_t j = 0; j < p->n_comp; ++j) {
            if (p->comp_slot[j] == slot) break;
            rv r;
            e.set = 0;
            if (!eval_general(&p->comp_expr[j], slots, 0.0, stack, &ar, &none, &r, &e)) slots[p->comp_slot[j]] = r;
        }
        rv r;
        e.set = 0;
        int ok = !eval_general(x, slots, 0.0, stack, &ar, &none, &r, &e) && !r.is_tuple;
        if (ok) *out = r.s.re;
        free(slots);
        free(stack);
        arena_free(&ar);
        return ok;
    }
    return 0;
}

orc_plan* orc_effective_plan_create(const obe_plan_desc* graph, const obe_effective_desc* d, char* err, size_t err_len) {
    errbuf e = {{0}, 0};
    if (!graph || !d) { snprintf(err, err_len, "null argument"); return NULL; }
    orc_plan* p = orc_plan_create(graph, err, err_len);
    if (!p) return NULL;
    if (d->n_grid < 1 || d->real_dim != 2 * (int64_t)p->n * p->n) {
        fail(&e, d->n_grid < 1 ? "field_grid length mismatch" : "real_dim must be 2 n_states^2");
        copy_err(&e, err, err_len);
        plan_free(p);
        return NULL;
    }
    p->eff = 1;
    p->N = d->real_dim;
    p->pop_stride = p->n + 1;
    p->eff_ngrid = d->n_grid;
    p->eff_grid = (double*)malloc(sizeof(double) * (size_t)d->n_grid);
    memcpy(p->eff_grid, d->field_grid, sizeof(double) * (size_t)d->n_grid);
    const obe_interp_operator* ops[3] = {&d->combined, &d->optical, &d->detuning};
    for (int k = 0; k < 3; ++k) {
        const int64_t nnz = ops[k]->nnz, nc = (int64_t)(d->n_grid > 1 ? d->n_grid - 1 : 0) * nnz * 4;
        p->eff_nnz[k] = nnz;
        p->eff_rows[k] = (int64_t*)malloc(sizeof(int64_t) * (size_t)(p->N + 1));
        memcpy(p->eff_rows[k], ops[k]->row_ptrs, sizeof(int64_t) * (size_t)(p->N + 1));
        p->eff_cols[k] = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nnz > 0 ? nnz : 1));
        if (nnz > 0) memcpy(p->eff_cols[k], ops[k]->col_indices, sizeof(int64_t) * (size_t)nnz);
        p->eff_coef[k] = (double*)malloc(sizeof(double) * (size_t)(nc > 0 ? nc : 1));
        if (nc > 0) memcpy(p->eff_coef[k], ops[k]->coeffs, sizeof(double) * (size_t)nc);
    }
    p->eff_field = d->field_slot;
    p->eff_rabi = d->rabi_slot;
    p->eff_det = d->detuning_slot;
    p->eff_rabi_const = eff_constant_slot(p, d->rabi_slot, &p->eff_rabi_val);
    p->eff_det_const = eff_constant_slot(p, d->detuning_slot, &p->eff_det_val);
    return p;
}

static int64_t upper_index(int32_t n, int32_t i, int32_t j) {
    /* row-major upper triangle including the diagonal (ir.py:463-475) */
    int64_t off = 0;
    for (int32_t r = 0; r < i; ++r) off += n - r;
    return off + (j - i);
}

orc_plan* orc_plan_create(const obe_plan_desc* d, char* err, size_t err_len) {
    errbuf e = {{0}, 0};
    orc_plan* p = (orc_plan*)calloc(1, sizeof(orc_plan));
    if (d->n_states <= 0) { fail(&e, "layout dimension must be positive"); goto bad; }
    p->n = d->n_states;
    p->N = (int64_t)p->n * p->n;
    p->U = (int64_t)p->n * (p->n + 1) / 2;
    p->pop_stride = 1;
    p->n_slots = d->n_slots;
    p->n_base = d->n_base;
    if (p->n_base > p->n_slots) { fail(&e, "more base values than slots"); goto bad; }
    /* base values */
    int64_t n_items = d->n_base > 0 && d->base_tuple_ptr ? d->base_tuple_ptr[d->n_base] : 0;
    p->tuple_items = (cx*)malloc(sizeof(cx) * (size_t)(n_items > 0 ? n_items : 1));
    for (int64_t i = 0; i < n_items; ++i) p->tuple_items[i] = C(d->base_tuple_items[2 * i], d->base_tuple_items[2 * i + 1]);
    p->base = (rv*)calloc((size_t)(p->n_base > 0 ? p->n_base : 1), sizeof(rv));
    for (int32_t i = 0; i < p->n_base; ++i) {
        if (d->base_is_tuple && d->base_is_tuple[i]) {
            p->base[i].is_tuple = 1;
            p->base[i].items = p->tuple_items + d->base_tuple_ptr[i];
            p->base[i].len = d->base_tuple_ptr[i + 1] - d->base_tuple_ptr[i];
        } else {
            p->base[i].s = C(d->base_scalar[2 * i], d->base_scalar[2 * i + 1]);
        }
    }
    /* compounds */
    p->n_comp = d->n_compounds;
    p->comp_slot = (int32_t*)malloc(sizeof(int32_t) * (size_t)(p->n_comp > 0 ? p->n_comp : 1));
    p->comp_expr = (expr_t*)calloc((size_t)(p->n_comp > 0 ? p->n_comp : 1), sizeof(expr_t));
    p->max_stack = 8;
    for (int32_t i = 0; i < p->n_comp; ++i) {
        p->comp_slot[i] = d->compound_slot[i];
        expr_from_desc(&p->comp_expr[i], &d->compound_expr[i]);
        if (p->comp_slot[i] < 0 || p->comp_slot[i] >= p->n_slots) { fail(&e, "compound slot %d out of bounds", p->comp_slot[i]); goto bad; }
        if (validate_expr(&p->comp_expr[i], p->n_slots, &e)) goto bad;
        if (p->comp_expr[i].n > p->max_stack) p->max_stack = p->comp_expr[i].n;
    }
    /* pchip tables */
    p->n_pchip = d->n_pchip;
    p->pchip = (pchip_table*)calloc((size_t)(p->n_pchip > 0 ? p->n_pchip : 1), sizeof(pchip_table));
    for (int64_t i = 0; i < p->n_pchip; ++i) {
        int64_t a = d->pchip_ptr[i], b = d->pchip_ptr[i + 1];
        if (pchip_build(&p->pchip[i], d->pchip_grid + a, d->pchip_values + a, b - a, &e)) goto bad;
    }
    /* coefficients */
    p->decomposed = d->hamiltonian_decomposed;
    p->n_coeff = d->n_coefficients;
    p->coeff_expr = (expr_t*)calloc((size_t)(p->n_coeff > 0 ? p->n_coeff : 1), sizeof(expr_t));
    p->coeff_dynamic = (uint8_t*)calloc((size_t)(p->n_coeff > 0 ? p->n_coeff : 1), 1);
    for (int32_t i = 0; i < p->n_coeff; ++i) {
        expr_from_desc(&p->coeff_expr[i], &d->coefficient_expr[i]);
        if (validate_expr(&p->coeff_expr[i], p->n_slots, &e)) goto bad;
        if (p->coeff_expr[i].n > p->max_stack) p->max_stack = p->coeff_expr[i].n;
    }
    /* dynamic detection (plan.rs:1240-1291) */
    {
        uint8_t* dyn_slot = (uint8_t*)calloc((size_t)(p->n_slots > 0 ? p->n_slots : 1), 1);
        int params_use_time = 0, ham_uses_time = 0;
        for (int32_t i = 0; i < p->n_comp; ++i) {
            int dyn = p->comp_expr[i].uses_time || expr_uses_dynamic_slot(&p->comp_expr[i], dyn_slot, p->n_slots);
            dyn_slot[p->comp_slot[i]] = (uint8_t)dyn;
            params_use_time |= p->comp_expr[i].uses_time;
        }
        for (int32_t i = 0; i < p->n_coeff; ++i) {
            p->coeff_dynamic[i] = (uint8_t)(p->coeff_expr[i].uses_time || expr_uses_dynamic_slot(&p->coeff_expr[i], dyn_slot, p->n_slots));
            ham_uses_time |= p->coeff_expr[i].uses_time;
        }
        p->time_dependent = params_use_time || ham_uses_time;
        free(dyn_slot);
    }
    /* expanded plan (plan.rs:1069-1153) */
    p->has_expanded = d->has_expanded;
    p->u2p = (pidx*)malloc(sizeof(pidx) * (size_t)p->U);
    {
        /* build_upper_to_packed_indices (rhs.rs:151-176) */
        for (int32_t i = 0; i < p->n; ++i) { pidx q = {i, NO_IM}; p->u2p[upper_index(p->n, i, i)] = q; }
        int64_t cursor = p->n;
        for (int32_t i = 0; i < p->n; ++i)
            for (int32_t j = i + 1; j < p->n; ++j) { pidx q = {cursor, cursor + 1}; p->u2p[upper_index(p->n, i, j)] = q; cursor += 2; }
    }
    if (p->has_expanded) {
        int64_t T = d->n_terms;
        p->T = T;
        if (d->output_ptrs[0] != 0 || d->output_ptrs[p->U] != T) { fail(&e, "expanded RHS output_ptrs must start at 0 and end at term count"); goto bad; }
        for (int64_t u = 0; u < p->U; ++u)
            if (d->output_ptrs[u] > d->output_ptrs[u + 1]) { fail(&e, "expanded RHS output_ptrs must be monotonic"); goto bad; }
        p->out_ptr = (int64_t*)malloc(sizeof(int64_t) * (size_t)(p->U + 1));
        memcpy(p->out_ptr, d->output_ptrs, sizeof(int64_t) * (size_t)(p->U + 1));
        size_t tn = (size_t)(T > 0 ? T : 1);
        p->in_idx = (int64_t*)malloc(sizeof(int64_t) * tn);
        p->c_idx = (int64_t*)malloc(sizeof(int64_t) * tn);
        p->c_conj = (uint8_t*)malloc(tn);
        p->in_conj = (uint8_t*)malloc(tn);
        p->factor = (cx*)malloc(sizeof(cx) * tn);
        for (int64_t t = 0; t < T; ++t) {
            int64_t in = d->input_indices[t];
            if (in < 0 || in >= p->U) { fail(&e, "expanded RHS input index %lld out of bounds for upper length %lld", (long long)in, (long long)p->U); goto bad; }
            int64_t ci = d->coeff_indices[t];
            if (ci >= 0 && ci >= p->n_coeff) { fail(&e, "expanded RHS coefficient index %lld out of bounds for %d coefficients", (long long)ci, p->n_coeff); goto bad; }
            p->in_idx[t] = in;
            p->c_idx[t] = ci < 0 ? -1 : ci;
            p->c_conj[t] = d->coeff_conj[t];
            p->in_conj[t] = d->input_conj[t];
            p->factor[t] = C(d->factors_re[t], d->factors_im[t]);
        }
        /* partitioned layout (rhs.rs:285-384) */
        p->sr_ptr = (int64_t*)calloc((size_t)(p->U + 1), sizeof(int64_t));
        p->sc_ptr = (int64_t*)calloc((size_t)(p->U + 1), sizeof(int64_t));
        p->dr_ptr = (int64_t*)calloc((size_t)(p->U + 1), sizeof(int64_t));
        p->dc_ptr = (int64_t*)calloc((size_t)(p->U + 1), sizeof(int64_t));
        p->sr = (static_term*)calloc(tn, sizeof(static_term));
        p->sc = (static_term*)calloc(tn, sizeof(static_term));
        p->dr = (dyn_term*)calloc(tn, sizeof(dyn_term));
        p->dc = (dyn_term*)calloc(tn, sizeof(dyn_term));
        key_rec* keys_r = (key_rec*)malloc(sizeof(key_rec) * tn);
        key_rec* keys_c = (key_rec*)malloc(sizeof(key_rec) * tn);
        key_rec* dk_r = (key_rec*)malloc(sizeof(key_rec) * tn);
        key_rec* dk_c = (key_rec*)malloc(sizeof(key_rec) * tn);
        for (int64_t u = 0; u < p->U; ++u) {
            int64_t nr = 0, nc = 0, ndr = 0, ndc = 0;
            for (int64_t t = p->out_ptr[u]; t < p->out_ptr[u + 1]; ++t) {
                int dynamic = p->c_idx[t] >= 0 && p->coeff_dynamic[p->c_idx[t]];
                pidx q = p->u2p[p->in_idx[t]];
                key_rec k;
                k.re = q.re;
                k.term = t;
                if (q.im == NO_IM) {
                    k.im = q.re; k.sign = 0;
                    if (dynamic) dk_r[ndr++] = k; else keys_r[nr++] = k;
                } else {
                    k.im = q.im; k.sign = p->in_conj[t] ? -1 : 1;
                    if (dynamic) dk_c[ndc++] = k; else keys_c[nc++] = k;
                }
            }
            qsort(keys_r, (size_t)nr, sizeof(key_rec), cmp_key_real);
            qsort(keys_c, (size_t)nc, sizeof(key_rec), cmp_key_complex);
            /* dynamic terms: stable sort by re (real) / (re, im) (complex) */
            for (int64_t i = 1; i < ndr; ++i) { key_rec k = dk_r[i]; int64_t j = i; while (j > 0 && dk_r[j - 1].re > k.re) { dk_r[j] = dk_r[j - 1]; --j; } dk_r[j] = k; }
            for (int64_t i = 1; i < ndc; ++i) {
                key_rec k = dk_c[i]; int64_t j = i;
                while (j > 0 && (dk_c[j - 1].re > k.re || (dk_c[j - 1].re == k.re && dk_c[j - 1].im > k.im))) { dk_c[j] = dk_c[j - 1]; --j; }
                dk_c[j] = k;
            }
            for (int64_t i = 0; i < nr;) {
                int64_t j = i;
                while (j < nr && keys_r[j].re == keys_r[i].re) ++j;
                static_term* s = &p->sr[p->n_sr++];
                s->n_src = j - i;
                s->src = (int64_t*)malloc(sizeof(int64_t) * (size_t)(j - i));
                for (int64_t q = i; q < j; ++q) s->src[q - i] = keys_r[q].term;
                qsort(s->src, (size_t)s->n_src, sizeof(int64_t), cmp_i64);
                s->re = keys_r[i].re; s->im = keys_r[i].re; s->sign = 0.0;
                i = j;
            }
            for (int64_t i = 0; i < nc;) {
                int64_t j = i;
                while (j < nc && keys_c[j].re == keys_c[i].re && keys_c[j].im == keys_c[i].im && keys_c[j].sign == keys_c[i].sign) ++j;
                static_term* s = &p->sc[p->n_sc++];
                s->n_src = j - i;
                s->src = (int64_t*)malloc(sizeof(int64_t) * (size_t)(j - i));
                for (int64_t q = i; q < j; ++q) s->src[q - i] = keys_c[q].term;
                qsort(s->src, (size_t)s->n_src, sizeof(int64_t), cmp_i64);
                s->re = keys_c[i].re; s->im = keys_c[i].im; s->sign = (double)keys_c[i].sign;
                i = j;
            }
            for (int64_t i = 0; i < ndr; ++i) { dyn_term* q = &p->dr[p->n_dr++]; q->term = dk_r[i].term; q->re = dk_r[i].re; q->im = dk_r[i].re; q->sign = 0.0; }
            for (int64_t i = 0; i < ndc; ++i) { dyn_term* q = &p->dc[p->n_dc++]; q->term = dk_c[i].term; q->re = dk_c[i].re; q->im = dk_c[i].im; q->sign = (double)dk_c[i].sign; }
            p->sr_ptr[u + 1] = p->n_sr; p->sc_ptr[u + 1] = p->n_sc;
            p->dr_ptr[u + 1] = p->n_dr; p->dc_ptr[u + 1] = p->n_dc;
        }
        free(keys_r); free(keys_c); free(dk_r); free(dk_c);
        /* grouped split-input layout (rhs.rs:207-250) */
        p->gr_ptr = (int64_t*)calloc((size_t)(p->U + 1), sizeof(int64_t));
        p->gc_ptr = (int64_t*)calloc((size_t)(p->U + 1), sizeof(int64_t));
        p->gr = (dyn_term*)calloc(tn, sizeof(dyn_term));
        p->gc = (dyn_term*)calloc(tn, sizeof(dyn_term));
        int64_t ngr = 0, ngc = 0;
        for (int64_t u = 0; u < p->U; ++u) {
            for (int64_t t = p->out_ptr[u]; t < p->out_ptr[u + 1]; ++t) {
                pidx q = p->u2p[p->in_idx[t]];
                if (q.im == NO_IM) { dyn_term g = {t, q.re, q.re, 0.0}; p->gr[ngr++] = g; }
                else { dyn_term g = {t, q.re, q.im, p->in_conj[t] ? -1.0 : 1.0}; p->gc[ngc++] = g; }
            }
            p->gr_ptr[u + 1] = ngr; p->gc_ptr[u + 1] = ngc;
        }
    }
    return p;
bad:
    copy_err(&e, err, err_len);
    plan_free(p);
    return NULL;
}

/* ------------------------------------------------------------------------------------------ */
/* per-trajectory workspace (rhs.rs:1057-1241)                                                 */

typedef struct {
    const orc_plan* p;
    rv* slots;
    cx* coeff;              /* coefficient values */
    cx* static_coef_r;      /* merged static coefficients (partitioned) */
    cx* static_coef_c;
    double* tv_re;          /* per-term values (dynamic / all terms) */
    double* tv_im;
    cx* sstack;
    rv* gstack;
    arena ar;
    cx** comp_tuple;        /* storage of tuple-valued compound results */
    int64_t* comp_tuple_cap;
    int64_t* pchip_hints;
    int32_t n_over;
    int64_t* over_slot;
    cx* over_val;
    int valid;              /* cached coefficients valid (time-independent plans) */
    int use_split_input;
    int64_t eff_hint;       /* the effective RHS's last field interval (rhs.rs: last_interval) */
    /* stop event */
    int ev_kind;
    expr_t ev_expr;
    int ev_has_expr;
    const int64_t* ev_idx;
    int32_t n_ev_idx;
    double ev_thr;
} workspace;

static void ws_init(workspace* w, const orc_plan* p, int use_split) {
    memset(w, 0, sizeof *w);
    w->p = p;
    w->slots = (rv*)calloc((size_t)(p->n_slots > 0 ? p->n_slots : 1), sizeof(rv));
    w->coeff = (cx*)calloc((size_t)(p->n_coeff > 0 ? p->n_coeff : 1), sizeof(cx));
    w->static_coef_r = (cx*)calloc((size_t)(p->n_sr > 0 ? p->n_sr : 1), sizeof(cx));
    w->static_coef_c = (cx*)calloc((size_t)(p->n_sc > 0 ? p->n_sc : 1), sizeof(cx));
    w->tv_re = (double*)calloc((size_t)(p->T > 0 ? p->T : 1), sizeof(double));
    w->tv_im = (double*)calloc((size_t)(p->T > 0 ? p->T : 1), sizeof(double));
    int64_t ms = p->max_stack + 4;
    w->sstack = (cx*)malloc(sizeof(cx) * (size_t)ms);
    w->gstack = (rv*)malloc(sizeof(rv) * (size_t)ms);
    w->pchip_hints = (int64_t*)calloc((size_t)(p->n_pchip > 0 ? p->n_pchip : 1), sizeof(int64_t));
    w->use_split_input = use_split;
    w->comp_tuple = (cx**)calloc((size_t)(p->n_comp > 0 ? p->n_comp : 1), sizeof(cx*));
    w->comp_tuple_cap = (int64_t*)calloc((size_t)(p->n_comp > 0 ? p->n_comp : 1), sizeof(int64_t));
}

static void ws_free(workspace* w) {
    free(w->slots); free(w->coeff); free(w->static_coef_r); free(w->static_coef_c);
    free(w->tv_re); free(w->tv_im); free(w->sstack); free(w->gstack); arena_free(&w->ar);
    for (int32_t i = 0; i < w->p->n_comp; ++i) free(w->comp_tuple[i]);
    free(w->comp_tuple); free(w->comp_tuple_cap);
    free(w->pchip_hints); free(w->over_slot); free(w->over_val);
    if (w->ev_has_expr) expr_free(&w->ev_expr);
}

static void ws_set_overrides(workspace* w, int32_t n, const int64_t* slots, const double* vals) {
    free(w->over_slot); free(w->over_val);
    w->n_over = n;
    w->over_slot = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    w->over_val = (cx*)malloc(sizeof(cx) * (size_t)(n > 0 ? n : 1));
    for (int32_t i = 0; i < n; ++i) { w->over_slot[i] = slots[i]; w->over_val[i] = C(vals[2 * i], vals[2 * i + 1]); }
    w->valid = 0;
}

/* ParameterGraph::evaluate_with_overrides_into (plan.rs:130-173) */
static int ws_eval_params(workspace* w, double t, errbuf* e) {
    const orc_plan* p = w->p;
    for (int32_t i = 0; i < p->n_base; ++i) w->slots[i] = p->base[i];
    for (int32_t i = 0; i < w->n_over; ++i) {
        int64_t s = w->over_slot[i];
        if (s < 0 || s >= p->n_base) return fail(e, "parameter override slot %lld is not a base parameter slot", (long long)s);
        w->slots[s].is_tuple = 0;
        w->slots[s].s = w->over_val[i];
    }
    for (int32_t i = p->n_base; i < p->n_slots; ++i) { w->slots[i].is_tuple = 0; w->slots[i].s = C(0.0, 0.0); }
    pchip_ctx pc = {p->pchip, p->n_pchip, w->pchip_hints};
    for (int32_t i = 0; i < p->n_comp; ++i) {
        const expr_t* x = &p->comp_expr[i];
        rv r;
        if (x->scalar_only) {
            r.is_tuple = 0;
            if (eval_scalar(x, w->slots, t, w->sstack, &r.s, e)) return 1;
        } else {
            if (eval_general(x, w->slots, t, w->gstack, &w->ar, &pc, &r, e)) return 1;
            if (r.is_tuple) {
                /* the arena is reset by the next evaluation: keep tuple compounds in storage */
                if (w->comp_tuple_cap[i] < r.len) {
                    free(w->comp_tuple[i]);
                    w->comp_tuple[i] = (cx*)malloc(sizeof(cx) * (size_t)r.len);
                    w->comp_tuple_cap[i] = r.len;
                }
                if (r.len > 0) memcpy(w->comp_tuple[i], r.items, sizeof(cx) * (size_t)r.len);
                r.items = w->comp_tuple[i];
            }
        }
        w->slots[p->comp_slot[i]] = r;
    }
    return 0;
}

/* evaluate_decomposed_coefficients_into (plan.rs:242-276) */
static int ws_eval_coeffs(workspace* w, double t, errbuf* e) {
    const orc_plan* p = w->p;
    if (!p->decomposed) return fail(e, "expanded sparse RHS requires a decomposed Hamiltonian plan");
    for (int32_t k = 0; k < p->n_coeff; ++k) {
        const expr_t* x = &p->coeff_expr[k];
        if (x->scalar_only) {
            if (eval_scalar(x, w->slots, t, w->sstack, &w->coeff[k], e)) return 1;
        } else {
            rv r;
            if (eval_general(x, w->slots, t, w->gstack, &w->ar, NULL, &r, e)) return 1;
            if (as_scalar(&r, &w->coeff[k], e)) return 1;
        }
    }
    return 0;
}

/* expanded_sparse_term_value (rhs.rs:878-899) */
static inline cx term_value(const orc_plan* p, int64_t t, const cx* coeff) {
    cx c = C(1.0, 0.0);
    if (p->c_idx[t] >= 0) {
        c = coeff[p->c_idx[t]];
        if (p->c_conj[t]) c = cx_conj(c);
    }
    return cx_mul(p->factor[t], c);
}

static inline void write_out(const orc_plan* p, double* out, int64_t u, double re, double im) {
    pidx q = p->u2p[u];
    out[q.re] = re;
    if (q.im != NO_IM) out[q.im] = im;
}

/* Rust's `{:.6e}`: six decimals, exponent without sign padding ("1.000000e2", "-3.500000e-1") */
static void fmt_rust_exp6(double v, char* out, size_t len) {
    char buf[64];
    snprintf(buf, sizeof buf, "%.6e", v);
    char* e = strchr(buf, 'e');
    if (!e) { snprintf(out, len, "%s", buf); return; }
    int ex = atoi(e + 1);
    *e = 0;
    snprintf(out, len, "%.24se%d", buf, ex);
}

/* find_interval_cached (effective_lindblad/rhs.rs:48-86) */
static int eff_find_interval(double x, const double* grid, int64_t n, int64_t* hint, int64_t* idx, errbuf* e) {
    if (n < 2) { *idx = 0; return 0; }
    const double tol = 1e-10 * fmax(fabs(grid[n - 1] - grid[0]), 1.0);
    char a[64], b[64];
    if (x < grid[0] - tol) {
        fmt_rust_exp6(x, a, sizeof a);
        fmt_rust_exp6(grid[0], b, sizeof b);
        return fail(e, "field coordinate %s is below the operator grid minimum %s", a, b);
    }
    if (x > grid[n - 1] + tol) {
        fmt_rust_exp6(x, a, sizeof a);
        fmt_rust_exp6(grid[n - 1], b, sizeof b);
        return fail(e, "field coordinate %s is above the operator grid maximum %s", a, b);
    }
    const double xc = x < grid[0] ? grid[0] : (x > grid[n - 1] ? grid[n - 1] : x);  /* NaN stays NaN */
    if (xc <= grid[0]) { *hint = 0; *idx = 0; return 0; }
    if (xc >= grid[n - 1]) { *hint = n - 2; *idx = n - 2; return 0; }
    const int64_t h = *hint;
    if (h < n - 1 && grid[h] <= xc && xc <= grid[h + 1]) { *idx = h; return 0; }
    int64_t cnt = 0;
    while (cnt < n && grid[cnt] <= xc) ++cnt;  /* partition_point(g <= x) */
    int64_t k = cnt > 0 ? cnt - 1 : 0;
    if (k > n - 2) k = n - 2;
    *hint = k;
    *idx = k;
    return 0;
}

/* SparseOperator::sparse_matvec_interpolated (effective_lindblad/plan.rs:19-42) */
static void eff_matvec(const orc_plan* p, int op, int64_t idx, double dx, double scale, const double* y, double* dy) {
    const int64_t nnz = p->eff_nnz[op];
    const int64_t interval = idx < p->eff_ngrid - 2 ? idx : (p->eff_ngrid >= 2 ? p->eff_ngrid - 2 : 0);
    const double* cb = p->eff_coef[op] + interval * nnz * 4;
    for (int64_t i = 0; i < p->N; ++i) {
        double sum = 0.0;
        for (int64_t q = p->eff_rows[op][i]; q < p->eff_rows[op][i + 1]; ++q) {
            const double* c = cb + q * 4;
            const double val = c[0] + dx * (c[1] + dx * (c[2] + dx * c[3]));
            sum += val * y[p->eff_cols[op][q]];
        }
        dy[i] += scale * sum;
    }
}

/* rhs_effective_lindblad (effective_lindblad/rhs.rs:88-137) */
static int ws_rhs_effective(workspace* w, double t, const double* y, double* out, errbuf* e) {
    const orc_plan* p = w->p;
    if (ws_eval_params(w, t, e)) return 1;
    const rv* fv = &w->slots[p->eff_field];
    if (fv->is_tuple) return fail(e, "field_coordinate must be scalar");
    const double x = fv->s.re;
    const rv* rvv = &w->slots[p->eff_rabi];
    const rv* dvv = &w->slots[p->eff_det];
    const double rabi = p->eff_rabi_const ? p->eff_rabi_val : (rvv->is_tuple ? 0.0 : rvv->s.re);
    const double det = p->eff_det_const ? p->eff_det_val : (dvv->is_tuple ? 0.0 : dvv->s.re);
    int64_t idx = 0;
    if (eff_find_interval(x, p->eff_grid, p->eff_ngrid, &w->eff_hint, &idx, e)) return 1;
    const double dx = x - p->eff_grid[idx];
    for (int64_t i = 0; i < p->N; ++i) out[i] = 0.0;
    eff_matvec(p, 0, idx, dx, 1.0, y, out);
    eff_matvec(p, 1, idx, dx, 0.5 * rabi, y, out);
    eff_matvec(p, 2, idx, dx, det, y, out);
    return 0;
}

/* rhs_packed_expanded_sparse_into_with_profile (rhs.rs:1789-1867) + the partitioned kernel
   (rhs.rs:815-876), or for n > 40 the split-input path (rhs.rs:1869-1968, 633-695) */
static int ws_rhs(workspace* w, double t, const double* y, double* out, errbuf* e) {
    const orc_plan* p = w->p;
    if (p->eff) return ws_rhs_effective(w, t, y, out, e);
    if (!p->has_expanded) return fail(e, "execution_mode='expanded_sparse' requires a decomposed Hamiltonian plan");
    if (p->n <= PARTITIONED_MAX_STATES) {
        int init = !w->valid;
        if (init || p->time_dependent) {
            if (ws_eval_params(w, t, e)) return 1;
            if (ws_eval_coeffs(w, t, e)) return 1;
            if (init) {
                for (int64_t i = 0; i < p->n_sr; ++i) {
                    cx c = C(0.0, 0.0);
                    for (int64_t k = 0; k < p->sr[i].n_src; ++k) c = cx_add(c, term_value(p, p->sr[i].src[k], w->coeff));
                    w->static_coef_r[i] = c;
                }
                for (int64_t i = 0; i < p->n_sc; ++i) {
                    cx c = C(0.0, 0.0);
                    for (int64_t k = 0; k < p->sc[i].n_src; ++k) c = cx_add(c, term_value(p, p->sc[i].src[k], w->coeff));
                    w->static_coef_c[i] = c;
                }
            }
            for (int64_t i = 0; i < p->n_dr; ++i) { cx c = term_value(p, p->dr[i].term, w->coeff); w->tv_re[p->dr[i].term] = c.re; w->tv_im[p->dr[i].term] = c.im; }
            for (int64_t i = 0; i < p->n_dc; ++i) { cx c = term_value(p, p->dc[i].term, w->coeff); w->tv_re[p->dc[i].term] = c.re; w->tv_im[p->dc[i].term] = c.im; }
            w->valid = 1;
        }
        for (int64_t u = 0; u < p->U; ++u) {
            double ar = 0.0, ai = 0.0;
            for (int64_t i = p->sr_ptr[u]; i < p->sr_ptr[u + 1]; ++i) {
                double v = y[p->sr[i].re];
                ar += w->static_coef_r[i].re * v;
                ai += w->static_coef_r[i].im * v;
            }
            for (int64_t i = p->sc_ptr[u]; i < p->sc_ptr[u + 1]; ++i) {
                double vr = y[p->sc[i].re], vi = p->sc[i].sign * y[p->sc[i].im];
                cx c = w->static_coef_c[i];
                ar += c.re * vr - c.im * vi;
                ai += c.re * vi + c.im * vr;
            }
            for (int64_t i = p->dr_ptr[u]; i < p->dr_ptr[u + 1]; ++i) {
                double v = y[p->dr[i].re];
                ar += w->tv_re[p->dr[i].term] * v;
                ai += w->tv_im[p->dr[i].term] * v;
            }
            for (int64_t i = p->dc_ptr[u]; i < p->dc_ptr[u + 1]; ++i) {
                double cr = w->tv_re[p->dc[i].term], ci = w->tv_im[p->dc[i].term];
                double vr = y[p->dc[i].re], vi = p->dc[i].sign * y[p->dc[i].im];
                ar += cr * vr - ci * vi;
                ai += cr * vi + ci * vr;
            }
            write_out(p, out, u, ar, ai);
        }
        return 0;
    }
    /* n > 40 */
    int can_skip = !p->time_dependent && w->valid;
    if (!can_skip) {
        if (ws_eval_params(w, t, e)) return 1;
        if (ws_eval_coeffs(w, t, e)) return 1;
        for (int64_t i = 0; i < p->T; ++i) { cx c = term_value(p, i, w->coeff); w->tv_re[i] = c.re; w->tv_im[i] = c.im; }
        w->valid = 1;
    }
    if (w->use_split_input) {
        for (int64_t u = 0; u < p->U; ++u) {
            double ar = 0.0, ai = 0.0;
            for (int64_t i = p->gr_ptr[u]; i < p->gr_ptr[u + 1]; ++i) {
                int64_t t = p->gr[i].term;
                double v = y[p->gr[i].re];
                ar += w->tv_re[t] * v;
                ai += w->tv_im[t] * v;
            }
            for (int64_t i = p->gc_ptr[u]; i < p->gc_ptr[u + 1]; ++i) {
                int64_t t = p->gc[i].term;
                double cr = w->tv_re[t], ci = w->tv_im[t];
                double vr = y[p->gc[i].re], vi = p->gc[i].sign * y[p->gc[i].im];
                ar += cr * vr - ci * vi;
                ai += cr * vi + ci * vr;
            }
            write_out(p, out, u, ar, ai);
        }
    } else {
        /* split coefficients, CSR order (rhs.rs:586-631) */
        for (int64_t u = 0; u < p->U; ++u) {
            double ar = 0.0, ai = 0.0;
            for (int64_t t = p->out_ptr[u]; t < p->out_ptr[u + 1]; ++t) {
                pidx q = p->u2p[p->in_idx[t]];
                double cr = w->tv_re[t], ci = w->tv_im[t];
                double vr = y[q.re];
                double vi = q.im == NO_IM ? 0.0 : (p->in_conj[t] ? -1.0 : 1.0) * y[q.im];
                ar += cr * vr - ci * vi;
                ai += cr * vi + ci * vr;
            }
            write_out(p, out, u, ar, ai);
        }
    }
    return 0;
}

/* LindbladRhs::event_value (ode_impl.rs:134-154) */
static int ws_event(workspace* w, double t, const double* y, int* has, double* g, errbuf* e) {
    *has = 0;
    if (w->ev_kind == OBE_EVENT_NONE) return 0;
    if (w->ev_kind == OBE_EVENT_POPULATION) {
        double v = 0.0;
        for (int32_t i = 0; i < w->n_ev_idx; ++i) {
            int64_t idx = w->ev_idx[i];
            if (idx < 0 || idx >= w->p->n) return fail(e, "population event index %lld out of bounds", (long long)idx);
            v += y[idx];
        }
        *g = v - w->ev_thr;
        *has = 1;
        return 0;
    }
    /* evaluate_runtime_expression_real (rhs.rs:1214-1240) */
    if (ws_eval_params(w, t, e)) return 1;
    pchip_ctx pc = {w->p->pchip, w->p->n_pchip, w->pchip_hints};
    rv r;
    if (eval_general(&w->ev_expr, w->slots, t, w->gstack, &w->ar, &pc, &r, e)) return 1;
    if (r.is_tuple) return fail(e, "event expression evaluated to a tuple");
    if (fabs(r.s.im) > 1e-12) return fail(e, "event expression evaluated to a complex value");
    *g = r.s.re;
    *has = 1;
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* outputs (ode/output.rs)                                                                     */

typedef struct {
    int kind;
    int store_trace;
    int64_t width;         /* values per point */
    int is_complex;
    int64_t capacity;      /* points */
    int64_t count;
    double* times;
    double* vals;          /* capacity * width * (1|2) */
    /* spec */
    const orc_plan* p;
    const obe_solve_options* opt;
    /* selected extraction: packed indices */
    int64_t* sel_re;
    int64_t* sel_im;
    int8_t* sel_kind;      /* 0 real, 1 pair, 2 conj pair */
    /* integral state */
    double integral, last_t, last_value;
    double last_time;      /* times[last] even when not stored */
    int has_last_time;
} sink;

static int64_t packed_upper_real_index(int32_t n, int64_t i, int64_t j) {
    int64_t off = 0;
    for (int64_t r = 0; r < i; ++r) off += n - r - 1;
    return n + 2 * (off + (j - i - 1));
}

int64_t orc_output_width(const orc_plan* plan, const obe_solve_options* opt, int32_t* is_complex) {
    *is_complex = opt->output == OBE_OUTPUT_SELECTED;
    switch (opt->output) {
    case OBE_OUTPUT_POPULATIONS: return plan->n;
    case OBE_OUTPUT_SELECTED: return opt->n_selected;
    case OBE_OUTPUT_FULL: return plan->N;
    default: return 1;
    }
}

static void sink_init(sink* s, const orc_plan* p, const obe_solve_options* opt, int64_t capacity, double* times, double* vals) {
    memset(s, 0, sizeof *s);
    s->p = p;
    s->opt = opt;
    s->kind = opt->output;
    s->store_trace = opt->store_trace;
    int32_t cplx;
    s->width = orc_output_width(p, opt, &cplx);
    s->is_complex = cplx;
    s->capacity = capacity;
    s->times = times;
    s->vals = vals;
    s->last_t = NAN;
    if (s->kind == OBE_OUTPUT_SELECTED) {
        int32_t m = opt->n_selected;
        s->sel_re = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
        s->sel_im = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
        s->sel_kind = (int8_t*)malloc((size_t)(m > 0 ? m : 1));
        for (int32_t k = 0; k < m; ++k) {
            int64_t i = opt->selected_i[k], j = opt->selected_j[k];
            if (p->eff) {
                /* split_real_selected_extractions (effective_lindblad/solver.rs:58-76) */
                const int64_t n = p->n;
                s->sel_kind[k] = i == j ? 0 : 1;
                s->sel_re[k] = i * n + j;
                s->sel_im[k] = i == j ? i * n + j : n * n + i * n + j;
                continue;
            }
            if (i == j) { s->sel_kind[k] = 0; s->sel_re[k] = i; s->sel_im[k] = i; }
            else if (i < j) { int64_t r = packed_upper_real_index(p->n, i, j); s->sel_kind[k] = 1; s->sel_re[k] = r; s->sel_im[k] = r + 1; }
            else { int64_t r = packed_upper_real_index(p->n, j, i); s->sel_kind[k] = 2; s->sel_re[k] = r; s->sel_im[k] = r + 1; }
        }
    }
}

static void sink_free(sink* s) { free(s->sel_re); free(s->sel_im); free(s->sel_kind); }

static double weighted(const sink* s, const double* y) {
    double v = 0.0;
    for (int32_t k = 0; k < s->opt->n_weights; ++k) v += s->opt->weight_value[k] * y[s->opt->weight_index[k]];
    return v;
}

/* number of points a sink reports (OdeOutput::times().len()) */
static int64_t sink_points(const sink* s) {
    if (s->kind == OBE_OUTPUT_WEIGHTED_INTEGRAL && !s->store_trace) return s->has_last_time ? 1 : 0;
    return s->count;
}

static double sink_last_time(const sink* s) { return s->last_time; }

static void sink_push(sink* s, double t, const double* y) {
    int64_t w = s->width;
    s->last_time = t;
    s->has_last_time = 1;
    switch (s->kind) {
    case OBE_OUTPUT_WEIGHTED_INTEGRAL: {
        double value = weighted(s, y);
        if (isfinite(s->last_t)) s->integral += 0.5 * (s->last_value + value) * (t - s->last_t);
        s->last_t = t;
        s->last_value = value;
        if (s->store_trace) {
            if (s->count < s->capacity) { s->times[s->count] = t; s->vals[s->count] = s->integral; }
            s->count++;
        } else {
            if (s->capacity > 0) { s->times[0] = t; s->vals[0] = s->integral; }
            s->count = 1;
        }
        return;
    }
    case OBE_OUTPUT_WEIGHTED_RATE:
        if (s->count < s->capacity) { s->times[s->count] = t; s->vals[s->count] = weighted(s, y); }
        s->count++;
        return;
    case OBE_OUTPUT_POPULATIONS:
        if (s->count < s->capacity) {
            s->times[s->count] = t;
            for (int64_t i = 0; i < w; ++i) s->vals[s->count * w + i] = y[i * s->p->pop_stride];
        }
        s->count++;
        return;
    case OBE_OUTPUT_FULL:
        if (s->count < s->capacity) {
            s->times[s->count] = t;
            memcpy(s->vals + s->count * w, y, sizeof(double) * (size_t)w);
        }
        s->count++;
        return;
    case OBE_OUTPUT_SELECTED:
        if (s->count < s->capacity) {
            s->times[s->count] = t;
            double* v = s->vals + 2 * s->count * w;
            for (int64_t k = 0; k < w; ++k) {
                if (s->sel_kind[k] == 0) { v[2 * k] = y[s->sel_re[k]]; v[2 * k + 1] = 0.0; }
                else if (s->sel_kind[k] == 1) { v[2 * k] = y[s->sel_re[k]]; v[2 * k + 1] = y[s->sel_im[k]]; }
                else { v[2 * k] = y[s->sel_re[k]]; v[2 * k + 1] = -y[s->sel_im[k]]; }
            }
        }
        s->count++;
        return;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* integrators (ode/common.rs, ode/dopri5.rs, ode/tsit5.rs)                                    */

static inline double time_tol(double t) { return 10.0 * 2.220446049250313e-16 * fmax(fabs(t), 1.0); }
static inline int close_to_start(double t, double t0) { return fabs(t - t0) <= time_tol(t0); }
static inline double sign_of(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }

typedef struct {
    double alpha, beta, facc1, facc2, fac_old, h_max, safety, posneg;
    int reject;
} controller;

static void ctrl_init(controller* c, double t0, double t1) {
    c->beta = 0.04;
    c->alpha = 0.2 - c->beta * 0.75;
    c->facc1 = 1.0 / 0.2;
    c->facc2 = 1.0 / 10.0;
    c->fac_old = 1.0e-4;
    c->h_max = fabs(t1 - t0);
    c->reject = 0;
    c->safety = 0.9;
    c->posneg = sign_of(1.0, t1 - t0);
}

/* Controller::accept (common.rs:48-69) */
static int ctrl_accept(controller* c, double err, double h, double* h_new_out) {
    double fac11 = pow(err, c->alpha);
    double fac = fac11 * pow(c->fac_old, -c->beta);
    fac = fmax(c->facc2, fmin(c->facc1, fac / c->safety));
    double h_new = h / fac;
    if (err <= 1.0) {
        c->fac_old = fmax(err, 1.0e-4);
        if (fabs(h_new) > c->h_max) h_new = c->posneg * c->h_max;
        if (c->reject) h_new = c->posneg * fmin(fabs(h_new), fabs(h));
        c->reject = 0;
        *h_new_out = h_new;
        return 1;
    }
    h_new = h / fmin(c->facc1, fac11 / c->safety);
    c->reject = 1;
    *h_new_out = h_new;
    return 0;
}

/* Dopri5 tableau (dopri5.rs:5-43; Hairer, Norsett & Wanner DOPRI5) */
static const double D_C2 = 1.0 / 5.0, D_C3 = 3.0 / 10.0, D_C4 = 4.0 / 5.0, D_C5 = 8.0 / 9.0;
static const double D_A21 = 1.0 / 5.0;
static const double D_A31 = 3.0 / 40.0, D_A32 = 9.0 / 40.0;
static const double D_A41 = 44.0 / 45.0, D_A42 = -56.0 / 15.0, D_A43 = 32.0 / 9.0;
static const double D_A51 = 19372.0 / 6561.0, D_A52 = -25360.0 / 2187.0, D_A53 = 64448.0 / 6561.0, D_A54 = -212.0 / 729.0;
static const double D_A61 = 9017.0 / 3168.0, D_A62 = -355.0 / 33.0, D_A63 = 46732.0 / 5247.0, D_A64 = 49.0 / 176.0, D_A65 = -5103.0 / 18656.0;
static const double D_A71 = 35.0 / 384.0, D_A72 = 0.0, D_A73 = 500.0 / 1113.0, D_A74 = 125.0 / 192.0, D_A75 = -2187.0 / 6784.0, D_A76 = 11.0 / 84.0;
static const double D_E1 = 71.0 / 57600.0, D_E3 = -71.0 / 16695.0, D_E4 = 71.0 / 1920.0, D_E5 = -17253.0 / 339200.0, D_E6 = 22.0 / 525.0, D_E7 = -1.0 / 40.0;
static const double D_D1 = -12715105075.0 / 11282082432.0, D_D3 = 87487479700.0 / 32700410799.0, D_D4 = -10690763975.0 / 1880347072.0;
static const double D_D5 = 701980252875.0 / 199316789632.0, D_D6 = -1453857185.0 / 822651844.0, D_D7 = 69997945.0 / 29380423.0;

/* Tsit5 tableau (tsit5.rs:5-60; Tsitouras 2011) */
static const double T_C2 = 0.161, T_C3 = 0.327, T_C4 = 0.9, T_C5 = 0.9800255409045097;
static const double T_A21 = 0.161;
static const double T_A31 = -0.008480655492356989, T_A32 = 0.335480655492357;
static const double T_A41 = 2.8971530571054935, T_A42 = -6.359448489975075, T_A43 = 4.3622954328695815;
static const double T_A51 = 5.325864828439257, T_A52 = -11.748883564062828, T_A53 = 7.4955393428898365, T_A54 = -0.09249506636175525;
static const double T_A61 = 5.86145544294642, T_A62 = -12.92096931784711, T_A63 = 8.159367898576159, T_A64 = -0.071584973281401, T_A65 = -0.028269050394068383;
static const double T_A71 = 0.09646076681806523, T_A72 = 0.01, T_A73 = 0.4798896504144996, T_A74 = 1.379008574103742, T_A75 = -3.290069515436081, T_A76 = 2.324710524099774;
static const double T_E1 = -0.0017800110522257771, T_E2 = -0.0008164344596567469, T_E3 = 0.007880878010261995, T_E4 = -0.1447110071732629;
static const double T_E5 = 0.5823571654525552, T_E6 = -0.458082105929187, T_E7 = 1.0 / 66.0;
static const double T_R11 = 1.0, T_R12 = -2.763706197274826, T_R13 = 2.9132554618219126, T_R14 = -1.0530884977290216;
static const double T_R22 = 0.1317, T_R23 = -0.2234, T_R24 = 0.1017;
static const double T_R32 = 3.9302962368947516, T_R33 = -5.941033872131505, T_R34 = 2.490627285651253;
static const double T_R42 = -12.411077166933676, T_R43 = 30.33818863028232, T_R44 = -16.548102889244902;
static const double T_R52 = 37.50931341651104, T_R53 = -88.1789048947664, T_R54 = 47.37952196281928;
static const double T_R62 = -27.896526289197286, T_R63 = 65.09189467479366, T_R64 = -34.87065786149661;
static const double T_R72 = 1.5, T_R73 = -4.0, T_R74 = 2.5;

typedef struct {
    int64_t dim;
    double *y, *yn, *yt, *ys, *ds, *r0, *r1, *r2, *r3, *r4, *f0, *f1, *k;
    double* ev_y;
} rk_buf;

static void rkb_init(rk_buf* b, int64_t dim) {
    b->dim = dim;
    size_t n = (size_t)dim;
    b->y = (double*)calloc(n, 8); b->yn = (double*)calloc(n, 8); b->yt = (double*)calloc(n, 8);
    b->ys = (double*)calloc(n, 8); b->ds = (double*)calloc(n, 8);
    b->r0 = (double*)calloc(n, 8); b->r1 = (double*)calloc(n, 8); b->r2 = (double*)calloc(n, 8);
    b->r3 = (double*)calloc(n, 8); b->r4 = (double*)calloc(n, 8);
    b->f0 = (double*)calloc(n, 8); b->f1 = (double*)calloc(n, 8);
    b->k = (double*)calloc(7 * n, 8);
    b->ev_y = (double*)calloc(n, 8);
}

static void rkb_free(rk_buf* b) {
    free(b->y); free(b->yn); free(b->yt); free(b->ys); free(b->ds); free(b->r0); free(b->r1);
    free(b->r2); free(b->r3); free(b->r4); free(b->f0); free(b->f1); free(b->k); free(b->ev_y);
}

/* hinit (common.rs:72-118) */
static int hinit(workspace* w, const double* y, double x, double x_end, double atol, double rtol,
                 double* f0, double* f1, double* ytmp, int64_t dim, double* h_out, errbuf* e) {
    if (ws_rhs(w, x, y, f0, e)) return 1;
    double posneg = sign_of(1.0, x_end - x);
    double h_max = fabs(x_end - x);
    double d0 = 0.0, d1 = 0.0;
    for (int64_t i = 0; i < dim; ++i) {
        double sci = atol + fabs(y[i]) * rtol;
        d0 += (y[i] / sci) * (y[i] / sci);
        d1 += (f0[i] / sci) * (f0[i] / sci);
    }
    double h0 = (d0 < 1.0e-10 || d1 < 1.0e-10) ? 1.0e-6 : 0.01 * sqrt(d0 / d1);
    h0 = fmin(h0, h_max);
    h0 = sign_of(h0, posneg);
    for (int64_t i = 0; i < dim; ++i) ytmp[i] = y[i] + f0[i] * h0;
    if (ws_rhs(w, x + h0, ytmp, f1, e)) return 1;
    double d2 = 0.0;
    for (int64_t i = 0; i < dim; ++i) {
        double sci = atol + fabs(y[i]) * rtol;
        d2 += ((f1[i] - f0[i]) / sci) * ((f1[i] - f0[i]) / sci);
    }
    d2 = sqrt(d2) / h0;
    double h1 = fmax(sqrt(d1), fabs(d2)) <= 1.0e-15 ? fmax(1.0e-6, fabs(h0) * 1.0e-3) : pow(0.01 / fmax(sqrt(d1), d2), 1.0 / 5.0);
    *h_out = sign_of(fmin(100.0 * fabs(h0), fmin(h1, h_max)), posneg);
    return 0;
}

/* build_save_plan (common.rs:124-151) -> times in *out (malloc'd), count in *n_out, or has=0 */
static int build_save_plan(const obe_solve_options* o, double t0, double t1, double** out, int64_t* n_out, errbuf* e) {
    *out = NULL;
    *n_out = 0;
    if (!o->has_saveat) return 0;
    int64_t n = o->n_saveat;
    double* times = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    int64_t c = 0;
    if (o->save_start) times[c++] = t0;
    for (int64_t i = 0; i < n; ++i) {
        double tm = o->saveat[i];
        if (o->save_start && close_to_start(tm, t0)) continue;
        if (!isfinite(tm)) { free(times); return fail(e, "saveat contains non-finite value"); }
        if (tm < t0 - time_tol(t0) || tm > t1 + time_tol(t1)) {
            char a[64], b[64], cbuf[64];
            fmt_f64(tm, a, sizeof a); fmt_f64(t0, b, sizeof b); fmt_f64(t1, cbuf, sizeof cbuf);
            free(times);
            return fail(e, "saveat value %s is outside [%s, %s]", a, b, cbuf);
        }
        times[c++] = tm;
    }
    *out = times;
    *n_out = c;
    return 0;
}

static inline int crossed_zero(double g0, double g1) {
    return g0 == 0.0 || g1 == 0.0 || (g0 < 0.0 && g1 > 0.0) || (g0 > 0.0 && g1 < 0.0);
}

/* push_unique (dopri5.rs:150-158) */
static void push_unique(sink* s, double t, const double* y) {
    if (sink_points(s) > 0 && fabs(sink_last_time(s) - t) <= time_tol(t)) return;
    sink_push(s, t, y);
}

/* dense outputs */
static void dopri_dense_prep(const rk_buf* b, double h) {
    int64_t dim = b->dim;
    const double* k = b->k;
    for (int64_t i = 0; i < dim; ++i) {
        b->r4[i] = h * (D_D1 * k[i] + D_D3 * k[2 * dim + i] + D_D4 * k[3 * dim + i] + D_D5 * k[4 * dim + i] + D_D6 * k[5 * dim + i] + D_D7 * k[6 * dim + i]);
    }
    for (int64_t i = 0; i < dim; ++i) {
        double d = b->yn[i] - b->y[i];
        double bb = k[i] * h - d;
        b->r0[i] = b->y[i];
        b->r1[i] = d;
        b->r2[i] = bb;
        b->r3[i] = -k[6 * dim + i] * h + d - bb;
    }
}

static void dopri_dense_out(const rk_buf* b, double th, double* out) {
    double th1 = 1.0 - th;
    for (int64_t i = 0; i < b->dim; ++i)
        out[i] = b->r0[i] + (b->r1[i] + (b->r2[i] + (b->r3[i] + b->r4[i] * th1) * th) * th1) * th;
}

static void tsit_dense_out(const rk_buf* b, double th, double h, double* out) {
    int64_t d = b->dim;
    const double* k = b->k;
    double t2 = th * th, t3 = t2 * th, t4 = t3 * th;
    double b1 = T_R11 * th + T_R12 * t2 + T_R13 * t3 + T_R14 * t4;
    double b2 = T_R22 * t2 + T_R23 * t3 + T_R24 * t4;
    double b3 = T_R32 * t2 + T_R33 * t3 + T_R34 * t4;
    double b4 = T_R42 * t2 + T_R43 * t3 + T_R44 * t4;
    double b5 = T_R52 * t2 + T_R53 * t3 + T_R54 * t4;
    double b6 = T_R62 * t2 + T_R63 * t3 + T_R64 * t4;
    double b7 = T_R72 * t2 + T_R73 * t3 + T_R74 * t4;
    for (int64_t i = 0; i < d; ++i)
        out[i] = b->y[i] + h * (b1 * k[i] + b2 * k[d + i] + b3 * k[2 * d + i] + b4 * k[3 * d + i] + b5 * k[4 * d + i] + b6 * k[5 * d + i] + b7 * k[6 * d + i]);
}

/* solve_dopri5 (dopri5.rs:160-379) and solve_tsit5 (tsit5.rs:159-363) */
static int solve_rk(workspace* w, int tsit, const double* y0, const obe_solve_options* o, sink* out, obe_traj_stats* st, errbuf* e) {
    const orc_plan* p = w->p;
    int64_t dim = p->N;
    double t0 = o->t0, t1 = o->t1;
    memset(st, 0, sizeof *st);
    st->event_time = NAN;
    if (o->maxiters <= 0) return fail(e, "maxiters must be positive");
    if (t1 < t0) return fail(e, "only forward integration");
    if (t1 == t0) {
        if (o->save_start) sink_push(out, t0, y0);
        st->n_points = sink_points(out);
        return 0;
    }
    double* sp = NULL;
    int64_t n_sp = 0;
    if (build_save_plan(o, t0, t1, &sp, &n_sp, e)) return 1;
    int has_sp = o->has_saveat;
    rk_buf b;
    rkb_init(&b, dim);
    int rc = 0;
    double* k = b.k;
    memcpy(b.y, y0, sizeof(double) * (size_t)dim);
    double x = t0, h;
    if (isfinite(o->dt) && o->dt > 0.0) {
        h = fmin(o->dt, t1 - t0);
    } else if ((rc = hinit(w, b.y, x, t1, o->abstol, o->reltol, b.f0, b.f1, b.yt, dim, &h, e))) {
        goto done;
    }
    controller ctrl;
    ctrl_init(&ctrl, t0, t1);
    double pn = sign_of(1.0, t1 - t0);
    if ((rc = ws_rhs(w, x, b.y, k, e))) goto done;
    st->rhs_calls += 1;
    int ev_old_has;
    double ev_old;
    if ((rc = ws_event(w, x, b.y, &ev_old_has, &ev_old, e))) goto done;
    int64_t si = 0;
    if (has_sp) {
        while (si < n_sp && close_to_start(sp[si], t0)) { sink_push(out, sp[si], b.y); ++si; }
    } else if (o->save_start) {
        sink_push(out, x, b.y);
    }
    int64_t ns = 0, nst = 0, ia = 0;
    int last = 0;
    char xs[64];
    while (!last) {
        if (ns > o->maxiters) { fmt_f64(x, xs, sizeof xs); rc = fail(e, "Stopped at x=%s. Need more than %lld steps.", xs, (long long)ns); goto done; }
        if (0.1 * fabs(h) <= 2.220446049250313e-16 * fabs(x)) { fmt_f64(x, xs, sizeof xs); rc = fail(e, "Stopped at x=%s. Step size underflow.", xs); goto done; }
        if ((x + 1.01 * h - t1) * pn > 0.0) { h = t1 - x; last = 1; }
        ++ns;
        double *y = b.y, *yt = b.yt, *yn = b.yn;
        if (!tsit) {
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * D_A21 * k[i];
            if ((rc = ws_rhs(w, x + h * D_C2, yt, k + dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (D_A31 * k[i] + D_A32 * k[dim + i]);
            if ((rc = ws_rhs(w, x + h * D_C3, yt, k + 2 * dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (D_A41 * k[i] + D_A42 * k[dim + i] + D_A43 * k[2 * dim + i]);
            if ((rc = ws_rhs(w, x + h * D_C4, yt, k + 3 * dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (D_A51 * k[i] + D_A52 * k[dim + i] + D_A53 * k[2 * dim + i] + D_A54 * k[3 * dim + i]);
            if ((rc = ws_rhs(w, x + h * D_C5, yt, k + 4 * dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (D_A61 * k[i] + D_A62 * k[dim + i] + D_A63 * k[2 * dim + i] + D_A64 * k[3 * dim + i] + D_A65 * k[4 * dim + i]);
            memcpy(b.ys, yt, sizeof(double) * (size_t)dim);
            if ((rc = ws_rhs(w, x + h * 1.0, yt, k + 5 * dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yn[i] = y[i] + h * (D_A71 * k[i] + D_A72 * k[dim + i] + D_A73 * k[2 * dim + i] + D_A74 * k[3 * dim + i] + D_A75 * k[4 * dim + i] + D_A76 * k[5 * dim + i]);
            if ((rc = ws_rhs(w, x + h * 1.0, yn, k + 6 * dim, e))) goto done;
        } else {
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * T_A21 * k[i];
            if ((rc = ws_rhs(w, x + h * T_C2, yt, k + dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (T_A31 * k[i] + T_A32 * k[dim + i]);
            if ((rc = ws_rhs(w, x + h * T_C3, yt, k + 2 * dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (T_A41 * k[i] + T_A42 * k[dim + i] + T_A43 * k[2 * dim + i]);
            if ((rc = ws_rhs(w, x + h * T_C4, yt, k + 3 * dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (T_A51 * k[i] + T_A52 * k[dim + i] + T_A53 * k[2 * dim + i] + T_A54 * k[3 * dim + i]);
            if ((rc = ws_rhs(w, x + h * T_C5, yt, k + 4 * dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (T_A61 * k[i] + T_A62 * k[dim + i] + T_A63 * k[2 * dim + i] + T_A64 * k[3 * dim + i] + T_A65 * k[4 * dim + i]);
            memcpy(b.ys, yt, sizeof(double) * (size_t)dim);
            if ((rc = ws_rhs(w, x + h * 1.0, yt, k + 5 * dim, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yn[i] = y[i] + h * (T_A71 * k[i] + T_A72 * k[dim + i] + T_A73 * k[2 * dim + i] + T_A74 * k[3 * dim + i] + T_A75 * k[4 * dim + i] + T_A76 * k[5 * dim + i]);
            if ((rc = ws_rhs(w, x + h * 1.0, yn, k + 6 * dim, e))) goto done;
        }
        st->rhs_calls += 6;
        double err = 0.0;
        for (int64_t i = 0; i < dim; ++i) {
            double sc = o->abstol + fmax(fabs(y[i]), fabs(yn[i])) * o->reltol;
            double ei;
            if (!tsit)
                ei = h * (D_E1 * k[i] + D_E3 * k[2 * dim + i] + D_E4 * k[3 * dim + i] + D_E5 * k[4 * dim + i] + D_E6 * k[5 * dim + i] + D_E7 * k[6 * dim + i]);
            else
                ei = h * (T_E1 * k[i] + T_E2 * k[dim + i] + T_E3 * k[2 * dim + i] + T_E4 * k[3 * dim + i] + T_E5 * k[4 * dim + i] + T_E6 * k[5 * dim + i] + T_E7 * k[6 * dim + i]);
            err += (ei / sc) * (ei / sc);
        }
        err = sqrt(err / (double)dim);
        double hn;
        int acc = ctrl_accept(&ctrl, err, h, &hn);
        if (acc) {
            st->accepted_steps += 1;
            if (st->accepted_steps % 1000 == 0 || ia > 0) {
                double n2 = 0.0, d2 = 0.0;
                for (int64_t i = 0; i < dim; ++i) {
                    double dk = k[6 * dim + i] - k[5 * dim + i];
                    double dy = yn[i] - b.ys[i];
                    n2 += dk * dk;
                    d2 += dy * dy;
                }
                double hl = d2 > 0.0 ? h * sqrt(n2 / d2) : 0.0;
                if (hl > 3.25) {
                    ++ia;
                    nst = 0;
                    if (ia == 15) { fmt_f64(x, xs, sizeof xs); rc = fail(e, "Stiff at x=%s.", xs); goto done; }
                } else {
                    ++nst;
                    if (nst == 6) ia = 0;
                }
            }
            double xo = x;
            x += h;
            int ev_new_has;
            double ev_new;
            if ((rc = ws_event(w, x, yn, &ev_new_has, &ev_new, e))) goto done;
            int hit = 0;
            double te = 0.0;
            const double* ye = NULL;
            int dense_ready = 0;
            if (ev_old_has && ev_new_has && crossed_zero(ev_old, ev_new)) {
                if (ev_old == 0.0) { hit = 1; te = xo; memcpy(b.ev_y, y, sizeof(double) * (size_t)dim); ye = b.ev_y; }
                else if (ev_new == 0.0) { hit = 1; te = x; memcpy(b.ev_y, yn, sizeof(double) * (size_t)dim); ye = b.ev_y; }
                else {
                    if (!tsit) { dopri_dense_prep(&b, h); dense_ready = 1; }
                    double lo = 0.0, hi = 1.0, glo = ev_old;
                    for (int it = 0; it < 60; ++it) {
                        double mid = 0.5 * (lo + hi);
                        if (!tsit) dopri_dense_out(&b, mid, b.ds); else tsit_dense_out(&b, mid, h, b.ds);
                        int has;
                        double gm;
                        if ((rc = ws_event(w, xo + mid * h, b.ds, &has, &gm, e))) goto done;
                        if (!has) { rc = fail(e, "event disappeared during root finding"); goto done; }
                        if (gm == 0.0) { lo = mid; hi = mid; break; }
                        if ((glo < 0.0 && gm > 0.0) || (glo > 0.0 && gm < 0.0)) hi = mid;
                        else { lo = mid; glo = gm; }
                    }
                    double theta = 0.5 * (lo + hi);
                    if (!tsit) dopri_dense_out(&b, theta, b.ds); else tsit_dense_out(&b, theta, h, b.ds);
                    memcpy(b.ev_y, b.ds, sizeof(double) * (size_t)dim);
                    hit = 1;
                    te = xo + theta * h;
                    ye = b.ev_y;
                }
            }
            if (has_sp) {
                double event_time = hit ? te : x;
                while (si < n_sp && sp[si] <= event_time + time_tol(event_time)) {
                    double ts = sp[si];
                    if (ts >= xo - time_tol(xo)) {
                        if (fabs(ts - xo) <= time_tol(xo)) sink_push(out, ts, y);
                        else if (fabs(ts - x) <= time_tol(x)) sink_push(out, ts, yn);
                        else {
                            if (!tsit) {
                                if (!dense_ready) { dopri_dense_prep(&b, h); dense_ready = 1; }
                                dopri_dense_out(&b, (ts - xo) / h, b.ds);
                            } else {
                                tsit_dense_out(&b, (ts - xo) / h, h, b.ds);
                            }
                            sink_push(out, ts, b.ds);
                        }
                    }
                    ++si;
                }
            } else if (!hit) {
                sink_push(out, x, yn);
            }
            if (hit) {
                push_unique(out, te, ye);
                st->event_triggered = 1;
                st->event_time = te;
                break;
            }
            double* tmp = b.y; b.y = b.yn; b.yn = tmp;
            memcpy(k, k + 6 * dim, sizeof(double) * (size_t)dim);
            ev_old_has = ev_new_has;
            ev_old = ev_new;
            if (last) break;
        } else {
            last = 0;
            if (st->accepted_steps >= 1) st->rejected_steps += 1;
        }
        h = hn;
    }
    if (has_sp && si != n_sp && !st->event_triggered) {
        rc = fail(e, "ended before all saveat: %lld of %lld", (long long)si, (long long)n_sp);
    }
done:
    st->n_points = sink_points(out);
    rkb_free(&b);
    free(sp);
    return rc;
}

/* solve_fixed_step (fixed.rs:133-249): dopri5 (fixed.rs:50-101), rk2 (:28-48) and rk4
 * (:103-131) steppers; the step is dt clipped to t1 and to the next saveat time
 * (next_step_limit, fixed.rs:16-26); no dense output, events end on the step that crosses. */
static int solve_fixed(workspace* w, int stepper, const double* y0, const obe_solve_options* o, sink* out, obe_traj_stats* st, errbuf* e) {
    const orc_plan* p = w->p;
    int64_t dim = p->N;
    double t0 = o->t0, t1 = o->t1;
    memset(st, 0, sizeof *st);
    st->event_time = NAN;
    if (o->maxiters <= 0) return fail(e, "maxiters must be positive");
    if (t1 < t0) return fail(e, "only forward integration");
    if (!isfinite(o->dt) || o->dt <= 0.0) return fail(e, "fixed-step solvers require positive finite dt");
    if (t1 == t0) {
        if (o->save_start) sink_push(out, t0, y0);
        st->n_points = sink_points(out);
        return 0;
    }
    double* sp = NULL;
    int64_t n_sp = 0;
    if (build_save_plan(o, t0, t1, &sp, &n_sp, e)) return 1;
    int has_sp = o->has_saveat;
    rk_buf b;
    rkb_init(&b, dim);
    int rc = 0;
    double *k = b.k, *k1 = k, *k2 = k + dim, *k3 = k + 2 * dim, *k4 = k + 3 * dim, *k5 = k + 4 * dim, *k6 = k + 5 * dim;
    memcpy(b.y, y0, sizeof(double) * (size_t)dim);
    double x = t0;
    int64_t si = 0;
    if (has_sp) {
        while (si < n_sp && close_to_start(sp[si], t0)) { sink_push(out, sp[si], b.y); ++si; }
    } else if (o->save_start) {
        sink_push(out, x, b.y);
    }
    int ev_old_has;
    double ev_old;
    if ((rc = ws_event(w, x, b.y, &ev_old_has, &ev_old, e))) goto done;
    int64_t steps = 0;
    char xs[64];
    while (x < t1 - time_tol(t1)) {
        if (steps >= o->maxiters) { fmt_f64(x, xs, sizeof xs); rc = fail(e, "Stopped at x=%s. Need more than %lld steps.", xs, (long long)steps); goto done; }
        double target = fmin(x + o->dt, t1);
        if (has_sp && si < n_sp && sp[si] > x + time_tol(x)) target = fmin(target, sp[si]);
        double h = target - x;
        if (h <= 0.0 || 0.1 * h <= 2.220446049250313e-16 * fmax(fabs(x), 1.0)) { fmt_f64(x, xs, sizeof xs); rc = fail(e, "Stopped at x=%s. Step size underflow.", xs); goto done; }
        double *y = b.y, *yt = b.yt, *yn = b.yn;
        if ((rc = ws_rhs(w, x, y, k1, e))) goto done;
        if (stepper == OBE_SOLVER_FIXED_RK2) {
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + 0.5 * h * k1[i];
            if ((rc = ws_rhs(w, x + 0.5 * h, yt, k2, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yn[i] = y[i] + h * k2[i];
            st->rhs_calls += 2;
        } else if (stepper == OBE_SOLVER_FIXED_RK4) {
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + 0.5 * h * k1[i];
            if ((rc = ws_rhs(w, x + 0.5 * h, yt, k2, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + 0.5 * h * k2[i];
            if ((rc = ws_rhs(w, x + 0.5 * h, yt, k3, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * k3[i];
            if ((rc = ws_rhs(w, x + h, yt, k4, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yn[i] = y[i] + h * (k1[i] + 2.0 * k2[i] + 2.0 * k3[i] + k4[i]) / 6.0;
            st->rhs_calls += 4;
        } else {
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * D_A21 * k1[i];
            if ((rc = ws_rhs(w, x + h * D_C2, yt, k2, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (D_A31 * k1[i] + D_A32 * k2[i]);
            if ((rc = ws_rhs(w, x + h * D_C3, yt, k3, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (D_A41 * k1[i] + D_A42 * k2[i] + D_A43 * k3[i]);
            if ((rc = ws_rhs(w, x + h * D_C4, yt, k4, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (D_A51 * k1[i] + D_A52 * k2[i] + D_A53 * k3[i] + D_A54 * k4[i]);
            if ((rc = ws_rhs(w, x + h * D_C5, yt, k5, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yt[i] = y[i] + h * (D_A61 * k1[i] + D_A62 * k2[i] + D_A63 * k3[i] + D_A64 * k4[i] + D_A65 * k5[i]);
            if ((rc = ws_rhs(w, x + h, yt, k6, e))) goto done;
            for (int64_t i = 0; i < dim; ++i) yn[i] = y[i] + h * (D_A71 * k1[i] + D_A73 * k3[i] + D_A74 * k4[i] + D_A75 * k5[i] + D_A76 * k6[i]);
            st->rhs_calls += 6;
        }
        st->accepted_steps += 1;
        ++steps;
        double xo = x;
        x += h;
        int ev_new_has;
        double ev_new;
        if ((rc = ws_event(w, x, yn, &ev_new_has, &ev_new, e))) goto done;
        int hit = 0;
        if (ev_old_has && ev_new_has && crossed_zero(ev_old, ev_new)) {
            hit = 1;
            st->event_triggered = 1;
            st->event_time = ev_old == 0.0 ? xo : x;
        }
        if (has_sp) {
            double stop_time = hit ? st->event_time : x;
            while (si < n_sp && sp[si] <= stop_time + time_tol(stop_time)) { sink_push(out, sp[si], yn); ++si; }
        } else if (!hit) {
            sink_push(out, x, yn);
        }
        if (hit) {
            sink_push(out, st->event_time, yn);
            break;
        }
        double* tmp = b.y; b.y = b.yn; b.yn = tmp;
        ev_old_has = ev_new_has;
        ev_old = ev_new;
    }
    if (has_sp && si != n_sp && !st->event_triggered) {
        rc = fail(e, "ended before all saveat: %lld of %lld", (long long)si, (long long)n_sp);
    }
done:
    st->n_points = sink_points(out);
    rkb_free(&b);
    free(sp);
    return rc;
}

static int solve_any(workspace* w, const double* y0, const obe_solve_options* o, sink* out, obe_traj_stats* st, errbuf* e) {
    w->eff_hint = 0;  /* a fresh RHS workspace per trajectory (effective_lindblad/rhs.rs:14-24) */
    if (o->solver == OBE_SOLVER_DOPRI5 || o->solver == OBE_SOLVER_TSIT5)
        return solve_rk(w, o->solver == OBE_SOLVER_TSIT5, y0, o, out, st, e);
    return solve_fixed(w, o->solver, y0, o, out, st, e);
}

static int setup_event(workspace* w, const obe_solve_options* o) {
    w->ev_kind = o->event_kind;
    if (o->event_kind == OBE_EVENT_POPULATION) {
        w->ev_idx = o->event_indices;
        w->n_ev_idx = o->n_event_indices;
        w->ev_thr = o->event_threshold;
    } else if (o->event_kind == OBE_EVENT_EXPRESSION) {
        expr_from_desc(&w->ev_expr, &o->event_expr);
        w->ev_has_expr = 1;
        if (w->ev_expr.n + 4 > w->p->max_stack + 4) {
            free(w->gstack);
            free(w->sstack);
            w->gstack = (rv*)malloc(sizeof(rv) * (size_t)(w->ev_expr.n + 4));
            w->sstack = (cx*)malloc(sizeof(cx) * (size_t)(w->ev_expr.n + 4));
        }
    }
    return 0;
}

static int check_solver(const obe_solve_options* o, errbuf* e) {
    if (o->solver < OBE_SOLVER_DOPRI5 || o->solver > OBE_SOLVER_FIXED_RK4)
        return fail(e, "solver must be 'dopri5', 'tsit5', 'fixed_dopri5', 'fixed_rk2', or 'fixed_rk4', got %d", o->solver);
    return 0;
}

int orc_rhs(const orc_plan* plan, int32_t n_override, const int64_t* override_slots, const double* override_values,
            double t, const double* y, double* dy, int32_t use_split_input_rhs, char* err, size_t err_len) {
    errbuf e = {{0}, 0};
    workspace w;
    ws_init(&w, plan, use_split_input_rhs);
    ws_set_overrides(&w, n_override, override_slots, override_values);
    int rc = ws_rhs(&w, t, y, dy, &e);
    if (rc) copy_err(&e, err, err_len);
    ws_free(&w);
    return rc;
}

int orc_coefficients(const orc_plan* plan, int32_t n_override, const int64_t* override_slots,
                     const double* override_values, double t, double* out, char* err, size_t err_len) {
    errbuf e = {{0}, 0};
    workspace w;
    ws_init(&w, plan, 1);
    ws_set_overrides(&w, n_override, override_slots, override_values);
    int rc = ws_eval_params(&w, t, &e) || ws_eval_coeffs(&w, t, &e);
    if (!rc)
        for (int32_t k = 0; k < plan->n_coeff; ++k) { out[2 * k] = w.coeff[k].re; out[2 * k + 1] = w.coeff[k].im; }
    else copy_err(&e, err, err_len);
    ws_free(&w);
    return rc;
}

int orc_solve_single(const orc_plan* plan, const obe_solve_options* opt, const double* rho0,
                     int32_t n_param_slots, const int64_t* param_slots, const double* param_values,
                     int64_t capacity, double* times, double* values, obe_traj_stats* stats,
                     int32_t use_split_input_rhs, char* err, size_t err_len) {
    errbuf e = {{0}, 0};
    if (check_solver(opt, &e)) { copy_err(&e, err, err_len); return 1; }
    workspace w;
    ws_init(&w, plan, use_split_input_rhs);
    if (n_param_slots > 0) ws_set_overrides(&w, n_param_slots, param_slots, param_values);
    setup_event(&w, opt);
    sink s;
    sink_init(&s, plan, opt, capacity, times, values);
    int rc = solve_any(&w, rho0, opt, &s, stats, &e);
    sink_free(&s);
    ws_free(&w);
    if (rc) copy_err(&e, err, err_len);
    return rc;
}

int orc_solve_batch(const orc_plan* plan, const obe_solve_options* opt, int64_t n_traj,
                    const double* rho0, int64_t rho0_stride, int32_t n_param_slots,
                    const int64_t* param_slots, const double* param_values, int64_t time_count,
                    int64_t width, double* values, double* out_times, obe_traj_stats* stats,
                    int32_t threads, int32_t use_split_input_rhs, char* err, size_t err_len) {
    errbuf first = {{0}, 0};
    if (check_solver(opt, &first)) { copy_err(&first, err, err_len); return 1; }
    int32_t cplx;
    int64_t wdt = orc_output_width(plan, opt, &cplx);
    if (wdt != width) { fail(&first, "output width mismatch: %lld vs %lld", (long long)wdt, (long long)width); copy_err(&first, err, err_len); return 1; }
    int64_t per = time_count * width * (cplx ? 2 : 1);
    int64_t first_bad = -1;
    char first_msg[512] = {0};
#ifdef _OPENMP
    int nthreads = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        workspace w;
        ws_init(&w, plan, use_split_input_rhs);
        setup_event(&w, opt);
        double* tbuf = (double*)malloc(sizeof(double) * (size_t)(time_count > 0 ? time_count : 1));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int64_t b = 0; b < n_traj; ++b) {
            errbuf e = {{0}, 0};
            if (n_param_slots > 0) ws_set_overrides(&w, n_param_slots, param_slots, param_values + 2 * b * n_param_slots);
            else w.valid = 0;
            sink s;
            sink_init(&s, plan, opt, time_count, tbuf, values + b * per);
            obe_traj_stats st;
            int rc = solve_any(&w, rho0 + b * rho0_stride, opt, &s, &st, &e);
            if (!rc && st.n_points != time_count)
                rc = fail(&e, "expected %lld output points, got %lld", (long long)time_count, (long long)st.n_points);
            st.status = rc;
            if (stats) stats[b] = st;
            if (!rc && b == 0 && out_times) memcpy(out_times, tbuf, sizeof(double) * (size_t)time_count);
            if (rc) {
#ifdef _OPENMP
#pragma omp critical
#endif
                {
                    if (first_bad < 0 || b < first_bad) {
                        first_bad = b;
                        snprintf(first_msg, sizeof first_msg, "%s", e.msg);
                    }
                }
            }
            sink_free(&s);
        }
        free(tbuf);
        ws_free(&w);
    }
    if (first_bad >= 0) {
        if (err && err_len) snprintf(err, err_len, "trajectory %lld: %s", (long long)first_bad, first_msg);
        return 1;
    }
    return 0;
}

int32_t orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Replay of a frozen step sequence (test support for the GPU adjoint): for each trajectory, the
 * given accepted steps (t_n, h_n) of Dopri5 (dopri5.rs:60-86) or Tsit5 (tsit5.rs:70-103), no step
 * control, no error estimate; outputs the weighted trapezoid integral of the pushed points
 * (output.rs:314-330; t0 pushed when save_start) or the final populations.  With event_hit[t] set
 * the last step is the one that ended on opt's stop event: its crossing is found again as the
 * solver finds it (dopri5.rs:280-317: the seventh stage, the 60-step bisection on the dense
 * output) and the output ends at that time and state (push_unique, dopri5.rs:149-158).  Central
 * finite differences of this map check the adjoint of the same frozen sequence. */
int orc_solve_replay(const orc_plan* plan, const obe_solve_options* opt, int64_t n_traj, const double* rho0, int64_t rho0_stride,
                     int32_t n_param_slots, const int64_t* param_slots, const double* param_values, const int64_t* n_steps,
                     const double* steps, int64_t max_steps, const int32_t* event_hit, int64_t width, double* values, char* err,
                     size_t err_len) {
    errbuf e = {{0}, 0};
    const int tsit = opt->solver == OBE_SOLVER_TSIT5;
    if (opt->solver != OBE_SOLVER_DOPRI5 && !tsit) { fail(&e, "replay supports dopri5 and tsit5"); copy_err(&e, err, err_len); return 1; }
    const int integral = opt->output == OBE_OUTPUT_WEIGHTED_INTEGRAL;
    const int64_t n = plan->n, N = plan->N;
    if (width != (integral ? 1 : n)) { fail(&e, "replay output width mismatch"); copy_err(&e, err, err_len); return 1; }
    workspace w;
    ws_init(&w, plan, 1);
    setup_event(&w, opt);
    rk_buf b;
    rkb_init(&b, N);
    int rc = 0;
    for (int64_t t = 0; t < n_traj && !rc; ++t) {
        const int ev_step = event_hit && event_hit[t] && opt->event_kind != OBE_EVENT_NONE && n_steps[t] > 0;
        const double* yout = NULL;
        if (n_param_slots > 0) ws_set_overrides(&w, n_param_slots, param_slots, param_values + 2 * t * n_param_slots);
        else w.valid = 0;
        double* y = b.y, *yt = b.yt, *yn = b.yn, *k = b.k;
        memcpy(y, rho0 + t * rho0_stride, sizeof(double) * (size_t)N);
        double integ = 0.0, last_t = 0.0, last_v = 0.0;
        int have_last = 0;
        if (integral && opt->save_start) {
            last_t = opt->t0;
            last_v = 0.0;
            for (int32_t q = 0; q < opt->n_weights; ++q) last_v += opt->weight_value[q] * y[opt->weight_index[q]];
            have_last = 1;
        }
        for (int64_t s = 0; s < n_steps[t] && !rc; ++s) {
            const double x = steps[2 * (t * max_steps + s)], h = steps[2 * (t * max_steps + s) + 1];
            if ((rc = ws_rhs(&w, x, y, k, &e))) break;
            if (!tsit) {
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * D_A21 * k[i];
                if ((rc = ws_rhs(&w, x + h * D_C2, yt, k + N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * (D_A31 * k[i] + D_A32 * k[N + i]);
                if ((rc = ws_rhs(&w, x + h * D_C3, yt, k + 2 * N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * (D_A41 * k[i] + D_A42 * k[N + i] + D_A43 * k[2 * N + i]);
                if ((rc = ws_rhs(&w, x + h * D_C4, yt, k + 3 * N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * (D_A51 * k[i] + D_A52 * k[N + i] + D_A53 * k[2 * N + i] + D_A54 * k[3 * N + i]);
                if ((rc = ws_rhs(&w, x + h * D_C5, yt, k + 4 * N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * (D_A61 * k[i] + D_A62 * k[N + i] + D_A63 * k[2 * N + i] + D_A64 * k[3 * N + i] + D_A65 * k[4 * N + i]);
                if ((rc = ws_rhs(&w, x + h, yt, k + 5 * N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yn[i] = y[i] + h * (D_A71 * k[i] + D_A72 * k[N + i] + D_A73 * k[2 * N + i] + D_A74 * k[3 * N + i] + D_A75 * k[4 * N + i] + D_A76 * k[5 * N + i]);
            } else {
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * T_A21 * k[i];
                if ((rc = ws_rhs(&w, x + h * T_C2, yt, k + N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * (T_A31 * k[i] + T_A32 * k[N + i]);
                if ((rc = ws_rhs(&w, x + h * T_C3, yt, k + 2 * N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * (T_A41 * k[i] + T_A42 * k[N + i] + T_A43 * k[2 * N + i]);
                if ((rc = ws_rhs(&w, x + h * T_C4, yt, k + 3 * N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * (T_A51 * k[i] + T_A52 * k[N + i] + T_A53 * k[2 * N + i] + T_A54 * k[3 * N + i]);
                if ((rc = ws_rhs(&w, x + h * T_C5, yt, k + 4 * N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yt[i] = y[i] + h * (T_A61 * k[i] + T_A62 * k[N + i] + T_A63 * k[2 * N + i] + T_A64 * k[3 * N + i] + T_A65 * k[4 * N + i]);
                if ((rc = ws_rhs(&w, x + h, yt, k + 5 * N, &e))) break;
                for (int64_t i = 0; i < N; ++i) yn[i] = y[i] + h * (T_A71 * k[i] + T_A72 * k[N + i] + T_A73 * k[2 * N + i] + T_A74 * k[3 * N + i] + T_A75 * k[4 * N + i] + T_A76 * k[5 * N + i]);
            }
            const double xn = x + h;
            if (ev_step && s == n_steps[t] - 1) {
                b.y = y;
                b.yn = yn;
                if ((rc = ws_rhs(&w, xn, yn, k + 6 * N, &e))) break;
                int has0, has1;
                double g0, g1, te;
                if ((rc = ws_event(&w, x, y, &has0, &g0, &e))) break;
                if ((rc = ws_event(&w, xn, yn, &has1, &g1, &e))) break;
                if (!has0 || !has1 || !crossed_zero(g0, g1)) { rc = fail(&e, "the replayed event step does not cross zero"); break; }
                if (g0 == 0.0) { te = x; yout = y; }
                else if (g1 == 0.0) { te = xn; yout = yn; }
                else {
                    if (!tsit) dopri_dense_prep(&b, h);
                    double lo = 0.0, hi = 1.0, glo = g0;
                    for (int it = 0; it < 60; ++it) {
                        double mid = 0.5 * (lo + hi);
                        if (!tsit) dopri_dense_out(&b, mid, b.ds); else tsit_dense_out(&b, mid, h, b.ds);
                        int has;
                        double gm;
                        if ((rc = ws_event(&w, x + mid * h, b.ds, &has, &gm, &e))) break;
                        if (!has) { rc = fail(&e, "event disappeared during root finding"); break; }
                        if (gm == 0.0) { lo = mid; hi = mid; break; }
                        if ((glo < 0.0 && gm > 0.0) || (glo > 0.0 && gm < 0.0)) hi = mid;
                        else { lo = mid; glo = gm; }
                    }
                    if (rc) break;
                    double theta = 0.5 * (lo + hi);
                    if (!tsit) dopri_dense_out(&b, theta, b.ds); else tsit_dense_out(&b, theta, h, b.ds);
                    te = x + theta * h;
                    yout = b.ds;
                }
                if (integral && !(have_last && fabs(last_t - te) <= time_tol(te))) {
                    double v = 0.0;
                    for (int32_t q = 0; q < opt->n_weights; ++q) v += opt->weight_value[q] * yout[opt->weight_index[q]];
                    if (have_last) integ += 0.5 * (last_v + v) * (te - last_t);
                }
                break;
            }
            if (integral) {
                double v = 0.0;
                for (int32_t q = 0; q < opt->n_weights; ++q) v += opt->weight_value[q] * yn[opt->weight_index[q]];
                if (have_last) integ += 0.5 * (last_v + v) * (xn - last_t);
                last_t = xn;
                last_v = v;
                have_last = 1;
            }
            double* tmp = y; y = yn; yn = tmp;
            b.y = y; b.yn = yn;
        }
        if (rc) break;
        if (!yout) yout = y;
        if (integral) values[t] = integ;
        else memcpy(values + t * n, yout, sizeof(double) * (size_t)n);
    }
    if (rc) copy_err(&e, err, err_len);
    rkb_free(&b);
    ws_free(&w);
    return rc;
}
