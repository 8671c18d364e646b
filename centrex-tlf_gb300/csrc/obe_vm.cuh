// obe_vm.cuh -- device expression VM for coefficient and parameter programs.
//
// Semantics follow rust/src/lindblad/eval.rs (opcodes :11-57, helpers :155-451 and :664-789,
// scalar evaluator :791-911).  Complex arithmetic is num-complex 0.4.6's published formulas
// (naive product/quotient, exp/sin/cos/tan from real functions) with one deliberate
// difference: a power whose exponent is a real integer |k| <= 64 is computed by repeated
// multiplication, as the reference's Python evaluator does (centrex_tlf/lindblad/ir.py:918-921,
// Python complex pow), so real operands give exactly real results.  num-complex's
// exp(y*ln x) form differs from it by rounding only (<= 1e-15 relative).
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>

#include "obe_internal.h"

namespace obe {

// A VM value: (re, im) in `v`, tuple id (>= 0, tuples are base-slot constants) in `tup`.
// The stack lives in memory the caller provides (shared memory in the integrator).
struct VStack {
    double2* v;
    int32_t* tup;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    double ns = b.x * b.x + b.y * b.y;
    double re = a.x * b.x + a.y * b.y;
    double im = a.y * b.x - a.x * b.y;
    return make_double2(re / ns, im / ns);
}
__device__ __forceinline__ double2 cexp(double2 z) {
    double re = z.x, im = z.y;
    if (isinf(re)) {
        if (re < 0.0) {
            if (!isfinite(im)) return make_double2(0.0, 0.0);
        } else if (im == 0.0 || !isfinite(im)) {
            if (isinf(im)) im = CUDART_NAN;
            return make_double2(re, im);
        }
    } else if (isnan(re) && im == 0.0) {
        return z;
    }
    double e = exp(re);
    if (im == 0.0) return make_double2(e, e * 0.0);
    double s, c;
    sincos(im, &s, &c);
    return make_double2(e * c, e * s);
}
__device__ __forceinline__ double2 cpow(double2 x, double2 y) {
    if (y.x == 0.0 && y.y == 0.0) return make_double2(1.0, 0.0);
    if (y.y == 0.0 && y.x == rint(y.x) && fabs(y.x) <= 64.0) {
        int k = static_cast<int>(fabs(y.x));
        double2 acc = make_double2(1.0, 0.0), b = x;
        bool first = true;
        while (k) {
            if (k & 1) {
                acc = first ? b : cmul(acc, b);
                first = false;
            }
            k >>= 1;
            if (k) b = cmul(b, b);
        }
        if (y.x < 0.0) {
            if (acc.y == 0.0) return make_double2(1.0 / acc.x, 0.0);
            return cdiv(make_double2(1.0, 0.0), acc);
        }
        return acc;
    }
    double2 ln = make_double2(log(hypot(x.x, x.y)), atan2(x.y, x.x));
    return cexp(cmul(y, ln));
}

__device__ __forceinline__ double rem_euclid(double a, double b) {
    double r = fmod(a, b);
    return r < 0.0 ? r + fabs(b) : r;
}

__device__ __forceinline__ double g2d(double x, double y, double a, double mx, double my, double sx, double sy) {
    double dx = x - mx, dy = y - my;
    return a * exp(-((dx * dx) / (2.0 * sx * sx) + (dy * dy) / (2.0 * sy * sy)));
}

__device__ __forceinline__ double rabi_from_intensity(double intensity, double coupling, double dipole) {
    const double hbar = 1.0545718176461565e-34, c = 299792458.0, eps0 = 8.8541878128e-12;
    return sqrt(intensity * 2.0 / (c * eps0)) * coupling * dipole / hbar;
}

constexpr double kPi = 3.14159265358979323846;
constexpr double kEdXtB = 0.315 * 1.602176634e-19 * 5.29177210544e-11;

static __device__ __noinline__ double2 helper_scalar(int fid, const double2* a, int argc) {
    auto S = [&](int i) { return i < argc ? a[i].x : 0.0; };
    switch (fid) {
    case 1: return make_double2(g2d(S(0), S(1), S(2), S(3), S(4), S(5), S(6)), 0.0);
    case 2: {
        double th = S(7), ct, st;
        sincos(th, &st, &ct);
        double sx = S(5), sy = S(6);
        double A = ct * ct / (2.0 * sx * sx) + st * st / (2.0 * sy * sy);
        double B = sin(2.0 * th) / (2.0 * sx * sx) - sin(2.0 * th) / (2.0 * sy * sy);
        double Cc = st * st / (2.0 * sx * sx) + ct * ct / (2.0 * sy * sy);
        double dx = S(0) - S(3), dy = S(1) - S(4);
        return make_double2(S(2) * exp(-(A * dx * dx + B * dx * dy + Cc * dy * dy)), 0.0);
    }
    case 3: {
        double phi = S(1) * sin(S(2) * S(0)), s, c;
        sincos(phi, &s, &c);
        return make_double2(c, s);
    }
    case 4: return make_double2(0.5 * (1.0 + (sin(S(1) * S(0) + S(2)) >= 0.0 ? 1.0 : -1.0)), 0.0);
    case 5: {
        double theta = 0.5 * S(1) * sin(S(2) * S(0));
        double v = 0.5 * (cos(theta) + sin(theta));
        return make_double2(v, v);
    }
    case 6: return make_double2(rem_euclid((S(1) * S(0) + S(2)) / (2.0 * kPi), 1.0), 0.0);
    case 7: {
        double period = S(1) + S(2), duty = S(1) / period;
        double frac = rem_euclid(2.0 * kPi * S(0) / period + S(3), 2.0 * kPi) / (2.0 * kPi);
        return make_double2(frac < duty ? 1.0 : 0.0, 0.0);
    }
    case 9: return make_double2(rabi_from_intensity(S(0), S(1), argc > 2 ? S(2) : kEdXtB), 0.0);
    case 11: {
        double inten = g2d(S(0), S(1), S(2), S(3), S(4), S(5), S(6));
        return make_double2(rabi_from_intensity(inten, S(7), argc > 8 ? S(8) : kEdXtB), 0.0);
    }
    case 12: {
        double frac = rem_euclid(S(0) * S(2) + S(3) / (2.0 * kPi), 1.0);
        if (frac <= 0.0) frac += 1.0;
        return make_double2(frac < S(1) ? 1.0 : 0.0, 0.0);
    }
    case 13: {
        double q = floor((S(0) - S(1)) / S(2));
        long long nq = isnan(q) ? 0 : (q >= 9.2e18 ? 9223372036854775807LL : (q <= -9.2e18 ? (-9223372036854775807LL - 1) : static_cast<long long>(q)));
        return make_double2(nq % 2 == 0 ? 1.0 : -1.0, 0.0);
    }
    case 15: {
        double dx = S(0) - S(1);
        return make_double2(exp(-dx * dx / (2.0 * S(2) * S(2))), 0.0);
    }
    default: return make_double2(0.0, 0.0);
    }
}

// PCHIP derivative d[i] of the direct form (eval.rs:322-333), computed locally.
static __device__ double pchip_d(const double2* g, const double2* v, int n, int i) {
    auto h = [&](int k) { return g[k + 1].x - g[k].x; };
    auto delta = [&](int k) { return (v[k + 1].x - v[k].x) / h(k); };
    if (i == 0) return delta(0);
    if (i == n - 1) return delta(n - 2);
    double d0 = delta(i - 1), d1 = delta(i);
    if (signbit(d0) != signbit(d1) || d0 == 0.0 || d1 == 0.0) return 0.0;
    double w1 = 2.0 * h(i) + h(i - 1), w2 = h(i) + 2.0 * h(i - 1);
    return (w1 + w2) / (w1 / d0 + w2 / d1);
}

__device__ __forceinline__ const double2* tuple_items(const DevPlan& P, int32_t id, int* len) {
    *len = P.tuple_ptr[id + 1] - P.tuple_ptr[id];
    return reinterpret_cast<const double2*>(P.tuple_items) + P.tuple_ptr[id];
}

static __device__ __noinline__ double2 helper_general(const DevPlan& P, int fid, const double2* a, const int32_t* tup, int argc) {
    if (fid == 8 || fid == 10) {
        int la, lx, ly;
        const double2* amp = tuple_items(P, tup[2], &la);
        const double2* xl = tuple_items(P, tup[3], &lx);
        const double2* yl = tuple_items(P, tup[4], &ly);
        double acc = 0.0;
        int m = min(la, min(lx, ly));
        for (int i = 0; i < m; ++i) acc += g2d(a[0].x, a[1].x, amp[i].x, xl[i].x, yl[i].x, a[5].x, a[6].x);
        if (fid == 8) return make_double2(acc, 0.0);
        return make_double2(rabi_from_intensity(acc, a[7].x, argc > 8 ? a[8].x : kEdXtB), 0.0);
    }
    if (fid == 14) {
        int lg, lv;
        const double2* g = tuple_items(P, tup[1], &lg);
        const double2* v = tuple_items(P, tup[2], &lv);
        double x = a[0].x;
        if (lg == 1) return make_double2(v[0].x, 0.0);
        if (x <= g[0].x) return make_double2(v[0].x, 0.0);
        for (int i = 0; i < lg - 1; ++i) {
            double left = g[i].x, right = g[i + 1].x;
            if (x <= right) {
                double frac = (x - left) / (right - left);
                return make_double2(v[i].x + frac * (v[i + 1].x - v[i].x), 0.0);
            }
        }
        return make_double2(v[lg - 1].x, 0.0);
    }
    if (fid == 16) {  // direct PCHIP (eval.rs:305-351)
        int n, lv;
        const double2* g = tuple_items(P, tup[1], &n);
        const double2* v = tuple_items(P, tup[2], &lv);
        double x = a[0].x;
        if (n == 1) return make_double2(v[0].x, 0.0);
        if (x <= g[0].x) return make_double2(v[0].x, 0.0);
        if (x >= g[n - 1].x) return make_double2(v[n - 1].x, 0.0);
        int idx = 0;
        for (int i = 0; i < n - 1; ++i)
            if (x < g[i + 1].x || i == n - 2) { idx = i; break; }
        double hh = g[idx + 1].x - g[idx].x;
        double t = (x - g[idx].x) / hh, t2 = t * t, t3 = t2 * t;
        double h00 = 2.0 * t3 - 3.0 * t2 + 1.0, h10 = t3 - 2.0 * t2 + t, h01 = -2.0 * t3 + 3.0 * t2, h11 = t3 - t2;
        return make_double2(h00 * v[idx].x + h10 * hh * pchip_d(g, v, n, idx) + h01 * v[idx + 1].x + h11 * hh * pchip_d(g, v, n, idx + 1), 0.0);
    }
    return helper_scalar(fid, a, argc);
}

// PchipTable::evaluate (plan.rs:82-115) without the search hint.
static __device__ __noinline__ double pchip_table_eval(const DevPlan& P, int table, double x) {
    int a = P.pchip_ptr[table], n = P.pchip_ptr[table + 1] - a;
    const double* g = P.pchip_grid + a;
    const double* coef = P.pchip_coef + P.pchip_cptr[table];
    if (x <= g[0]) return coef[0];
    if (x >= g[n - 1]) {
        int last = n - 2;
        double dx = g[n - 1] - g[last];
        const double* c = coef + 4 * last;
        return c[0] + dx * (c[1] + dx * (c[2] + dx * c[3]));
    }
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (g[mid] <= x) lo = mid + 1; else hi = mid;
    }
    int i = lo > 0 ? lo - 1 : 0;
    if (i > n - 2) i = n - 2;
    double dx = x - g[i];
    const double* c = coef + 4 * i;
    return c[0] + dx * (c[1] + dx * (c[2] + dx * c[3]));
}

// Evaluate one program.  Programs were kind-checked on the host, so tuples only reach the
// helpers that accept them and the result is a scalar.
static __device__ __noinline__ double2 vm_eval(const DevPlan& P, const int32_t* op, const int32_t* arg, const int32_t* fn,
                                        const double* val, int32_t start, int32_t len, const double2* slots, double t,
                                        VStack S) {
    double2* st = S.v;
    int32_t* tp = S.tup;
    int sp = 0;
    for (int32_t k = start; k < start + len; ++k) {
        int32_t o = op[k];
        switch (o) {
        case OP_CONST: st[sp] = make_double2(val[2 * k], val[2 * k + 1]); tp[sp++] = -1; break;
        case OP_SLOT: {
            int32_t s = arg[k];
            int32_t tid = s < P.n_base ? P.base_tuple[s] : -1;
            st[sp] = tid >= 0 ? make_double2(0.0, 0.0) : slots[s];
            tp[sp++] = tid;
            break;
        }
        case OP_TIME: st[sp] = make_double2(t, 0.0); tp[sp++] = -1; break;
        case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_POW: {
            double2 b = st[--sp], a = st[sp - 1], c;
            if (o == OP_ADD) c = make_double2(a.x + b.x, a.y + b.y);
            else if (o == OP_SUB) c = make_double2(a.x - b.x, a.y - b.y);
            else if (o == OP_MUL) c = cmul(a, b);
            else if (o == OP_DIV) c = cdiv(a, b);
            else c = cpow(a, b);
            st[sp - 1] = c;
            tp[sp - 1] = -1;
            break;
        }
        case OP_NEG: st[sp - 1] = make_double2(-st[sp - 1].x, -st[sp - 1].y); break;
        case OP_CONJ: st[sp - 1].y = -st[sp - 1].y; break;
        case OP_BUILTIN: {
            int argc = arg[k];
            double2 z = st[sp - argc], r;
            sp -= argc;
            switch (fn[k]) {
            case 1:
            case 2: {
                double sn, cs;
                sincos(z.x, &sn, &cs);
                double ch = z.y == 0.0 ? 1.0 : cosh(z.y), sh = z.y == 0.0 ? z.y : sinh(z.y);
                r = fn[k] == 1 ? make_double2(sn * ch, cs * sh) : make_double2(cs * ch, -sn * sh);
                break;
            }
            case 3: {
                double tr = z.x + z.x, ti = z.y + z.y, dd = cos(tr) + cosh(ti);
                r = make_double2(sin(tr) / dd, sinh(ti) / dd);
                break;
            }
            case 4: r = cexp(z); break;
            case 5: r = make_double2(hypot(z.x, z.y), 0.0); break;
            case 6: r = make_double2(z.x, 0.0); break;
            default: r = make_double2(z.y, 0.0); break;
            }
            st[sp] = r;
            tp[sp++] = -1;
            break;
        }
        case OP_HELPER: {
            int argc = arg[k];
            sp -= argc;
            double2 r = helper_general(P, fn[k], st + sp, tp + sp, argc);
            st[sp] = r;
            tp[sp++] = -1;
            break;
        }
        case OP_PCHIP_TABLE: {
            sp -= 3;
            double x = st[sp].x;
            st[sp] = make_double2(pchip_table_eval(P, fn[k], x), 0.0);
            tp[sp++] = -1;
            break;
        }
        default: {  // comparisons
            double r = st[sp - 1].x, l = st[sp - 2].x;
            sp -= 2;
            bool res = o == OP_GT ? l > r : o == OP_GE ? l >= r : o == OP_LT ? l < r : o == OP_LE ? l <= r : o == OP_EQ ? l == r : l != r;
            st[sp] = make_double2(res ? 1.0 : 0.0, 0.0);
            tp[sp++] = -1;
            break;
        }
        }
    }
    return st[0];
}

// The same programs on real values only, for expressions marked real_ok (obe_plan.cpp:
// expr_real_closed) when every slot of the trajectory is real.  Each case computes exactly what
// the complex case above yields for operands with zero imaginary parts -- the quotient as
// (a b) / (b b), tan(z) as sin(2z) / (cos(2z) + 1), integer powers by the same repeated
// multiplication -- so the two paths agree bit for bit while the real one issues a fraction of
// the double-precision instructions.  The stack is the caller's VM stack storage.
static __device__ __forceinline__ double vm_eval_real_inl(const DevPlan& P, const int32_t* op, const int32_t* arg,
                                                          const int32_t* fn, const double* val, int32_t start, int32_t len,
                                                          const double2* slots, double t, double* st) {
    int sp = 0;
    for (int32_t k = start; k < start + len; ++k) {
        const int32_t o = op[k];
        switch (o) {
        case OP_CONST: st[sp++] = val[2 * k]; break;
        case OP_SLOT: st[sp++] = slots[arg[k]].x; break;
        case OP_TIME: st[sp++] = t; break;
        case OP_ADD: { double b = st[--sp]; st[sp - 1] = st[sp - 1] + b; break; }
        case OP_SUB: { double b = st[--sp]; st[sp - 1] = st[sp - 1] - b; break; }
        case OP_MUL: { double b = st[--sp]; st[sp - 1] = st[sp - 1] * b; break; }
        case OP_DIV: { double b = st[--sp], a = st[sp - 1]; st[sp - 1] = (a * b) / (b * b); break; }
        case OP_POW: {
            const double y = st[--sp], x = st[sp - 1];
            double r;
            if (y == 0.0) {
                r = 1.0;
            } else {
                int kk = static_cast<int>(fabs(y));
                double acc = 1.0, b = x;
                bool first = true;
                while (kk) {
                    if (kk & 1) {
                        acc = first ? b : acc * b;
                        first = false;
                    }
                    kk >>= 1;
                    if (kk) b = b * b;
                }
                r = y < 0.0 ? 1.0 / acc : acc;
            }
            st[sp - 1] = r;
            break;
        }
        case OP_NEG: st[sp - 1] = -st[sp - 1]; break;
        case OP_CONJ: break;
        case OP_BUILTIN: {
            const double z = st[sp - 1];
            double r;
            switch (fn[k]) {
            case 1:
            case 2: {
                double sn, cs;
                sincos(z, &sn, &cs);  // as the complex case computes them
                r = fn[k] == 1 ? sn : cs;
                break;
            }
            case 3: { double tr = z + z; r = sin(tr) / (cos(tr) + 1.0); break; }
            case 4: r = exp(z); break;
            case 5: r = hypot(z, 0.0); break;
            case 6: r = z; break;
            default: r = 0.0; break;
            }
            st[sp - 1] = r;
            break;
        }
        default: {  // comparisons
            const double r = st[sp - 1], l = st[sp - 2];
            sp -= 2;
            const bool res = o == OP_GT ? l > r : o == OP_GE ? l >= r : o == OP_LT ? l < r : o == OP_LE ? l <= r : o == OP_EQ ? l == r : l != r;
            st[sp++] = res ? 1.0 : 0.0;
            break;
        }
        }
    }
    return st[0];
}

// the same as a call (the integrator's per-step coefficient rows inline it into their own call)
static __device__ __noinline__ double vm_eval_real(const DevPlan& P, const int32_t* op, const int32_t* arg, const int32_t* fn,
                                            const double* val, int32_t start, int32_t len, const double2* slots, double t,
                                            double* st) {
    return vm_eval_real_inl(P, op, arg, fn, val, start, len, slots, t, st);
}

}  // namespace obe
