// obe_adjoint.cuh -- discrete adjoint of the adaptive solve, double precision or the mixed form
// (gradients of the final populations or of a weighted time integral with respect to base
// parameters and to the initial state, through stop events).  No counterpart in the reference,
// whose Rust crate has no gradient path.
//
// The forward solve (integrate_kernel with a tape) records, for every accepted step n, its start
// time t_n, size h_n, start state y_n and the stage derivatives K_1..K_6.  With the step sequence
// frozen, one step of Dopri5/Tsit5 is the explicit six-stage map
//     Y_s = y_n + h sum_{l<s} a_sl K_l,   K_s = L(t_n + c_s h; p) Y_s,   y_{n+1} = y_n + h sum_s b_s K_s
// (the seventh, first-same-as-last stage only feeds the error estimate), and its reverse sweep is
//     lambda_s = h b_s ybar' + h sum_{m>s} a_ms mu_m,    mu_s = L(t_s)^T lambda_s,
//     ybar = ybar' + sum_s mu_s,                          pbar += sum_s lambda_s^T (dL/dp)(t_s) Y_s.
// L(t) = sum_f formula_f(c(t)) E_f, with each formula a sum of factor x coefficient-class
// products, so lambda^T (dL/dp) Y = sum_class Re(dc_class/dp * S_class) where S_class sums
// factor * Y_in' * conj(lambda_out) over the records and products of that class.  The
// coefficient derivatives dc/dp come from forward-mode (dual) evaluation of the parameter and
// coefficient programs.  The trapezoid rule of the integral outputs (sum over accepted steps of
// (t_{n+1} - t_n)(w.y_n + w.y_{n+1}) / 2) adds its weights to ybar at both ends of each segment.
//
// A step that a stop event ends maps y_n to the dense output at the event time (a seven-stage map
// with the interpolant's weights), and the event time's own dependence enters through the event
// function's derivatives (dense_weights and the event seed below).  The mixed form sweeps its
// single-precision tape with single-precision products and double-precision accumulation.
//
// One group of 32, 64, 128 or 256 threads per trajectory (the plan's width; above 45 states the
// stage-derivative adjoints and ybar move to a per-group slice of device memory, and the class
// sums too when shared memory cannot hold them, and the record streams are read from the plan's
// device image); the transposed product L^T lambda runs on a second, input-major record stream
// built by the packer.
#pragma once

#include "obe_kernels.cuh"

namespace obe {

constexpr int kMaxGrad = 8;

// per-trajectory adjoint status codes
enum AdjCode : int32_t { ADJ_OK = 0, ADJ_HELPER_DERIVATIVE = 1, ADJ_FORWARD_FAILED = 2, ADJ_EVENT_TANGENT = 3 };

struct AdjArgs {
    int n_grad;
    int grad_slot[kMaxGrad];    // base slots the gradient is taken with respect to
    const double* tape;
    long long tape_cap, tape_stride;
    // checkpointed tape (ckpt = C > 0, the integrator's tape_ckpt layout): each segment of C steps
    // is replayed from its start state into the group's segment buffer (seg + group * seg_stride:
    // C records of [t_n, h_n, y_n, K_1..K_6], rec_stride doubles apart) before its reverse sweep
    int ckpt;
    double* seg;
    long long seg_stride, rec_stride;
    // large systems (256 threads per trajectory): each group's mu, ybar and class sums live in a
    // slice of device memory, gscratch + group * gstride bytes
    unsigned char* gscratch;
    size_t gstride;
    const obe_traj_stats* fwd_stats;  // the forward solve's statistics (accepted-step counts)
    const double* out_grad;     // [traj][width]: d(loss)/d(output)
    double* param_grad;         // [traj][n_grad]
    double* rho0_grad;          // [traj][N] or null
    int32_t* adj_status;        // [traj]
    unsigned long long* counter;
};

// ------------------------------------------------------------------------------------------
// forward-mode evaluation: value and derivatives with respect to the n_grad parameters

// One program (instruction arrays op/arg/fn/val, entries start..start+len) in dual numbers.
// slots / dslots: values and derivatives ([slot * n_grad + g]) of the parameter slots; the stack
// holds values in sv, derivatives in sd ([depth * kMaxGrad]) and tuple ids in tp.  Returns the
// value and writes the derivatives to out_d[0..n_grad).  tseed >= 0 seeds d(time)/d(variable
// tseed) = 1 (the time derivative of the program).  A helper or table whose arguments carry a
// derivative sets *bad (its derivative is not implemented).
static __device__ __noinline__ double2 vm_eval_dual_prog(const DevPlan& P, const int32_t* op, const int32_t* arg,
                                                         const int32_t* fn, const double* val, int32_t start, int32_t len,
                                                         const double2* slots, const double2* dslots, int ng, double t,
                                                         double2* sv, double2* sd, int32_t* tp, double2* out_d, int* bad,
                                                         int tseed) {
    int sp = 0;
    auto D = [&](int i, int g) -> double2& { return sd[i * kMaxGrad + g]; };
    for (int32_t k = start; k < start + len; ++k) {
        const int32_t o = op[k];
        switch (o) {
        case OP_CONST:
            sv[sp] = make_double2(val[2 * k], val[2 * k + 1]);
            for (int g = 0; g < ng; ++g) D(sp, g) = make_double2(0.0, 0.0);
            tp[sp++] = -1;
            break;
        case OP_SLOT: {
            const int32_t s = arg[k];
            const int32_t tid = s < P.n_base ? P.base_tuple[s] : -1;
            sv[sp] = tid >= 0 ? make_double2(0.0, 0.0) : slots[s];
            for (int g = 0; g < ng; ++g) D(sp, g) = tid >= 0 ? make_double2(0.0, 0.0) : dslots[s * ng + g];
            tp[sp++] = tid;
            break;
        }
        case OP_TIME:
            sv[sp] = make_double2(t, 0.0);
            for (int g = 0; g < ng; ++g) D(sp, g) = make_double2(g == tseed ? 1.0 : 0.0, 0.0);
            tp[sp++] = -1;
            break;
        case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_POW: {
            const int ib = --sp, ia = sp - 1;
            const double2 a = sv[ia], b = sv[ib];
            double2 c;
            if (o == OP_ADD || o == OP_SUB) {
                const double sg = o == OP_ADD ? 1.0 : -1.0;
                c = make_double2(a.x + sg * b.x, a.y + sg * b.y);
                for (int g = 0; g < ng; ++g) D(ia, g) = make_double2(D(ia, g).x + sg * D(ib, g).x, D(ia, g).y + sg * D(ib, g).y);
            } else if (o == OP_MUL) {
                c = cmul(a, b);
                for (int g = 0; g < ng; ++g) {
                    const double2 x = cmul(D(ia, g), b), y = cmul(a, D(ib, g));
                    D(ia, g) = make_double2(x.x + y.x, x.y + y.y);
                }
            } else if (o == OP_DIV) {
                c = cdiv(a, b);
                // (a'/b) - (a b'/b^2) = (a' - c b') / b
                for (int g = 0; g < ng; ++g) {
                    const double2 cb = cmul(c, D(ib, g));
                    D(ia, g) = cdiv(make_double2(D(ia, g).x - cb.x, D(ia, g).y - cb.y), b);
                }
            } else {
                c = cpow(a, b);
                // integer exponent: k a^(k-1) a'; otherwise a^b (b' ln a + b a'/a)
                const bool int_exp = b.y == 0.0 && b.x == rint(b.x) && fabs(b.x) <= 64.0;
                double2 f1 = make_double2(0.0, 0.0), lna = make_double2(0.0, 0.0);
                if (int_exp) {
                    if (b.x != 0.0) f1 = cmul(make_double2(b.x, 0.0), cpow(a, make_double2(b.x - 1.0, 0.0)));
                } else {
                    lna = make_double2(log(hypot(a.x, a.y)), atan2(a.y, a.x));
                    f1 = cmul(c, cdiv(b, a));
                }
                for (int g = 0; g < ng; ++g) {
                    double2 dv = cmul(f1, D(ia, g));
                    if (!int_exp) {
                        const double2 t2 = cmul(c, cmul(D(ib, g), lna));
                        dv = make_double2(dv.x + t2.x, dv.y + t2.y);
                    } else if (D(ib, g).x != 0.0 || D(ib, g).y != 0.0) {
                        *bad = 1;
                    }
                    D(ia, g) = dv;
                }
            }
            sv[ia] = c;
            tp[ia] = -1;
            break;
        }
        case OP_NEG:
            sv[sp - 1] = make_double2(-sv[sp - 1].x, -sv[sp - 1].y);
            for (int g = 0; g < ng; ++g) D(sp - 1, g) = make_double2(-D(sp - 1, g).x, -D(sp - 1, g).y);
            break;
        case OP_CONJ:
            sv[sp - 1].y = -sv[sp - 1].y;
            for (int g = 0; g < ng; ++g) D(sp - 1, g).y = -D(sp - 1, g).y;  // the parameters are real
            break;
        case OP_BUILTIN: {
            const int argc = arg[k];
            const int iz = sp - argc;
            const double2 z = sv[iz];
            double2 r = make_double2(0.0, 0.0), dr = make_double2(0.0, 0.0);  // value and d(value)/dz
            switch (fn[k]) {
            case 1: {
                double sn, cs;
                sincos(z.x, &sn, &cs);
                const double ch = z.y == 0.0 ? 1.0 : cosh(z.y), sh = z.y == 0.0 ? z.y : sinh(z.y);
                r = make_double2(sn * ch, cs * sh);
                dr = make_double2(cs * ch, -sn * sh);  // cos z
                break;
            }
            case 2: {
                double sn, cs;
                sincos(z.x, &sn, &cs);
                const double ch = z.y == 0.0 ? 1.0 : cosh(z.y), sh = z.y == 0.0 ? z.y : sinh(z.y);
                r = make_double2(cs * ch, -sn * sh);
                dr = make_double2(-sn * ch, -cs * sh);  // -sin z
                break;
            }
            case 3: {
                const double tr = z.x + z.x, ti = z.y + z.y, dd = cos(tr) + cosh(ti);
                r = make_double2(sin(tr) / dd, sinh(ti) / dd);
                const double2 r2 = cmul(r, r);
                dr = make_double2(1.0 + r2.x, r2.y);  // 1 + tan^2 z
                break;
            }
            case 4: r = cexp(z); dr = r; break;
            case 5: r = make_double2(hypot(z.x, z.y), 0.0); break;
            case 6: r = make_double2(z.x, 0.0); break;
            default: r = make_double2(z.y, 0.0); break;
            }
            for (int g = 0; g < ng; ++g) {
                const double2 dz = D(iz, g);
                double2 dv;
                if (fn[k] <= 4) {
                    dv = cmul(dr, dz);
                } else if (fn[k] == 5) {  // |z|' = Re(conj(z) z') / |z|
                    const double m = hypot(z.x, z.y);
                    dv = make_double2(m > 0.0 ? (z.x * dz.x + z.y * dz.y) / m : 0.0, 0.0);
                } else if (fn[k] == 6) {
                    dv = make_double2(dz.x, 0.0);
                } else {
                    dv = make_double2(dz.y, 0.0);
                }
                D(iz, g) = dv;
            }
            sp = iz;
            sv[sp] = r;
            tp[sp++] = -1;
            break;
        }
        case OP_HELPER:
        case OP_PCHIP_TABLE: {
            const int argc = o == OP_PCHIP_TABLE ? 3 : arg[k];
            sp -= argc;
            for (int a = 0; a < argc; ++a)
                for (int g = 0; g < ng; ++g)
                    if (D(sp + a, g).x != 0.0 || D(sp + a, g).y != 0.0) *bad = 1;
            double2 r;
            if (o == OP_HELPER) r = helper_general(P, fn[k], sv + sp, tp + sp, argc);
            else r = make_double2(pchip_table_eval(P, fn[k], sv[sp].x), 0.0);
            sv[sp] = r;
            for (int g = 0; g < ng; ++g) D(sp, g) = make_double2(0.0, 0.0);
            tp[sp++] = -1;
            break;
        }
        default: {  // comparisons: piecewise constant
            const double r = sv[sp - 1].x, l = sv[sp - 2].x;
            sp -= 2;
            const bool res = o == OP_GT ? l > r : o == OP_GE ? l >= r : o == OP_LT ? l < r : o == OP_LE ? l <= r : o == OP_EQ ? l == r : l != r;
            sv[sp] = make_double2(res ? 1.0 : 0.0, 0.0);
            for (int g = 0; g < ng; ++g) D(sp, g) = make_double2(0.0, 0.0);
            tp[sp++] = -1;
            break;
        }
        }
    }
    for (int g = 0; g < ng; ++g) out_d[g] = D(0, g);
    return sv[0];
}

// a program of the plan's expression pool, derivatives with respect to the parameters
static __device__ __forceinline__ double2 vm_eval_dual(const DevPlan& P, int32_t start, int32_t len, const double2* slots,
                                                       const double2* dslots, int ng, double t, double2* sv, double2* sd,
                                                       int32_t* tp, double2* out_d, int* bad) {
    return vm_eval_dual_prog(P, P.ins_op, P.ins_arg, P.ins_fn, P.ins_val, start, len, slots, dslots, ng, t, sv, sd, tp, out_d,
                             bad, -1);
}

// ------------------------------------------------------------------------------------------
// shared-memory layout of one adjoint trajectory group (tpt threads)

struct AdjLayout {
    size_t tab, G, LS, MU, YB, slots, dslots, dts, sv, sd, tp, cstat, dcstat, cdyn, ddyn, dcls, S, red, traj, bytes;
    size_t tab32, YB32, dcls32;  // the mixed sweep's single-precision formula table, ybar copy, class derivatives
    size_t T4, cv;               // the mixed replay's deviation-form formula table and stage class values
    size_t gbytes;  // large systems: bytes of the group's device-memory slice (MU, YB, S)
    bool glob;
    bool s_shared;  // the class sums S in shared memory (always below 256 threads; above, when they fit)
};

// stages: 6, or 7 when a stop event can end the solve (the event step's dense output reads the
// first-same-as-last stage too)
__host__ __device__ inline AdjLayout adj_layout(int n, int N, int n_formula, int n_coeff, int n_dyn, int n_slots, int vm_depth,
                                                int tpt, int stages) {
    const size_t U = static_cast<size_t>(n) * (n + 1) / 2;
    const size_t nc = n_coeff > 0 ? n_coeff : 1, nd = n_dyn > 0 ? n_dyn : 1, ns = n_slots > 0 ? n_slots : 1;
    AdjLayout L{};
    L.glob = tpt >= 256;
    size_t o = 0, og = 0;
    size_t& om = L.glob ? og : o;  // cursor of the buffers that move to device memory
    L.tab = o; o = align16(o + (1 + n_formula) * 16);
    L.tab32 = o; o = align16(o + (1 + n_formula) * 8);
    L.G = o; o = align16(o + U * 16);
    L.LS = o; o = align16(o + U * 16);
    L.MU = om; om = align16(om + static_cast<size_t>(stages) * N * 8);
    L.YB = om; om = align16(om + static_cast<size_t>(N) * 8);
    L.YB32 = om; om = align16(om + static_cast<size_t>(N) * 4);
    L.T4 = om; om = align16(om + static_cast<size_t>(1 + n_formula) * 16);
    L.slots = o; o = align16(o + 6 * ns * 16);
    L.dslots = o; o = align16(o + 6 * ns * kMaxGrad * 16);
    L.dts = o; o = align16(o + ns * 16);
    L.sv = o; o = align16(o + 6 * static_cast<size_t>(vm_depth) * 16);
    L.sd = o; o = align16(o + 6 * static_cast<size_t>(vm_depth) * kMaxGrad * 16);
    L.tp = o; o = align16(o + 6 * static_cast<size_t>(vm_depth) * 4);
    L.cstat = o; o = align16(o + nc * 16);
    L.dcstat = o; o = align16(o + nc * kMaxGrad * 16);
    L.cdyn = o; o = align16(o + 6 * nd * 16);
    L.ddyn = o; o = align16(o + 6 * nd * kMaxGrad * 16);
    L.dcls = o; o = align16(o + 6 * 2 * nc * kMaxGrad * 16);
    L.dcls32 = o; o = align16(o + 6 * 2 * nc * kMaxGrad * 8);
    L.cv = o; o = align16(o + 5 * 2 * nc * 16);
    L.red = o; o = align16(o + (tpt / 32 + 4) * 8);
    L.traj = o; o = align16(o + 16);
    // the class sums take read-modify-writes at every formula end: shared memory whenever they fit
    // (large systems: within a 200 KB group, one group per CTA)
    const size_t s_bytes = align16(2 * nc * static_cast<size_t>(tpt) * 16);
    L.s_shared = !L.glob || o + s_bytes <= 200 * 1024;
    if (L.s_shared) {
        L.S = o;
        o += s_bytes;
    } else {
        L.S = og;
        og += s_bytes;
    }
    L.bytes = o;
    L.gbytes = og;
    return L;
}

// the record streams staged per CTA (large systems read them from the plan's device image)
__host__ __device__ inline size_t adj_plan_smem_bytes(const DevPlan& P, int tpt) {
    return tpt >= 256 ? 0 : align16(static_cast<size_t>(P.n_biter + P.n_titer + P.n_tin) * tpt * 4);
}

// The dense output of a step as stage weights: y(theta) = y_n + h sum_{j<7} w_j(theta) K_j, and
// dw_j = d w_j / d theta.  Dopri5 (M = 0, dopri5.rs:104-143): theta dd + theta(1-theta) bb +
// theta^2 (1-theta) r3 + theta^2 (1-theta)^2 r4 with dd = h sum b_j K_j, bb = h K_1 - dd,
// r3 = -h K_7 + dd - bb, r4 = h sum d_j K_j.  Tsit5 (M = 1, tsit5.rs:121-143): the interpolant's
// quartic polynomials.  b: the solution weights (b_7 = 0).
__device__ __forceinline__ void dense_weights(int M, double th, const double* b, double* w, double* dw) {
    if (M == 0) {
        const double t1 = 1.0 - th;
        const double p1 = th, p2 = th * t1, p3 = th * th * t1, p4 = th * th * t1 * t1;
        const double q1 = 1.0, q2 = 1.0 - 2.0 * th, q3 = th * (2.0 - 3.0 * th), q4 = 2.0 * th * t1 * (1.0 - 2.0 * th);
#pragma unroll
        for (int j = 0; j < 7; ++j) {
            const double bj = j < 6 ? b[j] : 0.0;
            const double e0 = j == 0 ? 1.0 : 0.0, e6 = j == 6 ? 1.0 : 0.0;
            const double dj = j == 1 ? 0.0 : kTab.dd[j];
            const double c2 = e0 - bj, c3 = 2.0 * bj - e0 - e6;
            w[j] = p1 * bj + p2 * c2 + p3 * c3 + p4 * dj;
            dw[j] = q1 * bj + q2 * c2 + q3 * c3 + q4 * dj;
        }
    } else {
        const double t2 = th * th, t3 = t2 * th, t4 = t3 * th;
#pragma unroll
        for (int j = 0; j < 7; ++j) {
            w[j] = kTab.r[j][0] * th + kTab.r[j][1] * t2 + kTab.r[j][2] * t3 + kTab.r[j][3] * t4;
            dw[j] = kTab.r[j][0] + 2.0 * kTab.r[j][1] * th + 3.0 * kTab.r[j][2] * t2 + 4.0 * kTab.r[j][3] * t3;
        }
    }
}

// ------------------------------------------------------------------------------------------
// the reverse sweep

// MIXED: the sweep of the mixed form's tape (single-precision records [y_n, k_1, d_2..d_7], the
// stage derivatives K_s = k_1 + d_s): stage inputs, adjoints lambda_s and mu_s, the transposed and
// bilinear products in single precision; ybar and the parameter gradient accumulate in double
// (each step's mu sum and class sums are added to them once, exactly converted).
template <int TPT, int EPT, bool MIXED>
__global__ void __launch_bounds__(256, 1) adjoint_kernel(const DevPlan P, const CallArgs A, const AdjArgs J, int gpb,
                                                         size_t group_bytes, int M) {
    static_assert(TPT >= 32 && TPT <= 256, "the adjoint runs 32, 64, 128 or 256 threads per trajectory");
    extern __shared__ __align__(16) unsigned char smem[];
    const int g = static_cast<int>(threadIdx.x) / TPT;
    const int lt = static_cast<int>(threadIdx.x) % TPT;
    const int n = P.n, N = P.N, U = P.U;
    const uint32_t* s_bil = P.bil;
    const uint32_t* s_trec = P.trec;
    const uint32_t* s_lin = P.lane_in;
    if constexpr (TPT < 256) {
        uint32_t* b = reinterpret_cast<uint32_t*>(smem);
        uint32_t* tr = b + static_cast<size_t>(P.n_biter) * TPT;
        uint32_t* li = tr + static_cast<size_t>(P.n_titer) * TPT;
        for (int i = threadIdx.x; i < P.n_biter * TPT; i += blockDim.x) b[i] = P.bil[i];
        for (int i = threadIdx.x; i < P.n_titer * TPT; i += blockDim.x) tr[i] = P.trec[i];
        for (int i = threadIdx.x; i < P.n_tin * TPT; i += blockDim.x) li[i] = P.lane_in[i];
        s_bil = b;
        s_trec = tr;
        s_lin = li;
    }
    __syncthreads();
    if (g >= gpb) return;

    const int n_stage_max = A.ev_kind != OBE_EVENT_NONE ? 7 : 6;
    const AdjLayout Lay = adj_layout(n, N, P.n_formula, P.n_coeff, P.n_dyn, P.n_slots, A.vm_depth, TPT, n_stage_max);
    unsigned char* gb = smem + adj_plan_smem_bytes(P, TPT) + static_cast<size_t>(g) * group_bytes;
    unsigned char* gm = Lay.glob ? J.gscratch + (static_cast<size_t>(blockIdx.x) * gpb + g) * J.gstride : gb;
    double2* s_tab = reinterpret_cast<double2*>(gb + Lay.tab);
    double2* s_G = reinterpret_cast<double2*>(gb + Lay.G);
    double* s_G64 = reinterpret_cast<double*>(gb + Lay.G);
    double2* s_LS = reinterpret_cast<double2*>(gb + Lay.LS);
    double* s_LS64 = reinterpret_cast<double*>(gb + Lay.LS);
    double* s_MU = reinterpret_cast<double*>(gm + Lay.MU);
    double* s_YB = reinterpret_cast<double*>(gm + Lay.YB);
    double2* s_cstat = reinterpret_cast<double2*>(gb + Lay.cstat);
    double2* s_dcstat = reinterpret_cast<double2*>(gb + Lay.dcstat);
    double2* s_cdyn = reinterpret_cast<double2*>(gb + Lay.cdyn);
    double2* s_ddyn = reinterpret_cast<double2*>(gb + Lay.ddyn);
    double2* s_dcls = reinterpret_cast<double2*>(gb + Lay.dcls);
    double2* s_S = reinterpret_cast<double2*>((Lay.s_shared ? gb : gm) + Lay.S);
    double* s_red = reinterpret_cast<double*>(gb + Lay.red);
    long long* s_traj = reinterpret_cast<long long*>(gb + Lay.traj);
    const int ns = P.n_slots > 0 ? P.n_slots : 1;
    const int nd = P.n_dyn > 0 ? P.n_dyn : 1;
    const int nc2 = 2 * P.n_coeff;
    const int ng = J.n_grad;
    const int S = P.n_static_formula, F = P.n_formula;
    const int vl = lt < 6 ? lt : 0;
    double2* slots = reinterpret_cast<double2*>(gb + Lay.slots) + vl * ns;
    double2* dslots = reinterpret_cast<double2*>(gb + Lay.dslots) + static_cast<size_t>(vl) * ns * kMaxGrad;
    double2* sv = reinterpret_cast<double2*>(gb + Lay.sv) + vl * A.vm_depth;
    double2* sd = reinterpret_cast<double2*>(gb + Lay.sd) + static_cast<size_t>(vl) * A.vm_depth * kMaxGrad;
    int32_t* tp = reinterpret_cast<int32_t*>(gb + Lay.tp) + vl * A.vm_depth;
    double2* dts = reinterpret_cast<double2*>(gb + Lay.dts);
    // single-precision views (mixed form)
    float2* s_tab32 = reinterpret_cast<float2*>(gb + Lay.tab32);
    float2* s_G32 = reinterpret_cast<float2*>(gb + Lay.G);
    float* s_G32f = reinterpret_cast<float*>(gb + Lay.G);
    float2* s_LS32 = reinterpret_cast<float2*>(gb + Lay.LS);
    float* s_LS32f = reinterpret_cast<float*>(gb + Lay.LS);
    float* s_MU32 = reinterpret_cast<float*>(gm + Lay.MU);
    float* s_YB32 = reinterpret_cast<float*>(gm + Lay.YB32);
    float2* s_dcls32 = reinterpret_cast<float2*>(gb + Lay.dcls32);
    float2* s_S32 = reinterpret_cast<float2*>((Lay.s_shared ? gb : gm) + Lay.S);
    const bool integral = A.output == OBE_OUTPUT_WEIGHTED_INTEGRAL;
    // solution weights b (row 5 of the stage table) and stage times c_s
    double bw[6], cs[6];
#pragma unroll
    for (int s = 0; s < 6; ++s) bw[s] = kTab.a[M][5][s];
    cs[0] = 0.0;
#pragma unroll
    for (int s = 1; s < 5; ++s) cs[s] = kTab.c[M][s - 1];
    cs[5] = 1.0;

    while (true) {
        if (lt == 0) *s_traj = static_cast<long long>(atomicAdd(J.counter, 1ull));
        gsync<TPT>(g);
        const long long traj = *s_traj;
        gsync<TPT>(g);
        if (traj >= A.n_traj) break;
        int bad = 0;
        const obe_traj_stats fst = J.fwd_stats[traj];
        const long long n_acc = fst.accepted_steps;
        const bool ev_hit = A.ev_kind != OBE_EVENT_NONE && fst.event_triggered != 0 && n_acc > 0;
        if (fst.status != 0 || n_acc > J.tape_cap) {
            if (lt == 0) J.adj_status[traj] = ADJ_FORWARD_FAILED;
            for (int q = lt; q < ng; q += TPT) J.param_grad[traj * ng + q] = CUDART_NAN;
            gsync<TPT>(g);
            continue;
        }

        // ---- parameters, derivative seeds, time-independent coefficients ----
        if (lt < 6) {
            init_slots(P, A, traj, slots);
            for (int s = 0; s < P.n_slots; ++s)
                for (int q = 0; q < ng; ++q)
                    dslots[s * ng + q] = make_double2(s == J.grad_slot[q] ? 1.0 : 0.0, 0.0);
            double2 dtmp[kMaxGrad];
            for (int c = 0; c < P.n_comp; ++c) {
                const DevExpr e = P.comp_expr[c];
                const int slot = P.comp_slot[c];
                slots[slot] = vm_eval_dual(P, e.start, e.len, slots, dslots, ng, A.t0, sv, sd, tp, dtmp, &bad);
                for (int q = 0; q < ng; ++q) dslots[slot * ng + q] = dtmp[q];
            }
        }
        if (lt == 0) {
            double2 dtmp[kMaxGrad];
            for (int k = 0; k < P.n_coeff; ++k) {
                if (P.coeff_dynamic[k]) {
                    s_cstat[k] = make_double2(0.0, 0.0);
                    for (int q = 0; q < ng; ++q) s_dcstat[k * kMaxGrad + q] = make_double2(0.0, 0.0);
                } else {
                    const DevExpr e = P.coeff_expr[k];
                    s_cstat[k] = vm_eval_dual(P, e.start, e.len, slots, dslots, ng, A.t0, sv, sd, tp, dtmp, &bad);
                    for (int q = 0; q < ng; ++q) s_dcstat[k * kMaxGrad + q] = dtmp[q];
                }
            }
            s_tab[0] = make_double2(0.0, 0.0);
        }
        for (int i = lt; i < U; i += TPT) {
            s_G[i] = make_double2(0.0, 0.0);
            s_LS[i] = make_double2(0.0, 0.0);
        }
        for (int i = lt; i < N; i += TPT) s_YB[i] = 0.0;
        gsync<TPT>(g);
        fill_formulas<TPT>(P, 1, 1 + S, s_cstat, s_cdyn, s_tab, lt);  // static entries: once
        if constexpr (MIXED) {
            gsync<TPT>(g);
            for (int f = lt; f < 1 + S; f += TPT) s_tab32[f] = make_float2(d2f(s_tab[f].x), d2f(s_tab[f].y));
        }

        // ---- the loss gradient at the final state ----
        const double* og = J.out_grad + traj * (integral ? 1 : n);
        const double gbar = integral ? og[0] : 0.0;
        if (!integral)
            for (int i = lt; i < n; i += TPT) s_YB[i] = og[i];
        if constexpr (MIXED) {
            gsync<TPT>(g);
            for (int i = lt; i < N; i += TPT) s_YB32[i] = d2f(s_YB[i]);
        }
        double pbar[kMaxGrad];
#pragma unroll
        for (int q = 0; q < kMaxGrad; ++q) pbar[q] = 0.0;
        gsync<TPT>(g);
        // ybar[i] += v on one thread (the mixed form keeps its single-precision copy in step)
        auto ybar_add = [&](int i, double v) {
            const double r = s_YB[i] + v;
            s_YB[i] = r;
            if constexpr (MIXED) s_YB32[i] = d2f(r);
        };
        // the trapezoid weight of a segment of length dt on one of its end states
        auto add_quadrature = [&](double dt) {
            if (lt == 0)
                for (int k = 0; k < A.n_weights; ++k) ybar_add(A.w_idx[k], gbar * A.w_val[k] * (0.5 * dt));
            gsync<TPT>(g);
        };

        // ---- the reverse sweep over the accepted steps, segment by segment ----
        const long long seg_len = J.ckpt > 0 ? J.ckpt : (n_acc > 0 ? n_acc : 1);
        const long long n_seg = J.ckpt > 0 ? (n_acc + seg_len - 1) / seg_len : 1;
        double* segbuf = J.ckpt > 0 ? J.seg + (static_cast<size_t>(blockIdx.x) * gpb + g) * J.seg_stride : nullptr;
        const double* tbase = J.tape + static_cast<size_t>(traj) * (J.ckpt > 0 ? J.tape_stride : J.tape_cap * J.tape_stride);
        for (long long sg = n_seg - 1; sg >= 0; --sg) {
        const long long s0 = sg * seg_len, s1 = s0 + seg_len < n_acc ? s0 + seg_len : n_acc;
        if (J.ckpt > 0 && MIXED) {
            // replay the segment's steps from its checkpointed start state as the mixed forward took
            // them: single-precision stage deviations d_2..d_7 (the same deviation-form gather) from
            // stage inputs summed in double, the solution, the trace renormalisation (trace-preserving
            // plans) and k_1 (first same as last, refreshed in double precision at the segment start
            // and every k1_refresh steps) in double; each step stored as a single-precision record
            // [y_n, k_1, d_2..d_7].  Scratch after the segment's records: y, k_1 (double), k_1 (single).
            double* yx = segbuf + static_cast<size_t>(J.ckpt + 1) * J.rec_stride;
            double* k1x = yx + N;
            float* k1fx = reinterpret_cast<float*>(yx + 2 * static_cast<size_t>(N));
            float* K32 = s_MU32;  // the step's stage deviations (the mu buffer is free here)
            float4* G4 = reinterpret_cast<float4*>(gb + Lay.G);
            float* G4f = reinterpret_cast<float*>(gb + Lay.G);
            float4* T4 = reinterpret_cast<float4*>(gm + Lay.T4);
            float4* cv = reinterpret_cast<float4*>(gb + Lay.cv);
            const double* ck = tbase + 2 * J.tape_cap + static_cast<size_t>(sg) * N;
            for (int i = lt; i < N; i += TPT) yx[i] = ck[i];
            // the trajectory's initial trace, which the forward restores after every accepted step
            const bool renorm = P.trace_preserving != 0;
            double tr0 = 1.0;
            bool renorm_t = false;
            if (renorm) {
                const double* r0 = A.rho0 + traj * A.rho0_stride;
                double tr = 0.0;
                for (int i = lt; i < n; i += TPT) tr += r0[i];
                tr0 = group_sum<TPT>(tr, s_red, lt, g);
                renorm_t = isfinite(tr0) && tr0 != 0.0;
            }
            // the table's fixed part: the records' zero coefficient and the time-independent formulas
            // (no change within a step); the formula stream refreshes the time-dependent ones per stage
            if (lt == 0) T4[0] = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int f = 1 + lt; f < 1 + S; f += TPT) T4[f] = make_float4(d2f(s_tab[f].x), d2f(s_tab[f].y), 0.f, 0.f);
            int since = 0;
            for (long long st = s0; st < s1; ++st) {
                const double tn = tbase[2 * st], h = tbase[2 * st + 1];
                // coefficient rows as the mixed forward keeps them: 0..4 at c_2..c_5, 1; 5 at t_n
                if (lt < 6) {
                    const double ts = lt < 5 ? tn + h * (lt < 4 ? kTab.c[M][lt] : 1.0) : tn;
                    double2 dtmp[kMaxGrad];
                    for (int c = 0; c < P.n_comp; ++c) {
                        if (!P.comp_dynamic[c]) continue;
                        const DevExpr e = P.comp_expr[c];
                        slots[P.comp_slot[c]] = vm_eval_dual(P, e.start, e.len, slots, dslots, 0, ts, sv, sd, tp, dtmp, &bad);
                    }
                    for (int j = 0; j < P.n_dyn; ++j) {
                        const DevExpr e = P.coeff_expr[P.dyn_ids[j]];
                        s_cdyn[lt * nd + j] = vm_eval_dual(P, e.start, e.len, slots, dslots, 0, ts, sv, sd, tp, dtmp, &bad);
                    }
                }
                gsync<TPT>(g);
                if (st == s0 || since >= A.k1_refresh) {
                    // k_1 = L(t_n) y_n in double precision
                    if (F > S) fill_formulas<TPT>(P, 1 + S, 1 + F, s_cstat, s_cdyn + 5 * nd, s_tab, lt);
                    for (int i = lt; i < N; i += TPT) {
                        if (i < n) s_G[i] = make_double2(yx[i], 0.0);
                        else s_G64[gslot64(i, n)] = yx[i];
                    }
                    gsync<TPT>(g);
                    gather_rhs<TPT, double, double2>(P, P.rec, P.lane_out, s_tab, s_G, k1x, lt);
                    gsync<TPT>(g);
                    for (int i = lt; i < N; i += TPT) k1fx[i] = d2f(k1x[i]);
                    since = 0;
                }
                stage_classes<TPT>(P, s_cstat, s_cdyn, nd, cv, lt);
                for (int s = 0; s < 6; ++s) {
                    const double hcs = h * kCsum.c[M][s];
                    for (int i = lt; i < N; i += TPT) {
                        double acc = hcs * k1x[i];
                        for (int j = 1; j <= s; ++j) acc = fma(h * kTab.a[M][s][j], f2d(K32[static_cast<size_t>(j - 1) * N + i]), acc);
                        const float dv = d2f(acc);
                        const float yv32 = d2f(yx[i]);
                        if (i < n) {
                            G4[i] = make_float4(dv, 0.f, yv32, 0.f);
                        } else {
                            const int q = gslot32(i, n);
                            G4f[q] = dv;
                            G4f[q + 2] = yv32;
                        }
                    }
                    gsync<TPT>(g);
                    fill_formulas_dev<TPT>(P.n_fiter, reinterpret_cast<const float4*>(P.fstream), cv + (s < 5 ? s : 4) * 2 * P.n_coeff,
                                           T4, lt);
                    gsync<TPT>(g);
                    gather_dev<TPT>(P, P.rec, P.lane_out, T4, G4, K32 + static_cast<size_t>(s) * N, lt);
                    gsync<TPT>(g);
                }
                double* out = segbuf + static_cast<size_t>(st - s0) * J.rec_stride;
                if (lt == 0) { out[0] = tn; out[1] = h; }
                float* fo = reinterpret_cast<float*>(out + 2);
                double tr = 0.0;
                for (int i = lt; i < N; i += TPT) {
                    fo[i] = d2f(yx[i]);
                    fo[N + i] = k1fx[i];
                    for (int r = 0; r < 6; ++r) fo[static_cast<size_t>(2 + r) * N + i] = K32[static_cast<size_t>(r) * N + i];
                    double acc = (h * kCsum.c[M][5]) * k1x[i];
                    for (int j = 1; j < 6; ++j) acc = fma(h * kTab.a[M][5][j], f2d(K32[static_cast<size_t>(j - 1) * N + i]), acc);
                    yx[i] = yx[i] + acc;
                    if (i < n) tr += yx[i];
                }
                double rf = 1.0;
                if (renorm_t) {
                    tr = group_sum<TPT>(tr, s_red, lt, g);
                    if (tr != 0.0 && isfinite(tr)) rf = tr0 / tr;
                }
                for (int i = lt; i < N; i += TPT) {
                    double k = k1x[i] + f2d(K32[static_cast<size_t>(5) * N + i]);
                    if (renorm_t) {
                        yx[i] *= rf;
                        k *= rf;
                    }
                    k1x[i] = k;
                    k1fx[i] = d2f(k);
                }
                ++since;
                gsync<TPT>(g);
            }
        } else if (J.ckpt > 0) {
            // replay the segment's steps from its checkpointed start state with the recorded
            // (t_n, h_n): the stage derivatives of the frozen steps, as the forward solve took them
            const double* ck = tbase + 2 * J.tape_cap + static_cast<size_t>(sg) * N;
            for (int i = lt; i < N; i += TPT) segbuf[2 + i] = ck[i];
            for (long long st = s0; st < s1; ++st) {
                double* rec = segbuf + static_cast<size_t>(st - s0) * J.rec_stride;
                const double tn = tbase[2 * st], h = tbase[2 * st + 1];
                if (lt == 0) { rec[0] = tn; rec[1] = h; }
                if (lt < 6) {
                    const double ts = tn + h * cs[lt];
                    double2 dtmp[kMaxGrad];
                    for (int c = 0; c < P.n_comp; ++c) {
                        if (!P.comp_dynamic[c]) continue;
                        const DevExpr e = P.comp_expr[c];
                        slots[P.comp_slot[c]] = vm_eval_dual(P, e.start, e.len, slots, dslots, 0, ts, sv, sd, tp, dtmp, &bad);
                    }
                    for (int j = 0; j < P.n_dyn; ++j) {
                        const DevExpr e = P.coeff_expr[P.dyn_ids[j]];
                        s_cdyn[lt * nd + j] = vm_eval_dual(P, e.start, e.len, slots, dslots, 0, ts, sv, sd, tp, dtmp, &bad);
                    }
                }
                gsync<TPT>(g);
                const double* yn_r = rec + 2;
                double* K_r = rec + 2 + N;
                for (int s = 0; s < 6; ++s) {
                    for (int i = lt; i < N; i += TPT) {
                        double acc = 0.0;
                        for (int l = 0; l < s; ++l) acc += kTab.a[M][s - 1][l] * K_r[static_cast<size_t>(l) * N + i];
                        const double v = s > 0 ? yn_r[i] + h * acc : yn_r[i];
                        // diagonal entries fill the whole complex slot (the buffer is shared)
                        if (i < n) s_G[i] = make_double2(v, 0.0);
                        else s_G64[gslot64(i, n)] = v;
                    }
                    gsync<TPT>(g);
                    if (F > S) fill_formulas<TPT>(P, 1 + S, 1 + F, s_cstat, s_cdyn + s * nd, s_tab, lt);
                    gsync<TPT>(g);
                    gather_rhs<TPT, double, double2>(P, P.rec, P.lane_out, s_tab, s_G, K_r + static_cast<size_t>(s) * N, lt);
                    gsync<TPT>(g);
                }
                if (ev_hit && st == n_acc - 1) {
                    // the event step's seventh stage K_7 = L(t_n + h) y_{n+1}, into the next record's
                    // state slot (the segment buffer holds one record more than a segment)
                    for (int i = lt; i < N; i += TPT) {
                        double acc = 0.0;
                        for (int s = 0; s < 6; ++s) acc += bw[s] * K_r[static_cast<size_t>(s) * N + i];
                        const double v = yn_r[i] + h * acc;
                        if (i < n) s_G[i] = make_double2(v, 0.0);
                        else s_G64[gslot64(i, n)] = v;
                    }
                    gsync<TPT>(g);
                    gather_rhs<TPT, double, double2>(P, P.rec, P.lane_out, s_tab, s_G, rec + J.rec_stride + 2, lt);
                    gsync<TPT>(g);
                }
                if (st + 1 < s1) {
                    double* yn_next = rec + J.rec_stride + 2;
                    for (int i = lt; i < N; i += TPT) {
                        double acc = 0.0;
                        for (int s = 0; s < 6; ++s) acc += bw[s] * K_r[static_cast<size_t>(s) * N + i];
                        yn_next[i] = yn_r[i] + h * acc;
                    }
                }
                gsync<TPT>(g);
            }
        }
        for (long long st = s1 - 1; st >= s0; --st) {
            const double* rec = J.ckpt > 0 ? segbuf + static_cast<size_t>(st - s0) * J.rec_stride
                                           : tbase + static_cast<size_t>(st) * J.tape_stride;
            const double tn = rec[0], h = rec[1];
            const double* yn_t = rec + 2;
            const double* Kt = rec + 2 + N;
            // The step that ended on the stop event maps y_n to the dense output at theta =
            // (t_e - t_n) / h: y(t_e) = y_n + h sum_{j<7} W_j(theta) K_j, a seven-stage explicit map
            // whose seventh stage K_7 = L(t_n + h) y_{n+1} has the input weights b.  Its final
            // weights W replace b; otherwise wgt = b.
            const bool ev_step = ev_hit && st == n_acc - 1;
            const int n_st = ev_step ? 7 : 6;
            const double* K7 = rec + J.rec_stride + 2;
            // single-precision record of the mixed form: y_n, k_1, d_2..d_7 (K_s = k_1 + d_s)
            const float* yf = reinterpret_cast<const float*>(rec + 2);
            const float* k1f = yf + N;
            const float* df = yf + 2 * static_cast<size_t>(N);
            // stage j's derivative and the start state as doubles, either record
            auto kv = [&](int j, int i) -> double {
                if constexpr (MIXED) return f2d(k1f[i]) + (j > 0 ? f2d(df[static_cast<size_t>(j - 1) * N + i]) : 0.0);
                else return j < 6 ? Kt[static_cast<size_t>(j) * N + i] : K7[i];
            };
            auto yv = [&](int i) -> double {
                if constexpr (MIXED) return f2d(yf[i]);
                else return yn_t[i];
            };
            double wgt[7], dwgt[7];
            double te = tn + h;
#pragma unroll
            for (int s = 0; s < 7; ++s) {
                wgt[s] = s < 6 ? bw[s] : 0.0;
                dwgt[s] = 0.0;
            }
            if (ev_step) {
                te = fst.event_time;
                double th = (te - tn) / h;
                th = th < 0.0 ? 0.0 : (th > 1.0 ? 1.0 : th);
                dense_weights(M, th, bw, wgt, dwgt);
            }
            const double dt = ev_step ? te - tn : (tn + h) - tn;
            const bool segment = integral && (st > 0 || A.save_start);
            if (segment) add_quadrature(dt);  // the end state y_{n+1} (or y(t_e))
            if (ev_step) {
                // t_e moves with the state and the parameters (g(t_e, y(t_e), p) = 0).  With
                // J_t = dJ/dt_e at fixed stages (the integral's end-point term plus ybar . y'(t_e)),
                // a population event g = e.y - threshold adds -J_t / (e.y'(t_e)) e to ybar(t_e); an
                // event program g(t, p) adds -J_t (dg/dp) / (dg/dt) to the parameter gradient.
                double part = 0.0;
                for (int i = lt; i < N; i += TPT) {
                    double yd = 0.0;
                    for (int j = 0; j < 7; ++j) yd += dwgt[j] * kv(j, i);
                    part += s_YB[i] * yd;
                }
                double jt = group_sum<TPT>(part, s_red, lt, g);
                if (lt == 0) {
                    auto y_te = [&](int i) {
                        double acc = 0.0;
                        for (int j = 0; j < 7; ++j) acc += wgt[j] * kv(j, i);
                        return yv(i) + h * acc;
                    };
                    auto yd_te = [&](int i) {
                        double acc = 0.0;
                        for (int j = 0; j < 7; ++j) acc += dwgt[j] * kv(j, i);
                        return acc;
                    };
                    if (segment) {
                        double wy = 0.0;
                        for (int k = 0; k < A.n_weights; ++k) wy += A.w_val[k] * (yv(A.w_idx[k]) + y_te(A.w_idx[k]));
                        jt += 0.5 * gbar * wy;
                    }
                    if (A.ev_kind == OBE_EVENT_POPULATION) {
                        double ey = 0.0;
                        for (int k = 0; k < A.n_ev; ++k) ey += yd_te(A.ev_idx[k]);
                        const double c = -jt / ey;
                        if (!isfinite(c)) bad = ADJ_EVENT_TANGENT;
                        else
                            for (int k = 0; k < A.n_ev; ++k) ybar_add(A.ev_idx[k], c);
                    } else if (ng > 0) {
                        // dg/dp: the time-dependent compounds and the event program at t_e in dual numbers
                        double2 dtmp[kMaxGrad], gp[kMaxGrad], gt;
                        int hb = 0;
                        for (int c = 0; c < P.n_comp; ++c) {
                            if (!P.comp_dynamic[c]) continue;
                            const DevExpr e = P.comp_expr[c];
                            const int slot = P.comp_slot[c];
                            slots[slot] = vm_eval_dual(P, e.start, e.len, slots, dslots, ng, te, sv, sd, tp, dtmp, &hb);
                            for (int q = 0; q < ng; ++q) dslots[slot * ng + q] = dtmp[q];
                        }
                        vm_eval_dual_prog(P, A.ev_op, A.ev_arg, A.ev_fn, A.ev_val, 0, A.ev_len, slots, dslots, ng, te, sv, sd,
                                          tp, gp, &hb, -1);
                        // dg/dt: the same programs with the time seeded (a compound whose time derivative
                        // goes through a helper, e.g. a square wave, gets NaN, which matters only if the
                        // event program reads it)
                        for (int q = 0; q < P.n_slots; ++q) dts[q] = make_double2(0.0, 0.0);
                        for (int c = 0; c < P.n_comp; ++c) {
                            if (!P.comp_dynamic[c]) continue;
                            const DevExpr e = P.comp_expr[c];
                            int hc = 0;
                            double2& dt_slot = dts[P.comp_slot[c]];
                            vm_eval_dual_prog(P, P.ins_op, P.ins_arg, P.ins_fn, P.ins_val, e.start, e.len, slots, dts, 1, te, sv,
                                              sd, tp, &dt_slot, &hc, 0);
                            if (hc) dt_slot = make_double2(CUDART_NAN, CUDART_NAN);
                        }
                        vm_eval_dual_prog(P, A.ev_op, A.ev_arg, A.ev_fn, A.ev_val, 0, A.ev_len, slots, dts, 1, te, sv, sd, tp, &gt,
                                          &hb, 0);
                        if (hb || !isfinite(gt.x)) bad = ADJ_HELPER_DERIVATIVE;
                        for (int q = 0; q < ng; ++q) {
                            const double c = -jt * gp[q].x / gt.x;
                            if (!isfinite(c)) bad = ADJ_EVENT_TANGENT;
                            else pbar[q] += c;
                        }
                    }
                }
                gsync<TPT>(g);
            }
            // coefficient values and derivatives at the six stage times, one VM lane each (the
            // seventh stage of an event step sits at t_n + h, as the sixth)
            if (lt < 6) {
                const double ts = tn + h * cs[lt];
                double2 dtmp[kMaxGrad];
                for (int c = 0; c < P.n_comp; ++c) {
                    if (!P.comp_dynamic[c]) continue;
                    const DevExpr e = P.comp_expr[c];
                    const int slot = P.comp_slot[c];
                    slots[slot] = vm_eval_dual(P, e.start, e.len, slots, dslots, ng, ts, sv, sd, tp, dtmp, &bad);
                    for (int q = 0; q < ng; ++q) dslots[slot * ng + q] = dtmp[q];
                }
                for (int j = 0; j < P.n_dyn; ++j) {
                    const DevExpr e = P.coeff_expr[P.dyn_ids[j]];
                    s_cdyn[lt * nd + j] = vm_eval_dual(P, e.start, e.len, slots, dslots, ng, ts, sv, sd, tp, dtmp, &bad);
                    for (int q = 0; q < ng; ++q) s_ddyn[(lt * nd + j) * kMaxGrad + q] = dtmp[q];
                }
            }
            gsync<TPT>(g);
            // per stage row and coefficient class: d(class value)/dp
            for (int q = lt; q < 6 * nc2 * ng; q += TPT) {
                const int row = q / (nc2 * ng), rem = q - row * nc2 * ng, cls = rem / ng, gi = rem - cls * ng;
                const int k = cls >> 1;
                const int pos = P.coeff_dyn_pos[k];
                double2 d = pos >= 0 ? s_ddyn[(row * nd + pos) * kMaxGrad + gi] : s_dcstat[k * kMaxGrad + gi];
                if (cls & 1) d.y = -d.y;
                s_dcls[(row * nc2 + cls) * kMaxGrad + gi] = d;
                if constexpr (MIXED) s_dcls32[(row * nc2 + cls) * kMaxGrad + gi] = make_float2(d2f(d.x), d2f(d.y));
            }
            gsync<TPT>(g);
            if constexpr (MIXED) {
                const float hf = d2f(h);
                float wf[7];
#pragma unroll
                for (int s = 0; s < 7; ++s) wf[s] = d2f(wgt[s]);
                float pst[kMaxGrad];  // this step's parameter-gradient terms
#pragma unroll
                for (int q = 0; q < kMaxGrad; ++q) pst[q] = 0.f;
                for (int s = n_st - 1; s >= 0; --s) {
                    const int row = s < 6 ? s : 5;
                    // lambda_s and the stage input Y_s = y_n + h (c_s k_1 + sum_l a_sl d_l) (the seventh
                    // stage's input is y_{n+1}: row 5, the solution weights)
                    // element i's lambda_s and Y_s; with the buffers in device memory (256 threads) the
                    // loads of kCh elements are issued before their first use (same arithmetic)
                    auto stage_in = [&](int i, float ybv, const float* muv, float yv, float k1v, const float* dfv) {
                        float lam = hf * wf[s] * ybv;
                        for (int m = s + 1; m < 6; ++m) lam = fmaf(hf * kTabF.a[M][m - 1][s], muv[m - 1], lam);
                        if (n_st == 7 && s < 6) lam = fmaf(hf * kTabF.a[M][5][s], muv[5], lam);
                        // diagonal entries (i < n) fill the whole complex slot: the double-precision
                        // replay reuses these buffers
                        if (i < n) s_LS32[i] = make_float2(lam, 0.f);
                        else s_LS32f[gslot64(i, n)] = lam;
                        float yin = yv;
                        if (s > 0) {
                            const int r = s - 1;
                            float acc = kTabF.csum[M][r] * k1v;
                            for (int l = 1; l < s; ++l) acc = fmaf(kTabF.a[M][r][l], dfv[l - 1], acc);
                            yin = fmaf(hf, acc, yin);
                        }
                        if (i < n) s_G32[i] = make_float2(yin, 0.f);
                        else s_G32f[gslot64(i, n)] = yin;
                    };
                    if constexpr (TPT >= 256) {
                        constexpr int kCh = 4;
                        for (int i0 = lt; i0 < N; i0 += kCh * TPT) {
                            float muv[kCh][6], dfv[kCh][5], ybv[kCh], yv[kCh], k1v[kCh];
#pragma unroll
                            for (int c = 0; c < kCh; ++c) {
                                const int i = i0 + c * TPT;
                                const bool in = i < N;
                                ybv[c] = in ? s_YB32[i] : 0.f;
                                yv[c] = in ? yf[i] : 0.f;
                                k1v[c] = in ? k1f[i] : 0.f;
#pragma unroll
                                for (int m = 1; m < 7; ++m)
                                    muv[c][m - 1] = (in && m > s && (m < 6 || n_st == 7)) ? s_MU32[static_cast<size_t>(m) * N + i] : 0.f;
#pragma unroll
                                for (int l = 1; l < 6; ++l) dfv[c][l - 1] = (in && l < s) ? df[static_cast<size_t>(l - 1) * N + i] : 0.f;
                            }
#pragma unroll
                            for (int c = 0; c < kCh; ++c)
                                if (i0 + c * TPT < N) stage_in(i0 + c * TPT, ybv[c], muv[c], yv[c], k1v[c], dfv[c]);
                        }
                    } else {
                        for (int i = lt; i < N; i += TPT) {
                            float lam = hf * wf[s] * s_YB32[i];
                            for (int m = s + 1; m < 6; ++m) lam = fmaf(hf * kTabF.a[M][m - 1][s], s_MU32[static_cast<size_t>(m) * N + i], lam);
                            if (n_st == 7 && s < 6) lam = fmaf(hf * kTabF.a[M][5][s], s_MU32[static_cast<size_t>(6) * N + i], lam);
                            if (i < n) s_LS32[i] = make_float2(lam, 0.f);
                            else s_LS32f[gslot64(i, n)] = lam;
                            float yin = yf[i];
                            if (s > 0) {
                                const int r = s - 1;
                                float acc = kTabF.csum[M][r] * k1f[i];
                                for (int l = 1; l < s; ++l) acc = fmaf(kTabF.a[M][r][l], df[static_cast<size_t>(l - 1) * N + i], acc);
                                yin = fmaf(hf, acc, yin);
                            }
                            if (i < n) s_G32[i] = make_float2(yin, 0.f);
                            else s_G32f[gslot64(i, n)] = yin;
                        }
                    }
                    if (F > S) {
                        fill_formulas<TPT>(P, 1 + S, 1 + F, s_cstat, s_cdyn + row * nd, s_tab, lt);
                        gsync<TPT>(g);
                        for (int f = 1 + S + lt; f < 1 + F; f += TPT) s_tab32[f] = make_float2(d2f(s_tab[f].x), d2f(s_tab[f].y));
                    }
                    gsync<TPT>(g);
                    // mu_s = L(t_s)^T lambda_s
                    {
                        float br = 0.f, bi = 0.f;
                        int o = 0;
                        const int n_tin = P.n_tin, n_titer = P.n_titer;
                        uint32_t dcur = n_tin > 0 ? s_lin[lt] : 0u;  // the next input slot loaded at each flush
                        auto tsum = [&](uint32_t w, float2 c, float2 u) {
                            const float tr = fmaf(c.x, u.x, c.y * u.y);
                            float ti = fmaf(c.x, u.y, -c.y * u.x);
                            if (w & kRecConj) ti = -ti;
                            br += tr;
                            bi += ti;
                            if (w & kRecFlush) {
                                s_MU32[static_cast<size_t>(s) * N + (dcur & 0xFFFFu)] = br;
                                if ((dcur >> 16) != kNoImag) s_MU32[static_cast<size_t>(s) * N + (dcur >> 16)] = bi;
                                br = 0.f;
                                bi = 0.f;
                                ++o;
                                dcur = o < n_tin ? s_lin[o * TPT + lt] : 0u;
                            }
                        };
                        // software-pipelined as the forward gather: two records per iteration, the
                        // next record's operands and the word two ahead in flight
                        uint32_t w0 = n_titer > 0 ? s_trec[lt] : 0u;
                        uint32_t w1 = n_titer > 1 ? s_trec[TPT + lt] : 0u;
                        float2 c0 = s_tab32[w0 >> kRecCoefShift];
                        float2 u0 = s_LS32[w0 & kRecIndexMask];
                        int it = 0;
                        for (; it + 1 < n_titer; it += 2) {
                            const uint32_t w2 = it + 2 < n_titer ? s_trec[(it + 2) * TPT + lt] : 0u;
                            const float2 c1 = s_tab32[w1 >> kRecCoefShift];
                            const float2 u1 = s_LS32[w1 & kRecIndexMask];
                            tsum(w0, c0, u0);
                            const uint32_t w3 = it + 3 < n_titer ? s_trec[(it + 3) * TPT + lt] : 0u;
                            c0 = s_tab32[w2 >> kRecCoefShift];
                            u0 = s_LS32[w2 & kRecIndexMask];
                            tsum(w1, c1, u1);
                            w0 = w2;
                            w1 = w3;
                        }
                        if (it < n_titer) tsum(w0, c0, u0);
                    }
                    // lambda_s^T (dL/dp) Y_s, formula by formula
                    for (int c = 0; c < nc2; ++c) s_S32[c * TPT + lt] = make_float2(0.f, 0.f);
                    {
                        float zr = 0.f, zi = 0.f;
                        auto bsum = [&](uint32_t w, float2 a, float2 lam) {
                            if (w & kBilEnd) {
                                const int f = static_cast<int>(w & ~kBilEnd);
                                for (int p = P.formula_ptr[f - 1]; p < P.formula_ptr[f]; ++p) {
                                    const int cls = P.prod_class[p];
                                    if (cls < 0) continue;
                                    const float fr = P.prod_factor32[2 * p], fi = P.prod_factor32[2 * p + 1];
                                    float2& acc = s_S32[cls * TPT + lt];
                                    acc.x += fr * zr - fi * zi;
                                    acc.y += fr * zi + fi * zr;
                                }
                                zr = 0.f;
                                zi = 0.f;
                            } else {
                                if (w & kBilConj) a.y = -a.y;
                                zr = fmaf(a.x, lam.x, fmaf(a.y, lam.y, zr));
                                zi = fmaf(a.y, lam.x, fmaf(-a.x, lam.y, zi));
                            }
                        };
                        // the operands of a record (slot 0 for a formula's end word, which reads none)
                        auto a_of = [&](uint32_t w) { return s_G32[(w & kBilEnd) ? 0u : (w & kBilSlotMask)]; };
                        auto l_of = [&](uint32_t w) { return s_LS32[(w & kBilEnd) ? 0u : ((w >> kBilOutShift) & kBilSlotMask)]; };
                        // software-pipelined as the gathers: two records per iteration
                        const int n_biter = P.n_biter;
                        uint32_t w0 = n_biter > 0 ? s_bil[lt] : 0u;
                        uint32_t w1 = n_biter > 1 ? s_bil[TPT + lt] : 0u;
                        float2 a0 = a_of(w0), l0 = l_of(w0);
                        int it = 0;
                        for (; it + 1 < n_biter; it += 2) {
                            const uint32_t w2 = it + 2 < n_biter ? s_bil[(it + 2) * TPT + lt] : 0u;
                            const float2 a1 = a_of(w1), l1 = l_of(w1);
                            bsum(w0, a0, l0);
                            const uint32_t w3 = it + 3 < n_biter ? s_bil[(it + 3) * TPT + lt] : 0u;
                            a0 = a_of(w2);
                            l0 = l_of(w2);
                            bsum(w1, a1, l1);
                            w0 = w2;
                            w1 = w3;
                        }
                        if (it < n_biter) bsum(w0, a0, l0);
                    }
                    for (int c = 0; c < nc2; ++c) {
                        const float2 Sv = s_S32[c * TPT + lt];
                        for (int q = 0; q < ng; ++q) {
                            const float2 d = s_dcls32[(row * nc2 + c) * kMaxGrad + q];
                            pst[q] = fmaf(d.x, Sv.x, fmaf(-d.y, Sv.y, pst[q]));
                        }
                    }
                    gsync<TPT>(g);
                }
                for (int q = 0; q < ng; ++q) pbar[q] += f2d(pst[q]);
                // ybar_n = ybar_{n+1} + sum_s mu_s (the stage sum in single precision)
                if constexpr (TPT >= 256) {
                    constexpr int kCh = 4;
                    for (int i0 = lt; i0 < N; i0 += kCh * TPT) {
                        float muv[kCh][7];
                        double ybv[kCh];
#pragma unroll
                        for (int c = 0; c < kCh; ++c) {
                            const int i = i0 + c * TPT;
#pragma unroll
                            for (int st7 = 0; st7 < 7; ++st7)
                                muv[c][st7] = (i < N && st7 < n_st) ? s_MU32[static_cast<size_t>(st7) * N + i] : 0.f;
                            ybv[c] = i < N ? s_YB[i] : 0.0;
                        }
#pragma unroll
                        for (int c = 0; c < kCh; ++c) {
                            const int i = i0 + c * TPT;
                            if (i < N) {
                                float acc = 0.f;
                                for (int st7 = 0; st7 < n_st; ++st7) acc += muv[c][st7];
                                const double r = ybv[c] + f2d(acc);
                                s_YB[i] = r;
                                s_YB32[i] = d2f(r);
                            }
                        }
                    }
                } else {
                    for (int i = lt; i < N; i += TPT) {
                        float acc = 0.f;
                        for (int s = 0; s < n_st; ++s) acc += s_MU32[static_cast<size_t>(s) * N + i];
                        ybar_add(i, f2d(acc));
                    }
                }
                gsync<TPT>(g);
            } else {
            for (int s = n_st - 1; s >= 0; --s) {
                const int row = s < 6 ? s : 5;
                // lambda_s (adjoint of K_s) into the lambda slot buffer; Y_s into the input buffer
                for (int i = lt; i < N; i += TPT) {
                    double lam = h * wgt[s] * s_YB[i];
                    for (int m = s + 1; m < 6; ++m) lam += h * kTab.a[M][m - 1][s] * s_MU[static_cast<size_t>(m) * N + i];
                    if (n_st == 7 && s < 6) lam += h * bw[s] * s_MU[static_cast<size_t>(6) * N + i];
                    s_LS64[gslot64(i, n)] = lam;
                    double acc = 0.0;
                    if (s < 6)
                        for (int l = 0; l < s; ++l) acc += kTab.a[M][s - 1][l] * Kt[static_cast<size_t>(l) * N + i];
                    else
                        for (int l = 0; l < 6; ++l) acc += bw[l] * Kt[static_cast<size_t>(l) * N + i];
                    s_G64[gslot64(i, n)] = s > 0 ? yn_t[i] + h * acc : yn_t[i];
                }
                gsync<TPT>(g);
                if (F > S) fill_formulas<TPT>(P, 1 + S, 1 + F, s_cstat, s_cdyn + row * nd, s_tab, lt);
                gsync<TPT>(g);
                // mu_s = L(t_s)^T lambda_s on the input-major stream
                {
                    double br = 0.0, bi = 0.0;
                    int o = 0;
                    const int n_tin = P.n_tin;
                    uint32_t dcur = n_tin > 0 ? s_lin[lt] : 0u;  // the next input slot loaded at each flush
                    for (int it = 0; it < P.n_titer; ++it) {
                        const uint32_t w = s_trec[it * TPT + lt];
                        const double2 c = s_tab[w >> kRecCoefShift];
                        const double2 u = s_LS[w & kRecIndexMask];
                        const double tr = c.x * u.x + c.y * u.y;
                        double ti = c.x * u.y - c.y * u.x;
                        if (w & kRecConj) ti = -ti;
                        br += tr;
                        bi += ti;
                        if (w & kRecFlush) {
                            s_MU[static_cast<size_t>(s) * N + (dcur & 0xFFFFu)] = br;
                            if ((dcur >> 16) != kNoImag) s_MU[static_cast<size_t>(s) * N + (dcur >> 16)] = bi;
                            br = 0.0;
                            bi = 0.0;
                            ++o;
                            dcur = o < n_tin ? s_lin[o * TPT + lt] : 0u;
                        }
                    }
                }
                // lambda_s^T (dL/dp) Y_s: per-class sums of factor * Y_in' * conj(lambda_out), formula
                // by formula: z = sum over the formula's records of Y_in' conj(lambda_out), then
                // each of its class products adds factor * z
                for (int c = 0; c < nc2; ++c) s_S[c * TPT + lt] = make_double2(0.0, 0.0);
                {
                    double zr = 0.0, zi = 0.0;
                    for (int it = 0; it < P.n_biter; ++it) {
                        const uint32_t w = s_bil[it * TPT + lt];
                        if (w & kBilEnd) {
                            const int f = static_cast<int>(w & ~kBilEnd);
                            for (int p = P.formula_ptr[f - 1]; p < P.formula_ptr[f]; ++p) {
                                const int cls = P.prod_class[p];
                                if (cls < 0) continue;
                                const double fr = P.prod_factor[2 * p], fi = P.prod_factor[2 * p + 1];
                                double2& acc = s_S[cls * TPT + lt];
                                acc.x += fr * zr - fi * zi;
                                acc.y += fr * zi + fi * zr;
                            }
                            zr = 0.0;
                            zi = 0.0;
                        } else {
                            double2 a = s_G[w & kBilSlotMask];
                            if (w & kBilConj) a.y = -a.y;
                            const double2 lam = s_LS[(w >> kBilOutShift) & kBilSlotMask];
                            zr += a.x * lam.x + a.y * lam.y;
                            zi += a.y * lam.x - a.x * lam.y;
                        }
                    }
                }
                for (int c = 0; c < nc2; ++c) {
                    const double2 Sv = s_S[c * TPT + lt];
                    for (int q = 0; q < ng; ++q) {
                        const double2 d = s_dcls[(row * nc2 + c) * kMaxGrad + q];
                        pbar[q] += d.x * Sv.x - d.y * Sv.y;
                    }
                }
                gsync<TPT>(g);
            }
            // ybar_n = ybar_{n+1} + sum_s mu_s
            for (int i = lt; i < N; i += TPT) {
                double acc = s_YB[i];
                for (int s = 0; s < n_st; ++s) acc += s_MU[static_cast<size_t>(s) * N + i];
                s_YB[i] = acc;
            }
            gsync<TPT>(g);
            }  // double-precision stages
            if (segment) add_quadrature(dt);  // the start state y_n
        }
        }  // segments

        // ---- outputs ----
        for (int q = 0; q < ng; ++q) {
            const double v = group_sum<TPT>(pbar[q], s_red, lt, g);
            if (lt == 0) J.param_grad[traj * ng + q] = v;
        }
        if (J.rho0_grad)
            for (int i = lt; i < N; i += TPT) J.rho0_grad[traj * N + i] = s_YB[i];
        const double any_bad = group_sum<TPT>(bad ? 1.0 : 0.0, s_red, lt, g);
        const double tangent = group_sum<TPT>(bad == ADJ_EVENT_TANGENT ? 1.0 : 0.0, s_red, lt, g);
        if (lt == 0) J.adj_status[traj] = tangent > 0.0 ? ADJ_EVENT_TANGENT : any_bad > 0.0 ? ADJ_HELPER_DERIVATIVE : ADJ_OK;
        gsync<TPT>(g);
    }
}

template <int TPT, int EPT, bool MIXED>
cudaError_t launch_adjoint_shape(const DevPlan& P, const CallArgs& A, const AdjArgs& J, int blocks, int gpb, size_t smem,
                                 size_t group_bytes, int method, cudaStream_t stream) {
    auto k = adjoint_kernel<TPT, EPT, MIXED>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    k<<<blocks, gpb * TPT, smem, stream>>>(P, A, J, gpb, group_bytes, method);
    return cudaGetLastError();
}

// the adjoint widths (the integrator shapes up to 256 threads per trajectory)
#define OBE_FOR_EACH_ADJOINT(X) X(32, 8) X(32, 16) X(64, 4) X(64, 16) X(128, 2) X(128, 12) X(128, 16) X(256, 24) X(256, 32)
#ifndef OBE_INSTANCE_TU
#define OBE_EXTERN_ADJOINT(T, E)                                                                                             \
    extern template cudaError_t launch_adjoint_shape<T, E, false>(const DevPlan&, const CallArgs&, const AdjArgs&, int, int, \
                                                                  size_t, size_t, int, cudaStream_t);                      \
    extern template cudaError_t launch_adjoint_shape<T, E, true>(const DevPlan&, const CallArgs&, const AdjArgs&, int, int,  \
                                                                 size_t, size_t, int, cudaStream_t);
OBE_FOR_EACH_ADJOINT(OBE_EXTERN_ADJOINT)
#undef OBE_EXTERN_ADJOINT
#endif

}  // namespace obe
