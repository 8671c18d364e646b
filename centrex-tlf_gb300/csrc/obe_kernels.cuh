// obe_kernels.cuh -- device side of the GB300 Lindblad expanded_sparse solver: a persistent
// kernel that owns whole trajectories (one trajectory per warp, or per group of warps for larger
// systems) and runs the Dopri5/Tsit5 (or fixed-step) loop, the packed-Hermitian RHS, the step
// controller, terminal events, saveat dense output and the observables on the device.
//
// Reference behaviour (CPU, Rust): rust/src/ode/dopri5.rs:160-379, rust/src/ode/tsit5.rs:159-363,
// rust/src/ode/fixed.rs, rust/src/ode/common.rs (controller, hinit, save plan),
// rust/src/ode/output.rs (observables), rust/src/lindblad/rhs.rs:815-876 and 1789-1867 (the
// expanded_sparse RHS), rust/src/lindblad/ode_batch.rs (batch/grid drivers).
//
// Layout of one trajectory group in shared memory: the coefficient-formula table (entry 0 = 0),
// the gather buffer (the stage input in 16-byte slots), the stage derivatives, a double push
// buffer, coefficient values and reduction scratch; the plan's gather stream is staged once per
// CTA.  Systems above 45 states keep the stage derivatives and the push buffer in a per-group
// slice of device memory.  The state y and the candidate yn stay in registers (EPT elements per
// thread, element i = lane + e * TPT).  In the mixed form the gather, the formula table and the
// stage deviations are single precision; the state, k_1, the solution update, the controller
// and the observables stay double.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>

#include <cstdint>
#include <type_traits>

#include "obe_internal.h"
#include "obe_vm.cuh"

namespace obe {

// ------------------------------------------------------------------------------------------
// tableaus (rust/src/ode/dopri5.rs:5-43, rust/src/ode/tsit5.rs:5-60)

// kTab.a[m][s][j]: stage s+2 input = y + h * sum_j kTab.a[m][s][j] K_{j+1}; row 5 is the solution.
// kC: stage times c2..c5 (c6 = c7 = 1).  kE: error weights e1..e7 (Dopri5 has no e2).
// kDd: Dopri5 dense output d1, d3..d7 (dopri5.rs:38-43).  kR: Tsit5 dense output r[i][1..4]
// (tsit5.rs:41-60).
struct Tableaus {
    double a[2][6][6];
    double c[2][4];
    double e[2][7];
    double dd[7];
    double r[7][4];
};
constexpr Tableaus kTabHost = {
    {{{1.0 / 5.0, 0, 0, 0, 0, 0},
      {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0},
      {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0},
      {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0},
      {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0},
      {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0}},
     {{0.161, 0, 0, 0, 0, 0},
      {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
      {2.8971530571054935, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
      {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
      {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
      {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}}},
    {{1.0 / 5.0, 3.0 / 10.0, 4.0 / 5.0, 8.0 / 9.0}, {0.161, 0.327, 0.9, 0.9800255409045097}},
    {{71.0 / 57600.0, 0.0, -71.0 / 16695.0, 71.0 / 1920.0, -17253.0 / 339200.0, 22.0 / 525.0, -1.0 / 40.0},
     {-0.0017800110522257771, -0.0008164344596567469, 0.007880878010261995, -0.1447110071732629,
      0.5823571654525552, -0.458082105929187, 1.0 / 66.0}},
    {-12715105075.0 / 11282082432.0, 0.0, 87487479700.0 / 32700410799.0, -10690763975.0 / 1880347072.0,
     701980252875.0 / 199316789632.0, -1453857185.0 / 822651844.0, 69997945.0 / 29380423.0},
    {{1.0, -2.763706197274826, 2.9132554618219126, -1.0530884977290216},
     {0.0, 0.1317, -0.2234, 0.1017},
     {0.0, 3.9302962368947516, -5.941033872131505, 2.490627285651253},
     {0.0, -12.411077166933676, 30.33818863028232, -16.548102889244902},
     {0.0, 37.50931341651104, -88.1789048947664, 47.37952196281928},
     {0.0, -27.896526289197286, 65.09189467479366, -34.87065786149661},
     {0.0, 1.5, -4.0, 2.5}}};

// single-precision copies for the mixed form's stage and error sums; csum = row sums of a
// (c_s up to rounding), summed in double left to right before rounding
struct TableausF {
    float a[2][6][6];
    float csum[2][6];
    float e[2][7];
};
constexpr TableausF make_tableaus_f() {
    TableausF t{};
    for (int m = 0; m < 2; ++m) {
        for (int r = 0; r < 6; ++r) {
            double sum = 0.0;
            for (int j = 0; j < 6; ++j) {
                t.a[m][r][j] = static_cast<float>(kTabHost.a[m][r][j]);
                sum += kTabHost.a[m][r][j];
            }
            t.csum[m][r] = static_cast<float>(sum);
        }
        for (int j = 0; j < 7; ++j) t.e[m][j] = static_cast<float>(kTabHost.e[m][j]);
    }
    return t;
}

// row sums of a in double (the k_1 weight of a stage input in the deviation form), summed left
// to right
struct RowSums {
    double c[2][6];
};
constexpr RowSums make_row_sums() {
    RowSums t{};
    for (int m = 0; m < 2; ++m)
        for (int r = 0; r < 6; ++r) {
            double sum = 0.0;
            for (int j = 0; j < 6; ++j) sum += kTabHost.a[m][r][j];
            t.c[m][r] = sum;
        }
    return t;
}

// compile-time tables, one copy per translation unit (no runtime initialisation)
static __constant__ Tableaus kTab = kTabHost;
static __constant__ TableausF kTabF = make_tableaus_f();
static __constant__ RowSums kCsum = make_row_sums();

constexpr int kMaxWeights = 64;
constexpr int kMaxSelected = 64;
constexpr int kMaxEventIdx = 32;
constexpr int kMaxParams = 16;

enum TrajCode : int32_t {
    ST_OK = 0,
    ST_MAXITERS = 1,
    ST_UNDERFLOW = 2,
    ST_STIFF = 3,
    ST_SAVEAT = 4,
    ST_EVENT_COMPLEX = 5,
    ST_EVENT_INDEX = 6,
    ST_POINTS = 7,
    ST_BAD_MAXITERS = 8,
    ST_BACKWARD = 9,
    ST_FIXED_DT = 10,
    ST_TAPE = 11,
    ST_FIELD_LOW = 12,   // effective plans: field coordinate below the operator grid (a = x, b = grid min)
    ST_FIELD_HIGH = 13   // ... above it (b = grid max)
};

struct TrajErr {
    double x;
    long long a, b;
};

// Per-call arguments (passed by value).  Pointers are device memory.
struct CallArgs {
    long long n_traj;
    double t0, t1, atol, rtol, dt;
    long long maxiters;
    int save_start, has_saveat, n_save;
    const double* save_times;
    int output, store_trace;
    int n_weights;
    const int* w_idx;
    const double* w_val;
    int n_sel;
    const int* sel_re;
    const int* sel_im;
    const int* sel_kind;
    int ev_kind, n_ev;
    const int* ev_idx;
    double ev_thr;
    int ev_len;  // event program in the call blob
    const int32_t* ev_op;
    const int32_t* ev_arg;
    const int32_t* ev_fn;
    const double* ev_val;
    const double* rho0;
    long long rho0_stride;
    int n_param;
    int param_slot[kMaxParams];
    const double* param_values;  // [traj][n_param] complex, or NULL (grid mode)
    int n_axes;
    long long axis_len[kMaxParams], axis_off[kMaxParams], axis_stride[kMaxParams];
    const double* axes;          // complex
    long long cap;               // output points per trajectory
    long long out_stride;        // doubles per trajectory in values
    double* values;
    double* times;               // [traj][cap] or NULL
    obe_traj_stats* stats;
    TrajErr* errs;
    unsigned long long* counter;
    int k1_refresh;  // mixed form: recompute k_1 in double every this many accepted steps
    const long long* order;   // queue position -> trajectory (cost-ordered launches), or null: identity
    unsigned char* gscratch;  // large systems: per-group global slices of the stage buffers
    size_t gstride;           // bytes per slice
    // gradient tape (double-precision adaptive solves), null when off.  tape_ckpt == 0: per
    // trajectory up to tape_cap accepted steps of [t_n, h_n, y_n (N), K_1..K_6 (6 N)], tape_stride
    // doubles apart.  tape_ckpt = C > 0: per trajectory (tape_stride doubles apart) the step log
    // [tape_cap][t_n, h_n], then y_n of every C-th step (steps 0, C, 2C, ...), N doubles each
    double* tape;
    long long tape_cap, tape_stride;
    int tape_ckpt;
    int vm_depth;    // VM stack depth of the plan's and the event's programs
    int fixed;       // 0: adaptive; else the fixed-step obe_solver value (double-precision form only)
    int ctrl32;      // mixed form: stage inputs, error norm and controller in single precision, no renormalisation
    int vm_smem;     // the compact time-dependent programs are staged in shared memory (PlanSmem::vprog..)
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Shared-memory layout of one trajectory group.  Gather inputs live in 16-byte slots (slot i:
// rho_ii, slot n + m: the m-th upper pair), so one record reads one input and one coefficient.
//   FP64 form: tab double2[1+F], G double2[U], K double[7][N]
//   mixed form: T4 float4[1+F] = (c, dc), G4 float4[U] = (y_s - y_n, y_n), K32 float[6][N]
//               (d_2..d_7), k1f float[N], k1 double[N]; the double-precision tab double2[1+F]
//               and G double2[U] serve only the k_1 refreshes, when K32 and k1f are dead, and
//               share their storage
//   both: ybuf double[N] (outputs, events; the mixed form's aliases G4), VM slot and stack
//   storage for the six VM lanes, coefficient rows, reduction scratch.
//   large systems (256 or 512 threads per trajectory, n > 45): the stage buffers K (k1, k1f) and ybuf --
//   and in the mixed form also the refresh buffers tab and G -- live in a per-group slice of
//   global memory (L2-resident: one trajectory per SM); `gbytes` is the slice's size.
struct GroupLayout {
    size_t tab, T4, cv, G, G4, K, k1, k1f, ybuf, vm_slots, vm_stack, vm_tup, cstat, cdyn, red, traj, bytes;
    size_t gbytes;
    bool kglob;    // K, k1, k1f, ybuf in the global slice
    bool tabglob;  // tab, G in the global slice
};

__host__ __device__ inline GroupLayout group_layout(int n, int N, int n_formula, int n_coeff, int n_dyn, int n_slots,
                                                    int vm_depth, int tpt, bool mixed) {
    // slot-buffer entries: the packed layout's n (n + 1) / 2, or N / 2 for a split-real state
    const size_t U_packed = static_cast<size_t>(n) * (n + 1) / 2, U_split = (static_cast<size_t>(N) + 1) / 2;
    const size_t U = U_packed > U_split ? U_packed : U_split;
    const bool big = tpt >= 256;
    GroupLayout L{};
    L.kglob = big;
    L.tabglob = big && mixed;
    size_t o = 0, og = 0;
    size_t& ok = big ? og : o;  // cursor of the stage buffers
    if (mixed) {
        L.T4 = o; o = align16(o + (1 + n_formula) * 16);
        L.cv = o; o = align16(o + 5 * 2 * static_cast<size_t>(n_coeff > 0 ? n_coeff : 1) * 16);
        L.G4 = o; o = align16(o + U * 16);
        const size_t k32 = align16(6 * 4 * static_cast<size_t>(N)), k1f = align16(4 * static_cast<size_t>(N));
        const size_t tab = align16((1 + n_formula) * 16), g = align16(U * 16);
        L.K = ok;
        L.k1f = ok + k32;
        L.tab = ok;
        L.G = ok + tab;
        ok += k32 + k1f > tab + g ? k32 + k1f : tab + g;
        L.k1 = ok; ok = align16(ok + static_cast<size_t>(N) * 8);
    } else {
        L.tab = o; o = align16(o + (1 + n_formula) * 16);
        L.G = o; o = align16(o + U * 16);
        L.K = ok; ok = align16(ok + 7 * 8 * static_cast<size_t>(N));
    }
    if (mixed && !big) {
        // the output / event buffer shares the deviation slot buffer G4 (U float4 >= N doubles):
        // the two are never live together, and G4's y_n halves and the diagonal slots' zero
        // imaginary halves are written again after every use of the buffer (restore_g4)
        L.ybuf = L.G4;
    } else {
        L.ybuf = ok; ok = align16(ok + static_cast<size_t>(N) * 8);
    }
    L.gbytes = og;
    L.vm_slots = o; o = align16(o + 6 * static_cast<size_t>(n_slots > 0 ? n_slots : 1) * 16);
    L.vm_stack = o; o = align16(o + 6 * static_cast<size_t>(vm_depth) * 16);
    L.vm_tup = o; o = align16(o + 6 * static_cast<size_t>(vm_depth) * 4);
    L.cstat = o; o = align16(o + static_cast<size_t>(n_coeff > 0 ? n_coeff : 1) * 16);
    L.cdyn = o; o = align16(o + 6 * static_cast<size_t>(n_dyn > 0 ? n_dyn : 1) * 16);
    L.red = o; o = align16(o + (tpt / 32 + 4) * 8);
    L.traj = o; o = align16(o + 16);
    L.bytes = o;
    return L;
}

// Per-CTA shared copy of the plan: the gather stream (records, output slots) and, for the
// time-dependent formulas, their product lists (offsets, coefficient classes, factors in the
// precision of the form).
struct PlanSmem {
    size_t rec, out, fstream, fptr, fcls, ffac, vprog, vval, vop, varg, vfn, bytes;
};

// with_vm: also the compact time-dependent programs (the per-step coefficient rows read their
// instructions from shared memory instead of through L1, which the local-memory traffic and the
// stage buffers keep busy)
__host__ __device__ inline PlanSmem plan_smem(const DevPlan& P, int tpt, bool mixed, bool with_vm = false) {
    PlanSmem L{};
    size_t o = 0;
    if (with_vm) {
        // at the start of the shared memory, where dyn_row finds it
        L.vprog = o; o = align16(o + static_cast<size_t>(P.n_vprog) * sizeof(DevExpr));
        L.vval = o; o = align16(o + static_cast<size_t>(P.n_vins) * 16);
        L.vop = o; o = align16(o + static_cast<size_t>(P.n_vins) * 4);
        L.varg = o; o = align16(o + static_cast<size_t>(P.n_vins) * 4);
        L.vfn = o; o = align16(o + static_cast<size_t>(P.n_vins) * 4);
    }
    L.rec = o; o += static_cast<size_t>(P.n_iter) * tpt * 4;
    L.out = o; o = align16(o + static_cast<size_t>(P.n_out) * tpt * 4);
    if (mixed) {
        L.fstream = o; o = align16(o + static_cast<size_t>(P.n_fiter) * tpt * 16);
    } else {
        L.fptr = o; o = align16(o + static_cast<size_t>(P.n_formula - P.n_static_formula + 1) * 4);
        L.fcls = o; o = align16(o + static_cast<size_t>(P.n_dyn_prod) * 4);
        L.ffac = o; o = align16(o + static_cast<size_t>(P.n_dyn_prod) * 16);
    }
    L.bytes = o;
    return L;
}

template <int TPT>
__device__ __forceinline__ void gsync(int g) {
    if constexpr (TPT == 32) {
        __syncwarp();
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(TPT) : "memory");
    }
}

// Sum over the group; every thread returns the same value (fixed reduction order).
template <int TPT>
__device__ __forceinline__ double group_sum(double v, double* red, int lt, int g) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if constexpr (TPT == 32) {
        return __shfl_sync(0xffffffffu, v, 0);
    } else {
        if ((lt & 31) == 0) red[lt >> 5] = v;
        gsync<TPT>(g);
        double tot = 0.0;
#pragma unroll
        for (int w = 0; w < TPT / 32; ++w) tot += red[w];
        gsync<TPT>(g);
        return tot;
    }
}

__device__ __forceinline__ double time_tol(double t) { return 10.0 * 2.220446049250313e-16 * fmax(fabs(t), 1.0); }

// double index of packed element i inside the slot buffer G (double2[U]) of the group
// binary32 <-> binary64 conversions by field arithmetic on the integer pipe.  On this GPU a
// conversion instruction occupies the FP64 pipe like a double-precision FMA (one warp
// instruction per ~20 SM cycles whatever its active lanes), so the mixed form's per-step
// conversions go through these.  Normal numbers and zeros take the integer path; subnormals,
// infinities and NaNs fall back to the hardware conversion.
__device__ __forceinline__ double f2d(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xFFu;
    if ((b & 0x7FFFFFFFu) == 0u) return __hiloint2double(static_cast<int>(b), 0);
    if (e == 0u || e == 0xFFu) return static_cast<double>(f);
    // exponent rebias 127 -> 1023; the 23 fraction bits become the top of the 52
    const uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
    return __hiloint2double(static_cast<int>(hi), static_cast<int>(b << 29));
}
// round to nearest, ties to even
__device__ __forceinline__ float d2f(double d) {
    const uint32_t hi = static_cast<uint32_t>(__double2hiint(d)), lo = static_cast<uint32_t>(__double2loint(d));
    const uint32_t sign = hi & 0x80000000u;
    const uint32_t e = (hi >> 20) & 0x7FFu;
    if ((hi & 0x7FFFFFFFu) == 0u && lo == 0u) return __uint_as_float(sign);
    if (e < 897u || e > 1150u) return static_cast<float>(d);  // below the normal float range, overflow, inf, nan
    // the 52 fraction bits: keep the top 23, round on the 29 dropped
    const uint32_t keep = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const uint32_t rest = lo & 0x1FFFFFFFu;
    uint32_t r = ((e - 896u) << 23) | keep;
    if (rest > 0x10000000u || (rest == 0x10000000u && (keep & 1u))) r += 1u;  // a carry bumps the exponent
    return __uint_as_float(sign | r);
}

// max(|a|, |b|) of two doubles by their bit patterns (integer pipe; for non-negative doubles the
// integer order of the bits is the numeric order)
__device__ __forceinline__ double max_abs(double a, double b) {
    const long long ia = __double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFLL;
    const long long ib = __double_as_longlong(b) & 0x7FFFFFFFFFFFFFFFLL;
    return __longlong_as_double(ia > ib ? ia : ib);
}

// 1 / x for x > 0: a single-precision reciprocal refined by one Newton-Raphson step in double
// (r1 = r0 + r0 (1 - x r0)), relative error ~(2^-23)^2; x outside the single-precision normal
// range takes the double division
__device__ __forceinline__ double recip_nr(double x) {
    const uint32_t e = (static_cast<uint32_t>(__double2hiint(x)) >> 20) & 0x7FFu;
    if (e < 898u || e > 1149u) return 1.0 / x;
    const double r0 = f2d(__frcp_rn(d2f(x)));
    return fma(r0, fma(-x, r0, 1.0), r0);
}

__device__ __forceinline__ int gslot64(int i, int n) { return i < n ? 2 * i : n + i; }
// float index of packed element i's deviation inside G4 (float4[U]); + 2 for y_n
__device__ __forceinline__ int gslot32(int i, int n) { return i < n ? 4 * i : 4 * (n + ((i - n) >> 1)) + ((i - n) & 1); }

// ------------------------------------------------------------------------------------------
// the VM side of a trajectory: six VM lanes, each with its own slot values and stack in
// shared memory

struct VMLane {
    double2* slots;
    VStack stack;
    bool real;  // every slot is real and the time-dependent compounds keep it so: real-only VM
};

static __device__ __noinline__ void init_slots(const DevPlan& P, const CallArgs& A, long long traj, double2* slots) {
    for (int i = 0; i < P.n_slots; ++i)
        slots[i] = i < P.n_base ? make_double2(P.base_val[2 * i], P.base_val[2 * i + 1]) : make_double2(0.0, 0.0);
    if (A.param_values) {
        for (int k = 0; k < A.n_param; ++k) {
            const double* v = A.param_values + 2 * (traj * A.n_param + k);
            slots[A.param_slot[k]] = make_double2(v[0], v[1]);
        }
    } else if (A.n_axes > 0) {
        // row-major grid decode, last axis fastest (ode_batch.rs:353-391)
        for (int k = 0; k < A.n_axes; ++k) {
            long long idx = (traj / A.axis_stride[k]) % A.axis_len[k];
            const double* v = A.axes + 2 * (A.axis_off[k] + idx);
            slots[A.param_slot[k]] = make_double2(v[0], v[1]);
        }
    }
}

__device__ __forceinline__ double2 eval_expr(const DevPlan& P, DevExpr e, const VMLane& L, double t) {
    if (L.real && e.real_ok)
        return make_double2(vm_eval_real(P, P.ins_op, P.ins_arg, P.ins_fn, P.ins_val, e.start, e.len, L.slots, t,
                                         reinterpret_cast<double*>(L.stack.v)),
                            0.0);
    return vm_eval(P, P.ins_op, P.ins_arg, P.ins_fn, P.ins_val, e.start, e.len, L.slots, t, L.stack);
}

// Evaluate the compounds (all of them, or only the time-dependent ones) at time t.
static __device__ __noinline__ void eval_compounds(const DevPlan& P, VMLane L, double t, bool only_dynamic) {
    for (int c = 0; c < P.n_comp; ++c)
        if (!only_dynamic || P.comp_dynamic[c]) L.slots[P.comp_slot[c]] = eval_expr(P, P.comp_expr[c], L, t);
}

// The compact time-dependent programs (DevPlan::vprog..), in shared or device memory.
struct VMProg {
    const DevExpr* prog;
    const int32_t* op;
    const int32_t* arg;
    const int32_t* fn;
    const double* val;
};

// The time-dependent compounds and coefficients at time t into one coefficient row, inlined
// with the real-only VM into the integrator (as a call, the registers live across it were saved
// and restored through local memory every step).  The programs come compacted in evaluation
// order: the compounds (into their slots) and then the coefficients (into the row).
static __device__ __forceinline__ void dyn_row(const DevPlan& P, int vm_smem, VMLane L, double t, double2* row) {
    VMProg V{P.vprog, P.vop, P.varg, P.vfn, P.vval};
    if (vm_smem) {
        // the copy the integrator staged at the start of its shared memory (plan_smem, with_vm)
        extern __shared__ __align__(16) unsigned char smem[];
        const PlanSmem PS = plan_smem(P, 0, false, true);
        V = VMProg{reinterpret_cast<const DevExpr*>(smem + PS.vprog), reinterpret_cast<const int32_t*>(smem + PS.vop),
                   reinterpret_cast<const int32_t*>(smem + PS.varg), reinterpret_cast<const int32_t*>(smem + PS.vfn),
                   reinterpret_cast<const double*>(smem + PS.vval)};
    }
    for (int q = 0; q < P.n_vprog; ++q) {
        const DevExpr e = V.prog[q];
        double2 v;
        if (L.real && e.real_ok)
            v = make_double2(vm_eval_real_inl(P, V.op, V.arg, V.fn, V.val, e.start, e.len, L.slots, t,
                                              reinterpret_cast<double*>(L.stack.v)),
                             0.0);
        else
            v = vm_eval(P, V.op, V.arg, V.fn, V.val, e.start, e.len, L.slots, t, L.stack);
        if (q < P.n_vcomp) L.slots[e.pad] = v;
        else row[e.pad] = v;
    }
}

__device__ __forceinline__ double2 coeff_value(const DevPlan& P, int cls, const double2* cstat, const double2* crow) {
    int k = cls >> 1;
    int pos = P.coeff_dyn_pos[k];
    double2 c = pos >= 0 ? crow[pos] : cstat[k];
    if (cls & 1) c.y = -c.y;
    return c;
}

// formula table entries [lo, hi) in double from coefficient values (cstat: time-independent
// coefficients, crow: the time-dependent ones at the current time)
template <int TPT>
__device__ __forceinline__ void fill_formulas(const DevPlan& P, int lo, int hi, const double2* cstat, const double2* crow,
                                              double2* tab, int lt) {
    for (int f = lo + lt; f < hi; f += TPT) {
        int a = P.formula_ptr[f - 1], b = P.formula_ptr[f];
        double2 acc = make_double2(0.0, 0.0);
        for (int p = a; p < b; ++p) {
            double2 fac = make_double2(P.prod_factor[2 * p], P.prod_factor[2 * p + 1]);
            int cls = P.prod_class[p];
            double2 c = cls < 0 ? make_double2(1.0, 0.0) : coeff_value(P, cls, cstat, crow);
            double2 v = cmul(fac, c);
            acc.x += v.x;
            acc.y += v.y;
        }
        tab[f] = acc;
    }
}

// The time-dependent formulas in double from the CTA's shared copy of their product lists.
template <int TPT>
__device__ __forceinline__ void fill_formulas_dyn(const DevPlan& P, const int32_t* __restrict__ fptr,
                                                  const int32_t* __restrict__ fcls, const double2* __restrict__ ffac,
                                                  const double2* cstat, const double2* crow, double2* tab, int lt) {
    const int S = P.n_static_formula;
    for (int f = 1 + S + lt; f < 1 + P.n_formula; f += TPT) {
        int a = fptr[f - 1 - S], b = fptr[f - S];
        double2 acc = make_double2(0.0, 0.0);
        for (int p = a; p < b; ++p) {
            double2 fac = ffac[p];
            int cls = fcls[p];
            double2 c = cls < 0 ? make_double2(1.0, 0.0) : coeff_value(P, cls, cstat, crow);
            double2 v = cmul(fac, c);
            acc.x += v.x;
            acc.y += v.y;
        }
        tab[f] = acc;
    }
}

// Single-precision formula values at a stage time (.xy) and their change since the step's
// start time (.zw).  cv holds, per coefficient class (k, conj), the value and the change as
// float4; the changes were taken in double before rounding, so they keep their relative
// precision.  Pure single-precision work per product.
// The time-dependent formulas' single-precision values at a stage time (.xy) and their changes
// since the step's start (.zw), from the CTA's shared thread-interleaved product stream: each
// thread sums the products of its own formulas and stores each entry when its last product is
// in.  cv holds the stage row's per-class values and changes.
template <int TPT>
__device__ __forceinline__ void fill_formulas_dev(int n_fiter, const float4* __restrict__ fs, const float4* __restrict__ cv,
                                                  float4* __restrict__ T4, int lt) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    // one product: factor (r.x, r.y) times the class value and change (c), or a static factor
    auto sum = [&](float4 r, float4 c) {
        const uint32_t meta = __float_as_uint(r.z);
        if ((meta & kFStreamClassMask) != 0u) {
            acc.x = fmaf(r.x, c.x, fmaf(-r.y, c.y, acc.x));
            acc.y = fmaf(r.x, c.y, fmaf(r.y, c.x, acc.y));
            acc.z = fmaf(r.x, c.z, fmaf(-r.y, c.w, acc.z));
            acc.w = fmaf(r.x, c.w, fmaf(r.y, c.z, acc.w));
        } else {
            acc.x += r.x;
            acc.y += r.y;
        }
        if (meta & kFStreamFlush) {
            T4[meta >> kFStreamFormulaShift] = acc;
            acc = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    // the class value of a product (any value for a static factor, which does not read it)
    auto cls_of = [&](float4 r) {
        const uint32_t k = __float_as_uint(r.z) & kFStreamClassMask;
        return cv[k != 0u ? k - 1 : 0];
    };
    if (n_fiter <= 0) return;
    // software-pipelined like the gather: the product two ahead and the class value of the next
    // one are in flight while the current product is summed, two products per iteration
    float4 r0 = fs[lt];
    float4 r1 = n_fiter > 1 ? fs[TPT + lt] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 c0 = cls_of(r0);
    int it = 0;
    for (; it + 1 < n_fiter; it += 2) {
        const float4 r2 = it + 2 < n_fiter ? fs[(it + 2) * TPT + lt] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 c1 = cls_of(r1);
        sum(r0, c0);
        const float4 r3 = it + 3 < n_fiter ? fs[(it + 3) * TPT + lt] : make_float4(0.f, 0.f, 0.f, 0.f);
        c0 = cls_of(r2);
        sum(r1, c1);
        r0 = r2;
        r1 = r3;
    }
    if (it < n_fiter) sum(r0, c0);
}

// Per-class single-precision values and changes since the step start for the five stage rows
// (cv[row * 2 n_coeff + class]); one pass over all rows so the double-precision differences and
// conversions cost one warp instruction each.
template <int TPT>
__device__ __forceinline__ void stage_classes(const DevPlan& P, const double2* cstat, const double2* cdyn, int nd,
                                              float4* cv, int lt) {
    const int nc = 2 * P.n_coeff;
    for (int q = lt; q < 5 * nc; q += TPT) {
        const int row = q / nc, cls = q - row * nc;
        const int k = cls >> 1;
        const int pos = P.coeff_dyn_pos[k];
        double2 c = pos >= 0 ? cdyn[row * nd + pos] : cstat[k];
        double2 c0 = pos >= 0 ? cdyn[5 * nd + pos] : c;
        double dre = c.x - c0.x, dim = c.y - c0.y;
        if (cls & 1) { c.y = -c.y; dim = -dim; }
        cv[q] = make_float4(static_cast<float>(c.x), static_cast<float>(c.y), static_cast<float>(dre), static_cast<float>(dim));
    }
}

// The interpolated effective-Hamiltonian RHS (effective_lindblad/rhs.rs:88-137): the field
// interval by the reference's cached search (rhs.rs:48-86; `hint` is the trajectory's
// last_interval), then dy_i = 1 * (L_c y)_i + Omega/2 (L_o y)_i + delta (L_d y)_i, each row a sum of
// cubic-in-dx entries times y[col].  Every lane sees the same x, so the interval, the hint and
// the first range error (kept in err, err_x, err_g) are the same on all lanes.
template <int TPT>
__device__ __forceinline__ void eff_rhs(const DevPlan& P, double x, double rabi, double det, const double* __restrict__ yv,
                                        double* __restrict__ out, int& hint, int& err, double& err_x, double& err_g, int lt) {
    const int ng = P.eff_ngrid;
    const double* grid = P.eff_grid;
    int idx = 0;
    if (ng >= 2) {
        const double tol = 1e-10 * fmax(fabs(grid[ng - 1] - grid[0]), 1.0);
        if (x < grid[0] - tol) {
            if (!err) { err = ST_FIELD_LOW; err_x = x; err_g = grid[0]; }
        } else if (x > grid[ng - 1] + tol) {
            if (!err) { err = ST_FIELD_HIGH; err_x = x; err_g = grid[ng - 1]; }
        } else {
            const double xc = x < grid[0] ? grid[0] : (x > grid[ng - 1] ? grid[ng - 1] : x);
            if (xc <= grid[0]) {
                hint = 0;
            } else if (xc >= grid[ng - 1]) {
                hint = ng - 2;
                idx = ng - 2;
            } else if (hint < ng - 1 && grid[hint] <= xc && xc <= grid[hint + 1]) {
                idx = hint;
            } else {
                int c = 0;
                while (c < ng && grid[c] <= xc) ++c;
                idx = c > 0 ? c - 1 : 0;
                if (idx > ng - 2) idx = ng - 2;
                hint = idx;
            }
        }
    }
    const double dx = x - grid[idx];
    const int interval = ng >= 2 && idx > ng - 2 ? ng - 2 : idx;
    const double scale[3] = {1.0, 0.5 * rabi, det};
    for (int i = lt; i < P.N; i += TPT) {
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int32_t* rows = P.eff_rows + static_cast<size_t>(k) * (P.N + 1);
            const int32_t* cols = P.eff_cols + P.eff_col_off[k];
            const double2* cb = reinterpret_cast<const double2*>(P.eff_coef + P.eff_coef_off[k] +
                                                                 static_cast<size_t>(interval) * P.eff_nnz[k] * 4);
            double sum = 0.0;
            for (int q = rows[i]; q < rows[i + 1]; ++q) {
                const double2 c01 = cb[2 * q], c23 = cb[2 * q + 1];
                const double val = c01.x + dx * (c01.y + dx * (c23.x + dx * c23.y));
                sum += val * yv[cols[q]];
            }
            acc += scale[k] * sum;
        }
        out[i] = acc;
    }
}

// coefficient k of stage row `row` (the effective RHS's field, Rabi rate, detuning)
__device__ __forceinline__ double coef_re(const DevPlan& P, const double2* cstat, const double2* cdyn_row, int k) {
    const int pos = P.coeff_dyn_pos[k];
    return pos >= 0 ? cdyn_row[pos].x : cstat[k].x;
}

// The packed expanded_sparse RHS: one record = one 16-byte coefficient and one 16-byte input.
// The formula table, the slot buffer and the output are disjoint (restrict), so the operand
// loads of later records can be issued ahead of the output stores of earlier ones.
template <int TPT, typename T, typename T2>
__device__ __forceinline__ void gather_rhs(const DevPlan& P, const uint32_t* __restrict__ s_rec, const uint32_t* __restrict__ s_out,
                                           const T2* __restrict__ tab, const T2* __restrict__ G, T* __restrict__ K, int lt) {
    T ar = 0, ai = 0;
    int o = 0;
    const int n_iter = P.n_iter, n_out = P.n_out;
    uint32_t dcur = n_out > 0 ? s_out[lt] : 0u;  // the lane's current output; the next one loaded at each flush
#pragma unroll 4
    for (int it = 0; it < n_iter; ++it) {
        uint32_t w = s_rec[it * TPT + lt];
        T2 c = tab[w >> kRecCoefShift];
        T2 v = G[w & kRecIndexMask];
        if (w & kRecConj) v.y = -v.y;
        ar = fma(c.x, v.x, ar);
        ar = fma(-c.y, v.y, ar);
        ai = fma(c.x, v.y, ai);
        ai = fma(c.y, v.x, ai);
        if (w & kRecFlush) {
            K[dcur & 0xFFFFu] = ar;
            const uint32_t im = dcur >> 16;
            if (im != kNoImag) K[im] = ai;
            ar = 0;
            ai = 0;
            ++o;
            dcur = o < n_out ? s_out[o * TPT + lt] : 0u;
        }
    }
}

// Stage deviation d_s = L(t_s) (y_s - y_n) + (L(t_s) - L(t_n)) y_n, all in single precision.
// Software-pipelined: the operands of the next record and the record word two ahead are in flight
// while the current record is summed (the loop is latency-bound otherwise).  Two records per
// iteration, so that the pipeline's operand registers alternate instead of being copied.
template <int TPT>
__device__ __forceinline__ void gather_dev(const DevPlan& P, const uint32_t* __restrict__ s_rec, const uint32_t* __restrict__ s_out,
                                           const float4* __restrict__ T4, const float4* __restrict__ G4, float* __restrict__ K,
                                           int lt) {
    float ar = 0.f, ai = 0.f;
    int o = 0;
    const int n_iter = P.n_iter;
    // one record: its product off the accumulator's chain (one add per record on ar / ai, so the
    // products of consecutive records overlap), then the output's store when it is the last
    // the lane's current output (packed re | im << 16), the next one loaded at each flush so that
    // the store never waits on it
    const int n_out = P.n_out;
    uint32_t dcur = n_out > 0 ? s_out[lt] : 0u;
    auto sum = [&](uint32_t w, float4 c, float4 v) {
        if (w & kRecConj) { v.y = -v.y; v.w = -v.w; }
        ar += fmaf(c.x, v.x, fmaf(-c.y, v.y, fmaf(c.z, v.z, -c.w * v.w)));
        ai += fmaf(c.x, v.y, fmaf(c.y, v.x, fmaf(c.z, v.w, c.w * v.z)));
        if (w & kRecFlush) {
            K[dcur & 0xFFFFu] = ar;
            const uint32_t im = dcur >> 16;
            if (im != kNoImag) K[im] = ai;
            ar = 0.f;
            ai = 0.f;
            ++o;
            dcur = o < n_out ? s_out[o * TPT + lt] : 0u;
        }
    };
    uint32_t w0 = s_rec[lt];
    uint32_t w1 = n_iter > 1 ? s_rec[TPT + lt] : 0u;
    float4 c0 = T4[w0 >> kRecCoefShift];
    float4 v0 = G4[w0 & kRecIndexMask];
    int it = 0;
    for (; it + 1 < n_iter; it += 2) {
        const uint32_t w2 = it + 2 < n_iter ? s_rec[(it + 2) * TPT + lt] : 0u;
        const float4 c1 = T4[w1 >> kRecCoefShift];
        const float4 v1 = G4[w1 & kRecIndexMask];
        sum(w0, c0, v0);
        const uint32_t w3 = it + 3 < n_iter ? s_rec[(it + 3) * TPT + lt] : 0u;
        c0 = T4[w2 >> kRecCoefShift];
        v0 = G4[w2 & kRecIndexMask];
        sum(w1, c1, v1);
        w0 = w2;
        w1 = w3;
    }
    if (it < n_iter) sum(w0, c0, v0);
}

// ------------------------------------------------------------------------------------------
// the integrator kernel
//
// FP64 form: K_1..K_7 in double, each stage a full double RHS.
// Mixed form: k_1 = f(t_n, y_n) in double, stage deviations d_2..d_7 in single precision.  The
// stage inputs and the embedded error estimate are sums of the d_j only (a_sj sums to c_s and
// the error weights to zero), so single-precision rounding does not reach the step-size
// controller.  k_1 of the next step is k_1 + d_7 (first-same-as-last), recomputed in double
// every k1_refresh accepted steps.

// Threads per CTA of the integrator: the mixed form's smaller per-trajectory footprint fits
// more trajectory groups per SM (shared memory), at a register budget of 65536 / threads.
constexpr int kThreadsFp64 = 256;
constexpr int kThreadsMixed = 384;

// C32: the mixed form's single-precision-control variant, compiled as a kernel of its own so that
// neither variant carries the other's registers and branches
template <int TPT, int EPT, bool MIXED, bool C32>
__global__ void __launch_bounds__(TPT > 256 ? TPT : MIXED && TPT < 256 ? kThreadsMixed : kThreadsFp64, 1) integrate_kernel(const DevPlan P, const CallArgs A, int gpb, size_t group_bytes, int M) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int g = static_cast<int>(threadIdx.x) / TPT;
    const int lt = static_cast<int>(threadIdx.x) % TPT;
    const int n = P.n, N = P.N, U = P.U;

    // stage the plan's gather stream and time-dependent formula products once per CTA
    const PlanSmem PS = plan_smem(P, TPT, MIXED, A.vm_smem != 0);
    // packed index -> double index in the slot buffer (identity for the split-real effective state)
    auto gsl = [&](int i) -> int {
        if constexpr (MIXED) return gslot64(i, P.n);
        else return P.eff ? i : gslot64(i, P.n);
    };
    uint32_t* s_rec = reinterpret_cast<uint32_t*>(smem + PS.rec);
    uint32_t* s_out = reinterpret_cast<uint32_t*>(smem + PS.out);
    int32_t* s_fptr = reinterpret_cast<int32_t*>(smem + PS.fptr);
    int32_t* s_fcls = reinterpret_cast<int32_t*>(smem + PS.fcls);
    double2* s_ffac64 = reinterpret_cast<double2*>(smem + PS.ffac);
    uint32_t* s_fstream = reinterpret_cast<uint32_t*>(smem + PS.fstream);
    // the per-step coefficient rows' programs: staged in shared memory when the host found room
    if (A.vm_smem) {
        DevExpr* s_vprog = reinterpret_cast<DevExpr*>(smem + PS.vprog);
        double* s_vval = reinterpret_cast<double*>(smem + PS.vval);
        int32_t* s_vop = reinterpret_cast<int32_t*>(smem + PS.vop);
        int32_t* s_varg = reinterpret_cast<int32_t*>(smem + PS.varg);
        int32_t* s_vfn = reinterpret_cast<int32_t*>(smem + PS.vfn);
        for (int i = threadIdx.x; i < P.n_vprog; i += blockDim.x) s_vprog[i] = P.vprog[i];
        for (int i = threadIdx.x; i < P.n_vins; i += blockDim.x) {
            s_vop[i] = P.vop[i];
            s_varg[i] = P.varg[i];
            s_vfn[i] = P.vfn[i];
            s_vval[2 * i] = P.vval[2 * i];
            s_vval[2 * i + 1] = P.vval[2 * i + 1];
        }
    }
    const int vm_smem = A.vm_smem;
    {
        for (int i = threadIdx.x; i < P.n_iter * TPT; i += blockDim.x) s_rec[i] = P.rec[i];
        for (int i = threadIdx.x; i < P.n_out * TPT; i += blockDim.x) s_out[i] = P.lane_out[i];
        if constexpr (MIXED) {
            for (int i = threadIdx.x; i < P.n_fiter * TPT * 4; i += blockDim.x) s_fstream[i] = P.fstream[i];
        } else {
            const int nf = P.n_formula - P.n_static_formula;
            for (int i = threadIdx.x; i <= nf; i += blockDim.x) s_fptr[i] = P.formula_ptr[P.n_static_formula + i] - P.dyn_prod0;
            for (int i = threadIdx.x; i < P.n_dyn_prod; i += blockDim.x) {
                const int q = P.dyn_prod0 + i;
                s_fcls[i] = P.prod_class[q];
                s_ffac64[i] = make_double2(P.prod_factor[2 * q], P.prod_factor[2 * q + 1]);
            }
        }
    }
    __syncthreads();
    if (g >= gpb) return;

    const int vm_depth = A.vm_depth;
    const GroupLayout Lay = group_layout(n, N, P.n_formula, P.n_coeff, P.n_dyn, P.n_slots, vm_depth, TPT, MIXED);
    unsigned char* gb = smem + PS.bytes + static_cast<size_t>(g) * group_bytes;
    // large systems: this group's slice of the global stage-buffer scratch
    unsigned char* gg = Lay.kglob ? A.gscratch + (static_cast<size_t>(blockIdx.x) * gpb + g) * A.gstride : gb;
    unsigned char* kb = Lay.kglob ? gg : gb;
    unsigned char* tb = Lay.tabglob ? gg : gb;
    double2* s_tab = reinterpret_cast<double2*>(tb + Lay.tab);
    double2* s_G = reinterpret_cast<double2*>(tb + Lay.G);
    double* s_G64 = reinterpret_cast<double*>(tb + Lay.G);
    double* s_K = reinterpret_cast<double*>(kb + Lay.K);      // FP64 form
    float* s_K32 = reinterpret_cast<float*>(kb + Lay.K);      // mixed form
    float4* s_T4 = reinterpret_cast<float4*>(gb + Lay.T4);
    float4* s_cv = reinterpret_cast<float4*>(gb + Lay.cv);
    float4* s_G4 = reinterpret_cast<float4*>(gb + Lay.G4);
    float* s_G4f = reinterpret_cast<float*>(gb + Lay.G4);
    double* s_k1 = reinterpret_cast<double*>(kb + Lay.k1);
    float* s_k1f = reinterpret_cast<float*>(kb + Lay.k1f);
    double* s_ybuf = reinterpret_cast<double*>(kb + Lay.ybuf);
    double2* s_cstat = reinterpret_cast<double2*>(gb + Lay.cstat);
    double2* s_cdyn = reinterpret_cast<double2*>(gb + Lay.cdyn);
    double* s_red = reinterpret_cast<double*>(gb + Lay.red);
    long long* s_traj = reinterpret_cast<long long*>(gb + Lay.traj);
    const int nd = P.n_dyn > 0 ? P.n_dyn : 1;
    const int S = P.n_static_formula, F = P.n_formula;
    // mixed form: single-precision stage inputs, error norm and controller (opt-in variant), and
    // the trace renormalisation of the double-precision-control form on trace-preserving plans
    constexpr bool ctrl32 = MIXED && C32;
    const bool renorm = MIXED && !ctrl32 && P.trace_preserving != 0;
    // weighted outputs of one-warp trajectories take each accepted step's value from the registers
    const bool weighted_regs = TPT == 32 && A.n_weights <= 16 &&
                               (A.output == OBE_OUTPUT_WEIGHTED_INTEGRAL || A.output == OBE_OUTPUT_WEIGHTED_RATE);

    // this thread's VM lane (lanes 0..5 only)
    VMLane L;
    L.real = false;
    {
        int vl = lt < 6 ? lt : 0;
        L.slots = reinterpret_cast<double2*>(gb + Lay.vm_slots) + vl * (P.n_slots > 0 ? P.n_slots : 1);
        L.stack.v = reinterpret_cast<double2*>(gb + Lay.vm_stack) + vl * vm_depth;
        L.stack.tup = reinterpret_cast<int32_t*>(gb + Lay.vm_tup) + vl * vm_depth;
    }

    while (true) {
        if (lt == 0) {
            const long long q = static_cast<long long>(atomicAdd(A.counter, 1ull));
            *s_traj = q < A.n_traj && A.order ? A.order[q] : q;
        }
        gsync<TPT>(g);
        const long long traj = *s_traj;
        gsync<TPT>(g);
        if (traj >= A.n_traj) break;

        // ---------------- per-trajectory setup ----------------
        const double t0 = A.t0, t1 = A.t1;
        if (lt < 6) {
            init_slots(P, A, traj, L.slots);
            L.real = false;
            eval_compounds(P, L, t0, false);
            bool real = P.dyn_real_closed != 0;
            for (int i = 0; i < P.n_slots && real; ++i) real = L.slots[i].y == 0.0;
            L.real = real;
        }
        if (lt == 0) {
            for (int k = 0; k < P.n_coeff; ++k)
                s_cstat[k] = P.coeff_dynamic[k] ? make_double2(0.0, 0.0) : eval_expr(P, P.coeff_expr[k], L, t0);
            for (int j = 0; j < P.n_dyn; ++j) s_cdyn[5 * nd + j] = eval_expr(P, P.coeff_expr[P.dyn_ids[j]], L, t0);
            s_tab[0] = make_double2(0.0, 0.0);
            if constexpr (MIXED) s_T4[0] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        // slot buffers start at zero (the imaginary halves of diagonal slots stay zero)
        for (int i = lt; i < U; i += TPT) {
            s_G[i] = make_double2(0.0, 0.0);
            if constexpr (MIXED) s_G4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        gsync<TPT>(g);
        // time-independent formulas: once per trajectory
        fill_formulas<TPT>(P, 1, 1 + S, s_cstat, s_cdyn + 5 * nd, s_tab, lt);
        if constexpr (MIXED) {
            for (int f = 1 + lt; f < 1 + S; f += TPT) {
                double2 v = s_tab[f];
                s_T4[f] = make_float4(static_cast<float>(v.x), static_cast<float>(v.y), 0.f, 0.f);
            }
        }

        double y[EPT], yn[EPT];
        const double* r0 = A.rho0 + traj * A.rho0_stride;
#pragma unroll
        for (int e = 0; e < EPT; ++e) {
            int i = lt + e * TPT;
            y[e] = i < N ? r0[i] : 0.0;
            yn[e] = 0.0;
            if (i < N) s_G64[gsl(i)] = y[e];
        }

        // the initial trace, restored after every accepted step when renormalising
        double tr0 = 1.0;
        bool renorm_t = false;
        if (renorm) {
            double tr = 0.0;
#pragma unroll
            for (int e = 0; e < EPT; ++e)
                if (lt + e * TPT < n) tr += y[e];
            tr0 = group_sum<TPT>(tr, s_red, lt, g);
            renorm_t = isfinite(tr0) && tr0 != 0.0;
        }

        long long accepted = 0, rejected = 0, rhs_calls = 0, count = 0;
        int status = ST_OK;
        double err_x = 0.0;
        long long err_a = 0, err_b = 0;
        // effective plans: the field interval hint and the first field-range error of this trajectory
        int eff_hint = 0, eff_err = 0;
        double eff_x = 0.0, eff_g = 0.0;
        auto eff_failed = [&]() {
            if (!eff_err) return false;
            status = eff_err;
            err_x = eff_x;
            err_a = __double_as_longlong(eff_g);
            return true;
        };
        int ev_triggered = 0;
        double ev_time = CUDART_NAN;
        double integral = 0.0, last_t = CUDART_NAN, last_value = 0.0, last_time = 0.0;
        bool has_last_time = false;
        double* out_vals = A.values + traj * A.out_stride;
        double* out_times = A.times ? A.times + traj * A.cap : nullptr;

        // push the group's state in s_ybuf (already written and synced) as one output point
        // lane 0: a weighted output's value at t (output.rs:314-330: the trapezoid of the integral)
        auto weighted_value = [&](double t, long long pt, bool store, double value) {
            if (A.output == OBE_OUTPUT_WEIGHTED_INTEGRAL) {
                if (isfinite(last_t)) integral += 0.5 * (last_value + value) * (t - last_t);
                last_t = t;
                last_value = value;
                if (A.store_trace && store) out_vals[pt] = integral;
            } else if (store) {
                out_vals[pt] = value;
            }
        };
        auto push = [&](double t) {
            last_time = t;
            has_last_time = true;
            const long long pt = count;
            const bool store = pt < A.cap;
            switch (A.output) {
            case OBE_OUTPUT_POPULATIONS:
                if (store)
                    for (int i = lt; i < n; i += TPT) out_vals[pt * n + i] = s_ybuf[static_cast<size_t>(i) * P.pop_stride];
                break;
            case OBE_OUTPUT_FULL:
                if (store)
                    for (int i = lt; i < N; i += TPT) out_vals[pt * N + i] = s_ybuf[i];
                break;
            case OBE_OUTPUT_SELECTED:
                if (store)
                    for (int k = lt; k < A.n_sel; k += TPT) {
                        double re = s_ybuf[A.sel_re[k]];
                        double im = A.sel_kind[k] == 0 ? 0.0 : (A.sel_kind[k] == 1 ? s_ybuf[A.sel_im[k]] : -s_ybuf[A.sel_im[k]]);
                        out_vals[2 * (pt * A.n_sel + k)] = re;
                        out_vals[2 * (pt * A.n_sel + k) + 1] = im;
                    }
                break;
            default: {
                if (lt == 0) {
                    double value = 0.0;
                    for (int k = 0; k < A.n_weights; ++k) value += A.w_val[k] * s_ybuf[A.w_idx[k]];
                    weighted_value(t, pt, store, value);
                }
                break;
            }
            }
            if (lt == 0 && out_times && store && !(A.output == OBE_OUTPUT_WEIGHTED_INTEGRAL && !A.store_trace)) out_times[pt] = t;
            if (A.output == OBE_OUTPUT_WEIGHTED_INTEGRAL && !A.store_trace) count = 1;
            else ++count;
            gsync<TPT>(g);
        };
        // push for a weighted output whose value lane 0 already holds (one-warp trajectories)
        auto push_weighted = [&](double t, double value) {
            last_time = t;
            has_last_time = true;
            const long long pt = count;
            const bool store = pt < A.cap;
            if (lt == 0) weighted_value(t, pt, store, value);
            if (lt == 0 && out_times && store && !(A.output == OBE_OUTPUT_WEIGHTED_INTEGRAL && !A.store_trace)) out_times[pt] = t;
            if (A.output == OBE_OUTPUT_WEIGHTED_INTEGRAL && !A.store_trace) count = 1;
            else ++count;
            __syncwarp();
        };
        auto stage_registers_to_buf = [&](const double* v) {
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                int i = lt + e * TPT;
                if (i < N) s_ybuf[i] = v[e];
            }
            gsync<TPT>(g);
        };

        // event function g(t, y) for the state in s_ybuf (synced); uniform result
        auto event_value = [&](double t, bool& has, double& gv) {
            has = false;
            if (A.ev_kind == OBE_EVENT_NONE) return;
            if (lt == 0) {
                double v = 0.0;
                int bad = 0;
                if (A.ev_kind == OBE_EVENT_POPULATION) {
                    for (int k = 0; k < A.n_ev; ++k) {
                        int idx = A.ev_idx[k];
                        if (idx < 0 || idx >= n) { bad = ST_EVENT_INDEX; break; }
                        v += s_ybuf[idx];
                    }
                    v -= A.ev_thr;
                } else {
                    eval_compounds(P, L, t, true);
                    double2 r = vm_eval(P, A.ev_op, A.ev_arg, A.ev_fn, A.ev_val, 0, A.ev_len, L.slots, t, L.stack);
                    if (fabs(r.y) > 1e-12) bad = ST_EVENT_COMPLEX;
                    v = r.x;
                }
                s_red[TPT / 32] = v;
                s_red[TPT / 32 + 1] = static_cast<double>(bad);
            }
            gsync<TPT>(g);
            gv = s_red[TPT / 32];
            int bad = static_cast<int>(s_red[TPT / 32 + 1]);
            gsync<TPT>(g);
            if (bad) {
                status = bad;
                return;
            }
            has = true;
        };

        // evaluate the time-dependent coefficients at t into row `row` of s_cdyn (lane 0)
        auto dyn_coeffs_at = [&](double t, int row) {
            if (P.n_dyn > 0 && lt == 0) {
                dyn_row(P, vm_smem, L, t, s_cdyn + row * nd);
            }
        };
        // one double-precision RHS from the slot buffer: formulas for coefficient row `row`, gather into out
        auto rhs64 = [&](int row, double* out) {
            if constexpr (MIXED) {
                // the table and slot buffer share storage with the stage deviations: rebuild
                // every entry, the zero coefficient and the diagonal slots' imaginary halves
                for (int i = lt; i < n; i += TPT) s_G64[2 * i + 1] = 0.0;
                if (lt == 0) s_tab[0] = make_double2(0.0, 0.0);
                gsync<TPT>(g);  // G written, coefficient row ready
                fill_formulas<TPT>(P, 1, 1 + F, s_cstat, s_cdyn + row * nd, s_tab, lt);
            } else {
                gsync<TPT>(g);  // G written, coefficient row ready
                if (P.eff) {
                    const double2* cr = s_cdyn + row * nd;
                    eff_rhs<TPT>(P, coef_re(P, s_cstat, cr, 0), coef_re(P, s_cstat, cr, 1), coef_re(P, s_cstat, cr, 2), s_G64,
                                 out, eff_hint, eff_err, eff_x, eff_g, lt);
                    gsync<TPT>(g);  // out complete, G free
                    return;
                }
                if (F > S) fill_formulas_dyn<TPT>(P, s_fptr, s_fcls, s_ffac64, s_cstat, s_cdyn + row * nd, s_tab, lt);
            }
            gsync<TPT>(g);
            gather_rhs<TPT, double, double2>(P, s_rec, s_out, s_tab, s_G, out, lt);
            gsync<TPT>(g);  // out complete, G free
        };
        // stage derivative j (0-based: K_1..K_7) at own element i, as double
        auto Kat = [&](int j, int i) -> double {
            if constexpr (MIXED) return j == 0 ? s_k1[i] : s_k1[i] + static_cast<double>(s_K32[static_cast<size_t>(j - 1) * N + i]);
            else return s_K[static_cast<size_t>(j) * N + i];
        };
        double* k1_out = MIXED ? s_k1 : s_K;  // where a full double RHS for K_1 goes

        bool done = false;
        if (A.maxiters <= 0) {
            status = ST_BAD_MAXITERS;
            done = true;
        } else if (t1 < t0) {
            status = ST_BACKWARD;
            done = true;
        } else if (A.fixed && !(isfinite(A.dt) && A.dt > 0.0)) {
            status = ST_FIXED_DT;
            done = true;
        } else if (t1 == t0) {
            if (A.save_start) {
                stage_registers_to_buf(y);
                push(t0);
            }
            done = true;
        }

        // ---------------- fixed-step solvers (fixed.rs:133-249), double precision ----------------
        if constexpr (!MIXED) {
            if (A.fixed && !done) {
                done = true;
                int fsi = 0;
                if (A.has_saveat) {
                    bool buffered = false;
                    while (fsi < A.n_save && fabs(A.save_times[fsi] - t0) <= time_tol(t0)) {
                        if (!buffered) { stage_registers_to_buf(y); buffered = true; }
                        push(A.save_times[fsi]);
                        ++fsi;
                    }
                } else if (A.save_start) {
                    stage_registers_to_buf(y);
                    push(t0);
                }
                bool ev_old_has = false;
                double ev_old = 0.0;
                if (A.ev_kind != OBE_EVENT_NONE) {
                    stage_registers_to_buf(y);
                    event_value(t0, ev_old_has, ev_old);
                }
                double x = t0;
                long long steps = 0;
                while (status == ST_OK && x < t1 - time_tol(t1)) {
                    if (eff_failed()) break;
                    if (steps >= A.maxiters) { status = ST_MAXITERS; err_x = x; err_a = steps; break; }
                    // next_step_limit (fixed.rs:16-26): dt, clipped to t1 and the next saveat time
                    double target = fmin(x + A.dt, t1);
                    if (A.has_saveat && fsi < A.n_save && A.save_times[fsi] > x + time_tol(x)) target = fmin(target, A.save_times[fsi]);
                    const double h = target - x;
                    if (h <= 0.0 || 0.1 * h <= 2.220446049250313e-16 * fmax(fabs(x), 1.0)) { status = ST_UNDERFLOW; err_x = x; break; }
                    // coefficients at the stage times, one VM lane each: row 5 is the step start;
                    // Dopri5 rows 0-4 are c_2..c_6, RK2/RK4 use row 0 (x + h/2) and row 4 (x + h)
                    if (P.n_dyn > 0 && lt < 6) {
                        const bool dp = A.fixed == OBE_SOLVER_FIXED_DOPRI5;
                        if (lt == 5 || lt == 0 || lt == 4 || dp) {
                            double ts = x;
                            if (lt < 5) ts = dp ? x + h * (lt < 4 ? kTab.c[0][lt] : 1.0) : (lt == 0 ? x + 0.5 * h : x + h);
                            dyn_row(P, vm_smem, L, ts, s_cdyn + lt * nd);
                        }
                    }
                    // k_1 = f(x, y)
#pragma unroll
                    for (int e = 0; e < EPT; ++e) {
                        int i = lt + e * TPT;
                        if (i < N) s_G64[gsl(i)] = y[e];
                    }
                    rhs64(5, s_K);
                    if (A.fixed == OBE_SOLVER_FIXED_RK2) {
                        // rk2_step (fixed.rs:28-48)
#pragma unroll
                        for (int e = 0; e < EPT; ++e) {
                            int i = lt + e * TPT;
                            if (i < N) s_G64[gsl(i)] = y[e] + 0.5 * h * s_K[i];
                        }
                        rhs64(0, s_K + N);
#pragma unroll
                        for (int e = 0; e < EPT; ++e) {
                            int i = lt + e * TPT;
                            if (i < N) yn[e] = y[e] + h * s_K[N + i];
                        }
                        rhs_calls += 2;
                    } else if (A.fixed == OBE_SOLVER_FIXED_RK4) {
                        // rk4_step (fixed.rs:103-131)
#pragma unroll 1
                        for (int s = 0; s < 3; ++s) {
                            const double c = s < 2 ? 0.5 * h : h;
#pragma unroll
                            for (int e = 0; e < EPT; ++e) {
                                int i = lt + e * TPT;
                                if (i < N) s_G64[gsl(i)] = y[e] + c * s_K[static_cast<size_t>(s) * N + i];
                            }
                            rhs64(s < 2 ? 0 : 4, s_K + static_cast<size_t>(s + 1) * N);
                        }
#pragma unroll
                        for (int e = 0; e < EPT; ++e) {
                            int i = lt + e * TPT;
                            if (i < N)
                                yn[e] = y[e] + h * (s_K[i] + 2.0 * s_K[N + i] + 2.0 * s_K[2 * N + i] + s_K[3 * N + i]) / 6.0;
                        }
                        rhs_calls += 4;
                    } else {
                        // dopri5_step (fixed.rs:50-101): the adaptive tableau without k_7
#pragma unroll 1
                        for (int s = 0; s < 6; ++s) {
#pragma unroll
                            for (int e = 0; e < EPT; ++e) {
                                int i = lt + e * TPT;
                                if (i < N) {
                                    double acc = 0.0;
#pragma unroll
                                    for (int j = 0; j < 6; ++j)
                                        if (j <= s) acc += kTab.a[0][s][j] * s_K[static_cast<size_t>(j) * N + i];
                                    double v = y[e] + h * acc;
                                    if (s == 5) yn[e] = v;
                                    else s_G64[gsl(i)] = v;
                                }
                            }
                            if (s < 5) rhs64(s, s_K + static_cast<size_t>(s + 1) * N);
                        }
                        rhs_calls += 6;
                    }
                    ++accepted;
                    ++steps;
                    const double xo = x;
                    x += h;
                    bool ev_new_has = false, hit = false;
                    double ev_new = 0.0;
                    if (A.ev_kind != OBE_EVENT_NONE) {
                        stage_registers_to_buf(yn);
                        event_value(x, ev_new_has, ev_new);
                        if (status) { err_x = x; break; }
                        if (ev_old_has && ev_new_has &&
                            (ev_old == 0.0 || ev_new == 0.0 || (ev_old < 0.0 && ev_new > 0.0) || (ev_old > 0.0 && ev_new < 0.0))) {
                            hit = true;
                            ev_triggered = 1;
                            ev_time = ev_old == 0.0 ? xo : x;
                        }
                    }
                    if (A.has_saveat) {
                        const double stop = hit ? ev_time : x;
                        bool buffered = false;
                        while (fsi < A.n_save && A.save_times[fsi] <= stop + time_tol(stop)) {
                            if (!buffered) { stage_registers_to_buf(yn); buffered = true; }
                            push(A.save_times[fsi]);
                            ++fsi;
                        }
                    } else if (!hit) {
                        stage_registers_to_buf(yn);
                        push(x);
                    }
                    if (hit) {
                        stage_registers_to_buf(yn);
                        push(ev_time);
                        break;
                    }
#pragma unroll
                    for (int e = 0; e < EPT; ++e) y[e] = yn[e];
                    ev_old_has = ev_new_has;
                    ev_old = ev_new;
                }
                if (status == ST_OK && A.has_saveat && fsi != A.n_save && !ev_triggered) {
                    status = ST_SAVEAT;
                    err_a = fsi;
                    err_b = A.n_save;
                }
            }
        }

        double x = t0, h = 0.0;
        if (!done) {
            // initial step (dopri5.rs:199-206)
            if (isfinite(A.dt) && A.dt > 0.0) {
                h = fmin(A.dt, t1 - t0);
            } else {
                // hinit (common.rs:72-118), in double: f0 into K_1's buffer, f1 into s_ybuf
                dyn_coeffs_at(x, 5);
                rhs64(5, k1_out);
                double d0 = 0.0, d1 = 0.0;
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    int i = lt + e * TPT;
                    if (i < N) {
                        double sci = A.atol + fabs(y[e]) * A.rtol;
                        double f0 = k1_out[i];
                        d0 += (y[e] / sci) * (y[e] / sci);
                        d1 += (f0 / sci) * (f0 / sci);
                    }
                }
                d0 = group_sum<TPT>(d0, s_red, lt, g);
                d1 = group_sum<TPT>(d1, s_red, lt, g);
                double posneg = (t1 - x) >= 0.0 ? 1.0 : -1.0;
                double h_max = fabs(t1 - x);
                double h0 = (d0 < 1.0e-10 || d1 < 1.0e-10) ? 1.0e-6 : 0.01 * sqrt(d0 / d1);
                h0 = fmin(h0, h_max);
                h0 = posneg * fabs(h0);
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    int i = lt + e * TPT;
                    if (i < N) s_G64[gsl(i)] = y[e] + k1_out[i] * h0;
                }
                dyn_coeffs_at(x + h0, 4);
                rhs64(4, s_ybuf);
                double d2 = 0.0;
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    int i = lt + e * TPT;
                    if (i < N) {
                        double sci = A.atol + fabs(y[e]) * A.rtol;
                        double df = s_ybuf[i] - k1_out[i];
                        d2 += (df / sci) * (df / sci);
                    }
                }
                d2 = sqrt(group_sum<TPT>(d2, s_red, lt, g)) / h0;
                double h1 = fmax(sqrt(d1), fabs(d2)) <= 1.0e-15 ? fmax(1.0e-6, fabs(h0) * 1.0e-3)
                                                                 : pow(0.01 / fmax(sqrt(d1), d2), 1.0 / 5.0);
                h = posneg * fabs(fmin(100.0 * fabs(h0), fmin(h1, h_max)));
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    int i = lt + e * TPT;
                    if (i < N) s_G64[gsl(i)] = y[e];
                }
            }
        }

        // controller state (common.rs:20-46)
        const double beta = 0.04, alpha = 0.2 - beta * 0.75, facc1 = 1.0 / 0.2, facc2 = 1.0 / 10.0, safety = 0.9;
        double fac_old = 1.0e-4;
        // log2(1e-4): the mixed form's controller keeps log2(fac_old)
        constexpr double kLog2Fac0 = -13.287712379549449;
        double lfac_old = kLog2Fac0;
        float fac_old32 = 1.0e-4f;
        const float atolf = static_cast<float>(A.atol), rtolf = static_cast<float>(A.rtol);  // mixed error norm
        const double h_maxc = fabs(t1 - t0);
        const double posneg = (t1 - t0) >= 0.0 ? 1.0 : -1.0;
        bool reject = false;
        bool ev_old_has = false;
        double ev_old = 0.0;
        int si = 0;

        // K_1 = f(t, y) in double from the slot buffer (which holds y)
        // the mixed form's G4 after the output buffer (its alias) was used: y_n's single-precision
        // halves and the diagonal slots' zero imaginary halves (deviation and y_n); the deviation
        // halves are written afresh by every stage
        auto restore_g4 = [&]() {
            if constexpr (MIXED && TPT < 256) {
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    const int i = lt + e * TPT;
                    if (i < N) s_G4f[gslot32(i, n) + 2] = d2f(y[e]);
                    if (i < n) {
                        s_G4f[4 * i + 1] = 0.f;
                        s_G4f[4 * i + 3] = 0.f;
                    }
                }
            }
        };
        auto refresh_k1 = [&](int row) {
            rhs64(row, k1_out);
            if constexpr (MIXED) {
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    int i = lt + e * TPT;
                    if (i < N) s_k1f[i] = d2f(s_k1[i]);
                }
                restore_g4();
                if constexpr (TPT >= 256) {
#pragma unroll
                    for (int e = 0; e < EPT; ++e) {
                        int i = lt + e * TPT;
                        if (i < N) s_G4f[gslot32(i, n) + 2] = d2f(y[e]);
                    }
                }
            }
        };
        if (!done) {
            dyn_coeffs_at(x, 5);
            refresh_k1(5);
            rhs_calls = 1;
            if (A.ev_kind != OBE_EVENT_NONE) {
                stage_registers_to_buf(y);
                event_value(x, ev_old_has, ev_old);
                if (status) done = true;
            }
        }
        if (!done) {
            if (A.has_saveat) {
                bool buffered = false;
                while (si < A.n_save && fabs(A.save_times[si] - t0) <= time_tol(t0)) {
                    if (!buffered) { stage_registers_to_buf(y); buffered = true; }
                    push(A.save_times[si]);
                    ++si;
                }
            } else if (A.save_start) {
                stage_registers_to_buf(y);
                push(x);
            }
        }

        if (!done) {
            gsync<TPT>(g);  // the start's event and output reads of the buffer are complete
            restore_g4();
        }
        long long ns = 0, nst = 0, ia = 0;
        int since_refresh = 0;
        bool last = false;
        while (!done && !last) {
            if (eff_failed()) break;
            if (ns > A.maxiters) { status = ST_MAXITERS; err_x = x; err_a = ns; break; }
            if (0.1 * fabs(h) <= 2.220446049250313e-16 * fabs(x)) { status = ST_UNDERFLOW; err_x = x; break; }
            if ((x + 1.01 * h - t1) * posneg > 0.0) {
                h = t1 - x;
                last = true;
            }
            ++ns;
            // coefficients at the five distinct stage times, one VM lane each
            if (P.n_dyn > 0 && lt < 5) {
                double c = lt < 4 ? kTab.c[M][lt] : 1.0;
                double ts = x + h * c;
                dyn_row(P, vm_smem, L, ts, s_cdyn + lt * nd);
            }
            if constexpr (MIXED) {
                gsync<TPT>(g);
                stage_classes<TPT>(P, s_cstat, s_cdyn, nd, s_cv, lt);
            }
            double err = 0.0;
            float err32 = 0.f;  // the mixed form's error norm
            if constexpr (!MIXED) {
                // stages 2..7 (stage 7 input is the solution yn)
#pragma unroll 1
                for (int s = 0; s < 6; ++s) {
                    // one copy per stage: stage s issues exactly its s + 1 products per element
                    auto stage_input = [&](auto stage) {
                        constexpr int sc = decltype(stage)::value;
#pragma unroll
                        for (int e = 0; e < EPT; ++e) {
                            const int i = lt + e * TPT;
                            if (i < N) {
                                double acc = 0.0;
#pragma unroll
                                for (int j = 0; j <= sc; ++j) acc += kTab.a[M][sc][j] * Kat(j, i);
                                const double v = y[e] + h * acc;
                                if constexpr (sc == 5) yn[e] = v;
                                s_G64[gsl(i)] = v;
                            }
                        }
                    };
                    switch (s) {
                    case 0: stage_input(std::integral_constant<int, 0>{}); break;
                    case 1: stage_input(std::integral_constant<int, 1>{}); break;
                    case 2: stage_input(std::integral_constant<int, 2>{}); break;
                    case 3: stage_input(std::integral_constant<int, 3>{}); break;
                    case 4: stage_input(std::integral_constant<int, 4>{}); break;
                    default: stage_input(std::integral_constant<int, 5>{}); break;
                    }
                    rhs64(s < 4 ? s : 4, s_K + static_cast<size_t>(s + 1) * N);
                }
                // error norm (dopri5.rs:88-102, tsit5.rs:104-119)
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    int i = lt + e * TPT;
                    if (i < N) {
                        double sc = A.atol + fmax(fabs(y[e]), fabs(yn[e])) * A.rtol;
                        double acc = 0.0;
#pragma unroll
                        for (int j = 0; j < 7; ++j)
                            if (M == 1 || j != 1) acc += kTab.e[M][j] * Kat(j, i);
                        double ei = h * acc;
                        double q = ei / sc;
                        err += q * q;
                    }
                }
            } else {
                const float hf = d2f(h);
#pragma unroll 1
                for (int s = 0; s < 6; ++s) {
                    // stage input deviation y_s - y_n = h (c_s k_1 + sum_j a_sj d_j) and the solution
                    // y_{n+1} = y_n + h (k_1 + sum_j b_j d_j): summed in double from the double k_1 and
                    // the single-precision d_j (exact conversions), the deviation then rounded once
                    // to single precision for the stage's products.  The single-precision-control
                    // variant (A.ctrl32) sums the deviation in single precision.
                    const float csum = kTabF.csum[M][s];
                    if (!ctrl32) {
                        // the step size folded into the stage's weights once per stage
                        const double hcs = h * kCsum.c[M][s];
                        double ha[5];
#pragma unroll
                        for (int j = 1; j < 6; ++j) ha[j - 1] = j <= s ? h * kTab.a[M][s][j] : 0.0;
                        if constexpr (TPT >= 256) {
                            // one copy per stage (stage s loads and combines exactly its s deviations)
                            auto stage_input64_big = [&](auto stage) {
                                constexpr int sc = decltype(stage)::value;
                                constexpr int kCh = EPT < 8 ? EPT : 8;
#pragma unroll
                                for (int e0 = 0; e0 < EPT; e0 += kCh) {
                                    float kv[kCh][sc > 0 ? sc : 1];
                                    double k1d[kCh];
#pragma unroll
                                    for (int c = 0; c < kCh; ++c) {
                                        const int i = lt + (e0 + c) * TPT;
                                        const bool in = i < N;
#pragma unroll
                                        for (int j = 1; j <= sc; ++j)
                                            kv[c][j - 1] = in ? s_K32[static_cast<size_t>(j - 1) * N + i] : 0.f;
                                        k1d[c] = in ? s_k1[i] : 0.0;
                                    }
#pragma unroll
                                    for (int c = 0; c < kCh; ++c) {
                                        const int e = e0 + c;
                                        const int i = lt + e * TPT;
                                        if (i < N) {
                                            double dv = hcs * k1d[c];
#pragma unroll
                                            for (int j = 1; j <= sc; ++j) dv = fma(ha[j - 1], f2d(kv[c][j - 1]), dv);
                                            if constexpr (sc == 5) yn[e] = y[e] + dv;
                                            s_G4f[gslot32(i, n)] = d2f(dv);
                                        }
                                    }
                                }
                            };
                            switch (s) {
                            case 0: stage_input64_big(std::integral_constant<int, 0>{}); break;
                            case 1: stage_input64_big(std::integral_constant<int, 1>{}); break;
                            case 2: stage_input64_big(std::integral_constant<int, 2>{}); break;
                            case 3: stage_input64_big(std::integral_constant<int, 3>{}); break;
                            case 4: stage_input64_big(std::integral_constant<int, 4>{}); break;
                            default: stage_input64_big(std::integral_constant<int, 5>{}); break;
                            }
                        } else {
#pragma unroll
                            for (int e = 0; e < EPT; ++e) {
                                const int i = lt + e * TPT;
                                if (i < N) {
                                    double dv = hcs * s_k1[i];
#pragma unroll
                                    for (int j = 1; j < 6; ++j)
                                        if (j <= s) dv = fma(ha[j - 1], f2d(s_K32[static_cast<size_t>(j - 1) * N + i]), dv);
                                    if (s == 5) yn[e] = y[e] + dv;
                                    s_G4f[gslot32(i, n)] = d2f(dv);
                                }
                            }
                        }
                    } else if constexpr (TPT >= 256) {
                        // the stage buffers live in device memory here: each batch of kCh elements
                        // issues all its loads before the first use, so the L2 round trips overlap
                        // (the same arithmetic as below)
                        // the stage buffers live in device memory here: each batch of kCh elements
                        // issues all its loads before the first use, so the L2 round trips overlap
                        // (the same arithmetic as below)
                        constexpr int kCh = EPT < 8 ? EPT : 8;
#pragma unroll
                        for (int e0 = 0; e0 < EPT; e0 += kCh) {
                            float kv[kCh][5], k1v[kCh];
                            double k1d[kCh];
#pragma unroll
                            for (int c = 0; c < kCh; ++c) {
                                const int i = lt + (e0 + c) * TPT;
                                const bool in = i < N;
#pragma unroll
                                for (int j = 1; j < 6; ++j)
                                    kv[c][j - 1] = (in && j <= s) ? s_K32[static_cast<size_t>(j - 1) * N + i] : 0.f;
                                k1v[c] = in ? s_k1f[i] : 0.f;
                                k1d[c] = (in && s == 5) ? s_k1[i] : 0.0;
                            }
#pragma unroll
                            for (int c = 0; c < kCh; ++c) {
                                const int e = e0 + c;
                                const int i = lt + e * TPT;
                                if (i < N) {
                                    float acc = 0.f;
#pragma unroll
                                    for (int j = 1; j < 6; ++j)
                                        if (j <= s) acc = fmaf(kTabF.a[M][s][j], kv[c][j - 1], acc);
                                    if (s == 5) yn[e] = y[e] + h * (k1d[c] + f2d(acc));
                                    s_G4f[gslot32(i, n)] = hf * fmaf(csum, k1v[c], acc);
                                }
                            }
                        }
                    } else {
                    // one copy per stage (the stage index a constant in each), so that stage s reads
                    // exactly its s deviations instead of issuing all five under predicates
                    auto stage_input = [&](auto stage) {
                        constexpr int sc = decltype(stage)::value;
#pragma unroll
                        for (int e = 0; e < EPT; ++e) {
                            const int i = lt + e * TPT;
                            if (i < N) {
                                float acc = 0.f;
#pragma unroll
                                for (int j = 1; j <= sc; ++j)
                                    acc = fmaf(kTabF.a[M][sc][j], s_K32[static_cast<size_t>(j - 1) * N + i], acc);
                                const float k1f = s_k1f[i];
                                if constexpr (sc == 5) yn[e] = y[e] + h * (s_k1[i] + f2d(acc));
                                s_G4f[gslot32(i, n)] = hf * fmaf(csum, k1f, acc);
                            }
                        }
                    };
                    switch (s) {
                    case 0: stage_input(std::integral_constant<int, 0>{}); break;
                    case 1: stage_input(std::integral_constant<int, 1>{}); break;
                    case 2: stage_input(std::integral_constant<int, 2>{}); break;
                    case 3: stage_input(std::integral_constant<int, 3>{}); break;
                    case 4: stage_input(std::integral_constant<int, 4>{}); break;
                    default: stage_input(std::integral_constant<int, 5>{}); break;
                    }
                    }
                    if (s < 5) {  // stage 7 shares stage 6's time
                        gsync<TPT>(g);
                        fill_formulas_dev<TPT>(P.n_fiter, reinterpret_cast<const float4*>(s_fstream), s_cv + s * 2 * P.n_coeff,
                                               s_T4, lt);
                    }
                    gsync<TPT>(g);
                    gather_dev<TPT>(P, s_rec, s_out, s_T4, s_G4, s_K32 + static_cast<size_t>(s) * N, lt);
                    gsync<TPT>(g);
                }
                // error estimate from the deviations alone (the error weights sum to zero): each
                // element's estimate h sum_j e_j d_j is a combination of the single-precision d_j,
                // summed in single precision and converted exactly; its scale from the double state,
                // the ratio, the sum of squares and the norm in double (the single-precision-control
                // variant: all in single precision)
                if (!ctrl32) {
                    if constexpr (TPT >= 256) {
                        constexpr int kCh = EPT < 8 ? EPT : 8;
#pragma unroll
                        for (int e0 = 0; e0 < EPT; e0 += kCh) {
                            float kv[kCh][6];
#pragma unroll
                            for (int c = 0; c < kCh; ++c) {
                                const int i = lt + (e0 + c) * TPT;
#pragma unroll
                                for (int j = 1; j < 7; ++j) kv[c][j - 1] = i < N ? s_K32[static_cast<size_t>(j - 1) * N + i] : 0.f;
                            }
#pragma unroll
                            for (int c = 0; c < kCh; ++c) {
                                const int e = e0 + c;
                                if (lt + e * TPT < N) {
                                    float acc = 0.f;
#pragma unroll
                                    for (int j = 1; j < 7; ++j)
                                        if (M == 1 || j != 1) acc = fmaf(kTabF.e[M][j], kv[c][j - 1], acc);
                                    const double sc = fma(max_abs(y[e], yn[e]), A.rtol, A.atol);
                                    const double q = h * f2d(acc) * recip_nr(sc);
                                    err = fma(q, q, err);
                                }
                            }
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < EPT; ++e) {
                            const int i = lt + e * TPT;
                            if (i < N) {
                                float acc = 0.f;
#pragma unroll
                                for (int j = 1; j < 7; ++j)
                                    if (M == 1 || j != 1) acc = fmaf(kTabF.e[M][j], s_K32[static_cast<size_t>(j - 1) * N + i], acc);
                                const double sc = fma(max_abs(y[e], yn[e]), A.rtol, A.atol);
                                const double q = h * f2d(acc) * recip_nr(sc);
                                err = fma(q, q, err);
                            }
                        }
                    }
                    err = sqrt(group_sum<TPT>(err, s_red, lt, g) / static_cast<double>(N));
                } else {
                float errf = 0.f;
                if constexpr (TPT >= 256) {
                    // device-memory stage buffers: batched loads, as in the stage inputs
                    constexpr int kCh = EPT < 8 ? EPT : 8;
#pragma unroll
                    for (int e0 = 0; e0 < EPT; e0 += kCh) {
                        float kv[kCh][6];
#pragma unroll
                        for (int c = 0; c < kCh; ++c) {
                            const int i = lt + (e0 + c) * TPT;
#pragma unroll
                            for (int j = 1; j < 7; ++j) kv[c][j - 1] = i < N ? s_K32[static_cast<size_t>(j - 1) * N + i] : 0.f;
                        }
#pragma unroll
                        for (int c = 0; c < kCh; ++c) {
                            const int i = lt + (e0 + c) * TPT;
                            if (i < N) {
                                float acc = 0.f;
#pragma unroll
                                for (int j = 1; j < 7; ++j)
                                    if (M == 1 || j != 1) acc = fmaf(kTabF.e[M][j], kv[c][j - 1], acc);
                                const int gi = gslot32(i, n);
                                const float yf = s_G4f[gi + 2];
                                const float ynf = yf + s_G4f[gi];
                                const float sc = fmaf(fmaxf(fabsf(yf), fabsf(ynf)), rtolf, atolf);
                                const float q = __fdividef(hf * acc, sc);
                                errf = fmaf(q, q, errf);
                            }
                        }
                    }
                } else {
#pragma unroll
                for (int e = 0; e < EPT; ++e) {
                    int i = lt + e * TPT;
                    if (i < N) {
                        float acc = 0.f;
#pragma unroll
                        for (int j = 1; j < 7; ++j)
                            if (M == 1 || j != 1) acc = fmaf(kTabF.e[M][j], s_K32[static_cast<size_t>(j - 1) * N + i], acc);
                        const int gi = gslot32(i, n);
                        const float yf = s_G4f[gi + 2];
                        const float ynf = yf + s_G4f[gi];
                        const float sc = fmaf(fmaxf(fabsf(yf), fabsf(ynf)), rtolf, atolf);
                        const float q = __fdividef(hf * acc, sc);
                        errf = fmaf(q, q, errf);
                    }
                }
                }
                // warp-level sum in single precision, broadcast from lane 0 (fixed order)
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) errf += __shfl_down_sync(0xffffffffu, errf, off);
                if constexpr (TPT == 32) {
                    errf = __shfl_sync(0xffffffffu, errf, 0);
                } else {
                    float* redf = reinterpret_cast<float*>(s_red);
                    if ((lt & 31) == 0) redf[lt >> 5] = errf;
                    gsync<TPT>(g);
                    errf = 0.f;
#pragma unroll
                    for (int w = 0; w < TPT / 32; ++w) errf += redf[w];
                    gsync<TPT>(g);
                }
                err32 = sqrtf(errf / static_cast<float>(N));
                }
            }
            rhs_calls += 6;
            if constexpr (!MIXED) err = sqrt(group_sum<TPT>(err, s_red, lt, g) / static_cast<double>(N));
            // controller (common.rs:48-69).  The mixed form runs it in single precision (its error
            // norm is single precision already) and scales h by the rounded factor: its step sizes
            // differ from a double-precision controller's by ~1e-7 relative.
            double fac11 = 0.0, hn;
            bool accept_step;
            if (MIXED && ctrl32) {
                const float f11 = exp2f(static_cast<float>(alpha) * log2f(err32));
                float facf = f11 * exp2f(static_cast<float>(-beta) * log2f(fac_old32));
                facf = fmaxf(static_cast<float>(facc2), fminf(static_cast<float>(facc1), facf / static_cast<float>(safety)));
                hn = h * f2d(1.0f / facf);
                accept_step = err32 <= 1.0f;
                if (accept_step) fac_old32 = fmaxf(err32, 1.0e-4f);
                else hn = h * f2d(1.0f / fminf(static_cast<float>(facc1), f11 / static_cast<float>(safety)));
            } else if (MIXED) {
                // the same controller in double as exp2 of logarithms, the old factor's logarithm
                // kept from the step that set it: err^alpha fac_old^-beta = 2^(alpha log2 err - beta log2 fac_old)
                const double lerr = log2(err);
                fac11 = exp2(alpha * lerr);
                double fac = exp2(alpha * lerr - beta * lfac_old);
                fac = fmax(facc2, fmin(facc1, fac / safety));
                hn = h / fac;
                accept_step = err <= 1.0;
                if (accept_step) lfac_old = fmax(lerr, kLog2Fac0);
            } else {
                fac11 = pow(err, alpha);
                double fac = fac11 * pow(fac_old, -beta);
                fac = fmax(facc2, fmin(facc1, fac / safety));
                hn = h / fac;
                accept_step = err <= 1.0;
                if (accept_step) fac_old = fmax(err, 1.0e-4);
            }
            if (accept_step) {
                if (fabs(hn) > h_maxc) hn = posneg * h_maxc;
                if (reject) hn = posneg * fmin(fabs(hn), fabs(h));
                reject = false;
                ++accepted;
                // stiffness detection (dopri5.rs:255-277)
                if (accepted % 1000 == 0 || ia > 0) {
                    double n2 = 0.0, dd2 = 0.0;
#pragma unroll
                    for (int e = 0; e < EPT; ++e) {
                        int i = lt + e * TPT;
                        if (i < N) {
                            // the stage-6 input, recomputed as in the stage loop
                            double acc6 = 0.0;
#pragma unroll
                            for (int j = 0; j < 6; ++j)
                                if (j <= 4) acc6 += kTab.a[M][4][j] * Kat(j, i);
                            double ys6 = y[e] + h * acc6;
                            double dk = Kat(6, i) - Kat(5, i);
                            double dy = yn[e] - ys6;
                            n2 += dk * dk;
                            dd2 += dy * dy;
                        }
                    }
                    n2 = group_sum<TPT>(n2, s_red, lt, g);
                    dd2 = group_sum<TPT>(dd2, s_red, lt, g);
                    double hl = dd2 > 0.0 ? h * sqrt(n2 / dd2) : 0.0;
                    if (hl > 3.25) {
                        ++ia;
                        nst = 0;
                        if (ia == 15) { status = ST_STIFF; err_x = x; break; }
                    } else {
                        ++nst;
                        if (nst == 6) ia = 0;
                    }
                }
                const double xo = x;
                x += h;
                // dense output of own elements at theta, written to the push buffer (synced)
                auto dense_to_buf = [&](double th) {
#pragma unroll
                    for (int e = 0; e < EPT; ++e) {
                        int i = lt + e * TPT;
                        if (i >= N) continue;
                        double v;
                        if (M == 0) {
                            double r4 = 0.0;
#pragma unroll
                            for (int j = 0; j < 7; ++j)
                                if (j != 1) r4 += kTab.dd[j] * Kat(j, i);
                            r4 *= h;
                            double dd = yn[e] - y[e];
                            double bb = Kat(0, i) * h - dd;
                            double r3 = -Kat(6, i) * h + dd - bb;
                            double th1 = 1.0 - th;
                            v = y[e] + (dd + (bb + (r3 + r4 * th1) * th) * th1) * th;
                        } else {
                            double t2 = th * th, t3 = t2 * th, t4 = t3 * th;
                            double acc = 0.0;
#pragma unroll
                            for (int j = 0; j < 7; ++j) {
                                double bj = kTab.r[j][0] * th + kTab.r[j][1] * t2 + kTab.r[j][2] * t3 + kTab.r[j][3] * t4;
                                acc += bj * Kat(j, i);
                            }
                            v = y[e] + h * acc;
                        }
                        s_ybuf[i] = v;
                    }
                    gsync<TPT>(g);
                };
                // which state the event point carries: 0 = y, 1 = yn, 2 = dense at ev_theta
                int ev_state = 0;
                double ev_theta = 0.0;
                bool ev_new_has = false;
                double ev_new = 0.0;
                bool hit = false;
                double te = 0.0;
                if (A.ev_kind != OBE_EVENT_NONE) {
                    stage_registers_to_buf(yn);
                    event_value(x, ev_new_has, ev_new);
                    if (status) { err_x = x; break; }
                    if (ev_old_has && ev_new_has &&
                        (ev_old == 0.0 || ev_new == 0.0 || (ev_old < 0.0 && ev_new > 0.0) || (ev_old > 0.0 && ev_new < 0.0))) {
                        hit = true;
                        if (ev_old == 0.0) {
                            te = xo;
                            ev_state = 0;
                        } else if (ev_new == 0.0) {
                            te = x;
                            ev_state = 1;
                        } else {
                            // 60-step bisection on the dense interpolant (dopri5.rs:289-315)
                            double lo = 0.0, hi = 1.0, glo = ev_old;
                            for (int itb = 0; itb < 60; ++itb) {
                                double mid = 0.5 * (lo + hi);
                                dense_to_buf(mid);
                                bool hs;
                                double gm;
                                event_value(xo + mid * h, hs, gm);
                                if (status) break;
                                if (gm == 0.0) { lo = mid; hi = mid; break; }
                                if ((glo < 0.0 && gm > 0.0) || (glo > 0.0 && gm < 0.0)) hi = mid;
                                else { lo = mid; glo = gm; }
                            }
                            if (status) { err_x = x; break; }
                            ev_theta = 0.5 * (lo + hi);
                            ev_state = 2;
                            te = xo + ev_theta * h;
                        }
                    }
                }
                if (A.has_saveat) {
                    double event_time = hit ? te : x;
                    while (si < A.n_save && A.save_times[si] <= event_time + time_tol(event_time)) {
                        double ts = A.save_times[si];
                        if (ts >= xo - time_tol(xo)) {
                            if (fabs(ts - xo) <= time_tol(xo)) stage_registers_to_buf(y);
                            else if (fabs(ts - x) <= time_tol(x)) stage_registers_to_buf(yn);
                            else dense_to_buf((ts - xo) / h);
                            push(ts);
                        }
                        ++si;
                    }
                } else if (!hit) {
                    if (TPT == 32 && weighted_regs) {
                        // the weighted value from the registers: each weight's element shuffled to
                        // lane 0 from the lane that holds it, summed in the weights' order as push
                        // sums them (the same value, without staging y_{n+1} in shared memory)
                        double value = 0.0;
                        for (int k = 0; k < A.n_weights; ++k) {
                            const int idx = A.w_idx[k];
                            const int e = idx / TPT;
                            double sel = 0.0;
#pragma unroll
                            for (int q = 0; q < EPT; ++q)
                                if (q == e) sel = yn[q];
                            const double yv = __shfl_sync(0xffffffffu, sel, idx % TPT);
                            value += A.w_val[k] * yv;
                        }
                        push_weighted(x, value);
                    } else {
                        stage_registers_to_buf(yn);
                        push(x);
                    }
                }
                // the step for the adjoint: start time, size, start state and stages 1-6 (or,
                // checkpointed, the step and every tape_ckpt-th start state).  The step that ends on
                // a stop event also leaves its seventh stage (the dense output's first-same-as-last
                // derivative) in the next record's state slot.
                if constexpr (!MIXED) {
                    if (A.tape) {
                        const bool k7 = hit && A.tape_ckpt == 0;
                        if (accepted + (k7 ? 1 : 0) > A.tape_cap) { status = ST_TAPE; err_a = A.tape_cap; break; }
                        const long long j = accepted - 1;
                        double* rec;
                        bool keep_y = true;
                        if (A.tape_ckpt == 0) {
                            rec = A.tape + (static_cast<size_t>(traj) * A.tape_cap + j) * A.tape_stride;
                            if (lt == 0) { rec[0] = xo; rec[1] = h; }
                            rec += 2;
                            for (int i = lt; i < (k7 ? 7 : 6) * N; i += TPT)
                                rec[i < 6 * N ? N + i : A.tape_stride + (i - 6 * N)] = s_K[i];
                        } else {
                            double* base = A.tape + static_cast<size_t>(traj) * A.tape_stride;
                            if (lt == 0) { base[2 * j] = xo; base[2 * j + 1] = h; }
                            keep_y = j % A.tape_ckpt == 0;
                            rec = base + 2 * A.tape_cap + static_cast<size_t>(j / A.tape_ckpt) * N;
                        }
                        if (keep_y) {
#pragma unroll
                            for (int e = 0; e < EPT; ++e) {
                                int i = lt + e * TPT;
                                if (i < N) rec[i] = y[e];
                            }
                        }
                    }
                } else {
                    // the mixed form's tape: single-precision records [t_n, h_n | y_n, k_1, d_2..d_7]
                    // (the stage derivatives as this step used them, K_s = k_1 + d_s); checkpointed,
                    // the step log and every tape_ckpt-th start state in double, as above
                    if (A.tape) {
                        if (accepted > A.tape_cap) { status = ST_TAPE; err_a = A.tape_cap; break; }
                        const long long j = accepted - 1;
                        if (A.tape_ckpt == 0) {
                            double* rec = A.tape + (static_cast<size_t>(traj) * A.tape_cap + j) * A.tape_stride;
                            if (lt == 0) { rec[0] = xo; rec[1] = h; }
                            float* fo = reinterpret_cast<float*>(rec + 2);
#pragma unroll
                            for (int e = 0; e < EPT; ++e) {
                                int i = lt + e * TPT;
                                if (i < N) fo[i] = d2f(y[e]);
                            }
                            for (int i = lt; i < N; i += TPT) fo[N + i] = s_k1f[i];
                            for (int i = lt; i < 6 * N; i += TPT) fo[2 * N + i] = s_K32[i];
                        } else {
                            double* base = A.tape + static_cast<size_t>(traj) * A.tape_stride;
                            if (lt == 0) { base[2 * j] = xo; base[2 * j + 1] = h; }
                            if (j % A.tape_ckpt == 0) {
                                double* rec = base + 2 * A.tape_cap + static_cast<size_t>(j / A.tape_ckpt) * N;
#pragma unroll
                                for (int e = 0; e < EPT; ++e) {
                                    int i = lt + e * TPT;
                                    if (i < N) rec[i] = y[e];
                                }
                            }
                        }
                    }
                }
                if (hit) {
                    // push_unique (dopri5.rs:150-158)
                    if (!(count > 0 && fabs(last_time - te) <= time_tol(te))) {
                        if (ev_state == 0) stage_registers_to_buf(y);
                        else if (ev_state == 1) stage_registers_to_buf(yn);
                        else dense_to_buf(ev_theta);
                        push(te);
                    }
                    ev_triggered = 1;
                    ev_time = te;
                    break;
                }
                // accept: y <- yn; K_1 <- K_7
                if constexpr (!MIXED) {
#pragma unroll
                    for (int e = 0; e < EPT; ++e) {
                        int i = lt + e * TPT;
                        y[e] = yn[e];
                        if (i < N) s_K[i] = s_K[static_cast<size_t>(6) * N + i];
                    }
                } else {
                    // the coefficients at t_{n+1} = x + h are row 4; they become the step-start row
                    if (lt < P.n_dyn) s_cdyn[5 * nd + lt] = s_cdyn[4 * nd + lt];
                    // trace renormalisation in double: the next step starts from y_{n+1} tr_0 / tr(y_{n+1})
                    // and, the RHS being linear, from k_1 scaled alike
                    double rf = 1.0;
                    if (renorm_t) {
                        double tr = 0.0;
#pragma unroll
                        for (int e = 0; e < EPT; ++e)
                            if (lt + e * TPT < n) tr += yn[e];
                        tr = group_sum<TPT>(tr, s_red, lt, g);
                        if (tr != 0.0 && isfinite(tr)) rf = tr0 / tr;
                    }
                    const bool refresh = !last && ++since_refresh >= A.k1_refresh;
                    if (refresh) gsync<TPT>(g);  // the slot buffer below overlays the stage deviations
                    if (TPT >= 256 && !refresh) {
                        // first-same-as-last with device-memory stage buffers: batched loads
                        constexpr int kCh = EPT < 8 ? EPT : 8;
#pragma unroll
                        for (int e0 = 0; e0 < EPT; e0 += kCh) {
                            double k1d[kCh];
                            float d7[kCh];
#pragma unroll
                            for (int c = 0; c < kCh; ++c) {
                                const int i = lt + (e0 + c) * TPT;
                                k1d[c] = i < N ? s_k1[i] : 0.0;
                                d7[c] = i < N ? s_K32[static_cast<size_t>(5) * N + i] : 0.f;
                            }
#pragma unroll
                            for (int c = 0; c < kCh; ++c) {
                                const int e = e0 + c;
                                const int i = lt + e * TPT;
                                y[e] = renorm_t ? yn[e] * rf : yn[e];
                                if (i < N) {
                                    double k = k1d[c] + f2d(d7[c]);
                                    if (renorm_t) k *= rf;
                                    s_k1[i] = k;
                                    s_k1f[i] = d2f(k);
                                    s_G4f[gslot32(i, n) + 2] = d2f(y[e]);
                                }
                            }
                        }
                    } else {
#pragma unroll
                    for (int e = 0; e < EPT; ++e) {
                        int i = lt + e * TPT;
                        y[e] = renorm_t ? yn[e] * rf : yn[e];
                        if (i < N) {
                            if (refresh) {
                                s_G64[gsl(i)] = y[e];
                            } else {
                                // first-same-as-last: k_1 of the next step is k_7 = k_1 + d_7
                                double k = s_k1[i] + f2d(s_K32[static_cast<size_t>(5) * N + i]);
                                if (renorm_t) k *= rf;
                                s_k1[i] = k;
                                s_k1f[i] = d2f(k);
                                s_G4f[gslot32(i, n) + 2] = d2f(y[e]);
                                if (TPT < 256 && i < n) {  // the output buffer's alias (restore_g4)
                                    s_G4f[4 * i + 1] = 0.f;
                                    s_G4f[4 * i + 3] = 0.f;
                                }
                            }
                        }
                    }
                    }
                    if (refresh) {
                        since_refresh = 0;
                        refresh_k1(4);
                    }
                }
                ev_old_has = ev_new_has;
                ev_old = ev_new;
                h = hn;
                if (last) break;
            } else {
                if (!MIXED || !ctrl32) hn = h / fmin(facc1, fac11 / safety);
                reject = true;
                last = false;
                if (accepted >= 1) ++rejected;
                h = hn;
            }
            gsync<TPT>(g);
        }
        if (status == ST_OK && A.has_saveat && si != A.n_save && !ev_triggered && !done) {
            status = ST_SAVEAT;
            err_a = si;
            err_b = A.n_save;
        }

        // ---------------- finalise ----------------
        if (status == ST_OK) eff_failed();  // a range error in the last step
        if (lt == 0) {
            if (A.output == OBE_OUTPUT_WEIGHTED_INTEGRAL && !A.store_trace && has_last_time && A.cap > 0) {
                out_vals[0] = integral;
                if (out_times) out_times[0] = last_time;
            }
            obe_traj_stats st;
            st.accepted_steps = accepted;
            st.rejected_steps = rejected;
            st.rhs_calls = rhs_calls;
            st.event_triggered = ev_triggered;
            st.status = status;
            st.event_time = ev_time;
            st.n_points = (A.output == OBE_OUTPUT_WEIGHTED_INTEGRAL && !A.store_trace) ? (has_last_time ? 1 : 0) : count;
            A.stats[traj] = st;
            TrajErr te;
            te.x = err_x;
            te.a = err_a;
            te.b = err_b;
            A.errs[traj] = te;
        }
        gsync<TPT>(g);
    }
}

// One RHS evaluation per state (lindblad_rhs_py), batched; overrides per state.  The mixed
// form evaluates the products in single precision.
template <int TPT, bool MIXED>
__global__ void __launch_bounds__(TPT > 256 ? TPT : 256) rhs_kernel(const DevPlan P, long long count, const double* ts, const double* ys,
                                                  int n_ov, const int* ov_slots, const double* ov_vals, double* dys,
                                                  int gpb, size_t group_bytes, int vm_depth, unsigned char* gscratch,
                                                  size_t gstride, double* errs) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int g = static_cast<int>(threadIdx.x) / TPT;
    const int lt = static_cast<int>(threadIdx.x) % TPT;
    const int n = P.n, N = P.N, U = P.U;
    const PlanSmem PS = plan_smem(P, TPT, false);  // the layout the host sized (double-precision form)
    uint32_t* s_rec = reinterpret_cast<uint32_t*>(smem + PS.rec);
    uint32_t* s_out = reinterpret_cast<uint32_t*>(smem + PS.out);
    for (int i = threadIdx.x; i < P.n_iter * TPT; i += blockDim.x) s_rec[i] = P.rec[i];
    for (int i = threadIdx.x; i < P.n_out * TPT; i += blockDim.x) s_out[i] = P.lane_out[i];
    __syncthreads();
    if (g >= gpb) return;
    const GroupLayout Lay = group_layout(n, N, P.n_formula, P.n_coeff, P.n_dyn, P.n_slots, vm_depth, TPT, false);
    unsigned char* gb = smem + PS.bytes + static_cast<size_t>(g) * group_bytes;
    unsigned char* kb = Lay.kglob ? gscratch + (static_cast<size_t>(blockIdx.x) * gpb + g) * gstride : gb;
    double2* s_tab = reinterpret_cast<double2*>(gb + Lay.tab);
    double2* s_G = reinterpret_cast<double2*>(gb + Lay.G);
    double* s_K = reinterpret_cast<double*>(kb + Lay.K);
    double2* s_cstat = reinterpret_cast<double2*>(gb + Lay.cstat);
    double2* s_cdyn = reinterpret_cast<double2*>(gb + Lay.cdyn);
    // single-precision views for the mixed form (inside the double buffers)
    float2* s_tab32 = reinterpret_cast<float2*>(kb + Lay.K);
    float2* s_G32 = s_tab32 + (1 + P.n_formula);
    float* s_K32 = reinterpret_cast<float*>(kb + Lay.ybuf);
    VMLane L;
    L.slots = reinterpret_cast<double2*>(gb + Lay.vm_slots);
    L.stack.v = reinterpret_cast<double2*>(gb + Lay.vm_stack);
    L.stack.tup = reinterpret_cast<int32_t*>(gb + Lay.vm_tup);
    L.real = false;
    CallArgs none{};
    for (long long st = static_cast<long long>(blockIdx.x) * gpb + g; st < count; st += static_cast<long long>(gridDim.x) * gpb) {
        const double t = ts[st];
        if (lt == 0) {
            init_slots(P, none, 0, L.slots);
            for (int k = 0; k < n_ov; ++k) L.slots[ov_slots[k]] = make_double2(ov_vals[2 * (st * n_ov + k)], ov_vals[2 * (st * n_ov + k) + 1]);
            eval_compounds(P, L, t, false);
            for (int k = 0; k < P.n_coeff; ++k) {
                double2 c = eval_expr(P, P.coeff_expr[k], L, t);
                s_cstat[k] = c;
                if (P.coeff_dyn_pos[k] >= 0) s_cdyn[P.coeff_dyn_pos[k]] = c;
            }
            s_tab[0] = make_double2(0.0, 0.0);
        }
        for (int i = lt; i < U; i += TPT) s_G[i] = make_double2(0.0, 0.0);
        gsync<TPT>(g);
        for (int i = lt; i < N; i += TPT) reinterpret_cast<double*>(s_G)[P.eff ? i : gslot64(i, n)] = ys[st * N + i];
        if (P.eff) {
            // the effective RHS at t (a fresh interval hint, as the reference's debug call builds a
            // new workspace); errs[st] = (status, x, grid bound) of a field-range error, then the
            // field, Rabi rate and detuning used and the interval
            gsync<TPT>(g);
            int hint = 0, err = 0;
            double ex = 0.0, eg = 0.0;
            eff_rhs<TPT>(P, s_cstat[0].x, s_cstat[1].x, s_cstat[2].x, reinterpret_cast<const double*>(s_G), dys + st * N, hint,
                         err, ex, eg, lt);
            if (lt == 0 && errs) {
                double* r = errs + 8 * st;
                r[0] = err;
                r[1] = ex;
                r[2] = eg;
                r[3] = s_cstat[0].x;
                r[4] = s_cstat[1].x;
                r[5] = s_cstat[2].x;
                r[6] = hint;
                r[7] = 0.0;
            }
            gsync<TPT>(g);
            continue;
        }
        fill_formulas<TPT>(P, 1, 1 + P.n_formula, s_cstat, s_cdyn, s_tab, lt);
        gsync<TPT>(g);
        if constexpr (MIXED) {
            for (int f = lt; f < 1 + P.n_formula; f += TPT) s_tab32[f] = make_float2(static_cast<float>(s_tab[f].x), static_cast<float>(s_tab[f].y));
            for (int i = lt; i < U; i += TPT) s_G32[i] = make_float2(static_cast<float>(s_G[i].x), static_cast<float>(s_G[i].y));
            gsync<TPT>(g);
            gather_rhs<TPT, float, float2>(P, s_rec, s_out, s_tab32, s_G32, s_K32, lt);
            gsync<TPT>(g);
            for (int i = lt; i < N; i += TPT) dys[st * N + i] = static_cast<double>(s_K32[i]);
        } else {
            gather_rhs<TPT, double, double2>(P, s_rec, s_out, s_tab, s_G, s_K, lt);
            gsync<TPT>(g);
            for (int i = lt; i < N; i += TPT) dys[st * N + i] = s_K[i];
        }
        gsync<TPT>(g);
    }
}


// ------------------------------------------------------------------------------------------
// launchers: obe_instance.cu instantiates each kernel shape in a translation unit of its own,
// so the shapes compile in parallel; the host code only calls them.

template <int TPT, int EPT, bool MIXED>
cudaError_t launch_integrate_shape(const DevPlan& P, const CallArgs& A, int blocks, int gpb, size_t smem, size_t group_bytes,
                                   int method, cudaStream_t stream) {
    auto k = integrate_kernel<TPT, EPT, MIXED, false>;
    if constexpr (MIXED) {
        if (A.ctrl32) k = integrate_kernel<TPT, EPT, true, true>;
    }
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    k<<<blocks, gpb * TPT, smem, stream>>>(P, A, gpb, group_bytes, method);
    return cudaGetLastError();
}

template <int TPT, bool MIXED>
cudaError_t launch_rhs_shape(const DevPlan& P, long long count, const double* ts, const double* ys, int n_ov, const int* ov_slots,
                             const double* ov_vals, double* dys, int blocks, int gpb, size_t smem, size_t group_bytes,
                             int vm_depth, unsigned char* gscratch, size_t gstride, double* errs) {
    auto k = rhs_kernel<TPT, MIXED>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    k<<<blocks, gpb * TPT, smem>>>(P, count, ts, ys, n_ov, ov_slots, ov_vals, dys, gpb, group_bytes, vm_depth, gscratch, gstride,
                                   errs);
    return cudaGetLastError();
}

// the integrator shapes (threads per trajectory, elements per thread) and the RHS widths; the
// build compiles obe_instance.cu once per shape (centrex_tlf_gb300/build.py: SHAPES, RHS_SHAPES)
#define OBE_FOR_EACH_SHAPE(X) X(32, 8) X(32, 16) X(64, 4) X(64, 16) X(128, 2) X(128, 12) X(128, 16) X(256, 24) X(256, 32) X(512, 12) X(512, 16)
#define OBE_FOR_EACH_RHS(X) X(32) X(64) X(128) X(256) X(512)
#ifndef OBE_INSTANCE_TU
#define OBE_EXTERN_SHAPE(T, E)                                                                                          \
    extern template cudaError_t launch_integrate_shape<T, E, false>(const DevPlan&, const CallArgs&, int, int, size_t,   \
                                                                    size_t, int, cudaStream_t);                         \
    extern template cudaError_t launch_integrate_shape<T, E, true>(const DevPlan&, const CallArgs&, int, int, size_t,    \
                                                                   size_t, int, cudaStream_t);
#define OBE_EXTERN_RHS(T)                                                                                               \
    extern template cudaError_t launch_rhs_shape<T, false>(const DevPlan&, long long, const double*, const double*, int, \
                                                           const int*, const double*, double*, int, int, size_t, size_t, \
                                                           int, unsigned char*, size_t, double*);                        \
    extern template cudaError_t launch_rhs_shape<T, true>(const DevPlan&, long long, const double*, const double*, int,  \
                                                          const int*, const double*, double*, int, int, size_t, size_t,  \
                                                          int, unsigned char*, size_t, double*);
OBE_FOR_EACH_SHAPE(OBE_EXTERN_SHAPE)
OBE_FOR_EACH_RHS(OBE_EXTERN_RHS)
#undef OBE_EXTERN_SHAPE
#undef OBE_EXTERN_RHS
#endif

}  // namespace obe
