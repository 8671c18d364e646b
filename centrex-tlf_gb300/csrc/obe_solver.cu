// obe_solver.cu -- host side of the GB300 Lindblad solver: plan upload, option validation,
// launch planning, the batch/grid/single drivers and the C ABI of include/obe_gb300.h
// (rust/src/lindblad/python_api.rs:271-799, rust/src/lindblad/ode_batch.rs).  The kernels are in
// obe_kernels.cuh, instantiated per shape in obe_instance.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "obe_adjoint.cuh"
#include "obe_kernels.cuh"

namespace obe {

// ------------------------------------------------------------------------------------------
// host side

namespace {

thread_local long long g_launches = 0;

bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
    return false;
}

template <typename T>
size_t put(std::vector<unsigned char>& blob, const std::vector<T>& v) {
    size_t off = align16(blob.size());
    blob.resize(off + std::max<size_t>(v.size() * sizeof(T), 16));
    if (!v.empty()) std::memcpy(blob.data() + off, v.data(), v.size() * sizeof(T));
    return off;
}

int k1_refresh_interval() {
    // every 32 accepted steps: measured on the 4096-point 16-state scan, 8 -> 32 is 5 % faster
    // at a population error against FP64 of 4.3e-9 (8.7e-10 at 8; 9.7e-8 with no refresh)
    static const int v = [] {
        const char* env = std::getenv("OBE_K1_REFRESH");
        return env ? std::max(1, std::atoi(env)) : 32;
    }();
    return v;
}

// The plan's device image serialised into `blob` on the host, and the DevPlan whose pointers
// address that image once it sits at device address `base`.
void build_plan_image(const obe_plan* p, std::vector<unsigned char>& blob, uintptr_t base, DevPlan& P) {
    const HostPacked& h = p->packed;
    size_t o_op = put(blob, h.ins_op), o_arg = put(blob, h.ins_arg), o_fn = put(blob, h.ins_fn), o_val = put(blob, h.ins_val);
    size_t o_bv = put(blob, h.base_val), o_bt = put(blob, h.base_tuple), o_tp = put(blob, h.tuple_ptr), o_ti = put(blob, h.tuple_items);
    size_t o_cs = put(blob, h.comp_slot), o_ce = put(blob, h.comp_expr), o_cd = put(blob, h.comp_dynamic);
    size_t o_ke = put(blob, h.coeff_expr), o_kd = put(blob, h.coeff_dynamic), o_di = put(blob, h.dyn_ids), o_dp = put(blob, h.coeff_dyn_pos);
    size_t o_pp = put(blob, h.pchip_ptr), o_pg = put(blob, h.pchip_grid), o_pc = put(blob, h.pchip_coef), o_pcp = put(blob, h.pchip_cptr);
    size_t o_fp = put(blob, h.formula_ptr), o_pf = put(blob, h.prod_factor), o_pcl = put(blob, h.prod_class), o_pf32 = put(blob, h.prod_factor32);
    size_t o_rec = put(blob, h.rec), o_lo = put(blob, h.lane_out), o_fs = put(blob, h.fstream);
    size_t o_tr = put(blob, h.trec), o_li = put(blob, h.lane_in), o_bil = put(blob, h.bil);
    size_t o_eg = put(blob, h.eff_grid), o_er = put(blob, h.eff_rows), o_ec = put(blob, h.eff_cols), o_ef = put(blob, h.eff_coef);
    size_t o_ks = put(blob, h.coeff_scale);
    // the time-dependent compounds and coefficients, their instructions copied contiguously
    std::vector<DevExpr> vprog;
    std::vector<int32_t> vop, varg, vfn;
    std::vector<double> vval;
    auto add_prog = [&](const DevExpr& e, int32_t target) {
        DevExpr c{static_cast<int32_t>(vop.size()), e.len, e.real_ok, target};
        for (int32_t k = e.start; k < e.start + e.len; ++k) {
            vop.push_back(h.ins_op[k]);
            varg.push_back(h.ins_arg[k]);
            vfn.push_back(h.ins_fn[k]);
            vval.push_back(h.ins_val[2 * k]);
            vval.push_back(h.ins_val[2 * k + 1]);
        }
        vprog.push_back(c);
    };
    for (size_t c = 0; c < h.comp_slot.size(); ++c)
        if (h.comp_dynamic[c]) add_prog(h.comp_expr[c], h.comp_slot[c]);
    const int32_t n_vcomp = static_cast<int32_t>(vprog.size());
    for (size_t j = 0; j < h.dyn_ids.size(); ++j) add_prog(h.coeff_expr[h.dyn_ids[j]], static_cast<int32_t>(j));
    size_t o_vp = put(blob, vprog), o_vo = put(blob, vop), o_va = put(blob, varg), o_vf = put(blob, vfn), o_vv = put(blob, vval);
    P = DevPlan{};
    P.n_vcomp = n_vcomp;
    P.n_vprog = static_cast<int32_t>(vprog.size());
    P.n_vins = static_cast<int32_t>(vop.size());
    P.vprog = reinterpret_cast<const DevExpr*>(base + o_vp);
    P.vop = reinterpret_cast<const int32_t*>(base + o_vo);
    P.varg = reinterpret_cast<const int32_t*>(base + o_va);
    P.vfn = reinterpret_cast<const int32_t*>(base + o_vf);
    P.vval = reinterpret_cast<const double*>(base + o_vv);
    P.n = p->n;
    P.N = static_cast<int32_t>(p->N);
    P.U = static_cast<int32_t>(p->U);
    P.ins_op = reinterpret_cast<const int32_t*>(base + o_op);
    P.ins_arg = reinterpret_cast<const int32_t*>(base + o_arg);
    P.ins_fn = reinterpret_cast<const int32_t*>(base + o_fn);
    P.ins_val = reinterpret_cast<const double*>(base + o_val);
    P.n_slots = std::max(p->n_slots, h.n_vm_slots);
    P.n_base = p->n_base;
    P.dyn_real_closed = h.dyn_real_closed;
    P.trace_preserving = h.trace_preserving;
    P.coeff_scale = reinterpret_cast<const double*>(base + o_ks);
    P.base_val = reinterpret_cast<const double*>(base + o_bv);
    P.base_tuple = reinterpret_cast<const int32_t*>(base + o_bt);
    P.tuple_ptr = reinterpret_cast<const int32_t*>(base + o_tp);
    P.tuple_items = reinterpret_cast<const double*>(base + o_ti);
    P.n_comp = static_cast<int32_t>(h.comp_slot.size());
    P.comp_slot = reinterpret_cast<const int32_t*>(base + o_cs);
    P.comp_expr = reinterpret_cast<const DevExpr*>(base + o_ce);
    P.comp_dynamic = reinterpret_cast<const uint8_t*>(base + o_cd);
    P.n_coeff = p->n_coeff;
    P.coeff_expr = reinterpret_cast<const DevExpr*>(base + o_ke);
    P.coeff_dynamic = reinterpret_cast<const uint8_t*>(base + o_kd);
    P.n_dyn = static_cast<int32_t>(h.dyn_ids.size());
    P.dyn_ids = reinterpret_cast<const int32_t*>(base + o_di);
    P.coeff_dyn_pos = reinterpret_cast<const int32_t*>(base + o_dp);
    P.time_dependent = p->time_dependent;
    P.max_stack = std::max(1, h.max_stack);
    P.n_pchip = static_cast<int32_t>(h.pchip_cptr.size());
    P.pchip_ptr = reinterpret_cast<const int32_t*>(base + o_pp);
    P.pchip_grid = reinterpret_cast<const double*>(base + o_pg);
    P.pchip_coef = reinterpret_cast<const double*>(base + o_pc);
    P.pchip_cptr = reinterpret_cast<const int32_t*>(base + o_pcp);
    P.n_formula = h.n_formula;
    P.n_static_formula = h.n_static_formula;
    P.formula_ptr = reinterpret_cast<const int32_t*>(base + o_fp);
    P.prod_factor = reinterpret_cast<const double*>(base + o_pf);
    P.prod_class = reinterpret_cast<const int32_t*>(base + o_pcl);
    P.prod_factor32 = reinterpret_cast<const float*>(base + o_pf32);
    P.dyn_prod0 = h.formula_ptr.empty() ? 0 : h.formula_ptr[h.n_static_formula];
    P.n_dyn_prod = h.formula_ptr.empty() ? 0 : h.formula_ptr[h.n_formula] - P.dyn_prod0;
    P.tpt = h.tpt;
    P.n_iter = h.n_iter;
    P.rec = reinterpret_cast<const uint32_t*>(base + o_rec);
    P.n_out = h.n_out;
    P.lane_out = reinterpret_cast<const uint32_t*>(base + o_lo);
    P.n_fiter = h.n_fiter;
    P.fstream = reinterpret_cast<const uint32_t*>(base + o_fs);
    P.n_titer = h.n_titer;
    P.trec = reinterpret_cast<const uint32_t*>(base + o_tr);
    P.n_tin = h.n_tin;
    P.lane_in = reinterpret_cast<const uint32_t*>(base + o_li);
    P.n_biter = h.n_biter;
    P.bil = reinterpret_cast<const uint32_t*>(base + o_bil);
    P.pop_stride = h.pop_stride;
    P.eff = h.eff;
    P.eff_ngrid = static_cast<int32_t>(h.eff_grid.size());
    P.eff_grid = reinterpret_cast<const double*>(base + o_eg);
    P.eff_rows = reinterpret_cast<const int32_t*>(base + o_er);
    P.eff_cols = reinterpret_cast<const int32_t*>(base + o_ec);
    P.eff_coef = reinterpret_cast<const double*>(base + o_ef);
    for (int k = 0; k < 3; ++k) {
        P.eff_nnz[k] = h.eff_nnz[k];
        P.eff_col_off[k] = h.eff_col_off[k];
        P.eff_coef_off[k] = h.eff_coef_off[k];
    }
}

obe_status upload_plan(obe_plan* p) {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return OBE_ERR_CUDA;
    if (p->d_blob && p->d_device == dev) return OBE_OK;
    if (p->d_blob) {
        cudaFree(p->d_blob);
        p->d_blob = nullptr;
    }
    std::vector<unsigned char> blob;
    DevPlan P;
    build_plan_image(p, blob, 0, P);  // sizes only
    void* d = nullptr;
    if (!cuda_ok(cudaMalloc(&d, blob.size()), "cudaMalloc(plan)")) return OBE_ERR_CUDA;
    blob.clear();
    build_plan_image(p, blob, reinterpret_cast<uintptr_t>(d), P);
    if (!cuda_ok(cudaMemcpy(d, blob.data(), blob.size(), cudaMemcpyHostToDevice), "cudaMemcpy(plan)")) {
        cudaFree(d);
        return OBE_ERR_CUDA;
    }
    p->dev = P;
    p->d_blob = d;
    p->d_device = dev;
    ++p->image_gen;
    return OBE_OK;
}

// grow-only device scratch of a plan
obe_status scratch(obe_plan* p, size_t bytes, unsigned char** out) {
    if (p->scratch_bytes < bytes) {
        if (p->d_scratch) cudaFree(p->d_scratch);
        p->d_scratch = nullptr;
        p->scratch_bytes = 0;
        size_t want = std::max<size_t>(bytes, 1 << 20);
        if (!cuda_ok(cudaMalloc(&p->d_scratch, want), "cudaMalloc(scratch)")) return OBE_ERR_CUDA;
        p->scratch_bytes = want;
    }
    *out = static_cast<unsigned char*>(p->d_scratch);
    return OBE_OK;
}

// elements per thread of the compiled shape of a width (OBE_FOR_EACH_SHAPE), the fewest that
// hold the state: 8 or 16 at 32 threads, 4 or 16 at 64, 2, 12 or 16 at 128, 24 or 32 at 256,
// 12 or 16 at 512 (a 76-state system: 5,776 elements, 24 per thread at 256 threads, 12 at 512)
int ept_for(int N, int tpt) {
    // OBE_EPT_WIDE=1: the widest compiled count of every width (runs those shapes on systems a
    // tighter one would take; read at every launch)
    if (const char* env = std::getenv("OBE_EPT_WIDE"); env && env[0] && env[0] != '0') return tpt == 256 ? 32 : 16;
    if (tpt == 32) return N <= 32 * 8 ? 8 : 16;
    if (tpt == 256) return N <= 256 * 24 ? 24 : 32;
    if (tpt == 512) return N <= 512 * 12 ? 12 : 16;
    // the compact shapes of a small system at a wide launch (latency-bound single solves): two or
    // four elements per thread instead of sixteen mostly idle ones
    if (tpt == 64 && N <= 64 * 4) return 4;
    if (tpt == 128 && N <= 128 * 2) return 2;
    if (tpt == 128 && N <= 128 * 12) return 12;
    return 16;
}

struct LaunchShape {
    int tpt, ept, gpb, blocks;
    size_t group_bytes, smem;
    size_t gstride;  // large systems: global stage-buffer bytes per group (0 otherwise)
    int vm_smem = 0; // the time-dependent programs staged in shared memory (CallArgs::vm_smem)
};

// grow-only global stage-buffer scratch of a plan (large systems)
obe_status kscratch(obe_plan* p, size_t bytes, unsigned char** out) {
    if (p->gk_bytes < bytes) {
        if (p->d_gk) cudaFree(p->d_gk);
        p->d_gk = nullptr;
        p->gk_bytes = 0;
        if (!cuda_ok(cudaMalloc(&p->d_gk, bytes), "cudaMalloc(stage buffers)")) return OBE_ERR_CUDA;
        p->gk_bytes = bytes;
    }
    *out = static_cast<unsigned char*>(p->d_gk);
    return OBE_OK;
}

// ---- cost-ordered launches ---------------------------------------------------------------
// A persistent launch pulls trajectories from a queue; in index order the launch lasts until its
// slowest warp has worked through whichever trajectories it happened to pull, and the long ones
// pulled last set that time (on the 16-state scan's 4096 points the makespan is 1.56x the
// evenly shared work).  The queue is therefore ordered longest-first by a cost estimate made from
// the inputs alone (no solve): the integral over the solve's time span of the Hamiltonian's
// coefficient magnitude, sqrt(sum_k (|c_k(t)| s_k)^2) with s_k the largest factor of the terms
// coefficient k multiplies (the generalised Rabi frequency of a driven transition), sampled at
// kCostSamples times and cut at a runtime-expression stop event's first sign change (the ragged
// end times).  Steps of an explicit adaptive solver scale with that phase; the order is a counting
// sort into kOrderBuckets logarithmic buckets (longest first; within a bucket in any order).  The
// results do not depend on the order: every trajectory's arithmetic is its own.
constexpr int kCostSamples = 32;
constexpr int kOrderBuckets = 1024;

__global__ void __launch_bounds__(128) cost_kernel(const DevPlan P, const CallArgs A, float* cost, unsigned int* range) {
    const long long traj = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (traj >= A.n_traj) return;
    double2 slots[kMaxSlots], stk[kMaxStack];
    int32_t tup[kMaxStack];
    VMLane L;
    L.slots = slots;
    L.stack.v = stk;
    L.stack.tup = tup;
    L.real = false;
    init_slots(P, A, traj, slots);
    eval_compounds(P, L, A.t0, false);
    bool real = P.dyn_real_closed != 0;
    for (int i = 0; i < P.n_slots && real; ++i) real = slots[i].y == 0.0;
    L.real = real;
    double w0 = 0.0;
    for (int k = 0; k < P.n_coeff; ++k) {
        if (P.coeff_dynamic[k]) continue;
        const double2 c = eval_expr(P, P.coeff_expr[k], L, A.t0);
        const double a = hypot(c.x, c.y) * P.coeff_scale[k];
        w0 += a * a;
    }
    const bool ev = A.ev_kind == OBE_EVENT_EXPRESSION && A.ev_len > 0;
    double g0 = 0.0;
    if (ev) g0 = vm_eval(P, A.ev_op, A.ev_arg, A.ev_fn, A.ev_val, 0, A.ev_len, L.slots, A.t0, L.stack).x;
    const double dt = (A.t1 - A.t0) / kCostSamples;
    double c = 0.0, span = 0.0;
    for (int q = 0; q < kCostSamples; ++q) {
        const double t = A.t0 + (q + 0.5) * dt;
        if (P.n_dyn > 0 || ev) eval_compounds(P, L, t, true);
        if (ev) {
            const double gq = vm_eval(P, A.ev_op, A.ev_arg, A.ev_fn, A.ev_val, 0, A.ev_len, L.slots, t, L.stack).x;
            if ((g0 < 0.0 && gq >= 0.0) || (g0 > 0.0 && gq <= 0.0)) break;
        }
        double w = w0;
        for (int j = 0; j < P.n_dyn; ++j) {
            const double2 cv = eval_expr(P, P.coeff_expr[P.dyn_ids[j]], L, t);
            const double a = hypot(cv.x, cv.y) * P.coeff_scale[P.dyn_ids[j]];
            w += a * a;
        }
        c += sqrt(w) * dt;
        span += dt;
    }
    // a trajectory without a drive still orders by the length of its span
    c += 1e-9 * span / (A.t1 - A.t0);
    const float cf = isfinite(c) && c > 1e-30 ? static_cast<float>(c) : 1e-30f;
    cost[traj] = cf;
    atomicMin(&range[0], __float_as_uint(cf));  // positive floats order like their bit patterns
    atomicMax(&range[1], __float_as_uint(cf));
}

__device__ __forceinline__ int cost_bucket(float c, const unsigned int* range) {
    const float lo = logf(__uint_as_float(range[0])), hi = logf(__uint_as_float(range[1]));
    if (!(hi > lo)) return 0;
    const int b = static_cast<int>((hi - logf(c)) / (hi - lo) * (kOrderBuckets - 1) + 0.5f);
    return b < 0 ? 0 : (b >= kOrderBuckets ? kOrderBuckets - 1 : b);
}

__global__ void order_histogram_kernel(long long n, const float* cost, const unsigned int* range, unsigned int* hist) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&hist[cost_bucket(cost[i], range)], 1u);
}

// exclusive scan of the bucket counts into bucket offsets, one thread (kOrderBuckets adds)
__global__ void order_scan_kernel(unsigned int* hist) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned int run = 0;
    for (int b = 0; b < kOrderBuckets; ++b) {
        const unsigned int c = hist[b];
        hist[b] = run;
        run += c;
    }
}

__global__ void order_scatter_kernel(long long n, const float* cost, const unsigned int* range, unsigned int* off,
                                     long long* order) {
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) order[atomicAdd(&off[cost_bucket(cost[i], range)], 1u)] = i;
}

bool ordering_enabled() {
    static const bool on = [] {
        const char* env = std::getenv("OBE_ORDER");
        return !(env && env[0] == '0');
    }();
    return on;
}

// Fills A.order with the longest-first queue of this launch on `stream` (4 small kernels), from a
// grow-only per-plan buffer; returns the number of launches issued.
obe_status order_queue(obe_plan* p, CallArgs& A, cudaStream_t stream, int* launches) {
    const long long n = A.n_traj;
    const size_t o_ord = 0, o_cost = align16(static_cast<size_t>(n) * 8), o_hist = align16(o_cost + static_cast<size_t>(n) * 4);
    const size_t o_rng = o_hist + kOrderBuckets * 4, bytes = align16(o_rng + 8);
    if (p->ord_bytes < bytes) {
        if (p->d_ord) cudaFree(p->d_ord);
        p->d_ord = nullptr;
        p->ord_bytes = 0;
        if (!cuda_ok(cudaMalloc(&p->d_ord, bytes), "cudaMalloc(queue order)")) return OBE_ERR_CUDA;
        p->ord_bytes = bytes;
    }
    unsigned char* b = static_cast<unsigned char*>(p->d_ord);
    long long* order = reinterpret_cast<long long*>(b + o_ord);
    float* cost = reinterpret_cast<float*>(b + o_cost);
    unsigned int* hist = reinterpret_cast<unsigned int*>(b + o_hist);
    unsigned int* range = reinterpret_cast<unsigned int*>(b + o_rng);
    if (!cuda_ok(cudaMemsetAsync(hist, 0, kOrderBuckets * 4 + 8, stream), "cudaMemsetAsync(order)")) return OBE_ERR_CUDA;
    if (!cuda_ok(cudaMemsetAsync(range, 0xFF, 4, stream), "cudaMemsetAsync(order)")) return OBE_ERR_CUDA;
    const unsigned int blocks = static_cast<unsigned int>((n + 127) / 128);
    cost_kernel<<<blocks, 128, 0, stream>>>(p->dev, A, cost, range);
    order_histogram_kernel<<<blocks, 128, 0, stream>>>(n, cost, range, hist);
    order_scan_kernel<<<1, 32, 0, stream>>>(hist);
    order_scatter_kernel<<<blocks, 128, 0, stream>>>(n, cost, range, hist, order);
    if (!cuda_ok(cudaGetLastError(), "order kernels")) return OBE_ERR_CUDA;
    A.order = order;
    *launches = 4;
    return OBE_OK;
}

template <bool MIXED>
cudaError_t dispatch_shape(const DevPlan& P, const CallArgs& A0, const LaunchShape& s, int method, cudaStream_t st) {
    CallArgs A = A0;
    A.vm_smem = s.vm_smem;
#define OBE_DISPATCH(T, E) \
    if (s.tpt == T && s.ept == E) return launch_integrate_shape<T, E, MIXED>(P, A, s.blocks, s.gpb, s.smem, s.group_bytes, method, st);
    OBE_FOR_EACH_SHAPE(OBE_DISPATCH)
#undef OBE_DISPATCH
    return cudaErrorInvalidConfiguration;
}

int sm_count() {
    static const int count = [] {
        int dev = 0, c = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
        return c > 0 ? c : 1;
    }();
    return count;
}

// gpb_fixed > 0: that many trajectories per CTA (at most what fits), else the automatic choice
obe_status plan_launch(const DevPlan& P, bool mixed, long long n_traj, int vm_depth, LaunchShape* s, int gpb_fixed = 0) {
    s->tpt = P.tpt;
    if (s->tpt > 512) {
        set_error("systems with more than 90 states are not supported by this build of the GPU solver");
        return OBE_ERR_UNSUPPORTED;
    }
    s->ept = ept_for(P.N, s->tpt);
    struct { size_t bytes; } L;
    const GroupLayout GL = group_layout(P.n, P.N, P.n_formula, P.n_coeff, P.n_dyn, P.n_slots, vm_depth, s->tpt, mixed);
    L.bytes = GL.bytes;
    s->group_bytes = L.bytes;
    s->gstride = GL.gbytes;
    size_t plan_bytes = plan_smem(P, s->tpt, mixed).bytes;
    const size_t limit = 227 * 1024;
    int gpb = std::max(1, (mixed ? kThreadsMixed : kThreadsFp64) / s->tpt);
    while (gpb > 1 && plan_bytes + gpb * L.bytes > limit) --gpb;
    if (plan_bytes + gpb * L.bytes > limit) {
        set_error("system too large for the GPU solver's shared-memory layout");
        return OBE_ERR_UNSUPPORTED;
    }
    if (gpb_fixed > 0) {
        gpb = std::min(gpb, gpb_fixed);
    } else {
        // fewer groups per CTA when the batch is small, so that every SM gets work
        long long per_sm = (n_traj + sm_count() - 1) / sm_count();
        while (gpb > 1 && gpb > per_sm) --gpb;
    }
    s->gpb = gpb;
    s->smem = plan_bytes + gpb * L.bytes;
    // the time-dependent programs in shared memory too, when that costs no trajectory group and
    // no resident CTA
    const size_t plan_vm = plan_smem(P, s->tpt, mixed, true).bytes;
    if (P.n_vprog > 0 && plan_vm + gpb * L.bytes <= limit && limit / (plan_vm + gpb * L.bytes) >= limit / s->smem) {
        s->vm_smem = 1;
        s->smem = plan_vm + gpb * L.bytes;
    }
    int blocks_per_sm = std::max<int>(1, static_cast<int>(limit / s->smem));
    long long want = (n_traj + gpb - 1) / gpb;
    long long cap = static_cast<long long>(sm_count()) * blocks_per_sm;
    s->blocks = static_cast<int>(std::max<long long>(1, std::min(want, cap)));
    return OBE_OK;
}

// Host-side save plan (common.rs:124-151).
obe_status save_plan(const obe_solve_options* o, std::vector<double>& times) {
    times.clear();
    if (!o->has_saveat) return OBE_OK;
    auto tol = [](double t) { return 10.0 * 2.220446049250313e-16 * std::fmax(std::fabs(t), 1.0); };
    if (o->save_start) times.push_back(o->t0);
    for (int64_t i = 0; i < o->n_saveat; ++i) {
        double t = o->saveat[i];
        if (o->save_start && std::fabs(t - o->t0) <= tol(o->t0)) continue;
        if (!std::isfinite(t)) {
            set_error("saveat contains non-finite value");
            return OBE_ERR_INVALID;
        }
        if (t < o->t0 - tol(o->t0) || t > o->t1 + tol(o->t1)) {
            set_error("saveat value " + fmt_f64(t) + " is outside [" + fmt_f64(o->t0) + ", " + fmt_f64(o->t1) + "]");
            return OBE_ERR_INVALID;
        }
        times.push_back(t);
    }
    return OBE_OK;
}

int64_t packed_upper_real_index(int32_t n, int64_t i, int64_t j) {
    int64_t off = 0;
    for (int64_t r = 0; r < i; ++r) off += n - r - 1;
    return n + 2 * (off + (j - i - 1));
}

// Rust's `{:.6e}` (six decimals, exponent without sign padding: 1.000000e2, -3.500000e-1)
std::string fmt_rust_exp6(double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.6e", v);
    char* ep = std::strchr(buf, 'e');
    if (!ep) return buf;
    const int ex = std::atoi(ep + 1);
    *ep = 0;
    return std::string(buf) + "e" + std::to_string(ex);
}

// effective_lindblad/rhs.rs:56-67
std::string field_range_message(bool above, double x, double bound) {
    return "field coordinate " + fmt_rust_exp6(x) + (above ? " is above the operator grid maximum " : " is below the operator grid minimum ") +
           fmt_rust_exp6(bound);
}

std::string traj_message(int code, const TrajErr& e) {
    switch (code) {
    case ST_MAXITERS: return "Stopped at x=" + fmt_f64(e.x) + ". Need more than " + std::to_string(e.a) + " steps.";
    case ST_UNDERFLOW: return "Stopped at x=" + fmt_f64(e.x) + ". Step size underflow.";
    case ST_STIFF: return "Stiff at x=" + fmt_f64(e.x) + ".";
    case ST_SAVEAT: return "ended before all saveat: " + std::to_string(e.a) + " of " + std::to_string(e.b);
    case ST_EVENT_COMPLEX: return "event expression evaluated to a complex value";
    case ST_EVENT_INDEX: return "population event index out of bounds";
    case ST_POINTS: return "expected " + std::to_string(e.a) + " output points, got " + std::to_string(e.b);
    case ST_BAD_MAXITERS: return "maxiters must be positive";
    case ST_BACKWARD: return "only forward integration";
    case ST_FIXED_DT: return "fixed-step solvers require positive finite dt";
    case ST_TAPE: return "the gradient tape holds " + std::to_string(e.a) + " accepted steps per trajectory; pass a larger max_steps";
    case ST_FIELD_LOW: case ST_FIELD_HIGH: {
        double g;
        std::memcpy(&g, &e.a, sizeof g);
        return field_range_message(code == ST_FIELD_HIGH, e.x, g);
    }
    default: return "trajectory failed with status " + std::to_string(code);
    }
}

// the mixed integrator (either control precision) runs the solve
inline bool is_mixed(int32_t precision) {
    return precision == OBE_PRECISION_MIXED || precision == OBE_PRECISION_MIXED_FP32_CONTROL;
}

// Everything a solve needs on the device besides the plan: the per-call blob of small arrays.
struct CallBlob {
    std::vector<unsigned char> bytes;
    size_t o_save = 0, o_widx = 0, o_wval = 0, o_sre = 0, o_sim = 0, o_skind = 0, o_evidx = 0, o_evop = 0, o_evarg = 0, o_evfn = 0, o_evval = 0;
    int ev_len = 0;
};

obe_status validate_options(const obe_plan* p, const obe_solve_options* o, std::vector<double>& save_times, CallBlob& cb,
                            int64_t* width_out, int* is_complex) {
    const bool eff = p->packed.eff != 0;
    if (o->precision != OBE_PRECISION_FP64 && !is_mixed(o->precision)) {
        set_error("precision must be 'fp64', 'mixed' or 'mixed_fp32_control'");
        return OBE_ERR_INVALID;
    }
    if (eff && is_mixed(o->precision)) {
        set_error("effective-Hamiltonian plans solve in double precision");
        return OBE_ERR_UNSUPPORTED;
    }
    if (eff && o->event_kind != OBE_EVENT_NONE) {
        set_error("effective-Hamiltonian solves take no stop event");
        return OBE_ERR_UNSUPPORTED;
    }
    if (!p->has_expanded && !eff) {
        set_error("execution_mode='expanded_sparse' requires a decomposed Hamiltonian plan");
        return OBE_ERR_INVALID;
    }
    if (o->solver < OBE_SOLVER_DOPRI5 || o->solver > OBE_SOLVER_FIXED_RK4) {
        set_error("solver must be 'dopri5', 'tsit5', 'fixed_dopri5', 'fixed_rk2', or 'fixed_rk4'");
        return OBE_ERR_INVALID;
    }
    if (o->solver >= OBE_SOLVER_FIXED_DOPRI5 && is_mixed(o->precision)) {
        set_error("precision='mixed' is implemented for the adaptive solvers 'dopri5' and 'tsit5'");
        return OBE_ERR_UNSUPPORTED;
    }
    obe_status st = save_plan(o, save_times);
    if (st != OBE_OK) return st;
    int64_t width = 0;
    *is_complex = 0;
    std::vector<int32_t> widx, sre, sim, skind, evidx;
    std::vector<double> wval;
    switch (o->output) {
    case OBE_OUTPUT_POPULATIONS: width = p->n; break;
    case OBE_OUTPUT_FULL: width = p->N; break;
    case OBE_OUTPUT_SELECTED:
        width = o->n_selected;
        *is_complex = 1;
        if (o->n_selected > kMaxSelected) { set_error("too many selected outputs for the GPU solver"); return OBE_ERR_UNSUPPORTED; }
        for (int k = 0; k < o->n_selected; ++k) {
            int64_t i = o->selected_i[k], j = o->selected_j[k];
            if (i < 0 || j < 0 || i >= p->n || j >= p->n) { set_error("selected output index out of bounds"); return OBE_ERR_INVALID; }
            if (eff) {
                // split_real_selected_extractions (effective_lindblad/solver.rs:58-76)
                const int64_t nn = p->n;
                sre.push_back(static_cast<int32_t>(i * nn + j));
                sim.push_back(static_cast<int32_t>(i == j ? i * nn + j : nn * nn + i * nn + j));
                skind.push_back(i == j ? 0 : 1);
                continue;
            }
            if (i == j) { sre.push_back(static_cast<int32_t>(i)); sim.push_back(static_cast<int32_t>(i)); skind.push_back(0); }
            else if (i < j) { int64_t r = packed_upper_real_index(p->n, i, j); sre.push_back(static_cast<int32_t>(r)); sim.push_back(static_cast<int32_t>(r + 1)); skind.push_back(1); }
            else { int64_t r = packed_upper_real_index(p->n, j, i); sre.push_back(static_cast<int32_t>(r)); sim.push_back(static_cast<int32_t>(r + 1)); skind.push_back(2); }
        }
        break;
    case OBE_OUTPUT_WEIGHTED_INTEGRAL:
    case OBE_OUTPUT_WEIGHTED_RATE:
        width = 1;
        if (o->n_weights > kMaxWeights) { set_error("too many integral weights for the GPU solver"); return OBE_ERR_UNSUPPORTED; }
        for (int k = 0; k < o->n_weights; ++k) {
            if (o->weight_index[k] < 0 || o->weight_index[k] >= p->N) { set_error("integral weight index out of bounds"); return OBE_ERR_INVALID; }
            widx.push_back(static_cast<int32_t>(o->weight_index[k]));
            wval.push_back(o->weight_value[k]);
        }
        break;
    default: set_error("unknown output mode"); return OBE_ERR_INVALID;
    }
    *width_out = width;
    std::vector<int32_t> evop, evarg, evfn;
    std::vector<double> evval;
    if (o->event_kind == OBE_EVENT_POPULATION) {
        if (o->n_event_indices > kMaxEventIdx) { set_error("too many population event indices"); return OBE_ERR_UNSUPPORTED; }
        for (int k = 0; k < o->n_event_indices; ++k) evidx.push_back(static_cast<int32_t>(o->event_indices[k]));
    } else if (o->event_kind == OBE_EVENT_EXPRESSION) {
        // kind-check the event program with the plan's slot kinds and keep it in the call blob
        const obe_expr& e = o->event_expr;
        for (int64_t k = 0; k < e.n_instr; ++k) {
            int32_t op = e.op[k];
            if (op == OP_TEMP || op < 1 || op > 19) { set_error("unsupported instruction in stop_event expression"); return OBE_ERR_UNSUPPORTED; }
            if (op == OP_SLOT && (e.index[k] < 0 || e.index[k] >= p->n_slots)) { set_error("stop_event slot index out of bounds"); return OBE_ERR_INVALID; }
            if (op == OP_SLOT && e.index[k] < p->n_base && p->base_is_tuple[e.index[k]]) {
                set_error("tuple-valued stop_event operands are not supported by the GPU solver");
                return OBE_ERR_UNSUPPORTED;
            }
            if (op == OP_HELPER && (e.function[k] == 8 || e.function[k] == 10 || e.function[k] == 14 || e.function[k] == 16)) {
                set_error("tuple helpers in stop_event expressions are not supported by the GPU solver");
                return OBE_ERR_UNSUPPORTED;
            }
            evop.push_back(op);
            evarg.push_back(op == OP_SLOT ? static_cast<int32_t>(e.index[k]) : (e.argc ? e.argc[k] : 0));
            evfn.push_back(e.function ? e.function[k] : 0);
            evval.push_back(e.value ? e.value[2 * k] : 0.0);
            evval.push_back(e.value ? e.value[2 * k + 1] : 0.0);
        }
        if (e.n_instr > kMaxStack) { set_error("stop_event expression too long for the GPU solver"); return OBE_ERR_UNSUPPORTED; }
        cb.ev_len = static_cast<int>(e.n_instr);
    }
    cb.o_save = put(cb.bytes, save_times);
    cb.o_widx = put(cb.bytes, widx);
    cb.o_wval = put(cb.bytes, wval);
    cb.o_sre = put(cb.bytes, sre);
    cb.o_sim = put(cb.bytes, sim);
    cb.o_skind = put(cb.bytes, skind);
    cb.o_evidx = put(cb.bytes, evidx);
    cb.o_evop = put(cb.bytes, evop);
    cb.o_evarg = put(cb.bytes, evarg);
    cb.o_evfn = put(cb.bytes, evfn);
    cb.o_evval = put(cb.bytes, evval);
    return OBE_OK;
}

void fill_call_args(CallArgs& A, const obe_solve_options* o, const std::vector<double>& save_times, const CallBlob& cb,
                    const unsigned char* d_blob) {
    std::memset(&A, 0, sizeof A);
    A.t0 = o->t0;
    A.t1 = o->t1;
    A.atol = o->abstol;
    A.rtol = o->reltol;
    A.dt = o->dt;
    A.maxiters = o->maxiters;
    A.save_start = o->save_start;
    A.has_saveat = o->has_saveat;
    A.n_save = static_cast<int>(save_times.size());
    A.save_times = reinterpret_cast<const double*>(d_blob + cb.o_save);
    A.output = o->output;
    A.store_trace = o->store_trace;
    A.n_weights = o->output == OBE_OUTPUT_WEIGHTED_INTEGRAL || o->output == OBE_OUTPUT_WEIGHTED_RATE ? o->n_weights : 0;
    A.w_idx = reinterpret_cast<const int*>(d_blob + cb.o_widx);
    A.w_val = reinterpret_cast<const double*>(d_blob + cb.o_wval);
    A.n_sel = o->output == OBE_OUTPUT_SELECTED ? o->n_selected : 0;
    A.sel_re = reinterpret_cast<const int*>(d_blob + cb.o_sre);
    A.sel_im = reinterpret_cast<const int*>(d_blob + cb.o_sim);
    A.sel_kind = reinterpret_cast<const int*>(d_blob + cb.o_skind);
    A.ev_kind = o->event_kind;
    A.n_ev = o->event_kind == OBE_EVENT_POPULATION ? o->n_event_indices : 0;
    A.ev_idx = reinterpret_cast<const int*>(d_blob + cb.o_evidx);
    A.ev_thr = o->event_threshold;
    A.ev_len = cb.ev_len;
    A.ev_op = reinterpret_cast<const int32_t*>(d_blob + cb.o_evop);
    A.ev_arg = reinterpret_cast<const int32_t*>(d_blob + cb.o_evarg);
    A.ev_fn = reinterpret_cast<const int32_t*>(d_blob + cb.o_evfn);
    A.ev_val = reinterpret_cast<const double*>(d_blob + cb.o_evval);
    A.fixed = o->solver >= OBE_SOLVER_FIXED_DOPRI5 ? o->solver : 0;
    A.ctrl32 = o->precision == OBE_PRECISION_MIXED_FP32_CONTROL ? 1 : 0;
    A.vm_smem = 0;  // set per launch shape (dispatch_shape)
}

cudaError_t launch_integrate(const obe_plan* p, const CallArgs& A, bool mixed, int solver, const LaunchShape& s, cudaStream_t st) {
    const int method = solver == OBE_SOLVER_TSIT5 ? 1 : 0;
    return mixed ? dispatch_shape<true>(p->dev, A, s, method, st) : dispatch_shape<false>(p->dev, A, s, method, st);
}

obe_status check_params(const obe_plan* p, int32_t n_param, const int64_t* slots) {
    if (n_param > kMaxParams) {
        set_error("too many scanned parameter slots for the GPU solver");
        return OBE_ERR_UNSUPPORTED;
    }
    for (int k = 0; k < n_param; ++k) {
        if (slots[k] < 0 || slots[k] >= p->n_base) {
            set_error("parameter override slot " + std::to_string(slots[k]) + " is not a base parameter slot");
            return OBE_ERR_TRAJECTORY;
        }
        if (p->base_is_tuple[slots[k]]) {
            set_error("scanning a tuple-valued parameter is not supported by the GPU solver");
            return OBE_ERR_UNSUPPORTED;
        }
    }
    return OBE_OK;
}

// Common device path: everything already on the device except the call blob, which goes into
// the front of the plan's scratch.  Stats and errors land in d_stats / d_errs.
obe_status solve_device(obe_plan* p, const obe_solve_options* o, long long n_traj, const double* d_rho0, long long rho0_stride,
                        int32_t n_param, const int64_t* param_slots, const double* d_param_values, int n_axes,
                        const int64_t* axis_len, const double* d_axes, long long cap, long long out_stride, double* d_values,
                        double* d_times, obe_traj_stats* d_stats, TrajErr* d_errs, unsigned char* d_blob_area,
                        const CallBlob& cb, const std::vector<double>& save_times, unsigned long long* d_counter,
                        cudaStream_t stream, double* d_tape = nullptr, long long tape_cap = 0, long long tape_stride = 0,
                        int tape_ckpt = 0, unsigned char* d_gscratch = nullptr) {
    CallArgs A;
    fill_call_args(A, o, save_times, cb, d_blob_area);
    A.n_traj = n_traj;
    A.rho0 = d_rho0;
    A.rho0_stride = rho0_stride;
    A.n_param = n_param;
    for (int k = 0; k < n_param; ++k) A.param_slot[k] = static_cast<int>(param_slots[k]);
    A.param_values = d_param_values;
    A.n_axes = n_axes;
    if (n_axes > 0) {
        long long off = 0, stride = 1;
        for (int k = n_axes - 1; k >= 0; --k) { A.axis_stride[k] = stride; stride *= axis_len[k]; }
        for (int k = 0; k < n_axes; ++k) { A.axis_len[k] = axis_len[k]; A.axis_off[k] = off; off += axis_len[k]; }
    }
    A.axes = d_axes;
    A.cap = cap;
    A.out_stride = out_stride;
    A.values = d_values;
    A.times = d_times;
    A.stats = d_stats;
    A.errs = d_errs;
    A.counter = d_counter;
    A.k1_refresh = k1_refresh_interval();
    A.vm_depth = std::max(p->dev.max_stack, std::max(cb.ev_len, 1));
    A.tape = d_tape;
    A.tape_cap = tape_cap;
    A.tape_stride = tape_stride;
    A.tape_ckpt = tape_ckpt;
    LaunchShape s;
    obe_status st = plan_launch(p->dev, is_mixed(o->precision), n_traj, A.vm_depth, &s, p->shape_gpb);
    if (st != OBE_OK) return st;
    if (s.gstride > 0) {
        // the large systems' per-trajectory stage buffers: the caller's (a recorded graph owns its
        // own) or the plan's grow-only scratch
        unsigned char* gk = d_gscratch;
        if (!gk && (st = kscratch(p, s.gstride * static_cast<size_t>(s.blocks) * s.gpb, &gk)) != OBE_OK) return st;
        A.gscratch = gk;
        A.gstride = s.gstride;
    }
    if (!cuda_ok(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), stream), "cudaMemsetAsync")) return OBE_ERR_CUDA;
    // longest-first queue when the batch runs in more than one wave (not while a graph records:
    // the order's buffer may have to grow)
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    if (!cuda_ok(cudaStreamIsCapturing(stream, &cap_status), "cudaStreamIsCapturing")) return OBE_ERR_CUDA;
    if (ordering_enabled() && !p->packed.eff && cap_status == cudaStreamCaptureStatusNone &&
        n_traj > static_cast<long long>(s.blocks) * s.gpb) {
        int n_order = 0;
        if ((st = order_queue(p, A, stream, &n_order)) != OBE_OK) return st;
        g_launches += n_order;
    }
    if (!cuda_ok(launch_integrate(p, A, is_mixed(o->precision), o->solver, s, stream), "kernel launch")) return OBE_ERR_CUDA;
    g_launches += 1;
    return OBE_OK;
}

// Holds the mutexes of several plans, taken in address order (every caller uses that order,
// so two multi-plan calls cannot deadlock); duplicates are taken once.
class PlanLocks {
  public:
    template <typename It>
    PlanLocks(It first, It last) : plans_(first, last) {
        std::sort(plans_.begin(), plans_.end());
        plans_.erase(std::unique(plans_.begin(), plans_.end()), plans_.end());
        for (obe_plan* p : plans_) p->mu.lock();
    }
    ~PlanLocks() {
        for (auto it = plans_.rbegin(); it != plans_.rend(); ++it) (*it)->mu.unlock();
    }
    PlanLocks(const PlanLocks&) = delete;
    PlanLocks& operator=(const PlanLocks&) = delete;

  private:
    std::vector<obe_plan*> plans_;
};

}  // namespace
}  // namespace obe

using namespace obe;

struct obe_result {
    std::vector<double> times, values;
    int64_t width = 0;
    int32_t is_complex = 0;
    obe_traj_stats stats{};
};

extern "C" {

int32_t obe_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int64_t obe_last_launch_count(void) { return g_launches; }

void obe_plan_destroy(obe_plan* plan) {
    if (!plan) return;
    if (plan->d_blob) cudaFree(plan->d_blob);
    if (plan->d_scratch) cudaFree(plan->d_scratch);
    if (plan->d_gk) cudaFree(plan->d_gk);
    if (plan->d_ord) cudaFree(plan->d_ord);
    if (plan->d_counter) cudaFree(plan->d_counter);
    delete plan;
}

static obe_status ensure_ready(obe_plan* p) {
    if (obe_device_count() <= 0) {
        set_error("no CUDA device is available: the GB300 solver has no CPU fallback");
        return OBE_ERR_CUDA;
    }
    obe_status st = upload_plan(p);
    if (st != OBE_OK) return st;
    if (!p->d_counter && !cuda_ok(cudaMalloc(&p->d_counter, 64), "cudaMalloc(counter)")) return OBE_ERR_CUDA;
    return OBE_OK;
}

static obe_status solve_batch_device_locked(obe_plan* p, const obe_solve_options* opt, int64_t n_traj, const double* d_rho0,
                                            int32_t n_param_slots, const int64_t* param_slots, const double* d_param_values,
                                            int64_t time_count, int64_t width, double* d_values, obe_traj_stats* d_stats,
                                            void* stream);

obe_status obe_solve_batch_device(const obe_plan* plan_c, const obe_solve_options* opt, int64_t n_traj, const double* d_rho0,
                                  int32_t n_param_slots, const int64_t* param_slots, const double* d_param_values,
                                  int64_t time_count, int64_t width, double* d_values, obe_traj_stats* d_stats, void* stream) {
    g_launches = 0;
    obe_plan* p = const_cast<obe_plan*>(plan_c);
    if (!p || !opt) { set_error("null argument"); return OBE_ERR_INVALID; }
    std::lock_guard<std::mutex> lock(p->mu);
    return solve_batch_device_locked(p, opt, n_traj, d_rho0, n_param_slots, param_slots, d_param_values, time_count, width,
                                     d_values, d_stats, stream);
}

static obe_status solve_batch_device_locked(obe_plan* p, const obe_solve_options* opt, int64_t n_traj, const double* d_rho0,
                                            int32_t n_param_slots, const int64_t* param_slots, const double* d_param_values,
                                            int64_t time_count, int64_t width, double* d_values, obe_traj_stats* d_stats,
                                            void* stream) {
    obe_status st = ensure_ready(p);
    if (st != OBE_OK) return st;
    if ((st = check_params(p, n_param_slots, param_slots)) != OBE_OK) return st;
    std::vector<double> save_times;
    CallBlob cb;
    int64_t w = 0;
    int cplx = 0;
    if ((st = validate_options(p, opt, save_times, cb, &w, &cplx)) != OBE_OK) return st;
    if (w != width) { set_error("output width mismatch"); return OBE_ERR_INVALID; }
    size_t errs_off = align16(cb.bytes.size());
    size_t need = errs_off + sizeof(TrajErr) * static_cast<size_t>(std::max<int64_t>(n_traj, 1));
    unsigned char* d = nullptr;
    if ((st = scratch(p, need, &d)) != OBE_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!cuda_ok(cudaMemcpyAsync(d, cb.bytes.data(), cb.bytes.size(), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(args)")) return OBE_ERR_CUDA;
    return solve_device(p, opt, n_traj, d_rho0, p->N, n_param_slots, param_slots, d_param_values, 0, nullptr, nullptr, time_count,
                        time_count * width * (cplx ? 2 : 1), d_values, nullptr, d_stats, reinterpret_cast<TrajErr*>(d + errs_off), d,
                        cb, save_times, static_cast<unsigned long long*>(p->d_counter), s);
}

// ---- launch-shape tuning ---------------------------------------------------------------------
namespace {
constexpr int kWidths[] = {32, 64, 128, 256, 512};  // the compiled threads-per-trajectory widths

// the automatic width: by the number of states, or by the state length for effective plans
int default_width(const obe_plan* p) {
    return p->packed.eff ? threads_per_trajectory_len(p->N) : threads_per_trajectory_for(p->n);
}

// Lays the plan's record streams out for `tpt` threads per trajectory; the device image follows
// on the next solve.
void relayout(obe_plan* p, int tpt) {
    if (p->packed.tpt == tpt) return;
    lay_out_lanes(p->packed, tpt);
    if (p->d_blob) cudaFree(p->d_blob);
    p->d_blob = nullptr;
    p->d_device = -1;
}
}  // namespace

obe_status obe_plan_set_shape(obe_plan* p, int32_t tpt, int32_t gpb) {
    if (!p) { set_error("null argument"); return OBE_ERR_INVALID; }
    if (tpt != 0 && shape_capacity(tpt) <= 0) {
        set_error("threads per trajectory must be 0 (automatic) or one of 32, 64, 128, 256, 512");
        return OBE_ERR_INVALID;
    }
    if (tpt != 0 && shape_capacity(tpt) < p->N) {
        set_error("a trajectory of " + std::to_string(tpt) + " threads holds at most " + std::to_string(shape_capacity(tpt)) +
                  " packed elements; this system has " + std::to_string(p->N));
        return OBE_ERR_INVALID;
    }
    if (gpb < 0) { set_error("trajectories per CTA must be non-negative"); return OBE_ERR_INVALID; }
    std::lock_guard<std::mutex> lock(p->mu);
    relayout(p, tpt > 0 ? tpt : default_width(p));
    p->shape_tpt = tpt;
    p->shape_gpb = gpb;
    return OBE_OK;
}

void obe_plan_get_shape(const obe_plan* p, int32_t* tpt, int32_t* gpb) {
    if (tpt) *tpt = p ? p->packed.tpt : 0;
    if (gpb) *gpb = p ? p->shape_gpb : 0;
}

obe_status obe_plan_autotune(obe_plan* p, const obe_solve_options* opt, int64_t n_traj, const double* d_rho0,
                             int32_t n_param_slots, const int64_t* param_slots, const double* d_param_values,
                             int64_t time_count, int64_t width, int32_t probe_steps, int32_t cand_cap, int32_t* cand_tpt,
                             int32_t* cand_gpb, float* cand_ms, int32_t* n_cand, void* stream) {
    g_launches = 0;
    if (!p || !opt) { set_error("null argument"); return OBE_ERR_INVALID; }
    if (n_traj <= 0) { set_error("autotuning needs a non-empty batch"); return OBE_ERR_INVALID; }
    if (probe_steps < 1) { set_error("probe_steps must be positive"); return OBE_ERR_INVALID; }
    std::lock_guard<std::mutex> lock(p->mu);
    const int gpb_before = p->shape_gpb;
    obe_status st = ensure_ready(p);
    if (st != OBE_OK) return st;
    if ((st = check_params(p, n_param_slots, param_slots)) != OBE_OK) return st;
    std::vector<double> save_times;
    CallBlob cb;
    int64_t w = 0;
    int cplx = 0;
    if ((st = validate_options(p, opt, save_times, cb, &w, &cplx)) != OBE_OK) return st;
    if (w != width) { set_error("output width mismatch"); return OBE_ERR_INVALID; }
    const bool mixed = is_mixed(opt->precision);
    const int vm_depth = std::max(p->dev.max_stack, std::max(cb.ev_len, 1));
    // candidates: the automatic width and the wider compiled ones up to 4x it, in the same
    // memory layout; each with as many trajectories per CTA as fit, half of that, and one
    const int w0 = default_width(p);
    std::vector<std::pair<int, int>> cands;
    for (int tw : kWidths) {
        if (tw < w0 || tw > 4 * w0 || shape_capacity(tw) < p->N || (tw >= 256) != (w0 >= 256)) continue;
        relayout(p, tw);
        if ((st = ensure_ready(p)) != OBE_OK) return st;
        LaunchShape s;
        if (plan_launch(p->dev, mixed, n_traj, vm_depth, &s, 1 << 20) != OBE_OK) continue;
        std::vector<int> gs = {s.gpb, (s.gpb + 1) / 2, 1};
        std::sort(gs.begin(), gs.end());
        gs.erase(std::unique(gs.begin(), gs.end()), gs.end());
        for (int g : gs) cands.emplace_back(tw, g);
    }
    if (cands.empty()) {
        relayout(p, p->shape_tpt > 0 ? p->shape_tpt : w0);
        set_error("no compiled launch shape holds this system");
        return OBE_ERR_UNSUPPORTED;
    }
    const size_t vals = static_cast<size_t>(n_traj) * static_cast<size_t>(std::max<int64_t>(time_count, 1)) *
                        static_cast<size_t>(std::max<int64_t>(width, 1)) * (cplx ? 2 : 1);
    double* d_vals = nullptr;
    obe_traj_stats* d_st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        if (d_vals) cudaFree(d_vals);
        if (d_st) cudaFree(d_st);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    if (!cuda_ok(cudaMalloc(&d_vals, vals * sizeof(double)), "cudaMalloc(probe values)") ||
        !cuda_ok(cudaMalloc(&d_st, static_cast<size_t>(n_traj) * sizeof(obe_traj_stats)), "cudaMalloc(probe stats)") ||
        !cuda_ok(cudaEventCreate(&e0), "cudaEventCreate") || !cuda_ok(cudaEventCreate(&e1), "cudaEventCreate")) {
        cleanup();
        relayout(p, p->shape_tpt > 0 ? p->shape_tpt : w0);
        return OBE_ERR_CUDA;
    }
    obe_solve_options probe = *opt;
    probe.maxiters = probe_steps;
    cudaStream_t sm = static_cast<cudaStream_t>(stream);
    std::vector<float> ms(cands.size(), 0.f);
    long long launches = 0;
    size_t best = 0;
    for (size_t c = 0; c < cands.size(); ++c) {
        relayout(p, cands[c].first);
        p->shape_gpb = cands[c].second;
        for (int rep = 0; rep < 2 && st == OBE_OK; ++rep) {  // one untimed run, one timed
            if (rep == 1 && !cuda_ok(cudaEventRecord(e0, sm), "cudaEventRecord")) st = OBE_ERR_CUDA;
            if (st == OBE_OK)
                st = solve_batch_device_locked(p, &probe, n_traj, d_rho0, n_param_slots, param_slots, d_param_values, time_count,
                                               width, d_vals, d_st, stream);
            launches += g_launches;
            if (st == OBE_OK && rep == 1 && !cuda_ok(cudaEventRecord(e1, sm), "cudaEventRecord")) st = OBE_ERR_CUDA;
        }
        if (st == OBE_OK && !cuda_ok(cudaEventSynchronize(e1), "probe solve")) st = OBE_ERR_CUDA;
        if (st == OBE_OK && !cuda_ok(cudaEventElapsedTime(&ms[c], e0, e1), "cudaEventElapsedTime")) st = OBE_ERR_CUDA;
        if (st != OBE_OK) break;
        if (ms[c] < ms[best]) best = c;
    }
    cleanup();
    if (st != OBE_OK) {
        relayout(p, p->shape_tpt > 0 ? p->shape_tpt : w0);
        p->shape_gpb = gpb_before;
        return st;
    }
    relayout(p, cands[best].first);
    p->shape_tpt = cands[best].first;
    p->shape_gpb = cands[best].second;
    if (n_cand) *n_cand = static_cast<int32_t>(cands.size());
    for (size_t c = 0; c < cands.size() && static_cast<int32_t>(c) < cand_cap; ++c) {
        if (cand_tpt) cand_tpt[c] = cands[c].first;
        if (cand_gpb) cand_gpb[c] = cands[c].second;
        if (cand_ms) cand_ms[c] = ms[c];
    }
    g_launches = launches;
    return OBE_OK;
}

// Streams of the heterogeneous batch: one non-blocking stream and completion event per job
// slot, created on the first multi-job call on a device and kept for the process.
namespace {
struct JobStreams {
    int device = -1;
    cudaStream_t s[OBE_MAX_JOBS] = {};
    cudaEvent_t done[OBE_MAX_JOBS] = {};
    cudaEvent_t start = nullptr;
};
JobStreams g_job_streams;
std::mutex g_multi_mutex;  // the job streams above: one heterogeneous batch at a time, taken before any plan's mutex

obe_status job_streams(int dev, JobStreams** out) {
    JobStreams& J = g_job_streams;
    if (J.device != dev) {
        if (J.device >= 0) {
            // another device is current: rebuild on this one (the old device's handles stay valid
            // only there, so release them under it)
            int cur = dev;
            cudaSetDevice(J.device);
            for (int k = 0; k < OBE_MAX_JOBS; ++k) {
                if (J.s[k]) cudaStreamDestroy(J.s[k]);
                if (J.done[k]) cudaEventDestroy(J.done[k]);
                J.s[k] = nullptr;
                J.done[k] = nullptr;
            }
            if (J.start) cudaEventDestroy(J.start);
            J.start = nullptr;
            cudaSetDevice(cur);
        }
        J.device = -1;
        for (int k = 0; k < OBE_MAX_JOBS; ++k) {
            if (!cuda_ok(cudaStreamCreateWithFlags(&J.s[k], cudaStreamNonBlocking), "cudaStreamCreateWithFlags")) return OBE_ERR_CUDA;
            if (!cuda_ok(cudaEventCreateWithFlags(&J.done[k], cudaEventDisableTiming), "cudaEventCreateWithFlags")) return OBE_ERR_CUDA;
        }
        if (!cuda_ok(cudaEventCreateWithFlags(&J.start, cudaEventDisableTiming), "cudaEventCreateWithFlags")) return OBE_ERR_CUDA;
        J.device = dev;
    }
    *out = &J;
    return OBE_OK;
}

struct PreparedJob {
    obe_plan* p;
    const obe_batch_job* j;
    std::vector<double> save_times;
    CallBlob cb;
    int cplx = 0;
    LaunchShape shape;
    unsigned char* d = nullptr;
    size_t errs_off = 0, need = 0;
};

obe_status job_fail(int k, obe_status st) {
    set_error("job " + std::to_string(k) + ": " + last_error_cstr());
    return st;
}

// Validation shared by the immediate and the graph-recorded heterogeneous batch (under the plan
// mutex): plans on the device, options checked, each job's argument block built and launch shape
// chosen; q.need = bytes of its argument block and error records.
obe_status prepare_jobs(int32_t n_jobs, const obe_batch_job* jobs, std::vector<PreparedJob>& pj) {
    for (int k = 0; k < n_jobs; ++k) {
        if (!jobs[k].plan || !jobs[k].opt) { set_error("null argument"); return job_fail(k, OBE_ERR_INVALID); }
        if (jobs[k].n_traj < 0) { set_error("n_traj must be non-negative"); return job_fail(k, OBE_ERR_INVALID); }
        for (int m = 0; m < k; ++m)
            if (jobs[m].plan == jobs[k].plan) {
                set_error("plan already used by job " + std::to_string(m) + " (one job per plan)");
                return job_fail(k, OBE_ERR_INVALID);
            }
    }
    pj.assign(n_jobs, PreparedJob{});
    for (int k = 0; k < n_jobs; ++k) {
        PreparedJob& q = pj[k];
        q.j = &jobs[k];
        q.p = const_cast<obe_plan*>(jobs[k].plan);
        obe_status st = ensure_ready(q.p);
        if (st != OBE_OK) return job_fail(k, st);
        if ((st = check_params(q.p, q.j->n_param_slots, q.j->param_slots)) != OBE_OK) return job_fail(k, st);
        int64_t w = 0;
        if ((st = validate_options(q.p, q.j->opt, q.save_times, q.cb, &w, &q.cplx)) != OBE_OK) return job_fail(k, st);
        if (w != q.j->width) { set_error("output width mismatch"); return job_fail(k, OBE_ERR_INVALID); }
        const int vm_depth = std::max(q.p->dev.max_stack, std::max(q.cb.ev_len, 1));
        if ((st = plan_launch(q.p->dev, is_mixed(q.j->opt->precision), std::max<int64_t>(q.j->n_traj, 1), vm_depth,
                              &q.shape, q.p->shape_gpb)) != OBE_OK)
            return job_fail(k, st);
        q.errs_off = align16(q.cb.bytes.size());
        q.need = q.errs_off + sizeof(TrajErr) * static_cast<size_t>(std::max<int64_t>(q.j->n_traj, 1));
    }
    return OBE_OK;
}

// largest systems first: their trajectories are the longest single pieces of work, so they take
// the SMs first and the small systems fill in behind them (longest-processing-time order)
std::vector<int> job_order(const std::vector<PreparedJob>& pj) {
    std::vector<int> order(pj.size());
    for (size_t k = 0; k < pj.size(); ++k) order[k] = static_cast<int>(k);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return pj[a].p->N > pj[b].p->N; });
    return order;
}

// job q's solve on stream js (its argument block already at q.d; d_gscratch: the large systems'
// stage buffers, or null for the plan's own)
obe_status launch_job(PreparedJob& q, cudaStream_t js, unsigned char* d_gscratch = nullptr) {
    return solve_device(q.p, q.j->opt, q.j->n_traj, q.j->d_rho0, q.p->N, q.j->n_param_slots, q.j->param_slots,
                        q.j->d_param_values, 0, nullptr, nullptr, q.j->time_count,
                        q.j->time_count * q.j->width * (q.cplx ? 2 : 1), q.j->d_values, nullptr, q.j->d_stats,
                        reinterpret_cast<TrajErr*>(q.d + q.errs_off), q.d, q.cb, q.save_times,
                        static_cast<unsigned long long*>(q.p->d_counter), js, nullptr, 0, 0, 0, d_gscratch);
}
}  // namespace

obe_status obe_solve_multi_device(int32_t n_jobs, const obe_batch_job* jobs, void* stream) {
    g_launches = 0;
    if (n_jobs < 0 || n_jobs > OBE_MAX_JOBS) {
        set_error("n_jobs must be between 0 and " + std::to_string(OBE_MAX_JOBS));
        return OBE_ERR_INVALID;
    }
    if (n_jobs == 0) return OBE_OK;
    if (!jobs) { set_error("null argument"); return OBE_ERR_INVALID; }
    std::lock_guard<std::mutex> multi_lock(g_multi_mutex);
    std::vector<obe_plan*> job_plans;
    for (int k = 0; k < n_jobs; ++k)
        if (jobs[k].plan) job_plans.push_back(const_cast<obe_plan*>(jobs[k].plan));
    PlanLocks plan_locks(job_plans.begin(), job_plans.end());
    std::vector<PreparedJob> pj;
    obe_status pst = prepare_jobs(n_jobs, jobs, pj);
    if (pst != OBE_OK) return pst;
    for (int k = 0; k < n_jobs; ++k)
        if ((pst = scratch(pj[k].p, pj[k].need, &pj[k].d)) != OBE_OK) return job_fail(k, pst);
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return OBE_ERR_CUDA;
    JobStreams* J = nullptr;
    obe_status st = job_streams(dev, &J);
    if (st != OBE_OK) return st;
    const std::vector<int> order = job_order(pj);
    cudaStream_t caller = static_cast<cudaStream_t>(stream);
    if (!cuda_ok(cudaEventRecord(J->start, caller), "cudaEventRecord")) return OBE_ERR_CUDA;
    long long launches = 0;
    for (int r = 0; r < n_jobs; ++r) {
        const int k = order[r];
        PreparedJob& q = pj[k];
        cudaStream_t js = J->s[r];
        if (!cuda_ok(cudaStreamWaitEvent(js, J->start, 0), "cudaStreamWaitEvent")) return OBE_ERR_CUDA;
        if (q.j->n_traj > 0) {
            if (!cuda_ok(cudaMemcpyAsync(q.d, q.cb.bytes.data(), q.cb.bytes.size(), cudaMemcpyHostToDevice, js), "cudaMemcpyAsync(args)"))
                return OBE_ERR_CUDA;
            st = launch_job(q, js);
            if (st != OBE_OK) return job_fail(k, st);
            launches += g_launches;
            g_launches = 0;
        }
        if (!cuda_ok(cudaEventRecord(J->done[r], js), "cudaEventRecord")) return OBE_ERR_CUDA;
        if (!cuda_ok(cudaStreamWaitEvent(caller, J->done[r], 0), "cudaStreamWaitEvent")) return OBE_ERR_CUDA;
    }
    g_launches = launches;
    return OBE_OK;
}

// The heterogeneous batch recorded once as a CUDA graph: argument blocks in graph-owned device
// memory, the queue resets and per-plan kernels captured on forked branches.
struct obe_multi_graph {
    int device = 0;
    // each plan and the generation of the device image it had when the launches were recorded (a
    // plan laid out again gets a new image, which the recorded kernels do not see)
    std::vector<std::pair<const obe_plan*, uint64_t>> images;
    std::vector<void*> bufs;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
};

void obe_multi_graph_destroy(obe_multi_graph* G) {
    if (!G) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(G->device);
    if (G->exec) cudaGraphExecDestroy(G->exec);
    if (G->graph) cudaGraphDestroy(G->graph);
    for (cudaEvent_t e : G->events) cudaEventDestroy(e);
    for (cudaStream_t st : G->streams) cudaStreamDestroy(st);
    for (void* b : G->bufs) cudaFree(b);
    cudaSetDevice(cur);
    delete G;
}

obe_status obe_multi_graph_create(int32_t n_jobs, const obe_batch_job* jobs, obe_multi_graph** out) {
    g_launches = 0;
    if (!out) { set_error("null argument"); return OBE_ERR_INVALID; }
    *out = nullptr;
    if (n_jobs < 1 || n_jobs > OBE_MAX_JOBS) {
        set_error("n_jobs must be between 1 and " + std::to_string(OBE_MAX_JOBS));
        return OBE_ERR_INVALID;
    }
    if (!jobs) { set_error("null argument"); return OBE_ERR_INVALID; }
    std::lock_guard<std::mutex> multi_lock(g_multi_mutex);
    std::vector<obe_plan*> job_plans;
    for (int k = 0; k < n_jobs; ++k)
        if (jobs[k].plan) job_plans.push_back(const_cast<obe_plan*>(jobs[k].plan));
    PlanLocks plan_locks(job_plans.begin(), job_plans.end());
    std::vector<PreparedJob> pj;
    obe_status st = prepare_jobs(n_jobs, jobs, pj);
    if (st != OBE_OK) return st;
    auto* G = new obe_multi_graph();
    auto bail = [&](obe_status code) {
        obe_multi_graph_destroy(G);
        return code;
    };
    if (!cuda_ok(cudaGetDevice(&G->device), "cudaGetDevice")) return bail(OBE_ERR_CUDA);
    // argument blocks copied once into memory the graph owns, and the large systems' per-trajectory
    // stage buffers allocated by the graph too (the plan's own grow and move with later calls), so
    // that nothing allocates while the launches are recorded
    std::vector<unsigned char*> gks(n_jobs, nullptr);
    for (int k = 0; k < n_jobs; ++k) {
        PreparedJob& q = pj[k];
        G->images.emplace_back(q.p, q.p->image_gen);
        void* b = nullptr;
        if (!cuda_ok(cudaMalloc(&b, q.need), "cudaMalloc(graph arguments)")) return bail(OBE_ERR_CUDA);
        G->bufs.push_back(b);
        q.d = static_cast<unsigned char*>(b);
        if (!cuda_ok(cudaMemcpy(q.d, q.cb.bytes.data(), q.cb.bytes.size(), cudaMemcpyHostToDevice), "cudaMemcpy(graph arguments)"))
            return bail(OBE_ERR_CUDA);
        if (q.shape.gstride > 0 && q.j->n_traj > 0) {
            void* gk = nullptr;
            if (!cuda_ok(cudaMalloc(&gk, q.shape.gstride * static_cast<size_t>(q.shape.blocks) * q.shape.gpb),
                         "cudaMalloc(graph stage buffers)"))
                return bail(OBE_ERR_CUDA);
            G->bufs.push_back(gk);
            gks[k] = static_cast<unsigned char*>(gk);
        }
    }
    cudaStream_t cs = nullptr;
    if (!cuda_ok(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate")) return bail(OBE_ERR_CUDA);
    G->streams.push_back(cs);
    cudaEvent_t start = nullptr;
    if (!cuda_ok(cudaEventCreateWithFlags(&start, cudaEventDisableTiming), "cudaEventCreate")) return bail(OBE_ERR_CUDA);
    G->events.push_back(start);
    for (int k = 0; k < n_jobs; ++k) {
        cudaStream_t js = nullptr;
        cudaEvent_t done = nullptr;
        if (!cuda_ok(cudaStreamCreateWithFlags(&js, cudaStreamNonBlocking), "cudaStreamCreate")) return bail(OBE_ERR_CUDA);
        G->streams.push_back(js);
        if (!cuda_ok(cudaEventCreateWithFlags(&done, cudaEventDisableTiming), "cudaEventCreate")) return bail(OBE_ERR_CUDA);
        G->events.push_back(done);
    }
    const std::vector<int> order = job_order(pj);
    if (!cuda_ok(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture")) return bail(OBE_ERR_CUDA);
    obe_status rec = OBE_OK;
    long long launches = 0;
    if (!cuda_ok(cudaEventRecord(start, cs), "cudaEventRecord")) rec = OBE_ERR_CUDA;
    for (int r = 0; r < n_jobs && rec == OBE_OK; ++r) {
        const int k = order[r];
        cudaStream_t js = G->streams[1 + r];
        cudaEvent_t done = G->events[1 + r];
        if (!cuda_ok(cudaStreamWaitEvent(js, start, 0), "cudaStreamWaitEvent")) { rec = OBE_ERR_CUDA; break; }
        if (pj[k].j->n_traj > 0) {
            g_launches = 0;
            if ((rec = launch_job(pj[k], js, gks[k])) != OBE_OK) { rec = job_fail(k, rec); break; }
            launches += g_launches;
        }
        if (!cuda_ok(cudaEventRecord(done, js), "cudaEventRecord") || !cuda_ok(cudaStreamWaitEvent(cs, done, 0), "cudaStreamWaitEvent"))
            rec = OBE_ERR_CUDA;
    }
    const std::string rec_msg = last_error_cstr();
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
    G->graph = graph;
    if (rec != OBE_OK) {
        set_error(rec_msg);
        return bail(rec);
    }
    if (!cuda_ok(ce, "cudaStreamEndCapture")) return bail(OBE_ERR_CUDA);
    if (!cuda_ok(cudaGraphInstantiate(&G->exec, G->graph, 0ull), "cudaGraphInstantiate")) return bail(OBE_ERR_CUDA);
    G->launches = launches;
    *out = G;
    g_launches = 0;
    set_error("");
    return OBE_OK;
}

obe_status obe_multi_graph_launch(obe_multi_graph* G, void* stream) {
    g_launches = 0;
    if (!G || !G->exec) { set_error("null argument"); return OBE_ERR_INVALID; }
    {
        std::vector<obe_plan*> gp;
        for (const auto& im : G->images) gp.push_back(const_cast<obe_plan*>(im.first));
        PlanLocks plan_locks(gp.begin(), gp.end());
        for (const auto& im : G->images)
            if (!im.first->d_blob || im.first->image_gen != im.second) {
                set_error("a plan of this graph was laid out again (launch shape changed) since it was recorded: "
                          "create the graph again");
                return OBE_ERR_INVALID;
            }
    }
    if (!cuda_ok(cudaGraphLaunch(G->exec, static_cast<cudaStream_t>(stream)), "cudaGraphLaunch")) return OBE_ERR_CUDA;
    g_launches = G->launches;
    return OBE_OK;
}

// Host-pointer batch/grid/single driver.
static obe_status solve_host(obe_plan* p, const obe_solve_options* o, long long n_traj, const double* rho0, long long rho0_stride,
                             int32_t n_param, const int64_t* param_slots, const double* param_values, int n_axes,
                             const int64_t* axis_slots, const int64_t* axis_len, const double* axes, long long time_count,
                             int64_t width, double* values, obe_traj_stats* stats_out, double* times_out, bool single,
                             std::vector<obe_traj_stats>* stats_vec) {
    g_launches = 0;
    std::lock_guard<std::mutex> lock(p->mu);
    obe_status st = ensure_ready(p);
    if (st != OBE_OK) return st;
    if (n_axes > 0) {
        if ((st = check_params(p, n_axes, axis_slots)) != OBE_OK) return st;
    } else if ((st = check_params(p, n_param, param_slots)) != OBE_OK) {
        return st;
    }
    std::vector<double> save_times;
    CallBlob cb;
    int64_t w = 0;
    int cplx = 0;
    if ((st = validate_options(p, o, save_times, cb, &w, &cplx)) != OBE_OK) return st;
    if (w != width) { set_error("output width mismatch"); return OBE_ERR_INVALID; }
    if (o->maxiters <= 0) {
        set_error(single ? "maxiters must be positive" : "trajectory 0: maxiters must be positive");
        return single ? OBE_ERR_INVALID : OBE_ERR_TRAJECTORY;
    }
    if (o->t1 < o->t0) {
        set_error(single ? "only forward integration" : "trajectory 0: only forward integration");
        return single ? OBE_ERR_INVALID : OBE_ERR_TRAJECTORY;
    }
    const long long per = time_count * width * (cplx ? 2 : 1);
    const size_t n_rho = static_cast<size_t>(rho0_stride ? n_traj * p->N : p->N);
    const size_t n_pv = param_values ? static_cast<size_t>(n_traj * n_param * 2) : 0;
    size_t n_ax = 0;
    for (int k = 0; k < n_axes; ++k) n_ax += static_cast<size_t>(axis_len[k]);
    // scratch layout: call blob | errs | stats | rho0 | params | axes | values | times
    size_t off = align16(cb.bytes.size());
    size_t o_errs = off; off = align16(off + sizeof(TrajErr) * n_traj);
    size_t o_stats = off; off = align16(off + sizeof(obe_traj_stats) * n_traj);
    size_t o_rho = off; off = align16(off + 8 * n_rho);
    size_t o_pv = off; off = align16(off + 8 * n_pv);
    size_t o_ax = off; off = align16(off + 16 * n_ax);
    size_t o_val = off; off = align16(off + 8 * static_cast<size_t>(n_traj * per));
    size_t o_tim = off; off = align16(off + (single ? 8 * static_cast<size_t>(time_count) : 0));
    unsigned char* d = nullptr;
    if ((st = scratch(p, off, &d)) != OBE_OK) return st;
    cudaStream_t s = nullptr;
    if (!cuda_ok(cudaMemcpyAsync(d, cb.bytes.data(), cb.bytes.size(), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(args)")) return OBE_ERR_CUDA;
    if (!cuda_ok(cudaMemcpyAsync(d + o_rho, rho0, 8 * n_rho, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(rho0)")) return OBE_ERR_CUDA;
    if (n_pv && !cuda_ok(cudaMemcpyAsync(d + o_pv, param_values, 8 * n_pv, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(params)")) return OBE_ERR_CUDA;
    if (n_ax && !cuda_ok(cudaMemcpyAsync(d + o_ax, axes, 16 * n_ax, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(axes)")) return OBE_ERR_CUDA;
    std::vector<int64_t> slots_v;
    if (n_axes > 0) slots_v.assign(axis_slots, axis_slots + n_axes);
    else if (n_param > 0) slots_v.assign(param_slots, param_slots + n_param);
    st = solve_device(p, o, n_traj, reinterpret_cast<double*>(d + o_rho), rho0_stride ? p->N : 0,
                      n_axes > 0 ? n_axes : n_param, slots_v.data(), n_pv ? reinterpret_cast<double*>(d + o_pv) : nullptr,
                      n_axes, axis_len, n_ax ? reinterpret_cast<double*>(d + o_ax) : nullptr, time_count, per,
                      reinterpret_cast<double*>(d + o_val), single ? reinterpret_cast<double*>(d + o_tim) : nullptr,
                      reinterpret_cast<obe_traj_stats*>(d + o_stats), reinterpret_cast<TrajErr*>(d + o_errs), d, cb, save_times,
                      static_cast<unsigned long long*>(p->d_counter), s);
    if (st != OBE_OK) return st;
    std::vector<obe_traj_stats> stats(static_cast<size_t>(n_traj));
    std::vector<TrajErr> errs(static_cast<size_t>(n_traj));
    if (!cuda_ok(cudaMemcpyAsync(values, d + o_val, 8 * static_cast<size_t>(n_traj * per), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(values)")) return OBE_ERR_CUDA;
    if (!cuda_ok(cudaMemcpyAsync(stats.data(), d + o_stats, sizeof(obe_traj_stats) * n_traj, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(stats)")) return OBE_ERR_CUDA;
    if (!cuda_ok(cudaMemcpyAsync(errs.data(), d + o_errs, sizeof(TrajErr) * n_traj, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(errs)")) return OBE_ERR_CUDA;
    if (single && times_out && !cuda_ok(cudaMemcpyAsync(times_out, d + o_tim, 8 * static_cast<size_t>(time_count), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync(times)")) return OBE_ERR_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(s), "kernel execution")) return OBE_ERR_CUDA;
    for (long long b = 0; b < n_traj; ++b) {
        int code = stats[b].status;
        if (code == ST_OK && !single && stats[b].n_points != time_count) {
            code = ST_POINTS;
            errs[b].a = time_count;
            errs[b].b = stats[b].n_points;
        }
        if (code != ST_OK) {
            set_error(single ? traj_message(code, errs[b]) : "trajectory " + std::to_string(b) + ": " + traj_message(code, errs[b]));
            return single ? OBE_ERR_INVALID : OBE_ERR_TRAJECTORY;
        }
    }
    if (stats_out) std::memcpy(stats_out, stats.data(), sizeof(obe_traj_stats) * n_traj);
    if (stats_vec) *stats_vec = std::move(stats);
    set_error("");
    return OBE_OK;
}

obe_status obe_solve_batch(const obe_plan* plan, const obe_solve_options* opt, int64_t n_traj, const double* rho0,
                           int32_t n_param_slots, const int64_t* param_slots, const double* param_values, int64_t time_count,
                           int64_t width, double* values, obe_traj_stats* stats) {
    if (!plan || !opt || !rho0 || !values || n_traj <= 0) { set_error("invalid batch arguments"); return OBE_ERR_INVALID; }
    return solve_host(const_cast<obe_plan*>(plan), opt, n_traj, rho0, 1, n_param_slots, param_slots, param_values, 0, nullptr,
                      nullptr, nullptr, time_count, width, values, stats, nullptr, false, nullptr);
}

obe_status obe_solve_grid(const obe_plan* plan, const obe_solve_options* opt, const double* rho0, int32_t n_axes,
                          const int64_t* axis_slots, const int64_t* axis_lengths, const double* axes, int64_t time_count,
                          int64_t width, double* values, obe_traj_stats* stats) {
    if (!plan || !opt || !rho0 || !values) { set_error("invalid grid arguments"); return OBE_ERR_INVALID; }
    if (n_axes <= 0) { set_error("parameter grid must contain at least one axis"); return OBE_ERR_INVALID; }
    if (n_axes > kMaxParams) { set_error("too many grid axes for the GPU solver"); return OBE_ERR_UNSUPPORTED; }
    long long count = 1;
    for (int k = 0; k < n_axes; ++k) {
        if (axis_lengths[k] <= 0) { set_error("parameter grid axes must be non-empty"); return OBE_ERR_INVALID; }
        count *= axis_lengths[k];
    }
    return solve_host(const_cast<obe_plan*>(plan), opt, count, rho0, 0, 0, nullptr, nullptr, n_axes, axis_slots, axis_lengths,
                      axes, time_count, width, values, stats, nullptr, false, nullptr);
}

obe_status obe_solve_single(const obe_plan* plan, const obe_solve_options* opt, const double* rho0, obe_result** out_result) {
    if (!plan || !opt || !rho0 || !out_result) { set_error("invalid single-solve arguments"); return OBE_ERR_INVALID; }
    *out_result = nullptr;
    obe_plan* p = const_cast<obe_plan*>(plan);
    int32_t cplx = opt->output == OBE_OUTPUT_SELECTED;
    int64_t width = opt->output == OBE_OUTPUT_POPULATIONS ? p->n : opt->output == OBE_OUTPUT_FULL ? p->N
                  : opt->output == OBE_OUTPUT_SELECTED ? opt->n_selected : 1;
    long long cap = opt->has_saveat ? opt->n_saveat + 2 : 4096;
    for (int attempt = 0; attempt < 8; ++attempt) {
        auto* r = new obe_result();
        r->width = width;
        r->is_complex = cplx;
        r->values.assign(static_cast<size_t>(cap * width * (cplx ? 2 : 1)), 0.0);
        r->times.assign(static_cast<size_t>(cap), 0.0);
        std::vector<obe_traj_stats> stv;
        // single solves run with time_count = capacity and accept any point count up to it
        obe_solve_options o = *opt;
        obe_status st = solve_host(p, &o, 1, rho0, 0, 0, nullptr, nullptr, 0, nullptr, nullptr, nullptr, cap, width,
                                   r->values.data(), nullptr, r->times.data(), true, &stv);
        if (st != OBE_OK) {
            delete r;
            return st;
        }
        long long pts = stv[0].n_points;
        if (pts <= cap) {
            r->times.resize(static_cast<size_t>(pts));
            r->values.resize(static_cast<size_t>(pts * width * (cplx ? 2 : 1)));
            r->stats = stv[0];
            *out_result = r;
            return OBE_OK;
        }
        delete r;
        cap = pts + 1;
    }
    set_error("single solve output did not fit after repeated growth");
    return OBE_ERR_INVALID;
}

void obe_result_shape(const obe_result* res, int64_t* n_times, int64_t* width, int32_t* is_complex) {
    if (n_times) *n_times = res ? static_cast<int64_t>(res->times.size()) : 0;
    if (width) *width = res ? res->width : 0;
    if (is_complex) *is_complex = res ? res->is_complex : 0;
}

void obe_result_stats(const obe_result* res, obe_traj_stats* stats) {
    if (res && stats) *stats = res->stats;
}

void obe_result_copy(const obe_result* res, double* times, double* values) {
    if (!res) return;
    if (times && !res->times.empty()) std::memcpy(times, res->times.data(), res->times.size() * 8);
    if (values && !res->values.empty()) std::memcpy(values, res->values.data(), res->values.size() * 8);
}

void obe_result_destroy(obe_result* res) { delete res; }

// ---- gradients: the forward solve with a tape, and the reverse sweep ----------------------

// the outputs and options a gradient supports; *width_out: 1 (weighted integral) or n
static obe_status grad_check(const obe_plan* p, const obe_solve_options* o, int64_t* width_out) {
    if (p->packed.eff) {
        set_error("gradients are implemented for expanded_sparse plans");
        return OBE_ERR_UNSUPPORTED;
    }
    if (!p->has_expanded) {
        set_error("execution_mode='expanded_sparse' requires a decomposed Hamiltonian plan");
        return OBE_ERR_INVALID;
    }
    if (o->precision != OBE_PRECISION_FP64 && o->precision != OBE_PRECISION_MIXED) {
        set_error("gradients are implemented for precision='fp64' and precision='mixed'");
        return OBE_ERR_UNSUPPORTED;
    }
    if (o->solver != OBE_SOLVER_DOPRI5 && o->solver != OBE_SOLVER_TSIT5) {
        set_error("gradients are implemented for the adaptive solvers 'dopri5' and 'tsit5'");
        return OBE_ERR_UNSUPPORTED;
    }
    if (p->packed.tpt > 256) {
        set_error("gradients need the plan at 256 threads per trajectory or fewer: call obe_plan_set_shape");
        return OBE_ERR_UNSUPPORTED;
    }
    if (o->output == OBE_OUTPUT_WEIGHTED_INTEGRAL && !o->store_trace && !o->has_saveat) {
        *width_out = 1;
        return OBE_OK;
    }
    if (o->output == OBE_OUTPUT_POPULATIONS && o->has_saveat && o->n_saveat == 1 && o->saveat[0] == o->t1 && !o->save_start) {
        *width_out = p->n;
        return OBE_OK;
    }
    set_error("gradients are implemented for final weighted integrals (output_when='final', saveat=None) and final "
              "populations");
    return OBE_ERR_UNSUPPORTED;
}

int64_t obe_grad_tape_doubles_per_step_for(const obe_plan* plan, int32_t precision) {
    if (!plan) return 0;
    // a double-precision record: t_n, h_n, y_n and K_1..K_6 in double; the mixed form's: t_n, h_n
    // in double, then y_n, k_1, d_2..d_7 in single precision
    const size_t N = static_cast<size_t>(plan->N);
    const size_t bytes = precision == OBE_PRECISION_MIXED ? 16 + 32 * N : (2 + 7 * N) * 8;
    return static_cast<int64_t>(align16(bytes) / 8);
}

int64_t obe_grad_tape_doubles_for(const obe_plan* plan, int64_t max_steps, int32_t checkpoint_every, int32_t precision) {
    if (!plan || max_steps <= 0 || checkpoint_every < 0) return 0;
    if (checkpoint_every == 0) return max_steps * obe_grad_tape_doubles_per_step_for(plan, precision);
    const int64_t n_ck = (max_steps + checkpoint_every - 1) / checkpoint_every;
    return static_cast<int64_t>(align16((2 * static_cast<size_t>(max_steps) + static_cast<size_t>(n_ck) * plan->N) * 8) / 8);
}

int64_t obe_grad_tape_doubles_per_step(const obe_plan* plan) {
    return obe_grad_tape_doubles_per_step_for(plan, OBE_PRECISION_FP64);
}

int64_t obe_grad_tape_doubles(const obe_plan* plan, int64_t max_steps, int32_t checkpoint_every) {
    return obe_grad_tape_doubles_for(plan, max_steps, checkpoint_every, OBE_PRECISION_FP64);
}

obe_status obe_grad_forward(const obe_plan* plan_c, const obe_solve_options* opt, int64_t n_traj, const double* d_rho0,
                            int32_t n_param_slots, const int64_t* param_slots, const double* d_param_values, int64_t max_steps,
                            int32_t checkpoint_every, double* d_tape, int64_t width, double* d_values, obe_traj_stats* d_stats,
                            void* stream) {
    g_launches = 0;
    obe_plan* p = const_cast<obe_plan*>(plan_c);
    if (!p || !opt || !d_tape || max_steps <= 0) { set_error("null argument or non-positive max_steps"); return OBE_ERR_INVALID; }
    if (checkpoint_every < 0) { set_error("checkpoint_every must be non-negative"); return OBE_ERR_INVALID; }
    int64_t gw = 0;
    obe_status st = grad_check(p, opt, &gw);
    if (st != OBE_OK) return st;
    if (gw != width) { set_error("output width mismatch"); return OBE_ERR_INVALID; }
    std::lock_guard<std::mutex> lock(p->mu);
    if ((st = ensure_ready(p)) != OBE_OK) return st;
    if ((st = check_params(p, n_param_slots, param_slots)) != OBE_OK) return st;
    std::vector<double> save_times;
    CallBlob cb;
    int64_t w = 0;
    int cplx = 0;
    if ((st = validate_options(p, opt, save_times, cb, &w, &cplx)) != OBE_OK) return st;
    size_t errs_off = align16(cb.bytes.size());
    size_t need = errs_off + sizeof(TrajErr) * static_cast<size_t>(std::max<int64_t>(n_traj, 1));
    unsigned char* d = nullptr;
    if ((st = scratch(p, need, &d)) != OBE_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!cuda_ok(cudaMemcpyAsync(d, cb.bytes.data(), cb.bytes.size(), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(args)")) return OBE_ERR_CUDA;
    return solve_device(p, opt, n_traj, d_rho0, p->N, n_param_slots, param_slots, d_param_values, 0, nullptr, nullptr, 1, width,
                        d_values, nullptr, d_stats, reinterpret_cast<TrajErr*>(d + errs_off), d, cb, save_times,
                        static_cast<unsigned long long*>(p->d_counter), s, d_tape, max_steps,
                        checkpoint_every > 0 ? obe_grad_tape_doubles_for(p, max_steps, checkpoint_every, opt->precision)
                                             : obe_grad_tape_doubles_per_step_for(p, opt->precision),
                        checkpoint_every);
}

obe_status obe_grad_backward(const obe_plan* plan_c, const obe_solve_options* opt, int64_t n_traj, const double* d_rho0,
                             int32_t n_param_slots, const int64_t* param_slots, const double* d_param_values, int32_t n_grad,
                             const int64_t* grad_slots, int64_t max_steps, int32_t checkpoint_every, const double* d_tape,
                             const obe_traj_stats* d_stats,
                             const double* d_out_grad, double* d_param_grad, double* d_rho0_grad, int32_t* d_adj_status,
                             void* stream) {
    g_launches = 0;
    obe_plan* p = const_cast<obe_plan*>(plan_c);
    if (!p || !opt || !d_tape || !d_stats || !d_out_grad || !d_adj_status || max_steps <= 0) {
        set_error("null argument or non-positive max_steps");
        return OBE_ERR_INVALID;
    }
    if (checkpoint_every < 0) { set_error("checkpoint_every must be non-negative"); return OBE_ERR_INVALID; }
    if (n_grad < 0 || n_grad > kMaxGrad || (n_grad > 0 && (!grad_slots || !d_param_grad))) {
        set_error("gradients are taken with respect to at most " + std::to_string(kMaxGrad) + " parameter slots");
        return OBE_ERR_INVALID;
    }
    int64_t gw = 0;
    obe_status st = grad_check(p, opt, &gw);
    if (st != OBE_OK) return st;
    for (int q = 0; q < n_grad; ++q) {
        if (grad_slots[q] < 0 || grad_slots[q] >= p->n_base || p->base_is_tuple[grad_slots[q]]) {
            set_error("gradient slot " + std::to_string(grad_slots[q]) + " is not a scalar base parameter slot");
            return OBE_ERR_INVALID;
        }
    }
    std::lock_guard<std::mutex> lock(p->mu);
    if ((st = ensure_ready(p)) != OBE_OK) return st;
    if ((st = check_params(p, n_param_slots, param_slots)) != OBE_OK) return st;
    std::vector<double> save_times;
    CallBlob cb;
    int64_t w = 0;
    int cplx = 0;
    if ((st = validate_options(p, opt, save_times, cb, &w, &cplx)) != OBE_OK) return st;
    unsigned char* d = nullptr;
    if ((st = scratch(p, align16(cb.bytes.size()), &d)) != OBE_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!cuda_ok(cudaMemcpyAsync(d, cb.bytes.data(), cb.bytes.size(), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(args)")) return OBE_ERR_CUDA;
    CallArgs A;
    fill_call_args(A, opt, save_times, cb, d);
    A.n_traj = n_traj;
    A.rho0 = d_rho0;
    A.rho0_stride = p->N;
    A.n_param = n_param_slots;
    for (int k = 0; k < A.n_param; ++k) A.param_slot[k] = static_cast<int>(param_slots[k]);
    A.param_values = d_param_values;
    A.vm_depth = std::max(p->dev.max_stack, std::max(cb.ev_len, 1));
    A.k1_refresh = k1_refresh_interval();  // the mixed form's checkpoint replay
    AdjArgs J{};
    J.n_grad = n_grad;
    for (int q = 0; q < n_grad; ++q) J.grad_slot[q] = static_cast<int>(grad_slots[q]);
    J.tape = d_tape;
    J.tape_cap = max_steps;
    J.ckpt = checkpoint_every;
    J.rec_stride = obe_grad_tape_doubles_per_step_for(p, opt->precision);
    J.tape_stride = checkpoint_every > 0 ? obe_grad_tape_doubles_for(p, max_steps, checkpoint_every, opt->precision)
                                         : J.rec_stride;
    J.fwd_stats = d_stats;
    J.out_grad = d_out_grad;
    J.param_grad = d_param_grad;
    J.rho0_grad = d_rho0_grad;
    J.adj_status = d_adj_status;
    J.counter = static_cast<unsigned long long*>(p->d_counter);
    const DevPlan& P = p->dev;
    const int tpt = P.tpt;
    const size_t plan_bytes = adj_plan_smem_bytes(P, tpt);
    const bool events = opt->event_kind != OBE_EVENT_NONE;
    const AdjLayout AL = adj_layout(P.n, P.N, P.n_formula, P.n_coeff, P.n_dyn, P.n_slots, A.vm_depth, tpt, events ? 7 : 6);
    const size_t group = AL.bytes;
    const size_t limit = 227 * 1024;
    int gpb = 256 / tpt;
    while (gpb > 1 && plan_bytes + gpb * group > limit) --gpb;
    if (plan_bytes + gpb * group > limit) { set_error("system too large for the adjoint's shared-memory layout"); return OBE_ERR_UNSUPPORTED; }
    const long long per_sm = (n_traj + sm_count() - 1) / sm_count();
    while (gpb > 1 && gpb > per_sm) --gpb;
    const size_t smem = plan_bytes + gpb * group;
    const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>((n_traj + gpb - 1) / gpb, sm_count())));
    // per resident trajectory group, in the plan's device scratch: one segment of full records
    // (checkpointed tape; one record more with a stop event, whose step's seventh stage goes
    // there) and the large systems' slice
    const size_t groups = static_cast<size_t>(blocks) * gpb;
    // (the mixed form: single-precision records, then the double-precision replay's scratch record)
    const size_t seg_recs = static_cast<size_t>(checkpoint_every) + (events || opt->precision == OBE_PRECISION_MIXED ? 1 : 0);
    const size_t seg_bytes =
        checkpoint_every > 0
            ? align16((seg_recs * J.rec_stride + (opt->precision == OBE_PRECISION_MIXED ? 2 + 8 * static_cast<size_t>(P.N) : 0)) * 8)
            : 0;
    if (seg_bytes + AL.gbytes > 0) {
        unsigned char* gk = nullptr;
        if ((st = kscratch(p, groups * (seg_bytes + AL.gbytes), &gk)) != OBE_OK) return st;
        J.seg = reinterpret_cast<double*>(gk);
        J.seg_stride = static_cast<long long>(seg_bytes / 8);
        J.gscratch = gk + groups * seg_bytes;
        J.gstride = AL.gbytes;
    }
    if (!cuda_ok(cudaMemsetAsync(J.counter, 0, sizeof(unsigned long long), s), "cudaMemsetAsync")) return OBE_ERR_CUDA;
    const int method = opt->solver == OBE_SOLVER_TSIT5 ? 1 : 0;
    const int ept = ept_for(P.N, tpt);
    cudaError_t e = cudaErrorInvalidConfiguration;
    const bool mixed = opt->precision == OBE_PRECISION_MIXED;
#define OBE_ADJ_DISPATCH(T, E)                                                                                    \
    if (tpt == T && ept == E)                                                                                     \
        e = mixed ? launch_adjoint_shape<T, E, true>(P, A, J, blocks, gpb, smem, group, method, s)               \
                  : launch_adjoint_shape<T, E, false>(P, A, J, blocks, gpb, smem, group, method, s);
    OBE_FOR_EACH_ADJOINT(OBE_ADJ_DISPATCH)
#undef OBE_ADJ_DISPATCH
    if (!cuda_ok(e, "adjoint kernel launch")) return OBE_ERR_CUDA;
    g_launches += 1;
    set_error("");
    return OBE_OK;
}

static obe_status rhs_eval(const obe_plan* plan, int64_t count, const double* t, const double* y, int32_t n_override_slots,
                           const int64_t* override_slots, const double* override_values, int32_t precision, double* dy,
                           double* eff_info);

obe_status obe_rhs_eval(const obe_plan* plan, int64_t count, const double* t, const double* y, int32_t n_override_slots,
                        const int64_t* override_slots, const double* override_values, int32_t precision, double* dy) {
    return rhs_eval(plan, count, t, y, n_override_slots, override_slots, override_values, precision, dy, nullptr);
}

obe_status obe_effective_rhs_debug(const obe_plan* plan, double t, const double* y, double* dy, double* info) {
    if (!plan || !plan->packed.eff) { set_error("not an effective-Hamiltonian plan"); return OBE_ERR_INVALID; }
    if (!info) { set_error("null argument"); return OBE_ERR_INVALID; }
    return rhs_eval(plan, 1, &t, y, 0, nullptr, nullptr, OBE_PRECISION_FP64, dy, info);
}

static obe_status rhs_eval(const obe_plan* plan, int64_t count, const double* t, const double* y, int32_t n_override_slots,
                           const int64_t* override_slots, const double* override_values, int32_t precision, double* dy,
                           double* eff_info) {
    g_launches = 0;
    obe_plan* p = const_cast<obe_plan*>(plan);
    if (!p || !t || !y || !dy || count <= 0) { set_error("invalid RHS arguments"); return OBE_ERR_INVALID; }
    if (!p->has_expanded && !p->packed.eff) { set_error("execution_mode='expanded_sparse' requires a decomposed Hamiltonian plan"); return OBE_ERR_INVALID; }
    if (p->packed.eff && is_mixed(precision)) { set_error("effective-Hamiltonian plans solve in double precision"); return OBE_ERR_UNSUPPORTED; }
    std::lock_guard<std::mutex> lock(p->mu);
    obe_status st = ensure_ready(p);
    if (st != OBE_OK) return st;
    if ((st = check_params(p, n_override_slots, override_slots)) != OBE_OK) return st;
    const bool mixed = is_mixed(precision);
    LaunchShape s;
    const int vm_depth = std::max(p->dev.max_stack, 1);
    // the RHS kernel keeps both forms in the double-precision group layout
    if ((st = plan_launch(p->dev, false, count, vm_depth, &s)) != OBE_OK) return st;
    unsigned char* gk = nullptr;
    if (s.gstride > 0 && (st = kscratch(p, s.gstride * static_cast<size_t>(s.blocks) * s.gpb, &gk)) != OBE_OK) return st;
    std::vector<int32_t> slots(override_slots, override_slots + n_override_slots);
    size_t off = 0;
    size_t o_t = off; off = align16(off + 8 * count);
    size_t o_y = off; off = align16(off + 8 * count * p->N);
    size_t o_dy = off; off = align16(off + 8 * count * p->N);
    size_t o_sl = off; off = align16(off + 4 * std::max<size_t>(slots.size(), 1));
    size_t o_ov = off; off = align16(off + 16 * count * std::max<int32_t>(n_override_slots, 1));
    size_t o_er = off; off = align16(off + 64 * count);
    unsigned char* d = nullptr;
    if ((st = scratch(p, off, &d)) != OBE_OK) return st;
    cudaMemcpy(d + o_t, t, 8 * count, cudaMemcpyHostToDevice);
    cudaMemcpy(d + o_y, y, 8 * count * p->N, cudaMemcpyHostToDevice);
    if (n_override_slots > 0) {
        cudaMemcpy(d + o_sl, slots.data(), 4 * slots.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(d + o_ov, override_values, 16 * count * n_override_slots, cudaMemcpyHostToDevice);
    }
    cudaError_t le = cudaErrorInvalidConfiguration;
#define OBE_RHS_DISPATCH(T)                                                                                               \
    if (s.tpt == T)                                                                                                       \
        le = (mixed ? launch_rhs_shape<T, true> : launch_rhs_shape<T, false>)(                                            \
            p->dev, count, reinterpret_cast<double*>(d + o_t), reinterpret_cast<double*>(d + o_y), n_override_slots,      \
            reinterpret_cast<int*>(d + o_sl), reinterpret_cast<double*>(d + o_ov), reinterpret_cast<double*>(d + o_dy),   \
            s.blocks, s.gpb, s.smem, s.group_bytes, vm_depth, gk, s.gstride, reinterpret_cast<double*>(d + o_er));
    OBE_FOR_EACH_RHS(OBE_RHS_DISPATCH)
#undef OBE_RHS_DISPATCH
    g_launches += 1;
    if (!cuda_ok(le, "rhs kernel launch")) return OBE_ERR_CUDA;
    if (!cuda_ok(cudaMemcpy(dy, d + o_dy, 8 * count * p->N, cudaMemcpyDeviceToHost), "rhs kernel")) return OBE_ERR_CUDA;
    if (p->packed.eff) {
        // effective plans: the first state whose field left the operator grid fails the call
        std::vector<double> errs(8 * static_cast<size_t>(count));
        if (!cuda_ok(cudaMemcpy(errs.data(), d + o_er, errs.size() * 8, cudaMemcpyDeviceToHost), "rhs kernel")) return OBE_ERR_CUDA;
        for (int64_t k = 0; k < count; ++k)
            if (errs[8 * k] != 0.0) {
                set_error(field_range_message(errs[8 * k] == ST_FIELD_HIGH, errs[8 * k + 1], errs[8 * k + 2]));
                return OBE_ERR_INVALID;
            }
        if (eff_info)
            for (int q = 0; q < 4; ++q) eff_info[q] = errs[3 + q];
    }
    set_error("");
    return OBE_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// Allocation-free batch solve.
//
// For callers that must not allocate device memory while they solve (a caller that owns all
// device memory up front through its own arena or a fixed memory budget, or that records its
// work into a CUDA graph, cannot let a library call cudaMalloc underneath it): the same
// integrator kernel as obe_solve_batch_device, but every byte of scratch it needs -- the
// plan's device image, the per-call argument block, the per-trajectory error records and the
// work-queue counter -- lives in one fixed, file-scope device array.  Every GPU that loads
// this library holds the array until the process exits.

namespace obe {
namespace {

constexpr size_t kNoAllocPlanBytes = 1u << 20;       // plan device image
constexpr size_t kNoAllocArgBytes = 64u << 10;       // per-call argument block
constexpr long long kNoAllocMaxTrajectories = 65536; // per-trajectory error records
constexpr size_t kNoAllocCounterOff = 0;
constexpr size_t kNoAllocPlanOff = 256;
constexpr size_t kNoAllocArgOff = kNoAllocPlanOff + kNoAllocPlanBytes;
constexpr size_t kNoAllocErrOff = kNoAllocArgOff + kNoAllocArgBytes;
constexpr size_t kNoAllocBytes = kNoAllocErrOff + sizeof(TrajErr) * static_cast<size_t>(kNoAllocMaxTrajectories);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mutex;
void* g_noalloc_base[64] = {nullptr};  // device address of g_noalloc_scratch, per device

}  // namespace
}  // namespace obe

extern "C" obe_status obe_solve_batch_device_noalloc(const obe_plan* plan, const obe_solve_options* opt, int64_t n_traj,
                                                     const double* d_rho0, int32_t n_param_slots, const int64_t* param_slots,
                                                     const double* d_param_values, int64_t time_count, int64_t width,
                                                     double* d_values, obe_traj_stats* d_stats, void* stream) {
    using namespace obe;
    g_launches = 0;
    obe_plan* p = const_cast<obe_plan*>(plan);
    if (!p || !opt || !d_rho0 || !d_values || !d_stats) { set_error("null argument"); return OBE_ERR_INVALID; }
    if (n_traj <= 0) { set_error("n_traj must be positive"); return OBE_ERR_INVALID; }
    if (n_param_slots < 0 || (n_param_slots > 0 && (!param_slots || !d_param_values))) {
        set_error("n_param_slots > 0 needs both param_slots and d_param_values");
        return OBE_ERR_INVALID;
    }
    if (n_traj > kNoAllocMaxTrajectories) {
        set_error("obe_solve_batch_device_noalloc handles at most " + std::to_string(kNoAllocMaxTrajectories) +
                  " trajectories per call, got " + std::to_string(n_traj));
        return OBE_ERR_INVALID;
    }
    if (!p->has_expanded && !p->packed.eff) { set_error("execution_mode='expanded_sparse' requires a decomposed Hamiltonian plan"); return OBE_ERR_INVALID; }
    if (obe_device_count() <= 0) { set_error("no CUDA device is available: the GB300 solver has no CPU fallback"); return OBE_ERR_CUDA; }
    // lock order: the scratch array, then the plan (obe_plan_set_shape / obe_plan_autotune change
    // the plan's launch shape and layout under the plan's mutex while this call reads them)
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    std::lock_guard<std::mutex> plan_lock(p->mu);
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return OBE_ERR_CUDA;
    if (dev < 0 || dev >= 64) { set_error("device index out of range for the allocation-free entry point"); return OBE_ERR_UNSUPPORTED; }
    // once per device, with that device current: the device address of the scratch array
    if (!g_noalloc_base[dev]) {
        void* base = nullptr;
        if (!cuda_ok(cudaGetSymbolAddress(&base, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)")) return OBE_ERR_CUDA;
        g_noalloc_base[dev] = base;
    }
    obe_status st = OBE_OK;
    if ((st = check_params(p, n_param_slots, param_slots)) != OBE_OK) return st;
    std::vector<double> save_times;
    CallBlob cb;
    int64_t w = 0;
    int cplx = 0;
    if ((st = validate_options(p, opt, save_times, cb, &w, &cplx)) != OBE_OK) return st;
    if (w != width) { set_error("output width mismatch"); return OBE_ERR_INVALID; }
    if (cb.bytes.size() > kNoAllocArgBytes) {
        set_error("per-call arguments (saveat, weights, selections, event program) exceed the " +
                  std::to_string(kNoAllocArgBytes) + "-byte block of the allocation-free entry point");
        return OBE_ERR_INVALID;
    }
    unsigned char* base = static_cast<unsigned char*>(g_noalloc_base[dev]);
    std::vector<unsigned char> image;
    DevPlan P;
    build_plan_image(p, image, reinterpret_cast<uintptr_t>(base + kNoAllocPlanOff), P);
    if (image.size() > kNoAllocPlanBytes) {
        set_error("plan device image (" + std::to_string(image.size()) + " bytes) exceeds the " +
                  std::to_string(kNoAllocPlanBytes) + "-byte plan block of the allocation-free entry point");
        return OBE_ERR_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!cuda_ok(cudaMemcpyAsync(base + kNoAllocPlanOff, image.data(), image.size(), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(plan image)")) return OBE_ERR_CUDA;
    if (!cuda_ok(cudaMemcpyAsync(base + kNoAllocArgOff, cb.bytes.data(), cb.bytes.size(), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(arguments)")) return OBE_ERR_CUDA;
    // the work-queue counter must start at zero on every call
    if (!cuda_ok(cudaMemsetAsync(base + kNoAllocCounterOff, 0, sizeof(unsigned long long), s), "cudaMemsetAsync(counter)")) return OBE_ERR_CUDA;

    CallArgs A;
    fill_call_args(A, opt, save_times, cb, base + kNoAllocArgOff);
    A.n_traj = n_traj;
    A.rho0 = d_rho0;
    A.rho0_stride = p->N;
    A.n_param = n_param_slots;
    for (int k = 0; k < A.n_param; ++k) A.param_slot[k] = static_cast<int>(param_slots[k]);
    A.param_values = d_param_values;
    A.n_axes = 0;
    A.axes = nullptr;
    A.cap = time_count;
    A.out_stride = time_count * width * (cplx ? 2 : 1);
    A.values = d_values;
    A.times = nullptr;
    A.stats = d_stats;
    A.errs = reinterpret_cast<TrajErr*>(base + kNoAllocErrOff);
    A.counter = reinterpret_cast<unsigned long long*>(base + kNoAllocCounterOff);
    A.k1_refresh = k1_refresh_interval();
    A.vm_depth = std::max(P.max_stack, std::max(cb.ev_len, 1));

    const bool mixed = is_mixed(opt->precision);
    LaunchShape shape;
    if ((st = plan_launch(P, mixed, n_traj, A.vm_depth, &shape, p->shape_gpb)) != OBE_OK) return st;
    if (shape.gstride > 0) {
        set_error("systems with more than 45 states keep per-trajectory stage buffers in device memory the library "
                  "allocates; solve them with obe_solve_batch_device");
        return OBE_ERR_UNSUPPORTED;
    }
    const int method = opt->solver == OBE_SOLVER_TSIT5 ? 1 : 0;
    cudaError_t e = mixed ? dispatch_shape<true>(P, A, shape, method, s) : dispatch_shape<false>(P, A, shape, method, s);
    if (!cuda_ok(e, "kernel launch")) return OBE_ERR_CUDA;
    g_launches += 1;
    // the host copy of the plan image may go: cudaMemcpyAsync from pageable memory returns only
    // once the source has been staged
    return OBE_OK;
}
