// obe_internal.h -- layouts shared by the host packer (obe_plan.cpp) and the CUDA solver
// (obe_solver.cu).  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/obe_gb300.h"

namespace obe {

// Expression VM opcodes (centrex_tlf/lindblad/ir.py:28-47; rust/src/lindblad/eval.rs:11-57).
enum : int32_t {
    OP_CONST = 1, OP_SLOT = 2, OP_TEMP = 3, OP_TIME = 4, OP_ADD = 5, OP_SUB = 6, OP_MUL = 7,
    OP_DIV = 8, OP_POW = 9, OP_NEG = 10, OP_CONJ = 11, OP_BUILTIN = 12, OP_HELPER = 13,
    OP_GT = 14, OP_GE = 15, OP_LT = 16, OP_LE = 17, OP_EQ = 18, OP_NE = 19,
    // device-only opcode: helper 16 resolved on the host to a PCHIP table (index in `fn`)
    OP_PCHIP_TABLE = 32
};

constexpr int kMaxStack = 48;      // device VM stack depth (host rejects deeper programs)
constexpr int kMaxSlots = 96;      // per-lane slot storage of the device VM
constexpr int kMaxDynCoeff = 16;   // time-dependent Hamiltonian coefficients per plan
constexpr int kMaxHelperArgs = 12;

// One expression in the device instruction pool.
struct DevExpr {
    int32_t start;
    int32_t len;
    int32_t real_ok;  // real operands give real results through every instruction (see vm_eval_real)
    int32_t pad;
};

// A record of the RHS gather stream.  Bits:
//   [0, 14)  input slot: i for the diagonal entry rho_ii, n + m for the m-th upper pair
//   14       complex input (off-diagonal) -- otherwise a real diagonal input
//   15       input conjugated (negate the imaginary part)
//   16       last record of the current output: flush the accumulator
//   [17, 32) index of the coefficient formula in the per-trajectory table
constexpr uint32_t kRecIndexMask = 0x3FFFu;
constexpr uint32_t kRecComplex = 1u << 14;
constexpr uint32_t kRecConj = 1u << 15;
constexpr uint32_t kRecFlush = 1u << 16;
constexpr int kRecCoefShift = 17;
constexpr uint32_t kFStreamClassMask = 0xFFFu;
constexpr uint32_t kFStreamFlush = 1u << 12;
constexpr int kFStreamFormulaShift = 13;
constexpr uint32_t kMaxFormulas = (1u << 15) - 1;
constexpr uint32_t kNoImag = 0xFFFFu;
// formula-major stream of the adjoint's parameter pass: record entries (input slot [0, 14),
// output slot [14, 28), conjugate input bit 28) follow each other per formula, then a formula
// entry (bit 31, formula index in the low bits) closes the formula
constexpr uint32_t kBilSlotMask = 0x3FFFu;
constexpr int kBilOutShift = 14;
constexpr uint32_t kBilConj = 1u << 28;
constexpr uint32_t kBilEnd = 1u << 31;

// Device view of a packed plan.  All pointers point into one device allocation.
struct DevPlan {
    int32_t n, N, U;
    // expression pool
    const int32_t* ins_op;
    const int32_t* ins_arg;      // slot index (SLOT) / argc (BUILTIN, HELPER)
    const int32_t* ins_fn;       // function id / PCHIP table index
    const double* ins_val;       // [2 * n_ins]
    // parameter graph
    int32_t n_slots, n_base;
    const double* base_val;      // [2 * n_base]
    const int32_t* base_tuple;   // [n_base] tuple id or -1
    const int32_t* tuple_ptr;    // [n_tuples + 1]
    const double* tuple_items;   // [2 * items]
    int32_t n_comp;
    const int32_t* comp_slot;
    const DevExpr* comp_expr;
    const uint8_t* comp_dynamic;
    int32_t n_coeff;
    const DevExpr* coeff_expr;
    const uint8_t* coeff_dynamic;
    int32_t n_dyn;               // time-dependent coefficients
    const int32_t* dyn_ids;      // [n_dyn] coefficient index
    const int32_t* coeff_dyn_pos;// [n_coeff] position in dyn_ids or -1
    int32_t time_dependent;
    int32_t max_stack;           // deepest VM stack of the plan's programs
    int32_t dyn_real_closed;     // every time-dependent compound maps real slots to real values
    // the time-dependent programs in evaluation order, compacted for the per-step coefficient rows:
    // n_vcomp compounds (pad = the compound's slot), then the n_dyn coefficients (pad = row
    // position); starts index the compact instruction arrays vop/varg/vfn/vval (n_vins entries)
    int32_t n_vcomp, n_vprog, n_vins;
    const DevExpr* vprog;
    const int32_t* vop;
    const int32_t* varg;
    const int32_t* vfn;
    const double* vval;          // [2 * n_vins]
    // PCHIP tables (plan.rs:27-116)
    int32_t n_pchip;
    const int32_t* pchip_ptr;
    const double* pchip_grid;
    const double* pchip_coef;    // [4 * segments]
    const int32_t* pchip_cptr;   // [n_pchip] offset of each table's coefficients
    // coefficient formulas: table entry f = sum over its products of factor * c(class)
    int32_t n_formula;           // entries 1..n_formula (entry 0 is the zero coefficient)
    int32_t n_static_formula;    // entries 1..n_static_formula are time independent
    const int32_t* formula_ptr;  // [n_formula + 1] into the product lists
    const double* prod_factor;   // [2 * n_prod]
    const int32_t* prod_class;   // [n_prod] -1 = constant 1, else coeff * 2 + conj
    const float* prod_factor32;  // [2 * n_prod] single-precision copy (mixed form)
    int32_t dyn_prod0, n_dyn_prod;  // the time-dependent formulas' products: [dyn_prod0, dyn_prod0 + n_dyn_prod)
    // gather stream, lane interleaved for `tpt` threads per trajectory
    int32_t tpt;
    int32_t n_iter;              // records per thread (padded)
    const uint32_t* rec;         // [n_iter * tpt]
    int32_t n_out;               // outputs per thread (padded)
    const uint32_t* lane_out;    // [n_out * tpt]: re | im << 16 (im = kNoImag on the diagonal)
    // time-dependent formulas as a thread-interleaved product stream (mixed form):
    // [n_fiter * tpt] of (factor re, factor im, meta, 0); meta = class + 1 (0: the constant 1)
    // | kFStreamFlush (last product of the formula) | formula << kFStreamFormulaShift
    int32_t n_fiter;
    const uint32_t* fstream;     // [n_fiter * tpt * 4]
    // the transposed gather stream (adjoint: v_bar = L^T u_bar), thread-interleaved: each record
    // reads an OUTPUT slot (the index field) and the formula of the forward record; each thread
    // accumulates the adjoint of its own INPUT slots, written to lane_in (re | im << 16)
    int32_t n_titer;
    const uint32_t* trec;        // [n_titer * tpt]
    int32_t n_tin;
    const uint32_t* lane_in;     // [n_tin * tpt]
    // the adjoint's parameter pass: the records of every formula with a parameter-dependent
    // product, formula-major and thread-interleaved (kBil* entries)
    int32_t n_biter;
    const uint32_t* bil;         // [n_biter * tpt]
    // populations are y[i * pop_stride] (1 packed; n + 1 for the split-real effective state)
    int32_t pop_stride;
    // the RHS keeps the trace for every coefficient value (sum over the diagonal outputs of every
    // input's and coefficient's products is zero): the mixed form renormalises the trace
    int32_t trace_preserving;
    // per Hamiltonian coefficient: the largest |factor| of the RHS terms it multiplies (the weight
    // of that coefficient's magnitude in the launch's cost estimate per trajectory)
    const double* coeff_scale;   // [n_coeff]
    // interpolated effective-Hamiltonian plans (eff != 0; N = real_dim): the RHS is
    // L_c(x) y + (Omega / 2) L_o(x) y + delta L_d(x) y with x, Omega, delta = coefficients 0, 1, 2
    int32_t eff;
    int32_t eff_ngrid;
    const double* eff_grid;      // [eff_ngrid]
    const int32_t* eff_rows;     // [3][N + 1], offsets within each operator
    const int32_t* eff_cols;     // operator k at eff_col_off[k]
    const double* eff_coef;      // operator k at eff_coef_off[k]: [(eff_ngrid - 1)][nnz_k][4]
    int32_t eff_nnz[3];
    int32_t eff_col_off[3];
    int64_t eff_coef_off[3];
};

// Host-side result of packing (owned by obe_plan).
struct HostPacked {
    std::vector<int32_t> ins_op, ins_arg, ins_fn;
    std::vector<double> ins_val;
    std::vector<double> base_val;
    std::vector<int32_t> base_tuple, tuple_ptr;
    std::vector<double> tuple_items;
    std::vector<int32_t> comp_slot;
    std::vector<DevExpr> comp_expr;
    std::vector<uint8_t> comp_dynamic;
    std::vector<DevExpr> coeff_expr;
    std::vector<uint8_t> coeff_dynamic;
    std::vector<int32_t> dyn_ids, coeff_dyn_pos;
    std::vector<int32_t> pchip_ptr;
    std::vector<double> pchip_grid, pchip_coef;
    std::vector<int32_t> pchip_cptr;
    std::vector<int32_t> formula_ptr, prod_class;
    std::vector<double> prod_factor;
    std::vector<float> prod_factor32;
    // width-independent record lists, laid out for a number of threads per trajectory by
    // lay_out_lanes: per output (upper index) its gather words without the flush bit, per input
    // slot its transposed words; *_lane_word is the lane_out / lane_in word of each
    std::vector<int64_t> g_ptr, t_ptr;  // [U + 1]
    std::vector<uint32_t> g_word, t_word, g_lane_word, t_lane_word;
    // the lane layout of the current width
    std::vector<uint32_t> rec, lane_out;
    std::vector<uint32_t> fstream;  // 4 words per entry
    std::vector<uint32_t> trec, lane_in;
    int32_t n_titer = 0, n_tin = 0;
    std::vector<uint32_t> bil;
    int32_t n_biter = 0;
    // effective-Hamiltonian plans
    int32_t pop_stride = 1;
    int32_t eff = 0;
    std::vector<double> eff_grid, eff_coef;
    std::vector<int32_t> eff_rows, eff_cols;
    int32_t eff_nnz[3] = {0, 0, 0};
    int32_t eff_col_off[3] = {0, 0, 0};
    int64_t eff_coef_off[3] = {0, 0, 0};
    int32_t n_iter = 0, n_out = 0, tpt = 32, n_fiter = 0;
    int32_t n_formula = 0, n_static_formula = 0;
    int32_t max_stack = 0;
    int32_t n_vm_slots = 0;     // parameter slots plus the hoisted static subexpressions
    int32_t dyn_real_closed = 0;  // every time-dependent compound is real_ok
    int32_t trace_preserving = 0;
    std::vector<double> coeff_scale;
};

}  // namespace obe

// Opaque handle of the public ABI.
struct obe_plan {
    int32_t n = 0;
    int64_t N = 0, U = 0;
    int32_t n_slots = 0, n_base = 0, n_coeff = 0;
    int32_t has_expanded = 0;
    int32_t time_dependent = 0;
    std::vector<int32_t> base_is_tuple;
    obe::HostPacked packed;
    // device copy (uploaded on first use, per device)
    void* d_blob = nullptr;
    int d_device = -1;
    uint64_t image_gen = 0;  // incremented with every device image uploaded (recorded graphs check it)
    obe::DevPlan dev{};
    // reusable device scratch of the host-pointer entry points
    void* d_scratch = nullptr;
    size_t scratch_bytes = 0;
    void* d_counter = nullptr;
    // global stage buffers of large systems (grow-only)
    void* d_gk = nullptr;
    size_t gk_bytes = 0;
    // the cost-ordered queue of a launch: per trajectory its cost estimate and the order (grow-only)
    void* d_ord = nullptr;
    size_t ord_bytes = 0;
    // launch shape fixed by obe_plan_set_shape / obe_plan_autotune (0: the automatic choice)
    int32_t shape_tpt = 0, shape_gpb = 0;
    // serialises the entry points that use this plan's layout, device image and scratch; calls on
    // different plans (e.g. one per device) run concurrently
    std::mutex mu;
};

namespace obe {
void set_error(const std::string& msg);
const char* last_error_cstr();  // the calling thread's last message
std::string fmt_f64(double v);  // Rust Display of f64
obe_status pack_plan(const obe_plan_desc* d, obe_plan* p);
int threads_per_trajectory_for(int32_t n);
int threads_per_trajectory_len(int64_t len);  // the same rule for a state of len doubles
int64_t shape_capacity(int tpt);  // packed elements one trajectory of that compiled width holds (0: none)
void lay_out_lanes(HostPacked& hp, int tpt);
}  // namespace obe
