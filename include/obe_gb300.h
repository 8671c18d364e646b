/*
 * obe_gb300.h -- C ABI of the GB300 Lindblad `expanded_sparse` solver.
 *
 * This is the native boundary that replaces the reference's PyO3 extension for the Lindblad
 * hot path (crate `centrex_tlf_rust`, rust/src/lindblad/python_api.rs).  Every entry point
 * takes plain pointers and sizes; nothing here names a Python, Rust or torch type.  All
 * arithmetic on the device is FP64 unless a solve asks for a mixed precision (obe_precision).
 *
 * Error convention: every function returns an obe_status.  On failure the message of the
 * matching reference error (a Python ValueError there) is available from obe_last_error()
 * in the calling thread until that thread's next call.
 */
#ifndef OBE_GB300_H
#define OBE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OBE_ABI_VERSION 2

typedef enum {
    OBE_OK = 0,
    OBE_ERR_INVALID = 1,      /* bad argument or payload (reference: ValueError)            */
    OBE_ERR_TRAJECTORY = 2,   /* a trajectory failed; message "trajectory {i}: {msg}"        */
    OBE_ERR_UNSUPPORTED = 3,  /* valid in the reference, outside this library's path          */
    OBE_ERR_CUDA = 4,         /* CUDA runtime error or no usable device                       */
    OBE_ERR_TIMEOUT = 5       /* a bounded device-side wait gave up                           */
} obe_status;

/* Solvers, rust/src/ode/batch.rs:8-30 (OdeSolver::from_str).  The fixed-step ones
 * (rust/src/ode/fixed.rs) run in double precision only. */
typedef enum {
    OBE_SOLVER_DOPRI5 = 0,
    OBE_SOLVER_TSIT5 = 1,
    OBE_SOLVER_FIXED_DOPRI5 = 2,
    OBE_SOLVER_FIXED_RK2 = 3,
    OBE_SOLVER_FIXED_RK4 = 4
} obe_solver;

/* Observables, rust/src/lindblad/ode_batch.rs:103-163 (OutputSpec). */
typedef enum {
    OBE_OUTPUT_POPULATIONS = 0,        /* y[0..n]                                           */
    OBE_OUTPUT_SELECTED = 1,           /* complex rho_ij for (i, j) pairs                   */
    OBE_OUTPUT_FULL = 2,               /* the packed state                                   */
    OBE_OUTPUT_WEIGHTED_INTEGRAL = 3,  /* trapezoid of sum w_i y_i over pushed points       */
    OBE_OUTPUT_WEIGHTED_RATE = 4       /* sum w_i y_i at each pushed point                   */
} obe_output_kind;

typedef enum { OBE_EVENT_NONE = 0, OBE_EVENT_POPULATION = 1, OBE_EVENT_EXPRESSION = 2 } obe_event_kind;

/*
 * Precision of an adaptive solve (no counterpart in the reference, which is FP64 throughout).
 *   OBE_PRECISION_FP64: every operation in double precision (the drop-in form).
 *   OBE_PRECISION_MIXED: the RHS coefficient products in single precision (as stage deviations
 *     d_s = K_s - K_1, see obe_kernels.cuh); the stage combinations, the state accumulation, the
 *     error norm and the step-size controller in double precision, and, for a trace-preserving
 *     plan, the trace renormalised in double precision after every accepted step.
 *   OBE_PRECISION_MIXED_FP32_CONTROL: as OBE_PRECISION_MIXED, but the stage inputs, the error
 *     norm and the controller in single precision and no renormalisation (faster, step sizes
 *     ~1e-7 relative from a double-precision controller's).  Forward solves only.
 */
typedef enum {
    OBE_PRECISION_FP64 = 0,
    OBE_PRECISION_MIXED = 1,
    OBE_PRECISION_MIXED_FP32_CONTROL = 2
} obe_precision;

/*
 * A compiled expression program: the reference's bytecode (centrex_tlf/lindblad/ir.py:28-47,
 * rust/src/lindblad/eval.rs:11-57) as parallel arrays.  `value` holds (re, im) pairs.
 */
typedef struct {
    int64_t n_instr;
    const int32_t* op;
    const int64_t* index;
    const int32_t* argc;
    const int32_t* function;
    const double* value;        /* [2 * n_instr] */
    int32_t scalar_only;
    int32_t output_is_tuple;
} obe_expr;

/*
 * Plan descriptor: the payload of prepare_lindblad_problem_py
 * (rust/src/lindblad/plan.rs:1155-1308; centrex_tlf/lindblad/plan_static.py:58-68) as flat
 * arrays.  The library copies what it needs; the caller may free these after create.
 */
typedef struct {
    int32_t n_states;

    /* parameter graph (plan.rs:19-25) */
    int32_t n_slots;                 /* len(slot_names)                                        */
    int32_t n_base;                  /* len(base_values)                                       */
    const int32_t* base_is_tuple;    /* [n_base]                                               */
    const double* base_scalar;       /* [2 * n_base]  (re, im) of scalar base values           */
    const int64_t* base_tuple_ptr;   /* [n_base + 1]  offsets into base_tuple_items            */
    const double* base_tuple_items;  /* [2 * base_tuple_ptr[n_base]]                           */
    int32_t n_compounds;
    const int32_t* compound_slot;    /* [n_compounds]                                          */
    const obe_expr* compound_expr;   /* [n_compounds]                                          */
    int32_t n_pchip;
    const int64_t* pchip_ptr;        /* [n_pchip + 1]                                          */
    const double* pchip_grid;        /* [pchip_ptr[n_pchip]]                                   */
    const double* pchip_values;      /* [pchip_ptr[n_pchip]]                                   */

    /* decomposed Hamiltonian coefficients (plan.rs:242-276) */
    int32_t hamiltonian_decomposed;  /* 1 for kind == "decomposed"                              */
    int32_t n_coefficients;
    const obe_expr* coefficient_expr;/* [n_coefficients]                                        */

    /* expanded_sparse RHS plan (plan.rs:1069-1153; ir.py:447-613); has_expanded == 0 when the
       payload's expanded_rhs_plan is None */
    int32_t has_expanded;
    int64_t n_terms;
    const int64_t* output_ptrs;      /* [n(n+1)/2 + 1]                                          */
    const int64_t* input_indices;    /* [n_terms] upper-triangle index                          */
    const int64_t* coeff_indices;    /* [n_terms] -1 = static                                   */
    const uint8_t* coeff_conj;       /* [n_terms]                                               */
    const uint8_t* input_conj;       /* [n_terms]                                               */
    const double* factors_re;        /* [n_terms]                                               */
    const double* factors_im;        /* [n_terms]                                               */

    /* dissipator (plan.rs:1174-1185), kept for validation of the payload */
    const double* source_decay_rates;/* [n_states]                                             */
} obe_plan_desc;

/*
 * Per-solve options: the arguments of solve_lindblad_ode_py / solve_lindblad_batch_ode_py /
 * solve_lindblad_grid_ode_py (python_api.rs:422-799) after the reference's option mapping
 * (python_api.rs:589-617): callers pass the *effective* saveat and save_start.
 */
typedef struct {
    double t0, t1, abstol, reltol, dt;
    int64_t maxiters;
    int32_t solver;                  /* obe_solver                                              */
    int32_t save_start;
    int32_t has_saveat;              /* 0 = saveat None                                         */
    int64_t n_saveat;
    const double* saveat;            /* [n_saveat]                                              */
    int32_t output;                  /* obe_output_kind                                         */
    int32_t store_trace;             /* integral outputs: 1 when output_when == "saveat"        */
    int32_t n_weights;
    const int64_t* weight_index;     /* [n_weights]                                             */
    const double* weight_value;      /* [n_weights]                                             */
    int32_t n_selected;
    const int64_t* selected_i;       /* [n_selected]                                            */
    const int64_t* selected_j;       /* [n_selected]                                            */
    int32_t event_kind;              /* obe_event_kind                                          */
    int32_t n_event_indices;
    const int64_t* event_indices;    /* population event                                        */
    double event_threshold;
    obe_expr event_expr;             /* runtime-expression event                                */
    int32_t precision;               /* obe_precision                                           */
} obe_solve_options;

/* Per-trajectory solver statistics (rust/src/ode/mod.rs:27-35). */
typedef struct {
    int64_t accepted_steps;
    int64_t rejected_steps;
    int64_t rhs_calls;
    int32_t event_triggered;
    int32_t status;                  /* 0 = ok, otherwise an internal code, see obe_last_error */
    double event_time;
    int64_t n_points;                /* points pushed into the output                          */
} obe_traj_stats;

typedef struct obe_plan obe_plan;
typedef struct obe_result obe_result;

/* Thread-local message of the last failure in this thread ("" if none). */
const char* obe_last_error(void);

/* ABI version of the loaded library (OBE_ABI_VERSION). */
int32_t obe_abi_version(void);

/* Number of CUDA devices the library can use; 0 without a GPU (never an error). */
int32_t obe_device_count(void);

/*
 * prepare_lindblad_problem_py (python_api.rs:271-274 -> plan.rs:1155-1308): validate the
 * payload and build the packed term tables (the coefficient packer).  Validation messages are
 * those of plan.rs:1096-1150.  Runs on the host; no device memory is touched until a solve.
 */
obe_status obe_plan_create(const obe_plan_desc* desc, obe_plan** out_plan);
void obe_plan_destroy(obe_plan* plan);

/* Packed length n*n and state count of a plan. */
int64_t obe_plan_packed_len(const obe_plan* plan);
int32_t obe_plan_n_states(const obe_plan* plan);
/* 1 when the plan's RHS keeps the trace of every state for every coefficient value (no
 * population leaves the system), as found by the packer; OBE_PRECISION_MIXED then renormalises the
 * trace after every accepted step.  No counterpart in the reference. */
int32_t obe_plan_trace_preserving(const obe_plan* plan);

/*
 * One RHS evaluation per state on the device: lindblad_rhs_py(plan, packed_state, t,
 * "expanded_sparse") (python_api.rs:294-316 -> rhs.rs:2090-2148), batched over `count`
 * states with optional per-state base-slot overrides.  Host pointers.
 *   y[count * N], t[count], overrides[count * n_slots * 2] (complex, may be NULL), dy[count * N]
 */
obe_status obe_rhs_eval(const obe_plan* plan, int64_t count, const double* t, const double* y,
                        int32_t n_override_slots, const int64_t* override_slots,
                        const double* override_values, int32_t precision, double* dy);

/*
 * solve_lindblad_ode_py (python_api.rs:422-528): one trajectory.  The number of output points
 * is not known in advance (every accepted step when saveat is None), so the result is a
 * library-owned object read with obe_result_*.  Host pointers.
 */
obe_status obe_solve_single(const obe_plan* plan, const obe_solve_options* opt, const double* rho0,
                            obe_result** out_result);
void obe_result_shape(const obe_result* res, int64_t* n_times, int64_t* width, int32_t* is_complex);
void obe_result_stats(const obe_result* res, obe_traj_stats* stats);
/* times[n_times]; values[n_times * width] (doubles, or interleaved re/im when is_complex) */
void obe_result_copy(const obe_result* res, double* times, double* values);
void obe_result_destroy(obe_result* res);

/*
 * solve_lindblad_batch_ode_py (python_api.rs:530-669 -> ode_batch.rs:176-351): B trajectories,
 * each with its own packed rho0 and optional scalar overrides of base slots.  Outputs have a
 * fixed count per trajectory (`time_count` points of `width` values; interleaved re/im for
 * OBE_OUTPUT_SELECTED), written to values[B * time_count * width (*2)].  Host pointers; the
 * copies to and from the device happen inside the call.
 *   rho0[B * N]; param_values[B * n_param_slots * 2] (complex) or NULL;
 *   stats[B] may be NULL; times[time_count] receives the output times (t1 for final outputs).
 */
obe_status obe_solve_batch(const obe_plan* plan, const obe_solve_options* opt, int64_t n_traj,
                           const double* rho0, int32_t n_param_slots, const int64_t* param_slots,
                           const double* param_values, int64_t time_count, int64_t width,
                           double* values, obe_traj_stats* stats);

/*
 * solve_lindblad_grid_ode_py (python_api.rs:671-799 -> ode_batch.rs:571-1040): a row-major
 * grid over scalar base slots (last axis fastest, ode_batch.rs:353-391) from one rho0.
 *   rho0[N]; axes[2 * sum(axis_lengths)] (complex); axis_lengths[n_axes].
 */
obe_status obe_solve_grid(const obe_plan* plan, const obe_solve_options* opt, const double* rho0,
                          int32_t n_axes, const int64_t* axis_slots, const int64_t* axis_lengths,
                          const double* axes, int64_t time_count, int64_t width, double* values,
                          obe_traj_stats* stats);

/*
 * Device-resident form of obe_solve_batch: every pointer is device memory and the call is
 * asynchronous on `stream` (a cudaStream_t, or NULL for the legacy default stream).  It does
 * not synchronise; statuses land in d_stats.  This is the call a GPU-side caller (and the
 * benchmark's device-resident timing) uses; it allocates nothing per call once a plan has
 * been uploaded by its first solve.
 */
obe_status obe_solve_batch_device(const obe_plan* plan, const obe_solve_options* opt,
                                  int64_t n_traj, const double* d_rho0, int32_t n_param_slots,
                                  const int64_t* param_slots, const double* d_param_values,
                                  int64_t time_count, int64_t width, double* d_values,
                                  obe_traj_stats* d_stats, void* stream);

/*
 * Interpolated effective-Hamiltonian Lindblad plans (rust/src/effective_lindblad: the native side
 * of centrex_tlf/effective_hamiltonian/rust_plan.py).  The state is the split-real density
 * matrix [Re rho (row-major n x n), Im rho] of real_dim = 2 n^2 doubles, and
 *     dy = L_c(x) y + (Omega / 2) L_o(x) y + delta L_d(x) y          (effective_lindblad/rhs.rs:88-137)
 * with x, Omega and delta the parameter-graph slots field_slot, rabi_slot and detuning_slot at
 * time t, and each operator a real CSR matrix whose entries are cubics in x on the field grid:
 * on interval k (grid[k] <= x <= grid[k + 1], found with the reference's cached search and its
 * 1e-10 range tolerance), entry p is c0 + dx (c1 + dx (c2 + dx c3)) with dx = x - grid[k] and
 * (c0..c3) = coeffs[(k * nnz + p) * 4 ..].  As in the reference, a Rabi or detuning slot that is a
 * base scalar, or a compound that does not depend on time, is fixed at plan creation to its value
 * from the base parameters (effective_lindblad/plan.rs: detect_constant_slot), so batch overrides
 * do not reach it.
 *
 * obe_effective_plan_create takes the parameter graph in `graph` (n_states and the parameter
 * fields; no Hamiltonian coefficients, no expanded plan) and the operators in `eff`.  The plan
 * then solves through obe_solve_single / obe_solve_batch / obe_solve_batch_device with the
 * effective API's output conventions: populations are the diagonal y[i (n + 1)], a selected
 * (i, j) is (y[i n + j], y[n^2 + i n + j]), full outputs and integral weights index the
 * real_dim-vector.  Double precision only; no stop events.  obe_rhs_eval evaluates its RHS
 * (debug_effective_lindblad_rhs_py), y and dy holding real_dim doubles per state.
 */
typedef struct {
    const int64_t* row_ptrs;     /* [real_dim + 1]                                            */
    const int64_t* col_indices;  /* [nnz]                                                     */
    const double* coeffs;        /* [(n_grid - 1) * nnz * 4], interval-major                  */
    int64_t nnz;
} obe_interp_operator;

typedef struct {
    int64_t real_dim;            /* 2 n_states^2                                              */
    int32_t n_grid;
    const double* field_grid;    /* [n_grid], increasing                                     */
    obe_interp_operator combined, optical, detuning;
    int32_t field_slot, rabi_slot, detuning_slot;
} obe_effective_desc;

obe_status obe_effective_plan_create(const obe_plan_desc* graph, const obe_effective_desc* eff,
                                     obe_plan** out_plan);
/* debug_effective_lindblad_rhs_py (effective_lindblad/python_api.rs:94-152): one RHS at t (host
 * pointers, y and dy of real_dim doubles) with info[4] = the field coordinate, Rabi rate and
 * detuning it used and the field interval. */
obe_status obe_effective_rhs_debug(const obe_plan* plan, double t, const double* y, double* dy, double* info);

/*
 * Launch-shape tuning (no counterpart in the reference, whose CPU path has no launch shape).
 * A solve runs each trajectory on a group of threads (32, 64, 128, 256 or 512: the compiled
 * widths; up to 16 packed elements per thread, 32 at 256 threads, the fewest of the compiled
 * counts that hold the state: 4 or 16 at 64 threads, 2, 12 or 16 at 128, 24 or 32 at 256,
 * 12 or 16 at 512) and puts one or more groups in a CTA.
 * By default the width is the smallest that holds the state (256 above 2,048 elements) and a
 * CTA takes as many groups as its shared memory fits, fewer for small batches.
 *
 * obe_plan_set_shape fixes both for every later solve of the plan: threads_per_trajectory 0 is
 * the default rule; trajectories_per_cta 0 is the automatic count, otherwise at most what fits.
 * A width that cannot hold the state is rejected.  Results of different widths differ by
 * rounding (another summation order), statistics by the steps that rounding moves.
 * obe_plan_get_shape reads the width in use and the fixed trajectories per CTA (0: automatic).
 *
 * obe_plan_autotune measures candidate shapes on a probe of the caller's own batch (arguments as
 * obe_solve_batch_device) and fixes the fastest, as obe_plan_set_shape would.  Each candidate
 * solves the batch with maxiters capped at probe_steps, once untimed and once timed with CUDA
 * events on `stream`.  Candidates: the default width and the wider compiled widths up to 4x it
 * in the same memory layout (stage buffers on chip below 256 threads, in device memory from
 * 256), each with as many trajectories per CTA as fit, half that, and one.  The candidates and
 * their probe times (ms) go to cand_tpt / cand_gpb / cand_ms (up to cand_cap entries; n_cand
 * receives the count).  Synchronises `stream`; allocates and frees its probe outputs.
 * Gradients need a plan width of 256 threads or fewer.  None of these may run while a solve of
 * the same plan is in flight on another thread.
 */
obe_status obe_plan_set_shape(obe_plan* plan, int32_t threads_per_trajectory, int32_t trajectories_per_cta);
void obe_plan_get_shape(const obe_plan* plan, int32_t* threads_per_trajectory, int32_t* trajectories_per_cta);
obe_status obe_plan_autotune(obe_plan* plan, const obe_solve_options* opt, int64_t n_traj,
                             const double* d_rho0, int32_t n_param_slots, const int64_t* param_slots,
                             const double* d_param_values, int64_t time_count, int64_t width,
                             int32_t probe_steps, int32_t cand_cap, int32_t* cand_tpt,
                             int32_t* cand_gpb, float* cand_ms, int32_t* n_cand, void* stream);

/*
 * Heterogeneous batch (no counterpart in the reference, which solves one prepared plan per
 * call, ode_batch.rs:176-351): several device-resident batches, each on its own plan (systems
 * of different sizes, different options, parameter slots and outputs), solved by one call.
 * Every job is what obe_solve_batch_device takes; all pointers inside are device memory except
 * `plan`, `opt` and `param_slots`.  The jobs' persistent kernels run concurrently, the largest
 * systems first, so the GPU is shared between the jobs and the smaller systems fill the SMs
 * that the larger ones leave while they drain.  Asynchronous on `stream`: the jobs start after
 * the work already queued on `stream` and later work on `stream` waits for all of them.  Each
 * plan may appear in at most one job (a plan's scratch serves one solve at a time); at most
 * OBE_MAX_JOBS jobs.  A validation failure names its job: "job {k}: {msg}", and nothing is
 * launched.
 */
#define OBE_MAX_JOBS 16
typedef struct {
    const obe_plan* plan;
    const obe_solve_options* opt;
    int64_t n_traj;
    const double* d_rho0;          /* [n_traj][N] */
    int32_t n_param_slots;
    const int64_t* param_slots;    /* host, [n_param_slots] */
    const double* d_param_values;  /* [n_traj][n_param_slots] complex, or NULL */
    int64_t time_count;
    int64_t width;
    double* d_values;              /* [n_traj][time_count][width] (x2 for selected) */
    obe_traj_stats* d_stats;       /* [n_traj] */
} obe_batch_job;
obe_status obe_solve_multi_device(int32_t n_jobs, const obe_batch_job* jobs, void* stream);

/*
 * The heterogeneous batch recorded once as a CUDA graph (no counterpart in the reference):
 * obe_multi_graph_create validates the jobs as obe_solve_multi_device does (same messages),
 * copies their per-call arguments into device memory the graph owns and records the work-queue
 * resets and the per-plan kernels (each plan on its own branch, largest systems first);
 * obe_multi_graph_launch replays the whole batch as one graph launch on `stream`.  The graph
 * keeps the jobs' device buffers by address: refill d_rho0 / d_param_values between launches and
 * read d_values / d_stats after them (a trajectory's failure is its stats' status).  The jobs'
 * host arrays (options, parameter slots) are read at creation only.  The graph owns its argument
 * blocks and the large systems' stage buffers.  The plans must outlive the graph; a plan's queue
 * counter serves one solve at a time, so no other call may use its plans while a launch is in
 * flight; a plan whose launch shape changes (obe_plan_set_shape, obe_plan_autotune) gets a new
 * device image, and a launch of a graph recorded before that fails with OBE_ERR_INVALID (record
 * it again).  obe_last_launch_count() after a launch: the kernels it ran.
 */
typedef struct obe_multi_graph obe_multi_graph;
obe_status obe_multi_graph_create(int32_t n_jobs, const obe_batch_job* jobs, obe_multi_graph** out_graph);
obe_status obe_multi_graph_launch(obe_multi_graph* graph, void* stream);
void obe_multi_graph_destroy(obe_multi_graph* graph);

/*
 * Gradients (no counterpart in the reference, whose Rust crate has no gradient path): the
 * discrete adjoint of the adaptive solve with its step sequence frozen, for final weighted
 * integrals (output_when="final", saveat None) and final populations, with respect to base
 * parameter slots and the initial state.  Device pointers, asynchronous on `stream`; every
 * system the solver takes (up to 90 states, a plan width of 256 threads or fewer), dopri5/tsit5,
 * precision fp64 or mixed (the mixed form's tape holds single-precision records and its reverse
 * sweep runs the transposed and parameter products in single precision, accumulating in double),
 * with or without a stop event (the event step maps to the dense output at the event time; the
 * event time's own dependence on the state and parameters is included).
 *
 * obe_grad_forward is obe_solve_batch_device that also records a tape per trajectory into d_tape
 * (caller-owned, n_traj * obe_grad_tape_doubles(plan, max_steps, checkpoint_every) doubles).
 * checkpoint_every = 0: every accepted step with its start time, size, start state and stage
 * derivatives 1-6 (obe_grad_tape_doubles_per_step doubles each; a double-precision trajectory
 * that a stop event ends also keeps that step's seventh stage in the next record, so it needs
 * one record more).  checkpoint_every = C > 0: the start time and size of every step and the
 * start state of every C-th step; the reverse sweep then replays each segment of C steps from
 * its start state (frozen steps; double precision, or the mixed form's own single-precision
 * deviation form) into a library-owned buffer of C records per resident trajectory before
 * sweeping it -- one more forward's arithmetic for a tape of 2 + N / C doubles per step.  A
 * trajectory with more than max_steps accepted steps ends with a status whose message asks for a
 * larger max_steps.
 * obe_grad_backward runs the reverse sweep on that tape (same options, max_steps and
 * checkpoint_every): given d(loss)/d(outputs) in d_out_grad ([n_traj][width]), it writes
 * d(loss)/d(parameter) to d_param_grad ([n_traj][n_grad], for the base slots grad_slots, at most
 * 8) and, if d_rho0_grad is not NULL, d(loss)/d(packed rho0) to d_rho0_grad ([n_traj][N]).
 * d_adj_status ([n_traj]): 0 = ok, 1 = a helper function or table received an argument that
 * depends on a differentiated parameter (not differentiable here), 2 = the forward trajectory
 * failed or overflowed the tape, 3 = the stop event's function has a zero time derivative at the
 * crossing.
 * The parameter arguments must be those of the forward call.
 */
int64_t obe_grad_tape_doubles_per_step(const obe_plan* plan);
int64_t obe_grad_tape_doubles(const obe_plan* plan, int64_t max_steps, int32_t checkpoint_every);
/* The same for the form `precision` (obe_precision): the mixed form's full-tape records are
 * single precision, 2 + 4N doubles of room instead of 2 + 7N (the two functions above give the
 * double-precision sizes, enough for either form); obe_grad_forward and obe_grad_backward lay
 * the tape out with these. */
int64_t obe_grad_tape_doubles_per_step_for(const obe_plan* plan, int32_t precision);
int64_t obe_grad_tape_doubles_for(const obe_plan* plan, int64_t max_steps, int32_t checkpoint_every, int32_t precision);
obe_status obe_grad_forward(const obe_plan* plan, const obe_solve_options* opt, int64_t n_traj,
                            const double* d_rho0, int32_t n_param_slots, const int64_t* param_slots,
                            const double* d_param_values, int64_t max_steps, int32_t checkpoint_every,
                            double* d_tape, int64_t width, double* d_values, obe_traj_stats* d_stats,
                            void* stream);
obe_status obe_grad_backward(const obe_plan* plan, const obe_solve_options* opt, int64_t n_traj,
                             const double* d_rho0, int32_t n_param_slots, const int64_t* param_slots,
                             const double* d_param_values, int32_t n_grad, const int64_t* grad_slots,
                             int64_t max_steps, int32_t checkpoint_every, const double* d_tape,
                             const obe_traj_stats* d_stats, const double* d_out_grad,
                             double* d_param_grad, double* d_rho0_grad, int32_t* d_adj_status,
                             void* stream);

/*
 * Allocation-free form of obe_solve_batch_device (no counterpart in the reference).  Some
 * callers cannot let a library allocate device memory while they solve: a caller that owns all
 * device memory up front through its own arena, or one that runs under a fixed memory budget
 * in which a cudaMalloc in the middle of a solve would fail or would have to be accounted for
 * after the fact.  This entry point calls no cudaMalloc/cudaFree (and no
 * allocating library routine); the caller passes every input and output in device memory.  All
 * scratch the integrator needs -- the plan's device image, the per-call argument block, the
 * per-trajectory error records and the work-queue counter -- lives in one fixed file-scope
 * device array of 2,687,232 bytes (about 2.6 MiB) that every GPU which loads this library holds until the process
 * exits.
 * Limits: at most 65,536 trajectories per call, a plan device image of at most 1 MiB and at
 * most 64 KiB of per-call arguments (saveat, weights, selections, event program); larger
 * requests are rejected with OBE_ERR_INVALID and a message saying which limit was hit.
 * Systems above 45 states are rejected with OBE_ERR_UNSUPPORTED: their per-trajectory stage
 * buffers need device memory of the order of a megabyte per trajectory in flight, far beyond the
 * fixed array; solve those with obe_solve_batch_device.
 * The first call on a device looks up the array's device address (once per device, with that
 * device current); make that first call before any stream capture begins.  The address is kept
 * for the life of the process: a cudaDeviceReset between calls is not supported.
 * n_param_slots > 0 needs both param_slots and d_param_values (OBE_ERR_INVALID otherwise).
 * Every call shares the one array and leaves its contents behind: calls whose GPU work overlaps
 * (other streams, other host threads) race on it and must be serialised by the caller.
 * Per-trajectory statuses land in d_stats as with obe_solve_batch_device.
 */
obe_status obe_solve_batch_device_noalloc(const obe_plan* plan, const obe_solve_options* opt,
                                          int64_t n_traj, const double* d_rho0, int32_t n_param_slots,
                                          const int64_t* param_slots, const double* d_param_values,
                                          int64_t time_count, int64_t width, double* d_values,
                                          obe_traj_stats* d_stats, void* stream);

/*
 * The dense batched commutator out = -i [H, rho] of `count` states on the tensor cores (no
 * counterpart in the reference; the measurement behind keeping the sparse gather at >= 64
 * states): H and rho Hermitian, n <= 80, [count][n][n] complex64 (re, im interleaved) in device
 * memory; tcgen05.mma kind::tf32 (products at TF32 precision, FP32 accumulation).  d_status[0]
 * counts states whose tensor-core wait gave up (0 on success); asynchronous on `stream`.
 */
obe_status obe_dense_commutator_tf32(int64_t count, int32_t n, const float* d_h, const float* d_rho, float* d_out,
                                     uint32_t* d_status, void* stream);

/* Number of kernel launches issued by the last solve in this thread (for accounting). */
int64_t obe_last_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* OBE_GB300_H */
