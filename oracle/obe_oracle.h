/*
 * obe_oracle.h -- CPU FP64 restatement of the reference's Lindblad `expanded_sparse` path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GPU solver and the
 * timed CPU baseline; only the tests, __graft_entry__.smoke() and the benchmark's CPU legs load
 * it.  Nothing in the product links or calls it.
 *
 * It restates, in C, the reference crate `centrex_tlf_rust` (rust/src, pinned by
 * rust/Cargo.lock): the expression VM (lindblad/eval.rs), the plan and coefficient packer
 * (lindblad/plan.rs, lindblad/rhs.rs), the partitioned and split-input RHS kernels
 * (lindblad/rhs.rs), the Dopri5 and Tsit5 integrators with their controller, dense output,
 * stiffness probe and terminal events (ode/dopri5.rs, ode/tsit5.rs, ode/common.rs), the output
 * accumulators (ode/output.rs) and the batch driver (lindblad/ode_batch.rs).  The Rust sources
 * cannot be built here (no Rust toolchain), so parity is pinned by the reference's own known
 * answers and by its Python FP64 evaluators (see tests/golden).
 */
#ifndef OBE_ORACLE_H
#define OBE_ORACLE_H

#include "../include/obe_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_plan orc_plan;

/* Build an oracle plan from the same descriptor the product consumes.  NULL on error. */
orc_plan* orc_plan_create(const obe_plan_desc* desc, char* err, size_t err_len);
void orc_plan_destroy(orc_plan* plan);

/* One RHS evaluation (rhs.rs:2090-2148, mode "expanded_sparse") with optional base-slot
   overrides (rhs.rs:1176-1197).  Returns 0 on success. */
int orc_rhs(const orc_plan* plan, int32_t n_override, const int64_t* override_slots,
            const double* override_values, double t, const double* y, double* dy,
            int32_t use_split_input_rhs, char* err, size_t err_len);

/* Evaluate the decomposed Hamiltonian coefficients at t (plan.rs:242-276). out[2*n_coeff]. */
int orc_coefficients(const orc_plan* plan, int32_t n_override, const int64_t* override_slots,
                     const double* override_values, double t, double* out, char* err,
                     size_t err_len);

/*
 * Batch solve (ode_batch.rs:176-351 via ode/batch.rs:31-53).  Trajectory b starts from
 * rho0 + b*rho0_stride (stride 0 = one shared state) with base-slot overrides
 * param_values + b*n_param_slots*2.  Each trajectory must produce exactly time_count points of
 * width values (x2 doubles when complex); they go to values + b*time_count*width*(1|2).
 * out_times (may be NULL) receives the times of trajectory 0.  threads <= 0: all cores.
 * Returns 0, or 1 with "trajectory {i}: {msg}" for the first failing trajectory.
 */
int orc_solve_batch(const orc_plan* plan, const obe_solve_options* opt, int64_t n_traj,
                    const double* rho0, int64_t rho0_stride, int32_t n_param_slots,
                    const int64_t* param_slots, const double* param_values, int64_t time_count,
                    int64_t width, double* values, double* out_times, obe_traj_stats* stats,
                    int32_t threads, int32_t use_split_input_rhs, char* err, size_t err_len);

/*
 * Single solve (python_api.rs:422-528) into caller buffers of `capacity` points.  On return
 * stats->n_points holds the number of points the solve produced; when that exceeds capacity
 * only the first `capacity` were written and the caller re-runs with a larger buffer.
 */
int orc_solve_single(const orc_plan* plan, const obe_solve_options* opt, const double* rho0,
                     int32_t n_param_slots, const int64_t* param_slots, const double* param_values,
                     int64_t capacity, double* times, double* values, obe_traj_stats* stats,
                     int32_t use_split_input_rhs, char* err, size_t err_len);

/* Width of an output spec (ode_batch.rs:150-157) and whether it is complex. */
int64_t orc_output_width(const orc_plan* plan, const obe_solve_options* opt, int32_t* is_complex);

/* An interpolated effective-Hamiltonian plan (effective_lindblad/plan.rs): the parameter graph in
 * `graph`, the operators in `eff` (include/obe_gb300.h).  It solves and evaluates its RHS through
 * the functions above with the effective API's output conventions (split-real state). */
orc_plan* orc_effective_plan_create(const obe_plan_desc* graph, const obe_effective_desc* eff, char* err, size_t err_len);

/* Threads OpenMP will use for a batch with threads <= 0. */
int32_t orc_max_threads(void);

/* Frozen-step replay (test support for gradients): steps[traj][max_steps][2] = (t_n, h_n),
 * n_steps[traj] of them; event_hit[traj] (or null): the last step ended on the stop event;
 * width 1 (weighted integral) or n (final populations). */
int orc_solve_replay(const orc_plan* plan, const obe_solve_options* opt, int64_t n_traj, const double* rho0, int64_t rho0_stride,
                     int32_t n_param_slots, const int64_t* param_slots, const double* param_values, const int64_t* n_steps,
                     const double* steps, int64_t max_steps, const int32_t* event_hit, int64_t width, double* values, char* err,
                     size_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* OBE_ORACLE_H */
