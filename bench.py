"""Benchmark: batched OBE trajectories/s of the 4096-point 16-state TlF parameter scan.

Workload (the scan configuration of the reference's headline metric): the 16-state X J=1 + B
J'=1 F'=1 (+ lumped X J=3) system, Gaussian Rabi pulse (peak Γ·10^U[-1,1], σ = 20/Γ, centre
100/Γ), detuning U[-5Γ, 5Γ], polarisation angle U[0, π], 4096 seeded points, Tsit5 with
rtol 1e-8 / atol 1e-11 over [0, 200/Γ], observable = time-integrated excited population.  The
plan payload is the reference builders' own output (tests/golden/plan_q1_16.json).

A "step" is one solve of the whole 4096-point batch.  The default precision is the mixed form
(single-precision RHS products, double-precision state, error norm and controller); its final
populations are compared with the plain FP64 path on every point, and the FP64 path is timed on
the same batch beside it (`fp64_gpu`).  `value` times the device-resident entry
point (obe_solve_batch_device) with CUDA events on its stream and the L2 flushed between steps;
`e2e` times the reference-facing call solve_lindblad_batch_ode_py with host arrays (copies in
the timed region).  Beside the headline the line carries the adjoint's cost against the forward
solve (`gradient`), the heterogeneous batch of 16-, 39- and 76-state systems in one call
(`heterogeneous`) and the interpolated effective-Hamiltonian path (`effective`).  `--impl reference` times the CPU path of the reference restated in C
(the oracle) on the host cores, on a bounded sample of the same scan.
"""

from __future__ import annotations

import argparse
import contextlib
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for sub in ("centrex-tlf_gb300", "oracle", "tests/golden"):
    sys.path.insert(0, str(ROOT / sub))

METRIC = "batched OBE trajectories/s at <=1e-6 pop. error vs plain FP64"
# DRAM bytes (read + write) per trajectory of integrate_kernel, from ncu captures of this
# workload (dram__bytes_read.sum + dram__bytes_write.sum over the trajectories of the captured
# launch): the mixed forms at 4096 points, FP64 at 1536 points; see profiles/.
TRAFFIC_BYTES_PER_TRAJECTORY = {"mixed": (14_186_752 + 158_208) / 4096, "fp64": 3_467_008 / 1536}
W_EXCITED = [(13, 1.0), (14, 1.0), (15, 1.0)]


def workload(points: int, seed: int = 20241203):
    import codec

    d = codec.load("plan_q1_16")
    gamma = d["gamma"]
    rng = np.random.default_rng(seed)
    params = np.stack(
        [gamma * 10 ** rng.uniform(-1.0, 1.0, points), rng.uniform(-5.0, 5.0, points) * gamma, rng.uniform(0.0, np.pi, points)],
        axis=1,
    ).astype(np.complex128)
    slots = [d["payload"]["parameter_graph"]["slot_names"].index(s) for s in ("rabi", "detuning", "theta")]
    return d, params, slots


def flops_per_step_unit(payload) -> tuple[int, int]:
    """Algorithmic work: F_rhs = 4*(diagonal-input terms) + 8*(complex-input terms); one
    attempted step = 6*F_rhs + 60*N."""
    e = payload["expanded_rhs_plan"]
    n = payload["n_states"]
    diag = {i * n - i * (i - 1) // 2 for i in range(n)}  # upper index of (i, i)
    inp = np.asarray(e["input_indices"])
    n_diag = int(np.isin(inp, list(diag)).sum())
    f_rhs = 4 * n_diag + 8 * (inp.size - n_diag)
    return f_rhs, 6 * f_rhs + 60 * n * n


class ClockSampler:
    def __init__(self, path: Path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self, device_index: int) -> dict:
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9 or parts[0] != str(device_index):
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_oracle_rate(d, params, slots, sample: int, threads: int = 0) -> dict:
    import oracle

    op = oracle.OraclePlan(d["payload"])
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    o = op.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, saveat=None, save_start=True,
                   maxiters=100000, solver="tsit5", output="excited_population", output_indices=None,
                   output_when="final", integral_weights=W_EXCITED, stop_event=None)
    p = params[:sample]
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), p.shape[0], axis=0)
    start = time.perf_counter()
    vals, _, _ = op.solve_batch(o, rho0, slots, p, threads=threads)
    dt = time.perf_counter() - start
    cores = threads if threads > 0 else oracle.max_threads()
    return {"value": p.shape[0] / dt, "unit": "trajectories/s", "cores": int(cores), "kind": "port",
            "sample": f"{p.shape[0]} of the {params.shape[0]} scan points, all {cores} host threads, C FP64 oracle",
            "seconds": dt, "values": vals.reshape(-1)}


def cpu_oracle_populations(d, params, slots, sample: int) -> np.ndarray:
    """Final populations of the first `sample` scan points from the FP64 oracle (accuracy check only)."""
    import oracle

    op = oracle.OraclePlan(d["payload"])
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    # final populations: saveat=[t1], save_start=False, as the reference maps them (python_api.rs:589-617)
    o = op.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, saveat=np.array([t1]), save_start=False,
                   maxiters=100000, solver="tsit5", output="populations", output_indices=None,
                   output_when="final", integral_weights=None, stop_event=None)
    p = params[:sample]
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), p.shape[0], axis=0)
    vals, _, _ = op.solve_batch(o, rho0, slots, p)
    return vals.reshape(p.shape[0], -1)


def run_reference(args) -> None:
    """The reference arm: the reference's CPU path (its Rust solver restated in C, the oracle) on
    all host threads, timed on the whole configured scan (`--points`, 4096 by default) every step,
    warm-up steps included."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    d, params, slots = workload(args.points)
    for _ in range(args.warmup):
        cpu_oracle_rate(d, params, slots, args.points)
    secs = []
    for _ in range(args.steps):
        r = cpu_oracle_rate(d, params, slots, args.points)
        secs.append(r["seconds"])
    value = float(args.points * args.steps / sum(secs))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "trajectories/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(secs)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"q1_16state_gaussian_scan_{args.points}pt_tsit5", "points": args.points,
                   "points_per_step": args.points, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "trajectories/s", "cores": r["cores"], "kind": "port",
                         "sample": f"the whole {args.points}-point scan every step, all {r['cores']} host threads, "
                                   "C FP64 oracle (-O3)"},
        "e2e": {"value": value, "unit": "trajectories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own path is Rust (PyO3); no Rust toolchain exists here or on the GPU box, so the "
                "reference arm times its C restatement (oracle/) on all host threads",
    }
    print(json.dumps(line))


def measure_gemm_peak(torch, dev, dtype) -> float:
    """Best-of-3 dense GEMM rate in TFLOP/s: float64 (the FP64 pipe) or float32 with TF32 off
    (the FP32 CUDA-core pipe)."""
    n = 4096
    a = torch.randn(n, n, dtype=dtype, device=dev)
    b = torch.randn(n, n, dtype=dtype, device=dev)
    tf32 = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        for _ in range(2):
            torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(3):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            torch.matmul(a, b)
            e.record()
            torch.cuda.synchronize()
            best = max(best, 2.0 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = tf32
    return best


def measure_gradient(torch, d, params_all, dev, n_traj: int = 256, reps: int = 3) -> dict:
    """The adjoint workload: n_traj points of the scan, d(excited-population integral)/d(rabi,
    detuning, theta, t_center) through the discrete adjoint (FP64, Tsit5); the forward-with-tape
    plus reverse-sweep time against the plain FP64 forward solve of the same points."""
    from centrex_tlf_gb300.autograd import solve_batch_with_grad
    from centrex_tlf_gb300.native import NativePlan

    gamma, (t0, t1) = d["gamma"], d["t_span"]
    names = d["payload"]["parameter_graph"]["slot_names"]
    slots = [names.index(s) for s in ("rabi", "detuning", "theta", "t_center")]
    p = np.concatenate([params_all[:n_traj].real, np.full((n_traj, 1), 100.0 / gamma)], axis=1)
    plan = NativePlan(d["payload"])
    opts = plan.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, saveat=None, save_start=True,
                        maxiters=100000, solver="tsit5", output="excited_population", output_indices=None,
                        output_when="final", integral_weights=W_EXCITED, stop_event=None)
    d_rho = torch.from_numpy(np.repeat(d["rho0_packed"].reshape(1, -1), n_traj, axis=0)).to(dev)
    d_par = torch.from_numpy(np.ascontiguousarray(p.astype(np.complex128)).view(np.float64).reshape(-1)).to(dev)
    d_val = torch.zeros(n_traj, dtype=torch.float64, device=dev)
    d_st = torch.zeros(n_traj * 6, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def fwd():
        plan.solve_batch_device(opts, n_traj, d_rho.data_ptr(), slots, d_par.data_ptr(), 1, d_val.data_ptr(),
                                d_st.data_ptr(), stream.cuda_stream)

    def grad(checkpoint_every=0, precision="fp64"):
        pt = torch.tensor(p, dtype=torch.float64, device=dev, requires_grad=True)
        j = solve_batch_with_grad(plan, d["rho0_packed"], (t0, t1), pt, slots, dt=1e-3 / gamma, integral_weights=W_EXCITED,
                                  max_steps=2048, checkpoint_every=checkpoint_every, precision=precision)
        j.sum().backward()
        grad.last_values = j.detach()
        return pt.grad

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            start = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - start)
        return best

    def grad_width(precision):
        # the launch width at which the gradient (taped forward and reverse sweep, checkpoints
        # every 512 steps) is fastest: the autotuner tunes the plain forward, and the reverse
        # sweep's best width need not be the forward's
        best = None
        for w in (32, 64, 128):
            plan.set_shape(w, 0)
            t = timed(lambda: grad(512, precision=precision))
            if best is None or t < best[1]:
                best = (w, t)
        plan.set_shape(best[0], 0)
        return best

    t_fwd = timed(fwd)
    t_grad = timed(grad)
    # the forward at the launch shape the autotuner picks for this batch; the gradient at the
    # width where it is fastest (the ratio: the fastest gradient over the fastest forward)
    cands = plan.autotune(opts, n_traj, d_rho.data_ptr(), slots, d_par.data_ptr(), 1, probe_steps=64,
                          stream=stream.cuda_stream)
    t_fwd_t = timed(fwd)
    w_grad, t_grad_ck = grad_width("fp64")
    t_grad_t = timed(grad)
    g64 = grad().cpu().numpy()
    j64 = grad.last_values.cpu().numpy()
    # the mixed form (FP32-RHS forward with a single-precision tape, single-precision transposed
    # and parameter products in the reverse sweep, FP64 accumulation): the forward at the shape the
    # autotuner picks for it, the gradient at its own fastest width
    opts_m = plan.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, saveat=None, save_start=True,
                          maxiters=100000, solver="tsit5", output="excited_population", output_indices=None,
                          output_when="final", integral_weights=W_EXCITED, stop_event=None, precision="mixed")

    def fwd_m():
        plan.solve_batch_device(opts_m, n_traj, d_rho.data_ptr(), slots, d_par.data_ptr(), 1, d_val.data_ptr(),
                                d_st.data_ptr(), stream.cuda_stream)

    cands_m = plan.autotune(opts_m, n_traj, d_rho.data_ptr(), slots, d_par.data_ptr(), 1, probe_steps=64,
                            stream=stream.cuda_stream)
    t_fwd_m = timed(fwd_m)
    w_grad_m, t_grad_m_ck = grad_width("mixed")
    t_grad_m = timed(lambda: grad(precision="mixed"))
    gm = grad(precision="mixed").cpu().numpy()
    plan.set_shape(0, 0)
    # the mixed gradients against the FP64 ones (each form on its own frozen step sequence), on
    # each derivative's natural scale |J| / |p|
    natural = np.abs(j64)[:, None] / np.maximum(np.abs(p), 1e-300)
    mixed_vs_64 = float(np.max(np.abs(gm - g64) / natural))
    return {"workload": f"{n_traj} scan points, d(excited-population integral)/d(rabi, detuning, theta, t_center), "
                        "Tsit5 discrete adjoint", "fwd_ms": 1e3 * t_fwd, "fwd_plus_grad_ms": 1e3 * t_grad,
            "grad_over_fwd": t_grad / t_fwd,
            "autotuned": {"threads_per_trajectory": cands[0]["threads_per_trajectory"],
                          "trajectories_per_cta": cands[0]["trajectories_per_cta"], "fwd_ms": 1e3 * t_fwd_t,
                          "gradient_threads_per_trajectory": w_grad,
                          "fwd_plus_grad_ms": 1e3 * t_grad_t, "grad_over_fwd": t_grad_t / t_fwd_t,
                          "checkpointed_512": {"fwd_plus_grad_ms": 1e3 * t_grad_ck, "grad_over_fwd": t_grad_ck / t_fwd_t,
                                               "tape_bytes_per_trajectory": 8 * plan.grad_tape_doubles(2048, 512),
                                               "full_tape_bytes_per_trajectory": 8 * plan.grad_tape_doubles(2048, 0)}},
            "mixed": {"threads_per_trajectory": cands_m[0]["threads_per_trajectory"],
                      "trajectories_per_cta": cands_m[0]["trajectories_per_cta"], "fwd_ms": 1e3 * t_fwd_m,
                      "gradient_threads_per_trajectory": w_grad_m,
                      "fwd_plus_grad_ms": 1e3 * t_grad_m, "grad_over_fwd": t_grad_m / t_fwd_m,
                      "grad_vs_fp64_fwd": t_grad_m / t_fwd_t,
                      "checkpointed_512": {"fwd_plus_grad_ms": 1e3 * t_grad_m_ck, "grad_over_fwd": t_grad_m_ck / t_fwd_m},
                      "max_grad_diff_vs_fp64_natural_scale": mixed_vs_64,
                      "note": "difference on the scale |J|/|p|, each form on its own step sequence; against central "
                              "differences of its own frozen steps the mixed adjoint agrees to <= 3e-6 relative for "
                              "rabi, detuning and angle, and to ~4e-7 of |J|/|p| for the pulse centre (a derivative "
                              "that cancels to ~1e-4 of that scale) (tests/test_gpu_adjoint.py)"}}


def measure_single(torch, dev, reps: int = 5) -> dict:
    """One trajectory of the 16-state system at its base parameters (peak Rabi Γ, zero detuning,
    z polarisation, Gaussian pulse σ = 20/Γ centred at 100/Γ), Dopri5 rtol 1e-8 atol 1e-11 over
    [0, 200/Γ]: final populations and the excited-population integral through the reference-facing
    single-solve call (host arrays, one call per output as the reference makes them), FP64 and the
    mixed forms, at the automatic launch width (32 threads) and at 64 and 128 threads; against the oracle
    solving the same trajectory on one host thread."""
    import codec
    import oracle
    from centrex_tlf_gb300 import centrex_tlf_rust as api

    d = codec.load("plan_q1_16")
    g, (t0, t1) = d["gamma"], d["t_span"]
    plan = api.prepare_lindblad_problem_py(d["payload"])
    rho0 = d["rho0_packed"]

    def solve(precision):
        # final populations as the reference's solve_lindblad passes them: saveat [t1], no start point
        _, pops, _, st = api.solve_lindblad_ode_py(plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / g, np.array([t1]), False,
                                                   100000, "expanded_sparse", "dopri5", "populations", None, "final",
                                                   None, precision=precision)
        _, integ, _, _ = api.solve_lindblad_ode_py(plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / g, None, True, 100000,
                                                   "expanded_sparse", "dopri5", "excited_population", None, "final",
                                                   W_EXCITED, precision=precision)
        return np.asarray(pops), float(np.asarray(integ).reshape(-1)[-1]), st

    def timed(precision):
        solve(precision)
        best = float("inf")
        for _ in range(reps):
            start = time.perf_counter()
            out = solve(precision)
            best = min(best, time.perf_counter() - start)
        return best, out

    # the fixed cost of one reference-facing call: a solve over one initial step
    _, _, _, st1 = api.solve_lindblad_ode_py(plan, rho0, t0, t0 + 1e-3 / g, 1e-11, 1e-8, 1e-3 / g, None, True, 100000,
                                             "expanded_sparse", "dopri5", "excited_population", None, "final", W_EXCITED)
    call_ms = float("inf")
    for _ in range(reps):
        start = time.perf_counter()
        api.solve_lindblad_ode_py(plan, rho0, t0, t0 + 1e-3 / g, 1e-11, 1e-8, 1e-3 / g, None, True, 100000,
                                  "expanded_sparse", "dopri5", "excited_population", None, "final", W_EXCITED)
        call_ms = min(call_ms, 1e3 * (time.perf_counter() - start))
    res = {}
    for width in (0, 64, 128):
        plan.native.set_shape(width, 0)
        for precision in ("fp64", "mixed", "mixed_fp32_control"):
            res[(width, precision)] = timed(precision)
    plan.native.set_shape(0, 0)
    op = oracle.OraclePlan(d["payload"])
    common = dict(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=None, save_start=True, maxiters=100000,
                  solver="dopri5", output_indices=None, output_when="final", stop_event=None)
    o_pop = op.options(output="populations", integral_weights=None, **{**common, "saveat": np.array([t1]), "save_start": False})
    o_int = op.options(output="excited_population", integral_weights=W_EXCITED, **common)
    cpu_best = float("inf")
    for _ in range(reps):
        start = time.perf_counter()
        _, rp, rst = op.solve_single(o_pop, rho0)
        _, ri, _ = op.solve_single(o_int, rho0)
        cpu_best = min(cpu_best, time.perf_counter() - start)
    ref_pops, ref_int = rp.reshape(-1), float(ri.reshape(-1)[-1])
    out = {"workload": "16-state system at its base parameters, one trajectory, Dopri5 rtol 1e-8 atol 1e-11 over "
                       "[0, 200/Γ]; final populations + excited-population integral (two reference-facing calls, host "
                       "arrays)",
           "oracle_ms": 1e3 * cpu_best, "oracle_cores": 1, "accepted_steps": int(rst["accepted_steps"]),
           "one_step_call_ms": call_ms, "one_step_call_steps": int(st1["accepted_steps"]),
           "rejected_steps": int(rst["rejected_steps"])}
    for (width, precision), (t, (pops, integ, st)) in res.items():
        key = f"{precision}_{'auto_32_threads' if width == 0 else f'{width}_threads'}"
        out[key] = {"ms": 1e3 * t, "vs_oracle_speed": cpu_best / t,
                    "max_population_error_vs_oracle": float(np.max(np.abs(pops - ref_pops))),
                    "excited_integral_rel_error_vs_oracle": abs(integ - ref_int) / abs(ref_int),
                    "accepted_steps": int(st["accepted_steps"])}
    out["note"] = ("one trajectory occupies one thread group: a single solve is latency-bound on the GPU, the batch "
                   "entry points are the throughput path")
    return out


def ragged76_job(total: int, seed: int = 20241205):
    """The ragged 76-state scan: `total` trajectories of the X J=0-3 + B J'=1 system (R(0) and
    P(2) lasers, polarisations switched by 1 MHz square waves), per-laser Rabi U[0.5, 3]Γ and
    detuning N(0, 0.5Γ), end times U[20, 100] µs through a `Time() - t_end` stop event; Tsit5,
    rtol 1e-8, atol 1e-11, final populations."""
    import codec

    d = codec.load("plan_rc_76")
    g = d["gamma"]
    names = d["payload"]["parameter_graph"]["slot_names"]
    rng = np.random.default_rng(seed)
    t_end = rng.uniform(20e-6, 100e-6, total)
    params = np.stack([rng.uniform(0.5, 3.0, total) * g, rng.uniform(0.5, 3.0, total) * g,
                       rng.normal(0.0, 0.5, total) * g, rng.normal(0.0, 0.5, total) * g, t_end], axis=1).astype(np.complex128)
    ev = {"kind": "runtime_expression",
          "expression": {"instructions": [{"op": 4}, {"op": 2, "index": names.index("t_end")}, {"op": 6}],
                         "scalar_only": True, "output_is_tuple": False}}
    return {"d": d, "params": params, "slots": [names.index(s) for s in ("Ω0", "Ω1", "δ0", "δ1", "t_end")],
            "event": ev, "t1": 1.01e-4}


def measure_ragged76(torch, dev, total: int = 1024, cpu_sample: int = 32, fp64_sample: int = 1024) -> dict:
    """The ragged 76-state scan in one persistent launch per form (device-resident, final
    populations at each trajectory's own end time): the mixed forms on all `total` trajectories,
    FP64 on the first `fp64_sample` (its rate and the mixed forms' error against it), each at the
    launch width the autotuner picks on a probe of the batch; the oracle solves the first
    `cpu_sample` trajectories on all host threads, for its rate and for every form's error."""
    import oracle
    from centrex_tlf_gb300.native import NativePlan

    job = ragged76_job(total)
    d, g = job["d"], job["d"]["gamma"]
    f_rhs, per_step = flops_per_step_unit(d["payload"])
    plan = NativePlan(d["payload"])
    stream = torch.cuda.current_stream(dev)
    rho = torch.from_numpy(np.repeat(d["rho0_packed"].reshape(1, -1), total, axis=0)).to(dev)
    par = torch.from_numpy(np.ascontiguousarray(job["params"]).view(np.float64).reshape(-1)).to(dev)
    val = torch.zeros(total * 76, dtype=torch.float64, device=dev)
    st = torch.zeros(total * 6, dtype=torch.int64, device=dev)
    res = {}
    for precision in ("fp64", "mixed", "mixed_fp32_control"):
        count = min(total, fp64_sample) if precision == "fp64" else total
        o = plan.options(t0=0.0, t1=job["t1"], abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=np.array([job["t1"]]),
                         save_start=False, maxiters=1000000, solver="tsit5", output="populations", output_indices=None,
                         output_when="final", integral_weights=None, stop_event=job["event"], precision=precision)
        plan.set_shape(0, 0)
        cands = plan.autotune(o, count, rho.data_ptr(), job["slots"], par.data_ptr(), 1, probe_steps=64,
                              stream=stream.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.solve_batch_device(o, count, rho.data_ptr(), job["slots"], par.data_ptr(), 1, val.data_ptr(),
                                st.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        stv = st.view(-1, 6)[:count].cpu().numpy()
        if np.any(stv[:, 3] >> 32):
            raise RuntimeError(f"{int(np.count_nonzero(stv[:, 3] >> 32))} 76-state trajectories failed ({precision})")
        ms = e0.elapsed_time(e1)
        attempted = int(stv[:, 0].sum()) + int(stv[:, 1].sum())
        res[precision] = {"ms": ms, "trajectories": count, "value": count / (ms * 1e-3), "unit": "trajectories/s",
                          "threads_per_trajectory": cands[0]["threads_per_trajectory"],
                          "accepted_steps": int(stv[:, 0].sum()), "rejected_steps": int(stv[:, 1].sum()),
                          # algorithmic work (6 F_rhs + 60 N per attempted step) over the launch
                          "achieved_tflops": attempted * per_step / (ms * 1e-3) / 1e12,
                          "pops": val.view(total, 76)[:count].cpu().numpy().copy()}
    plan.set_shape(0, 0)
    op = oracle.OraclePlan(d["payload"])
    o = op.options(t0=0.0, t1=job["t1"], abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=np.array([job["t1"]]),
                   save_start=False, maxiters=1000000, solver="tsit5", output="populations", output_indices=None,
                   output_when="final", integral_weights=None, stop_event=job["event"])
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), cpu_sample, axis=0)
    start = time.perf_counter()
    ref, _, rst = op.solve_batch(o, rho0, job["slots"], job["params"][:cpu_sample])
    cpu_s = time.perf_counter() - start
    ref = ref.reshape(cpu_sample, 76)
    out = {"workload": f"{total} trajectories of the 76-state system, square-wave polarisation switching at 1 MHz, "
                       "end times U[20, 100] µs by stop event, Tsit5 rtol 1e-8 atol 1e-11, final populations; "
                       f"device-resident, one launch per form (FP64 on the first {min(total, fp64_sample)})",
           "cpu_oracle": {"value": cpu_sample / cpu_s, "unit": "trajectories/s", "cores": int(oracle.max_threads()),
                          "sample": f"first {cpu_sample} trajectories", "accepted_steps": int(rst["accepted_steps"].sum())}}
    for precision, r in res.items():
        pops = r.pop("pops")
        r["max_population_error_vs_oracle"] = float(np.max(np.abs(pops[:cpu_sample] - ref)))
        r["max_trace_drift"] = float(np.max(np.abs(pops.sum(axis=1) - 1.0)))
        r["speedup_vs_cpu_oracle"] = r["value"] / out["cpu_oracle"]["value"]
        out[precision] = r
        res[precision]["_pops"] = pops
    nf = res["fp64"]["_pops"].shape[0]
    for precision in ("mixed", "mixed_fp32_control"):
        out[precision]["max_population_error_vs_fp64_gpu"] = float(np.max(np.abs(res[precision]["_pops"][:nf] - res["fp64"]["_pops"])))
        out[precision]["speedup_vs_fp64_gpu"] = out[precision]["value"] / out["fp64"]["value"]
    for r in res.values():
        r.pop("_pops", None)
    out["note"] = ("the square-wave switching makes the RHS discontinuous; solves agree with the oracle to the "
                   "solver tolerance there (step landings at the jumps), not to rounding; achieved_tflops counts "
                   f"6*F_rhs + 60*N flop per attempted step (F_rhs = {f_rhs}, N = {76 * 76})")
    return out


def hetero_oracle_sample(spec, prepared, torch, dev, per_plan: int = 6) -> dict:
    """The oracle on the first `per_plan` instances of each plan of the heterogeneous batch (all
    host threads): its rate, and the max final-population error of both GPU forms against it."""
    import oracle

    stream = torch.cuda.current_stream(dev)
    total_s, total_n, errs = 0.0, 0, {"mixed": 0.0, "fp64": 0.0}
    for j, (plan, _, b, rho, slots, par, _, st) in zip(spec, prepared):
        k = min(per_plan, b)
        if k == 0:
            continue
        d, g = j["d"], j["d"]["gamma"]
        n = d["payload"]["n_states"]
        o_kw = dict(t0=0.0, t1=j["t1"], abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=np.array([j["t1"]]),
                    save_start=False, maxiters=1000000, solver="tsit5", output="populations", output_indices=None,
                    output_when="final", integral_weights=None, stop_event=j["event"])
        op = oracle.OraclePlan(d["payload"])
        rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), k, axis=0)
        start = time.perf_counter()
        ref, _, _ = op.solve_batch(op.options(**o_kw), rho0, j["slots"], j["params"][:k])
        total_s += time.perf_counter() - start
        total_n += k
        pv = torch.zeros(k * n, dtype=torch.float64, device=dev)
        for prec in errs:
            plan.solve_batch_device(plan.options(precision=prec, **o_kw), k, rho.data_ptr(), slots, par.data_ptr(), 1,
                                    pv.data_ptr(), st.data_ptr(), stream.cuda_stream)
            torch.cuda.synchronize()
            errs[prec] = max(errs[prec], float(np.max(np.abs(pv.view(k, n).cpu().numpy() - ref.reshape(k, n)))))
    return {"cpu_oracle": {"value": total_n / total_s, "unit": "trajectories/s", "cores": int(oracle.max_threads()),
                           "sample": f"first {per_plan} instances of each plan ({total_n} in all)"},
            "max_population_error_vs_oracle": errs}


HETERO_PLANS = (("plan_q1_16_tend", 6), ("plan_r0_39", 3), ("plan_rc_76", 1))
FORMS = ("fp64", "mixed", "mixed_fp32_control")
FORM_NOTES = {
    "fp64": "every operation in double precision (the drop-in form)",
    "mixed": "single-precision RHS products (stage deviations); stage combinations, state accumulation, error "
             "norm (ratios, sum, norm) and step-size controller in double, trace renormalised in double",
    "mixed_fp32_control": "single-precision RHS products and stage inputs, error norm and controller in single "
                          "precision; state accumulation in double; no renormalisation",
}


def hetero_jobs(total: int, seed: int = 20241204, t_end_range=(50.0, 300.0)):
    """The heterogeneous batch: `total` instances drawn 6:3:1 from the 16-state (Q(1)), 39-state
    (R(0), X J=0-2) and 76-state (R(0) + P(2), square-wave polarisation) plans; parameters as in
    the 16-state scan (peak Rabi Γ·10^U[-1,1], detuning U[-5Γ, 5Γ], angle U[0, π]) or, for the
    76-state plan, per-laser Rabi U[0.5, 3]Γ and detuning N(0, 0.5Γ); end times U[50, 300]/Γ through
    a `Time() - t_end` stop event; Tsit5, rtol 1e-8, atol 1e-11, excited-population integral."""
    import codec

    rng = np.random.default_rng(seed)
    kinds = rng.choice(len(HETERO_PLANS), size=total, p=np.array([w for _, w in HETERO_PLANS]) / 10.0)
    jobs = []
    for k, (name, _) in enumerate(HETERO_PLANS):
        count = int(np.sum(kinds == k))
        d = codec.load(name)
        g = d["gamma"]
        names = d["payload"]["parameter_graph"]["slot_names"]
        if name == "plan_rc_76":
            slot_names = ["Ω0", "Ω1", "δ0", "δ1", "t_end"]
            cols = [rng.uniform(0.5, 3.0, count) * g, rng.uniform(0.5, 3.0, count) * g,
                    rng.normal(0.0, 0.5, count) * g, rng.normal(0.0, 0.5, count) * g]
        else:
            slot_names = ["rabi", "detuning", "theta", "t_end"]
            cols = [g * 10 ** rng.uniform(-1.0, 1.0, count), rng.uniform(-5.0, 5.0, count) * g,
                    rng.uniform(0.0, np.pi, count)]
        t_end = rng.uniform(*t_end_range, count) / g
        params = np.stack(cols + [t_end], axis=1).astype(np.complex128)
        ev = {"kind": "runtime_expression",
              "expression": {"instructions": [{"op": 4}, {"op": 2, "index": names.index("t_end")}, {"op": 6}],
                             "scalar_only": True, "output_is_tuple": False}}
        jobs.append({"name": name, "d": d, "count": count, "params": params,
                     "slots": [names.index(s) for s in slot_names], "event": ev,
                     "t1": 1.01 * t_end_range[1] / g, "weights": [(i, 1.0) for i in d["excited_indices"]]})
    return jobs


def measure_heterogeneous(torch, dev, total: int = 8192, reps: int = 1) -> dict:
    """The heterogeneous batch, device-resident, through obe_solve_multi_device (one call, the
    three plans' kernels concurrent): the mixed form timed after one untimed call, the same jobs
    as three single-plan calls in a row on one stream (what a caller of the reference's
    one-plan-per-call API does), and the FP64 form once, for the error of the mixed form."""
    from centrex_tlf_gb300.native import MultiGraph, NativePlan, multi_solve_device

    spec = hetero_jobs(total)
    stream = torch.cuda.current_stream(dev)
    prepared = []
    for j in spec:
        d = j["d"]
        plan = NativePlan(d["payload"])
        g = d["gamma"]
        opts = {prec: plan.options(t0=0.0, t1=j["t1"], abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=None,
                                   save_start=True, maxiters=1000000, solver="tsit5", output="excited_population",
                                   output_indices=None, output_when="final", integral_weights=j["weights"],
                                   stop_event=j["event"], precision=prec)
                for prec in ("mixed", "fp64")}
        b = j["count"]
        rho = torch.from_numpy(np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0)).to(dev)
        par = torch.from_numpy(np.ascontiguousarray(j["params"]).view(np.float64).reshape(-1)).to(dev)
        val = {prec: torch.zeros(b, dtype=torch.float64, device=dev) for prec in opts}
        st = torch.zeros(b * 6, dtype=torch.int64, device=dev)
        prepared.append((plan, opts, b, rho, j["slots"], par, val, st))

    def multi(prec):
        return multi_solve_device([(pl, o[prec], b, r.data_ptr(), sl, pa.data_ptr(), 1, v[prec].data_ptr(), s.data_ptr())
                                   for pl, o, b, r, sl, pa, v, s in prepared], stream.cuda_stream)

    def sequential(prec):
        for pl, o, b, r, sl, pa, v, s in prepared:
            pl.solve_batch_device(o[prec], b, r.data_ptr(), sl, pa.data_ptr(), 1, v[prec].data_ptr(), s.data_ptr(),
                                  stream.cuda_stream)
        return len(prepared)

    def timed(fn, prec, warm=True):
        if warm:
            fn(prec)
            torch.cuda.synchronize()
        best, launches = float("inf"), 0
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            launches = fn(prec)
            e1.record(stream)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) * 1e-3)
        return best, launches

    t_multi, launches = timed(multi, "mixed")
    failed = sum(int(np.count_nonzero(s.view(-1, 6)[:, 3].cpu().numpy() >> 32)) for *_, s in prepared)
    steps = [int(s.view(-1, 6)[:, 0].sum().item()) for *_, s in prepared]
    t_seq, _ = timed(sequential, "mixed", warm=False)
    # the same batch recorded once as a CUDA graph (obe_multi_graph), replayed as one launch
    graph = MultiGraph([(pl, o["mixed"], b, r.data_ptr(), sl, pa.data_ptr(), 1, v["mixed"].data_ptr(), s.data_ptr())
                        for pl, o, b, r, sl, pa, v, s in prepared])
    t_graph, _ = timed(lambda prec: graph.launch(stream.cuda_stream), "mixed")
    graph.close()
    t_64, _ = timed(multi, "fp64", warm=False)
    sample = hetero_oracle_sample(spec, prepared, torch, dev)
    err = 0.0
    for j, (*_, val, _) in zip(spec, prepared):
        t_end = j["params"][:, -1].real
        dv = (val["mixed"] - val["fp64"]).abs().cpu().numpy()
        err = max(err, float(np.max(dv / t_end)))
    return {
        "workload": f"{total} instances, 16/39/76-state plans drawn 6:3:1, end times U[50, 300]/Γ by stop event, "
                    "Tsit5 rtol 1e-8 atol 1e-11, excited-population integral; mixed precision; device-resident",
        "value": total / t_multi, "unit": "trajectories/s", "ms": 1e3 * t_multi, "gpu_launches": launches,
        "instances": {j["name"]: j["count"] for j in spec},
        "accepted_steps": {j["name"]: n for j, n in zip(spec, steps)},
        "failed_trajectories": failed,
        "one_call_per_plan_ms": 1e3 * t_seq, "concurrency_gain": t_seq / t_multi,
        "cuda_graph_ms": 1e3 * t_graph,
        "fp64_ms": 1e3 * t_64, "speedup_of_mixed": t_64 / t_multi,
        "max_time_averaged_population_error_vs_fp64": err,
        "cpu_oracle": sample["cpu_oracle"],
        "speedup_vs_cpu_oracle": (total / t_multi) / sample["cpu_oracle"]["value"],
        "max_population_error_vs_oracle": sample["max_population_error_vs_oracle"],
        "note": "fp64 timed on its first call (plans already on the device); the time-averaged error is |integral "
                "difference| / t_end; the population errors are final populations at each instance's end time on "
                "the oracle's sample",
    }


def measure_hetero_gradient(torch, dev, total: int = 8192, precision: str = "mixed", reps: int = 1) -> dict:
    """Forward plus adjoint of the heterogeneous batch: for each of the three plans,
    d(excited-population integral)/d(its scanned slots, the end time included) through the
    discrete adjoint (the event step and the event time's derivative included), checkpointed tape
    (a start state every 512 steps) where the full one would pass 4 GiB; against the same plans'
    plain forward solves, one call per plan."""
    from centrex_tlf_gb300.autograd import solve_batch_with_grad
    from centrex_tlf_gb300.native import NativePlan

    spec = hetero_jobs(total)
    stream = torch.cuda.current_stream(dev)
    runs = []
    for j in spec:
        d = j["d"]
        plan = NativePlan(d["payload"])
        g = d["gamma"]
        opts = plan.options(t0=0.0, t1=j["t1"], abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=None, save_start=True,
                            maxiters=1000000, solver="tsit5", output="excited_population", output_indices=None,
                            output_when="final", integral_weights=j["weights"], stop_event=j["event"], precision=precision)
        b = j["count"]
        rho = torch.from_numpy(np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0)).to(dev)
        par = torch.from_numpy(np.ascontiguousarray(j["params"]).view(np.float64).reshape(-1)).to(dev)
        val = torch.zeros(b, dtype=torch.float64, device=dev)
        st = torch.zeros(b * 6, dtype=torch.int64, device=dev)
        runs.append((j, plan, opts, b, rho, par, val, st))

    def fwd():
        for j, plan, opts, b, rho, par, val, st in runs:
            plan.solve_batch_device(opts, b, rho.data_ptr(), j["slots"], par.data_ptr(), 1, val.data_ptr(), st.data_ptr(),
                                    stream.cuda_stream)

    per_plan = {}
    grads = {}
    ckpts = {}  # the tape length and checkpoint interval the wrapper chose per plan

    def max_steps_of(j):
        return 8192 if j["name"] == "plan_rc_76" else 2048

    def grad():
        for j, plan, opts, b, rho, par, val, st in runs:
            t = time.perf_counter()
            pt = torch.tensor(j["params"].real, dtype=torch.float64, device=dev, requires_grad=True)
            out, tape = solve_batch_with_grad(plan, rho, (0.0, j["t1"]), pt, j["slots"], dt=1e-3 / j["d"]["gamma"],
                                              maxiters=1000000, integral_weights=j["weights"], stop_event=j["event"],
                                              precision=precision, max_steps=max_steps_of(j), return_tape=True)
            ckpts[j["name"]] = (tape.max_steps, tape.checkpoint_every)
            out.sum().backward()
            torch.cuda.synchronize()
            assert bool(torch.isfinite(pt.grad).all()), j["name"]
            per_plan[j["name"]] = 1e3 * (time.perf_counter() - t)
            grads[j["name"]] = pt.grad

    # the three plans' gradients concurrently: each plan's taped forward and reverse sweep on its
    # own stream through the C ABI (obe_grad_forward / obe_grad_backward), one host synchronisation
    # between the forwards and the reverse sweeps
    conc = []
    for j, plan, opts, b, rho, par, val, st in runs:
        ms = max_steps_of(j)
        conc.append(dict(j=j, plan=plan, opts=opts, b=b, rho=rho, ms=ms, stream=torch.cuda.Stream(dev),
                         stats=torch.zeros(b * 6, dtype=torch.int64, device=dev),
                         pv=torch.from_numpy(np.ascontiguousarray(j["params"]).view(np.float64).reshape(-1)).to(dev),
                         out=torch.zeros(b, dtype=torch.float64, device=dev), og=torch.ones(b, dtype=torch.float64, device=dev),
                         pg=torch.zeros(b, len(j["slots"]), dtype=torch.float64, device=dev),
                         ast=torch.zeros(b, dtype=torch.int32, device=dev)))

    def grad_concurrent():
        for c in conc:
            if "tape" not in c:
                c["ms"], c["ck"] = ckpts[c["j"]["name"]]
                c["tape"] = torch.empty(c["b"] * c["plan"].grad_tape_doubles(c["ms"], c["ck"], precision),
                                        dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        for c in conc:
            c["plan"].grad_forward(c["opts"], c["b"], c["rho"].data_ptr(), c["j"]["slots"], c["pv"].data_ptr(), c["ms"],
                                   c["tape"].data_ptr(), c["out"].data_ptr(), c["stats"].data_ptr(), c["stream"].cuda_stream,
                                   checkpoint_every=c["ck"])
        torch.cuda.synchronize()
        for c in conc:
            stv = c["stats"].view(-1, 6).cpu().numpy()
            assert not np.any(stv[:, 3] >> 32) and int(stv[:, 0].max()) < c["ms"], c["j"]["name"]
            c["plan"].grad_backward(c["opts"], c["b"], c["rho"].data_ptr(), c["j"]["slots"], c["pv"].data_ptr(),
                                    c["j"]["slots"], c["ms"], c["tape"].data_ptr(), c["stats"].data_ptr(), c["og"].data_ptr(),
                                    c["pg"].data_ptr(), None, c["ast"].data_ptr(), c["stream"].cuda_stream,
                                    checkpoint_every=c["ck"])
        torch.cuda.synchronize()
        for c in conc:
            assert not bool(c["ast"].any()), c["j"]["name"]

    def timed(fn):
        best = float("inf")
        for _ in range(reps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t)
        return best

    fwd()
    torch.cuda.synchronize()
    t_fwd = timed(fwd)
    grad()  # untimed: device buffers (tapes, segment buffers) allocated once
    t_grad = timed(grad)
    grad_concurrent()  # untimed, as above
    t_conc = timed(grad_concurrent)
    # the same gradients either way (each trajectory's arithmetic does not depend on the schedule)
    same = all(torch.equal(c["pg"], grads[c["j"]["name"]]) for c in conc)
    return {"workload": f"{total} instances of the heterogeneous batch (16/39/76-state plans 6:3:1, end times "
                        "U[50, 300]/Γ by a Time() - t_end stop event); d(excited-population integral)/d(Rabi rates, "
                        "detunings, angle, t_end) per instance, Tsit5 discrete adjoint, " + precision,
            "instances": {j["name"]: j["count"] for j in spec}, "fwd_ms": 1e3 * t_fwd, "fwd_plus_grad_ms": 1e3 * t_grad,
            "grad_over_fwd": t_grad / t_fwd, "fwd_plus_grad_ms_per_plan": per_plan,
            "concurrent_fwd_plus_grad_ms": 1e3 * t_conc, "concurrent_grad_over_fwd": t_conc / t_fwd,
            "concurrent_gradients_identical": bool(same),
            "note": "forward = the three plans' plain solves one call each (device-resident); gradient = "
                    "solve_batch_with_grad + backward per plan (host-synchronised between the tape check and the "
                    "reverse sweep), timed after one untimed call; concurrent = the three plans' taped forwards on "
                    "their own streams, one synchronisation, then their reverse sweeps on their streams; the "
                    "76-state trajectories (checkpointed tape) dominate both"}


def measure_effective(torch, dev, total: int = 4096, cpu_sample: int = 256, reps: int = 2) -> dict:
    """The interpolated effective-Hamiltonian path (solve_effective_lindblad_batch_py): the R(0)
    compact model of tests/golden/plan_eff_r0.json (10 states, split-real state of 200 doubles,
    field oscillating across the 100-200 V/cm operator grid), `total` trajectories with seeded
    Rabi rates U[0.3, 2]·1e7 and detunings U[-5, 5]·1e6, Tsit5 rtol 1e-7 atol 1e-9 over 5 µs, the
    excited-population integral; host arrays in and out (the reference-facing call), against the
    FP64 oracle on a sample on all host threads."""
    import codec
    import oracle
    from centrex_tlf_gb300 import centrex_tlf_rust as api

    d = codec.load("plan_eff_r0")
    plan = api.prepare_effective_lindblad_plan_py(d["plan"])
    rng = np.random.default_rng(20241205)
    pb = np.stack([rng.uniform(0.3e7, 2.0e7, total), rng.uniform(-5e6, 5e6, total)], axis=1)
    w = [(i * 11, 1.0) for i in (7, 8, 9)]
    t0, t1 = d["t_span"]

    def run():
        return api.solve_effective_lindblad_batch_py(plan, d["y0"], t0, t1, 1e-9, 1e-7, 1e-10, None, True, 100000, "tsit5",
                                                     "excited_population", None, w, [0, 1], pb, total)

    run()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        start = time.perf_counter()
        out = run()
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - start)
    op = oracle.EffectiveOraclePlan(d["plan"])
    o = op.options(t0=t0, t1=t1, abstol=1e-9, reltol=1e-7, dt=1e-10, saveat=None, save_start=True, maxiters=100000,
                   solver="tsit5", output="excited_population", output_indices=None, integral_weights=w,
                   output_when="final")
    start = time.perf_counter()
    ref, _, _ = op.solve_batch(o, d["y0"], [0, 1], pb[:cpu_sample].astype(complex))
    cpu_s = time.perf_counter() - start
    vals = np.asarray(out[1])[:cpu_sample]
    rel = float(np.max(np.abs(vals - ref.reshape(-1)) / np.abs(ref.reshape(-1))))
    return {"workload": f"{total} trajectories of the 10-state R(0) interpolated effective model, Tsit5, "
                        "excited-population integral, host arrays in and out",
            "value": total / best, "unit": "trajectories/s", "ms": 1e3 * best,
            "accepted_steps": int(out[4]["accepted_steps"]),
            "cpu_oracle": {"value": cpu_sample / cpu_s, "unit": "trajectories/s", "cores": int(oracle.max_threads()),
                           "sample": cpu_sample},
            "max_rel_err_vs_cpu_oracle": rel}


def run_gpu(args) -> None:
    import torch

    from centrex_tlf_gb300 import _abi
    from centrex_tlf_gb300 import centrex_tlf_rust as api

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    from centrex_tlf_gb300.sharding import max_over_ranks, shard_bounds

    d, params_all, slots = workload(args.points * world)
    lo, hi = shard_bounds(args.points, rank)  # weak scaling: one shard of the scan per rank
    params = params_all[lo:hi]
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    b = params.shape[0]
    plan = api.prepare_lindblad_problem_py(d["payload"])
    native = plan.native
    opts = native.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, saveat=None, save_start=True,
                          maxiters=100000, solver="tsit5", output="excited_population", output_indices=None,
                          output_when="final", integral_weights=W_EXCITED, stop_event=None, precision=args.precision)
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0)
    d_rho = torch.from_numpy(rho0).to(dev)
    d_par = torch.from_numpy(np.ascontiguousarray(params).view(np.float64).reshape(-1)).to(dev)
    d_val = torch.zeros(b, dtype=torch.float64, device=dev)
    d_st = torch.zeros(b * 6, dtype=torch.int64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    stream = torch.cuda.current_stream(dev)

    def timed(o, steps, sampler=None):
        """Warm-up, then `steps` device-resident solves of the batch, L2 flushed before each;
        returns (per-step ms, attempted steps of the last solve)."""
        def step():
            native.solve_batch_device(o, b, d_rho.data_ptr(), slots, d_par.data_ptr(), 1, d_val.data_ptr(),
                                      d_st.data_ptr(), stream.cuda_stream)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        with sampler if sampler is not None else contextlib.nullcontext():
            torch.cuda.synchronize()
            for i in range(steps):
                flush.zero_()
                starts[i].record(stream)
                step()
                ends[i].record(stream)
            torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        st = d_st.view(b, 6).cpu().numpy()
        status = st[:, 3] >> 32
        if np.any(status != 0):
            raise RuntimeError(f"{int(np.count_nonzero(status))} trajectories failed on the GPU")
        return [s.elapsed_time(e) for s, e in zip(starts, ends)], int(st[:, 0].sum() + st[:, 1].sum())

    clock_path = Path(tempfile.gettempdir()) / f"obe_clocks_{os.getpid()}.csv"
    sampler = ClockSampler(clock_path)
    ms, attempted = timed(opts, args.steps, sampler)
    launches_per_step = native.launches()  # the integrator and, for a batch in several waves, its queue ordering
    # the other precision forms on the same batch: the plain FP64 path (the speed ratios' base) and
    # the mixed forms not timed as the headline
    form_ms = {args.precision: (ms, attempted)}
    if not args.no_fp64_compare:
        for form in FORMS:
            if form in form_ms:
                continue
            o_f = native.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma, saveat=None, save_start=True,
                                 maxiters=100000, solver="tsit5", output="excited_population", output_indices=None,
                                 output_when="final", integral_weights=W_EXCITED, stop_event=None, precision=form)
            form_ms[form] = timed(o_f, args.steps)
    other = form_ms.get("fp64") if args.precision != "fp64" else None
    total_s = sum(ms) * 1e-3
    total64_s = sum(other[0]) * 1e-3 if other else 0.0
    total_s, total64_s = max_over_ranks([total_s, total64_s], device=dev)
    value = b * world * args.steps / total_s
    launches = args.steps * launches_per_step  # obe_last_launch_count of the headline solve, per step

    # e2e: the reference-facing call with host arrays, copies inside the timed region
    e2e_s = []
    h2d = rho0.nbytes + params.nbytes + b * 0
    for i in range(args.steps + 1):
        torch.cuda.synchronize()
        t_s = time.perf_counter()
        out = api.solve_lindblad_batch_ode_py(plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / gamma, solver="tsit5",
                                              output="excited_population", integral_weights=W_EXCITED,
                                              parameter_slot_indices=slots, parameter_batch=params,
                                              precision=args.precision)
        torch.cuda.synchronize()
        if i > 0:
            e2e_s.append(time.perf_counter() - t_s)
    d2h = b * 8 + b * _abi.TRAJ_STATS_DTYPE.itemsize + b * 24
    e2e_value = b * world * len(e2e_s) / sum(e2e_s)

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # accuracy of this precision against the plain FP64 GPU path (final populations, all points)
    def pops(precision):
        _, v, _, _, _ = api.solve_lindblad_batch_ode_py(plan, rho0, t0, t1, 1e-11, 1e-8, 1e-3 / gamma, solver="tsit5",
                                                        output="populations", parameter_slot_indices=slots,
                                                        parameter_batch=params, precision=precision)
        return np.asarray(v).reshape(b, 16)

    p64 = pops("fp64")
    pm = p64 if args.precision == "fp64" else pops(args.precision)
    max_pop_err = float(np.max(np.abs(pm - p64)))
    form_pops = {f: (p64 if f == "fp64" else (pm if f == args.precision else pops(f))) for f in form_ms}
    # per-result diagnostics the solve reports beside its error: trace drift of the final state
    # (|sum of populations - 1|; rho0 has unit trace) for both forms, and the error of both forms
    # against the FP64 oracle on the CPU-baseline sample
    p_orc = cpu_oracle_populations(d, params, slots, args.cpu_sample)
    accuracy = {
        "max_population_error_vs_fp64_gpu": max_pop_err,
        "max_population_error_vs_fp64_oracle": float(np.max(np.abs(pm[: args.cpu_sample] - p_orc))),
        "max_population_error_fp64_gpu_vs_fp64_oracle": float(np.max(np.abs(p64[: args.cpu_sample] - p_orc))),
        "max_trace_drift": float(np.max(np.abs(pm.sum(axis=1) - 1.0))),
        "max_trace_drift_fp64_gpu": float(np.max(np.abs(p64.sum(axis=1) - 1.0))),
        "hermiticity_residual": 0.0,
        "hermiticity_note": "the state is the packed upper triangle (real diagonal, re/im pairs above it), "
                            "so the density matrix it stands for is Hermitian by construction",
        "oracle_sample": args.cpu_sample,
    }
    # and the observable against the CPU oracle on a sample (also the CPU baseline)
    cpu = cpu_oracle_rate(d, params, slots, args.cpu_sample)
    gradient = measure_gradient(torch, d, params, dev) if not args.no_gradient else None
    hetero = measure_heterogeneous(torch, dev, total=args.hetero_instances) if args.hetero_instances > 0 else None
    effective = measure_effective(torch, dev) if not args.no_effective else None
    single = measure_single(torch, dev) if not args.no_single else None
    ragged = measure_ragged76(torch, dev, total=args.ragged_instances) if args.ragged_instances > 0 else None
    hetero_grad = (measure_hetero_gradient(torch, dev, total=args.hetero_grad_instances)
                   if args.hetero_grad_instances > 0 else None)
    gpu_obs = np.asarray(out[1])[: args.cpu_sample]
    obs_rel = float(np.max(np.abs(gpu_obs - cpu["values"]) / np.maximum(np.abs(cpu["values"]), 1e-300)))
    accuracy["observable_max_rel_err_vs_cpu_oracle"] = obs_rel
    forms = {}
    rate64 = b * world * args.steps / (sum(form_ms["fp64"][0]) * 1e-3) if "fp64" in form_ms else None
    for f, (f_ms, f_att) in form_ms.items():
        rate = b * world * args.steps / (sum(f_ms) * 1e-3)
        fp = form_pops[f]
        forms[f] = {"value": rate, "unit": "trajectories/s", "ms_per_step": sum(f_ms) / len(f_ms),
                    "attempted_steps_per_launch": f_att, "speedup_vs_fp64_gpu": rate / rate64 if rate64 else None,
                    "max_population_error_vs_fp64_gpu": float(np.max(np.abs(fp - p64))),
                    "max_population_error_vs_fp64_oracle": float(np.max(np.abs(fp[: args.cpu_sample] - p_orc))),
                    "max_trace_drift": float(np.max(np.abs(fp.sum(axis=1) - 1.0))),
                    "note": FORM_NOTES[f]}
    f_rhs, per_step = flops_per_step_unit(d["payload"])
    flops_per_launch = attempted * per_step
    kernel_s = (sum(ms) / len(ms)) * 1e-3
    achieved = flops_per_launch / kernel_s / 1e12
    mixed = args.precision != "fp64"
    peak = measure_gemm_peak(torch, dev, torch.float32 if mixed else torch.float64)
    clocks = sampler.summary(local)
    # the HBM view of the same launch against the measured copy bandwidth (MEASURED_PEAKS.json,
    # else the machine's fallback figure): how far the kernel is from being memory-bound
    peaks_file = Path(__file__).resolve().parent / "MEASURED_PEAKS.json"
    hbm_peak, hbm_src = 6800.0, "fallback"
    if peaks_file.exists():
        try:
            hbm_peak, hbm_src = float(json.loads(peaks_file.read_text())["hbm_gbs"]), "measured"
        except (ValueError, KeyError):
            pass
    traffic_launch = TRAFFIC_BYTES_PER_TRAJECTORY["fp64" if args.precision == "fp64" else "mixed"] * b
    hbm_achieved = traffic_launch / kernel_s / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "trajectories/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum(ms) / len(ms), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32-rhs/f64-accumulate",
        "data": "synthetic (seeded scan of the reference-built 16-state plan)",
        "config": {"workload": f"q1_16state_gaussian_scan_{args.points}pt_tsit5", "points_per_gpu": b, "solver": "tsit5",
                   "rtol": 1e-8, "atol": 1e-11, "precision": args.precision, "l2": "flushed (256 MB write) between steps",
                   "attempted_steps_per_launch": attempted},
        "e2e": {"value": e2e_value, "unit": "trajectories/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "api": "centrex_tlf_rust.solve_lindblad_batch_ode_py (host numpy in/out)"},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32" if mixed else "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     "traffic": TRAFFIC_BYTES_PER_TRAJECTORY["fp64" if args.precision == "fp64" else "mixed"] * b,
                     "note": "algorithmic FLOPs (6*F_rhs + 60*N per attempted step, F_rhs = "
                             f"{f_rhs}) / mean launch time; peak = cuBLAS "
                             + ("SGEMM (TF32 off: the FP32 pipe the mixed form's products run on)" if mixed else "DGEMM")
                             + " measured in this run (the driver's peak file has HBM and bf16 only); traffic = ncu DRAM "
                             "read+write bytes per trajectory of this kernel, scaled to the launch",
                     "hbm": {"bound": "hbm", "achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s",
                             "frac": hbm_achieved / hbm_peak, "traffic": traffic_launch,
                             "peak_source": hbm_src + " copy bandwidth",
                             "note": "DRAM bytes per launch (ncu) / mean launch time: the kernel is not HBM-bound"}},
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "fp64_gpu": ({"value": b * world * args.steps / total64_s, "unit": "trajectories/s",
                      "ms_per_step": sum(other[0]) / len(other[0]), "attempted_steps_per_launch": other[1],
                      "speedup_of_this_precision": (b * world * args.steps / total_s) / (b * world * args.steps / total64_s)}
                     if other else None),
        "accuracy": accuracy,
        "forms": forms,
        "clocks": clocks,
        "gradient": gradient,
        "heterogeneous": hetero,
        "heterogeneous_gradient": hetero_grad,
        "effective": effective,
        "single_solve": single,
        "ragged_76": ragged,
    }
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def measure_dense76(torch, dev, total: int = 1024, reps: int = 5) -> dict:
    """The tensor-core question for the 76-state system: the dense commutator -i[H, rho] of a batch of
    states, H = static + sum_k c_k B_k assembled per state, as batched complex GEMMs on cuBLAS
    (complex64 with TF32 tensor cores, complex64 on the FP32 pipe, and the real/imaginary split in
    bf16 on the tensor cores, the fastest and least precise stand-in), against this package's
    sparse gather RHS (obe_rhs_eval, FP64 and the mixed form's single-precision products) on the
    same states.  Device times of every kernel come from an ncu launch list of this case."""
    import codec
    from centrex_tlf_gb300.native import NativePlan

    d = codec.load("plan_rc_76")
    hp = d["payload"]["hamiltonian_plan"]
    n = int(d["payload"]["n_states"])
    basis = []
    for c in hp["coefficients"]:
        m = np.zeros((n, n), dtype=np.complex128)
        for t in c["basis_terms"]:
            m[t["i"], t["j"]] += t["re"] + 1j * t["im"]
        basis.append(m)
    k = len(basis)
    rng = np.random.default_rng(76)
    g = d["gamma"]
    coeffs = (rng.normal(size=(total, k)) + 1j * rng.normal(size=(total, k))) * g
    rho = rng.normal(size=(total, n, n)) + 1j * rng.normal(size=(total, n, n))
    rho = (rho + rho.conj().transpose(0, 2, 1)) / (2 * n)
    S = torch.tensor(np.asarray(hp["static_matrix"]), dtype=torch.complex64, device=dev)
    Bk = torch.tensor(np.stack(basis).reshape(k, n * n), dtype=torch.complex64, device=dev)
    C = torch.tensor(coeffs, dtype=torch.complex64, device=dev)
    R = torch.tensor(rho, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def commutator():
        H = (C @ Bk).view(total, n, n) + S
        return -1j * (torch.bmm(H, R) - torch.bmm(R, H))

    def commutator_bf16():
        H = (C @ Bk).view(total, n, n) + S
        hr, hi = H.real.to(torch.bfloat16), H.imag.to(torch.bfloat16)
        rr, ri = R.real.to(torch.bfloat16), R.imag.to(torch.bfloat16)
        a_re = torch.bmm(hr, rr) - torch.bmm(hi, ri)
        a_im = torch.bmm(hr, ri) + torch.bmm(hi, rr)
        b_re = torch.bmm(rr, hr) - torch.bmm(ri, hi)
        b_im = torch.bmm(rr, hi) + torch.bmm(ri, hr)
        return (a_im - b_im), -(a_re - b_re)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    tf32 = torch.backends.cuda.matmul.allow_tf32
    try:
        torch.backends.cuda.matmul.allow_tf32 = True
        t_tf32 = timed(commutator)
        torch.backends.cuda.matmul.allow_tf32 = False
        t_fp32 = timed(commutator)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = tf32
    t_bf16 = timed(commutator_bf16)
    # this package's tcgen05 kernel on the same states (H assembled by the same GEMM)
    import ctypes

    from centrex_tlf_gb300 import _abi

    lib = _abi.load_library()
    H_all = ((C @ Bk).view(total, n, n) + S).contiguous()
    out_tc = torch.empty_like(R)
    status = torch.zeros(1, dtype=torch.int32, device=dev)

    def commutator_tcgen05():
        H = ((C @ Bk).view(total, n, n) + S).contiguous()
        rc = lib.obe_dense_commutator_tf32(total, n, H.data_ptr(), R.data_ptr(), out_tc.data_ptr(), status.data_ptr(),
                                           ctypes.c_void_p(stream.cuda_stream))
        if rc != _abi.OBE_OK:
            raise RuntimeError("obe_dense_commutator_tf32 failed")

    t_tc = timed(commutator_tcgen05)
    if int(status.item()) != 0:
        raise RuntimeError("the tensor-core commutator's wait gave up")
    ref = -1j * (torch.bmm(H_all.to(torch.complex128), R.to(torch.complex128))
                 - torch.bmm(R.to(torch.complex128), H_all.to(torch.complex128)))
    tc_err = float((out_tc.to(torch.complex128) - ref).abs().max() / ref.abs().max())
    # the sparse RHS on the same states (host arrays; the ncu launch list has the kernel alone)
    plan = NativePlan(d["payload"])
    idx = np.triu_indices(n, 1)
    packed = np.concatenate([rho.diagonal(axis1=1, axis2=2).real,
                             np.stack([rho[:, idx[0], idx[1]].real, rho[:, idx[0], idx[1]].imag], axis=-1).reshape(total, -1)],
                            axis=1)
    walls = {}
    for prec in ("fp64", "mixed"):
        plan.rhs(packed[:4], 0.0, precision=prec)
        best = float("inf")
        for _ in range(reps):
            start = time.perf_counter()
            plan.rhs(packed, 0.0, precision=prec)
            best = min(best, time.perf_counter() - start)
        walls[prec] = 1e3 * best
    f_rhs, _ = flops_per_step_unit(d["payload"])
    dense_flop = 16 * n ** 3
    return {"workload": f"{total} states of the 76-state system: one RHS each", "states": total,
            "dense_flop_per_state": dense_flop, "sparse_flop_per_state": f_rhs, "flop_ratio": dense_flop / f_rhs,
            "dense_ms": {"complex64_tf32_tensor": t_tf32, "complex64_fp32": t_fp32, "bf16_split_tensor": t_bf16,
                         "tcgen05_tf32_this_package": t_tc},
            "tcgen05_max_error_of_largest_element": tc_err,
            "sparse_obe_rhs_eval_wall_ms_with_copies": walls,
            "note": "device times per kernel: ncu launch list of `bench.py --case dense76`"}


def run_case(args) -> None:
    """One workload on its own, for profiling: `gradient` (the adjoint workload at a fixed launch
    width), `heterogeneous` (the 16/39/76-state batch) or `large` (one wave of 76-state
    trajectories, end times U[15, 20]/Γ).  Runs it `--steps` times and prints the times."""
    import torch

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    times = []
    if args.case == "dense76":
        print(json.dumps({"case": args.case, **measure_dense76(torch, dev, total=args.points, reps=max(1, args.steps))}))
        return
    if args.case == "heterogeneous":
        r = measure_heterogeneous(torch, dev, total=args.points, reps=max(1, args.steps))
        print(json.dumps({"case": args.case, **r}))
        return
    if args.case == "hetero-gradient":
        r = measure_hetero_gradient(torch, dev, total=args.points, precision=args.precision, reps=max(1, args.steps))
        print(json.dumps({"case": args.case, **r}))
        return
    if args.case == "gradient":
        from centrex_tlf_gb300.autograd import solve_batch_with_grad
        from centrex_tlf_gb300.native import NativePlan

        d, params_all, _ = workload(max(args.points, 1))
        gamma, (t0, t1) = d["gamma"], d["t_span"]
        names = d["payload"]["parameter_graph"]["slot_names"]
        slots = [names.index(s) for s in ("rabi", "detuning", "theta", "t_center")]
        p = np.concatenate([params_all.real, np.full((params_all.shape[0], 1), 100.0 / gamma)], axis=1)
        plan = NativePlan(d["payload"])
        plan.set_shape(args.threads_per_trajectory, 0)
        for _ in range(args.steps):
            pt = torch.tensor(p, dtype=torch.float64, device=dev, requires_grad=True)
            start = time.perf_counter()
            j = solve_batch_with_grad(plan, d["rho0_packed"], (t0, t1), pt, slots, dt=1e-3 / gamma,
                                      integral_weights=W_EXCITED, max_steps=2048, precision=args.precision,
                                      checkpoint_every=args.checkpoint_every)
            j.sum().backward()
            torch.cuda.synchronize()
            times.append(1e3 * (time.perf_counter() - start))
            assert bool(torch.isfinite(pt.grad).all())
        print(json.dumps({"case": args.case, "points": p.shape[0], "threads_per_trajectory": plan.shape()[0],
                          "precision": args.precision, "checkpoint_every": args.checkpoint_every,
                          "fwd_plus_grad_ms": times}))
        return
    # large: one wave of the 76-state system through the device entry point
    from centrex_tlf_gb300.native import NativePlan

    spec = [j for j in hetero_jobs(args.points * 10, t_end_range=(15.0, 20.0)) if j["name"] == "plan_rc_76"][0]
    d, g, b = spec["d"], spec["d"]["gamma"], spec["count"]
    plan = NativePlan(d["payload"])
    plan.set_shape(args.threads_per_trajectory, 0)
    o = plan.options(t0=0.0, t1=spec["t1"], abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=None, save_start=True,
                     maxiters=1000000, solver="tsit5", output="excited_population", output_indices=None,
                     output_when="final", integral_weights=spec["weights"], stop_event=spec["event"],
                     precision=args.precision)
    rho = torch.from_numpy(np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0)).to(dev)
    par = torch.from_numpy(np.ascontiguousarray(spec["params"]).view(np.float64).reshape(-1)).to(dev)
    val = torch.zeros(b, dtype=torch.float64, device=dev)
    st = torch.zeros(b * 6, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.solve_batch_device(o, b, rho.data_ptr(), spec["slots"], par.data_ptr(), 1, val.data_ptr(), st.data_ptr(),
                                stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    stv = st.view(-1, 6).cpu().numpy()
    assert not np.any(stv[:, 3] >> 32), "a 76-state trajectory failed"
    print(json.dumps({"case": args.case, "trajectories": b, "precision": args.precision,
                      "threads_per_trajectory": plan.shape()[0], "ms": times,
                      "accepted_steps": int(stv[:, 0].sum()), "rejected_steps": int(stv[:, 1].sum())}))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--precision", choices=["fp64", "mixed", "mixed_fp32_control"], default="mixed_fp32_control",
                    help="the headline form (every form is timed beside it; all hold the 1e-6 population bar)")
    ap.add_argument("--no-fp64-compare", action="store_true", help="skip timing the plain FP64 path beside mixed")
    ap.add_argument("--no-gradient", action="store_true", help="skip timing the adjoint beside the forward solve")
    ap.add_argument("--no-effective", action="store_true", help="skip timing the effective-Hamiltonian path")
    ap.add_argument("--no-single", action="store_true", help="skip timing the single 16-state solve")
    ap.add_argument("--ragged-instances", type=int, default=1024,
                    help="trajectories of the ragged 76-state scan timed beside the scan (0 skips it)")
    ap.add_argument("--hetero-instances", type=int, default=8192,
                    help="instances of the heterogeneous 16/39/76-state batch timed beside the scan (0 skips it)")
    ap.add_argument("--hetero-grad-instances", type=int, default=512,
                    help="instances of the heterogeneous batch timed forward plus adjoint (0: skip; the full "
                         "8192-instance batch: --case hetero-gradient --points 8192)")
    ap.add_argument("--points", type=int, default=4096)
    ap.add_argument("--checkpoint-every", type=int, default=None,
                    help="--case gradient: the tape's checkpoint interval (default: full tape while it fits)")
    ap.add_argument("--cpu-sample", type=int, default=128)
    ap.add_argument("--case", choices=["scan", "gradient", "heterogeneous", "hetero-gradient", "large", "dense76"], default="scan",
                    help="scan: the benchmark line; the others run one workload alone (profiling)")
    ap.add_argument("--threads-per-trajectory", type=int, default=0,
                    help="launch width of the gradient and large cases (0: automatic)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.case != "scan":
        run_case(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
