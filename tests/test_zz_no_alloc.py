"""The allocation-free batch entry point (obe_solve_batch_device_noalloc).

It exists for callers that cannot let a library allocate device memory while they solve -- a
caller that owns all device memory up front (its own arena) or that runs under a fixed memory
budget.  It must produce exactly what the allocating device entry point produces, call after
call, although every call reuses the same fixed device scratch array; the first case is also
checked against the oracle directly.

This file is collected last, so that a run that stops at the first failure has already run
every other test; it also passes on its own in a fresh process.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle
from centrex_tlf_gb300 import _abi
from centrex_tlf_gb300 import centrex_tlf_rust as api

pytestmark = pytest.mark.gpu

W_EXCITED = [(13, 1.0), (14, 1.0), (15, 1.0)]


def _noalloc(lib):
    fn = lib.obe_solve_batch_device_noalloc
    fn.argtypes = [
        ctypes.c_void_p, ctypes.POINTER(_abi.ObeSolveOptions), ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32,
        _abi.c_i64p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
    ]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("precision,output", [("fp64", "populations"), ("mixed", "excited_population")])
def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(golden, precision, output):
    torch = pytest.importorskip("torch")
    d = golden("plan_q1_16")
    gamma, (t0, t1) = d["gamma"], d["t_span"]
    plan = api.prepare_lindblad_problem_py(d["payload"])
    native = plan.native
    slot_names = d["payload"]["parameter_graph"]["slot_names"]
    slots = [slot_names.index(s) for s in ("rabi", "detuning", "theta")]
    rng = np.random.default_rng(5)
    b = 48
    params = np.stack([gamma * 10 ** rng.uniform(-1, 1, b), rng.uniform(-5, 5, b) * gamma, rng.uniform(0, np.pi, b)],
                      axis=1).astype(np.complex128)
    final_pops = output == "populations"
    opts = native.options(
        t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma,
        saveat=np.array([t1]) if final_pops else None, save_start=not final_pops, maxiters=100000, solver="tsit5",
        output=output, output_indices=None, output_when="final",
        integral_weights=None if final_pops else W_EXCITED, stop_event=None, precision=precision,
    )
    width = opts.width
    dev = torch.device("cuda:0")
    d_rho = torch.from_numpy(np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0)).to(dev)
    d_par = torch.from_numpy(np.ascontiguousarray(params).view(np.float64).reshape(-1)).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    slots_arr = np.asarray(slots, dtype=np.int64)

    # the allocating device entry point: the expected result
    ref_vals = torch.zeros(b * width, dtype=torch.float64, device=dev)
    ref_stats = torch.zeros(b * 6, dtype=torch.int64, device=dev)
    native.solve_batch_device(opts, b, d_rho.data_ptr(), slots, d_par.data_ptr(), 1, ref_vals.data_ptr(),
                              ref_stats.data_ptr(), stream)
    torch.cuda.synchronize()

    lib = _abi.load_library()
    fn = _noalloc(lib)
    for call in range(2):
        vals = torch.full((b * width,), float("nan"), dtype=torch.float64, device=dev)
        stats = torch.full((b * 6,), -1, dtype=torch.int64, device=dev)
        st = fn(native.handle, ctypes.byref(opts.opts), b, d_rho.data_ptr(), len(slots),
                slots_arr.ctypes.data_as(_abi.c_i64p), d_par.data_ptr(), 1, width, vals.data_ptr(), stats.data_ptr(),
                ctypes.c_void_p(stream))
        assert st == _abi.OBE_OK, _abi.last_error(lib)
        torch.cuda.synchronize()
        # same kernel, same inputs: the tolerance of the FP64 parity tests, met exactly here
        np.testing.assert_allclose(vals.cpu().numpy(), ref_vals.cpu().numpy(), rtol=1e-12, atol=0.0,
                                   err_msg=f"call {call}")
        np.testing.assert_array_equal(stats.cpu().numpy(), ref_stats.cpu().numpy())
        status = stats.view(b, 6)[:, 3].cpu().numpy() >> 32
        assert np.all(status == 0)

    # and the oracle on the same points: FP64 populations to 1e-9, the mixed integrals to 1e-6
    op = oracle.OraclePlan(d["payload"])
    o = op.options(t0=t0, t1=t1, abstol=1e-11, reltol=1e-8, dt=1e-3 / gamma,
                   saveat=np.array([t1]) if final_pops else None, save_start=not final_pops, maxiters=100000,
                   solver="tsit5", output=output, output_indices=None, output_when="final",
                   integral_weights=None if final_pops else W_EXCITED, stop_event=None)
    ref, _, _ = op.solve_batch(o, np.repeat(d["rho0_packed"].reshape(1, -1), b, axis=0), slots, params)
    got = vals.cpu().numpy().reshape(ref.shape)
    if final_pops:
        assert np.max(np.abs(got - ref)) <= 1e-9
    else:
        np.testing.assert_allclose(got, ref, rtol=1e-6)


def _both_entry_points(native, opts, b, rho0, slots, params, time_count):
    """(values, stats) of the allocating device entry point and of two allocation-free calls."""
    import torch

    dev = torch.device("cuda:0")
    width = opts.width
    per = time_count * width * (2 if opts.is_complex else 1)
    d_rho = torch.from_numpy(np.ascontiguousarray(rho0)).to(dev)
    d_par = None
    if params is not None:
        d_par = torch.from_numpy(np.ascontiguousarray(np.asarray(params, dtype=np.complex128)).view(np.float64).reshape(-1)).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    ref_vals = torch.zeros(b * per, dtype=torch.float64, device=dev)
    ref_stats = torch.zeros(b * 6, dtype=torch.int64, device=dev)
    native.solve_batch_device(opts, b, d_rho.data_ptr(), slots, None if d_par is None else d_par.data_ptr(), time_count,
                              ref_vals.data_ptr(), ref_stats.data_ptr(), stream)
    torch.cuda.synchronize()
    fn = _noalloc(_abi.load_library())
    slots_arr = np.asarray(slots if slots else [0], dtype=np.int64)
    runs = []
    for _ in range(2):
        vals = torch.full((b * per,), float("nan"), dtype=torch.float64, device=dev)
        stats = torch.full((b * 6,), -1, dtype=torch.int64, device=dev)
        st = fn(native.handle, ctypes.byref(opts.opts), b, d_rho.data_ptr(), len(slots) if d_par is not None else 0,
                slots_arr.ctypes.data_as(_abi.c_i64p), None if d_par is None else d_par.data_ptr(), time_count, width,
                vals.data_ptr(), stats.data_ptr(), ctypes.c_void_p(stream))
        assert st == _abi.OBE_OK, _abi.last_error(_abi.load_library())
        torch.cuda.synchronize()
        runs.append((vals.cpu().numpy(), stats.cpu().numpy()))
    return (ref_vals.cpu().numpy(), ref_stats.cpu().numpy()), runs


def test_noalloc_stop_event_batch(golden):
    """Per-trajectory stop events (event flags and times in the stats) through the allocation-free
    call, against the allocating one."""
    pytest.importorskip("torch")
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    native = plan.native
    ev = {"kind": "population", "indices": [1], "threshold": 0.05}
    opts = native.options(t0=0.0, t1=5.0, abstol=1e-10, reltol=1e-8, dt=1e-3, saveat=np.array([5.0]), save_start=False,
                          maxiters=100000, solver="dopri5", output="populations", output_indices=None,
                          output_when="final", integral_weights=None, stop_event=ev)
    det = np.array([[0.0], [0.05], [3.0], [-1.5]], dtype=np.complex128)
    slot = d["payload"]["parameter_graph"]["slot_names"].index("delta")
    rho0 = np.repeat(d["rho0_packed"].reshape(1, -1), 4, axis=0)
    (ref_v, ref_s), runs = _both_entry_points(native, opts, 4, rho0, [slot], det, 1)
    for vals, stats in runs:
        np.testing.assert_allclose(vals, ref_v, rtol=1e-12, atol=0.0)
        np.testing.assert_array_equal(stats, ref_s)


def test_noalloc_effective_plan(golden):
    """An interpolated effective-Hamiltonian plan (split-real state) through the allocation-free
    call, against the allocating one."""
    pytest.importorskip("torch")
    d = golden("plan_eff_r0")
    plan = api.prepare_effective_lindblad_plan_py(d["plan"])
    native = plan.native
    t0, t1 = d["t_span"]
    saveat = np.linspace(t0, t1, 5)
    opts = native.options(t0=t0, t1=t1, abstol=1e-9, reltol=1e-7, dt=1e-10, saveat=saveat, save_start=True,
                          maxiters=100000, solver="tsit5", output="populations", output_indices=None,
                          output_when="final", integral_weights=None, stop_event=None)
    rho0 = np.repeat(np.asarray(d["y0"], dtype=np.float64).reshape(1, -1), 3, axis=0)
    rabi = np.array([[0.8e7], [1.0e7], [1.3e7]], dtype=np.complex128)
    (ref_v, ref_s), runs = _both_entry_points(native, opts, 3, rho0, [0], rabi, 5)
    for vals, stats in runs:
        np.testing.assert_allclose(vals, ref_v, rtol=1e-12, atol=0.0)
        np.testing.assert_array_equal(stats, ref_s)


def test_noalloc_rejects_oversized_arguments_and_missing_parameters(golden):
    """Host-side refusals before any device work: a saveat beyond the 64 KiB argument block, and
    scanned slots without their values."""
    torch = pytest.importorskip("torch")
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    native = plan.native
    lib = _abi.load_library()
    fn = _noalloc(lib)
    dev = torch.device("cuda:0")
    rho = torch.zeros(4, dtype=torch.float64, device=dev)
    st_buf = torch.zeros(6, dtype=torch.int64, device=dev)
    saveat = np.linspace(0.0, 0.5, 9000)  # 72,000 bytes of save times
    opts = native.options(t0=0.0, t1=0.5, abstol=1e-10, reltol=1e-8, dt=1e-3, saveat=saveat, save_start=True,
                          maxiters=100000, solver="dopri5", output="populations", output_indices=None,
                          output_when="saveat", integral_weights=None, stop_event=None)
    out = torch.zeros(9000 * 2, dtype=torch.float64, device=dev)
    st = fn(native.handle, ctypes.byref(opts.opts), 1, rho.data_ptr(), 0, None, None, 9000, 2, out.data_ptr(),
            st_buf.data_ptr(), None)
    assert st == _abi.OBE_ERR_INVALID
    assert "65536-byte block" in _abi.last_error(lib)
    opts = native.options(t0=0.0, t1=0.5, abstol=1e-10, reltol=1e-8, dt=1e-3, saveat=np.array([0.5]), save_start=False,
                          maxiters=100000, solver="dopri5", output="populations", output_indices=None,
                          output_when="final", integral_weights=None, stop_event=None)
    slots = np.array([0], dtype=np.int64)
    st = fn(native.handle, ctypes.byref(opts.opts), 1, rho.data_ptr(), 1, slots.ctypes.data_as(_abi.c_i64p), None, 1, 2,
            out.data_ptr(), st_buf.data_ptr(), None)
    assert st == _abi.OBE_ERR_INVALID
    assert "needs both param_slots and d_param_values" in _abi.last_error(lib)


def test_noalloc_rejects_sizes_beyond_its_limit(golden):
    torch = pytest.importorskip("torch")
    d = golden("plan_two_level")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    native = plan.native
    opts = native.options(t0=0.0, t1=0.5, abstol=1e-10, reltol=1e-8, dt=1e-3, saveat=np.array([0.5]), save_start=False,
                          maxiters=100000, solver="dopri5", output="populations", output_indices=None,
                          output_when="final", integral_weights=None, stop_event=None)
    lib = _abi.load_library()
    fn = _noalloc(lib)
    dev = torch.device("cuda:0")
    too_many = 65537
    rho = torch.zeros(4, dtype=torch.float64, device=dev)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    st_buf = torch.zeros(6, dtype=torch.int64, device=dev)
    st = fn(native.handle, ctypes.byref(opts.opts), too_many, rho.data_ptr(), 0, None, None, 1, 2, out.data_ptr(),
            st_buf.data_ptr(), None)
    assert st == _abi.OBE_ERR_INVALID
    assert "at most 65536 trajectories" in _abi.last_error(lib)


def test_noalloc_rejects_systems_above_45_states(golden):
    """The 76-state system keeps its stage buffers in device memory the library allocates, so the
    allocation-free entry point refuses it, naming the entry point that can solve it."""
    torch = pytest.importorskip("torch")
    d = golden("plan_rc_76")
    plan = api.prepare_lindblad_problem_py(d["payload"])
    native = plan.native
    g = d["gamma"]
    opts = native.options(t0=0.0, t1=1.0 / g, abstol=1e-11, reltol=1e-8, dt=1e-3 / g, saveat=np.array([1.0 / g]),
                          save_start=False, maxiters=1000, solver="tsit5", output="populations", output_indices=None,
                          output_when="final", integral_weights=None, stop_event=None)
    lib = _abi.load_library()
    fn = _noalloc(lib)
    dev = torch.device("cuda:0")
    rho = torch.from_numpy(d["rho0_packed"].reshape(1, -1).copy()).to(dev)
    out = torch.zeros(76, dtype=torch.float64, device=dev)
    st_buf = torch.zeros(6, dtype=torch.int64, device=dev)
    st = fn(native.handle, ctypes.byref(opts.opts), 1, rho.data_ptr(), 0, None, None, 1, 76, out.data_ptr(),
            st_buf.data_ptr(), None)
    assert st == _abi.OBE_ERR_UNSUPPORTED
    assert "obe_solve_batch_device" in _abi.last_error(lib)
