"""Generate the golden fixtures under tests/golden/ from the reference's own Python code.

Run where a CeNTREX-TlF reference checkout exists, naming it with ``--reference PATH`` or the
``CENTREX_REFERENCE`` environment variable (there is no default path):

    python tests/golden/make_fixtures.py --reference PATH/TO/CeNTREX-TlF

What it writes (all JSON through ``codec.py``):

* ``plan_<name>.json``: the plan payload dict exactly as the reference's
  ``PreparedLindbladProblem.to_payload()`` returns it (centrex_tlf/lindblad/plan_static.py:58-68),
  built by the reference's unchanged builders (``prepare_lindblad_problem`` with
  ``backend="python"``, centrex_tlf/lindblad/plan_static.py:137-185), plus the packed initial
  state, the time span and the metadata a test needs.
* ``rhs_<name>.json``: packed states, times, base-parameter overrides and the packed RHS from
  the reference's Python FP64 evaluators ``structured_rhs`` and ``reference_rhs``
  (centrex_tlf/lindblad/reference_dense.py:60-77) for each of them.
* ``rk45_<name>.json``: trajectories from the reference's SciPy RK45 solve
  (``solve_lindblad(..., backend="python")``, centrex_tlf/lindblad/solve.py:155-199):
  tolerance-level anchors for whole solves.
* ``plan_rc_76.json`` / ``rhs_rc_76.json``: the 76-state rotational-cooling system (dense collapse
  operators dropped: the expanded_sparse path does not read them).
* ``kat_fixed_step.json``: the reference's recorded fixed-step solver runs
  (benchmarks/fixed_step_solver_results/fixed_step_solver_report.md and
  fixed_step_solver_validation.csv): step and RHS counts per case, and the photon-integral
  difference of each fixed-step run from the adaptive Dopri5 run.
* ``ffi_calls.json``: the positional arguments the reference's Python surface
  (solve.py:419, batch.py:235, batch.py:440) passes across its native boundary, recorded by
  installing a recording stand-in module as ``centrex_tlf.centrex_tlf_rust``.

pandas and matplotlib are stubbed: the reference imports them only for DataFrames and plotting
(centrex_tlf/couplings/branching.py:5, centrex_tlf/utils/plotting.py:9-13).
"""

from __future__ import annotations

import copy
import importlib.abc
import importlib.machinery
import os
import sys
import time
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import codec  # noqa: E402


def _reference_path() -> Path:
    """The reference checkout: ``--reference PATH`` or ``CENTREX_REFERENCE``; no default."""
    if "--reference" in sys.argv:
        i = sys.argv.index("--reference")
        if i + 1 >= len(sys.argv):
            raise SystemExit("--reference needs a path")
        return Path(sys.argv[i + 1])
    env = os.environ.get("CENTREX_REFERENCE")
    if not env:
        raise SystemExit("name the CeNTREX-TlF checkout with --reference PATH or CENTREX_REFERENCE")
    return Path(env)


REFERENCE = Path()  # set by _import_reference()

# Γ for the benchmark configurations: 2π·1.56 MHz, passed explicitly to the builders.
GAMMA = 2.0 * np.pi * 1.56e6


class _StubModule(types.ModuleType):
    def __getattr__(self, attr):
        if attr.startswith("__"):
            raise AttributeError(attr)
        return type(attr, (), {"__init__": lambda self, *a, **k: None})


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in ("pandas", "matplotlib"):
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        module = _StubModule(spec.name)
        module.__path__ = []
        return module

    def exec_module(self, module):
        pass


def _import_reference():
    global REFERENCE
    REFERENCE = _reference_path()
    sys.meta_path.insert(0, _StubFinder())
    sys.path.insert(0, str(REFERENCE))
    import sympy as smp  # noqa: F401

    import centrex_tlf  # noqa: F401

    return centrex_tlf


def _hermitian(rng: np.random.Generator, n: int, scale: float = 1.0) -> np.ndarray:
    m = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return scale * (m + m.conj().T)


def _density(rng: np.random.Generator, n: int) -> np.ndarray:
    m = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    rho = m @ m.conj().T
    return rho / np.trace(rho).real


def build_two_level(centrex_tlf, omega=0.6, delta=0.0, time_dependent=False):
    """Two-level system of the reference's benchmark and tests
    (benchmarks/bench_expanded_sparse_packed_rhs_kernels.py:102-157,
    tests/lindblad/test_rust_backend.py:35-58)."""
    import sympy as smp
    from centrex_tlf.lindblad.plan_static import prepare_lindblad_problem
    from centrex_tlf.lindblad.utils_setup import OBESystem

    om, de = smp.symbols("Omega delta", real=True)
    hamiltonian = smp.Matrix([[0, om / 2], [smp.conjugate(om) / 2, -de]])
    c_array = np.zeros((1, 2, 2), dtype=np.complex128)
    c_array[0, 0, 1] = np.sqrt(0.3)
    zeros = np.zeros((2, 2), dtype=np.complex128)
    system = OBESystem(
        ground=[], excited=[], QN=[], H_int=zeros, V_ref_int=zeros, couplings=[],
        H_symbolic=hamiltonian, C_array=c_array, system=None,
        coupling_symbols=[om, de], polarization_symbols=[],
    )
    if time_dependent:
        params = {
            "omega0": 1.0,
            "modulation_depth": 0.5,
            "modulation_frequency": 1.9,
            "delta": -0.1,
            "Omega": "omega0*phase_modulation(t, modulation_depth, modulation_frequency)",
        }
    else:
        params = {"Omega": omega, "delta": delta}
    return prepare_lindblad_problem(system, params, backend="python", hamiltonian_representation="decomposed")


def build_chain(centrex_tlf, n_states: int):
    """Nearest-neighbour chain of the reference's partition-gate test
    (tests/lindblad/test_rust_backend.py:489-568)."""
    import sympy as smp
    from centrex_tlf.lindblad.plan_static import prepare_lindblad_problem
    from centrex_tlf.lindblad.utils_setup import OBESystem

    om, de = smp.symbols("Omega delta", real=True)
    hamiltonian = smp.zeros(n_states, n_states)
    for i in range(n_states):
        hamiltonian[i, i] = de * i
    for i in range(n_states - 1):
        hamiltonian[i, i + 1] = om / 2
        hamiltonian[i + 1, i] = smp.conjugate(om) / 2
    c_array = np.zeros((n_states - 1, n_states, n_states), dtype=np.complex128)
    for i in range(n_states - 1):
        c_array[i, i, i + 1] = np.sqrt(0.1)
    zeros = np.zeros((n_states, n_states), dtype=np.complex128)
    system = OBESystem(
        ground=[], excited=[], QN=[], H_int=zeros, V_ref_int=zeros, couplings=[],
        H_symbolic=hamiltonian, C_array=c_array, system=None,
        coupling_symbols=[om, de], polarization_symbols=[],
    )
    params = {
        "omega0": 1.0,
        "modulation_depth": 0.5,
        "modulation_frequency": 1.9,
        "delta": 0.2,
        "Omega": "omega0*phase_modulation(t, modulation_depth, modulation_frequency)",
    }
    return prepare_lindblad_problem(system, params, backend="python", hamiltonian_representation="decomposed")


def build_q1_16(centrex_tlf, with_t_end: bool = False):
    """The 16-state TlF system of the single-solve and scan benchmarks.

    X J=1 (12 hyperfine states) + B J'=1 F1'=1/2 F'=1 (3 mF states) + the X J=3 level the
    B state also decays to, lumped into one state by the builder's own ``qn_compact=True``
    (centrex_tlf/lindblad/utils_setup.py:515-629).  Q(1) F'=1 drive with z- and x-linear
    polarisation components; a Gaussian-in-time Rabi pulse; Γ = 2π·1.56 MHz.  With
    ``with_t_end`` the parameter graph also holds a scalar ``t_end`` that a `Time() - t_end` stop
    event can read (ragged end times in a batch); the Hamiltonian does not depend on it.
    """
    from centrex_tlf import couplings, lindblad, transitions
    from centrex_tlf.lindblad.parameters import LindbladParameters
    from centrex_tlf.lindblad.plan_static import prepare_lindblad_problem

    trans = [transitions.Q1_F1_1o2_F1]
    selectors = couplings.generate_transition_selectors(
        trans, [[couplings.polarization_Z, couplings.polarization_X]]
    )
    obe = lindblad.generate_OBE_system_transitions(trans, selectors, qn_compact=True, Γ=GAMMA)
    params = LindbladParameters.from_kwargs(**_gaussian_pulse_parameters(with_t_end))
    prepared = prepare_lindblad_problem(obe, params, backend="python", hamiltonian_representation="decomposed")
    labels = [str(s.largest) for s in obe.QN]
    return prepared, labels


def _gaussian_pulse_parameters(with_t_end: bool) -> dict:
    kw = dict(
        rabi=GAMMA,
        detuning=0.0,
        theta=0.0,
        t_center=100.0 / GAMMA,
        sigma=20.0 / GAMMA,
    )
    if with_t_end:
        kw["t_end"] = 200.0 / GAMMA
    kw.update(
        Ω0="rabi*exp(-(t-t_center)**2/(2*sigma**2))",
        δ0="detuning",
        PZ0="cos(theta)",
        PX0="sin(theta)",
    )
    return kw


def build_r0_39(centrex_tlf):
    """The 39-state system of the heterogeneous batch: X J=0-2 (36 hyperfine states) + B J'=1
    F1'=1/2 F'=1 (P=-1, 3 mF states), driven on R(0) F1'=1/2 F'=1 with z- and x-linear
    polarisation components by the same Gaussian pulse and parameters as the 16-state system,
    plus a scalar ``t_end`` for a `Time() - t_end` stop event; Γ = 2π·1.56 MHz.
    """
    from centrex_tlf import couplings, lindblad, states, transitions
    from centrex_tlf.lindblad.parameters import LindbladParameters
    from centrex_tlf.lindblad.plan_static import prepare_lindblad_problem

    X = [states.QuantumSelector(J=j, electronic=states.ElectronicState.X) for j in (0, 1, 2)]
    B = [states.QuantumSelector(J=1, F1=0.5, F=1, P=-1, electronic=states.ElectronicState.B)]
    trans = [transitions.R0_F1_1o2_F1]
    selectors = couplings.generate_transition_selectors(trans, [[couplings.polarization_Z, couplings.polarization_X]])
    obe = lindblad.generate_OBE_system(X, B, selectors, Γ=GAMMA)
    params = LindbladParameters.from_kwargs(**_gaussian_pulse_parameters(True))
    prepared = prepare_lindblad_problem(obe, params, backend="python", hamiltonian_representation="decomposed")
    labels = [str(s.largest) for s in obe.QN]
    return prepared, labels


def save_multi(centrex_tlf) -> None:
    """plan_r0_39.json and plan_q1_16_tend.json: the two smaller systems of the heterogeneous
    batch (the 76-state one is plan_rc_76), each with a scannable t_end slot; rhs_r0_39.json:
    the reference's Python RHS on the 39-state payload."""
    # rho0: equal populations over the driven ground level (X J=0 for R(0), X J=1 for Q(1))
    for name, (prep, labels), driven in (("plan_r0_39", build_r0_39(centrex_tlf), "J = 0,"),
                                         ("plan_q1_16_tend", build_q1_16(centrex_tlf, with_t_end=True), "J = 1,")):
        n = len(labels)
        ground = [i for i, lab in enumerate(labels) if lab.startswith("|X") and driven in lab]
        rho = np.zeros((n, n), dtype=np.complex128)
        for i in ground:
            rho[i, i] = 1.0 / len(ground)
        payload = prep.to_payload()
        payload["dense_c_array"] = np.zeros((0, n, n), dtype=np.complex128)
        codec.save(name, {
            "payload": payload, "rho0_packed": prep.layout.pack(rho), "gamma": GAMMA, "state_labels": labels,
            "excited_indices": [i for i, lab in enumerate(labels) if "B" in lab],
            "scan_slots": ["rabi", "detuning", "theta", "t_end"],
        })
        if name == "plan_r0_39":
            slots = prep.parameter_graph["slot_names"]
            ov = [{}, {slots.index("rabi"): 2.5 * GAMMA, slots.index("detuning"): -1.5 * GAMMA, slots.index("theta"): 0.9}]
            cases = rhs_vectors(prep, [0.0, 80.0 / GAMMA, 100.0 / GAMMA], ov, seed=39, scale=0.05)
            codec.save("rhs_r0_39", {"cases": cases})


def build_r2_38(centrex_tlf):
    """The 38-state R(2) system of the reference's expanded_sparse solve benchmark
    (benchmarks/bench_expanded_sparse_packed_rhs_kernels.py:36-47 constants, :162-300 construction):
    R(2) F1'=7/2 F'=3 with x polarisation, ground and excited mains X J=2 F1=5/2 F=2 mF=0 and
    B F'=3 mF=1, opposite-parity levels retained, E = 200 V/cm and B = 1e-5 G along z, the Rabi
    rate of 60 mW in a 2 cm x 2 cm rectangular beam, zero detuning; rho0 = the lowest-energy
    X J=2 F1=5/2 F=2 mF=0 state; photon integral with weight Γ on every B state over 0.02 m /
    184 m/s.  The reference records its Rust solve of this system
    (benchmarks/expanded_sparse_static_dynamic_results/validation.csv, solve_timings.csv,
    grid_timings.csv).  Those records predate the reference's 0.2.4 constants (CHANGELOG.md:118-123:
    Γ = 1/τ_B instead of the hard-coded 2π·1.56 MHz, a new X rotational model), so the system is
    built with Γ = 2π·1.56 MHz, the value of `hamiltonian.Γ` then; with it the recorded step and
    RHS counts are reproduced exactly and the photon integral to 1e-4 (the X-model change).
    """
    from centrex_tlf import couplings, lindblad, states, transitions
    from centrex_tlf.lindblad.parameters import LindbladParameters
    from centrex_tlf.lindblad.plan_static import prepare_lindblad_problem
    from centrex_tlf.utils.rabi import power_to_rabi_rectangular_beam

    tr = transitions.R2_F1_7o2_F3
    gamma_ref = GAMMA  # 2π·1.56 MHz (see above)
    x_main = 1 * next(iter(states.generate_coupled_states_X(states.QuantumSelector(
        electronic=states.ElectronicState.X, J=tr.J_ground, F1=5 / 2, F=2, mF=0, P=tr.P_ground))))
    b_main = 1 * next(iter(states.generate_coupled_states_B(states.QuantumSelector(
        electronic=states.ElectronicState.B, J=tr.J_excited, F1=tr.F1_excited, F=tr.F_excited, mF=1,
        P=tr.P_excited))))
    selectors = couplings.generate_transition_selectors(
        transitions=[tr], polarizations=[[couplings.polarization_X]], ground_mains=[x_main], excited_mains=[b_main])
    import warnings
    with warnings.catch_warnings():
        warnings.filterwarnings("ignore", message="Low overlap detected.*")
        system = lindblad.generate_OBE_system_transitions(
            [tr], selectors, qn_compact=True, E=np.array([0.0, 0.0, 200.0]), B=np.array([0.0, 0.0, 1e-5]),
            retain_opposite_parity_levels=True, Γ=gamma_ref)
    rabi_rad_s = power_to_rabi_rectangular_beam(60e-3, abs(system.couplings[0].main_coupling), 0.02, 0.02)
    params = LindbladParameters()
    rabi = params.real("rabi", rabi_rad_s)
    detuning = params.real("detuning", 0.0)
    det_symbol = getattr(selectors[0], "\u03b4")
    for sym in system.H_symbolic.free_symbols:
        if sym in system.coupling_symbols:
            params.bind(sym, rabi, finalize=False)
        elif sym == det_symbol:
            params.bind(sym, detuning, finalize=False)
        else:
            params.real(str(sym), 0.0)
    for group in system.polarization_symbols:
        for sym in (group if isinstance(group, (list, tuple)) else [group]):
            params.bind(sym, 1.0, finalize=False)
    params._finalize()
    prepared = prepare_lindblad_problem(system, params, backend="python", hamiltonian_representation="decomposed")
    cands = [i for i, st in enumerate(system.QN)
             if st.largest.electronic_state == states.ElectronicState.X and st.largest.J == tr.J_ground
             and st.largest.F1 == 5 / 2 and st.largest.F == 2 and st.largest.mF == 0]
    start = min(cands, key=lambda i: float(np.real(system.H_int[i, i])))
    excited = [i for i, st in enumerate(system.QN) if st.largest.electronic_state == states.ElectronicState.B]
    return prepared, start, excited, gamma_ref


def save_r2_38(centrex_tlf) -> None:
    """plan_r2_38.json: the 38-state R(2) benchmark system with the reference's recorded Rust
    results for it (single photon integral, step and RHS counts; 9-point detuning grid counts)."""
    prep, start, excited, gamma_ref = build_r2_38(centrex_tlf)
    payload = prep.to_payload()
    n = payload["n_states"]
    payload["dense_c_array"] = np.zeros((0, n, n), dtype=np.complex128)  # never read on this path
    rho = np.zeros((n, n), dtype=np.complex128)
    rho[start, start] = 1.0
    codec.save("plan_r2_38", {
        "payload": payload, "rho0_packed": prep.layout.pack(rho), "gamma": gamma_ref,
        "t_span": [0.0, 0.02 / 184.0],
        # benchmarks/expanded_sparse_static_dynamic_results: validation.csv (static_dynamic =
        # expanded_sparse), solve_timings.csv:7, grid_timings.csv:7
        "kat": {"photon_integral": 1.2128563927511686, "accepted_steps": 28651, "rejected_steps": 0,
                "rhs_calls": 171907, "abstol": 1e-9, "reltol": 1e-7, "dt": 1e-9, "solver": "dopri5",
                "weights": [[int(i), gamma_ref] for i in excited]},
        "kat_grid": {"detuning": 2 * np.pi * 1e6 * np.linspace(-80.0, 80.0, 9), "accepted_steps": 329395,
                     "rejected_steps": 0, "rhs_calls": 1976397},
    })


def build_effective_r0(centrex_tlf, detuning_expr: str):
    """An interpolated effective-Hamiltonian model (centrex_tlf/effective_hamiltonian): R(0)
    F1'=1/2 F'=1 with z polarisation, compact Lindblad-safe model on the field grid 100, 150,
    200 V/cm (B = 1e-3 G along z, master field 150 V/cm; as tests/effective_hamiltonian/
    test_interpolated_preparation.py builds one), and the payload that the reference's
    prepare_effective_lindblad_rust_plan (effective_hamiltonian/rust_plan.py:42-200) hands to its
    native prepare_effective_lindblad_plan_py, captured by a stand-in for that native function.
    Parameters: the field oscillates inside the grid, Ez = 150 + 40 sin(2π·1e5 t) V/cm; a Gaussian
    Rabi pulse Ω0 = rabi exp(-(t - 2.5e-6)² / (2 (1e-6)²)); δ0 = `detuning_expr`.  Also returns the
    split-real superoperators at the grid nodes (the reference's own _hamiltonian_superoperator and
    dissipator), from which the golden RHS values are made."""
    import types

    import centrex_tlf as ct
    from centrex_tlf import couplings, transitions
    from centrex_tlf.effective_hamiltonian._superoperators import _hamiltonian_superoperator
    from centrex_tlf.effective_hamiltonian.preparation import prepare_lindblad_safe_compact_interpolated_model
    from centrex_tlf.effective_hamiltonian.rust_plan import (
        _complex_superop_to_split_real,
        prepare_effective_lindblad_rust_plan,
    )
    from centrex_tlf.lindblad.parameters import LindbladParameters

    pol = couplings.Polarization(np.array([0.0, 0.0, 1.0], dtype=np.complex128), name="Z")
    model = prepare_lindblad_safe_compact_interpolated_model(
        field_points=(100.0, 150.0, 200.0), transition=transitions.R0_F1_1o2_F1, optical_polarization=pol,
        magnetic_field=(0.0, 0.0, 1e-3), master_field=150.0)
    params = LindbladParameters.from_kwargs(
        rabi=1.0e7, detuning=0.0, chirp=2.0e11, Ez="150.0 + 40.0*sin(2*pi*1e5*t)",
        Ω0="rabi*exp(-(t - 2.5e-6)**2/(2*(1e-6)**2))", δ0=detuning_expr)
    saved = sys.modules.get("centrex_tlf.centrex_tlf_rust")
    stub = types.ModuleType("centrex_tlf.centrex_tlf_rust")
    stub.prepare_effective_lindblad_plan_py = lambda d: d  # capture the payload
    sys.modules["centrex_tlf.centrex_tlf_rust"] = stub
    ct.centrex_tlf_rust = stub
    try:
        plan = prepare_effective_lindblad_rust_plan(model, params, operator_interpolation="linear")
    finally:
        if saved is not None:
            sys.modules["centrex_tlf.centrex_tlf_rust"] = saved
    nodes = []
    for field_z in model.field_points.tolist():
        b = model.effective_bundle(float(field_z))
        nodes.append({
            "combined": _complex_superop_to_split_real(_hamiltonian_superoperator(b.h_internal) + b.dissipator_superoperator()),
            "optical": _complex_superop_to_split_real(_hamiltonian_superoperator(b.h_opt)),
            "detuning": _complex_superop_to_split_real(_hamiltonian_superoperator(b.h_det)),
        })
    return model, plan, nodes


def save_effective(centrex_tlf) -> None:
    """plan_eff_r0.json: the effective model's payload, a split-real initial state (the ground
    main state), and golden RHS values dy = (L_c(x) + Ω/2 L_o(x) + δ L_d(x)) y from the
    reference's node superoperators -- at the nodes and, between them, their linear interpolation
    (the payload's `linear` coefficients); plan_eff_r0_static.json: the same model with a
    time-independent detuning program δ0 = detuning, which the reference's plan freezes at its
    base value (effective_lindblad/plan.rs: detect_constant_slot)."""
    model, plan, nodes = build_effective_r0(centrex_tlf, "detuning + chirp*(t - 2.5e-6)")
    n = plan["n_states"]
    rho = np.zeros((n, n), dtype=np.complex128)
    g = int(model.ground_main_index)
    rho[g, g] = 1.0
    y0 = np.concatenate([rho.real.reshape(-1), rho.imag.reshape(-1)])
    grid = np.asarray(plan["field_grid"], dtype=np.float64)
    rng = np.random.default_rng(210)
    cases = []
    # the field program Ez(t) = 150 + 40 sin(2π·1e5 t) spans [110, 190]: cases at the middle node
    # and between the nodes, each at the time t where Ez(t) = x, with the base values (rabi,
    # detuning) that give the wanted Ω0(t) and δ0(t)
    for x, om, de in ((150.0, 1.3e7, 2.0e6), (123.4, 8.0e6, 1.0e6), (187.9, 2.5e6, -3.0e6), (110.0, 0.0, -5.0e6),
                      (176.5, 4.0e6, 0.0)):
        t = float(np.arcsin((x - 150.0) / 40.0) / (2 * np.pi * 1e5)) % 1e-5
        x = 150.0 + 40.0 * np.sin(2 * np.pi * 1e5 * t)
        pulse = np.exp(-(t - 2.5e-6) ** 2 / (2 * (1e-6) ** 2))
        rabi, det = om / pulse, de - 2.0e11 * (t - 2.5e-6)
        om = rabi * pulse
        de = det + 2.0e11 * (t - 2.5e-6)
        k = min(int(np.searchsorted(grid, x, side="right")) - 1, grid.size - 2)
        w = (x - grid[k]) / (grid[k + 1] - grid[k])
        mats = {key: (1.0 - w) * nodes[k][key] + w * nodes[k + 1][key] for key in ("combined", "optical", "detuning")}
        y = rng.normal(size=2 * n * n) * 0.1
        dy = mats["combined"] @ y + 0.5 * om * (mats["optical"] @ y) + de * (mats["detuning"] @ y)
        cases.append({"t": t, "field": x, "rabi": om, "detuning": de, "base_rabi": rabi, "base_detuning": det,
                      "y": y, "dy": dy})
    codec.save("plan_eff_r0", {"plan": plan, "y0": y0, "ground_main": g, "rhs_cases": cases,
                               "t_span": [0.0, 5.0e-6]})
    _, plan_s, _ = build_effective_r0(centrex_tlf, "detuning")
    codec.save("plan_eff_r0_static", {"plan": plan_s, "y0": y0})


def build_rc_76(centrex_tlf):
    """The 76-state rotational-cooling-sized system: X J=0-3 (64 hyperfine states) + B J'=1
    F1'=1/2, 3/2 (P=-1, 12 states), driven by R(0) F1'=1/2 F'=1 and P(2) F1'=3/2 F'=1 with x and z
    polarisation components; Γ = 2π·1.56 MHz.  Each laser's polarisation switches between x and
    z as a 1 MHz square wave (the second a quarter period later), and a scanned end time t_end
    can feed a `Time() - t_end` stop event.  (R(0) with Q(1) over 12 B states of one parity does
    not build in the reference; R(0) with P(2) is the exact-size construction that does.)
    """
    from centrex_tlf import couplings, lindblad, states, transitions
    from centrex_tlf.lindblad.parameters import LindbladParameters
    from centrex_tlf.lindblad.plan_static import prepare_lindblad_problem

    X = [states.QuantumSelector(J=j, electronic=states.ElectronicState.X) for j in (0, 1, 2, 3)]
    B = [states.QuantumSelector(J=1, F1=f1, P=-1, electronic=states.ElectronicState.B) for f1 in (0.5, 1.5)]
    trans = [transitions.R0_F1_1o2_F1, transitions.P2_F1_3o2_F1]
    pol = [couplings.polarization_X, couplings.polarization_Z]
    selectors = couplings.generate_transition_selectors(trans, [pol, pol])
    obe = lindblad.generate_OBE_system(X, B, selectors, Γ=GAMMA)
    quarter = 0.5 * np.pi
    params = LindbladParameters.from_kwargs(
        Ω0=GAMMA, Ω1=GAMMA, δ0=0.0, δ1=0.0, omega_pol=2.0 * np.pi * 1e6, t_end=50e-6,
        PX0="square_wave(t, omega_pol, 0.0)", PZ0="1 - square_wave(t, omega_pol, 0.0)",
        PX1=f"square_wave(t, omega_pol, {quarter!r})", PZ1=f"1 - square_wave(t, omega_pol, {quarter!r})",
    )
    prepared = prepare_lindblad_problem(obe, params, backend="python", hamiltonian_representation="decomposed")
    labels = [str(s.largest) for s in obe.QN]
    return prepared, labels


def save_rc_76(centrex_tlf) -> None:
    """plan_rc_76.json and rhs_rc_76.json: the 76-state system of build_rc_76."""
    rc, labels = build_rc_76(centrex_tlf)
    payload = rc.to_payload()
    # the expanded_sparse path never reads the dense collapse operators (154 x 76 x 76 complex,
    # 14 MB): keep their shape contract with zero operators
    payload["dense_c_array"] = np.zeros((0, 76, 76), dtype=np.complex128)
    n_x = sum(1 for lab in labels if "X" in lab)
    rho = np.zeros((76, 76), dtype=np.complex128)
    for i in range(n_x):
        rho[i, i] = 1.0 / n_x
    codec.save(
        "plan_rc_76",
        {
            "payload": payload, "rho0_packed": rc.layout.pack(rho), "gamma": GAMMA, "state_labels": labels,
            "n_ground": n_x, "excited_indices": [i for i, lab in enumerate(labels) if "B" in lab],
            "scan_slots": ["Ω0", "Ω1", "δ0", "δ1", "t_end"],
        },
    )
    cases = rhs_vectors(rc, [0.0, 3.1e-7, 7.7e-7], [{}, {0: 2.0 * GAMMA, 2: 0.3 * GAMMA}], seed=76, scale=0.02)
    codec.save("rhs_rc_76", {"cases": cases})


def _with_base_overrides(prepared, overrides: dict[int, complex]):
    """A shallow stand-in of ``prepared`` whose parameter graph has some base values replaced
    (what the batch drivers' scalar overrides do, rust/src/lindblad/rhs.rs:1176-1197)."""
    graph = copy.deepcopy(prepared.parameter_graph)
    for slot, value in overrides.items():
        graph["base_values"][slot] = {"kind": "scalar", "re": float(np.real(value)), "im": float(np.imag(value))}
    return types.SimpleNamespace(
        layout=prepared.layout,
        parameter_graph=graph,
        hamiltonian_plan=prepared.hamiltonian_plan,
        structured_jumps=prepared.structured_jumps,
        source_decay_rates=prepared.source_decay_rates,
        dense_c_array=prepared.dense_c_array,
    )


def rhs_vectors(prepared, times, overrides_list, seed, scale=1.0):
    from centrex_tlf.lindblad.reference_dense import reference_rhs, structured_rhs

    rng = np.random.default_rng(seed)
    n = prepared.layout.n
    cases = []
    for overrides in overrides_list:
        view = _with_base_overrides(prepared, overrides)
        for t in times:
            rho = _hermitian(rng, n, scale)
            packed = prepared.layout.pack(rho)
            cases.append(
                {
                    "t": float(t),
                    "override_slots": np.array(sorted(overrides), dtype=np.int64),
                    "override_values": np.array([overrides[k] for k in sorted(overrides)], dtype=np.complex128),
                    "packed": packed,
                    "structured": structured_rhs(view, packed, float(t)),
                    "reference": reference_rhs(view, packed, float(t)),
                }
            )
    return cases


def rk45_solve(prepared, rho0, t_span, saveat, abstol, reltol, overrides=None):
    from centrex_tlf.lindblad.solve import solve_lindblad

    target = prepared if not overrides else _reprepared(prepared, overrides)
    result = solve_lindblad(
        target, rho0, t_span, backend="python", abstol=abstol, reltol=reltol, saveat=saveat
    )
    return {"t": np.asarray(result.t), "packed_y": np.asarray(result.packed_y)}


def _reprepared(prepared, overrides):
    view = copy.copy(prepared)
    view.parameter_graph = _with_base_overrides(prepared, overrides).parameter_graph
    return view


def record_ffi_calls(centrex_tlf, prepared, rho0):
    """Run the reference's Python surface with a recording stand-in for its native module and
    keep the positional arguments of each call."""
    import centrex_tlf.lindblad.batch as batch_mod
    import centrex_tlf.lindblad.solve as solve_mod

    calls = []
    n = prepared.layout.n
    N = prepared.layout.packed_len

    class _Plan:
        pass

    def _solve_single(*args):
        calls.append({"fn": "solve_lindblad_ode_py", "args": list(args[1:])})
        output = args[12]
        if output == "full":
            width = N
        elif output == "populations":
            width = n
        elif output == "selected":
            width = len(args[13])
        else:
            width = 1
        return np.array([args[3]]), np.zeros(width), width, {"accepted_steps": 0, "rejected_steps": 0, "rhs_calls": 0, "event_triggered": False}

    def _solve_batch(*args):
        calls.append({"fn": "solve_lindblad_batch_ode_py", "args": list(args[1:])})
        b = args[1].shape[0]
        output = args[12]
        width = n if output == "populations" else (len(args[13]) if output == "selected" else 1)
        tc = 1 if args[14] == "final" else len(args[7])
        vals = np.zeros(b * tc * width, dtype=np.complex128 if output == "selected" else np.float64)
        return np.array([args[3]]), vals, width, tc, {"accepted_steps": 0, "rejected_steps": 0, "rhs_calls": 0, "event_triggered": False, "event_triggered_by_trajectory": [False] * b, "event_times": [args[3]] * b, "event_count": 0}

    def _solve_grid(*args):
        calls.append({"fn": "solve_lindblad_grid_ode_py", "args": list(args[1:])})
        b = int(np.prod(args[9]))
        output = args[15]
        width = n if output == "populations" else (len(args[16]) if output == "selected" else 1)
        tc = 1 if args[17] == "final" else len(args[10])
        vals = np.zeros(b * tc * width, dtype=np.complex128 if output == "selected" else np.float64)
        return np.array([args[3]]), vals, width, tc, {"accepted_steps": 0, "rejected_steps": 0, "rhs_calls": 0, "event_triggered": False, "event_triggered_by_trajectory": [False] * b, "event_times": [args[3]] * b, "event_count": 0}

    stand_in = types.ModuleType("centrex_tlf.centrex_tlf_rust")
    stand_in.solve_lindblad_ode_py = _solve_single
    stand_in.solve_lindblad_batch_ode_py = _solve_batch
    stand_in.solve_lindblad_grid_ode_py = _solve_grid
    sys.modules["centrex_tlf.centrex_tlf_rust"] = stand_in
    view = copy.copy(prepared)
    view.rust_plan = _Plan()
    view.backend = "rust"
    t_span = (0.0, 200.0 / GAMMA)
    weights = [(13, 1.0), (14, 1.0), (15, 1.0)]
    slots = prepared.parameter_graph["slot_names"]
    solve_mod.solve_lindblad(view, rho0, t_span, solver="dopri5", abstol=1e-11, reltol=1e-8, dt=1e-3 / GAMMA,
                             output="populations", output_when="final")
    solve_mod.solve_lindblad(view, rho0, t_span, solver="tsit5", abstol=1e-11, reltol=1e-8, dt=1e-3 / GAMMA,
                             output="excited_population", output_when="final", integral_weights=weights)
    solve_mod.solve_lindblad(view, rho0, t_span, solver="dopri5", abstol=1e-11, reltol=1e-8, dt=1e-3 / GAMMA,
                             output="selected", output_indices=[(0, 13), (14, 2), (5, 5)],
                             saveat=np.linspace(0.0, t_span[1], 11))
    pb = np.array([[GAMMA * 0.5, 0.3 * GAMMA, 0.2], [GAMMA * 2.0, -1.0 * GAMMA, 1.1]], dtype=np.complex128)
    batch_mod.parameter_scan(view, rho0, t_span, parameter_slots=["rabi", "detuning", "theta"], parameter_batch=pb,
                             solver="tsit5", abstol=1e-11, reltol=1e-8, dt=1e-3 / GAMMA,
                             output="excited_population", integral_weights=weights)
    batch_mod.solve_lindblad_batch(view, np.stack([rho0, rho0]), t_span, solver="dopri5", abstol=1e-11, reltol=1e-8,
                                   dt=1e-3 / GAMMA, output="populations", output_when="saveat",
                                   saveat=np.linspace(0.0, t_span[1], 5))
    batch_mod.grid_scan(view, rho0, t_span, scan={"detuning": np.linspace(-GAMMA, GAMMA, 3), "rabi": [GAMMA, 2 * GAMMA]},
                        solver="dopri5", abstol=1e-11, reltol=1e-8, dt=1e-3 / GAMMA,
                        output="photon_integral", integral_weights=[(13, GAMMA), (14, GAMMA), (15, GAMMA)])
    del sys.modules["centrex_tlf.centrex_tlf_rust"]
    return {"slot_names": slots, "calls": calls}


def fixed_step_kat() -> dict:
    """Known answers of the reference's fixed-step benchmark (benchmarks/bench_fixed_step_solvers.py:
    two-level system with Omega=0.8, delta=0, t in [0, 0.8], photon_integral with weights
    [(1, 0.3)], output_when="final", saveat None; adaptive Dopri5 at rtol 1e-8, atol 1e-10,
    dt 1e-3 as the reference run; the detuning grid is linspace(-2, 2, 201))."""
    import csv

    res = _reference_path() / "benchmarks" / "fixed_step_solver_results"
    counts = {}
    runtime_table = (res / "fixed_step_solver_report.md").read_text().split("## Validation")[0]
    for line in runtime_table.splitlines():
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) == 7 and cells[1] in ("single", "grid") and cells[5].isdigit():
            counts[(cells[0], cells[1], int(cells[2]))] = (int(cells[5]), int(cells[6]))
    cases = {}
    for label, mode, threads in counts:
        if threads == 4:
            continue
        solver, dt = "dopri5", 1e-3
        if label != "adaptive_dopri5":
            solver = label.rsplit("_dt", 1)[0]
            dt = float(label.rsplit("_dt", 1)[1].replace("p", "."))
        c = cases.setdefault(label, {"solver": solver, "dt": dt})
        c[f"{mode}_accepted_steps"], c[f"{mode}_rhs_calls"] = counts[(label, mode, threads)]
    with open(res / "fixed_step_solver_validation.csv") as f:
        for row in csv.DictReader(f):
            if row["mode"] == "single":
                cases[row["case"]]["abs_error_vs_adaptive"] = float(row["photon_integral_abs_error"])
                cases[row["case"]]["rel_error_vs_adaptive"] = float(row["photon_integral_rel_error"])
    return {
        "omega": 0.8, "delta": 0.0, "t_span": [0.0, 0.8], "weights": [[1, 0.3]], "abstol": 1e-10, "reltol": 1e-8,
        "grid_detuning": np.linspace(-2.0, 2.0, 201), "cases": cases,
    }


# The coefficient helpers of the expression VM (centrex_tlf/lindblad/helper_functions.py:35-51),
# each driving the Rabi coupling of a two-level system as a function of time, with the argument
# sets of the reference's own helper tests (tests/lindblad/test_parameter_helper_wrappers.py)
# and some arguments as parameter slots (so overrides reach them).
def _helper_cases():
    from centrex_tlf.lindblad import parameters as P

    def tup(p, name, v):
        return p.real(name, v)

    return [
        (1, "gaussian_2d", lambda p: P.gaussian_2d(p.time(), p.real("y", -0.2), p.real("amp", 1.3), 0.0, 0.1, 0.5, 0.7)),
        (2, "gaussian_2d_rotated",
         lambda p: P.gaussian_2d_rotated(p.time(), -0.2, 1.3, p.real("x0", 0.0), 0.1, 0.5, 0.7, p.real("angle", 0.3))),
        (2, "gaussian_2d_theta", lambda p: P.gaussian_2d(p.time(), -0.1, 1.3, 0.0, 0.1, 0.5, 0.7, theta=0.3)),
        (3, "phase_modulation", lambda p: P.phase_modulation(p.time(), p.real("beta", 3.8), p.real("omega_m", 1.2))),
        (4, "square_wave", lambda p: P.square_wave(p.time(), p.real("omega_s", 1.2), 0.3)),
        (5, "resonant_polarization_modulation",
         lambda p: P.resonant_polarization_modulation(p.time(), p.real("gamma_m", 0.4), 1.2)),
        (6, "sawtooth_wave", lambda p: P.sawtooth_wave(p.time(), 1.2, p.real("phase", 0.3))),
        (7, "variable_on_off", lambda p: P.variable_on_off(p.time(), p.real("ton", 0.1), 0.3, 0.0)),
        (8, "multipass_2d_intensity",
         lambda p: P.multipass_2d_intensity(p.time(), -0.2, tup(p, "amps", (1.0, 0.5)), tup(p, "xlocs", (-0.3, 0.4)),
                                            tup(p, "ylocs", (0.25, -0.1)), 0.7, 0.9)),
        (9, "rabi_from_intensity", lambda p: 1e-5 * P.rabi_from_intensity(2.0 + p.time() * p.time(), p.real("coupling", 0.4))),
        (10, "multipass_2d_rabi",
         lambda p: 1e-5 * P.multipass_2d_rabi(p.time(), -0.2, tup(p, "amps", (1.0, 0.5)), tup(p, "xlocs", (-0.3, 0.4)),
                                              tup(p, "ylocs", (0.25, -0.1)), 0.7, 0.9, 0.35)),
        (11, "gaussian_beam_rabi",
         lambda p: 1e-5 * P.gaussian_beam_rabi(p.time(), -0.2, p.real("intensity", 2.0), -0.3, 0.4, 0.7, 0.9, 0.35)),
        (12, "variable_on_off_duty", lambda p: P.variable_on_off_duty(p.time(), p.real("duty", 0.25), 2.5, 0.1)),
        (12, "variable_on_off_duty_invT", lambda p: P.variable_on_off_duty_invT(p.time(), 0.25, 1.3, 0.7)),
        (13, "alternating_sign", lambda p: P.alternating_sign(p.time(), 0.0, p.real("width", 0.5))),
        (14, "linear_interp",
         lambda p: P.linear_interp(p.time(), tup(p, "grid", (0.0, 0.5, 1.0, 2.0)), tup(p, "values", (2.0, 3.0, 4.0, 3.5)))),
        (15, "gaussian_1d", lambda p: P.gaussian_1d(p.time(), p.real("center", 0.0), 0.5)),
        # the first two and last two intervals have equal slopes: there SciPy's three-point end
        # derivative (Python helper) and plan.rs:55-56's end secant (Rust) coincide
        (16, "pchip_interp",
         lambda p: P.pchip_interp(p.time(), tup(p, "grid", (0.0, 0.5, 1.0, 1.5, 2.0, 2.5)),
                                  tup(p, "values", (2.0, 3.0, 4.0, 2.5, 1.0, -0.5)))),
    ]


def save_helpers(centrex_tlf) -> None:
    """``helpers.json``: one two-level plan per helper case, and packed states, times, overrides and
    the reference's Python RHS (``structured_rhs``, reference_dense.py:68-77, whose coefficients come
    from the reference's Python parameter graph and Hamiltonian fill, ir.py:882-1026) at times that
    span several periods of the periodic helpers and the ends of the interpolation tables.  Times
    within 1e-7 of a discontinuity (where the last bit decides the side) are left out.

    Beyond the ends of a ``pchip_interp`` table the reference's two evaluators disagree: the Rust
    VM holds the end values (rust/src/lindblad/plan.rs:90-100, eval.rs:306-311), SciPy's
    ``PchipInterpolator(extrapolate=True)`` in the Python helper extrapolates the end cubic.  The
    hot path is the Rust one, so those cases record the Python RHS at the clamped time (the
    plan depends on time only through the helper) and say so in ``convention``."""
    import sympy as smp
    from centrex_tlf.lindblad.parameters import LindbladParameters
    from centrex_tlf.lindblad.plan_static import prepare_lindblad_problem
    from centrex_tlf.lindblad.reference_dense import structured_rhs
    from centrex_tlf.lindblad.utils_setup import OBESystem

    om, de = smp.symbols("Omega delta", real=True)
    hamiltonian = smp.Matrix([[0, om / 2], [smp.conjugate(om) / 2, -de]])
    c_array = np.zeros((1, 2, 2), dtype=np.complex128)
    c_array[0, 0, 1] = np.sqrt(0.3)
    zeros = np.zeros((2, 2), dtype=np.complex128)
    times = [-1.93, -1.21, -0.77, -0.31, 0.0, 0.137, 0.41, 0.66, 0.93, 1.37, 1.81, 2.44, 3.1, 5.27]
    rng = np.random.default_rng(1616)
    out = []
    for helper_id, name, build in _helper_cases():
        system = OBESystem(ground=[], excited=[], QN=[], H_int=zeros, V_ref_int=zeros, couplings=[],
                           H_symbolic=hamiltonian, C_array=c_array, system=None, coupling_symbols=[om, de],
                           polarization_symbols=[])
        params = LindbladParameters()
        params.bind(om, build(params), finalize=False)
        params.bind(de, 0.1)
        prepared = prepare_lindblad_problem(system, params, backend="python", hamiltonian_representation="decomposed")
        slots = prepared.parameter_graph["slot_names"]
        scalar_slots = [i for i, v in enumerate(prepared.parameter_graph["base_values"]) if v.get("kind") != "tuple"]
        overrides = [{}]
        if scalar_slots:
            k = scalar_slots[0]
            base = prepared.parameter_graph["base_values"][k]["re"]
            overrides.append({k: complex(base * 1.15 + 0.05)})
        cases = []
        for over in overrides:
            view = _with_base_overrides(prepared, over)
            for t in times:
                rho = _hermitian(rng, 2, 0.5)
                packed = prepared.layout.pack(rho)
                t_eval, convention = float(t), "python"
                if name == "pchip_interp" and not 0.0 <= t <= 2.5:
                    t_eval, convention = min(max(float(t), 0.0), 2.5), "rust end clamp"
                dy = structured_rhs(view, packed, t_eval)
                jump = max(np.max(np.abs(structured_rhs(view, packed, t_eval + s) - dy)) for s in (-1e-7, 1e-7))
                if jump > 1e-4 * max(float(np.max(np.abs(dy))), 1e-300):
                    continue
                cases.append({
                    "t": float(t),
                    "override_slots": np.array(sorted(over), dtype=np.int64),
                    "override_values": np.array([over[k] for k in sorted(over)], dtype=np.complex128),
                    "packed": packed,
                    "structured": dy,
                    "convention": convention,
                })
        out.append({"helper_id": helper_id, "name": name, "slot_names": slots, "payload": prepared.to_payload(),
                    "cases": cases})
    codec.save("helpers", {"helpers": out})


def main() -> None:
    if "--helpers" in sys.argv:
        save_helpers(_import_reference())
        return
    if "--kat-fixed-step" in sys.argv:
        codec.save("kat_fixed_step", fixed_step_kat())
        return
    if "--rc-76" in sys.argv:
        save_rc_76(_import_reference())
        return
    if "--multi" in sys.argv:
        save_multi(_import_reference())
        return
    if "--r2-38" in sys.argv:
        save_r2_38(_import_reference())
        return
    if "--effective" in sys.argv:
        save_effective(_import_reference())
        return
    centrex_tlf = _import_reference()
    started = time.perf_counter()

    # --- two-level known-answer system -----------------------------------------------------
    two = build_two_level(centrex_tlf, omega=0.6, delta=0.0)
    rho2 = np.zeros((2, 2), dtype=np.complex128)
    rho2[0, 0] = 1.0
    codec.save(
        "plan_two_level",
        {
            "payload": two.to_payload(),
            "rho0_packed": two.layout.pack(rho2),
            "t_span": [0.0, 0.5],
            # benchmarks/expanded_sparse_packed_rhs_results/validation.csv:6 and
            # solve_timings.csv:2 (Rust FP64 Dopri5, rtol 1e-8, atol 1e-10, dt 1e-3,
            # photon_integral weights [(1, 0.3)], output_when="final").
            "kat": {
                "photon_integral": 0.001068126891997914,
                "accepted_steps": 10,
                "rejected_steps": 0,
                "rhs_calls": 61,
                "abstol": 1e-10,
                "reltol": 1e-8,
                "dt": 1e-3,
                "weights": [[1, 0.3]],
            },
            # grid_timings.csv:2: 25-point detuning grid, 4 threads.
            "kat_grid": {"detuning": np.linspace(-0.4, 0.4, 25), "accepted_steps": 252, "rejected_steps": 0, "rhs_calls": 1537},
        },
    )
    codec.save("rhs_two_level", {"cases": rhs_vectors(two, [0.0, 0.41], [{}, {0: 0.9, 1: 0.2}], seed=1)})
    codec.save("rk45_two_level", rk45_solve(two, rho2, (0.0, 0.5), np.linspace(0.0, 0.5, 11), 1e-10, 1e-8))

    two_td = build_two_level(centrex_tlf, time_dependent=True)
    codec.save("plan_two_level_td", {"payload": two_td.to_payload(), "rho0_packed": two_td.layout.pack(rho2), "t_span": [0.0, 5.0]})
    codec.save("rhs_two_level_td", {"cases": rhs_vectors(two_td, [0.0, 0.41, 2.3], [{}], seed=2)})
    codec.save("rk45_two_level_td", rk45_solve(two_td, rho2, (0.0, 5.0), np.linspace(0.0, 5.0, 21), 1e-10, 1e-8))

    # --- chains on both sides of the 40-state partition gate -------------------------------
    for n_states in (3, 45):
        chain = build_chain(centrex_tlf, n_states)
        rho_c = np.zeros((n_states, n_states), dtype=np.complex128)
        rho_c[0, 0] = 1.0
        codec.save(
            f"plan_chain{n_states}",
            {"payload": chain.to_payload(), "rho0_packed": chain.layout.pack(rho_c), "t_span": [0.0, 4.0]},
        )
        codec.save(f"rhs_chain{n_states}", {"cases": rhs_vectors(chain, [0.0, 0.41], [{}, {3: 0.35}], seed=3 + n_states)})
        if n_states == 3:
            codec.save("rk45_chain3", rk45_solve(chain, rho_c, (0.0, 4.0), np.linspace(0.0, 4.0, 9), 1e-10, 1e-8))

    # --- 16-state TlF Q(1) system ----------------------------------------------------------
    q1, labels = build_q1_16(centrex_tlf)
    rho_q = np.zeros((16, 16), dtype=np.complex128)
    for i in range(12):
        rho_q[i, i] = 1.0 / 12.0
    slots = q1.parameter_graph["slot_names"]
    codec.save(
        "plan_q1_16",
        {
            "payload": q1.to_payload(),
            "rho0_packed": q1.layout.pack(rho_q),
            "t_span": [0.0, 200.0 / GAMMA],
            "gamma": GAMMA,
            "state_labels": labels,
            "excited_indices": [13, 14, 15],
            "scan_slots": ["rabi", "detuning", "theta", "t_center"],
        },
    )
    ov = [
        {},
        {slots.index("rabi"): 3.0 * GAMMA, slots.index("detuning"): -2.0 * GAMMA, slots.index("theta"): 0.7},
        {slots.index("rabi"): 0.2 * GAMMA, slots.index("detuning"): 4.5 * GAMMA, slots.index("theta"): 2.9},
    ]
    codec.save("rhs_q1_16", {"cases": rhs_vectors(q1, [0.0, 80.0 / GAMMA, 100.0 / GAMMA, 130.0 / GAMMA], ov, seed=16, scale=0.05)})
    t_q = (0.0, 200.0 / GAMMA)
    rk = {}
    for key, over in (("nominal", {}), ("detuned", ov[1])):
        rk[key] = rk45_solve(q1, rho_q, t_q, np.linspace(0.0, t_q[1], 9), 1e-11, 1e-8, overrides=over)
        rk[key]["override_slots"] = np.array(sorted(over), dtype=np.int64)
        rk[key]["override_values"] = np.array([over[k] for k in sorted(over)], dtype=np.complex128)
    codec.save("rk45_q1_16", rk)

    codec.save("kat_fixed_step", fixed_step_kat())

    # --- 76-state rotational-cooling system (the large-system path, n > 45) ------------------
    save_rc_76(centrex_tlf)
    save_multi(centrex_tlf)
    save_r2_38(centrex_tlf)
    save_effective(centrex_tlf)
    save_helpers(centrex_tlf)

    # --- the native-boundary call contract of the reference's Python surface ----------------
    codec.save("ffi_calls", record_ffi_calls(centrex_tlf, q1, rho_q))
    print(f"fixtures written in {time.perf_counter() - started:.1f} s")


if __name__ == "__main__":
    main()
