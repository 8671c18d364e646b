"""The reference's own Python surface driving this package (CPU side of the drop-in).

With ``centrex_tlf_rust.install()`` the reference's unchanged ``prepare_lindblad_problem``
(plan_static.py:137-185, ``backend="rust"``), ``solve_lindblad`` (solve.py:504-694),
``parameter_scan`` (batch.py:313-340), ``solve_lindblad_batch`` (batch.py:143-301) and
``grid_scan`` (batch.py:343-519) reach this package's native-call functions.  Without a GPU the
calls end in this package's "no CUDA device" refusal, which shows that each one got through the
reference's validation and marshalling to the GB300 boundary and that nothing fell back to a CPU
solver.  The same calls' arguments are replayed on the GPU in test_gpu_dropin_replay.py.

Needs a CeNTREX-TlF checkout named by ``CENTREX_REFERENCE``; skipped otherwise (the reference is
not shipped with this repository).
"""

from __future__ import annotations

import os
import sys

import numpy as np
import pytest

REF = os.environ.get("CENTREX_REFERENCE")
pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="CENTREX_REFERENCE names no checkout")


@pytest.fixture(scope="module")
def surface():
    import make_fixtures
    from centrex_tlf_gb300 import _abi
    from centrex_tlf_gb300 import centrex_tlf_rust as api

    if _abi.load_library().obe_device_count() > 0:
        pytest.skip("a GPU is present: the solves would run (the GPU replay covers them)")
    centrex_tlf = make_fixtures._import_reference()
    saved = sys.modules.get("centrex_tlf.centrex_tlf_rust")
    api.install()
    try:
        from centrex_tlf import couplings, lindblad, transitions
        from centrex_tlf.lindblad.parameters import LindbladParameters
        from centrex_tlf.lindblad.plan_static import prepare_lindblad_problem

        trans = [transitions.Q1_F1_1o2_F1]
        sel = couplings.generate_transition_selectors(trans, [[couplings.polarization_Z, couplings.polarization_X]])
        obe = lindblad.generate_OBE_system_transitions(trans, sel, qn_compact=True, Γ=make_fixtures.GAMMA)
        params = LindbladParameters.from_kwargs(**make_fixtures._gaussian_pulse_parameters(False))
        prepared = prepare_lindblad_problem(obe, params, backend="rust", hamiltonian_representation="decomposed")
        yield centrex_tlf, prepared
    finally:
        if saved is None:
            sys.modules.pop("centrex_tlf.centrex_tlf_rust", None)
        else:
            sys.modules["centrex_tlf.centrex_tlf_rust"] = saved


def test_prepare_builds_this_package_plan(surface, golden):
    from centrex_tlf_gb300 import centrex_tlf_rust as api

    _, prepared = surface
    assert isinstance(prepared.rust_plan, api.PreparedLindbladPlan)
    assert prepared.rust_plan.n_states() == 16
    ref = golden("plan_q1_16")["payload"]
    got = prepared.to_payload()["expanded_rhs_plan"]
    for key in ("output_ptrs", "input_indices", "coeff_indices"):
        assert np.asarray(got[key]).tolist() == np.asarray(ref["expanded_rhs_plan"][key]).tolist()


def _rho0():
    rho = np.zeros((16, 16), dtype=np.complex128)
    for i in range(12):
        rho[i, i] = 1.0 / 12.0
    return rho


def test_surface_calls_reach_the_gpu_boundary(surface):
    import make_fixtures

    centrex_tlf, prepared = surface
    from centrex_tlf.lindblad import batch as batch_mod
    from centrex_tlf.lindblad import solve as solve_mod

    g = make_fixtures.GAMMA
    t_span = (0.0, 200.0 / g)
    w = [(13, 1.0), (14, 1.0), (15, 1.0)]
    common = dict(abstol=1e-11, reltol=1e-8, dt=1e-3 / g)
    calls = [
        lambda: solve_mod.solve_lindblad(prepared, _rho0(), t_span, solver="dopri5", output="populations",
                                         output_when="final", **common),
        lambda: batch_mod.parameter_scan(prepared, _rho0(), t_span, parameter_slots=["rabi", "detuning", "theta"],
                                         parameter_batch=np.array([[g, 0.0, 0.1]], dtype=np.complex128),
                                         solver="tsit5", output="excited_population", integral_weights=w, **common),
        lambda: batch_mod.solve_lindblad_batch(prepared, np.stack([_rho0(), _rho0()]), t_span, solver="dopri5",
                                               output="populations", **common),
        lambda: batch_mod.grid_scan(prepared, _rho0(), t_span, scan={"detuning": np.linspace(-g, g, 3)},
                                    solver="dopri5", output="photon_integral", integral_weights=w, **common),
    ]
    for call in calls:
        with pytest.raises(RuntimeError, match="no CUDA device"):
            call()
