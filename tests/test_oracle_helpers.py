"""Pin the oracle's expression-VM helpers against the reference's Python evaluator.

``tests/golden/helpers.json`` (made by ``make_fixtures.py --helpers``) holds one two-level plan
per coefficient helper of the reference's VM (helper IDs 1-16,
centrex_tlf/lindblad/helper_functions.py:35-51, including the tuple helpers
``multipass_2d_*``, ``linear_interp`` and ``pchip_interp``), with the argument sets of the
reference's own helper tests (tests/lindblad/test_parameter_helper_wrappers.py), and the
reference's Python RHS at times across several periods and beyond the tables' ends, with and
without a base-slot override.  The RHS is linear in the helper's value, so agreement of the RHS
is agreement of the helper.  Tolerance: 1e-13 of the case's largest element (libm against
Python's math module; both FP64).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle

HELPER_IDS = set(range(1, 17))


def _helper_ids(payload):
    ids = set()
    for comp in payload["parameter_graph"]["compounds"]:
        for ins in comp["expression"]["instructions"]:
            if "function" in ins and ins["function"] is not None:
                ids.add(int(ins["function"]))
    return ids


def test_every_helper_id_is_covered(golden):
    found = set()
    for h in golden("helpers")["helpers"]:
        ids = _helper_ids(h["payload"])
        assert h["helper_id"] in ids, h["name"]
        found |= ids
        assert len(h["cases"]) >= 10
    assert HELPER_IDS <= found


@pytest.mark.parametrize("index", range(18))
def test_oracle_helper_rhs_matches_python_reference(golden, index):
    h = golden("helpers")["helpers"][index]
    plan = oracle.OraclePlan(h["payload"])
    for case in h["cases"]:
        dy = plan.rhs(case["packed"], case["t"], case["override_slots"], case["override_values"])
        ref = case["structured"]
        scale = float(np.max(np.abs(ref)))
        assert np.max(np.abs(dy - ref)) <= 1e-13 * scale, (h["name"], case["t"])
