"""The CPU oracle against the reference's pose-term unit tests: the enabled
cases of test_six_dof_block_transformation_error_term_with_extrinsics.cc and
the minimization of test_pose_parameterization_test.cc, rebuilt and checked
by tests/pose_reference_scenarios.py with the tests' own assertions and
tolerances."""
import numpy as np
import pytest

import oracle_lib as O
import pose_reference_scenarios as P
from maplab_gb300 import _native as N


def test_fixture_holds_the_enabled_cases():
    assert P.SCEN["source"].endswith("test_six_dof_block_transformation_error_term_with_extrinsics.cc")
    assert [c["name"] for c in P.CASES] == ["TestPosePriorErrorTermZeroCost",
                                            "TestPosePriorErrorTermIdentityFixBIFixGIk"]
    assert all("T_B_I" in c["fixed"] for c in P.CASES)  # the extrinsics are constant in both
    assert P.PARAM["source"].endswith("test_pose_parameterization_test.cc")


@pytest.mark.parametrize("case", P.CASES, ids=[c["name"] for c in P.CASES])
def test_reference_pose_extrinsics_case(case):
    own = P.extrinsics_problem(case)
    o = O.OracleProblem(own.desc)
    s = o.solve(P.extrinsics_options(N.default_solver_options, device=False))
    fails = P.extrinsics_check(case, own, s, o.read_state()["kf_q_IM_p_MI"])
    assert not fails, fails


def test_planted_extrinsics_convention_error_fails_the_zero_cost_case():
    """The extrinsics block given as q_B_I instead of its inverse: the
    composed measurement no longer matches, so the zero-cost assertion fails."""
    case = P.CASES[0]
    own = P.extrinsics_problem(case)
    q = np.asarray(P.SCEN["fixture"]["q_B_I"])
    own.a["pe_ext"][:4] = q
    o = O.OracleProblem(own.desc)
    s = o.solve(P.extrinsics_options(N.default_solver_options, device=False))
    assert P.extrinsics_check(case, own, s, o.read_state()["kf_q_IM_p_MI"])


def test_reference_pose_parameterization_minimization():
    own = P.parameterization_problem()
    o = O.OracleProblem(own.desc)
    s = o.solve(P.parameterization_options(N.default_solver_options, device=False))
    fails = P.parameterization_check(s, o.read_state()["kf_q_IM_p_MI"])
    assert not fails, fails
