"""The oracle against the reference's own cost-term test scenarios, verbatim.

Every TEST_F of test_visual_term_test.cc (kLocalMission),
test_mission_baseframe_visual_term_test.cc (kGlobal, non-identity mission
baseframes), test_inertial_term_test.cc and test_3keyframe_inertial_term_test.cc
(algorithms/ceres-error-terms/test/) is rebuilt from the extracted fixture
(tests/golden/error_term_scenarios.json) and solved by the oracle's LM with
the tests' own solver settings; the tests' own assertions and tolerances are
checked on the result (final cost below 1e-15 / 1e-12, recovered blocks to
1e-15 ... 1e-4, iteration counts).  These are the only reference-held numbers
that pin the visual term's frame chains (store / observer keyframes, mission
baseframes, camera extrinsics) and the inertial term end to end.
"""
import pytest

import oracle_lib as O
import reference_scenarios as R
from maplab_gb300 import _native as N

SCENARIOS = R.all_scenarios()


def test_every_reference_test_was_extracted():
    counts = {fam: len(R.GOLDEN[fam]["scenarios"]) for fam in R.FAMILIES}
    assert counts == {"visual_local_mission": 8, "visual_global": 10, "inertial_two_keyframes": 12,
                      "inertial_three_keyframes": 5}


@pytest.mark.parametrize("item", SCENARIOS, ids=R.scenario_id)
def test_reference_scenario_on_the_oracle(item):
    fam, sc = item
    b = R.build(fam, sc)
    if b.requires:
        pytest.skip("needs " + ", ".join(b.requires))
    o = O.OracleProblem(b.desc)
    s = o.solve(R.solver_options(N.default_solver_options, device=False))
    fails = R.check(b, sc, s, o.read_state(), o.read_calibration())
    assert not fails, fails
