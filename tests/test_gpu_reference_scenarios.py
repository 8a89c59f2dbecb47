"""The device solver against the reference's own cost-term test scenarios.

The scenarios of test_visual_term_test.cc, test_mission_baseframe_visual_term_
test.cc, test_inertial_term_test.cc and test_3keyframe_inertial_term_test.cc
(algorithms/ceres-error-terms/test/), rebuilt from tests/golden/
error_term_scenarios.json, solved on the GPU with the tests' solver settings
(block-Jacobi PCG to 1e-14 in place of DENSE_SCHUR), and checked with the
tests' own assertions and tolerances.
"""
import pytest

import reference_scenarios as R
from maplab_gb300 import ba

pytestmark = pytest.mark.gpu

SCENARIOS = R.all_scenarios()


@pytest.mark.parametrize("item", SCENARIOS, ids=R.scenario_id)
def test_reference_scenario_on_the_device(item):
    fam, sc = item
    b = R.build(fam, sc)
    if b.requires:
        pytest.skip("needs " + ", ".join(b.requires))
    with ba.BundleAdjuster(b.desc) as g:
        s = g.solve(R.solver_options(ba.default_options, device=True))
        st = g.read_state()
        cal = g.read_calibration()
    fails = R.check(b, sc, s, st, cal)
    assert not fails, fails
