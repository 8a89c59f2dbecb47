"""The device solver against the reference's pose-term unit tests (the cases
of tests/pose_reference_scenarios.py), solved on the GPU with the tests'
settings (PCG to 1e-14 in place of DENSE_SCHUR) and checked with the tests'
own assertions and tolerances."""
import pytest

import pose_reference_scenarios as P
from maplab_gb300 import ba

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", P.CASES, ids=[c["name"] for c in P.CASES])
def test_reference_pose_extrinsics_case_on_the_device(case):
    own = P.extrinsics_problem(case)
    with ba.BundleAdjuster(own.desc) as g:
        s = g.solve(P.extrinsics_options(ba.default_options, device=True))
        st = g.read_state()
    fails = P.extrinsics_check(case, own, s, st["kf_q_IM_p_MI"])
    assert not fails, fails


def test_reference_pose_parameterization_on_the_device():
    own = P.parameterization_problem()
    with ba.BundleAdjuster(own.desc) as g:
        s = g.solve(P.parameterization_options(ba.default_options, device=True))
        st = g.read_state()
    fails = P.parameterization_check(s, st["kf_q_IM_p_MI"])
    assert not fails, fails
