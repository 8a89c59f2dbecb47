"""Landmark quality filter (isVisualLandmarkWellConstrained) on the device
against the oracle: identical flags with the elq_* defaults, with the
reprojection bound switched on, and at a perturbed state."""
import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["c1", "multi", "c2"])
def qmap(request):
    if request.param == "c1":
        return synth.generate("c1")
    if request.param == "c2":
        return synth.generate("c2", keyframes_per_mission=400, num_landmarks=40000)
    return synth.generate("c4", num_missions=3, keyframes_per_mission=60, num_landmarks=1500,
                          shared_landmark_fraction=0.3)


@pytest.mark.parametrize("kw", [{}, {"max_reprojection_error_px": 2.0}, {"min_observers": 6, "min_observation_angle_deg": 10.0}])
def test_landmark_quality_matches_oracle(qmap, kw):
    o = O.OracleProblem(qmap.desc)
    ref = o.landmark_quality(ba.default_landmark_quality_options(**kw))
    with ba.BundleAdjuster(qmap.desc) as g:
        got = g.landmark_quality(**kw)
    assert (got != ref).sum() == 0, np.flatnonzero(got != ref)[:10]
    if not kw:  # the defaults keep some landmarks and drop others on these maps
        assert 0 < got.sum() < len(got)


def test_landmark_quality_follows_the_state():
    """Evaluated at the handle's current state: after a solve the verdicts are
    those of the oracle at the same (written-back) state."""
    m = synth.generate("c1")
    with ba.BundleAdjuster(m.desc) as g:
        g.solve(ba.default_options(max_num_iterations=5, check_tolerances=0))
        st = g.read_state()
        got = g.landmark_quality()
    o = O.OracleProblem(m.desc)
    o.write_state(st)
    ref = o.landmark_quality(ba.default_landmark_quality_options())
    assert (got != ref).sum() == 0
