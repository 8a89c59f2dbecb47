"""The synthetic map generator (host library): shapes of the benchmark
configurations, determinism, visibility of every measurement, gauge fixes."""
import numpy as np

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import synth


def test_c1_shapes_and_determinism():
    a = synth.generate("c1")
    b = synth.generate("c1")
    s = a.sizes
    assert s["keyframes"] == 100 and s["landmarks"] == 2000 and s["imu_edges"] == 99
    assert 8000 < s["observations"] < 12000  # U{2..8} per landmark, about 10k
    assert s["imu_samples"] == 99 * 21
    np.testing.assert_array_equal(a.array("obs_uv"), b.array("obs_uv"))
    np.testing.assert_array_equal(a.array("kf_q_IM_p_MI"), b.array("kf_q_IM_p_MI"))
    c = synth.generate("c1", seed=7)
    assert not np.array_equal(a.array("obs_uv"), c.array("obs_uv"))


def test_c1_track_lengths_and_store_keyframe():
    m = synth.generate("c1")
    lm = m.array("obs_landmark")
    counts = np.bincount(lm, minlength=m.desc.num_landmarks)
    assert counts.min() >= 2 and counts.max() <= 8
    # each landmark's store keyframe is one of its observers
    kf = m.array("obs_keyframe")
    store = m.array("lm_store_keyframe")
    for l in range(0, m.desc.num_landmarks, 97):
        assert store[l] in set(kf[lm == l])


def test_gauge_flags_vi_single_mission():
    m = synth.generate("c1")
    f = m.array("kf_flags")
    assert f[0] == (N.MBA_KF_GAUGE_ROLL_PITCH | N.MBA_KF_POSITION_CONSTANT)
    assert np.all(f[1:] == 0)


def test_ground_truth_cost_matches_noise_level():
    """At ground truth the cost is about half the number of residuals (unit
    whitened noise): pixel noise N(0,1) and the IMU noise model."""
    m = synth.generate("c1")
    o = O.OracleProblem(m.desc)
    o.write_state(m.ground_truth())
    c = o.cost()
    n_res = 2 * m.desc.num_observations + 15 * m.desc.num_imu_edges
    assert 0.4 * n_res < c < 0.6 * n_res, (c, n_res)


def test_multi_mission_shared_landmarks_produce_global_terms():
    m = synth.generate("c4", keyframes_per_mission=60, num_landmarks=3000, shared_landmark_fraction=0.3)
    kf = m.array("obs_keyframe")
    lm = m.array("obs_landmark")
    mis = m.array("kf_mission")
    store = m.array("lm_store_keyframe")
    glob = mis[kf] != mis[store[lm]]
    assert glob.sum() > 100
    # one cluster: only the first keyframe of mission 0 carries the gauge fix
    flags = m.array("kf_flags")
    assert (flags != 0).sum() == 1 and flags[0] != 0
