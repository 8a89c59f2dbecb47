"""Gauge fixes of the optimization builder (mba_gauge_fixes, host only):
mission clusters by co-observation and loop closures, observability of
scale / position / yaw / roll-pitch from the constraints every mission of a
cluster has, and the fixes on the cluster's first keyframe in the problem."""
import ctypes

import numpy as np
import pytest

from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth


def fixes(m, keep_flags=False):
    """Gauge fixes of m's descriptor with its own fix flags and constant
    landmarks removed (unless keep_flags)."""
    d = N.ProblemDesc()
    ctypes.memmove(ctypes.byref(d), ctypes.byref(m.desc), ctypes.sizeof(d))
    if not keep_flags:
        d.kf_flags = None
        d.lm_constant = None
    kf = np.zeros(d.num_keyframes, dtype=np.uint32)
    lm = np.zeros(max(1, d.num_landmarks), dtype=np.uint8)
    nc = ctypes.c_int32()
    st = ba.lib().mba_gauge_fixes(ctypes.byref(d), kf.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                  lm.ctypes.data_as(N.c_uint8_p), ctypes.byref(nc))
    assert st == 0
    return kf, lm[:d.num_landmarks], nc.value


def first_kf_of(m, mission):
    return int(np.flatnonzero(m.array("kf_mission") == mission)[0])


def test_visual_inertial_mission_fixes_yaw_and_position():
    m = synth.generate("c1")
    kf, lm, nc = fixes(m)
    assert nc == 1
    assert kf[0] == N.MBA_KF_GAUGE_ROLL_PITCH | N.MBA_KF_POSITION_CONSTANT
    assert not kf[1:].any() and not lm.any()
    # the generator applies the same rule
    np.testing.assert_array_equal(kf, m.array("kf_flags"))


def test_visual_only_mission_fixes_pose_and_scale():
    m = synth.generate("c1", include_inertial=0)
    kf, lm, nc = fixes(m)
    assert kf[0] & N.MBA_KF_POSE_CONSTANT and kf[0] & N.MBA_KF_POSITION_CONSTANT
    assert not kf[1:].any()
    store = m.array("lm_store_keyframe")
    assert lm.sum() == 1 and store[np.flatnonzero(lm)[0]] == 0
    np.testing.assert_array_equal(lm.astype(bool), m.array("lm_constant").astype(bool))


def test_co_registered_missions_form_one_cluster():
    m = synth.generate("c4", num_missions=3, keyframes_per_mission=60, num_landmarks=1500,
                       shared_landmark_fraction=0.3)
    kf, lm, nc = fixes(m)
    assert nc == 1
    assert np.flatnonzero(kf).tolist() == [first_kf_of(m, 0)]


def test_independent_missions_are_separate_clusters():
    m = synth.generate("c3", num_missions=4, kf_min=40, kf_max=60)
    kf, lm, nc = fixes(m)
    assert nc == 4
    assert np.flatnonzero(kf).tolist() == [first_kf_of(m, q) for q in range(4)]


def test_loop_closures_join_missions():
    base = dict(num_missions=2, keyframes_per_mission=60, num_landmarks=1000, co_registered=0)
    m = synth.generate("c4", **base, shared_landmark_fraction=0.0)
    assert fixes(m)[2] == 2
    m = synth.generate("c4", **base, shared_landmark_fraction=0.0, loop_closure_stride=10)
    kf, lm, nc = fixes(m)
    assert nc == 1 and np.flatnonzero(kf).tolist() == [first_kf_of(m, 0)]


def test_absolute_terms_make_the_gauge_observable():
    m = synth.generate("c1", absolute_pose_stride=25)
    kf, lm, nc = fixes(m)
    assert not kf.any() and not lm.any()
    # visual only with two absolute terms: scale observable, nothing fixed
    m = synth.generate("c1", include_inertial=0, absolute_pose_stride=50)
    kf, lm, nc = fixes(m)
    assert not kf.any() and not lm.any()


def test_odometry_makes_scale_observable():
    m = synth.generate("c1", include_inertial=0, pose_edges=1)
    kf, lm, nc = fixes(m)
    assert kf[0] & N.MBA_KF_POSE_CONSTANT and not lm.any()


def test_existing_flags_are_kept():
    m = synth.generate("c1", include_inertial=0)
    kf, lm, _ = fixes(m, keep_flags=True)
    assert (kf & m.array("kf_flags")).tolist() == m.array("kf_flags").tolist()
