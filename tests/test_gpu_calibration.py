"""Camera calibration and mission baseframes as variables on the device
against the oracle.

maplab frees the intrinsics / distortion and the camera extrinsics with
ba_fix_ncamera_intrinsics / ba_fix_ncamera_extrinsics_* = false
(vi-optimization-builder.cc:24-35, optimization-terms-addition.cc:203-234),
and the mission baseframes when they are not fixed (:366-371, with
JplYawOnlyPoseParameterization).  Bar: the device LM (block-Jacobi PCG run to
1e-12) matches the oracle's exact-Schur LM per iteration to 1e-6 in cost, and
the recovered calibration agrees.
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu

ALL_CAM = N.MBA_CAM_INTRINSICS_FREE | N.MBA_CAM_DISTORTION_FREE | N.MBA_CAM_ROTATION_FREE | N.MBA_CAM_TRANSLATION_FREE


def _set_flags(m, cam_flags=None, mis_flags=None):
    keep = {}
    if cam_flags is not None:
        keep["cam"] = np.ascontiguousarray(cam_flags, dtype=np.uint32)
        m.desc.camera_flags = N.ptr(keep["cam"], ctypes.c_uint32)
    if mis_flags is not None:
        keep["mis"] = np.ascontiguousarray(mis_flags, dtype=np.uint32)
        m.desc.mission_flags = N.ptr(keep["mis"], ctypes.c_uint32)
    m._flag_arrays = keep


def _oracle_opts(iters):
    o = N.default_solver_options()
    o.max_num_iterations = iters
    o.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    o.check_tolerances = 0
    o.reject_outliers_every_n_iters = 0
    return o


def _gpu_opts(iters, **kw):
    return ba.default_options(max_num_iterations=iters, check_tolerances=0, reject_outliers_every_n_iters=0,
                              linear_tolerance=1e-12, max_linear_iterations=6000, **kw)


def _compare(m, iters=6, **kw):
    so = O.OracleProblem(m.desc)
    s_o = so.solve(_oracle_opts(iters))
    cal_o = so.read_calibration()
    with ba.BundleAdjuster(m.desc) as g:
        s_g = g.solve(_gpu_opts(iters, **kw))
        cal_g = g.read_calibration()
    assert abs(s_g["initial_cost"] - s_o["initial_cost"]) <= 1e-12 * s_o["initial_cost"]
    for a, b in zip(s_g["iterations"], s_o["iterations"]):
        assert abs(a["cost"] - b["cost"]) <= 1e-6 * b["cost"], (a, b)
        assert a["ok"] == b["ok"]
    assert abs(s_g["final_cost"] - s_o["final_cost"]) <= 1e-6 * s_o["final_cost"]
    return s_g, s_o, cal_g, cal_o


def test_free_camera_calibration_matches_oracle():
    """One camera of a visual-inertial map with every calibration block free,
    starting from perturbed intrinsics and extrinsics."""
    m = synth.generate("c1", keyframes_per_mission=30, num_landmarks=600)
    cam = m.desc.cameras[0]
    cam.intrinsics[0] += 4.0
    cam.intrinsics[1] -= 3.0
    cam.intrinsics[2] += 2.0
    cam.intrinsics[3] -= 1.5
    for a, d in enumerate((0.01, -0.008, 0.005)):
        cam.q_CI_p_CI[4 + a] += d
    _set_flags(m, cam_flags=[ALL_CAM] * m.desc.num_cameras)
    s_g, s_o, cal_g, cal_o = _compare(m)
    assert s_g["final_cost"] < 0.5 * s_g["initial_cost"]
    np.testing.assert_allclose(cal_g["intrinsics"], cal_o["intrinsics"], rtol=0, atol=1e-4)
    np.testing.assert_allclose(cal_g["distortion"], cal_o["distortion"], rtol=0, atol=1e-7)
    np.testing.assert_allclose(cal_g["q_CI"], cal_o["q_CI"], rtol=0, atol=1e-7)
    np.testing.assert_allclose(cal_g["p_CI"], cal_o["p_CI"], rtol=0, atol=1e-7)


def test_free_baseframes_match_oracle():
    """Three co-registered missions (kGlobal terms): mission 1's baseframe
    free with maplab's yaw + position parameterization, mission 2's with the
    full pose parameterization; their keyframe poses held, so the baseframes
    carry the cross-mission alignment."""
    m = synth.generate("c4", num_missions=3, keyframes_per_mission=30, num_landmarks=1500,
                       shared_landmark_fraction=0.3, include_inertial=0)
    mis = m.array("mission_q_GM_p_GM")
    mis[1, 4:] += [0.05, -0.03, 0.02]
    mis[2, 4:] += [-0.04, 0.02, 0.01]
    kf_mis = m.array("kf_mission")
    flags = m.array("kf_flags")
    flags[kf_mis > 0] |= N.MBA_KF_POSE_CONSTANT
    _set_flags(m, mis_flags=[0, N.MBA_MIS_BASEFRAME_YAW_POSITION, N.MBA_MIS_BASEFRAME_POSE])
    s_g, s_o, cal_g, cal_o = _compare(m)
    np.testing.assert_allclose(cal_g["baseframes"], cal_o["baseframes"], rtol=0, atol=1e-7)
    assert np.abs(cal_g["baseframes"][0] - mis[0]).max() == 0.0  # the constant baseframe is untouched
    assert np.abs(cal_g["baseframes"][1:] - mis[1:]).max() > 1e-4  # the free ones moved


def test_free_calibration_refused_in_mixed_precision():
    m = synth.generate("c1", keyframes_per_mission=20, num_landmarks=200)
    _set_flags(m, cam_flags=[N.MBA_CAM_INTRINSICS_FREE] * m.desc.num_cameras)
    with ba.BundleAdjuster(m.desc) as g:
        with pytest.raises(ba.BAError) as e:
            g.solve(ba.default_options(max_num_iterations=2, precision=N.MBA_PRECISION_MIXED))
        assert e.value.status == N.MBA_ERR_INVALID_ARG
