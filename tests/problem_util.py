"""Helpers to build small problem descriptors from numpy arrays (tests only)."""
import ctypes

import numpy as np

from maplab_gb300 import _native as N


class OwnedDesc:
    """A ProblemDesc plus the numpy arrays it points into."""

    def __init__(self, *, obs_uv, obs_sigma, obs_landmark, obs_keyframe, obs_camera, lm_p_B, lm_store_keyframe,
                 kf_q_IM_p_MI, kf_v_M=None, kf_b_g=None, kf_b_a=None, kf_mission=None, kf_flags=None,
                 mission_q_GM_p_GM=None, cameras=(), lm_constant=None, edge_from=None, edge_to=None,
                 edge_sample_offset=None, imu_timestamp_ns=None, imu_acc_gyro=None, imu_sigmas=(0.1, 0.1, 0.1, 0.1),
                 gravity=9.81, use_huber=1, camera_flags=None, mission_flags=None):
        f64 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64))
        i32 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.int32))
        nk = len(kf_q_IM_p_MI)
        self.a = {}
        a = self.a
        a["obs_uv"] = f64(obs_uv).reshape(-1, 2)
        a["obs_sigma"] = f64(obs_sigma)
        a["obs_landmark"] = i32(obs_landmark)
        a["obs_keyframe"] = i32(obs_keyframe)
        a["obs_camera"] = i32(obs_camera)
        a["lm_p_B"] = f64(lm_p_B).reshape(-1, 3)
        a["lm_store_keyframe"] = i32(lm_store_keyframe)
        a["lm_constant"] = np.ascontiguousarray(np.asarray(lm_constant if lm_constant is not None
                                                           else np.zeros(len(a["lm_p_B"])), dtype=np.uint8))
        a["kf_q_IM_p_MI"] = f64(kf_q_IM_p_MI).reshape(-1, 7)
        a["kf_v_M"] = f64(kf_v_M if kf_v_M is not None else np.zeros((nk, 3)))
        a["kf_b_g"] = f64(kf_b_g if kf_b_g is not None else np.zeros((nk, 3)))
        a["kf_b_a"] = f64(kf_b_a if kf_b_a is not None else np.zeros((nk, 3)))
        a["kf_mission"] = i32(kf_mission if kf_mission is not None else np.zeros(nk))
        a["kf_flags"] = np.ascontiguousarray(np.asarray(kf_flags if kf_flags is not None else np.zeros(nk),
                                                        dtype=np.uint32))
        a["mission_q_GM_p_GM"] = f64(mission_q_GM_p_GM if mission_q_GM_p_GM is not None
                                     else [[0, 0, 0, 1, 0, 0, 0]]).reshape(-1, 7)
        cams = (N.Camera * len(cameras))(*cameras)
        self.cams = cams
        ne = 0 if edge_from is None else len(edge_from)
        if ne:
            a["edge_from"] = i32(edge_from)
            a["edge_to"] = i32(edge_to)
            a["edge_sample_offset"] = np.ascontiguousarray(np.asarray(edge_sample_offset, dtype=np.int64))
            a["imu_timestamp_ns"] = np.ascontiguousarray(np.asarray(imu_timestamp_ns, dtype=np.int64))
            a["imu_acc_gyro"] = f64(imu_acc_gyro).reshape(-1, 6)
        d = N.ProblemDesc()
        d.num_keyframes = nk
        d.num_landmarks = len(a["lm_p_B"])
        d.num_observations = len(a["obs_sigma"])
        d.num_cameras = len(cameras)
        d.num_missions = len(a["mission_q_GM_p_GM"])
        d.num_imu_edges = ne
        d.num_imu_samples = len(a["imu_timestamp_ns"]) if ne else 0
        d.obs_uv = N.ptr(a["obs_uv"]); d.obs_sigma = N.ptr(a["obs_sigma"])
        d.obs_landmark = N.ptr(a["obs_landmark"], ctypes.c_int32)
        d.obs_keyframe = N.ptr(a["obs_keyframe"], ctypes.c_int32)
        d.obs_camera = N.ptr(a["obs_camera"], ctypes.c_int32)
        d.lm_p_B = N.ptr(a["lm_p_B"]); d.lm_store_keyframe = N.ptr(a["lm_store_keyframe"], ctypes.c_int32)
        d.lm_constant = N.ptr(a["lm_constant"], ctypes.c_uint8)
        d.kf_q_IM_p_MI = N.ptr(a["kf_q_IM_p_MI"]); d.kf_v_M = N.ptr(a["kf_v_M"])
        d.kf_b_g = N.ptr(a["kf_b_g"]); d.kf_b_a = N.ptr(a["kf_b_a"])
        d.kf_mission = N.ptr(a["kf_mission"], ctypes.c_int32)
        d.kf_flags = N.ptr(a["kf_flags"], ctypes.c_uint32)
        d.mission_q_GM_p_GM = N.ptr(a["mission_q_GM_p_GM"])
        d.cameras = ctypes.cast(cams, ctypes.POINTER(N.Camera))
        if ne:
            d.edge_from = N.ptr(a["edge_from"], ctypes.c_int32)
            d.edge_to = N.ptr(a["edge_to"], ctypes.c_int32)
            d.edge_sample_offset = N.ptr(a["edge_sample_offset"], ctypes.c_int64)
            d.imu_timestamp_ns = N.ptr(a["imu_timestamp_ns"], ctypes.c_int64)
            d.imu_acc_gyro = N.ptr(a["imu_acc_gyro"])
        d.gyro_noise_sigma, d.gyro_bias_sigma, d.acc_noise_sigma, d.acc_bias_sigma = imu_sigmas
        d.gravity_magnitude = gravity
        d.use_huber = use_huber
        d.huber_delta_local = 3.0
        d.huber_delta_global = 10.0
        if camera_flags is not None:
            a["camera_flags"] = np.ascontiguousarray(np.asarray(camera_flags, dtype=np.uint32))
            d.camera_flags = N.ptr(a["camera_flags"], ctypes.c_uint32)
        if mission_flags is not None:
            a["mission_flags"] = np.ascontiguousarray(np.asarray(mission_flags, dtype=np.uint32))
            d.mission_flags = N.ptr(a["mission_flags"], ctypes.c_uint32)
        self.desc = d


def camera(fu=460.0, fv=460.0, cu=376.0, cv=240.0, w=752, h=480, dtype=N.MBA_DISTORTION_RADTAN,
           dist=(-0.28, 0.07, 0.0, 0.0), q_CI=(0, 0, 0, 1), p_CI=(0, 0, 0)):
    c = N.Camera()
    for i, v in enumerate((fu, fv, cu, cv)):
        c.intrinsics[i] = v
    for i, v in enumerate(dist):
        c.distortion[i] = v
    c.distortion_type = dtype
    c.width, c.height = w, h
    q = np.asarray(q_CI, dtype=np.float64)
    q = q / np.linalg.norm(q)
    for i in range(4):
        c.q_CI_p_CI[i] = q[i]
    for i in range(3):
        c.q_CI_p_CI[4 + i] = p_CI[i]
    return c


def unit_quat(x, y, z, w):
    q = np.array([x, y, z, w], dtype=np.float64)
    q /= np.linalg.norm(q)
    return q * (1 if q[3] >= 0 else -1)


def ridders(f, x0, h=1e-3, ntab=10, con=1.4):
    """Ridders' polynomial extrapolation of the derivative of f at x0
    (the method of ceres-error-terms/test/parameterization-numerical-diff-inl.h)."""
    con2 = con * con
    a = np.zeros((ntab, ntab), dtype=object)
    a[0, 0] = (f(x0 + h) - f(x0 - h)) / (2 * h)
    best = a[0, 0]
    err = np.inf
    hh = h
    for i in range(1, ntab):
        hh /= con
        a[0, i] = (f(x0 + hh) - f(x0 - hh)) / (2 * hh)
        fac = con2
        for j in range(1, i + 1):
            a[j, i] = (a[j - 1, i] * fac - a[j - 1, i - 1]) / (fac - 1)
            fac *= con2
            e = max(np.max(np.abs(a[j, i] - a[j - 1, i])), np.max(np.abs(a[j, i] - a[j - 1, i - 1])))
            if e <= err:
                err = e
                best = a[j, i]
        if np.max(np.abs(a[i, i] - a[i - 1, i - 1])) >= 2 * err:
            break
    return np.asarray(best, dtype=np.float64)
