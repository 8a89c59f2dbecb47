"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure only: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use it as the checker; the product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

from maplab_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        subprocess.check_call(["make", "-s", "-C", ORACLE_DIR])
    lib = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    dp = N.c_double_p
    sig = {
        "oracle_create": (ctypes.c_int, [ctypes.POINTER(N.ProblemDesc), ctypes.POINTER(vp)]),
        "oracle_destroy": (None, [vp]),
        "oracle_set_threads": (None, [vp, ctypes.c_int]),
        "oracle_evaluate_visual": (ctypes.c_int, [vp, dp, ctypes.POINTER(dp)]),
        "oracle_evaluate_inertial": (ctypes.c_int, [vp, dp, ctypes.POINTER(dp)]),
        "oracle_linearize_visual": (ctypes.c_int, [vp, dp, dp, dp, dp, dp]),
        "oracle_solve": (ctypes.c_int, [vp, ctypes.POINTER(N.SolverOptions), ctypes.POINTER(N.Summary)]),
        "oracle_read_state": (ctypes.c_int, [vp, dp, dp, dp, dp, dp]),
        "oracle_read_calibration": (ctypes.c_int, [vp, ctypes.POINTER(N.Camera), dp]),
        "oracle_linearize_pose_edges": (ctypes.c_int, [vp, dp, dp, dp]),
        "oracle_pose_edge": (ctypes.c_int, [dp, dp, dp, dp, dp, dp, dp, dp]),
        "oracle_loop_closure": (ctypes.c_int, [dp, dp, dp, dp, dp, dp, dp, dp, dp]),
        "oracle_absolute_pose": (ctypes.c_int, [dp, dp, dp, dp, dp, dp, dp]),
        "oracle_read_switches": (ctypes.c_int, [vp, dp]),
        "oracle_landmark_quality": (ctypes.c_int, [vp, ctypes.POINTER(N.LandmarkQualityOptions),
                                                   ctypes.POINTER(ctypes.c_uint8)]),
        "oracle_reduced_system": (ctypes.c_int, [vp, ctypes.POINTER(N.SolverOptions), ctypes.c_double, dp, dp]),
        "oracle_write_state": (ctypes.c_int, [vp, dp, dp, dp, dp, dp]),
        "oracle_time_visual": (ctypes.c_double, [vp, ctypes.c_int, ctypes.c_int64, ctypes.c_int]),
        "oracle_imu_integrate": (None, [dp, dp, dp, ctypes.c_double, dp, dp, dp]),
        "oracle_quat_jacobian": (None, [dp, dp]),
        "oracle_quat_plus": (None, [dp, dp, dp]),
        "oracle_yaw_plus": (None, [dp, dp, dp]),
        "oracle_yaw_jacobian": (None, [dp, dp]),
        "oracle_rollpitch_plus": (None, [dp, dp, dp, dp]),
        "oracle_rollpitch_jacobian": (None, [dp, dp, dp]),
        "oracle_rotation_matrix": (None, [dp, dp]),
        "oracle_visual_term": (ctypes.c_int, [ctypes.POINTER(dp), dp, ctypes.c_double, ctypes.c_int,
                                              ctypes.POINTER(N.Camera), dp, ctypes.POINTER(dp),
                                              ctypes.POINTER(ctypes.c_int)]),
        "oracle_inertial_term": (ctypes.c_int, [dp, ctypes.POINTER(dp), ctypes.c_int, N.c_int64_p, dp, dp,
                                                ctypes.POINTER(dp)]),
        "oracle_project": (ctypes.c_int, [ctypes.POINTER(N.Camera), dp, dp, dp, dp, dp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def arr(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


def ptr_array(arrays):
    """ctypes array of double* from a list of arrays / None."""
    out = (N.c_double_p * len(arrays))()
    for i, a in enumerate(arrays):
        out[i] = N.ptr(a) if a is not None else None
    return out


class OracleProblem:
    VISUAL_BLOCK_SIZES = [6, 14, 14, 14, 14, 8, 6, 8, 8]
    INERTIAL_BLOCK_SIZES = [105, 45, 45, 45, 105, 45, 45, 45]

    def __init__(self, desc, threads=None):
        self.lib = load()
        self.desc = desc
        h = ctypes.c_void_p()
        st = self.lib.oracle_create(ctypes.byref(desc), ctypes.byref(h))
        if st != 0:
            raise RuntimeError(f"oracle_create failed: {st}")
        self.h = h
        if threads:
            self.lib.oracle_set_threads(self.h, threads)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    def evaluate_visual(self):
        n = self.desc.num_observations
        r = np.zeros((n, 2))
        J = [np.zeros((n, s)) for s in self.VISUAL_BLOCK_SIZES]
        self.lib.oracle_evaluate_visual(self.h, N.ptr(r), ptr_array(J))
        return r, J

    def evaluate_inertial(self):
        n = self.desc.num_imu_edges
        r = np.zeros((n, 15))
        J = [np.zeros((n, s)) for s in self.INERTIAL_BLOCK_SIZES]
        st = self.lib.oracle_evaluate_inertial(self.h, N.ptr(r), ptr_array(J))
        return st, r, J

    def linearize_visual(self):
        n = self.desc.num_observations
        r = np.zeros((n, 2)); Jl = np.zeros((n, 6)); Js = np.zeros((n, 12)); Jo = np.zeros((n, 12))
        c = ctypes.c_double()
        self.lib.oracle_linearize_visual(self.h, N.ptr(r), N.ptr(Jl), N.ptr(Js), N.ptr(Jo), ctypes.byref(c))
        return r, Jl, Js, Jo, c.value

    def cost(self):
        c = ctypes.c_double()
        self.lib.oracle_linearize_visual(self.h, None, None, None, None, ctypes.byref(c))
        return c.value

    def solve(self, opts):
        s = N.make_summary(256)
        st = self.lib.oracle_solve(self.h, ctypes.byref(opts), ctypes.byref(s))
        if st != 0:
            raise RuntimeError(f"oracle_solve failed: {st}")
        return N.summary_dict(s)

    def reduced_system(self, opts, radius):
        """Dense damped, Jacobi-scaled reduced camera system (A, b) of the
        first LM iteration at trust-region radius `radius`."""
        n = 15 * self.desc.num_keyframes
        A = np.zeros((n, n)); b = np.zeros(n)
        st = self.lib.oracle_reduced_system(self.h, ctypes.byref(opts), radius, N.ptr(A), N.ptr(b))
        if st != 0:
            raise RuntimeError(f"oracle_reduced_system failed: {st}")
        return A, b

    def landmark_quality(self, opts):
        good = np.zeros(max(1, self.desc.num_landmarks), dtype=np.uint8)
        self.lib.oracle_landmark_quality(self.h, ctypes.byref(opts), good.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        return good[:self.desc.num_landmarks].astype(bool)

    def read_switches(self):
        s = np.zeros(self.desc.num_pose_edges)
        self.lib.oracle_read_switches(self.h, N.ptr(s))
        return s

    def linearize_pose_edges(self):
        n = self.desc.num_pose_edges
        r = np.zeros((n, 6)); Jf = np.zeros((n, 36)); Jt = np.zeros((n, 36))
        self.lib.oracle_linearize_pose_edges(self.h, N.ptr(r), N.ptr(Jf), N.ptr(Jt))
        return r, Jf, Jt

    def read_state(self):
        d = self.desc
        kx = np.zeros((d.num_keyframes, 7)); kv = np.zeros((d.num_keyframes, 3))
        kbg = np.zeros((d.num_keyframes, 3)); kba = np.zeros((d.num_keyframes, 3))
        lp = np.zeros((d.num_landmarks, 3))
        self.lib.oracle_read_state(self.h, N.ptr(kx), N.ptr(kv), N.ptr(kbg), N.ptr(kba), N.ptr(lp))
        return dict(kf_q_IM_p_MI=kx, kf_v_M=kv, kf_b_g=kbg, kf_b_a=kba, lm_p_B=lp)

    def read_calibration(self):
        """Cameras and mission baseframes of the current state."""
        d = self.desc
        cams = (N.Camera * d.num_cameras)()
        mis = np.zeros((d.num_missions, 7))
        self.lib.oracle_read_calibration(self.h, cams, N.ptr(mis))
        return N.calibration_dict(cams, mis)

    def write_state(self, st):
        self.lib.oracle_write_state(self.h, N.ptr(st.get("kf_q_IM_p_MI")), N.ptr(st.get("kf_v_M")),
                                    N.ptr(st.get("kf_b_g")), N.ptr(st.get("kf_b_a")), N.ptr(st.get("lm_p_B")))

    def time_visual(self, threads, sample, reps=1):
        return self.lib.oracle_time_visual(self.h, threads, sample, reps)
