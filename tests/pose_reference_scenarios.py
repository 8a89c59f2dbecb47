"""Problems and checks of the reference's pose-term unit tests (tests only).

* The relative pose term with extrinsics (SixDoFBlockPoseErrorTermWithExtrinsics,
  the optimization builder's odometry term): the enabled cases of
  algorithms/ceres-error-terms/test/test_six_dof_block_transformation_error_term_with_extrinsics.cc,
  from tests/golden/pose_extrinsics_scenarios.json.  Each is the test's
  two-keyframe problem: keyframe blocks q_G_I | p_G_I (Hamilton coefficients,
  as the term reads them), the extrinsics block q_I_B | p_B_I, one measured
  T_Bk_Bkp1 with identity covariance, the listed blocks held constant.
* JplPoseParameterization's minimization test
  (algorithms/ceres-error-terms/test/test_pose_parameterization_test.cc, from
  tests/golden/pose_parameterization_scenario.json): a pose block pulled onto
  a reference transformation by the error (2 vec(q (x) q_ref^-1) | p - p_ref)
  under Ceres' default options.  That error is the absolute 6-DoF term
  (BlockPosePriorErrorTermV2) with an identity baseframe, identity sensor
  extrinsics and identity covariance (its rows in the other order and, where
  w < 0, with the opposite sign: the same cost and minimum), so the case runs
  as one keyframe with one absolute pose edge.

Both fixtures are written by tests/golden/make_golden.py from the test files.
"""
import ctypes
import json
import os

import numpy as np

import problem_util as U
from maplab_gb300 import _native as N

HERE = os.path.dirname(os.path.abspath(__file__))
SCEN = json.load(open(os.path.join(HERE, "golden", "pose_extrinsics_scenarios.json")))
PARAM = json.load(open(os.path.join(HERE, "golden", "pose_parameterization_scenario.json")))
CASES = [c for c in SCEN["tests"] if "skipped" not in c]


def _hrot(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def matrix(q, p):
    """4x4 transformation of a Hamilton quaternion (x y z w) and a position."""
    T = np.eye(4)
    T[:3, :3] = _hrot(np.asarray(q) / np.linalg.norm(q))
    T[:3, 3] = p
    return T


def quat_of(T):
    """Hamilton quaternion (x y z w, w >= 0) of a rotation matrix."""
    R = T[:3, :3]
    w = 0.5 * np.sqrt(max(0.0, 1 + R[0, 0] + R[1, 1] + R[2, 2]))
    if w > 1e-6:
        q = np.array([(R[2, 1] - R[1, 2]) / (4 * w), (R[0, 2] - R[2, 0]) / (4 * w), (R[1, 0] - R[0, 1]) / (4 * w), w])
    else:
        i = int(np.argmax(np.diag(R)))
        j, k = (i + 1) % 3, (i + 2) % 3
        s = np.sqrt(max(0.0, 1 + R[i, i] - R[j, j] - R[k, k]))
        q = np.zeros(4)
        q[i] = 0.5 * s
        q[j] = (R[j, i] + R[i, j]) / (2 * s)
        q[k] = (R[k, i] + R[i, k]) / (2 * s)
        q[3] = (R[k, j] - R[j, k]) / (2 * s)
    q /= np.linalg.norm(q)
    return q if q[3] >= 0 else -q


def _hprod(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz])


def disparity_angle(a, b):
    """Rotation angle between two Hamilton quaternions (either sign), as
    kindr's getDisparityAngle."""
    d = _hprod(np.asarray(a) / np.linalg.norm(a), np.array([-b[0], -b[1], -b[2], b[3]]) / np.linalg.norm(b))
    return 2.0 * np.arctan2(np.linalg.norm(d[:3]), abs(d[3]))


def _pose_graph_desc(kf, flags, meas, ext, edge_type):
    """One pose edge on keyframe 0 (to keyframe 1 unless absolute), identity
    covariance, no landmarks or IMU, one (unused) camera."""
    own = U.OwnedDesc(obs_uv=np.zeros((0, 2)), obs_sigma=np.zeros(0), obs_landmark=np.zeros(0),
                      obs_keyframe=np.zeros(0), obs_camera=np.zeros(0), lm_p_B=np.zeros((0, 3)),
                      lm_store_keyframe=np.zeros(0), kf_q_IM_p_MI=kf, kf_flags=flags, cameras=[U.camera()])
    a = own.a
    a["pe_from"] = np.array([0], dtype=np.int32)
    a["pe_to"] = np.array([0 if edge_type == N.MBA_POSE_EDGE_ABSOLUTE else 1], dtype=np.int32)
    a["pe_type"] = np.array([edge_type], dtype=np.int32)
    a["pe_meas"] = np.ascontiguousarray(meas, dtype=np.float64)
    a["pe_cov"] = np.ascontiguousarray(np.eye(6).ravel())
    a["pe_ext"] = np.ascontiguousarray(ext, dtype=np.float64)
    d = own.desc
    d.num_pose_edges = 1
    d.pose_edge_from = N.ptr(a["pe_from"], ctypes.c_int32)
    d.pose_edge_to = N.ptr(a["pe_to"], ctypes.c_int32)
    d.pose_edge_type = N.ptr(a["pe_type"], ctypes.c_int32)
    d.pose_edge_T_Bk_Bkp1 = N.ptr(a["pe_meas"])
    d.pose_edge_covariance = N.ptr(a["pe_cov"])
    d.pose_edge_q_I_B_p_B_I = N.ptr(a["pe_ext"])
    return own


def extrinsics_problem(case):
    """The case's problem (arrays owned by the returned object, .desc)."""
    f = SCEN["fixture"]
    T = {"T_G_Ik": matrix(f["q_G_Ik"], f["p_G_Ik"]), "T_G_Ikp1": matrix(f["q_G_Ikp1"], f["p_G_Ikp1"]),
         "T_B_I": matrix(f["q_B_I"], f["p_B_I"])}
    M = np.eye(4)
    for name, sign in case["measurement"]:
        M = M @ (T[name] if sign > 0 else np.linalg.inv(T[name]))
    kf = np.array([list(f["q_G_Ik"]) + list(f["p_G_Ik"]), list(f["q_G_Ikp1"]) + list(f["p_G_Ikp1"])])
    flags = [N.MBA_KF_POSE_CONSTANT if "T_G_Ik" in case["fixed"] else 0,
             N.MBA_KF_POSE_CONSTANT if "T_G_Ikp1" in case["fixed"] else 0]
    qBI = np.asarray(f["q_B_I"])
    ext = np.concatenate([[-qBI[0], -qBI[1], -qBI[2], qBI[3]], f["p_B_I"]])  # q_B_I's inverse | p_B_I
    return _pose_graph_desc(kf, flags, np.concatenate([quat_of(M), M[:3, 3]]), ext, N.MBA_POSE_EDGE_RELATIVE)


def extrinsics_check(case, own, summary, kf_state):
    """The case's assertions (list of failures)."""
    final = {"T_G_Ik": matrix(kf_state[0, :4], kf_state[0, 4:]), "T_G_Ikp1": matrix(kf_state[1, :4], kf_state[1, 4:])}
    fails = []
    for e in case["expect"]:
        if e["what"] in ("initial_cost", "final_cost"):
            if not abs(summary[e["what"]] - e["value"]) <= e["tol"]:
                fails.append((e, summary[e["what"]]))
        elif e["what"] == "same_transform":
            if not np.abs(final[e["a"]] - final[e["b"]]).max() <= e["tol"]:
                fails.append(e)
        else:
            fails.append(("unknown assertion", e))
    if "T_G_Ik" in case["fixed"] and not np.array_equal(kf_state[0], np.asarray(own.a["kf_q_IM_p_MI"][0])):
        fails.append("the constant keyframe moved")
    return fails


def extrinsics_options(lib_default, device):
    """The test's solve(): parameter, gradient and function tolerance 1e-14
    (DENSE_SCHUR; the device runs PCG to a tight tolerance)."""
    o = lib_default()
    o.max_num_iterations = 100
    o.function_tolerance = 1e-14
    o.parameter_tolerance = 1e-14
    o.gradient_tolerance = 1e-14
    o.reject_outliers_every_n_iters = 0
    if device:
        o.linear_solver = N.MBA_LINEAR_SOLVER_PCG
        o.linear_tolerance = 1e-14
        o.max_linear_iterations = 1000
    else:
        o.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    return o


def parameterization_problem():
    kf = [list(PARAM["x_q"]) + list(PARAM["x_p"])]
    meas = np.concatenate([PARAM["reference_q"], PARAM["reference_p"]])  # T_G_S
    ext = [0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0]  # T_S_B = identity
    return _pose_graph_desc(kf, [0], meas, ext, N.MBA_POSE_EDGE_ABSOLUTE)


def parameterization_options(lib_default, device):
    """Ceres' default ceres::Solver::Options (the test sets none)."""
    o = lib_default()
    o.max_num_iterations = 50
    o.function_tolerance = 1e-6
    o.gradient_tolerance = 1e-10
    o.parameter_tolerance = 1e-8
    o.initial_trust_region_radius = 1e4
    o.reject_outliers_every_n_iters = 0
    if device:
        o.linear_solver = N.MBA_LINEAR_SOLVER_PCG
        o.linear_tolerance = 1e-14
        o.max_linear_iterations = 1000
    else:
        o.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    return o


def parameterization_check(summary, kf_state):
    x = kf_state[0]
    fails = []
    if not summary["initial_cost"] > 1.0:
        fails.append(("initial cost", summary["initial_cost"]))
    ang = disparity_angle(x[:4], PARAM["reference_q"])
    if not ang <= PARAM["tol_rotation"]:
        fails.append(("rotation", ang))
    dp = np.abs(x[4:] - np.asarray(PARAM["reference_p"])).max()
    if not dp <= PARAM["tol_position"]:
        fails.append(("position", dp))
    return fails
