"""The reference's own unit test of the relative pose term with extrinsics
(SixDoFBlockPoseErrorTermWithExtrinsics, the optimization builder's odometry
term), run through the CPU oracle: its enabled cases from
tests/golden/pose_extrinsics_scenarios.json (extracted from
algorithms/ceres-error-terms/test/test_six_dof_block_transformation_error_term_with_extrinsics.cc
by tests/golden/make_golden.py).

Each case is the reference's two-keyframe problem: keyframe blocks
q_G_I | p_G_I (Hamilton coefficients, as the term reads them), the extrinsics
block q_I_B | p_B_I, one measured T_Bk_Bkp1 with identity covariance, the
listed blocks held constant; the oracle's LM solve must meet the case's
assertions at the case's tolerances."""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle_lib as O
import problem_util as U
from maplab_gb300 import _native as N

HERE = os.path.dirname(os.path.abspath(__file__))
SCEN = json.load(open(os.path.join(HERE, "golden", "pose_extrinsics_scenarios.json")))


def _hrot(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _matrix(q, p):
    """4x4 transformation of a Hamilton quaternion (x y z w) and a position."""
    T = np.eye(4)
    T[:3, :3] = _hrot(np.asarray(q) / np.linalg.norm(q))
    T[:3, 3] = p
    return T


def _quat_of(T):
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


def _fixture_transforms():
    f = SCEN["fixture"]
    return {"T_G_Ik": _matrix(f["q_G_Ik"], f["p_G_Ik"]), "T_G_Ikp1": _matrix(f["q_G_Ikp1"], f["p_G_Ikp1"]),
            "T_B_I": _matrix(f["q_B_I"], f["p_B_I"])}


def _problem(case):
    """The case's problem as a descriptor (arrays owned by the returned object)."""
    f = SCEN["fixture"]
    T = _fixture_transforms()
    M = np.eye(4)
    for name, sign in case["measurement"]:
        M = M @ (T[name] if sign > 0 else np.linalg.inv(T[name]))
    qm = _quat_of(M)
    kf = np.array([list(f["q_G_Ik"]) + list(f["p_G_Ik"]), list(f["q_G_Ikp1"]) + list(f["p_G_Ikp1"])])
    flags = [N.MBA_KF_POSE_CONSTANT if "T_G_Ik" in case["fixed"] else 0,
             N.MBA_KF_POSE_CONSTANT if "T_G_Ikp1" in case["fixed"] else 0]
    own = U.OwnedDesc(obs_uv=np.zeros((0, 2)), obs_sigma=np.zeros(0), obs_landmark=np.zeros(0),
                      obs_keyframe=np.zeros(0), obs_camera=np.zeros(0), lm_p_B=np.zeros((0, 3)),
                      lm_store_keyframe=np.zeros(0), kf_q_IM_p_MI=kf, kf_flags=flags, cameras=[U.camera()])
    qBI = np.asarray(f["q_B_I"])
    a = own.a
    a["pe_from"] = np.array([0], dtype=np.int32)
    a["pe_to"] = np.array([1], dtype=np.int32)
    a["pe_meas"] = np.ascontiguousarray(np.concatenate([qm, M[:3, 3]]))
    a["pe_cov"] = np.ascontiguousarray(np.eye(6).ravel())
    # the extrinsics block: coefficients of q_B_I's inverse | p_B_I
    a["pe_ext"] = np.ascontiguousarray(np.concatenate([[-qBI[0], -qBI[1], -qBI[2], qBI[3]], f["p_B_I"]]))
    d = own.desc
    d.num_pose_edges = 1
    d.pose_edge_from = N.ptr(a["pe_from"], ctypes.c_int32)
    d.pose_edge_to = N.ptr(a["pe_to"], ctypes.c_int32)
    d.pose_edge_T_Bk_Bkp1 = N.ptr(a["pe_meas"])
    d.pose_edge_covariance = N.ptr(a["pe_cov"])
    d.pose_edge_q_I_B_p_B_I = N.ptr(a["pe_ext"])
    return own


CASES = [c for c in SCEN["tests"] if "skipped" not in c]


def test_fixture_holds_the_enabled_cases():
    assert SCEN["source"].endswith("test_six_dof_block_transformation_error_term_with_extrinsics.cc")
    assert [c["name"] for c in CASES] == ["TestPosePriorErrorTermZeroCost", "TestPosePriorErrorTermIdentityFixBIFixGIk"]
    assert all("T_B_I" in c["fixed"] for c in CASES)  # the extrinsics are constant in both


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_reference_pose_extrinsics_case(case):
    own = _problem(case)
    o = O.OracleProblem(own.desc)
    opts = N.default_solver_options()
    opts.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    opts.max_num_iterations = 100
    # the reference's solve(): parameter, gradient and function tolerance 1e-14
    opts.function_tolerance = 1e-14
    opts.parameter_tolerance = 1e-14
    opts.gradient_tolerance = 1e-14
    s = o.solve(opts)
    state = o.read_state()["kf_q_IM_p_MI"]
    final = {"T_G_Ik": _matrix(state[0, :4], state[0, 4:]), "T_G_Ikp1": _matrix(state[1, :4], state[1, 4:])}
    for e in case["expect"]:
        if e["what"] in ("initial_cost", "final_cost"):
            assert abs(s[e["what"]] - e["value"]) <= e["tol"], (e, s[e["what"]])
        elif e["what"] == "same_transform":
            assert np.abs(final[e["a"]] - final[e["b"]]).max() <= e["tol"], e
        else:
            raise AssertionError(f"unknown assertion {e}")
    # the constant keyframe did not move
    if "T_G_Ik" in case["fixed"]:
        assert np.array_equal(state[0], np.asarray(own.a["kf_q_IM_p_MI"][0]))


# JplPoseParameterization's own test (test_pose_parameterization_test.cc,
# tests/golden/pose_parameterization_scenario.json): a pose block pulled onto
# a reference transformation by the error (2 vec(q (x) q_ref^-1) | p - p_ref)
# under the pose parameterization, Ceres' default options.  That error is the
# absolute 6-DoF term (BlockPosePriorErrorTermV2) with an identity baseframe,
# identity sensor extrinsics and identity covariance (its rows in the other
# order and, where w < 0, with the opposite sign: the same cost and minimum),
# so the case runs as one keyframe with one absolute pose edge.
PARAM = json.load(open(os.path.join(HERE, "golden", "pose_parameterization_scenario.json")))


def _hprod(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz])


def _disparity_angle(a, b):
    """Rotation angle between two Hamilton quaternions (either sign)."""
    d = _hprod(np.asarray(a) / np.linalg.norm(a), np.array([-b[0], -b[1], -b[2], b[3]]) / np.linalg.norm(b))
    return 2.0 * np.arctan2(np.linalg.norm(d[:3]), abs(d[3]))


def test_reference_pose_parameterization_minimization():
    assert PARAM["source"].endswith("test_pose_parameterization_test.cc")
    own = U.OwnedDesc(obs_uv=np.zeros((0, 2)), obs_sigma=np.zeros(0), obs_landmark=np.zeros(0),
                      obs_keyframe=np.zeros(0), obs_camera=np.zeros(0), lm_p_B=np.zeros((0, 3)),
                      lm_store_keyframe=np.zeros(0), kf_q_IM_p_MI=[list(PARAM["x_q"]) + list(PARAM["x_p"])],
                      cameras=[U.camera()])
    a = own.a
    a["pe_from"] = np.array([0], dtype=np.int32)
    a["pe_to"] = np.array([0], dtype=np.int32)
    a["pe_type"] = np.array([N.MBA_POSE_EDGE_ABSOLUTE], dtype=np.int32)
    a["pe_meas"] = np.ascontiguousarray(np.concatenate([PARAM["reference_q"], PARAM["reference_p"]]))  # T_G_S
    a["pe_cov"] = np.ascontiguousarray(np.eye(6).ravel())
    a["pe_ext"] = np.ascontiguousarray([0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0])  # T_S_B = identity
    d = own.desc
    d.num_pose_edges = 1
    d.pose_edge_from = N.ptr(a["pe_from"], ctypes.c_int32)
    d.pose_edge_to = N.ptr(a["pe_to"], ctypes.c_int32)
    d.pose_edge_type = N.ptr(a["pe_type"], ctypes.c_int32)
    d.pose_edge_T_Bk_Bkp1 = N.ptr(a["pe_meas"])
    d.pose_edge_covariance = N.ptr(a["pe_cov"])
    d.pose_edge_q_I_B_p_B_I = N.ptr(a["pe_ext"])
    o = O.OracleProblem(d)
    opts = N.default_solver_options()
    opts.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    # Ceres' defaults (ceres::Solver::Options)
    opts.max_num_iterations = 50
    opts.function_tolerance = 1e-6
    opts.gradient_tolerance = 1e-10
    opts.parameter_tolerance = 1e-8
    opts.initial_trust_region_radius = 1e4
    s = o.solve(opts)
    x = o.read_state()["kf_q_IM_p_MI"][0]
    assert s["initial_cost"] > 1.0
    assert _disparity_angle(x[:4], PARAM["reference_q"]) <= PARAM["tol_rotation"]
    assert np.abs(x[4:] - np.asarray(PARAM["reference_p"])).max() <= PARAM["tol_position"]
