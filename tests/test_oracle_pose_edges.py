"""Relative 6-DoF pose edges (odometry / wheel odometry) in the CPU oracle:
SixDoFBlockPoseErrorTermWithExtrinsics restated with forward-mode dual
numbers (as Ceres' AutoDiffCostFunction).  Checks: zero residual for a
noise-free measurement of the true state, ambient Jacobians against central
differences, the square-root information against numpy, and an LM solve of a
map with odometry edges lowering the cost."""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import synth


def _lib():
    return O.load()


def _edge(xk, xk1, ext, meas, cov):
    lib = _lib()
    r = np.zeros(6); Jk = np.zeros(42); Jk1 = np.zeros(42)
    st = lib.oracle_pose_edge(N.ptr(np.ascontiguousarray(xk)), N.ptr(np.ascontiguousarray(xk1)), N.ptr(ext),
                              N.ptr(meas), N.ptr(cov), N.ptr(r), N.ptr(Jk), N.ptr(Jk1))
    assert st == 0
    return r, Jk.reshape(6, 7), Jk1.reshape(6, 7)


def _map():
    m = synth.generate("c1", pose_edges=1, pose_edge_sigma_p=0.0, pose_edge_sigma_q=0.0)
    return m


def test_noise_free_measurement_has_zero_residual():
    m = _map()
    gt = m.ground_truth()["kf_q_IM_p_MI"]
    f, t = m.array("pose_edge_from"), m.array("pose_edge_to")
    meas, ext = m.array("pose_edge_T_Bk_Bkp1"), m.array("pose_edge_q_I_B_p_B_I")
    cov = np.diag([1e-4, 1e-4, 1e-4, 1e-5, 1e-5, 1e-5]).ravel()
    assert len(f) == m.desc.num_keyframes - 1
    for j in (0, 17, len(f) - 1):
        r, _, _ = _edge(gt[f[j]], gt[t[j]], ext[j].copy(), meas[j].copy(), cov)
        assert np.abs(r).max() < 1e-9, r


def test_ambient_jacobians_match_central_differences():
    m = _map()
    x = m.array("kf_q_IM_p_MI")
    rng = np.random.default_rng(0)
    ext = m.array("pose_edge_q_I_B_p_B_I")[3].copy()
    meas = m.array("pose_edge_T_Bk_Bkp1")[3].copy()
    A = rng.normal(size=(6, 6))
    cov = (A @ A.T + 6 * np.eye(6)).ravel() * 1e-3
    xk, xk1 = x[3].copy(), x[4].copy()
    r, Jk, Jk1 = _edge(xk, xk1, ext, meas, cov)
    h = 1e-6
    for which, J in ((0, Jk), (1, Jk1)):
        for c in range(7):
            a, b = xk.copy(), xk1.copy()
            (a if which == 0 else b)[c] += h
            rp = _edge(a, b, ext, meas, cov)[0]
            a, b = xk.copy(), xk1.copy()
            (a if which == 0 else b)[c] -= h
            rm = _edge(a, b, ext, meas, cov)[0]
            fd = (rp - rm) / (2 * h)
            np.testing.assert_allclose(J[:, c], fd, rtol=1e-6, atol=1e-6 * max(1.0, np.abs(fd).max()))


def test_sqrt_information_is_inverse_cholesky_applied_as_row_vector():
    m = _map()
    x = m.array("kf_q_IM_p_MI")
    ext = m.array("pose_edge_q_I_B_p_B_I")[0].copy()
    meas = m.array("pose_edge_T_Bk_Bkp1")[0].copy()
    rng = np.random.default_rng(1)
    A = rng.normal(size=(6, 6))
    C = A @ A.T + 6 * np.eye(6)
    r_c, _, _ = _edge(x[0].copy(), x[1].copy(), ext, meas, C.ravel())
    r_i, _, _ = _edge(x[0].copy(), x[1].copy(), ext, meas, np.eye(6).ravel())
    Minv = np.linalg.inv(np.linalg.cholesky(C))
    np.testing.assert_allclose(r_c, r_i @ Minv, rtol=1e-12, atol=1e-12)  # e_w = e^T L^-1


def test_oracle_solve_with_odometry_edges_lowers_cost():
    m = synth.generate("c1", pose_edges=1)
    o = O.OracleProblem(m.desc)
    opts = N.default_solver_options()
    opts.max_num_iterations = 5
    opts.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    opts.check_tolerances = 0
    s = o.solve(opts)
    assert s["final_cost"] < 0.01 * s["initial_cost"]


@pytest.mark.parametrize("what, status", [("covariance", N.MBA_ERR_NOT_SPD), ("index", N.MBA_ERR_OUT_OF_RANGE_INDEX),
                                          ("self", N.MBA_ERR_OUT_OF_RANGE_INDEX), ("quaternion", N.MBA_ERR_INVALID_ARG),
                                          ("nan", N.MBA_ERR_NON_FINITE)])
def test_library_validates_pose_edges_before_any_device_work(what, status):
    """mba_create checks the pose edges on the host (no GPU needed): a
    covariance that is not positive definite, keyframe indices out of range or
    equal, a measured rotation that is not a unit quaternion, non-finite
    values."""
    from maplab_gb300 import ba
    m = synth.generate("c1", pose_edges=1)
    j = 5
    if what == "covariance":
        cov = m.array("pose_edge_covariance")
        cov[j] = 0.0
        cov[j, 0] = -1.0
    elif what == "index":
        m.array("pose_edge_to")[j] = m.desc.num_keyframes
    elif what == "self":
        m.array("pose_edge_to")[j] = m.array("pose_edge_from")[j]
    elif what == "quaternion":
        m.array("pose_edge_T_Bk_Bkp1")[j, 3] = 2.0
    else:
        m.array("pose_edge_q_I_B_p_B_I")[j, 5] = np.nan
    h = ctypes.c_void_p()
    st = ba.lib().mba_create(ctypes.byref(m.desc), 0, ctypes.byref(h))
    assert st == status
    assert not h.value
