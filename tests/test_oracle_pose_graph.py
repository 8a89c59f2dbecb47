"""Pose-graph terms in the CPU oracle: LoopClosureEdgeErrorTerm with switch
variables and SwitchPriorErrorTerm, BlockPosePriorErrorTermV2 (absolute 6-DoF).

Checks: zero residual for noise-free measurements of the true state (the
generator's measurement models are written independently of the oracle's
residuals), ambient Jacobians against central differences (including the
three non-trace branches of the rotation-to-quaternion conversion), switch
variables turning gross loop-closure outliers off in an LM solve, and the
library's host validation of the new descriptor fields."""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import synth

IDENT = np.array([0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0])


def _inv_rot(T):
    """Eigen's inverse of the measured rotation (conjugate / squared norm), as
    the library stores loop-closure and absolute measurements."""
    q = T[:4]
    n2 = q @ q
    return np.concatenate([-q[:3] / n2, [q[3] / n2], T[4:]])


def _lc(bA, bB, xA, xB, meas, cov):
    lib = O.load()
    r = np.zeros(6); JA = np.zeros(42); JB = np.zeros(42)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (bA, bB, xA, xB, meas, cov)]
    assert lib.oracle_loop_closure(*[N.ptr(a) for a in args], N.ptr(r), N.ptr(JA), N.ptr(JB)) == 0
    return r, JA.reshape(6, 7), JB.reshape(6, 7)


def _abs(bf, x, ext, meas, cov):
    lib = O.load()
    r = np.zeros(6); J = np.zeros(42)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (bf, x, ext, meas, cov)]
    assert lib.oracle_absolute_pose(*[N.ptr(a) for a in args], N.ptr(r), N.ptr(J)) == 0
    return r, J.reshape(6, 7)


@pytest.fixture(scope="module")
def noise_free():
    return synth.generate("c1", keyframes_per_mission=150, num_missions=2, loop_closure_stride=10,
                          absolute_pose_stride=25, loop_closure_sigma_p=0.0, loop_closure_sigma_q=0.0,
                          absolute_pose_sigma_p=0.0, absolute_pose_sigma_q=0.0)


def test_noise_free_measurements_have_zero_residual(noise_free):
    m = noise_free
    gt = m.ground_truth()["kf_q_IM_p_MI"]
    ty, f, t = m.array("pose_edge_type"), m.array("pose_edge_from"), m.array("pose_edge_to")
    T, ext = m.array("pose_edge_T_Bk_Bkp1"), m.array("pose_edge_q_I_B_p_B_I")
    mis, kfm = m.array("mission_q_GM_p_GM"), m.array("kf_mission")
    cov = np.diag([1e-2, 1e-2, 1e-2, 1e-3, 1e-3, 1e-3]).ravel()
    n_lc = n_abs = n_cross = 0
    for j in range(m.desc.num_pose_edges):
        if ty[j] == N.MBA_POSE_EDGE_LOOP_CLOSURE:
            same = kfm[f[j]] == kfm[t[j]]
            n_cross += not same
            bA = IDENT if same else mis[kfm[f[j]]]
            bB = IDENT if same else mis[kfm[t[j]]]
            r, _, _ = _lc(bA, bB, gt[f[j]], gt[t[j]], _inv_rot(T[j]), cov)
            n_lc += 1
        elif ty[j] == N.MBA_POSE_EDGE_ABSOLUTE:
            r, _ = _abs(mis[kfm[f[j]]], gt[f[j]], ext[j], _inv_rot(T[j]), cov)
            n_abs += 1
        else:
            continue
        assert np.abs(r).max() < 1e-9, (j, r)
    assert n_lc > 0 and n_abs > 0 and n_cross > 0


def _fd_check(fn, x0, J, h=1e-6):
    for c in range(7):
        a, b = x0.copy(), x0.copy()
        a[c] += h
        b[c] -= h
        fd = (fn(a) - fn(b)) / (2 * h)
        np.testing.assert_allclose(J[:, c], fd, rtol=1e-6, atol=1e-6 * max(1.0, np.abs(fd).max()))


def test_loop_closure_jacobians_match_central_differences():
    rng = np.random.default_rng(3)
    A = rng.normal(size=(6, 6))
    cov = (A @ A.T + 6 * np.eye(6)).ravel() * 1e-3

    def rq(scale):
        v = rng.normal(size=3) * scale
        th = np.linalg.norm(v)
        return np.concatenate([np.sin(th / 2) * v / th, [np.cos(th / 2)]])
    bA = np.concatenate([rq(0.3), rng.normal(size=3)])
    bB = np.concatenate([rq(0.3), rng.normal(size=3)])
    xA = np.concatenate([rq(1.0), rng.normal(size=3) * 5])
    xB = np.concatenate([rq(1.0), rng.normal(size=3) * 5])
    meas = np.concatenate([rq(0.5), rng.normal(size=3)])
    for ba, bb in ((bA, bB), (IDENT, IDENT)):
        r, JA, JB = _lc(ba, bb, xA, xB, meas, cov)
        _fd_check(lambda x: _lc(ba, bb, x, xB, meas, cov)[0], xA, JA)
        _fd_check(lambda x: _lc(ba, bb, xA, x, meas, cov)[0], xB, JB)


@pytest.mark.parametrize("axis", [0, 1, 2, None])
def test_absolute_pose_jacobians_match_central_differences(axis):
    """axis: a 2.6 rad vertex rotation about x / y / z puts R_G_S's trace
    below zero (the largest-diagonal branches); None: trace branch."""
    rng = np.random.default_rng(5)
    A = rng.normal(size=(6, 6))
    cov = (A @ A.T + 6 * np.eye(6)).ravel() * 1e-3
    q = np.array([0.0, 0.0, 0.0, 1.0])
    if axis is not None:
        q[axis] = np.sin(1.3)
        q[3] = np.cos(1.3)
    else:
        q[:3] = [0.1, -0.2, 0.05]
        q /= np.linalg.norm(q)
    x = np.concatenate([q, [1.0, -2.0, 0.5]])
    bf = np.array([0.0, 0.0, np.sin(0.05), np.cos(0.05), 1.0, 2.0, 0.0])
    ext = np.array([np.sin(0.02), 0.0, 0.0, np.cos(0.02), 0.2, 0.0, -0.1])
    meas = np.concatenate([[0.1, 0.2, -0.1, 0.97], [0.5, 0.5, 0.5]])
    meas[:4] /= np.linalg.norm(meas[:4])
    r, J = _abs(bf, x, ext, meas, cov)
    _fd_check(lambda xx: _abs(bf, xx, ext, meas, cov)[0], x, J)


def test_switch_variables_turn_off_outlier_loop_closures():
    """SwitchPriorErrorTerm + bounds [0, 1]: the LM drives the switches of
    gross outliers (residual at the true state > 20 sigma) towards 0 and
    keeps the inliers' near 1; the trajectory ends closer to the truth than
    with the switches held at 1."""
    kw = dict(keyframes_per_mission=130, num_landmarks=1000, pose_edges=1, loop_closure_stride=4,
              loop_closure_outlier_fraction=0.35, seed=11)
    opts = N.default_solver_options()
    opts.max_num_iterations = 8
    opts.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    opts.check_tolerances = 0
    err = {}
    for var in (0.0, 1e-2):
        m = synth.generate("c1", loop_closure_switch_variance=var, **kw)
        o = O.OracleProblem(m.desc)
        gt = m.ground_truth()
        st0 = o.read_state()
        o.write_state(gt)
        r, _, _ = o.linearize_pose_edges()
        o.write_state(st0)
        ty = m.array("pose_edge_type")
        outlier = np.linalg.norm(r, axis=1)[ty == N.MBA_POSE_EDGE_LOOP_CLOSURE] > 20
        assert outlier.any() and (~outlier).any()
        s = o.solve(opts)
        assert s["final_cost"] < 1e-3 * s["initial_cost"]
        sw = o.read_switches()[ty == N.MBA_POSE_EDGE_LOOP_CLOSURE]
        if var > 0:
            assert sw[outlier].max() < 0.1, sw
            assert sw[~outlier].min() > 0.8, sw
        else:
            assert np.all(sw == 1.0)
        p = o.read_state()["kf_q_IM_p_MI"][:, 4:]
        err[var] = np.linalg.norm(p - gt["kf_q_IM_p_MI"][:, 4:], axis=1).mean()
    assert err[1e-2] < 0.5 * err[0.0], err


@pytest.mark.parametrize("what, status", [("type", N.MBA_ERR_INVALID_ARG), ("switch", N.MBA_ERR_INVALID_ARG),
                                          ("variance", N.MBA_ERR_INVALID_ARG),
                                          ("switch_nan", N.MBA_ERR_NON_FINITE),
                                          ("abs_ext", N.MBA_ERR_INVALID_ARG)])
def test_library_validates_pose_graph_fields(what, status):
    from maplab_gb300 import ba
    m = synth.generate("c1", loop_closure_stride=10, keyframes_per_mission=130, absolute_pose_stride=20)
    ty = m.array("pose_edge_type")
    lc = int(np.flatnonzero(ty == N.MBA_POSE_EDGE_LOOP_CLOSURE)[0])
    ab = int(np.flatnonzero(ty == N.MBA_POSE_EDGE_ABSOLUTE)[0])
    if what == "type":
        ty[lc] = 7
    elif what == "switch":
        m.array("pose_edge_switch")[lc] = 1.5
    elif what == "variance":
        m.array("pose_edge_switch_variance")[lc] = -1.0
    elif what == "switch_nan":
        m.array("pose_edge_switch")[lc] = np.nan
    else:
        m.array("pose_edge_q_I_B_p_B_I")[ab, 3] = 3.0  # sensor extrinsics not a unit quaternion
    h = ctypes.c_void_p()
    assert ba.lib().mba_create(ctypes.byref(m.desc), 0, ctypes.byref(h)) == status
    assert not h.value


def pose_graph_only(m):
    """m's descriptor without landmarks and observations (a pure pose graph:
    odometry, loop closures, absolute terms); the arrays stay owned by m."""
    d = N.ProblemDesc()
    ctypes.memmove(ctypes.byref(d), ctypes.byref(m.desc), ctypes.sizeof(d))
    d.num_landmarks = 0
    d.num_observations = 0
    for f in ("obs_uv", "obs_sigma", "obs_landmark", "obs_keyframe", "obs_camera", "lm_p_B", "lm_store_keyframe",
              "lm_constant"):
        setattr(d, f, None)
    return d


def test_oracle_solves_a_pure_pose_graph():
    m = synth.generate("c1", include_inertial=0, keyframes_per_mission=150, pose_edges=1, loop_closure_stride=5,
                       loop_closure_outlier_fraction=0.2, absolute_pose_stride=30, seed=13)
    d = pose_graph_only(m)
    o = O.OracleProblem(d)
    opts = N.default_solver_options()
    opts.max_num_iterations = 10
    opts.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    opts.check_tolerances = 0
    s = o.solve(opts)
    assert s["final_cost"] < 1e-2 * s["initial_cost"]
