"""Oracle self-checks restated from the reference's unit tests.

* test_quaternion_parameterization_test.cc:13-103 — analytic local
  parameterization Jacobians against Ridders numeric Jacobians of Plus, 1e-10.
* The visual / inertial ambient Jacobians, lifted to the tangent space by the
  local parameterization (what Ceres uses), against numeric derivatives of the
  restated residuals.
* test_visual_term_test.cc / test_mission_baseframe_visual_term_test.cc /
  test_inertial_term_test.cc style recovery: perturb one block of a
  ground-truth problem and let the restated LM recover it.
"""
import ctypes
import math

import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from problem_util import OwnedDesc, camera, ridders, unit_quat

dp = N.c_double_p


def _plus(q, d):
    out = np.zeros(4)
    O.load().oracle_quat_plus(N.ptr(O.arr(q)), N.ptr(O.arr(d)), N.ptr(out))
    return out


def _jq(q):
    J = np.zeros(12)
    O.load().oracle_quat_jacobian(N.ptr(O.arr(q)), N.ptr(J))
    return J.reshape(4, 3)


def test_jpl_quaternion_jacobian_numeric():
    # Eigen::Quaterniond q_AB(1, 1, 0, 1) -> xyzw (1, 0, 1, 1) normalized
    q = unit_quat(1, 0, 1, 1)
    J = _jq(q)
    Jn = np.stack([ridders(lambda t, k=k: _plus(q, np.eye(3)[k] * t), 0.0) for k in range(3)], axis=1)
    np.testing.assert_allclose(J, Jn, atol=1e-10)


def test_jpl_yaw_jacobian_numeric():
    lib = O.load()
    q = unit_quat(1, 0, 1, 1)
    J = np.zeros(4)
    lib.oracle_yaw_jacobian(N.ptr(O.arr(q)), N.ptr(J))

    def f(t):
        out = np.zeros(4)
        lib.oracle_yaw_plus(N.ptr(O.arr(q)), N.ptr(O.arr([t])), N.ptr(out))
        return out
    np.testing.assert_allclose(J, ridders(f, 0.0), atol=1e-10)


def _rpy_jpl(q):
    """getRollPitchYawFromQuaternionJpl: R = toRotationMatrixJPL(q), then
    RotationMatrixToRollPitchYaw (maplab-common geometry-inl.h:40-60)."""
    R = np.zeros(9)
    O.load().oracle_rotation_matrix(N.ptr(O.arr(q)), N.ptr(R))
    R = R.reshape(3, 3)
    pitch = math.atan2(-R[2, 0], math.sqrt(R[0, 0] ** 2 + R[1, 0] ** 2))
    c = math.cos(pitch)
    assert abs(c) > 1e-12
    return np.array([math.atan2(R[2, 1] / c, R[2, 2] / c), pitch, math.atan2(R[1, 0] / c, R[0, 0] / c)])


def test_jpl_yaw_plus_keeps_roll_pitch():
    """test_quaternion_parameterization_test.cc:33-58 (JplYawQuaternionParameterization.Plus):
    deltas -0.5, 0, 0.5, 1 applied in turn keep roll and pitch to 1e-6, and the
    yaw returns to its start exactly when the deltas sum to zero."""
    lib = O.load()
    q = unit_quat(1, 0, 1, 1)  # Eigen::Quaterniond(1, 1, 0, 1), xyzw
    rpy0 = _rpy_jpl(q)
    total = 0.0
    for delta in (-0.5, 0.0, 0.5, 1.0):
        out = np.zeros(4)
        lib.oracle_yaw_plus(N.ptr(O.arr(q)), N.ptr(O.arr([delta])), N.ptr(out))
        total += delta
        q = out
        rpy = _rpy_jpl(q)
        assert abs(rpy[0] - rpy0[0]) <= 1e-6 and abs(rpy[1] - rpy0[1]) <= 1e-6
        if total == 0.0:
            assert abs(rpy[2] - rpy0[2]) <= 1e-6
        else:
            assert rpy[2] != rpy0[2]


def test_jpl_roll_pitch_jacobian_numeric():
    lib = O.load()
    # Eigen::Quaterniond q_IM(1, 1, 5, 0), q_GM(1, 5, 0, 2) (w first).
    q_IM = unit_quat(1, 5, 0, 1)
    q_GM = unit_quat(5, 0, 2, 1)
    J = np.zeros(8)
    lib.oracle_rollpitch_jacobian(N.ptr(O.arr(q_GM)), N.ptr(O.arr(q_IM)), N.ptr(J))
    J = J.reshape(4, 2)

    def f(k):
        def g(t):
            out = np.zeros(4)
            d = np.zeros(2)
            d[k] = t
            lib.oracle_rollpitch_plus(N.ptr(O.arr(q_GM)), N.ptr(O.arr(q_IM)), N.ptr(d), N.ptr(out))
            return out
        return g
    Jn = np.stack([ridders(f(k), 0.0) for k in range(2)], axis=1)
    np.testing.assert_allclose(J, Jn, atol=1e-10)


def test_jpl_plus_properties():
    rng = np.random.default_rng(0)
    for _ in range(50):
        q = unit_quat(*rng.normal(size=4))
        for scale in (1e-3, 0.3, 1.5):  # both branches of the small-angle threshold
            d = rng.normal(size=3) * scale
            out = _plus(q, d)
            assert abs(np.linalg.norm(out) - 1) < 1e-14
            assert out[3] >= 0


def _visual_setup(error_type, dtype):
    rng = np.random.default_rng(7 + error_type + 10 * dtype)
    cam = camera(dtype=dtype, dist=(-0.28, 0.07, 0.001, -0.002) if dtype == N.MBA_DISTORTION_RADTAN
                 else (-0.01, 0.005, -0.001, 0.0001), q_CI=unit_quat(0.5, -0.5, 0.5, -0.5), p_CI=(0.05, -0.02, 0.1))
    # A point roughly 8 m in front of the observer camera (camera looks along I_x).
    p_B = np.array([8.0, 0.4, -0.3])
    store = np.concatenate([unit_quat(*rng.normal(size=3) * 0.05, 1.0), rng.normal(size=3) * 0.2])
    obs = np.concatenate([unit_quat(*rng.normal(size=3) * 0.05, 1.0), rng.normal(size=3) * 0.2])
    # Baseframe translations are zero here: the reference's baseframe rotation
    # Jacobians (visual-error-term-inl.h:207-209) use skew(p_G_fi), which is
    # the tangent derivative only when p_G_LM = p_G_M = 0; see
    # test_visual_term_baseframe_rotation_formula for the general case.
    mis_l = np.concatenate([unit_quat(0, 0, 0.05, 1), [0.0, 0.0, 0.0]])
    mis_o = np.concatenate([unit_quat(0, 0, -0.04, 1), [0.0, 0.0, 0.0]])
    if error_type == N.MBA_LOCAL_KEYFRAME:
        obs = store
    return cam, p_B, store, obs, mis_l, mis_o


def _visual_eval(cam, blocks, error_type, meas=(300.0, 200.0), sigma=0.7, want_jac=True):
    lib = O.load()
    P = (dp * 9)(*[N.ptr(b) for b in blocks])
    r = np.zeros(2)
    J = [np.zeros(s) for s in O.OracleProblem.VISUAL_BLOCK_SIZES]
    Jp = (dp * 9)(*[N.ptr(j) for j in J]) if want_jac else None
    failed = ctypes.c_int()
    lib.oracle_visual_term(P, N.ptr(O.arr(meas)), sigma, error_type, ctypes.byref(cam), N.ptr(r), Jp,
                           ctypes.byref(failed))
    return r, J, failed.value


@pytest.mark.parametrize("dtype", [N.MBA_DISTORTION_RADTAN, N.MBA_DISTORTION_EQUIDISTANT, N.MBA_DISTORTION_NONE])
@pytest.mark.parametrize("error_type", [N.MBA_LOCAL_KEYFRAME, N.MBA_LOCAL_MISSION, N.MBA_GLOBAL])
def test_visual_term_tangent_jacobians_numeric(error_type, dtype):
    cam, p_B, store, obs, mis_l, mis_o = _visual_setup(error_type, dtype)
    q_CI = np.array(cam.q_CI_p_CI[:4]); p_CI = np.array(cam.q_CI_p_CI[4:])
    intr = np.array(cam.intrinsics[:]); dist = np.array(cam.distortion[:])
    base = [p_B, store, mis_l, mis_o, obs, q_CI, p_CI, intr, dist]
    base = [O.arr(b) for b in base]
    r0, J, failed = _visual_eval(cam, base, error_type)
    assert failed == 0

    def residual_with(block, kind, k):
        def f(t):
            bl = [b.copy() for b in base]
            if kind == "q":
                bl[block][:4] = _plus(base[block][:4], np.eye(3)[k] * t)
            elif kind == "p":
                bl[block][4 + k] += t
            else:
                bl[block][k] += t
            if error_type == N.MBA_LOCAL_KEYFRAME and block in (1, 4):
                bl[1] = bl[4] = bl[block]
            return _visual_eval(cam, bl, error_type, want_jac=False)[0]
        return f

    checks = [(0, "v", 3)]
    if error_type != N.MBA_LOCAL_KEYFRAME:
        checks += [(1, "pose", None), (4, "pose", None)]
    if error_type == N.MBA_GLOBAL:
        checks += [(2, "pose", None), (3, "pose", None)]
    checks += [(6, "v", 3), (7, "v", 4)]
    if dtype != N.MBA_DISTORTION_NONE:
        checks += [(8, "v", 4)]
    for block, kind, n in checks:
        if kind == "pose":
            Jamb = J[block].reshape(2, 7)
            Jt = np.concatenate([Jamb[:, :4] @ _jq(base[block][:4]), Jamb[:, 4:]], axis=1)
            Jn = np.stack([ridders(residual_with(block, "q", k), 0.0) for k in range(3)] +
                          [ridders(residual_with(block, "p", k), 0.0) for k in range(3)], axis=1)
        else:
            Jt = J[block].reshape(2, n)
            Jn = np.stack([ridders(residual_with(block, "v", k), 0.0) for k in range(n)], axis=1)
        scale = max(1.0, np.abs(Jn).max())
        np.testing.assert_allclose(Jt, Jn, atol=1e-6 * scale, err_msg=f"block {block}")
    # q_C_I block (2x4 ambient) through its quaternion parameterization
    Jt = J[5].reshape(2, 4) @ _jq(q_CI)

    def fq(k):
        def f(t):
            bl = [b.copy() for b in base]
            bl[5] = _plus(base[5], np.eye(3)[k] * t)
            return _visual_eval(cam, bl, error_type, want_jac=False)[0]
        return f
    Jn = np.stack([ridders(fq(k), 0.0) for k in range(3)], axis=1)
    np.testing.assert_allclose(Jt, Jn, atol=1e-6 * max(1.0, np.abs(Jn).max()))


def test_visual_term_baseframe_rotation_formula():
    """With non-zero baseframe translations the restatement keeps the
    reference's formula J_q_G_LM = J_p_G_LM skew(p_G_fi) (visual-error-term-inl.h:208)."""
    cam, p_B, store, obs, _, _ = _visual_setup(N.MBA_GLOBAL, N.MBA_DISTORTION_RADTAN)
    mis_l = np.concatenate([unit_quat(0, 0, 0.05, 1), [0.3, -0.2, 0.1]])
    mis_o = np.concatenate([unit_quat(0, 0, -0.04, 1), [-0.1, 0.25, 0.0]])
    base = [O.arr(b) for b in [p_B, store, mis_l, mis_o, obs, cam.q_CI_p_CI[:4], cam.q_CI_p_CI[4:],
                               cam.intrinsics[:], cam.distortion[:]]]
    r, J, failed = _visual_eval(cam, base, N.MBA_GLOBAL)
    assert failed == 0
    lib = O.load()

    def R(q):
        m = np.zeros(9)
        lib.oracle_rotation_matrix(N.ptr(O.arr(q)), N.ptr(m))
        return m.reshape(3, 3)
    p_LM = R(store[:4]).T @ p_B + store[4:]
    p_G = R(mis_l[:4]) @ p_LM + mis_l[4:]
    S = np.array([[0, -p_G[2], p_G[1]], [p_G[2], 0, -p_G[0]], [-p_G[1], p_G[0], 0]])
    Jp = J[2].reshape(2, 7)[:, 4:]  # J_kp * J_p_G_LM / sigma
    Jq_amb = J[2].reshape(2, 7)[:, :4]
    np.testing.assert_allclose(Jq_amb @ _jq(mis_l[:4]), Jp @ S * (mis_l[:4] @ mis_l[:4]), atol=1e-9)


def test_visual_term_failure_zeroes_everything():
    cam, p_B, store, obs, mis_l, mis_o = _visual_setup(N.MBA_LOCAL_KEYFRAME, N.MBA_DISTORTION_RADTAN)
    p_behind = np.array([-5.0, 0.0, 0.0])  # behind the camera (optical axis = I_x)
    base = [O.arr(b) for b in [p_behind, store, mis_l, mis_o, store, cam.q_CI_p_CI[:4], cam.q_CI_p_CI[4:],
                               cam.intrinsics[:], cam.distortion[:]]]
    r, J, failed = _visual_eval(cam, base, N.MBA_LOCAL_KEYFRAME)
    assert failed == 1
    assert np.all(r == 0) and all(np.all(j == 0) for j in J)


def _inertial_problem_blocks(seed=0, ns=21):
    rng = np.random.default_rng(seed)
    dt_ns = 5_000_000
    ts = np.arange(ns, dtype=np.int64) * dt_ns
    imu = np.zeros((ns, 6))
    imu[:, 0:3] = rng.normal(size=(ns, 3)) * 0.3 + [0, 0, 9.81]
    imu[:, 3:6] = rng.normal(size=(ns, 3)) * 0.2
    qf = unit_quat(*rng.normal(size=3) * 0.1, 1.0)
    pf = rng.normal(size=3)
    bg, v, ba = rng.normal(size=3) * 0.01, rng.normal(size=3), rng.normal(size=3) * 0.05
    # The 'to' state is the integrated end state plus a small offset: the
    # reference's Jacobians (inertial-error-term.cc:188-230) are first order
    # in the residual, so they are checked near a consistent pair of states.
    lib = O.load()
    s = O.arr(np.concatenate([qf, bg, v, ba, pf]))
    noise = O.arr([0.0, 0.0, 0.0, 0.0, 9.81])
    for i in range(ns - 1):
        rd = O.arr(np.concatenate([imu[i, :3] - ba, imu[i, 3:] - bg, imu[i + 1, :3] - ba, imu[i + 1, 3:] - bg]))
        nxt = np.zeros(16)
        lib.oracle_imu_integrate(N.ptr(noise), N.ptr(s), N.ptr(rd), ctypes.c_double(dt_ns * 1e-9), N.ptr(nxt),
                                 None, None)
        s = nxt
    q_end = _plus(s[:4] / np.linalg.norm(s[:4]), rng.normal(size=3) * 1e-3)
    blocks = [np.concatenate([qf, pf]), bg, v, ba,
              np.concatenate([q_end, s[13:16] + rng.normal(size=3) * 1e-3]),
              s[4:7] + rng.normal(size=3) * 1e-4, s[7:10] + rng.normal(size=3) * 1e-3,
              s[10:13] + rng.normal(size=3) * 1e-4]
    return [O.arr(b) for b in blocks], ts, O.arr(imu)


def _inertial_eval(blocks, ts, imu, noise=(0.01, 0.001, 0.02, 0.002, 9.81), want_jac=True):
    lib = O.load()
    P = (dp * 8)(*[N.ptr(b) for b in blocks])
    r = np.zeros(15)
    J = [np.zeros(s) for s in O.OracleProblem.INERTIAL_BLOCK_SIZES]
    Jp = (dp * 8)(*[N.ptr(j) for j in J]) if want_jac else None
    st = lib.oracle_inertial_term(N.ptr(O.arr(noise)), P, len(ts), ts.ctypes.data_as(N.c_int64_p), N.ptr(imu),
                                  N.ptr(r), Jp)
    return st, r, J


def test_inertial_term_tangent_jacobians_numeric():
    blocks, ts, imu = _inertial_problem_blocks()
    st, r0, J = _inertial_eval(blocks, ts, imu)
    assert st == 0

    def f(block, kind, k):
        def g(t):
            bl = [b.copy() for b in blocks]
            if kind == "q":
                bl[block][:4] = _plus(blocks[block][:4], np.eye(3)[k] * t)
            elif kind == "p":
                bl[block][4 + k] += t
            else:
                bl[block][k] += t
            return _inertial_eval(bl, ts, imu, want_jac=False)[1]
        return g

    for side in (0, 4):
        Jamb = J[side].reshape(15, 7)
        Jt = np.concatenate([Jamb[:, :4] @ _jq(blocks[side][:4]), Jamb[:, 4:]], axis=1)
        Jn = np.stack([ridders(f(side, "q", k), 0.0) for k in range(3)] +
                      [ridders(f(side, "p", k), 0.0) for k in range(3)], axis=1)
        # J_begin uses the RK4-propagated transition (first order in the
        # error state), so agreement is to the integrator's linearization.
        np.testing.assert_allclose(Jt, Jn, atol=1e-3 * np.abs(Jn).max())
        for b in range(1, 4):
            Jt = J[side + b].reshape(15, 3)
            Jn = np.stack([ridders(f(side + b, "v", k), 0.0) for k in range(3)], axis=1)
            np.testing.assert_allclose(Jt, Jn, atol=1e-3 * max(1.0, np.abs(Jn).max()))


def test_inertial_unordered_timestamps_rejected():
    blocks, ts, imu = _inertial_problem_blocks()
    ts = ts.copy()
    ts[5], ts[6] = ts[6], ts[5]
    st, _, _ = _inertial_eval(blocks, ts, imu)
    assert st == N.MBA_ERR_UNORDERED_IMU


def _project(cam, p_C):
    kp = np.zeros(2)
    O.load().oracle_project(ctypes.byref(cam), N.ptr(O.arr(p_C)), N.ptr(kp), None, None, None)
    return kp


def test_visual_recovery_landmark_two_cameras():
    """test_visual_term_test.cc style: two observing keyframes, perturbed
    landmark, both poses fixed; LM recovers the landmark and the cost -> 0."""
    cam = camera(q_CI=unit_quat(0.5, -0.5, 0.5, -0.5))
    kx = np.array([[0, 0, 0, 1, 0, 0, 0], np.concatenate([unit_quat(0, 0, 0.05, 1), [0.0, 0.5, 0.0]])])
    p_true_M = np.array([6.0, 0.3, -0.2])
    uv, lmk, kfs = [], [], []
    for k in range(2):
        R = np.zeros(9)
        O.load().oracle_rotation_matrix(N.ptr(O.arr(kx[k][:4])), N.ptr(R))
        p_I = R.reshape(3, 3) @ (p_true_M - kx[k][4:])
        Rc = np.zeros(9)
        O.load().oracle_rotation_matrix(N.ptr(O.arr(cam.q_CI_p_CI[:4])), N.ptr(Rc))
        uv.append(_project(cam, Rc.reshape(3, 3) @ p_I))
        lmk.append(0)
        kfs.append(k)
    p_B_true = p_true_M  # store keyframe 0 is the identity pose
    od = OwnedDesc(obs_uv=uv, obs_sigma=[0.7, 0.7], obs_landmark=lmk, obs_keyframe=kfs, obs_camera=[0, 0],
                   lm_p_B=[p_B_true + [0.3, -0.2, 0.25]], lm_store_keyframe=[0], kf_q_IM_p_MI=kx,
                   kf_flags=[N.MBA_KF_POSE_CONSTANT] * 2, cameras=[cam])
    o = O.OracleProblem(od.desc)
    opts = N.default_solver_options()
    opts.max_num_iterations = 50
    opts.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    opts.function_tolerance = 1e-50
    opts.parameter_tolerance = 1e-50
    s = o.solve(opts)
    st = o.read_state()
    assert s["final_cost"] < 1e-15
    np.testing.assert_allclose(st["lm_p_B"][0], p_B_true, atol=1e-6)
