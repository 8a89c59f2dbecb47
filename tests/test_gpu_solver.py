"""Device Levenberg-Marquardt against the oracle's restated LM.

Bar (FP64 path): final cost within 1e-6 relative of the oracle after the same
iteration count, per-iteration costs likewise.  The oracle solves the reduced
camera system by dense Cholesky; the device by block-Jacobi PCG run to a tight
tolerance (1e-10) so both compute the same LM steps.
"""
import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth
from problem_util import OwnedDesc, camera, unit_quat

pytestmark = pytest.mark.gpu


def _oracle_opts(iters):
    o = N.default_solver_options()
    o.max_num_iterations = iters
    o.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    o.check_tolerances = 0
    return o


def _gpu_opts(iters, **kw):
    kw.setdefault("linear_tolerance", 1e-10)
    kw.setdefault("max_linear_iterations", 500)
    return ba.default_options(max_num_iterations=iters, check_tolerances=0, **kw)


@pytest.fixture(scope="module")
def c1_oracle_run():
    m = synth.generate("c1")
    o = O.OracleProblem(m.desc)
    s = o.solve(_oracle_opts(10))
    return m, s, o.read_state()


def test_c1_fp64_matches_oracle_dense(c1_oracle_run):
    """Same LM iterations as the oracle's exact (dense Cholesky) Schur solve:
    the device PCG is run to convergence (tolerance 1e-10, up to 6000 its)."""
    m, so, st_o = c1_oracle_run
    with ba.BundleAdjuster(m.desc) as g:
        sg = g.solve(_gpu_opts(10, max_linear_iterations=6000))
        st_g = g.read_state()
    assert abs(sg["initial_cost"] - so["initial_cost"]) <= 1e-12 * so["initial_cost"]
    assert abs(sg["final_cost"] - so["final_cost"]) <= 1e-6 * so["final_cost"], (sg["final_cost"], so["final_cost"])
    for a, b in zip(sg["iterations"], so["iterations"]):
        assert abs(a["cost"] - b["cost"]) <= 1e-6 * b["cost"], (a, b)
        assert a["ok"] == b["ok"]
    # Equal cost to 1e-6; the states agree to what the cost constrains
    # (flat directions move by ~1e-5 m between equally good solutions).
    np.testing.assert_allclose(st_g["kf_q_IM_p_MI"], st_o["kf_q_IM_p_MI"], atol=2e-4)
    np.testing.assert_allclose(st_g["lm_p_B"], st_o["lm_p_B"], atol=5e-3)


def test_fp64_pcg_matches_oracle_pcg():
    """Same block-Jacobi PCG settings on both sides (capped at 60 iterations,
    so the iteration cap, not the tolerance, ends most solves)."""
    m = synth.generate("c1", keyframes_per_mission=40, num_landmarks=800)
    o = O.OracleProblem(m.desc)
    oo = _oracle_opts(8)
    oo.linear_solver = N.MBA_LINEAR_SOLVER_PCG
    oo.linear_tolerance = 1e-10
    oo.max_linear_iterations = 60
    so = o.solve(oo)
    with ba.BundleAdjuster(m.desc) as g:
        sg = g.solve(_gpu_opts(8, max_linear_iterations=60))
    for a, b in zip(sg["iterations"], so["iterations"]):
        assert abs(a["cost"] - b["cost"]) <= 1e-6 * b["cost"], (a, b)
        assert a["lin_iters"] == b["lin_iters"]


def test_c1_eager_and_graph_agree():
    m = synth.generate("c1", keyframes_per_mission=40, num_landmarks=800)
    with ba.BundleAdjuster(m.desc) as g:
        s1 = g.solve(_gpu_opts(5, use_cuda_graph=1))
    with ba.BundleAdjuster(m.desc) as g:
        s2 = g.solve(_gpu_opts(5, use_cuda_graph=0))
    # Floating-point atomics in the assembly accumulate in a run-dependent
    # order, so the two runs agree to rounding amplified by the capped PCG.
    assert abs(s1["final_cost"] - s2["final_cost"]) <= 1e-5 * s2["final_cost"]
    assert s1["num_iterations"] == s2["num_iterations"]


def test_c1_mixed_precision_reaches_fp64_cost():
    """The mixed path (FP32 Jacobians / Schur / PCG, FP64 retraction, cost and
    gain ratio) reaches the plain FP64 path's final cost within 1e-6 relative."""
    m = synth.generate("c1")
    opts = dict(linear_tolerance=1e-6, max_linear_iterations=100)
    with ba.BundleAdjuster(m.desc) as g:
        s64 = g.solve(_gpu_opts(10, **opts))
    target = s64["final_cost"] * (1 + 1e-6)
    with ba.BundleAdjuster(m.desc) as g:
        s32 = g.solve(_gpu_opts(30, precision=N.MBA_PRECISION_MIXED, stop_cost=target, **opts))
    assert s32["final_cost"] <= target, (s32["final_cost"], s64["final_cost"])
    assert s32["termination"] == 6  # stopped on reaching the cost tolerance


def test_visual_only_problem_matches_oracle():
    m = synth.generate("c1", keyframes_per_mission=30, num_landmarks=600, include_inertial=0)
    o = O.OracleProblem(m.desc)
    so = o.solve(_oracle_opts(6))
    with ba.BundleAdjuster(m.desc) as g:
        sg = g.solve(_gpu_opts(6, max_linear_iterations=6000))
    assert abs(sg["final_cost"] - so["final_cost"]) <= 1e-6 * so["final_cost"], (sg["final_cost"], so["final_cost"])


def test_multi_mission_global_terms_match_oracle():
    m = synth.generate("c4", num_missions=3, keyframes_per_mission=40, num_landmarks=1500,
                       shared_landmark_fraction=0.3)
    o = O.OracleProblem(m.desc)
    so = o.solve(_oracle_opts(5))
    with ba.BundleAdjuster(m.desc) as g:
        sg = g.solve(_gpu_opts(5, max_linear_iterations=6000))
    assert abs(sg["final_cost"] - so["final_cost"]) <= 1e-6 * so["final_cost"], (sg["final_cost"], so["final_cost"])


def test_landmark_recovery_two_observers():
    """test_visual_term_test.cc style ground-truth recovery on the device."""
    cam = camera(q_CI=unit_quat(0.5, -0.5, 0.5, -0.5))
    kx = np.array([[0, 0, 0, 1, 0, 0, 0], np.concatenate([unit_quat(0, 0, 0.05, 1), [0.0, 0.5, 0.0]])])
    uv = [[353.02323456, 255.31784363], [437.32659405, 255.37958988]]  # projections of (6, 0.3, -0.2)
    od = OwnedDesc(obs_uv=uv, obs_sigma=[0.7, 0.7], obs_landmark=[0, 0], obs_keyframe=[0, 1], obs_camera=[0, 0],
                   lm_p_B=[[6.3, 0.1, 0.05]], lm_store_keyframe=[0], kf_q_IM_p_MI=kx,
                   kf_flags=[N.MBA_KF_POSE_CONSTANT] * 2, cameras=[cam])
    with ba.BundleAdjuster(od.desc) as g:
        s = g.solve(_gpu_opts(30, function_tolerance=0.0, parameter_tolerance=0.0))
        st = g.read_state()
    assert s["final_cost"] < 1e-12
    np.testing.assert_allclose(st["lm_p_B"][0], [6.0, 0.3, -0.2], atol=1e-6)


def test_zero_iterations_returns_cost():
    m = synth.generate("c1", keyframes_per_mission=20, num_landmarks=200)
    o = O.OracleProblem(m.desc)
    with ba.BundleAdjuster(m.desc) as g:
        s = g.solve(_gpu_opts(0))
    assert abs(s["final_cost"] - o.cost()) <= 1e-12 * o.cost()


def test_chain_preconditioner_matches_oracle_dense(c1_oracle_run):
    """The chain-corrected preconditioner changes only how fast PCG converges:
    run to 1e-10 it gives the oracle's exact-Schur LM trajectory, in far fewer
    linear iterations than block-Jacobi."""
    m, so, _ = c1_oracle_run
    with ba.BundleAdjuster(m.desc) as g:
        sc = g.solve(_gpu_opts(10, max_linear_iterations=6000, preconditioner=N.MBA_PRECOND_CHAIN))
    with ba.BundleAdjuster(m.desc) as g:
        sb = g.solve(_gpu_opts(10, max_linear_iterations=6000))
    assert abs(sc["final_cost"] - so["final_cost"]) <= 1e-6 * so["final_cost"], (sc["final_cost"], so["final_cost"])
    for a, b in zip(sc["iterations"], so["iterations"]):
        assert abs(a["cost"] - b["cost"]) <= 1e-6 * b["cost"], (a, b)
    assert sc["linear_iterations"] < 0.5 * sb["linear_iterations"], (sc["linear_iterations"], sb["linear_iterations"])


@pytest.mark.parametrize("product", [1, 2])
def test_pcg_product_variants_match_oracle_dense(c1_oracle_run, product):
    """Both PCG products (each stored pose block read once with the transposed
    part added by atomics, or read from both of its rows) give the oracle's
    exact-Schur LM trajectory when PCG is run to 1e-10."""
    m, so, _ = c1_oracle_run
    with ba.BundleAdjuster(m.desc) as g:
        g.set_tuning(pcg_product=product)
        sg = g.solve(_gpu_opts(10, max_linear_iterations=6000, preconditioner=N.MBA_PRECOND_CHAIN))
    assert abs(sg["final_cost"] - so["final_cost"]) <= 1e-6 * so["final_cost"], (sg["final_cost"], so["final_cost"])
    for a, b in zip(sg["iterations"], so["iterations"]):
        assert abs(a["cost"] - b["cost"]) <= 1e-6 * b["cost"], (a, b)


def test_pcg_product_variants_agree_mixed():
    """Mixed precision on a 3-mission map with shared landmarks: the two
    products give the same capped-PCG solve to rounding."""
    m = synth.generate("c4", num_missions=3, keyframes_per_mission=100, num_landmarks=5000,
                       shared_landmark_fraction=0.2)
    out = []
    for product in (1, 2):
        with ba.BundleAdjuster(m.desc) as g:
            g.set_tuning(pcg_product=product)
            out.append(g.solve(_gpu_opts(6, max_linear_iterations=25, linear_tolerance=1e-6,
                                         precision=N.MBA_PRECISION_MIXED, preconditioner=N.MBA_PRECOND_CHAIN)))
    assert abs(out[0]["final_cost"] - out[1]["final_cost"]) <= 1e-5 * out[1]["final_cost"], (out[0], out[1])


def test_chain_preconditioner_mixed_reaches_fp64_cost():
    m = synth.generate("c1")
    with ba.BundleAdjuster(m.desc) as g:
        s64 = g.solve(_gpu_opts(10, max_linear_iterations=100, linear_tolerance=1e-6))
    target = s64["final_cost"] * (1 + 1e-6)
    with ba.BundleAdjuster(m.desc) as g:
        s = g.solve(_gpu_opts(30, max_linear_iterations=100, linear_tolerance=1e-6, stop_cost=target,
                              precision=N.MBA_PRECISION_MIXED, preconditioner=N.MBA_PRECOND_CHAIN))
    assert s["termination"] == 6, s
    assert s["final_cost"] <= target


def test_outlier_rejection_matches_oracle():
    """maplab's outlier-rejection solve (every 3 iterations, depth <= 0):
    ten landmarks flipped behind their store camera are rejected at the first
    restart on both sides, the rejected sets agree, and the LM trajectories
    (exact Schur vs PCG to 1e-10) match to 1e-6."""
    m = synth.generate("c1")
    lp = m.array("lm_p_B")
    flipped = np.arange(0, 2000, 200)
    lp[flipped] *= -3.0
    oo = _oracle_opts(7)
    oo.reject_outliers_every_n_iters = 3
    so = O.OracleProblem(m.desc).solve(oo)
    with ba.BundleAdjuster(m.desc) as g:
        sg = g.solve(_gpu_opts(7, max_linear_iterations=6000, reject_outliers_every_n_iters=3))
        flags, count = g.rejected_landmarks()
    assert so["rejected_landmarks"] == sg["rejected_landmarks"] == count == len(flipped)
    assert set(np.nonzero(flags)[0]) == set(flipped)
    for a, b in zip(sg["iterations"], so["iterations"]):
        assert abs(a["cost"] - b["cost"]) <= 1e-6 * b["cost"], (a, b)


def test_outlier_rejection_off_keeps_all_landmarks():
    m = synth.generate("c1")
    m.array("lm_p_B")[:5] *= -3.0
    with ba.BundleAdjuster(m.desc) as g:
        s = g.solve(_gpu_opts(4, reject_outliers_every_n_iters=0))
        _, count = g.rejected_landmarks()
    assert s["rejected_landmarks"] == 0 and count == 0
