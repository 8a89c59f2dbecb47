"""Relative 6-DoF pose edges (SixDoFBlockPoseErrorTermWithExtrinsics) on the
device against the oracle.

Bars: per-edge whitened residual and tangent Jacobians within 1e-9 (relative
to the largest entry) of the oracle; total cost within 1e-12 relative; the
damped reduced camera system with the pose-edge blocks within 1e-9; LM with
the same iterations as the oracle's dense Schur solve within 1e-6 relative.
Maps: the visual-inertial map with odometry edges between consecutive
keyframes, and a visual-only map where the odometry edges replace the IMU.
"""
import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["vi", "visual_only"])
def pose_map(request):
    return synth.generate("c1", pose_edges=1, include_inertial=0 if request.param == "visual_only" else 1)


def _close(a, b, tol):
    scale = max(1.0, float(np.abs(b).max()))
    err = float(np.abs(a - b).max())
    assert err <= tol * scale, (err, scale)


def test_pose_edge_linearization_matches_oracle(pose_map):
    m = pose_map
    assert m.desc.num_pose_edges > 0
    o = O.OracleProblem(m.desc)
    ro, Jfo, Jto = o.linearize_pose_edges()
    with ba.BundleAdjuster(m.desc) as g:
        r, Jf, Jt = g.linearize_pose_edges()
    _close(r, ro, 1e-9)
    _close(Jf, Jfo, 1e-9)
    _close(Jt, Jto, 1e-9)
    # the edge from the gauge keyframe uses the roll/pitch (or fixed) pose block
    assert np.abs(ro).max() > 0


def test_cost_with_pose_edges_matches_oracle(pose_map):
    m = pose_map
    o = O.OracleProblem(m.desc)
    with ba.BundleAdjuster(m.desc) as g:
        c = g.cost()
    co = o.cost()
    assert abs(c - co) <= 1e-12 * co, (c, co)


def test_reduced_system_with_pose_edges_matches_oracle(pose_map):
    from test_gpu_schur import _dense
    m = pose_map
    o = O.OracleProblem(m.desc)
    radius = 1e4
    Ao, bo = o.reduced_system(N.default_solver_options(), radius)
    with ba.BundleAdjuster(m.desc) as g:
        s = g.reduced_system(N.MBA_PRECISION_FP64, radius)
    assert len(s["inertial"]) == m.desc.num_imu_edges + m.desc.num_pose_edges
    A = _dense(s, m.desc.num_keyframes)
    rel = np.linalg.norm(A - Ao) / np.linalg.norm(Ao)
    assert rel <= 1e-9, rel
    relb = np.linalg.norm(s["rhs"].ravel() - bo) / np.linalg.norm(bo)
    assert relb <= 1e-9, relb


def test_lm_with_pose_edges_matches_oracle_dense(pose_map):
    m = pose_map
    o = O.OracleProblem(m.desc)
    oo = N.default_solver_options()
    oo.max_num_iterations = 8
    oo.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    oo.check_tolerances = 0
    so = o.solve(oo)
    with ba.BundleAdjuster(m.desc) as g:
        sg = g.solve(ba.default_options(max_num_iterations=8, check_tolerances=0, linear_tolerance=1e-10,
                                        max_linear_iterations=6000))
    assert abs(sg["initial_cost"] - so["initial_cost"]) <= 1e-12 * so["initial_cost"]
    for a, b in zip(sg["iterations"], so["iterations"]):
        assert abs(a["cost"] - b["cost"]) <= 1e-6 * b["cost"], (a, b)
        assert a["ok"] == b["ok"]
    assert abs(sg["final_cost"] - so["final_cost"]) <= 1e-6 * so["final_cost"]
    assert sg["final_cost"] < 0.01 * sg["initial_cost"]


def test_mixed_chain_solve_with_pose_edges_reaches_fp64_cost():
    """The added forms (mixed precision, chain preconditioner) keep working
    with pose edges in the inertial-block slots."""
    m = synth.generate("c1", pose_edges=1)
    with ba.BundleAdjuster(m.desc) as g:
        s64 = g.solve(ba.default_options(max_num_iterations=15, check_tolerances=0))
    with ba.BundleAdjuster(m.desc) as g:
        smx = g.solve(ba.default_options(max_num_iterations=15, check_tolerances=0,
                                         precision=N.MBA_PRECISION_MIXED, preconditioner=N.MBA_PRECOND_CHAIN))
    assert smx["final_cost"] <= s64["final_cost"] * (1 + 1e-6), (smx["final_cost"], s64["final_cost"])
