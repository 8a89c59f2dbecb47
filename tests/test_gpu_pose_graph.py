"""Pose-graph terms on the device against the oracle: loop closures with
switch variables (LoopClosureEdgeErrorTerm + SwitchPriorErrorTerm, within a
mission and across missions), absolute 6-DoF terms (BlockPosePriorErrorTermV2)
and odometry, and the pose-graph relaxation (VIMapRelaxation::solveRelaxation).

Bars: per-edge residuals and tangent Jacobians within 1e-9 of the oracle, cost
within 1e-12, the reduced camera system (switches eliminated) within 1e-9, LM
per-iteration costs within 1e-6 of the oracle's dense Schur solve and the
final switch values within 1e-5.
"""
import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu

ONE_MISSION = dict(keyframes_per_mission=130, num_landmarks=1000, pose_edges=1, loop_closure_stride=4,
                   loop_closure_outlier_fraction=0.35, absolute_pose_stride=20, seed=11)
TWO_MISSIONS = dict(num_missions=2, keyframes_per_mission=120, num_landmarks=1500, pose_edges=1,
                    loop_closure_stride=6, loop_closure_outlier_fraction=0.2, absolute_pose_stride=30, seed=12)


def _map(kw, spread_switches=True):
    m = synth.generate("c1", **kw)
    if spread_switches:  # switches away from 1 so that the switch factor is exercised
        ty = m.array("pose_edge_type")
        sw = m.array("pose_edge_switch")
        rng = np.random.default_rng(0)
        lc = ty == N.MBA_POSE_EDGE_LOOP_CLOSURE
        sw[lc] = rng.uniform(0.2, 1.0, size=lc.sum())
    return m


@pytest.fixture(scope="module", params=["one_mission", "two_missions"])
def graph_map(request):
    return _map(ONE_MISSION if request.param == "one_mission" else TWO_MISSIONS)


def _close(a, b, tol):
    scale = max(1.0, float(np.abs(b).max()))
    err = float(np.abs(a - b).max())
    assert err <= tol * scale, (err, scale)


def test_pose_graph_linearization_matches_oracle(graph_map):
    m = graph_map
    ty = m.array("pose_edge_type")
    assert (ty == N.MBA_POSE_EDGE_LOOP_CLOSURE).any() and (ty == N.MBA_POSE_EDGE_ABSOLUTE).any()
    o = O.OracleProblem(m.desc)
    ro, Jfo, Jto = o.linearize_pose_edges()
    with ba.BundleAdjuster(m.desc) as g:
        r, Jf, Jt = g.linearize_pose_edges()
        np.testing.assert_array_equal(g.read_switch_variables(), o.read_switches())
    _close(r, ro, 1e-9)
    _close(Jf, Jfo, 1e-9)
    _close(Jt, Jto, 1e-9)
    assert np.abs(Jt[ty == N.MBA_POSE_EDGE_ABSOLUTE]).max() == 0.0


def test_pose_graph_cost_matches_oracle(graph_map):
    m = graph_map
    o = O.OracleProblem(m.desc)
    with ba.BundleAdjuster(m.desc) as g:
        c = g.cost()
    co = o.cost()
    assert abs(c - co) <= 1e-12 * co, (c, co)


def test_reduced_system_with_switches_matches_oracle(graph_map):
    from test_gpu_schur import _dense
    m = graph_map
    o = O.OracleProblem(m.desc)
    radius = 1e4
    Ao, bo = o.reduced_system(N.default_solver_options(), radius)
    with ba.BundleAdjuster(m.desc) as g:
        s = g.reduced_system(N.MBA_PRECISION_FP64, radius)
    A = _dense(s, m.desc.num_keyframes)
    rel = np.linalg.norm(A - Ao) / np.linalg.norm(Ao)
    assert rel <= 1e-9, rel
    relb = np.linalg.norm(s["rhs"].ravel() - bo) / np.linalg.norm(bo)
    assert relb <= 1e-9, relb


def _oracle_opts(iters):
    o = N.default_solver_options()
    o.max_num_iterations = iters
    o.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    o.check_tolerances = 0
    return o


def _gpu_opts(iters, **kw):
    return ba.default_options(max_num_iterations=iters, check_tolerances=0, linear_tolerance=1e-10,
                              max_linear_iterations=6000, **kw)


def _compare_runs(sg, so):
    assert abs(sg["initial_cost"] - so["initial_cost"]) <= 1e-12 * so["initial_cost"]
    for a, b in zip(sg["iterations"], so["iterations"]):
        assert abs(a["cost"] - b["cost"]) <= 1e-6 * b["cost"], (a, b)
        assert a["ok"] == b["ok"]
    assert abs(sg["final_cost"] - so["final_cost"]) <= 1e-6 * so["final_cost"]


def test_lm_with_switches_matches_oracle_dense():
    m = _map(ONE_MISSION, spread_switches=False)
    o = O.OracleProblem(m.desc)
    so = o.solve(_oracle_opts(8))
    with ba.BundleAdjuster(m.desc) as g:
        sg = g.solve(_gpu_opts(8))
        swg = g.read_switch_variables()
    _compare_runs(sg, so)
    np.testing.assert_allclose(swg, o.read_switches(), atol=1e-5)
    ty = m.array("pose_edge_type")
    lc = swg[ty == N.MBA_POSE_EDGE_LOOP_CLOSURE]
    assert lc.min() < 0.1 and lc.max() > 0.9  # outliers switched off, inliers kept


def test_relaxation_matches_oracle_dense():
    m = _map(ONE_MISSION, spread_switches=False)
    rp = ba.RelaxationProblem(m.desc)
    o = O.OracleProblem(rp.desc)
    so = o.solve(_oracle_opts(8))
    sg, st, sw = ba.relax(m.desc, _gpu_opts(8))
    _compare_runs(sg, so)
    np.testing.assert_allclose(sw, o.read_switches(), atol=1e-5)
    # landmarks, velocities and biases stay where they were
    np.testing.assert_array_equal(st["lm_p_B"], m.array("lm_p_B"))
    np.testing.assert_array_equal(st["kf_v_M"], m.array("kf_v_M"))


def test_mixed_chain_solve_with_pose_graph_reaches_fp64_cost():
    m = _map(ONE_MISSION, spread_switches=False)
    with ba.BundleAdjuster(m.desc) as g:
        s64 = g.solve(ba.default_options(max_num_iterations=15, check_tolerances=0))
    with ba.BundleAdjuster(m.desc) as g:
        smx = g.solve(ba.default_options(max_num_iterations=15, check_tolerances=0,
                                         precision=N.MBA_PRECISION_MIXED, preconditioner=N.MBA_PRECOND_CHAIN))
    assert smx["final_cost"] <= s64["final_cost"] * (1 + 1e-6), (smx["final_cost"], s64["final_cost"])


def test_switch_write_read_round_trip_and_cost():
    m = _map(ONE_MISSION, spread_switches=False)
    ty = m.array("pose_edge_type")
    with ba.BundleAdjuster(m.desc) as g:
        sw = g.read_switch_variables()
        assert np.all(sw == 1.0)
        sw[ty == N.MBA_POSE_EDGE_LOOP_CLOSURE] = 0.5
        g.write_switch_variables(sw)
        np.testing.assert_array_equal(g.read_switch_variables(), sw)
        c = g.cost()
        bad = sw.copy()
        bad[np.flatnonzero(ty == N.MBA_POSE_EDGE_LOOP_CLOSURE)[0]] = 1.5
        with pytest.raises(ba.BAError):
            g.write_switch_variables(bad)
    m.array("pose_edge_switch")[ty == N.MBA_POSE_EDGE_LOOP_CLOSURE] = 0.5
    co = O.OracleProblem(m.desc).cost()
    assert abs(c - co) <= 1e-12 * co, (c, co)


@pytest.mark.parametrize("graph_mode", [0, 1, 2])
def test_pure_pose_graph_matches_oracle_dense(graph_mode):
    """No landmarks, no observations: odometry, loop closures with switches
    and absolute terms only (the kernels of the visual part launch nothing).
    Every step's gain ratio rests on the pose edges' model cost change alone,
    in each loop mode (direct launches, graph per iteration, device loop)."""
    from test_oracle_pose_graph import pose_graph_only
    m = synth.generate("c1", include_inertial=0, keyframes_per_mission=150, pose_edges=1, loop_closure_stride=5,
                       loop_closure_outlier_fraction=0.2, absolute_pose_stride=30, seed=13)
    d = pose_graph_only(m)
    o = O.OracleProblem(d)
    so = o.solve(_oracle_opts(8))
    with ba.BundleAdjuster(d) as g:
        sg = g.solve(_gpu_opts(8, use_cuda_graph=graph_mode))
        swg = g.read_switch_variables()
    _compare_runs(sg, so)
    np.testing.assert_allclose(swg, o.read_switches(), atol=1e-5)
    with ba.BundleAdjuster(d) as g:
        smx = g.solve(ba.default_options(max_num_iterations=15, check_tolerances=0, precision=N.MBA_PRECISION_MIXED,
                                         preconditioner=N.MBA_PRECOND_CHAIN, use_cuda_graph=2))
    assert smx["final_cost"] <= sg["final_cost"] * (1 + 1e-3)
