"""Per-term parity of the CUDA evaluation kernels against the CPU oracle.

Bar: FP64 path within 1e-9 relative per Jacobian block and per term
(|a - b| / max(|b|, tiny), block-wise), exact zeros where the reference writes
zeros (failed projections, dummy blocks); the FP32 (mixed) linearization within
the tolerance stated in test_mixed_precision_visual_linearization.
"""
import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu

REL = 1e-9


def _blockwise_rel(a, b):
    """Per-row relative error of two (n, k) arrays; rows where b is exactly
    zero must be exactly zero in a."""
    nb = np.linalg.norm(b, axis=1)
    na = np.linalg.norm(a - b, axis=1)
    zero = nb == 0
    assert np.all(np.linalg.norm(a[zero], axis=1) == 0), "non-zero output where the reference writes zeros"
    if (~zero).sum() == 0:
        return 0.0
    return float((na[~zero] / nb[~zero]).max())


@pytest.fixture(scope="module")
def c1():
    return synth.generate("c1")


@pytest.fixture(scope="module")
def multi():
    # Two cameras (radtan + equidistant), 4 co-registered missions with shared
    # landmarks: kLocalKeyframe, kLocalMission and kGlobal terms all occur.
    return synth.generate("c4", num_missions=4, keyframes_per_mission=80, num_landmarks=4000,
                          shared_landmark_fraction=0.3)


@pytest.mark.parametrize("which", ["c1", "multi"])
def test_visual_ambient_parity(which, request):
    m = request.getfixturevalue(which)
    o = O.OracleProblem(m.desc)
    with ba.BundleAdjuster(m.desc) as g:
        r_g, J_g = g.evaluate_visual()
    r_o, J_o = o.evaluate_visual()
    assert _blockwise_rel(r_g, r_o) < REL
    for b in range(9):
        assert _blockwise_rel(J_g[b], J_o[b]) < REL, f"block {b}"


def test_visual_failed_projection_zeroes():
    m = synth.generate("c1", keyframes_per_mission=30, num_landmarks=200)
    p = m.array("lm_p_B")
    p[:20] = [-5.0, 0.0, 0.0]  # behind the store keyframe's camera -> failed projections
    o = O.OracleProblem(m.desc)
    with ba.BundleAdjuster(m.desc) as g:
        r_g, J_g = g.evaluate_visual()
    r_o, J_o = o.evaluate_visual()
    failed = np.all(r_o == 0, axis=1)
    assert failed.sum() >= 20
    assert np.all(r_g[failed] == 0)
    for b in range(9):
        assert np.all(J_g[b][failed] == 0)


@pytest.mark.parametrize("which", ["c1", "multi"])
def test_inertial_ambient_parity(which, request):
    m = request.getfixturevalue(which)
    o = O.OracleProblem(m.desc)
    with ba.BundleAdjuster(m.desc) as g:
        r_g, J_g = g.evaluate_inertial()
    st, r_o, J_o = o.evaluate_inertial()
    assert st == 0
    assert _blockwise_rel(r_g, r_o) < REL
    for b in range(8):
        assert _blockwise_rel(J_g[b], J_o[b]) < REL, f"block {b}"


@pytest.mark.parametrize("which", ["c1", "multi"])
def test_tangent_linearization_parity_fp64(which, request):
    """Solver-path Jacobians (local parameterization applied, Huber corrector)."""
    m = request.getfixturevalue(which)
    o = O.OracleProblem(m.desc)
    with ba.BundleAdjuster(m.desc) as g:
        r_g, Jl_g, Js_g, Jo_g = g.linearize_visual(N.MBA_PRECISION_FP64)
        cost_g = g.cost()
    r_o, Jl_o, Js_o, Jo_o, cost_o = o.linearize_visual()
    assert _blockwise_rel(r_g, r_o) < REL
    assert _blockwise_rel(Jl_g, Jl_o) < REL
    assert _blockwise_rel(Js_g, Js_o) < REL
    assert _blockwise_rel(Jo_g, Jo_o) < REL
    assert abs(cost_g - cost_o) <= 1e-12 * cost_o


def test_mixed_precision_visual_linearization(c1):
    """FP32 Jacobians: stated error against the FP64 oracle (median and max
    block-relative error over all observations)."""
    o = O.OracleProblem(c1.desc)
    with ba.BundleAdjuster(c1.desc) as g:
        r_g, Jl_g, Js_g, Jo_g = g.linearize_visual(N.MBA_PRECISION_MIXED)
    r_o, Jl_o, Js_o, Jo_o, _ = o.linearize_visual()
    for a, b in ((Jl_g, Jl_o), (Js_g, Js_o), (Jo_g, Jo_o)):
        nb = np.linalg.norm(b, axis=1)
        rel = np.linalg.norm(a - b, axis=1)[nb > 0] / nb[nb > 0]
        assert np.median(rel) < 1e-5 and rel.max() < 1e-2, (np.median(rel), rel.max())
    # residuals: absolute pixel error (sigma = 1 px)
    assert np.abs(r_g - r_o).max() < 1e-3


@pytest.mark.parametrize("precision", [N.MBA_PRECISION_FP64, N.MBA_PRECISION_MIXED])
def test_linearize_visual_into_pinned_host_memory(multi, precision):
    """Page-locked destinations are written by the gather kernel directly;
    pageable ones through the device staging buffer and copies.  Both give the
    same rows, bit for bit, also with some outputs omitted."""
    import ctypes
    import torch
    n = multi.desc.num_observations
    with ba.BundleAdjuster(multi.desc) as g:
        ref = g.linearize_visual(precision)
        pinned = [torch.full((n, c), np.nan, dtype=torch.float64).pin_memory() for c in (2, 6, 12, 12)]
        P = lambda t: ctypes.cast(t.data_ptr(), N.c_double_p) if t is not None else None
        assert ba.lib().mba_linearize_visual(g.handle, precision, *[P(t) for t in pinned]) == 0
        for a, b in zip(pinned, ref):
            np.testing.assert_array_equal(a.numpy(), b)
        sub = [pinned[0], None, pinned[2], None]
        for t in sub:
            if t is not None:
                t.fill_(np.nan)
        assert ba.lib().mba_linearize_visual(g.handle, precision, *[P(t) for t in sub]) == 0
        np.testing.assert_array_equal(sub[0].numpy(), ref[0])
        np.testing.assert_array_equal(sub[2].numpy(), ref[2])


def test_linearize_visual_chunked_into_pinned_host_memory():
    """FP64 rows into page-locked memory for a map of 32,768 observations or
    more go in eight chunks evaluated from caller-ordered copies of the
    observations, each chunk copied out while the next is evaluated.  The
    rows equal the single-pass rows into pageable memory bit for bit, also
    with outputs omitted and after the state has changed."""
    import ctypes
    import torch
    m = synth.generate("c2", keyframes_per_mission=200, num_landmarks=20000)
    n = m.desc.num_observations
    assert n >= 8 * 4096
    P = lambda t: ctypes.cast(t.data_ptr(), N.c_double_p) if t is not None else None
    with ba.BundleAdjuster(m.desc) as g:
        for step in range(2):
            ref = g.linearize_visual(N.MBA_PRECISION_FP64)
            pinned = [torch.full((n, c), np.nan, dtype=torch.float64).pin_memory() for c in (2, 6, 12, 12)]
            assert ba.lib().mba_linearize_visual(g.handle, N.MBA_PRECISION_FP64, *[P(t) for t in pinned]) == 0
            for a, b in zip(pinned, ref):
                np.testing.assert_array_equal(a.numpy(), b)
            sub = [None, pinned[1], None, pinned[3]]
            for t in sub:
                if t is not None:
                    t.fill_(np.nan)
            assert ba.lib().mba_linearize_visual(g.handle, N.MBA_PRECISION_FP64, *[P(t) for t in sub]) == 0
            np.testing.assert_array_equal(sub[1].numpy(), ref[1])
            np.testing.assert_array_equal(sub[3].numpy(), ref[3])
            if step == 0:
                o = N.default_solver_options()
                o.max_num_iterations = 2
                g.solve(o)


@pytest.mark.parametrize("pipelined, min_blocks, block", [(2, 1, 256), (2, 3, 64), (1, 1, 128), (1, 2, 256), (1, 2, 64)])
def test_evaluation_kernel_variants_agree(multi, pipelined, min_blocks, block):
    """The pipelined persistent loop and the register-capped variants run the
    same arithmetic as the one-thread-per-observation kernel.  FP64 agrees to
    1e-12 per row; FP32 Jacobians to 1e-4 relative per row and residuals to
    1e-4 px (sigma = 1 px): contraction into fused multiply-adds may differ
    between the inlined copies, and r = (projection - z) / sigma cancels
    ~400 px coordinates."""
    with ba.BundleAdjuster(multi.desc) as g:
        ref64 = g.linearize_visual(N.MBA_PRECISION_FP64)
        ref32 = g.linearize_visual(N.MBA_PRECISION_MIXED)
        g.set_tuning(visual_pipelined=pipelined, visual_min_blocks=min_blocks, visual_block=block)
        out64 = g.linearize_visual(N.MBA_PRECISION_FP64)
        out32 = g.linearize_visual(N.MBA_PRECISION_MIXED)
    for a, b in zip(out64, ref64):
        assert _blockwise_rel(a, b) <= 1e-12
    assert np.abs(out32[0] - ref32[0]).max() <= 1e-4
    for a, b in zip(out32[1:], ref32[1:]):
        assert _blockwise_rel(a, b) <= 1e-4


def test_state_roundtrip(c1):
    with ba.BundleAdjuster(c1.desc) as g:
        st = g.read_state()
        np.testing.assert_array_equal(st["kf_q_IM_p_MI"], c1.array("kf_q_IM_p_MI"))
        np.testing.assert_array_equal(st["lm_p_B"], c1.array("lm_p_B"))
        gt = c1.ground_truth()
        g.write_state(gt)
        st2 = g.read_state()
        for k in gt:
            np.testing.assert_array_equal(st2[k], gt[k])
