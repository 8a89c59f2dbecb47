"""Device-driven LM loop (the whole solve as one CUDA graph with a while
condition evaluated on the device) and per-problem autotuning."""
import threading
import time

import numpy as np
import pytest

from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu


def _opts(**kw):
    kw.setdefault("max_num_iterations", 10)
    kw.setdefault("check_tolerances", 0)
    return ba.default_options(**kw)


@pytest.mark.parametrize("precision", [N.MBA_PRECISION_FP64, N.MBA_PRECISION_MIXED])
def test_device_loop_matches_host_loop(precision):
    """Direct launches, one graph per iteration and the device-driven loop
    run the same iterations: costs, and the gain ratios (model cost change of
    the visual and the inertial terms) of every step, on a fresh handle each.
    FP64 within 1e-6; the mixed path assembles with FP32 atomics (summation
    order differs from run to run) and stops PCG at its iteration cap, so its
    runs agree within 1e-3."""
    m = synth.generate("c1")
    runs = []
    for mode in (0, 1, 2):
        with ba.BundleAdjuster(m.desc) as g:
            runs.append(g.solve(_opts(use_cuda_graph=mode, precision=precision)))
    plain, host, dev = runs
    tol = 1e-6 if precision == N.MBA_PRECISION_FP64 else 1e-3
    for other in (host, dev):
        assert other["num_iterations"] == plain["num_iterations"]
        assert other["rejected_landmarks"] == plain["rejected_landmarks"]
        for a, b in zip(other["iterations"], plain["iterations"]):
            assert a["ok"] == b["ok"]
            assert abs(a["cost"] - b["cost"]) <= tol * b["cost"], (a, b)
            if precision == N.MBA_PRECISION_FP64:
                assert abs(a["relative_decrease"] - b["relative_decrease"]) <= 1e-6, (a, b)
    times = [it["time_ms"] for it in dev["iterations"][1:]]
    assert all(t > 0 for t in times) and times == sorted(times)


def test_device_loop_stop_cost_and_mixed():
    m = synth.generate("c1")
    with ba.BundleAdjuster(m.desc) as g:
        s64 = g.solve(_opts(max_num_iterations=10))
    target = s64["final_cost"] * (1 + 1e-6)
    with ba.BundleAdjuster(m.desc) as g:
        s = g.solve(_opts(max_num_iterations=30, use_cuda_graph=2, stop_cost=target, precision=N.MBA_PRECISION_MIXED,
                          preconditioner=N.MBA_PRECOND_CHAIN, max_linear_iterations=25))
    assert s["termination"] == 6 and s["final_cost"] <= target
    assert 0 < s["time_to_stop_cost_ms"] <= s["iterations"][-1]["time_ms"] + 1e-9


def test_device_loop_cancel():
    m = synth.generate("c2", keyframes_per_mission=1000, num_landmarks=100000)
    with ba.BundleAdjuster(m.desc) as g:
        out = {}

        def run():
            out["s"] = None
            try:
                out["s"] = g.solve(_opts(max_num_iterations=200, use_cuda_graph=2, max_linear_iterations=100,
                                         reject_outliers_every_n_iters=0))
            except ba.BAError as e:
                out["err"] = e

        t = threading.Thread(target=run)
        t.start()
        time.sleep(0.3)
        g.cancel()
        t.join(timeout=120)
        assert not t.is_alive()
    assert "err" in out and out["err"].status == 7  # MBA_ERR_CANCELLED


def test_autotune_keeps_results():
    m = synth.generate("c1")
    with ba.BundleAdjuster(m.desc) as g:
        base = g.solve(_opts())
    with ba.BundleAdjuster(m.desc) as g:
        tun = g.autotune(N.MBA_PRECISION_FP64)
        assert tun["visual_block"] in (64, 128, 256) and tun["visual_min_blocks"] in (1, 2, 3, 4)
        assert tun["visual_pipelined"] in (1, 2)
        assert tun["schur_chunk"] in (4, 8, 16, 32, 64)
        assert tun["chain_tail_nodes"] in (32, 64, 128, 256, 512)
        assert tun["chain_segment"] in (1, 16, 32, 64, 128, 256)
        assert tun["chain_tail_smem"] in (1, 2)
        assert tun["pcg_product"] in (1, 2)
        assert tun["schur_split"] in (1, 2)
        assert tun["visual_ms"] > 0 and tun["schur_ms"] > 0 and tun["chain_apply_ms"] > 0
        tuned = g.solve(_opts())
    assert abs(tuned["final_cost"] - base["final_cost"]) <= 1e-6 * base["final_cost"]
    with ba.BundleAdjuster(m.desc) as g:
        g.set_tuning(visual_block=64, schur_chunk=4, chain_tail_nodes=32)
        s = g.solve(_opts())
    assert abs(s["final_cost"] - base["final_cost"]) <= 1e-6 * base["final_cost"]


def test_mixed_candidate_cost_agrees_with_fp64():
    """The mixed path evaluates candidate costs from FP32 residuals (FP64 sum);
    its final cost agrees with the full FP64 evaluation of the same state."""
    m = synth.generate("c2", keyframes_per_mission=500, num_landmarks=50000)
    with ba.BundleAdjuster(m.desc) as g:
        s = g.solve(_opts(max_num_iterations=8, precision=N.MBA_PRECISION_MIXED, preconditioner=N.MBA_PRECOND_CHAIN,
                          max_linear_iterations=25, use_cuda_graph=2))
        c64 = g.cost()
    assert abs(s["final_cost"] - c64) <= 1e-6 * c64, (s["final_cost"], c64)
