"""Learned chain preconditioner on the device against the numpy oracle
(oracle/gnn_oracle.py) and its effect on the solve.

Bars: coefficients of the forward pass within 2e-3 (BF16 activations on both
sides, FP32 vs FP64 accumulation); loss within 1e-3 relative; gradient per
parameter tensor within 5e-2 relative (BF16 pre-activation gradients);
training lowers the probe loss; the learned preconditioner needs fewer PCG
iterations than block-Jacobi at equal tolerance and reaches the FP64 path's
cost.
"""
import os
import sys

import numpy as np
import pytest

from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import gnn_oracle as G  # noqa: E402

pytestmark = pytest.mark.gpu

RADIUS = 1e4


@pytest.fixture(scope="module")
def c1_case():
    m = synth.generate("c1")
    g = ba.BundleAdjuster(m.desc)
    model = ba.PreconditionerModel(seed=11)
    rng = np.random.default_rng(5)
    w = model.parameters()
    w += rng.normal(size=w.size).astype(np.float32) * 0.05  # move off the initial head bias
    model.set_parameters(w)
    sysd = g.reduced_system(N.MBA_PRECISION_MIXED, RADIUS)
    perm, le, lb = g.chain_structure()
    cp = G.ChainProblem(sysd, perm, le, lb)
    probes = rng.normal(size=(2, 15 * m.desc.num_keyframes)).astype(np.float32)
    yield m, g, model, cp, probes
    g.close()
    model.close()


def test_forward_coefficients_match_oracle(c1_case):
    _, g, model, cp, probes = c1_case
    _, _, coef = g.preconditioner_gradient(model, RADIUS, probes=probes)
    f = G.forward(cp, model.parameters().astype(np.float64), use_bf16=True)
    np.testing.assert_allclose(coef, f["coef"], atol=2e-3)


def test_loss_and_gradient_match_oracle(c1_case):
    _, g, model, cp, probes = c1_case
    loss, grad, _ = g.preconditioner_gradient(model, RADIUS, probes=probes)
    lo, go, _, _ = G.loss_and_grad(cp, model.parameters().astype(np.float64), probes.astype(np.float64), True)
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    L, _ = G.layout()
    for name, (off, shp) in L.items():
        a, b = grad[off:off + int(np.prod(shp))], go[off:off + int(np.prod(shp))]
        nb_ = np.linalg.norm(b)
        if nb_ < 1e-12 * max(1.0, np.linalg.norm(go)):
            continue
        assert np.linalg.norm(a - b) <= 5e-2 * nb_, (name, np.linalg.norm(a - b) / nb_)


def test_training_lowers_probe_loss():
    m = synth.generate("c1")
    with ba.BundleAdjuster(m.desc) as g:
        model = ba.PreconditionerModel(seed=3)
        losses = g.train_preconditioner(model, RADIUS, nprobe=4, steps=40, lr=3e-3, seed=1)
        after = g.train_preconditioner(model, RADIUS, nprobe=4, steps=1, lr=0.0, seed=1)
        model.close()
    assert np.all(np.isfinite(losses))
    assert after[0] < losses[0], (losses[0], after[0])


def test_trained_network_gain_over_block_jacobi():
    """What the trained network gains over the method without it (plain
    block-Jacobi PCG): with PCG capped at 25 iterations, the mixed path with
    the shipped trained model reaches the FP64 path's 20-iteration cost in at
    most 10 LM iterations; block-Jacobi does not reach it in 40.  The
    fixed-coefficient chain (gamma = 1, alpha = 0) is run beside it as the
    ablation of the learned coefficients."""
    from maplab_gb300 import train_preconditioner as TP
    model = TP.load_default_model()
    assert model is not None, "trained weights missing"
    m = synth.generate("c1")
    opts = lambda **kw: ba.default_options(check_tolerances=0, linear_tolerance=1e-6, **kw)
    with ba.BundleAdjuster(m.desc) as g:
        s64 = g.solve(opts(max_num_iterations=20, max_linear_iterations=100))
    target = s64["final_cost"] * (1 + 1e-6)
    runs = {}
    for name, pre in (("bj", N.MBA_PRECOND_BLOCK_JACOBI), ("chain", N.MBA_PRECOND_CHAIN),
                      ("learned", N.MBA_PRECOND_LEARNED)):
        with ba.BundleAdjuster(m.desc) as g:
            g.set_preconditioner_model(model)
            runs[name] = g.solve(opts(max_num_iterations=40, max_linear_iterations=25, stop_cost=target,
                                      precision=N.MBA_PRECISION_MIXED, preconditioner=pre))
    model.close()
    assert runs["learned"]["termination"] == 6 and runs["learned"]["num_iterations"] - 1 <= 10, runs["learned"]
    assert runs["bj"]["termination"] != 6, runs["bj"]
    assert runs["chain"]["termination"] == 6


def test_learned_without_model_is_rejected():
    m = synth.generate("c1")
    with ba.BundleAdjuster(m.desc) as g:
        with pytest.raises(ba.BAError):
            g.solve(ba.default_options(max_num_iterations=2, precision=N.MBA_PRECISION_MIXED,
                                       preconditioner=N.MBA_PRECOND_LEARNED))
