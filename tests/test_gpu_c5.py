"""The largest configuration on one GPU: 40 missions, 50,000 keyframes, 5M
landmarks, 27M observations with power-law track lengths (capped at 200),
15-dimensional keyframe states with inertial edges.  Size-independent checks
of the mixed path (FP32 Jacobians, Schur complement and PCG; FP64 cost sums
and state): every accepted LM step lowers the cost, the final cost the solve
reports agrees with an FP64 re-evaluation of the final state to 1e-6, the
device memory the handle holds stays within the 180 GB budget, and the
chain-preconditioned device loop ends by its own rules."""
import pytest

from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu


def test_c5_mixed_solve_at_full_size():
    m = synth.generate("c5")
    d = m.desc
    assert (d.num_keyframes, d.num_landmarks, d.num_missions) == (50000, 5000000, 40)
    assert d.num_observations > 2.5e7 and d.num_imu_edges > 4.9e4
    opts = ba.default_options(max_num_iterations=4, check_tolerances=0, precision=N.MBA_PRECISION_MIXED,
                              preconditioner=N.MBA_PRECOND_CHAIN, max_linear_iterations=25, use_cuda_graph=2)
    with ba.BundleAdjuster(d) as g:
        s = g.solve(opts)
        c64 = g.cost()
        st = g.stats()
    assert st["device_bytes"] < 180e9, st["device_bytes"]
    assert s["termination"] == 0 and s["num_iterations"] == 5
    costs = [s["initial_cost"]] + [it["cost"] for it in s["iterations"][1:]]
    assert all(b <= a for a, b in zip(costs, costs[1:])), costs
    assert s["final_cost"] < 0.5 * s["initial_cost"], (s["initial_cost"], s["final_cost"])
    assert abs(s["final_cost"] - c64) <= 1e-6 * c64, (s["final_cost"], c64)
