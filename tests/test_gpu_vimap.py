"""The map-folder path on the GPU: vimap.optimize (load the map folder,
export the problem, solve, write the state back, save) against solving the
synthetic problem it was written from.  The exported problem holds the same
terms in another order, so the LM runs agree to summation order: costs
within 1e-6, keyframe and landmark states and loop-closure switches within
1e-6 after reloading the saved map."""
import ctypes

import numpy as np
import pytest

from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth, vimap
from test_vimap_io import ALL_TERMS, arr, synth_index
from vimap_writer import write_map

pytestmark = pytest.mark.gpu


def _opts():
    return ba.default_options(max_num_iterations=8, check_tolerances=0, linear_tolerance=1e-10,
                              max_linear_iterations=6000)


@pytest.mark.parametrize("case", ["vi", "multi_mission_graph"])
def test_optimize_map_folder_matches_direct_solve(tmp_path, case):
    if case == "vi":
        m = synth.generate("c1")
        export = dict(landmark_selection=N.MBA_VIMAP_LANDMARKS_ALL)
    else:
        m = synth.generate("c4", num_missions=2, keyframes_per_mission=60, num_landmarks=1500,
                           shared_landmark_fraction=0.3, pose_edges=1, loop_closure_stride=6,
                           loop_closure_outlier_fraction=0.2, absolute_pose_stride=20)
        export = dict(ALL_TERMS)
    src, out = tmp_path / "map", tmp_path / "optimized"
    write_map(m, str(src))
    # the direct problem with the gauge fixes the export applies
    from test_gauge_fixes import fixes
    kf_flags, lm_const, _ = fixes(m)
    direct = N.ProblemDesc()
    ctypes.memmove(ctypes.byref(direct), ctypes.byref(m.desc), ctypes.sizeof(direct))
    direct.kf_flags = kf_flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    direct.lm_constant = N.ptr(lm_const, ctypes.c_uint8)
    with ba.BundleAdjuster(direct) as g:
        s0 = g.solve(_opts())
        st0 = g.read_state()
        sw0 = g.read_switch_variables() if m.desc.num_pose_edges else None
    s1 = vimap.optimize(str(src), str(out), _opts(), **export)
    assert abs(s1["initial_cost"] - s0["initial_cost"]) <= 1e-12 * s0["initial_cost"]
    assert abs(s1["final_cost"] - s0["final_cost"]) <= 1e-6 * s0["final_cost"], (s1["final_cost"], s0["final_cost"])
    with vimap.VIMap(str(out)) as vm:
        d = vm.export(**export)
        ids = vm.export_ids()
        ki, li = synth_index(ids["keyframes"]), synth_index(ids["landmarks"])
        kx = arr(d, "kf_q_IM_p_MI", (d.num_keyframes, 7))
        np.testing.assert_allclose(kx, st0["kf_q_IM_p_MI"][ki], rtol=0, atol=1e-6)
        np.testing.assert_allclose(arr(d, "kf_v_M", (d.num_keyframes, 3)), st0["kf_v_M"][ki], rtol=0, atol=1e-6)
        np.testing.assert_allclose(arr(d, "lm_p_B", (d.num_landmarks, 3)), st0["lm_p_B"][li], rtol=0, atol=1e-6)
        if sw0 is not None:
            ty = m.array("pose_edge_type")
            lc = ty == N.MBA_POSE_EDGE_LOOP_CLOSURE
            dty = arr(d, "pose_edge_type", (d.num_pose_edges,), np.int32)
            sw1 = arr(d, "pose_edge_switch", (d.num_pose_edges,))[dty == N.MBA_POSE_EDGE_LOOP_CLOSURE]
            np.testing.assert_allclose(sw1, sw0[lc], rtol=0, atol=1e-6)  # loop closures keep the synthetic order
            assert sw1.min() < 0.5  # outliers switched off and written back
