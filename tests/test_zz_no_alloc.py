"""mba_visual_cost_noalloc: the allocation-free cost entry point for callers
that may not allocate device memory while running (a real-time estimator
thread that must not stall on cudaMalloc's synchronization or fail on an
out-of-memory error mid-mission; an application whose device memory belongs
to another allocator's pool).

The inputs and the output live in device memory that this test allocates on
the caller's behalf; the entry point itself allocates nothing and keeps its
intermediates in a fixed file-scope device array.  Its result must equal the
handle-based mba_cost on the same problem, to the 1e-12 relative tolerance the
other cost tests use, on two calls in a row (the second call reuses the scratch
array the first one left behind).  This file is collected last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu


def _device_batch(m, torch):
    d = m.desc

    def dev(name, dtype):
        return torch.from_numpy(np.ascontiguousarray(m.array(name), dtype=dtype)).cuda()

    cams = (N.Camera * d.num_cameras)()
    ctypes.memmove(cams, d.cameras, ctypes.sizeof(cams))
    keep = {
        "obs_uv": dev("obs_uv", np.float64), "obs_sigma": dev("obs_sigma", np.float64),
        "obs_landmark": dev("obs_landmark", np.int32), "obs_keyframe": dev("obs_keyframe", np.int32),
        "obs_camera": dev("obs_camera", np.int32), "lm_store_keyframe": dev("lm_store_keyframe", np.int32),
        "lm_p_B": dev("lm_p_B", np.float64), "kf_q_IM_p_MI": dev("kf_q_IM_p_MI", np.float64),
        "kf_mission": dev("kf_mission", np.int32), "mission_q_GM_p_GM": dev("mission_q_GM_p_GM", np.float64),
        "cameras": torch.frombuffer(bytearray(bytes(cams)), dtype=torch.uint8).cuda(),
    }
    b = N.VisualBatchDevice()
    b.num_observations, b.num_landmarks = d.num_observations, d.num_landmarks
    b.num_keyframes, b.num_missions, b.num_cameras = d.num_keyframes, d.num_missions, d.num_cameras
    for k, t in keep.items():
        setattr(b, k, t.data_ptr())
    b.use_huber = d.use_huber
    b.huber_delta_local, b.huber_delta_global = d.huber_delta_local, d.huber_delta_global
    return b, keep


def test_noalloc_cost_matches_handle_cost_on_two_calls():
    torch = pytest.importorskip("torch")
    # Visual-only (no IMU edges), several missions with shared landmarks: the
    # batch holds kLocalKeyframe, kLocalMission and kGlobal terms.
    m = synth.generate("c4", num_missions=4, keyframes_per_mission=60, num_landmarks=3000,
                       shared_landmark_fraction=0.3, include_inertial=0)
    with ba.BundleAdjuster(m.desc) as g:
        expected = g.cost()
    lib = ba.lib()
    batch, keep = _device_batch(m, torch)
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        st = lib.mba_visual_cost_noalloc(ctypes.byref(batch), torch.cuda.current_device(), None,
                                         ctypes.c_void_p(out.data_ptr()))
        assert st == N.MBA_OK, f"call {call}: status {st}"
        got = float(out.item())
        assert abs(got - expected) <= 1e-12 * expected, (call, got, expected)
        out.fill_(float("nan"))
        torch.cuda.synchronize()


def test_noalloc_rejects_batches_above_the_scratch_limit():
    torch = pytest.importorskip("torch")
    lib = ba.lib()
    b = N.VisualBatchDevice()
    b.num_observations = 65536 * 256 + 1
    b.num_landmarks = b.num_keyframes = b.num_missions = b.num_cameras = 1
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.mba_visual_cost_noalloc(ctypes.byref(b), torch.cuda.current_device(), None,
                                       ctypes.c_void_p(out.data_ptr())) == N.MBA_ERR_INVALID_ARG
