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


def _small_map():
    return synth.generate("c4", num_missions=3, keyframes_per_mission=30, num_landmarks=800,
                          shared_landmark_fraction=0.3, include_inertial=0)


def test_noalloc_cost_matches_the_oracle():
    """The same cost straight against the CPU oracle's robustified cost."""
    torch = pytest.importorskip("torch")
    import oracle_lib
    m = _small_map()
    expected = oracle_lib.OracleProblem(m.desc).cost()
    batch, keep = _device_batch(m, torch)
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = ba.lib().mba_visual_cost_noalloc(ctypes.byref(batch), torch.cuda.current_device(), None,
                                          ctypes.c_void_p(out.data_ptr()))
    assert st == N.MBA_OK
    got = float(out.item())
    assert abs(got - expected) <= 1e-12 * expected, (got, expected)


def test_noalloc_reports_bad_index_and_non_finite_then_clears_the_flags():
    """A batch with one landmark index past the end (skipped on the device)
    reports MBA_ERR_OUT_OF_RANGE_INDEX; one NaN uncertainty reports
    MBA_ERR_NON_FINITE; a valid call right after each reports MBA_OK with
    the right cost, so the flags the bad call left are cleared."""
    torch = pytest.importorskip("torch")
    import oracle_lib
    m = _small_map()
    expected = oracle_lib.OracleProblem(m.desc).cost()
    lib = ba.lib()
    dev = torch.cuda.current_device()
    batch, keep = _device_batch(m, torch)
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")

    def call():
        torch.cuda.synchronize()
        return lib.mba_visual_cost_noalloc(ctypes.byref(batch), dev, None, ctypes.c_void_p(out.data_ptr()))

    good_lm = keep["obs_landmark"][5].item()
    keep["obs_landmark"][5] = m.desc.num_landmarks  # one past the end: never read
    assert call() == N.MBA_ERR_OUT_OF_RANGE_INDEX
    keep["obs_landmark"][5] = good_lm
    assert call() == N.MBA_OK
    assert abs(float(out.item()) - expected) <= 1e-12 * expected

    r, _ = oracle_lib.OracleProblem(m.desc).evaluate_visual()
    i = int(np.flatnonzero(np.any(r != 0.0, axis=1))[0])  # a projection that succeeds
    good_sigma = keep["obs_sigma"][i].item()
    keep["obs_sigma"][i] = float("nan")
    assert call() == N.MBA_ERR_NON_FINITE
    keep["obs_sigma"][i] = good_sigma
    assert call() == N.MBA_OK
    assert abs(float(out.item()) - expected) <= 1e-12 * expected


def test_noalloc_rejects_batches_above_the_scratch_limit():
    torch = pytest.importorskip("torch")
    lib = ba.lib()
    b = N.VisualBatchDevice()
    b.num_observations = 65536 * 256 + 1
    b.num_landmarks = b.num_keyframes = b.num_missions = b.num_cameras = 1
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.mba_visual_cost_noalloc(ctypes.byref(b), torch.cuda.current_device(), None,
                                       ctypes.c_void_p(out.data_ptr())) == N.MBA_ERR_INVALID_ARG
