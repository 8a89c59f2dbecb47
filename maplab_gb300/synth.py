"""Seeded synthetic maps for the benchmark configurations (libmba_synth.so).

Presets follow the benchmark configurations of the VI bundle-adjustment
workload (shapes, noise and perturbation model of maplab's
test/vi-map-generator-6dof recipe):

* ``c1``: 100 keyframes on a 20 m circle, 10 Hz keyframes, 200 Hz IMU, one
  pinhole-radtan camera 752x480 (fu=fv=460, k1=-0.28, k2=0.07), 2,000
  landmarks uniform in a 30x30x5 m box, each seen by U{2..8} keyframes.
* ``c2``: 2,000 keyframes, 200k landmarks, track length geometric (mean 8,
  cap 40), two cameras (radtan + equidistant k=[-0.01, 0.005, -0.001, 1e-4]).
* ``c3``: 64 independent missions, keyframes log-uniform in [50, 1500], 100
  landmarks per keyframe, missions alternate radtan / equidistant cameras.
* ``c4``: 10 co-registered missions (2,000 keyframes each), 2M landmarks,
  10 % of landmarks shared between two missions (kGlobal terms).
* ``c5``: 40 missions x 1,250 keyframes, 5M landmarks, power-law tracks
  (alpha 2.2, lengths 3 to 200).
"""
import ctypes

import numpy as np

from . import _native as N


def config(preset="c1", seed=None, **overrides):
    lib = N.load_synth()
    c = N.SynthConfig()
    lib.mba_synth_default_config(ctypes.byref(c))
    if preset == "c1":
        c.seed = 1
    elif preset == "c2":
        c.seed = 2
        c.keyframes_per_mission = 2000
        c.num_landmarks = 200_000
        c.landmark_mode = N.MBA_SYNTH_LANDMARKS_FRUSTUM
        c.track_model = N.MBA_SYNTH_TRACK_GEOMETRIC
        c.track_mean = 8.0
        c.track_max = 40
        c.num_cameras = 2
    elif preset == "c3":
        c.seed = 3
        c.num_missions = 64
        c.kf_min, c.kf_max = 50, 1500
        c.landmarks_per_keyframe = 100
        c.landmark_mode = N.MBA_SYNTH_LANDMARKS_FRUSTUM
        c.track_model = N.MBA_SYNTH_TRACK_GEOMETRIC
        c.track_max = 40
        c.num_cameras = 2
        c.camera_per_mission = 1
        c.co_registered = 0
    elif preset == "c4":
        c.seed = 4
        c.num_missions = 10
        c.keyframes_per_mission = 2000
        c.num_landmarks = 2_000_000
        c.landmark_mode = N.MBA_SYNTH_LANDMARKS_FRUSTUM
        c.track_model = N.MBA_SYNTH_TRACK_GEOMETRIC
        c.track_max = 40
        c.num_cameras = 2
        c.shared_landmark_fraction = 0.1
    elif preset == "c5":
        c.seed = 5
        c.num_missions = 40
        c.keyframes_per_mission = 1250
        c.num_landmarks = 5_000_000
        c.landmark_mode = N.MBA_SYNTH_LANDMARKS_FRUSTUM
        c.track_model = N.MBA_SYNTH_TRACK_POWER_LAW
        c.track_alpha = 2.2
        c.track_min = 3  # lower cut-off of the power law: mean track about 8.8, about 44M observations
        c.track_max = 200
        c.num_cameras = 2
        c.shared_landmark_fraction = 0.02
    else:
        raise ValueError(f"unknown preset {preset!r}")
    if seed is not None:
        c.seed = seed
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


class SyntheticMap:
    """Owns a generated map; ``desc`` points into it (valid while alive)."""

    def __init__(self, cfg):
        self._lib = N.load_synth()
        h = ctypes.c_void_p()
        st = self._lib.mba_synth_generate(ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            raise RuntimeError(f"mba_synth_generate failed with status {st}")
        self._h = h
        self.cfg = cfg
        self.desc = N.ProblemDesc()
        self._lib.mba_synth_describe(self._h, ctypes.byref(self.desc))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.mba_synth_free(h)
            self._h = None

    @property
    def sizes(self):
        d = self.desc
        return dict(keyframes=d.num_keyframes, landmarks=d.num_landmarks, observations=d.num_observations,
                    cameras=d.num_cameras, missions=d.num_missions, imu_edges=d.num_imu_edges,
                    imu_samples=d.num_imu_samples)

    def array(self, name):
        """Numpy view of one descriptor array (no copy)."""
        d = self.desc
        shapes = {
            "obs_uv": (d.num_observations, 2), "obs_sigma": (d.num_observations,),
            "obs_landmark": (d.num_observations,), "obs_keyframe": (d.num_observations,),
            "obs_camera": (d.num_observations,), "lm_p_B": (d.num_landmarks, 3),
            "lm_store_keyframe": (d.num_landmarks,), "lm_constant": (d.num_landmarks,),
            "kf_q_IM_p_MI": (d.num_keyframes, 7), "kf_v_M": (d.num_keyframes, 3),
            "kf_b_g": (d.num_keyframes, 3), "kf_b_a": (d.num_keyframes, 3),
            "kf_mission": (d.num_keyframes,), "kf_flags": (d.num_keyframes,),
            "mission_q_GM_p_GM": (d.num_missions, 7), "edge_from": (d.num_imu_edges,),
            "edge_to": (d.num_imu_edges,), "edge_sample_offset": (d.num_imu_edges + 1,),
            "imu_timestamp_ns": (d.num_imu_samples,), "imu_acc_gyro": (d.num_imu_samples, 6),
            "pose_edge_from": (d.num_pose_edges,), "pose_edge_to": (d.num_pose_edges,),
            "pose_edge_T_Bk_Bkp1": (d.num_pose_edges, 7), "pose_edge_covariance": (d.num_pose_edges, 36),
            "pose_edge_q_I_B_p_B_I": (d.num_pose_edges, 7), "pose_edge_type": (d.num_pose_edges,),
            "pose_edge_switch": (d.num_pose_edges,), "pose_edge_switch_variance": (d.num_pose_edges,),
        }
        p = getattr(d, name)
        n = int(np.prod(shapes[name]))
        if n == 0:
            return np.zeros(shapes[name])
        return np.ctypeslib.as_array(p, shape=(n,)).reshape(shapes[name])

    def ground_truth(self):
        d = self.desc
        kx = np.zeros((d.num_keyframes, 7)); kv = np.zeros((d.num_keyframes, 3))
        kbg = np.zeros((d.num_keyframes, 3)); kba = np.zeros((d.num_keyframes, 3))
        lp = np.zeros((d.num_landmarks, 3))
        self._lib.mba_synth_ground_truth(self._h, N.ptr(kx), N.ptr(kv), N.ptr(kbg), N.ptr(kba), N.ptr(lp))
        return dict(kf_q_IM_p_MI=kx, kf_v_M=kv, kf_b_g=kbg, kf_b_a=kba, lm_p_B=lp)


def generate(preset="c1", seed=None, **overrides):
    return SyntheticMap(config(preset, seed, **overrides))
