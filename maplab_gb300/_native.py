"""ctypes mirrors of include/maplab_ba.h and include/maplab_ba_synth.h.

The structures below follow the C declarations field by field; ctypes applies
the platform C alignment rules, so the layouts match on x86_64 and aarch64.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_HERE, "_build")

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int32_p = ctypes.POINTER(ctypes.c_int32)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_uint8_p = ctypes.POINTER(ctypes.c_uint8)
c_uint32_p = ctypes.POINTER(ctypes.c_uint32)

# mba_status
MBA_OK = 0
MBA_ERR_INVALID_ARG = 1
MBA_ERR_OUT_OF_RANGE_INDEX = 2
MBA_ERR_NON_FINITE = 3
MBA_ERR_NOT_SPD = 4
MBA_ERR_CUDA = 5
MBA_ERR_TIMEOUT = 6
MBA_ERR_CANCELLED = 7
MBA_POSE_EDGE_RELATIVE = 0
MBA_POSE_EDGE_LOOP_CLOSURE = 1
MBA_POSE_EDGE_ABSOLUTE = 2
MBA_ERR_NO_DEVICE = 8
MBA_ERR_UNORDERED_IMU = 9

MBA_LOCAL_KEYFRAME, MBA_LOCAL_MISSION, MBA_GLOBAL = 0, 1, 2
MBA_DISTORTION_NONE, MBA_DISTORTION_RADTAN, MBA_DISTORTION_EQUIDISTANT, MBA_DISTORTION_FOV = 0, 1, 2, 3

MBA_CAM_INTRINSICS_FREE = 1 << 0
MBA_CAM_DISTORTION_FREE = 1 << 1
MBA_CAM_ROTATION_FREE = 1 << 2
MBA_CAM_TRANSLATION_FREE = 1 << 3
MBA_MIS_BASEFRAME_YAW_POSITION = 1 << 0
MBA_MIS_BASEFRAME_POSE = 1 << 1

MBA_KF_POSE_CONSTANT = 1 << 0
MBA_KF_GAUGE_ROLL_PITCH = 1 << 1
MBA_KF_VELOCITY_CONSTANT = 1 << 2
MBA_KF_GYRO_BIAS_CONSTANT = 1 << 3
MBA_KF_ACCEL_BIAS_CONSTANT = 1 << 4
MBA_KF_POSITION_CONSTANT = 1 << 5
MBA_KF_ROTATION_CONSTANT = 1 << 6

MBA_LINEAR_SOLVER_PCG, MBA_LINEAR_SOLVER_DENSE_SCHUR = 0, 1
MBA_PRECOND_BLOCK_JACOBI, MBA_PRECOND_LEARNED, MBA_PRECOND_CHAIN = 0, 1, 2
MBA_PRECISION_FP64, MBA_PRECISION_MIXED = 0, 1

MBA_SYNTH_LANDMARKS_BOX, MBA_SYNTH_LANDMARKS_FRUSTUM = 0, 1
MBA_SYNTH_TRACK_UNIFORM, MBA_SYNTH_TRACK_GEOMETRIC, MBA_SYNTH_TRACK_POWER_LAW = 0, 1, 2


class Camera(ctypes.Structure):
    _fields_ = [
        ("intrinsics", ctypes.c_double * 4),
        ("distortion", ctypes.c_double * 4),
        ("distortion_type", ctypes.c_int32),
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("q_CI_p_CI", ctypes.c_double * 7),
    ]


class ProblemDesc(ctypes.Structure):
    _fields_ = [
        ("num_keyframes", ctypes.c_int64),
        ("num_landmarks", ctypes.c_int64),
        ("num_observations", ctypes.c_int64),
        ("num_cameras", ctypes.c_int64),
        ("num_missions", ctypes.c_int64),
        ("num_imu_edges", ctypes.c_int64),
        ("num_imu_samples", ctypes.c_int64),
        ("obs_uv", c_double_p),
        ("obs_sigma", c_double_p),
        ("obs_landmark", c_int32_p),
        ("obs_keyframe", c_int32_p),
        ("obs_camera", c_int32_p),
        ("lm_p_B", c_double_p),
        ("lm_store_keyframe", c_int32_p),
        ("lm_constant", c_uint8_p),
        ("kf_q_IM_p_MI", c_double_p),
        ("kf_v_M", c_double_p),
        ("kf_b_g", c_double_p),
        ("kf_b_a", c_double_p),
        ("kf_mission", c_int32_p),
        ("kf_flags", c_uint32_p),
        ("mission_q_GM_p_GM", c_double_p),
        ("cameras", ctypes.POINTER(Camera)),
        ("edge_from", c_int32_p),
        ("edge_to", c_int32_p),
        ("edge_sample_offset", c_int64_p),
        ("imu_timestamp_ns", c_int64_p),
        ("imu_acc_gyro", c_double_p),
        ("gyro_noise_sigma", ctypes.c_double),
        ("gyro_bias_sigma", ctypes.c_double),
        ("acc_noise_sigma", ctypes.c_double),
        ("acc_bias_sigma", ctypes.c_double),
        ("gravity_magnitude", ctypes.c_double),
        ("use_huber", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("huber_delta_local", ctypes.c_double),
        ("huber_delta_global", ctypes.c_double),
        ("num_pose_edges", ctypes.c_int64),
        ("pose_edge_from", c_int32_p),
        ("pose_edge_to", c_int32_p),
        ("pose_edge_T_Bk_Bkp1", c_double_p),
        ("pose_edge_covariance", c_double_p),
        ("pose_edge_q_I_B_p_B_I", c_double_p),
        ("pose_edge_type", c_int32_p),
        ("pose_edge_switch", c_double_p),
        ("pose_edge_switch_variance", c_double_p),
        ("camera_flags", c_uint32_p),
        ("mission_flags", c_uint32_p),
    ]


class SolverOptions(ctypes.Structure):
    _fields_ = [
        ("max_num_iterations", ctypes.c_int32),
        ("jacobi_scaling", ctypes.c_int32),
        ("initial_trust_region_radius", ctypes.c_double),
        ("max_trust_region_radius", ctypes.c_double),
        ("min_trust_region_radius", ctypes.c_double),
        ("function_tolerance", ctypes.c_double),
        ("gradient_tolerance", ctypes.c_double),
        ("parameter_tolerance", ctypes.c_double),
        ("min_relative_decrease", ctypes.c_double),
        ("min_lm_diagonal", ctypes.c_double),
        ("max_lm_diagonal", ctypes.c_double),
        ("linear_solver", ctypes.c_int32),
        ("max_linear_iterations", ctypes.c_int32),
        ("linear_tolerance", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("preconditioner", ctypes.c_int32),
        ("use_cuda_graph", ctypes.c_int32),
        ("check_tolerances", ctypes.c_int32),
        ("stop_cost", ctypes.c_double),
        ("reject_outliers_every_n_iters", ctypes.c_int32),
        ("outlier_use_reprojection_error", ctypes.c_int32),
        ("outlier_max_reprojection_error_px", ctypes.c_double),
    ]


class IterationSummary(ctypes.Structure):
    _fields_ = [
        ("iteration", ctypes.c_int32),
        ("step_is_successful", ctypes.c_int32),
        ("linear_solver_iterations", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("cost", ctypes.c_double),
        ("cost_change", ctypes.c_double),
        ("gradient_max_norm", ctypes.c_double),
        ("step_norm", ctypes.c_double),
        ("relative_decrease", ctypes.c_double),
        ("trust_region_radius", ctypes.c_double),
        ("iteration_time_ms", ctypes.c_double),
    ]


class Summary(ctypes.Structure):
    _fields_ = [
        ("num_iterations", ctypes.c_int32),
        ("num_successful_steps", ctypes.c_int32),
        ("termination", ctypes.c_int32),
        ("total_linear_iterations", ctypes.c_int32),
        ("initial_cost", ctypes.c_double),
        ("final_cost", ctypes.c_double),
        ("total_time_ms", ctypes.c_double),
        ("time_to_stop_cost_ms", ctypes.c_double),
        ("max_iterations_capacity", ctypes.c_int32),
        ("num_rejected_landmarks", ctypes.c_int32),
        ("iterations", ctypes.POINTER(IterationSummary)),
    ]


class LandmarkQualityOptions(ctypes.Structure):
    _fields_ = [
        ("min_observers", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("min_observation_angle_deg", ctypes.c_double),
        ("max_distance_from_closest_observer", ctypes.c_double),
        ("min_distance_from_closest_observer", ctypes.c_double),
        ("max_reprojection_error_px", ctypes.c_double),
    ]


class VimapInfo(ctypes.Structure):
    """mba_vimap_info (include/maplab_vimap.h)."""
    _fields_ = [(n, ctypes.c_int64) for n in (
        "num_missions", "num_vertices", "num_landmarks", "num_keypoints", "num_viwls_edges", "num_odometry_edges",
        "num_wheel_odometry_edges", "num_loop_closure_edges", "num_other_edges", "num_absolute_measurements",
        "num_sensors", "num_cameras")]


class VimapExportOptions(ctypes.Structure):
    """mba_vimap_export_options (include/maplab_vimap.h)."""
    _fields_ = [
        ("num_missions", ctypes.c_int32),
        ("pad0_", ctypes.c_int32),
        ("missions", ctypes.POINTER(ctypes.c_int32)),
        ("add_visual_constraints", ctypes.c_int32),
        ("add_inertial_constraints", ctypes.c_int32),
        ("add_6dof_odometry_constraints", ctypes.c_int32),
        ("add_wheel_odometry_constraints", ctypes.c_int32),
        ("add_absolute_pose_constraints", ctypes.c_int32),
        ("add_loop_closure_edges", ctypes.c_int32),
        ("fix_landmark_positions", ctypes.c_int32),
        ("fix_velocity", ctypes.c_int32),
        ("fix_gyro_bias", ctypes.c_int32),
        ("fix_accel_bias", ctypes.c_int32),
        ("fix_vertices", ctypes.c_int32),
        ("min_landmarks_per_frame", ctypes.c_int32),
        ("feature_type", ctypes.c_int32),
        ("apply_gauge_fixes", ctypes.c_int32),
        ("landmark_selection", ctypes.c_int32),
        ("pad1_", ctypes.c_int32),
        ("landmark_keep", ctypes.POINTER(ctypes.c_uint8)),
        ("quality", LandmarkQualityOptions),
        ("gravity_magnitude", ctypes.c_double),
        ("use_huber", ctypes.c_int32),
        ("pad2_", ctypes.c_int32),
    ]


MBA_VIMAP_LANDMARKS_QUALITY = 0
MBA_VIMAP_LANDMARKS_ALL = 1
MBA_VIMAP_LANDMARKS_MASK = 2


class Tuning(ctypes.Structure):
    _fields_ = [
        ("visual_block", ctypes.c_int32),
        ("schur_chunk", ctypes.c_int32),
        ("chain_tail_nodes", ctypes.c_int32),
        ("visual_min_blocks", ctypes.c_int32),
        ("visual_ms", ctypes.c_double),
        ("schur_ms", ctypes.c_double),
        ("chain_apply_ms", ctypes.c_double),
        ("visual_pipelined", ctypes.c_int32),
        ("chain_segment", ctypes.c_int32),
        ("chain_tail_smem", ctypes.c_int32),
        ("pcg_product", ctypes.c_int32),
        ("schur_split", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
    ]


class ProblemStats(ctypes.Structure):
    _fields_ = [
        ("num_keyframes", ctypes.c_int64),
        ("num_landmarks", ctypes.c_int64),
        ("num_observations", ctypes.c_int64),
        ("num_imu_edges", ctypes.c_int64),
        ("num_schur_pose_blocks", ctypes.c_int64),
        ("device_bytes", ctypes.c_int64),
        ("num_pose_edges", ctypes.c_int64),
    ]


class VisualBatchDevice(ctypes.Structure):
    _fields_ = [
        ("num_observations", ctypes.c_int64),
        ("num_landmarks", ctypes.c_int64),
        ("num_keyframes", ctypes.c_int64),
        ("num_missions", ctypes.c_int64),
        ("num_cameras", ctypes.c_int64),
        ("obs_uv", ctypes.c_void_p),
        ("obs_sigma", ctypes.c_void_p),
        ("obs_landmark", ctypes.c_void_p),
        ("obs_keyframe", ctypes.c_void_p),
        ("obs_camera", ctypes.c_void_p),
        ("lm_store_keyframe", ctypes.c_void_p),
        ("lm_p_B", ctypes.c_void_p),
        ("kf_q_IM_p_MI", ctypes.c_void_p),
        ("kf_mission", ctypes.c_void_p),
        ("mission_q_GM_p_GM", ctypes.c_void_p),
        ("cameras", ctypes.c_void_p),
        ("use_huber", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("huber_delta_local", ctypes.c_double),
        ("huber_delta_global", ctypes.c_double),
    ]


class SynthConfig(ctypes.Structure):
    _fields_ = [
        ("seed", ctypes.c_uint64),
        ("num_missions", ctypes.c_int32),
        ("keyframes_per_mission", ctypes.c_int32),
        ("kf_min", ctypes.c_int32),
        ("kf_max", ctypes.c_int32),
        ("landmarks_per_keyframe", ctypes.c_int32),
        ("num_landmarks", ctypes.c_int64),
        ("landmark_mode", ctypes.c_int32),
        ("track_model", ctypes.c_int32),
        ("track_min", ctypes.c_int32),
        ("track_max", ctypes.c_int32),
        ("track_mean", ctypes.c_double),
        ("track_alpha", ctypes.c_double),
        ("num_cameras", ctypes.c_int32),
        ("camera_per_mission", ctypes.c_int32),
        ("camera0_distortion", ctypes.c_int32),
        ("camera1_distortion", ctypes.c_int32),
        ("radius_m", ctypes.c_double),
        ("box_half_xy", ctypes.c_double),
        ("box_half_z", ctypes.c_double),
        ("keyframes_per_lap", ctypes.c_double),
        ("kf_rate_hz", ctypes.c_double),
        ("imu_rate_hz", ctypes.c_double),
        ("pixel_sigma", ctypes.c_double),
        ("acc_noise", ctypes.c_double),
        ("gyro_noise", ctypes.c_double),
        ("acc_bias_rw", ctypes.c_double),
        ("gyro_bias_rw", ctypes.c_double),
        ("rot_perturb", ctypes.c_double),
        ("pos_perturb", ctypes.c_double),
        ("lm_perturb", ctypes.c_double),
        ("vel_perturb", ctypes.c_double),
        ("shared_landmark_fraction", ctypes.c_double),
        ("include_inertial", ctypes.c_int32),
        ("co_registered", ctypes.c_int32),
        ("pose_edges", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("pose_edge_sigma_p", ctypes.c_double),
        ("pose_edge_sigma_q", ctypes.c_double),
        ("loop_closure_stride", ctypes.c_int32),
        ("absolute_pose_stride", ctypes.c_int32),
        ("loop_closure_sigma_p", ctypes.c_double),
        ("loop_closure_sigma_q", ctypes.c_double),
        ("loop_closure_outlier_fraction", ctypes.c_double),
        ("loop_closure_switch_variance", ctypes.c_double),
        ("absolute_pose_sigma_p", ctypes.c_double),
        ("absolute_pose_sigma_q", ctypes.c_double),
    ]


def ptr(a, ctype=ctypes.c_double):
    """Pointer to a contiguous numpy array (None for None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _declare(lib, name, restype, argtypes):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = argtypes
    return f


def load_synth():
    path = os.path.join(BUILD_DIR, "libmba_synth.so")
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run __graft_entry__.build() first")
    lib = ctypes.CDLL(path)
    _declare(lib, "mba_synth_default_config", None, [ctypes.POINTER(SynthConfig)])
    _declare(lib, "mba_synth_generate", ctypes.c_int, [ctypes.POINTER(SynthConfig), ctypes.POINTER(ctypes.c_void_p)])
    _declare(lib, "mba_synth_free", None, [ctypes.c_void_p])
    _declare(lib, "mba_synth_describe", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ProblemDesc)])
    _declare(lib, "mba_synth_ground_truth", ctypes.c_int, [ctypes.c_void_p] + [c_double_p] * 5)
    return lib


def load_ba():
    """Loads the CUDA back-end (libmaplab_ba.so); raises if it is not built."""
    path = os.path.join(BUILD_DIR, "libmaplab_ba.so")
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: the CUDA back-end is not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    _declare(lib, "mba_abi_version", ctypes.c_int32, [])
    _declare(lib, "mba_default_solver_options", None, [ctypes.POINTER(SolverOptions)])
    _declare(lib, "mba_status_string", ctypes.c_char_p, [ctypes.c_int])
    _declare(lib, "mba_create", ctypes.c_int, [ctypes.POINTER(ProblemDesc), ctypes.c_int32, ctypes.POINTER(vp)])
    _declare(lib, "mba_destroy", None, [vp])
    _declare(lib, "mba_evaluate_visual", ctypes.c_int, [vp, c_double_p, ctypes.POINTER(c_double_p)])
    _declare(lib, "mba_evaluate_inertial", ctypes.c_int, [vp, c_double_p, ctypes.POINTER(c_double_p)])
    _declare(lib, "mba_linearize_visual", ctypes.c_int, [vp, ctypes.c_int32] + [c_double_p] * 4)
    _declare(lib, "mba_linearize_pose_edges", ctypes.c_int, [vp] + [c_double_p] * 3)
    _declare(lib, "mba_read_switch_variables", ctypes.c_int, [vp, c_double_p])
    _declare(lib, "mba_default_landmark_quality_options", None, [ctypes.POINTER(LandmarkQualityOptions)])
    _declare(lib, "mba_landmark_quality", ctypes.c_int, [vp, ctypes.POINTER(LandmarkQualityOptions), c_uint8_p])
    _declare(lib, "mba_gauge_fixes", ctypes.c_int, [ctypes.POINTER(ProblemDesc), ctypes.POINTER(ctypes.c_uint32),
                                                    c_uint8_p, ctypes.POINTER(ctypes.c_int32)])
    _declare(lib, "mba_relaxation_flags", ctypes.c_int, [ctypes.POINTER(ProblemDesc), ctypes.POINTER(ctypes.c_uint32),
                                                         ctypes.POINTER(ctypes.c_uint8)])
    _declare(lib, "mba_write_switch_variables", ctypes.c_int, [vp, c_double_p])
    _declare(lib, "mba_cost", ctypes.c_int, [vp, ctypes.c_int32, c_double_p])
    _declare(lib, "mba_solve", ctypes.c_int, [vp, ctypes.POINTER(SolverOptions), ctypes.POINTER(Summary)])
    _declare(lib, "mba_read_state", ctypes.c_int, [vp] + [c_double_p] * 5)
    _declare(lib, "mba_read_calibration", ctypes.c_int, [vp, ctypes.POINTER(Camera), c_double_p])
    _declare(lib, "mba_write_calibration", ctypes.c_int, [vp, ctypes.POINTER(Camera), c_double_p])
    _declare(lib, "mba_write_state", ctypes.c_int, [vp] + [c_double_p] * 5)
    _declare(lib, "mba_cancel", None, [vp])
    _declare(lib, "mba_time_visual_kernel", ctypes.c_int, [vp, ctypes.c_int32, ctypes.c_int32, c_double_p])
    _declare(lib, "mba_measure_fp64_peak", ctypes.c_int, [ctypes.c_int32, c_double_p])
    _declare(lib, "mba_get_stats", ctypes.c_int, [vp, ctypes.POINTER(ProblemStats)])
    i32p = ctypes.POINTER(ctypes.c_int32)
    f32p = ctypes.POINTER(ctypes.c_float)
    _declare(lib, "mba_gnn_num_parameters", ctypes.c_int64, [])
    _declare(lib, "mba_gnn_create", ctypes.c_int, [ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(vp)])
    _declare(lib, "mba_gnn_destroy", None, [vp])
    _declare(lib, "mba_gnn_get_parameters", ctypes.c_int, [vp, f32p])
    _declare(lib, "mba_gnn_set_parameters", ctypes.c_int, [vp, f32p])
    _declare(lib, "mba_set_preconditioner_model", ctypes.c_int, [vp, vp])
    _declare(lib, "mba_gnn_train", ctypes.c_int, [vp, vp, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.c_float, ctypes.c_uint64, c_double_p])
    _declare(lib, "mba_gnn_gradient", ctypes.c_int, [vp, vp, ctypes.c_double, ctypes.c_int32, f32p, ctypes.c_uint64,
                                                     f32p, c_double_p, c_double_p])
    _declare(lib, "mba_autotune", ctypes.c_int, [vp, ctypes.c_int32, ctypes.POINTER(Tuning)])
    _declare(lib, "mba_set_tuning", ctypes.c_int, [vp, ctypes.POINTER(Tuning)])
    _declare(lib, "mba_chain_structure", ctypes.c_int, [vp, i32p, i32p, i32p])
    _declare(lib, "mba_chain_apply", ctypes.c_int, [vp, ctypes.c_int32, ctypes.c_double, c_double_p, c_double_p])
    _declare(lib, "mba_rejected_landmarks", ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_int64)])
    _declare(lib, "mba_reduced_system", ctypes.c_int,
             [vp, ctypes.c_int32, ctypes.c_double, c_double_p, ctypes.POINTER(ctypes.c_int32), c_double_p,
              c_double_p, c_double_p])
    _declare(lib, "mba_visual_cost_noalloc", ctypes.c_int,
             [ctypes.POINTER(VisualBatchDevice), ctypes.c_int32, vp, vp])
    u16p = ctypes.POINTER(ctypes.c_uint16)
    _declare(lib, "mba_gnn_gemm", ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, u16p, u16p, u16p, u16p,
                                                 ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), u16p])
    _declare(lib, "mba_gnn_gemm_wait_check", ctypes.c_int, [ctypes.c_int32])
    u64p = ctypes.POINTER(ctypes.c_uint64)
    _declare(lib, "mba_vimap_load", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(vp)])
    _declare(lib, "mba_vimap_destroy", None, [vp])
    _declare(lib, "mba_vimap_get_info", ctypes.c_int, [vp, ctypes.POINTER(VimapInfo)])
    _declare(lib, "mba_vimap_mission_ids", ctypes.c_int, [vp, u64p])
    _declare(lib, "mba_vimap_default_export_options", None, [ctypes.POINTER(VimapExportOptions)])
    _declare(lib, "mba_vimap_export", ctypes.c_int, [vp, ctypes.POINTER(VimapExportOptions), ctypes.POINTER(ProblemDesc)])
    _declare(lib, "mba_vimap_export_ids", ctypes.c_int, [vp, u64p, u64p, u64p, u64p])
    _declare(lib, "mba_vimap_landmark_ids", ctypes.c_int, [vp, u64p])
    _declare(lib, "mba_vimap_import_state", ctypes.c_int, [vp] + [c_double_p] * 6)
    _declare(lib, "mba_vimap_save", ctypes.c_int, [vp, ctypes.c_char_p])
    return lib


def default_solver_options(lib=None):
    """ba_* flag defaults (solver-options.cc:3-52) without needing the CUDA library."""
    o = SolverOptions()
    o.max_num_iterations = 30
    o.jacobi_scaling = 1
    o.initial_trust_region_radius = 1e5
    o.max_trust_region_radius = 1e20
    o.min_trust_region_radius = 1e-32
    o.function_tolerance = 1e-12
    o.gradient_tolerance = 1e-10
    o.parameter_tolerance = 1e-8
    o.min_relative_decrease = 1e-3
    o.min_lm_diagonal = 1e-6
    o.max_lm_diagonal = 1e32
    o.linear_solver = MBA_LINEAR_SOLVER_PCG
    o.max_linear_iterations = 100
    o.linear_tolerance = 1e-6
    o.precision = MBA_PRECISION_FP64
    o.preconditioner = MBA_PRECOND_BLOCK_JACOBI
    o.use_cuda_graph = 1
    o.check_tolerances = 1
    o.stop_cost = 0.0
    o.reject_outliers_every_n_iters = 3
    o.outlier_use_reprojection_error = 0
    o.outlier_max_reprojection_error_px = 50.0
    return o


def make_summary(capacity=64):
    s = Summary()
    its = (IterationSummary * capacity)()
    s.max_iterations_capacity = capacity
    s.iterations = ctypes.cast(its, ctypes.POINTER(IterationSummary))
    s._its = its  # keep alive
    return s


def calibration_dict(cams, mis):
    """Per-camera and per-mission blocks as arrays: intrinsics [N_cam][4],
    distortion [N_cam][4], q_CI [N_cam][4], p_CI [N_cam][3], baseframes
    [N_mis][7]."""
    return {"intrinsics": np.array([list(c.intrinsics) for c in cams]).reshape(-1, 4),
            "distortion": np.array([list(c.distortion) for c in cams]).reshape(-1, 4),
            "q_CI": np.array([list(c.q_CI_p_CI)[:4] for c in cams]).reshape(-1, 4),
            "p_CI": np.array([list(c.q_CI_p_CI)[4:] for c in cams]).reshape(-1, 3),
            "baseframes": np.asarray(mis, dtype=np.float64).reshape(-1, 7)}


def summary_dict(s):
    n = min(s.num_iterations, s.max_iterations_capacity)
    its = []
    for i in range(n):
        it = s.iterations[i]
        its.append({"iteration": it.iteration, "ok": bool(it.step_is_successful), "cost": it.cost,
                    "lin_iters": it.linear_solver_iterations, "radius": it.trust_region_radius,
                    "relative_decrease": it.relative_decrease, "time_ms": it.iteration_time_ms,
                    "cost_change": it.cost_change, "step_norm": it.step_norm})
    return {"num_iterations": s.num_iterations, "successful": s.num_successful_steps,
            "termination": s.termination, "linear_iterations": s.total_linear_iterations,
            "initial_cost": s.initial_cost, "final_cost": s.final_cost, "total_time_ms": s.total_time_ms,
            "time_to_stop_cost_ms": s.time_to_stop_cost_ms, "rejected_landmarks": s.num_rejected_landmarks,
            "iterations": its}
