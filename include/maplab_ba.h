/*
 * maplab_ba.h — C ABI of the GB300 visual-inertial bundle-adjustment back-end.
 *
 * Plain C types only (no Eigen, no Ceres, no torch).  All arrays are
 * structure-of-arrays, row-major, FP64 unless stated.  Quaternions are stored
 * xyzw and interpreted as JPL (passive), exactly like maplab's
 * OptimizationStateBuffer.  Poses are 7-vectors [q_xyzw, p].
 *
 * The entry points replace three reference interfaces:
 *   1. map_optimization::VIMapOptimizer::optimize
 *        algorithms/map-optimization/include/map-optimization/vi-map-optimizer.h:21-39
 *        algorithms/map-optimization/src/vi-map-optimizer.cc:34-78
 *      and map_optimization::solve (src/solver.cc:14-44)      -> mba_create + mba_solve
 *   2. ceres::CostFunction::Evaluate of VisualReprojectionError and
 *      InertialErrorTerm
 *        algorithms/ceres-error-terms/include/ceres-error-terms/visual-error-term-inl.h:12-379
 *        algorithms/ceres-error-terms/src/inertial-error-term.cc:77-286
 *                                         -> mba_evaluate_visual / mba_evaluate_inertial
 *   3. ceres_error_terms::ProblemInformation + OptimizationStateBuffer
 *        algorithms/ceres-error-terms/include/ceres-error-terms/problem-information.h:18-140
 *        algorithms/map-optimization/src/optimization-state-buffer.cc:42-264
 *                                         -> mba_problem_desc, mba_read_state / mba_write_state
 *
 * Errors are returned as mba_status codes; no entry point aborts the process.
 * One handle per host thread; every handle owns one CUDA stream.
 */
#ifndef MAPLAB_BA_H_
#define MAPLAB_BA_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MBA_ABI_VERSION 2

typedef enum mba_status {
  MBA_OK = 0,
  MBA_ERR_INVALID_ARG = 1,
  MBA_ERR_OUT_OF_RANGE_INDEX = 2,
  MBA_ERR_NON_FINITE = 3,
  MBA_ERR_NOT_SPD = 4,
  MBA_ERR_CUDA = 5,
  MBA_ERR_TIMEOUT = 6,
  MBA_ERR_CANCELLED = 7,
  MBA_ERR_NO_DEVICE = 8,
  MBA_ERR_UNORDERED_IMU = 9
} mba_status;

/* ceres_error_terms::LandmarkErrorType (ceres-error-terms/common.h:14). */
enum { MBA_LOCAL_KEYFRAME = 0, MBA_LOCAL_MISSION = 1, MBA_GLOBAL = 2 };

/* aslam::Distortion::Type subset: pinhole + {none, radtan, equidistant,
 * fisheye}.  MBA_DISTORTION_FOV is aslam's FisheyeDistortion (the
 * field-of-view model, aslam_cv_cameras/src/distortion-fisheye.cc) with its
 * one parameter w in distortion[0]; w^2 < 1e-5 is the identity map. */
enum { MBA_DISTORTION_NONE = 0, MBA_DISTORTION_RADTAN = 1, MBA_DISTORTION_EQUIDISTANT = 2, MBA_DISTORTION_FOV = 3 };

/* Camera calibration blocks left free in the solve (camera_flags).  maplab's
 * builder sets the intrinsics and distortion blocks constant unless
 * ba_fix_ncamera_intrinsics = false, and q_C_I / p_C_I unless
 * ba_fix_ncamera_extrinsics_rotation / _translation = false
 * (vi-optimization-builder.cc:24-35, optimization-terms-addition.cc:
 * 203-234); the cost-term tests free each block on its own.  Intrinsics and
 * distortion are plain additive blocks, q_C_I uses JplQuaternion-
 * Parameterization. */
enum {
  MBA_CAM_INTRINSICS_FREE = 1u << 0,
  MBA_CAM_DISTORTION_FREE = 1u << 1,
  MBA_CAM_ROTATION_FREE = 1u << 2,
  MBA_CAM_TRANSLATION_FREE = 1u << 3
};
/* Mission baseframe T_G_M left free (mission_flags).  maplab fixes all
 * baseframes (fixAllBaseframesInProblem) unless absolute 6-DoF terms are in
 * the problem and fix_baseframes is off (vi-optimization-builder.cc:
 * 366-371); it then uses JplYawOnlyPoseParameterization (yaw + position,
 * optimization-problem.cc:90-91).  The mission-baseframe tests use
 * JplPoseParameterization (6 dof).  A free baseframe enters the kGlobal
 * visual terms; problems that also have absolute 6-DoF or cross-mission
 * loop-closure terms must keep their baseframes constant. */
enum { MBA_MIS_BASEFRAME_YAW_POSITION = 1u << 0, MBA_MIS_BASEFRAME_POSE = 1u << 1 };

/* Per-keyframe fix flags (kf_flags).  They restate the Ceres parameter-block
 * constness and local parameterizations chosen by the problem builder:
 * ba_fix_vertices / ba_fix_velocity / ba_fix_gyro_bias / ba_fix_accel_bias
 * (map-optimization/src/vi-optimization-builder.cc:36-47) and the gauge fix of
 * the first vertex of a mission cluster (src/optimization-problem.cc:19-75). */
enum {
  MBA_KF_POSE_CONSTANT = 1u << 0,       /* whole 7-dof pose block constant */
  MBA_KF_GAUGE_ROLL_PITCH = 1u << 1,    /* JplRollPitchQuaternionParameterization + position fixed */
  MBA_KF_VELOCITY_CONSTANT = 1u << 2,
  MBA_KF_GYRO_BIAS_CONSTANT = 1u << 3,
  MBA_KF_ACCEL_BIAS_CONSTANT = 1u << 4,
  MBA_KF_POSITION_CONSTANT = 1u << 5,   /* SubsetParameterization(3,{0,1,2}) on the position */
  MBA_KF_ROTATION_CONSTANT = 1u << 6    /* FixedRotationDoF::kAll: rotation constant */
};

typedef struct mba_camera {
  double intrinsics[4];   /* fu, fv, cu, cv */
  double distortion[4];   /* radtan: k1 k2 p1 p2; equidistant: k1 k2 k3 k4 */
  int32_t distortion_type;/* MBA_DISTORTION_* */
  int32_t width, height;  /* image size in pixels (isKeypointVisible) */
  int32_t pad_;
  double q_CI_p_CI[7];    /* extrinsics: JPL q_C_I, then p_C_I */
} mba_camera;

typedef struct mba_problem_desc {
  int64_t num_keyframes;
  int64_t num_landmarks;
  int64_t num_observations;
  int64_t num_cameras;
  int64_t num_missions;
  int64_t num_imu_edges;      /* 0 => purely visual problem */
  int64_t num_imu_samples;    /* total samples over all edges */

  /* Visual observations (one VisualReprojectionError each). */
  const double* obs_uv;       /* [N_obs][2] distorted keypoint measurement */
  const double* obs_sigma;    /* [N_obs] keypoint uncertainty in px (> 0) */
  const int32_t* obs_landmark;/* [N_obs] */
  const int32_t* obs_keyframe;/* [N_obs] observer vertex */
  const int32_t* obs_camera;  /* [N_obs] */

  /* Landmarks: p_B expressed in the IMU frame of their store vertex. */
  const double* lm_p_B;             /* [N_lm][3] */
  const int32_t* lm_store_keyframe; /* [N_lm] */
  const uint8_t* lm_constant;       /* [N_lm] or NULL (ba_fix_landmark_positions) */

  /* Keyframes (vertices). */
  const double* kf_q_IM_p_MI; /* [N_kf][7] */
  const double* kf_v_M;       /* [N_kf][3] */
  const double* kf_b_g;       /* [N_kf][3] */
  const double* kf_b_a;       /* [N_kf][3] */
  const int32_t* kf_mission;  /* [N_kf] */
  const uint32_t* kf_flags;   /* [N_kf] MBA_KF_* bits, or NULL */

  /* Missions: baseframe pose q_G_M (JPL) | p_G_M; always constant here. */
  const double* mission_q_GM_p_GM; /* [N_mis][7] */

  const mba_camera* cameras;  /* [N_cam]; intrinsics/extrinsics constant */

  /* Inertial edges (one InertialErrorTerm each). Samples of edge e are
   * imu_*[edge_sample_offset[e] .. edge_sample_offset[e+1]). */
  const int32_t* edge_from;          /* [N_e] */
  const int32_t* edge_to;            /* [N_e] */
  const int64_t* edge_sample_offset; /* [N_e + 1] */
  const int64_t* imu_timestamp_ns;   /* [N_s] */
  const double* imu_acc_gyro;        /* [N_s][6]: acc xyz, gyro xyz */
  double gyro_noise_sigma, gyro_bias_sigma, acc_noise_sigma, acc_bias_sigma;
  double gravity_magnitude;

  /* Robust loss on visual terms (optimization-terms-addition.cc:189-198):
   * HuberLoss(delta * sigma) with delta = 3 (local) or 10 (global).
   * use_huber = 0 disables the loss (plain least squares). */
  int32_t use_huber;
  int32_t pad_;
  double huber_delta_local;
  double huber_delta_global;
  /* Pose-graph terms ("pose edges"), no loss, sensor extrinsics and mission
   * baseframes constant.  Kind per edge (pose_edge_type):
   *  MBA_POSE_EDGE_RELATIVE: odometry / wheel-odometry TransformationEdge
   *    (addRelativePoseTermsForEdges, optimization-terms-addition.cc:543-640),
   *    SixDoFBlockPoseErrorTermWithExtrinsics; measurement T_Bk_Bkp1,
   *    extrinsics q_I_B | p_B_I, covariance get_T_A_B_Covariance_p_q.
   *  MBA_POSE_EDGE_LOOP_CLOSURE: LoopClosureEdge (augment-loopclosure.cc:
   *    10-164), LoopClosureEdgeErrorTerm times a switch variable in [0, 1];
   *    measurement T_A_B, covariance get_T_A_B_Covariance; extrinsics unused.
   *    With a switch variance > 0 the switch is a variable with
   *    SwitchPriorErrorTerm(1, variance) and bounds [0, 1]; with 0 it is held
   *    at its given value.
   *  MBA_POSE_EDGE_ABSOLUTE: Absolute6DoFMeasurement of keyframe `from`
   *    (addAbsolutePoseConstraintTermsForVertices, :650-738),
   *    BlockPosePriorErrorTermV2 with the keyframe mission's baseframe;
   *    measurement T_G_S, covariance get_T_G_S_covariance, extrinsics the
   *    sensor block q_S_B | p_S_B (JPL); pose_edge_to ignored.
   * Measurements are aslam::Transformation values: q (x y z w, Hamilton) | p. */
  int64_t num_pose_edges;
  const int32_t* pose_edge_from;       /* [N_pe] keyframe A (T_Bk, the vertex of an absolute term) */
  const int32_t* pose_edge_to;         /* [N_pe] keyframe B (T_Bkp1) */
  const double* pose_edge_T_Bk_Bkp1;   /* [N_pe][7] measurement q (x y z w) | p */
  const double* pose_edge_covariance;  /* [N_pe][36] row-major, residual order (p, q) */
  const double* pose_edge_q_I_B_p_B_I; /* [N_pe][7] extrinsics block (see above) */
  const int32_t* pose_edge_type;       /* [N_pe] MBA_POSE_EDGE_*; NULL = all RELATIVE */
  const double* pose_edge_switch;      /* [N_pe] initial switch of a loop closure; NULL = 1 */
  const double* pose_edge_switch_variance; /* [N_pe] switch prior variance; NULL = all 0 */
  /* Calibration and baseframes as variables (NULL = all constant, maplab's
   * defaults).  FP64 solves only: a mixed-precision solve of a problem with
   * a free block returns MBA_ERR_INVALID_ARG. */
  const uint32_t* camera_flags;  /* [N_cam] MBA_CAM_* bits */
  const uint32_t* mission_flags; /* [N_mis] MBA_MIS_BASEFRAME_* (at most one bit) */
} mba_problem_desc;

enum { MBA_POSE_EDGE_RELATIVE = 0, MBA_POSE_EDGE_LOOP_CLOSURE = 1, MBA_POSE_EDGE_ABSOLUTE = 2 };

/* Subset of ceres::Solver::Options used by map_optimization
 * (include/map-optimization/solver-options.h:26-75), same names and defaults
 * as the ba_* gflags (src/solver-options.cc:3-52). */
enum { MBA_LINEAR_SOLVER_PCG = 0, MBA_LINEAR_SOLVER_DENSE_SCHUR = 1 };
/* Preconditioners of the reduced camera system's PCG: block-Jacobi (15x15
 * keyframe blocks, the plain method); CHAIN: block-Jacobi corrected by the
 * couplings between consecutive keyframes of each trajectory (a
 * block-tridiagonal matrix solved by cyclic reduction, fixed coefficients);
 * LEARNED: the same correction with coefficients predicted per keyframe by a
 * graph network over the co-visibility graph.  CHAIN and LEARNED fall back to
 * block-Jacobi for any LM iteration whose correction is not positive definite. */
enum { MBA_PRECOND_BLOCK_JACOBI = 0, MBA_PRECOND_LEARNED = 1, MBA_PRECOND_CHAIN = 2 };
enum { MBA_PRECISION_FP64 = 0, MBA_PRECISION_MIXED = 1 };

typedef struct mba_solver_options {
  int32_t max_num_iterations;          /* ba_num_iterations = 30 */
  int32_t jacobi_scaling;              /* ba_use_jacobi_scaling = 1 */
  double initial_trust_region_radius;  /* 1e5 */
  double max_trust_region_radius;      /* 1e20 */
  double min_trust_region_radius;      /* 1e-32 */
  double function_tolerance;           /* 1e-12 */
  double gradient_tolerance;           /* 1e-10 */
  double parameter_tolerance;          /* 1e-8 */
  double min_relative_decrease;        /* 1e-3 (Ceres default) */
  double min_lm_diagonal;              /* 1e-6 (Ceres default) */
  double max_lm_diagonal;              /* 1e32 (Ceres default) */
  int32_t linear_solver;               /* MBA_LINEAR_SOLVER_* */
  int32_t max_linear_iterations;       /* PCG cap (100) */
  double linear_tolerance;             /* PCG relative residual tolerance (1e-6) */
  int32_t precision;                   /* MBA_PRECISION_* */
  int32_t preconditioner;              /* MBA_PRECOND_* */
  int32_t use_cuda_graph;              /* capture each LM iteration as a graph */
  int32_t check_tolerances;            /* 1: stop on function/gradient/parameter tolerance */
  double stop_cost;                    /* >0: stop as soon as cost <= stop_cost */
  /* Outlier-landmark rejection (outlier-rejection-solver.cc): every n
   * iterations the solve restarts after removing the landmarks seen at depth
   * <= 0 (or, optionally, with a reprojection error above the threshold).
   * ba_use_visual_outlier_rejection_solver = true, n = 3; 0 disables. */
  int32_t reject_outliers_every_n_iters;     /* ba_outlier_rejection_reject_every_n_iters = 3 */
  int32_t outlier_use_reprojection_error;    /* ba_outlier_rejection_use_reprojection_error = 0 */
  double outlier_max_reprojection_error_px;  /* ba_outlier_rejection_max_reprojection_error_px = 50 */
} mba_solver_options;

/* Mirrors the columns of ceres::IterationSummary printed by maplab's
 * OutlierRejectionCallback (outlier-rejection-solver.h:29-68). */
typedef struct mba_iteration_summary {
  int32_t iteration;
  int32_t step_is_successful;
  int32_t linear_solver_iterations;
  int32_t pad_;
  double cost;
  double cost_change;
  double gradient_max_norm;
  double step_norm;
  double relative_decrease;
  double trust_region_radius;
  double iteration_time_ms;
} mba_iteration_summary;

typedef struct mba_summary {
  int32_t num_iterations;         /* entries written to `iterations` */
  int32_t num_successful_steps;
  int32_t termination;            /* 0 max iterations, 1 function tol, 2 gradient tol,
                                     3 parameter tol, 4 min radius, 5 cancelled, 6 stop_cost */
  int32_t total_linear_iterations;
  double initial_cost;
  double final_cost;
  double total_time_ms;
  double time_to_stop_cost_ms;    /* -1 if stop_cost was not reached */
  int32_t max_iterations_capacity;/* caller sets: length of `iterations` */
  int32_t num_rejected_landmarks; /* outlier landmarks removed during this solve */
  mba_iteration_summary* iterations; /* caller-owned, may be NULL */
} mba_summary;

typedef struct mba_handle mba_handle;

/* Library / ABI version (MBA_ABI_VERSION). */
int32_t mba_abi_version(void);

/* Fills opts with the maplab ba_* flag defaults (solver-options.cc:3-52). */
void mba_default_solver_options(mba_solver_options* opts);

/* Text for a status code. */
const char* mba_status_string(mba_status s);

/* Validates the descriptor (indices in range, sigmas > 0, quaternions unit
 * within 1e-5 like assertValidQuaternion, IMU timestamps ordered), copies all
 * arrays to device memory and builds the Schur pattern.  Caller arrays are not
 * retained.  Replaces constructOptimizationProblem + OptimizationStateBuffer::
 * importStatesOfMissions (vi-optimization-builder.cc:154-374,
 * optimization-state-buffer.cc:153-264). */
mba_status mba_create(const mba_problem_desc* desc, int32_t device, mba_handle** out);

void mba_destroy(mba_handle* h);

/* Batched ceres::CostFunction::Evaluate of every VisualReprojectionError at the
 * current state (visual-error-term-inl.h:12-379).  residuals: [N_obs][2] or
 * NULL.  jacobians: NULL or an array of 9 pointers (landmark p [N][2x3],
 * landmark-base pose [N][2x7], landmark-mission baseframe [N][2x7],
 * observer-mission baseframe [N][2x7], observer pose [N][2x7], q_C_I [N][2x4],
 * p_C_I [N][2x3], intrinsics [N][2x4], distortion [N][2x4]), each NULL to
 * skip, in the ambient row-major layout Ceres receives.  Host pointers.  The
 * raw (un-robustified) residual is returned, as Evaluate does. */
mba_status mba_evaluate_visual(mba_handle* h, double* residuals, double* const* jacobians);

/* Batched InertialErrorTerm::Evaluate (inertial-error-term.cc:77-286).
 * residuals: [N_e][15] or NULL; jacobians: NULL or 8 pointers (pose_from
 * [N][15x7], b_g_from [N][15x3], v_from, b_a_from, pose_to, b_g_to, v_to,
 * b_a_to), each NULL to skip.  Host pointers. */
mba_status mba_evaluate_inertial(mba_handle* h, double* residuals, double* const* jacobians);

/* Tangent-space (post local-parameterization) Jacobians the solver uses, with
 * the Huber correction applied, for parity tests of the solver path.
 * precision MBA_PRECISION_FP64 or MBA_PRECISION_MIXED (FP32 Jacobians).
 * Outputs (host, FP64, may be NULL): r [N][2], J_landmark [N][2x3],
 * J_store [N][2x6], J_observer [N][2x6]. */
mba_status mba_linearize_visual(mba_handle* h, int32_t precision, double* r,
                                double* J_landmark, double* J_store, double* J_observer);

/* Pose edges at the current state: whitened residual [N_pe][6] (times the
 * switch for loop closures) and tangent Jacobians [N_pe][6x6] w.r.t. the
 * (theta, p) tangent of the from / to keyframe (Ceres: autodiff ambient
 * Jacobian times the JPL pose parameterization's ComputeJacobian; J_to is
 * zero for absolute terms).  Host pointers, each may be NULL. */
mba_status mba_linearize_pose_edges(mba_handle* h, double* r, double* J_from, double* J_to);

/* Switch variables of the pose edges [N_pe] (1 for edges without one).
 * Writing clamps nothing: values must lie in [0, 1]. */
mba_status mba_read_switch_variables(mba_handle* h, double* s);
mba_status mba_write_switch_variables(mba_handle* h, const double* s);

/* Ceres-style total cost 0.5 * sum rho(|r|^2) at the current state. */
mba_status mba_cost(mba_handle* h, int32_t precision, double* cost);

/* Runs Levenberg-Marquardt on the device (ceres::Solve with the options of
 * solver-options.h:26-75).  The state stays on the device; read it back with
 * mba_read_state.  summary may be NULL.
 * MBA_ERR_TIMEOUT means a bounded device wait ran out (the learned
 * preconditioner's tensor-core pipeline): copies or MMAs it guarded may still
 * have been in flight, so the device state is undefined.  The handle is then
 * poisoned: later mba_solve, mba_gnn_train and mba_gnn_gradient calls on it
 * return MBA_ERR_TIMEOUT without launching anything, and the caller should
 * destroy its handles and treat the CUDA context as unusable. */
mba_status mba_solve(mba_handle* h, const mba_solver_options* opts, mba_summary* summary);

/* OptimizationStateBuffer analogue: copy the optimized state out / in.
 * Any pointer may be NULL.  Shapes as in mba_problem_desc. */
mba_status mba_read_state(mba_handle* h, double* kf_q_IM_p_MI, double* kf_v_M,
                          double* kf_b_g, double* kf_b_a, double* lm_p_B);
mba_status mba_write_state(mba_handle* h, const double* kf_q_IM_p_MI, const double* kf_v_M,
                           const double* kf_b_g, const double* kf_b_a, const double* lm_p_B);

/* Camera calibration and mission baseframes of the handle's current state
 * (the blocks that mba_problem_desc's camera_flags / mission_flags leave
 * free move during a solve): cameras [N_cam] (every field copied) and
 * mission_q_GM_p_GM [N_mis][7].  Either pointer may be NULL.  Writing sets
 * the intrinsics, distortion parameters, q_C_I | p_C_I and baseframes;
 * quaternions must be unit within 1e-5 and distortion types and image sizes
 * must match the descriptor's.  The OptimizationStateBuffer analogue for the
 * sensor and baseframe blocks (optimization-state-buffer.cc:42-152). */
mba_status mba_read_calibration(mba_handle* h, mba_camera* cameras, double* mission_q_GM_p_GM);
mba_status mba_write_calibration(mba_handle* h, const mba_camera* cameras, const double* mission_q_GM_p_GM);

/* Thread-safe request to stop after the current LM iteration (the SIGINT
 * handler of ceres-error-terms/src/ceres-signal-handler.cc:12-56). */
void mba_cancel(mba_handle* h);

/* Timing of the visual evaluation kernel alone over `iters` launches with
 * the inputs resident on the device (CUDA events on the handle's stream).
 * mode 0: FP64 tangent linearization, 1: FP32 tangent linearization.
 * Writes the mean milliseconds per launch. */
mba_status mba_time_visual_kernel(mba_handle* h, int32_t mode, int32_t iters, double* ms_per_launch);

/* Measured FP64 arithmetic rate of `device` in TFLOP/s (one FMA = 2 FLOPs):
 * independent FMA chains on every SM, timed with CUDA events.  The
 * denominator of the FP64 evaluation kernel's roofline; no counterpart in
 * the reference (a measurement aid). */
mba_status mba_measure_fp64_peak(int32_t device, double* tflops);

/* The damped reduced camera system of the current state, as one LM iteration
 * builds it (the matrix Ceres's SchurEliminator forms internally for
 * SPARSE_SCHUR / ITERATIVE_SCHUR, linear_solver/schur_eliminator.h; maplab has
 * no interface to it, so this entry point has no reference counterpart).
 * Jacobi-scaled like the solver's system, LM-damped with trust-region radius
 * `radius`, fixed tangent dims as identity rows with zero right-hand side.
 * Keyframe blocks are 15x15 in the order (theta, p, v, b_g, b_a).
 * Host outputs, FP64, each may be NULL:
 *   diag [N_kf][15][15];
 *   upper_ij [N_pu][2] keyframe pairs (i < j) and upper [N_pu][6][6], the
 *     pose-pose (theta, p) block of row i, column j,
 *     N_pu = mba_problem_stats.num_schur_pose_blocks / 2;
 *   inertial [N_edge][15][15] (IMU edges, then pose edges), row = edge's
 *   from keyframe, column = to;
 *   rhs [N_kf][15].
 * precision MBA_PRECISION_FP64 or MBA_PRECISION_MIXED (FP32 system). */
mba_status mba_reduced_system(mba_handle* h, int32_t precision, double radius, double* diag, int32_t* upper_ij,
                              double* upper, double* inertial, double* rhs);

/* Landmarks rejected as outliers by the solves run on this handle so far
 * (Landmark::Quality::kBad in maplab): flags [N_lm] (1 = rejected, may be
 * NULL) and their count.  Rejected landmarks stay out of later solves. */
mba_status mba_rejected_landmarks(mba_handle* h, uint8_t* flags, int64_t* count);

/* ---- Learned preconditioner (no reference counterpart: maplab's Ceres path
 * uses SCHUR_JACOBI).  A 3-layer message-passing network (hidden 64, BF16
 * weights, FP32 accumulation) over the co-visibility graph of the reduced
 * camera system predicts, per keyframe, the coefficients of the chain
 * correction to block-Jacobi (MBA_PRECOND_LEARNED).  The model is trained on
 * the device on reduced systems this library builds. */
typedef struct mba_gnn mba_gnn;
int64_t mba_gnn_num_parameters(void);
/* Randomly initialised model on `device` (head biased towards the plain chain). */
mba_status mba_gnn_create(int32_t device, uint64_t seed, mba_gnn** out);
void mba_gnn_destroy(mba_gnn* m);
/* FP32 master parameters [mba_gnn_num_parameters()]; set resets the optimizer. */
mba_status mba_gnn_get_parameters(mba_gnn* m, float* params);
mba_status mba_gnn_set_parameters(mba_gnn* m, const float* params);
/* Model used by MBA_PRECOND_LEARNED solves on this handle (NULL detaches; the
 * caller keeps ownership).  Solves asking for LEARNED without a model fail
 * with MBA_ERR_INVALID_ARG. */
mba_status mba_set_preconditioner_model(mba_handle* h, mba_gnn* m);
/* Training on the reduced system of the handle's current state (FP32 system,
 * LM radius `radius`): `steps` Adam steps (learning rate lr) on the probe
 * loss mean |T^-1 S w - w|^2 over nprobe normal probes w (T: the chain matrix
 * with the model's coefficients).  losses [steps] receives the loss before
 * each step (may be NULL). */
mba_status mba_gnn_train(mba_handle* h, mba_gnn* m, double radius, int32_t nprobe, int32_t steps, float lr,
                         uint64_t seed, double* losses);
/* Loss and its gradient for given probes (host [nprobe][15 N_kf], or seeded
 * draws if NULL) without updating the model: grad [num_parameters], loss,
 * coef [N_kf][3] per chain position (gamma_ine, gamma_vis, alpha).  For
 * gradient checks. */
mba_status mba_gnn_gradient(mba_handle* h, mba_gnn* m, double radius, int32_t nprobe, const float* probes,
                            uint64_t seed, float* grad, double* loss, double* coef);
/* Keyframe chain order used by the chain preconditioner: perm [N_kf] chain
 * position -> keyframe; link_edge [N_kf] inertial edge coupling position p to
 * p - 1 (-1: none); link_blk [N_kf] index of the (kf(p), kf(p-1)) pose block
 * among the 2 N_pu oriented blocks (upper j < N_pu, else the transpose of
 * upper j - N_pu; -1: none).  Any pointer may be NULL. */
mba_status mba_chain_structure(mba_handle* h, int32_t* perm, int32_t* link_edge, int32_t* link_blk);
/* z = T^-1 r for the exact chain matrix T (gamma = 1, alpha = 0) of the
 * reduced system at the current state (built as mba_reduced_system does, with
 * trust-region radius `radius`), through the handle's chain sweeps.  r and z
 * [N_kf][15] in keyframe order, host memory.  MBA_ERR_NOT_SPD if a pivot of
 * the factorization failed.  For checking the sweeps. */
mba_status mba_chain_apply(mba_handle* h, int32_t precision, double radius, const double* r, double* z);

/* Launch and schedule parameters of one problem (no reference counterpart).
 * mba_autotune times each candidate on the handle's own data with CUDA
 * events and keeps the fastest; later solves on the handle use them. */
typedef struct mba_tuning {
  int32_t visual_block;         /* threads per block of the evaluation kernel (64, 128, 256) */
  int32_t schur_chunk;          /* slot pairs summed per thread by the Schur pair kernel */
  int32_t chain_tail_nodes;     /* chain positions below which one block finishes a chain sweep */
  int32_t visual_min_blocks;    /* register cap of the evaluation kernel: blocks of 256 per SM (1 = none;
                                 * one thread per observation: 1, 3 or 4; pipelined: 1 or 2) */
  double visual_ms;             /* per launch, chosen setting */
  double schur_ms;
  double chain_apply_ms;
  int32_t visual_pipelined;     /* 1: software-pipelined persistent evaluation kernel, 2: one thread per
                                 * observation (0 in mba_set_tuning keeps the current setting) */
  int32_t chain_segment;        /* chain sweeps: positions one block takes through the lower levels (a power
                                 * of two from 2 to 256; three launches per apply), or 1: one launch per
                                 * level (0 in mba_set_tuning keeps the current setting) */
  int32_t chain_tail_smem;      /* 1: the one-block tail keeps the survivors' vectors in shared memory,
                                 * 2: in global memory (0 in mba_set_tuning keeps the current setting) */
  int32_t pcg_product;          /* PCG product: 1 reads each stored pose block once (transposed part by
                                 * atomics), 2 reads it from both of its rows (0 keeps the setting) */
  int32_t schur_split;          /* Schur pair kernel: 1 two threads per chunk (half the output columns
                                 * each), 2 one thread per chunk (0 keeps the setting) */
  int32_t pad_;
} mba_tuning;
mba_status mba_autotune(mba_handle* h, int32_t precision, mba_tuning* out);
/* Applies tuning values (e.g. cached from an earlier mba_autotune of a
 * problem of the same shape); a field of 0 keeps the current setting. */
mba_status mba_set_tuning(mba_handle* h, const mba_tuning* t);

/* Problem statistics (for reports): sizes of the reduced camera system. */
typedef struct mba_problem_stats {
  int64_t num_keyframes, num_landmarks, num_observations, num_imu_edges;
  int64_t num_schur_pose_blocks;   /* off-diagonal 6x6 pose-pose blocks (both triangles) */
  int64_t device_bytes;            /* bytes held on the device by the handle */
  int64_t num_pose_edges;          /* relative pose edges (after the IMU edges) */
} mba_problem_stats;
mba_status mba_get_stats(mba_handle* h, mba_problem_stats* stats);

/* Pose-graph relaxation (VIMapRelaxation::solveRelaxation,
 * vi-map-relaxation.cc:97-151): the same solve with velocities, biases and
 * landmark positions fixed (intrinsics and extrinsics are always fixed here)
 * and the loop-closure edges added.  Host only: fills kf_flags_out [N_kf]
 * with desc's flags plus the velocity / bias fixes and lm_constant_out [N_lm]
 * with 1; the caller points a copy of desc at them and solves with
 * mba_create / mba_solve as usual. */
mba_status mba_relaxation_flags(const mba_problem_desc* desc, uint32_t* kf_flags_out, uint8_t* lm_constant_out);

/* Gauge fixes of constructOptimizationProblem (vi-optimization-builder.cc:
 * 240-361, OptimizationProblem::applyGaugeFixesForInitialVertices,
 * optimization-problem.cc:19-176).  Missions are clustered by co-observed
 * landmarks and loop closures; per cluster the observability of scale,
 * global position, yaw and roll/pitch follows from the constraints every
 * mission of the cluster has (IMU edges, visual observations, odometry edges,
 * absolute 6-DoF terms), and the first keyframe in the problem of the
 * cluster's first mission gets the open degrees of freedom fixed: rotation
 * all (pose constant), yaw (roll/pitch parameterization), position; an
 * unobservable scale fixes the first landmark stored at that keyframe.
 * Host only: kf_flags_out [N_kf] = desc's flags plus the fixes,
 * lm_constant_out [N_lm] = desc's constants plus the fixes (either output may
 * be NULL); *num_clusters (may be NULL) receives the cluster count. */
mba_status mba_gauge_fixes(const mba_problem_desc* desc, uint32_t* kf_flags_out, uint8_t* lm_constant_out,
                           int32_t* num_clusters);

/* Landmark quality (isVisualLandmarkWellConstrained,
 * map-structure/vi-map/src/landmark-quality-metrics.cc:103-166), the filter
 * constructOptimizationProblem applies before adding a landmark's terms:
 * enough observers, closest observing camera (signed by the landmark's depth
 * in it) within a distance band, wide enough maximum disparity angle between
 * the incidence rays, optionally every reprojection error below a bound.
 * Evaluated on the device at the handle's current state; flags [N_lm], 1 =
 * well constrained.  The defaults are the elq_* gflags. */
typedef struct mba_landmark_quality_options {
  int32_t min_observers;                     /* elq_min_observers (4) */
  int32_t pad_;
  double min_observation_angle_deg;          /* elq_min_observation_angle_deg (5) */
  double max_distance_from_closest_observer; /* elq_max_distance_from_closest_observer (40 m) */
  double min_distance_from_closest_observer; /* elq_min_distance_from_closest_observer (0.05 m) */
  double max_reprojection_error_px;          /* elq_max_reprojection_error_px (-1: no test) */
} mba_landmark_quality_options;
void mba_default_landmark_quality_options(mba_landmark_quality_options* o);
mba_status mba_landmark_quality(mba_handle* h, const mba_landmark_quality_options* o, uint8_t* well_constrained);

/* Visual observations and the state they depend on, all in DEVICE memory
 * owned by the caller, laid out as in mba_problem_desc (state arrays in the
 * caller's layout: kf_q_IM_p_MI [N_kf][7], lm_p_B [N_lm][3], ...). */
typedef struct mba_visual_batch_device {
  int64_t num_observations;
  int64_t num_landmarks, num_keyframes, num_missions, num_cameras;
  const double* obs_uv;            /* [N_obs][2] */
  const double* obs_sigma;         /* [N_obs] */
  const int32_t* obs_landmark;     /* [N_obs] */
  const int32_t* obs_keyframe;     /* [N_obs] */
  const int32_t* obs_camera;       /* [N_obs] */
  const int32_t* lm_store_keyframe;/* [N_lm] */
  const double* lm_p_B;            /* [N_lm][3] */
  const double* kf_q_IM_p_MI;      /* [N_kf][7] */
  const int32_t* kf_mission;       /* [N_kf] */
  const double* mission_q_GM_p_GM; /* [N_mis][7] */
  const mba_camera* cameras;       /* [N_cam] */
  int32_t use_huber;
  int32_t pad_;
  double huber_delta_local, huber_delta_global;
} mba_visual_batch_device;

/* Robustified visual cost 0.5 * sum rho(|r|^2) of a batch, computed without
 * allocating any memory.  This entry point has no counterpart in the
 * reference; it serves callers that may not allocate device memory while
 * running: a real-time visual-inertial estimator thread must not block on the
 * device-wide synchronization of cudaMalloc/cudaFree or fail on an
 * out-of-memory error mid-mission, and an application whose device memory is
 * owned by another allocator's pool cannot have it fragmented by foreign
 * cudaMalloc calls.  The caller passes device pointers for every input and
 * for the output (*cost_out_device, one double).  Intermediates live in a
 * fixed 512 KiB file-scope device array that each GPU loading the library
 * keeps until the process exits; batches above 16,777,216 observations are
 * rejected with MBA_ERR_INVALID_ARG.  All calls share that array, so calls
 * that overlap on the GPU (other streams or threads) race; serialize them.
 * The first call on a device looks up the array's device address with that
 * device current; make that first call before any stream capture.  Runs on
 * `stream` (a cudaStream_t, NULL = legacy default stream); every call copies
 * two status flags to host memory and synchronizes `stream` before it
 * returns.  Out-of-range indices are skipped on the device and reported as
 * MBA_ERR_OUT_OF_RANGE_INDEX; non-finite costs as MBA_ERR_NON_FINITE (the
 * flags are cleared at the start of every call).  A CUDA error already
 * pending when the call starts is left in place and reported as
 * MBA_ERR_CUDA without a launch. */
mba_status mba_visual_cost_noalloc(const mba_visual_batch_device* batch, int32_t device, void* stream,
                                   double* cost_out_device);

/* The learned preconditioner's node update on the tensor cores
 * (tcgen05, TMA): Z = A W^T + A2 W2^T + bias, H = bf16(relu(Z)), for
 * kernel-level checks.  Host buffers: A, A2 [n][k] and W, W2 [64][k] as BF16
 * bit patterns (A2 / W2 may be NULL), bias [64] (may be NULL), Z [n][64],
 * H [n][64] BF16 bit patterns (may be NULL); k = 32 or 64.  No counterpart
 * in the reference (maplab preconditions with SCHUR_JACOBI). */
mba_status mba_gnn_gemm(int32_t device, int64_t n, int32_t k, const uint16_t* A, const uint16_t* W,
                        const uint16_t* A2, const uint16_t* W2, const float* bias, float* Z, uint16_t* H);

/* Failure detection without a fault: launches the tensor-core node update
 * with its operand copies left out, so that the kernel's bounded wait on the
 * load barrier runs out (a barrier nothing signals).  Returns MBA_ERR_TIMEOUT
 * when the kernel reported the timeout and the device stayed usable (a
 * following synchronize succeeds); MBA_OK would mean the timeout went
 * unreported. */
mba_status mba_gnn_gemm_wait_check(int32_t device);

#ifdef __cplusplus
}
#endif

#endif /* MAPLAB_BA_H_ */
