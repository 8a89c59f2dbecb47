/*
 * maplab_ba_synth.h — seeded synthetic visual-inertial maps (host library
 * libmba_synth.so, no CUDA).
 *
 * Restates the recipe of maplab's test map generator
 * (test/vi-map-generator-6dof/src/6dof-test-trajectory-gen.cc:32-215,
 * src/6dof-pose-graph-gen.cc:33-60 and 205-399, src/6dof-vi-map-gen.cc:22-161):
 * a circular trajectory with roll/pitch/height excitation, 200 Hz IMU with
 * discrete white noise sigma/sqrt(dt) and bias random walks sigma*sqrt(dt)
 * drawn from std::mt19937 + std::normal_distribution, landmarks stored in
 * their first observer's IMU frame, pixel noise N(0, sigma^2), and initial
 * poses/landmarks perturbed by normal noise (first keyframe of each mission
 * left at ground truth as the gauge).  Gravity magnitude follows
 * common::GravityProvider (common/maplab-common/src/gravity-provider.cc).
 * The mission-cluster gauge fixes restate vi-optimization-builder.cc:243-371
 * and optimization-problem.cc:19-75.
 */
#ifndef MAPLAB_BA_SYNTH_H_
#define MAPLAB_BA_SYNTH_H_

#include "maplab_ba.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { MBA_SYNTH_LANDMARKS_BOX = 0, MBA_SYNTH_LANDMARKS_FRUSTUM = 1 };
enum { MBA_SYNTH_TRACK_UNIFORM = 0, MBA_SYNTH_TRACK_GEOMETRIC = 1, MBA_SYNTH_TRACK_POWER_LAW = 2 };

typedef struct mba_synth_config {
  uint64_t seed;
  int32_t num_missions;
  int32_t keyframes_per_mission;  /* used when kf_min == 0 */
  int32_t kf_min, kf_max;         /* > 0: keyframes per mission log-uniform in [kf_min, kf_max] */
  int32_t landmarks_per_keyframe; /* > 0: landmarks = this * keyframes, else num_landmarks */
  int64_t num_landmarks;
  int32_t landmark_mode;          /* MBA_SYNTH_LANDMARKS_* */
  int32_t track_model;            /* MBA_SYNTH_TRACK_* */
  int32_t track_min, track_max;   /* uniform bounds; power law: [max(2, track_min), cap]; geometric: [2, cap] */
  double track_mean;              /* geometric mean */
  double track_alpha;             /* power-law exponent */
  int32_t num_cameras;            /* 1 or 2 */
  int32_t camera_per_mission;     /* 1: mission m uses camera m % num_cameras */
  int32_t camera0_distortion;     /* MBA_DISTORTION_* of camera 0 */
  int32_t camera1_distortion;     /* MBA_DISTORTION_* of camera 1 */
  double radius_m;                /* circle radius (20) */
  double box_half_xy, box_half_z; /* landmark box (15, 2.5) for MBA_SYNTH_LANDMARKS_BOX */
  double keyframes_per_lap;       /* 100 */
  double kf_rate_hz, imu_rate_hz; /* 10, 200 */
  double pixel_sigma;             /* 1 px */
  double acc_noise, gyro_noise, acc_bias_rw, gyro_bias_rw;
  double rot_perturb, pos_perturb, lm_perturb, vel_perturb;
  double shared_landmark_fraction;/* co-registered missions: fraction of landmarks seen by two missions */
  int32_t include_inertial;
  int32_t co_registered;          /* missions share one circle (overlapping trajectories) */
  int32_t pose_edges;             /* 1: odometry edge between consecutive keyframes of a mission */
  int32_t pad_;
  double pose_edge_sigma_p;       /* odometry position noise (m) */
  double pose_edge_sigma_q;       /* odometry rotation noise (rad) */
  /* > 0: a loop closure every this many keyframes, to the keyframe one lap
   * later in the same mission and to the same-index keyframe of the next
   * mission. */
  int32_t loop_closure_stride;
  int32_t absolute_pose_stride;   /* > 0: an absolute 6-DoF measurement every this many keyframes */
  double loop_closure_sigma_p, loop_closure_sigma_q;
  double loop_closure_outlier_fraction; /* loop closures replaced by a wrong transform (0.5 rad, 3 m noise) */
  double loop_closure_switch_variance;  /* > 0: switchable loop closures; 0: switch held at 1 */
  double absolute_pose_sigma_p, absolute_pose_sigma_q;
} mba_synth_config;

typedef struct mba_synth_map mba_synth_map;

/* Fills cfg with the 100-keyframe single-mission defaults. */
void mba_synth_default_config(mba_synth_config* cfg);

/* Generates a map; returns MBA_OK or MBA_ERR_INVALID_ARG. */
mba_status mba_synth_generate(const mba_synth_config* cfg, mba_synth_map** out);

void mba_synth_free(mba_synth_map* map);

/* Points desc at the map's arrays (valid until mba_synth_free). */
mba_status mba_synth_describe(const mba_synth_map* map, mba_problem_desc* desc);

/* Ground-truth state (any pointer may be NULL); shapes as in mba_problem_desc. */
mba_status mba_synth_ground_truth(const mba_synth_map* map, double* kf_q_IM_p_MI, double* kf_v_M,
                                  double* kf_b_g, double* kf_b_a, double* lm_p_B);

#ifdef __cplusplus
}
#endif

#endif /* MAPLAB_BA_SYNTH_H_ */
