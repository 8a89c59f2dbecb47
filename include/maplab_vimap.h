/* VIMap map-folder reader, problem exporter and state write-back.
 *
 * Replaces, for the bundle-adjustment path, the map side of maplab's
 * optimizer:
 *   - vi_map::serialization::loadMapFromFolder
 *     (map-structure/vi-map/src/vi-map-serialization.cc:318-364): the
 *     vi_map/ folder (text metadata, binary vi_map.proto VIMap messages for
 *     missions, vertices*, edges*, landmark_index) and vi_map/sensors.yaml;
 *   - map_optimization::constructOptimizationProblem
 *     (algorithms/map-optimization/src/vi-optimization-builder.cc:154-374)
 *     with OptimizationStateBuffer::importStatesOfMissions
 *     (src/optimization-state-buffer.cc:153-300): the SoA problem of
 *     maplab_ba.h for a set of missions;
 *   - OptimizationStateBuffer::copyAllStatesBackToMap
 *     (src/optimization-state-buffer.cc:42-78) and
 *     vi_map::serialization::saveMapToFolder (vi-map-serialization.cc:366-435):
 *     the optimized state written into the map and the map saved.
 *
 * Host code only (no device).  Errors are status codes, never aborts: a
 * malformed file or a dangling id makes the call fail with
 * MBA_ERR_INVALID_ARG / MBA_ERR_OUT_OF_RANGE_INDEX where maplab would CHECK.
 */
#ifndef MAPLAB_VIMAP_H_
#define MAPLAB_VIMAP_H_

#include "maplab_ba.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mba_vimap mba_vimap;

typedef struct mba_vimap_info {
  int64_t num_missions;
  int64_t num_vertices;
  int64_t num_landmarks;
  int64_t num_keypoints;             /* keypoints of set frames */
  int64_t num_viwls_edges;
  int64_t num_odometry_edges;        /* 6-DoF odometry TransformationEdge */
  int64_t num_wheel_odometry_edges;
  int64_t num_loop_closure_edges;
  int64_t num_other_edges;           /* generic transformation / cklam edges (not used by BA) */
  int64_t num_absolute_measurements; /* Absolute6DoFMeasurement over all vertices */
  int64_t num_sensors;               /* entries of sensors.yaml (cameras inside an ncamera not counted) */
  int64_t num_cameras;               /* cameras over all ncameras */
} mba_vimap_info;

/* Reads `map_folder`/vi_map/{vi_map_metadata, sensors.yaml, files listed in
 * the metadata}.  The map is validated (every id a vertex, edge, landmark
 * index entry or mission refers to exists) and kept in memory with the raw
 * message bytes, so that mba_vimap_save rewrites only the optimized fields. */
mba_status mba_vimap_load(const char* map_folder, mba_vimap** out);
void mba_vimap_destroy(mba_vimap* m);
mba_status mba_vimap_get_info(const mba_vimap* m, mba_vimap_info* info);

/* Mission ids (2 x uint64 each, aslam::proto::Id words) in the order of the
 * missions file. */
mba_status mba_vimap_mission_ids(const mba_vimap* m, uint64_t* ids /* [2 * num_missions] */);

/* Which landmarks the visual terms use (isLandmarkWellConstrained,
 * map-structure/vi-map/src/landmark-quality-metrics.cc:75-103). */
enum {
  MBA_VIMAP_LANDMARKS_QUALITY = 0, /* kGood kept, kBad dropped, kUnknown evaluated (quality options) */
  MBA_VIMAP_LANDMARKS_ALL = 1,     /* every landmark with a valid store vertex */
  MBA_VIMAP_LANDMARKS_MASK = 2     /* the caller's landmark_keep mask (map landmark order) */
};

/* ViProblemOptions as maplab's flags set them (vi-optimization-builder.cc:
 * 9-75); defaults from mba_vimap_default_export_options. */
typedef struct mba_vimap_export_options {
  int32_t num_missions;          /* 0 = every mission of the map */
  int32_t pad0_;
  const int32_t* missions;       /* [num_missions] indices into the missions file order */
  int32_t add_visual_constraints;        /* ba_include_visual, 1 */
  int32_t add_inertial_constraints;      /* ba_include_inertial, 1 */
  int32_t add_6dof_odometry_constraints; /* ba_include_6dof_odometry, 0 */
  int32_t add_wheel_odometry_constraints;/* ba_include_wheel_odometry, 0 */
  int32_t add_absolute_pose_constraints; /* ba_include_absolute_pose_constraints, 0 */
  int32_t add_loop_closure_edges;        /* ba_include_loop_closure_edges, 0 */
  int32_t fix_landmark_positions;        /* ba_fix_landmark_positions, 0 */
  int32_t fix_velocity;                  /* ba_fix_velocity, 0 */
  int32_t fix_gyro_bias;                 /* ba_fix_gyro_bias, 0 */
  int32_t fix_accel_bias;                /* ba_fix_accel_bias, 0 */
  int32_t fix_vertices;                  /* ba_fix_vertices, 0 */
  int32_t min_landmarks_per_frame;       /* ba_min_landmarks_per_frame, 0 */
  int32_t feature_type;                  /* ba_feature_type: 0 = kBinary (default), -1 = every visual type */
  int32_t apply_gauge_fixes;             /* 1: kf_flags / lm_constant from mba_gauge_fixes */
  int32_t landmark_selection;            /* MBA_VIMAP_LANDMARKS_* */
  int32_t pad1_;
  const uint8_t* landmark_keep;          /* [num_landmarks of the map] for MBA_VIMAP_LANDMARKS_MASK */
  mba_landmark_quality_options quality;  /* elq_* flags for kUnknown landmarks */
  double gravity_magnitude;              /* default GravityProvider(392 m, 47.22 deg) of ba_altitude_meters /
                                            ba_latitude; <= 0: the mission IMU's gravity_magnitude_mps2 */
  int32_t use_huber;                     /* visual Huber loss (optimization-terms-addition.cc:189-198), 1 */
  int32_t pad2_;
} mba_vimap_export_options;

void mba_vimap_default_export_options(mba_vimap_export_options* o);

/* Builds the SoA problem of the selected missions into `desc`.  Every array
 * `desc` points to is owned by `m` and stays valid until the next export or
 * mba_vimap_destroy.  Index order: keyframes mission by mission along the
 * backbone from the root vertex (getAllVertexIdsInMissionAlongGraph,
 * vi-map.cc:2281-2316); landmarks by store keyframe, then store order;
 * observations by observer keyframe, frame, keypoint; inertial edges along
 * the backbone; pose edges wheel odometry, 6-DoF odometry, absolute, loop
 * closures (the builder's order). */
mba_status mba_vimap_export(mba_vimap* m, const mba_vimap_export_options* o, mba_problem_desc* desc);

/* Ids of the last export's rows (2 x uint64 each; NULL skips an array):
 * keyframe vertex ids, landmark ids, mission ids, and per pose edge the edge
 * id (relative and loop-closure terms) or the vertex id (absolute terms). */
mba_status mba_vimap_export_ids(const mba_vimap* m, uint64_t* kf_vertex_ids, uint64_t* landmark_ids,
                                uint64_t* mission_ids, uint64_t* pose_edge_ids);

/* Map landmark order (store vertices in file order, then store order): the
 * ids, for building a landmark_keep mask. */
mba_status mba_vimap_landmark_ids(const mba_vimap* m, uint64_t* ids /* [2 * num_landmarks] */);

/* Writes the optimized state of the last export back into the map
 * (copyAllKeyframePosesBackToMap: q_M_I = q_IM (JPL) coefficient for
 * coefficient, p_M_I; velocity, biases, landmark p_B, and the loop closures'
 * switch variables).  Arrays in the layout of mba_problem_desc; each may be
 * NULL. */
mba_status mba_vimap_import_state(mba_vimap* m, const double* kf_q_IM_p_MI, const double* kf_v_M,
                                  const double* kf_b_g, const double* kf_b_a, const double* lm_p_B,
                                  const double* pose_edge_switch);

/* Writes the map to `map_folder`/vi_map/ (created; an existing vi_map/
 * folder is refused, as saveMapToFolder refuses without overwrite).  The
 * message bytes are the loaded ones with only the state fields re-encoded. */
mba_status mba_vimap_save(const mba_vimap* m, const char* map_folder);

#ifdef __cplusplus
}
#endif

#endif /* MAPLAB_VIMAP_H_ */
