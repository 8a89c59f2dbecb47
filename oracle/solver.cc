// CPU ORACLE — test infrastructure only (see oracle.h).
//
// Problem-level restatement: the maplab VI problem as built by
// map_optimization::constructOptimizationProblem (vi-optimization-builder.cc:
// 154-374, optimization-terms-addition.cc:22-241 and 421-495) over the SoA
// descriptor of include/maplab_ba.h, and the Ceres trust-region
// Levenberg-Marquardt minimizer configured by solver-options.h:26-75.
// The LM restatement follows Ceres' published algorithm (TrustRegionMinimizer +
// LevenbergMarquardtStrategy): Jacobi scaling from the initial Jacobian,
// D = sqrt(clamp(diag(J^T J), 1e-6, 1e32) / radius), model cost change
// -J d.(r + J d / 2), acceptance at relative decrease > 1e-3, Nielsen radius
// update radius /= max(1/3, 1 - (2 rho - 1)^3), rejection radius /= 2^k.
// Landmarks are eliminated by the Schur complement; the reduced camera system
// is solved by dense Cholesky or by block-Jacobi PCG.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <thread>
#include <unordered_map>
#include <vector>

#include "oracle.h"

namespace oracle {

static void parallelFor(int64_t n, int threads, const std::function<void(int64_t, int64_t)>& fn) {
  if (threads <= 1 || n < 1024) { fn(0, n); return; }
  std::vector<std::thread> ts;
  const int64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int64_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    ts.emplace_back(fn, b, e);
  }
  for (auto& t : ts) t.join();
}

struct Problem {
  int64_t nkf = 0, nlm = 0, nobs = 0, ncam = 0, nmis = 0, nedge = 0, nsamp = 0;
  int64_t nimu = 0;  // edges [0, nimu) are IMU edges, [nimu, nedge) relative pose edges
  std::vector<double> pe_meas, pe_M, pe_ext;  // per pose edge: [7], [36] sqrt information, [7]
  std::vector<int32_t> pe_type, pe_swi;       // per pose edge: MBA_POSE_EDGE_*, switch variable (-1: none)
  std::vector<double> pe_swc;                 // switch value of an edge without a switch variable
  std::vector<double> sw, sw_w;               // switch variables and their prior's sqrt information
  std::vector<double> obs_uv, obs_sigma;
  std::vector<int32_t> obs_lm, obs_kf, obs_cam;
  std::vector<uint8_t> obs_type;
  std::vector<double> lm_p;
  std::vector<int32_t> lm_store;
  std::vector<uint8_t> lm_const;
  std::vector<double> kf_x, kf_v, kf_bg, kf_ba;
  std::vector<int32_t> kf_mis;
  std::vector<uint32_t> kf_flags;
  std::vector<double> mis;
  std::vector<mba_camera> cams;
  std::vector<int32_t> e_from, e_to;
  std::vector<int64_t> e_off, ts;
  std::vector<double> imu;
  ImuNoise noise{};
  int use_huber = 1;
  double hub_local = 3.0, hub_global = 10.0;
  int threads = 1;
  std::vector<int64_t> lm_obs_off, lm_obs_idx;
  std::vector<uint8_t> kf_mask;  // 15 per keyframe, 1 = active tangent dim
  std::vector<uint8_t> lm_mask;  // 1 = active landmark
  std::vector<uint8_t> lm_off;   // 1 = rejected outlier: its terms are out of the problem
  // Calibration / baseframe variables ("global nodes"): one 15-dim block per
  // camera with a free calibration block and per mission with a free
  // baseframe, after the keyframes in the reduced system (node g is block
  // nkf + g).  Camera node dims: intrinsics 0-3, distortion 4-7 (the model's
  // parameter count), theta_C_I 8-10, p_C_I 11-13.  Mission node dims:
  // theta 0-2 (yaw only: 0), p_G_M 3-5.
  int64_t ng = 0;
  std::vector<uint32_t> cam_flags, mis_flags;
  std::vector<int32_t> cam_node, mis_node;   // -1: constant
  std::vector<int32_t> node_cam, node_mis;   // node -> camera / mission (-1)
  std::vector<uint8_t> g_mask;               // 15 per node
};

// Distortion parameters per model (aslam): radtan 4, equidistant 4, FOV 1.
static int distortionParams(int type) {
  return type == MBA_DISTORTION_RADTAN || type == MBA_DISTORTION_EQUIDISTANT ? 4 : (type == MBA_DISTORTION_FOV ? 1 : 0);
}

int createProblem(const mba_problem_desc* d, Problem** out) {
  if (!d || !out) return MBA_ERR_INVALID_ARG;
  auto* p = new Problem();
  p->nkf = d->num_keyframes; p->nlm = d->num_landmarks; p->nobs = d->num_observations;
  p->ncam = d->num_cameras; p->nmis = d->num_missions; p->nedge = d->num_imu_edges;
  p->nsamp = d->num_imu_samples;
  p->obs_uv.assign(d->obs_uv, d->obs_uv + 2 * p->nobs);
  p->obs_sigma.assign(d->obs_sigma, d->obs_sigma + p->nobs);
  p->obs_lm.assign(d->obs_landmark, d->obs_landmark + p->nobs);
  p->obs_kf.assign(d->obs_keyframe, d->obs_keyframe + p->nobs);
  p->obs_cam.assign(d->obs_camera, d->obs_camera + p->nobs);
  p->lm_p.assign(d->lm_p_B, d->lm_p_B + 3 * p->nlm);
  p->lm_store.assign(d->lm_store_keyframe, d->lm_store_keyframe + p->nlm);
  p->lm_const.assign(p->nlm, 0);
  if (d->lm_constant) p->lm_const.assign(d->lm_constant, d->lm_constant + p->nlm);
  p->kf_x.assign(d->kf_q_IM_p_MI, d->kf_q_IM_p_MI + 7 * p->nkf);
  p->kf_v.assign(d->kf_v_M, d->kf_v_M + 3 * p->nkf);
  p->kf_bg.assign(d->kf_b_g, d->kf_b_g + 3 * p->nkf);
  p->kf_ba.assign(d->kf_b_a, d->kf_b_a + 3 * p->nkf);
  p->kf_mis.assign(d->kf_mission, d->kf_mission + p->nkf);
  p->kf_flags.assign(p->nkf, 0u);
  if (d->kf_flags) p->kf_flags.assign(d->kf_flags, d->kf_flags + p->nkf);
  p->mis.assign(d->mission_q_GM_p_GM, d->mission_q_GM_p_GM + 7 * p->nmis);
  p->cams.assign(d->cameras, d->cameras + p->ncam);
  p->nimu = p->nedge;
  if (p->nimu > 0) {
    p->e_from.assign(d->edge_from, d->edge_from + p->nimu);
    p->e_to.assign(d->edge_to, d->edge_to + p->nimu);
    p->e_off.assign(d->edge_sample_offset, d->edge_sample_offset + p->nimu + 1);
    p->ts.assign(d->imu_timestamp_ns, d->imu_timestamp_ns + p->nsamp);
    p->imu.assign(d->imu_acc_gyro, d->imu_acc_gyro + 6 * p->nsamp);
  }
  // Relative pose edges follow the IMU edges.
  // Loop closures store the measured rotation as JPL coefficients (the
  // Hamilton inverse, augment-loopclosure.cc:44-49) and absolute terms as the
  // inverse measured rotation q_S_G (block-pose-prior-error-term-v2.cc:13-16);
  // both inverses as Eigen computes them (conjugate / squared norm).
  for (int64_t j = 0; j < d->num_pose_edges; ++j) {
    const int type = d->pose_edge_type ? d->pose_edge_type[j] : MBA_POSE_EDGE_RELATIVE;
    const int32_t f = d->pose_edge_from[j];
    p->e_from.push_back(f);
    p->e_to.push_back(type == MBA_POSE_EDGE_ABSOLUTE ? f : d->pose_edge_to[j]);
    p->pe_type.push_back(type);
    double T[7];
    std::memcpy(T, d->pose_edge_T_Bk_Bkp1 + 7 * j, sizeof(T));
    if (type != MBA_POSE_EDGE_RELATIVE) {
      const double n2 = T[0] * T[0] + T[1] * T[1] + T[2] * T[2] + T[3] * T[3];
      for (int i = 0; i < 3; ++i) T[i] = -T[i] / n2;
      T[3] = T[3] / n2;
    }
    p->pe_meas.insert(p->pe_meas.end(), T, T + 7);
    p->pe_ext.insert(p->pe_ext.end(), d->pose_edge_q_I_B_p_B_I + 7 * j, d->pose_edge_q_I_B_p_B_I + 7 * j + 7);
    double M[36];
    if (!poseEdgeSqrtInfo(d->pose_edge_covariance + 36 * j, M)) { delete p; return MBA_ERR_NOT_SPD; }
    p->pe_M.insert(p->pe_M.end(), M, M + 36);
    const double s0 = (type == MBA_POSE_EDGE_LOOP_CLOSURE && d->pose_edge_switch) ? d->pose_edge_switch[j] : 1.0;
    const double var = (type == MBA_POSE_EDGE_LOOP_CLOSURE && d->pose_edge_switch_variance)
                           ? d->pose_edge_switch_variance[j] : 0.0;
    if (var > 0.0) {
      p->pe_swi.push_back((int32_t)p->sw.size());
      p->sw.push_back(s0);
      p->sw_w.push_back(std::sqrt(1.0 / var));  // SwitchPriorErrorTerm (switch-prior-error-term.h:17-20)
    } else {
      p->pe_swi.push_back(-1);
    }
    p->pe_swc.push_back(s0);
  }
  p->nedge = p->nimu + d->num_pose_edges;
  p->noise = {d->gyro_noise_sigma, d->gyro_bias_sigma, d->acc_noise_sigma, d->acc_bias_sigma,
              d->gravity_magnitude};
  p->use_huber = d->use_huber;
  p->hub_local = d->huber_delta_local;
  p->hub_global = d->huber_delta_global;
  // Error type selection (optimization-terms-addition.cc:68-78).
  p->obs_type.resize(p->nobs);
  for (int64_t i = 0; i < p->nobs; ++i) {
    const int l = p->obs_lm[i], k = p->obs_kf[i];
    if (l < 0 || l >= p->nlm || k < 0 || k >= p->nkf || p->obs_cam[i] < 0 || p->obs_cam[i] >= p->ncam) {
      delete p;
      return MBA_ERR_OUT_OF_RANGE_INDEX;
    }
    const int s = p->lm_store[l];
    if (k == s) p->obs_type[i] = MBA_LOCAL_KEYFRAME;
    else if (p->kf_mis[k] == p->kf_mis[s]) p->obs_type[i] = MBA_LOCAL_MISSION;
    else p->obs_type[i] = MBA_GLOBAL;
  }
  // landmark -> observations
  p->lm_obs_off.assign(p->nlm + 1, 0);
  for (int64_t i = 0; i < p->nobs; ++i) p->lm_obs_off[p->obs_lm[i] + 1]++;
  for (int64_t l = 0; l < p->nlm; ++l) p->lm_obs_off[l + 1] += p->lm_obs_off[l];
  p->lm_obs_idx.resize(p->nobs);
  {
    std::vector<int64_t> fill(p->lm_obs_off.begin(), p->lm_obs_off.end() - 1);
    for (int64_t i = 0; i < p->nobs; ++i) p->lm_obs_idx[fill[p->obs_lm[i]]++] = i;
  }
  // Active tangent dims.  KF tangent order: theta(3), p(3), v(3), b_g(3), b_a(3).
  p->kf_mask.assign(15 * p->nkf, 1);
  std::vector<uint8_t> in_inertial(p->nkf, 0), in_visual(p->nkf, 0);
  for (int64_t e = 0; e < p->nimu; ++e) { in_inertial[p->e_from[e]] = 1; in_inertial[p->e_to[e]] = 1; }
  // a pose edge constrains the pose blocks only (the keyframe's pose is in the
  // problem, its speed and biases are not unless an IMU edge uses them)
  for (int64_t e = p->nimu; e < p->nedge; ++e) { in_visual[p->e_from[e]] = 1; in_visual[p->e_to[e]] = 1; }
  for (int64_t i = 0; i < p->nobs; ++i) {
    if (p->obs_type[i] != MBA_LOCAL_KEYFRAME) { in_visual[p->obs_kf[i]] = 1; in_visual[p->lm_store[p->obs_lm[i]]] = 1; }
  }
  for (int64_t k = 0; k < p->nkf; ++k) {
    uint8_t* m = &p->kf_mask[15 * k];
    const uint32_t f = p->kf_flags[k];
    if (!in_inertial[k] && !in_visual[k]) for (int i = 0; i < 6; ++i) m[i] = 0;
    if (!in_inertial[k]) for (int i = 6; i < 15; ++i) m[i] = 0;
    if (f & MBA_KF_POSE_CONSTANT) for (int i = 0; i < 6; ++i) m[i] = 0;
    if (f & MBA_KF_ROTATION_CONSTANT) for (int i = 0; i < 6; ++i) m[i] = 0;
    if (f & MBA_KF_POSITION_CONSTANT) for (int i = 3; i < 6; ++i) m[i] = 0;
    if (f & MBA_KF_GAUGE_ROLL_PITCH) { m[2] = 0; m[3] = m[4] = m[5] = 0; }
    if (f & MBA_KF_VELOCITY_CONSTANT) for (int i = 6; i < 9; ++i) m[i] = 0;
    if (f & MBA_KF_GYRO_BIAS_CONSTANT) for (int i = 9; i < 12; ++i) m[i] = 0;
    if (f & MBA_KF_ACCEL_BIAS_CONSTANT) for (int i = 12; i < 15; ++i) m[i] = 0;
  }
  p->lm_mask.assign(p->nlm, 1);
  p->lm_off.assign(p->nlm, 0);
  for (int64_t l = 0; l < p->nlm; ++l) if (p->lm_const[l] || p->lm_obs_off[l + 1] == p->lm_obs_off[l]) p->lm_mask[l] = 0;
  // Calibration / baseframe variables.
  p->cam_flags.assign(p->ncam, 0u);
  if (d->camera_flags) p->cam_flags.assign(d->camera_flags, d->camera_flags + p->ncam);
  p->mis_flags.assign(p->nmis, 0u);
  if (d->mission_flags) p->mis_flags.assign(d->mission_flags, d->mission_flags + p->nmis);
  p->cam_node.assign(p->ncam, -1);
  p->mis_node.assign(p->nmis, -1);
  for (int64_t c = 0; c < p->ncam; ++c) {
    const uint32_t f = p->cam_flags[c];
    if (!(f & 0xfu)) continue;
    std::vector<uint8_t> m(15, 0);
    if (f & MBA_CAM_INTRINSICS_FREE) for (int a = 0; a < 4; ++a) m[a] = 1;
    if (f & MBA_CAM_DISTORTION_FREE) for (int a = 0; a < distortionParams(p->cams[c].distortion_type); ++a) m[4 + a] = 1;
    if (f & MBA_CAM_ROTATION_FREE) for (int a = 8; a < 11; ++a) m[a] = 1;
    if (f & MBA_CAM_TRANSLATION_FREE) for (int a = 11; a < 14; ++a) m[a] = 1;
    p->cam_node[c] = (int32_t)p->ng++;
    p->node_cam.push_back((int32_t)c);
    p->node_mis.push_back(-1);
    p->g_mask.insert(p->g_mask.end(), m.begin(), m.end());
  }
  for (int64_t mi = 0; mi < p->nmis; ++mi) {
    const uint32_t f = p->mis_flags[mi];
    if (!f) continue;
    if (f != MBA_MIS_BASEFRAME_YAW_POSITION && f != MBA_MIS_BASEFRAME_POSE) { delete p; return MBA_ERR_INVALID_ARG; }
    std::vector<uint8_t> m(15, 0);
    m[0] = 1;
    if (f == MBA_MIS_BASEFRAME_POSE) m[1] = m[2] = 1;
    m[3] = m[4] = m[5] = 1;
    p->mis_node[mi] = (int32_t)p->ng++;
    p->node_cam.push_back(-1);
    p->node_mis.push_back((int32_t)mi);
    p->g_mask.insert(p->g_mask.end(), m.begin(), m.end());
  }
  // A free baseframe enters the visual terms only: absolute 6-DoF terms and
  // cross-mission loop closures keep their baseframes constant.
  for (int64_t e = p->nimu; e < p->nedge; ++e) {
    const int type = p->pe_type[e - p->nimu];
    const int mf = p->kf_mis[p->e_from[e]], mt = p->kf_mis[p->e_to[e]];
    const bool uses_bf = type == MBA_POSE_EDGE_ABSOLUTE || (type == MBA_POSE_EDGE_LOOP_CLOSURE && mf != mt);
    if (uses_bf && (p->mis_node[mf] >= 0 || p->mis_node[mt] >= 0)) { delete p; return MBA_ERR_INVALID_ARG; }
  }
  p->threads = std::max(1u, std::thread::hardware_concurrency());
  *out = p;
  return MBA_OK;
}

// Local parameterization Jacobian (7x6) of keyframe k's pose block mapped to
// the 6-dim tangent [theta, p] (masked dims zero).
static void poseParam(const Problem& p, int64_t k, double* P76) {
  std::memset(P76, 0, 42 * sizeof(double));
  const double* q = &p.kf_x[7 * k];
  const uint8_t* m = &p.kf_mask[15 * k];
  if (p.kf_flags[k] & MBA_KF_GAUGE_ROLL_PITCH) {
    double J42[8];
    jplRollPitchJacobian(&p.mis[7 * p.kf_mis[k]], q, J42);
    for (int r = 0; r < 4; ++r) {
      P76[6 * r + 0] = m[0] ? J42[2 * r] : 0.0;
      P76[6 * r + 1] = m[1] ? J42[2 * r + 1] : 0.0;
    }
  } else {
    double Jq[12];
    jplQuaternionJacobian(q, Jq);
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 3; ++c) P76[6 * r + c] = m[c] ? Jq[3 * r + c] : 0.0;
  }
  for (int i = 0; i < 3; ++i) P76[6 * (4 + i) + 3 + i] = m[3 + i] ? 1.0 : 0.0;
}

static void visualParams(const Problem& p, int64_t i, const double** P) {
  const int l = p.obs_lm[i], k = p.obs_kf[i], s = p.lm_store[l];
  const mba_camera& c = p.cams[p.obs_cam[i]];
  P[0] = &p.lm_p[3 * l];
  P[1] = &p.kf_x[7 * s];
  P[2] = &p.mis[7 * p.kf_mis[s]];
  P[3] = &p.mis[7 * p.kf_mis[k]];
  P[4] = &p.kf_x[7 * k];
  P[5] = c.q_CI_p_CI;
  P[6] = c.q_CI_p_CI + 4;
  P[7] = c.intrinsics;
  P[8] = c.distortion;
}

static double huberA(const Problem& p, int64_t i) {
  return (p.obs_type[i] == MBA_GLOBAL ? p.hub_global : p.hub_local) * p.obs_sigma[i];
}

void evaluateVisualAmbient(const Problem& p, double* res, double* const* jac) {
  parallelFor(p.nobs, p.threads, [&](int64_t b, int64_t e) {
    static const int sz[9] = {6, 14, 14, 14, 14, 8, 6, 8, 8};
    for (int64_t i = b; i < e; ++i) {
      const double* P[9];
      visualParams(p, i, P);
      double r[2];
      double* J[9];
      bool any = false;
      for (int k = 0; k < 9; ++k) { J[k] = (jac && jac[k]) ? jac[k] + sz[k] * i : nullptr; any |= J[k] != nullptr; }
      visualEvaluate(P, &p.obs_uv[2 * i], p.obs_sigma[i], p.obs_type[i], p.cams[p.obs_cam[i]], r,
                     any ? J : nullptr, nullptr);
      if (res) { res[2 * i] = r[0]; res[2 * i + 1] = r[1]; }
    }
  });
}

static void inertialParams(const Problem& p, int64_t e, const double** P) {
  const int f = p.e_from[e], t = p.e_to[e];
  P[0] = &p.kf_x[7 * f]; P[1] = &p.kf_bg[3 * f]; P[2] = &p.kf_v[3 * f]; P[3] = &p.kf_ba[3 * f];
  P[4] = &p.kf_x[7 * t]; P[5] = &p.kf_bg[3 * t]; P[6] = &p.kf_v[3 * t]; P[7] = &p.kf_ba[3 * t];
}

int evaluateInertialAmbient(const Problem& p, double* res, double* const* jac) {
  int status = 0;
  parallelFor(p.nimu, p.threads, [&](int64_t b, int64_t e) {
    static const int sz[8] = {105, 45, 45, 45, 105, 45, 45, 45};
    for (int64_t i = b; i < e; ++i) {
      const double* P[8];
      inertialParams(p, i, P);
      double r[15];
      double* J[8];
      bool any = false;
      for (int k = 0; k < 8; ++k) { J[k] = (jac && jac[k]) ? jac[k] + sz[k] * i : nullptr; any |= J[k] != nullptr; }
      const int64_t o = p.e_off[i];
      const int st = inertialEvaluate(p.noise, P, (int)(p.e_off[i + 1] - o), &p.ts[o], &p.imu[6 * o], r,
                                      any ? J : nullptr);
      if (st) status = st;
      if (res) std::memcpy(res + 15 * i, r, sizeof(r));
    }
  });
  return status;
}

// ------------------------------------------------------------ linearization
struct Linearization {
  std::vector<double> vr, vJl, vJs, vJo;  // visual: 2, 2x3, 2x6, 2x6 per obs
  std::vector<double> ir, iJf, iJt;       // inertial: 15, 15x15, 15x15 per edge
  std::vector<double> sJ;                 // pose edges: d residual / d switch [6] (= unswitched residual)
  // Global nodes (only when the problem has some): per observation up to 3
  // node ids (camera; the landmark's and the observer's mission baseframes
  // of a kGlobal term; -1 = none) and their 2 x 15 tangent Jacobians.
  std::vector<int32_t> vGn;               // 3 per obs
  std::vector<double> vG;                 // 3 x 30 per obs
  double cost = 0.0;
};

// Tangent Jacobians (2 x 15 in node dims, masked dims zero) of observation i
// with respect to its global nodes, from the ambient blocks of
// VisualReprojectionError::Evaluate: intrinsics and distortion are additive
// blocks, q_C_I goes through JplQuaternionParameterization, a baseframe
// through JplPoseParameterization or JplYawOnlyPoseParameterization.
static void nodeJacobians(const Problem& p, int64_t i, const double* Jbf_lm, const double* Jbf_obs,
                          const double* Jq_CI, const double* Jp_CI, const double* Jintr, const double* Jdist,
                          int32_t* nid, double* JN) {
  std::memset(JN, 0, 90 * sizeof(double));
  nid[0] = nid[1] = nid[2] = -1;
  const int c = p.obs_cam[i];
  const int cn = p.cam_node[c];
  if (cn >= 0) {
    nid[0] = cn;
    const uint8_t* m = &p.g_mask[15 * cn];
    double Jq[12];
    jplQuaternionJacobian(p.cams[c].q_CI_p_CI, Jq);
    for (int r = 0; r < 2; ++r) {
      double* o = JN + 15 * r;
      for (int a = 0; a < 4; ++a) o[a] = m[a] ? Jintr[4 * r + a] : 0.0;
      for (int a = 0; a < 4; ++a) o[4 + a] = m[4 + a] ? Jdist[4 * r + a] : 0.0;
      for (int a = 0; a < 3; ++a) {
        double s = 0.0;
        for (int k = 0; k < 4; ++k) s += Jq_CI[4 * r + k] * Jq[3 * k + a];
        o[8 + a] = m[8 + a] ? s : 0.0;
        o[11 + a] = m[11 + a] ? Jp_CI[3 * r + a] : 0.0;
      }
    }
  }
  if (p.obs_type[i] != MBA_GLOBAL) return;
  const int l = p.obs_lm[i];
  const int mis[2] = {p.kf_mis[p.lm_store[l]], p.kf_mis[p.obs_kf[i]]};
  const double* Jb[2] = {Jbf_lm, Jbf_obs};
  for (int s = 0; s < 2; ++s) {
    const int g = p.mis_node[mis[s]];
    if (g < 0) continue;
    nid[1 + s] = g;
    double* O = JN + 30 * (1 + s);
    const uint8_t* m = &p.g_mask[15 * g];
    const double* q = &p.mis[7 * mis[s]];
    if (p.mis_flags[mis[s]] == MBA_MIS_BASEFRAME_YAW_POSITION) {
      double Jy[4];
      jplYawJacobian(q, Jy);
      for (int r = 0; r < 2; ++r) {
        double v = 0.0;
        for (int k = 0; k < 4; ++k) v += Jb[s][7 * r + k] * Jy[k];
        O[15 * r] = v;
      }
    } else {
      double Jq[12];
      jplQuaternionJacobian(q, Jq);
      for (int r = 0; r < 2; ++r)
        for (int a = 0; a < 3; ++a) {
          double v = 0.0;
          for (int k = 0; k < 4; ++k) v += Jb[s][7 * r + k] * Jq[3 * k + a];
          O[15 * r + a] = m[a] ? v : 0.0;
        }
    }
    for (int r = 0; r < 2; ++r)
      for (int a = 0; a < 3; ++a) O[15 * r + 3 + a] = Jb[s][7 * r + 4 + a];
  }
}

// Ceres Corrector (third-party, restated from Triggs et al. "Bundle
// adjustment: a modern synthesis" as documented by Ceres): returns the
// residual scaling and applies the Jacobian correction to J (2 x cols).
static void applyCorrector(double sq, const double* rho, double* r, double** Js, const int* cols, int nJ) {
  const double sqrt_rho1 = std::sqrt(rho[1]);
  double residual_scaling, alpha_sq_norm;
  if (sq == 0.0 || rho[2] <= 0.0) {
    residual_scaling = sqrt_rho1;
    alpha_sq_norm = 0.0;
  } else {
    const double D = 1.0 + 2.0 * sq * rho[2] / rho[1];
    const double alpha = 1.0 - std::sqrt(D);
    residual_scaling = sqrt_rho1 / (1.0 - alpha);
    alpha_sq_norm = alpha / sq;
  }
  for (int j = 0; j < nJ; ++j) {
    double* J = Js[j];
    const int C = cols[j];
    for (int c = 0; c < C; ++c) {
      const double rtJ = r[0] * J[c] + r[1] * J[C + c];
      J[c] = sqrt_rho1 * (J[c] - alpha_sq_norm * r[0] * rtJ);
      J[C + c] = sqrt_rho1 * (J[C + c] - alpha_sq_norm * r[1] * rtJ);
    }
  }
  r[0] *= residual_scaling;
  r[1] *= residual_scaling;
}

// Robustified, tangent-space linearization of every term.  want_jac=false
// only computes the cost.
int linearize(const Problem& p, bool want_jac, Linearization* L) {
  if (want_jac) {
    L->vr.assign(2 * p.nobs, 0.0); L->vJl.assign(6 * p.nobs, 0.0);
    L->vJs.assign(12 * p.nobs, 0.0); L->vJo.assign(12 * p.nobs, 0.0);
    L->ir.assign(15 * p.nedge, 0.0); L->iJf.assign(225 * p.nedge, 0.0); L->iJt.assign(225 * p.nedge, 0.0);
    L->sJ.assign(6 * (p.nedge - p.nimu), 0.0);
    if (p.ng > 0) {
      L->vGn.assign(3 * p.nobs, -1);
      L->vG.assign(90 * p.nobs, 0.0);
    }
  }
  const int T = p.threads;
  std::vector<double> part(T + 1, 0.0);
  // visual
  {
    std::vector<std::thread> ts;
    const int64_t chunk = (p.nobs + T - 1) / T;
    auto workRange = [&](int t, int64_t b, int64_t e) {
      double acc = 0.0;
      for (int64_t i = b; i < e; ++i) {
        if (p.lm_off[p.obs_lm[i]]) continue;  // rejected: zero residual and Jacobians
        const double* P[9];
        visualParams(p, i, P);
        double r[2], Jl[6], Js7[14], Jo7[14];
        double Jbl[14], Jbo[14], Jqc[8], Jpc[6], Jin[8], Jdi[8];
        const bool nodes = want_jac && p.ng > 0;
        double* J[9] = {Jl, Js7, nodes ? Jbl : nullptr, nodes ? Jbo : nullptr, Jo7, nodes ? Jqc : nullptr,
                        nodes ? Jpc : nullptr, nodes ? Jin : nullptr, nodes ? Jdi : nullptr};
        visualEvaluate(P, &p.obs_uv[2 * i], p.obs_sigma[i], p.obs_type[i], p.cams[p.obs_cam[i]], r,
                       want_jac ? J : nullptr, nullptr);
        const double sq = r[0] * r[0] + r[1] * r[1];
        double rho[3] = {sq, 1.0, 0.0};
        if (p.use_huber) huberLoss(huberA(p, i), sq, rho);
        acc += 0.5 * rho[0];
        if (!want_jac) continue;
        double Jst[12], Jot[12], P76[42];
        std::memset(Jst, 0, sizeof(Jst)); std::memset(Jot, 0, sizeof(Jot));
        const int l = p.obs_lm[i];
        if (!p.lm_mask[l]) std::memset(Jl, 0, sizeof(Jl));
        if (p.obs_type[i] != MBA_LOCAL_KEYFRAME) {
          const int64_t s = p.lm_store[l], k = p.obs_kf[i];
          poseParam(p, s, P76);
          for (int rr = 0; rr < 2; ++rr)
            for (int c = 0; c < 6; ++c) {
              double a = 0.0, b2 = 0.0;
              for (int m = 0; m < 7; ++m) a += Js7[7 * rr + m] * P76[6 * m + c];
              Jst[6 * rr + c] = a;
              (void)b2;
            }
          poseParam(p, k, P76);
          for (int rr = 0; rr < 2; ++rr)
            for (int c = 0; c < 6; ++c) {
              double a = 0.0;
              for (int m = 0; m < 7; ++m) a += Jo7[7 * rr + m] * P76[6 * m + c];
              Jot[6 * rr + c] = a;
            }
        }
        double JN[90];
        int32_t nid[3] = {-1, -1, -1};
        if (nodes) nodeJacobians(p, i, Jbl, Jbo, Jqc, Jpc, Jin, Jdi, nid, JN);
        if (p.use_huber) {
          double* Js_[6] = {Jl, Jst, Jot, JN, JN + 30, JN + 60};
          const int cols[6] = {3, 6, 6, 15, 15, 15};
          applyCorrector(sq, rho, r, Js_, cols, nodes ? 6 : 3);
        }
        if (nodes) {
          std::memcpy(&L->vGn[3 * i], nid, sizeof(nid));
          std::memcpy(&L->vG[90 * i], JN, sizeof(JN));
        }
        std::memcpy(&L->vr[2 * i], r, sizeof(r));
        std::memcpy(&L->vJl[6 * i], Jl, sizeof(Jl));
        std::memcpy(&L->vJs[12 * i], Jst, sizeof(Jst));
        std::memcpy(&L->vJo[12 * i], Jot, sizeof(Jot));
      }
      part[t] = acc;
    };
    if (p.nobs < 2048) {
      // serial: one worker covering every observation
      std::fill(part.begin(), part.end(), 0.0);
      workRange(0, 0, p.nobs);
    } else {
      for (int t = 0; t < T; ++t)
        ts.emplace_back(workRange, t, std::min<int64_t>(p.nobs, t * chunk), std::min<int64_t>(p.nobs, (t + 1) * chunk));
      for (auto& t : ts) t.join();
    }
  }
  double cost = 0.0;
  for (double v : part) cost += v;
  // inertial
  std::vector<double> ipart(T + 1, 0.0);
  int status = 0;
  {
    std::vector<std::thread> ts;
    const int64_t chunk = (p.nimu + T - 1) / T;
    auto workRange = [&](int t, int64_t b, int64_t e) {
      double acc = 0.0;
      for (int64_t i = b; i < e; ++i) {
        const double* P[8];
        inertialParams(p, i, P);
        double r[15], Jp[2][105], Jg[2][45], Jv[2][45], Ja[2][45];
        double* J[8] = {Jp[0], Jg[0], Jv[0], Ja[0], Jp[1], Jg[1], Jv[1], Ja[1]};
        const int64_t o = p.e_off[i];
        const int st = inertialEvaluate(p.noise, P, (int)(p.e_off[i + 1] - o), &p.ts[o], &p.imu[6 * o], r,
                                        want_jac ? J : nullptr);
        if (st) { status = st; continue; }
        double sq = 0.0;
        for (int k = 0; k < 15; ++k) sq += r[k] * r[k];
        acc += 0.5 * sq;
        if (!want_jac) continue;
        std::memcpy(&L->ir[15 * i], r, sizeof(r));
        for (int s = 0; s < 2; ++s) {
          const int64_t k = s == 0 ? p.e_from[i] : p.e_to[i];
          double* out = s == 0 ? &L->iJf[225 * i] : &L->iJt[225 * i];
          double P76[42];
          poseParam(p, k, P76);
          const uint8_t* m = &p.kf_mask[15 * k];
          for (int rr = 0; rr < 15; ++rr) {
            for (int c = 0; c < 6; ++c) {
              double a = 0.0;
              for (int mm = 0; mm < 7; ++mm) a += Jp[s][7 * rr + mm] * P76[6 * mm + c];
              out[15 * rr + c] = a;
            }
            for (int c = 0; c < 3; ++c) {
              out[15 * rr + 6 + c] = m[6 + c] ? Jv[s][3 * rr + c] : 0.0;
              out[15 * rr + 9 + c] = m[9 + c] ? Jg[s][3 * rr + c] : 0.0;
              out[15 * rr + 12 + c] = m[12 + c] ? Ja[s][3 * rr + c] : 0.0;
            }
          }
        }
      }
      ipart[t] = acc;
    };
    if (p.nimu < 64) workRange(0, 0, p.nimu);
    else {
      for (int t = 0; t < T; ++t)
        ts.emplace_back(workRange, t, std::min<int64_t>(p.nimu, t * chunk), std::min<int64_t>(p.nimu, (t + 1) * chunk));
      for (auto& t : ts) t.join();
    }
  }
  for (double v : ipart) cost += v;
  // pose edges: residual rows 0-5, tangent columns (theta, p) through the
  // pose parameterization (ambient Jacobian x ComputeJacobian); loop closures
  // scaled by their switch, whose prior adds 0.5 ((1 - s) w)^2.
  static const double kIdentityPose[7] = {0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0};
  for (int64_t i = p.nimu; i < p.nedge; ++i) {
    const int64_t j = i - p.nimu, f = p.e_from[i], t = p.e_to[i];
    double r[6], Jf7[42] = {}, Jt7[42] = {};
    const int type = p.pe_type[j];
    const double* xf = &p.kf_x[7 * f];
    const double* xt = &p.kf_x[7 * t];
    if (type == MBA_POSE_EDGE_LOOP_CLOSURE) {
      const bool same = p.kf_mis[f] == p.kf_mis[t];
      const double* bfA = same ? kIdentityPose : &p.mis[7 * p.kf_mis[f]];
      const double* bfB = same ? kIdentityPose : &p.mis[7 * p.kf_mis[t]];
      loopClosureEvaluate(bfA, bfB, xf, xt, &p.pe_meas[7 * j], &p.pe_M[36 * j], r, want_jac ? Jf7 : nullptr,
                          want_jac ? Jt7 : nullptr);
    } else if (type == MBA_POSE_EDGE_ABSOLUTE) {
      absolutePoseEvaluate(&p.mis[7 * p.kf_mis[f]], xf, &p.pe_ext[7 * j], &p.pe_meas[7 * j], &p.pe_M[36 * j], r,
                           want_jac ? Jf7 : nullptr);
    } else {
      poseEdgeEvaluate(xf, xt, &p.pe_ext[7 * j], &p.pe_meas[7 * j], &p.pe_M[36 * j], r, want_jac ? Jf7 : nullptr,
                       want_jac ? Jt7 : nullptr);
    }
    const int q = p.pe_swi[j];
    const double sw = q >= 0 ? p.sw[q] : p.pe_swc[j];
    double sq = 0.0;
    for (int k = 0; k < 6; ++k) sq += (sw * r[k]) * (sw * r[k]);
    cost += 0.5 * sq;
    if (q >= 0) {
      const double rp = (1.0 - sw) * p.sw_w[q];
      cost += 0.5 * rp * rp;
    }
    if (!want_jac) continue;
    for (int k = 0; k < 6; ++k) { L->ir[15 * i + k] = sw * r[k]; L->sJ[6 * j + k] = r[k]; }
    for (int k = 0; k < 42; ++k) { Jf7[k] *= sw; Jt7[k] *= sw; }
    for (int s2 = 0; s2 < 2; ++s2) {
      const int64_t k = s2 == 0 ? f : t;
      const double* J7 = s2 == 0 ? Jf7 : Jt7;
      double* out = s2 == 0 ? &L->iJf[225 * i] : &L->iJt[225 * i];
      double P76[42];
      poseParam(p, k, P76);
      for (int rr = 0; rr < 6; ++rr)
        for (int c = 0; c < 6; ++c) {
          double a = 0.0;
          for (int mm = 0; mm < 7; ++mm) a += J7[7 * rr + mm] * P76[6 * mm + c];
          out[15 * rr + c] = a;
        }
    }
  }
  L->cost = cost;
  if (!std::isfinite(cost) && status == 0) status = MBA_ERR_NON_FINITE;
  return status;
}

// ------------------------------------------------------------ block system
struct BlockSystem {
  int64_t nkf = 0;
  std::unordered_map<uint64_t, int64_t> index;  // (i<<32|j), i<=j -> block
  std::vector<int32_t> bi, bj;
  std::vector<double> blocks;  // 225 per block
  int64_t find(int64_t i, int64_t j) const {
    if (i > j) std::swap(i, j);
    auto it = index.find(((uint64_t)i << 32) | (uint64_t)j);
    return it == index.end() ? -1 : it->second;
  }
  int64_t add(int64_t i, int64_t j) {
    if (i > j) std::swap(i, j);
    const uint64_t key = ((uint64_t)i << 32) | (uint64_t)j;
    auto it = index.find(key);
    if (it != index.end()) return it->second;
    const int64_t b = (int64_t)bi.size();
    index.emplace(key, b);
    bi.push_back((int32_t)i); bj.push_back((int32_t)j);
    return b;
  }
};

// Global nodes touched by observation i (block indices nkf + g), up to 3.
static int obsNodes(const Problem& p, int64_t i, int64_t* out) {
  int n = 0;
  const int cn = p.cam_node[p.obs_cam[i]];
  if (cn >= 0) out[n++] = p.nkf + cn;
  if (p.obs_type[i] == MBA_GLOBAL) {
    const int gl = p.mis_node[p.kf_mis[p.lm_store[p.obs_lm[i]]]], go = p.mis_node[p.kf_mis[p.obs_kf[i]]];
    if (gl >= 0) out[n++] = p.nkf + gl;
    if (go >= 0) out[n++] = p.nkf + go;
  }
  return n;
}

// Tangent dim d of block k (keyframe or global node) is active.
static bool dimActive(const Problem& p, int64_t k, int d) {
  return k < p.nkf ? p.kf_mask[15 * k + d] != 0 : p.g_mask[15 * (k - p.nkf) + d] != 0;
}

static void buildPattern(const Problem& p, BlockSystem* S) {
  S->nkf = p.nkf;
  for (int64_t k = 0; k < p.nkf + p.ng; ++k) S->add(k, k);
  for (int64_t e = 0; e < p.nedge; ++e) S->add(p.e_from[e], p.e_to[e]);
  std::vector<int64_t> ks;
  for (int64_t l = 0; l < p.nlm; ++l) {
    ks.clear();
    ks.push_back(p.lm_store[l]);
    for (int64_t a = p.lm_obs_off[l]; a < p.lm_obs_off[l + 1]; ++a) {
      ks.push_back(p.obs_kf[p.lm_obs_idx[a]]);
      if (p.ng > 0) {
        int64_t g[3];
        const int n = obsNodes(p, p.lm_obs_idx[a], g);
        for (int b = 0; b < n; ++b) ks.push_back(g[b]);
      }
    }
    std::sort(ks.begin(), ks.end());
    ks.erase(std::unique(ks.begin(), ks.end()), ks.end());
    for (size_t a = 0; a < ks.size(); ++a)
      for (size_t b = a; b < ks.size(); ++b) S->add(ks[a], ks[b]);
  }
  S->blocks.assign(S->bi.size() * 225, 0.0);
}

// Adds A^T B (A: R x 15-padded rows of width ca at column offset, etc.).
// Helper: block(i,j) += s * Ja^T Jb where Ja is R x 15, Jb is R x 15 (row-major).
static void addJtJ(BlockSystem* S, int64_t i, int64_t j, const double* Ja, const double* Jb, int R, double s) {
  const int64_t b = S->find(i, j);
  double* B = &S->blocks[225 * b];
  const bool swap = i > j;
  for (int r = 0; r < 15; ++r)
    for (int c = 0; c < 15; ++c) {
      double a = 0.0;
      for (int k = 0; k < R; ++k) a += Ja[15 * k + r] * Jb[15 * k + c];
      if (!swap) B[15 * r + c] += s * a;
      else B[15 * c + r] += s * a;
    }
}

static bool cholN(std::vector<double>& A, int n) {
  for (int j = 0; j < n; ++j) {
    double d = A[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) d -= A[(size_t)j * n + k] * A[(size_t)j * n + k];
    if (!(d > 0.0)) return false;
    const double l = std::sqrt(d);
    A[(size_t)j * n + j] = l;
    for (int i = j + 1; i < n; ++i) {
      double s = A[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) s -= A[(size_t)i * n + k] * A[(size_t)j * n + k];
      A[(size_t)i * n + j] = s / l;
    }
  }
  return true;
}
static void cholSolve(const std::vector<double>& L, int n, double* x) {
  for (int i = 0; i < n; ++i) {
    double s = x[i];
    for (int k = 0; k < i; ++k) s -= L[(size_t)i * n + k] * x[k];
    x[i] = s / L[(size_t)i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = x[i];
    for (int k = i + 1; k < n; ++k) s -= L[(size_t)k * n + i] * x[k];
    x[i] = s / L[(size_t)i * n + i];
  }
}
static bool inv3(const double* A, double* B) {
  const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                     A[2] * (A[3] * A[7] - A[4] * A[6]);
  if (!(std::fabs(det) > 0.0)) return false;
  const double id = 1.0 / det;
  B[0] = (A[4] * A[8] - A[5] * A[7]) * id; B[1] = (A[2] * A[7] - A[1] * A[8]) * id; B[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  B[3] = (A[5] * A[6] - A[3] * A[8]) * id; B[4] = (A[0] * A[8] - A[2] * A[6]) * id; B[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  B[6] = (A[3] * A[7] - A[4] * A[6]) * id; B[7] = (A[1] * A[6] - A[0] * A[7]) * id; B[8] = (A[0] * A[4] - A[1] * A[3]) * id;
  return true;
}

struct StepResult {
  std::vector<double> dc, dl, ds;  // scaled step (keyframes 15N, landmarks 3N, switches)
  int linear_iterations = 0;
  int status = 0;
};

struct Scaled {
  std::vector<double> skf, slm, ssw;  // Jacobi scale per tangent dim and per switch variable
};

// block(i, j) += s u v^T for 15-vectors u (rows of i) and v (rows of j).
static void addOuter(BlockSystem* S, int64_t i, int64_t j, const double* u, const double* v, double s) {
  double* B = &S->blocks[225 * S->find(i, j)];
  const bool swap = i > j;
  for (int r = 0; r < 15; ++r)
    for (int c = 0; c < 15; ++c) {
      if (!swap) B[15 * r + c] += s * u[r] * v[c];
      else B[15 * c + r] += s * u[r] * v[c];
    }
}

// Per switch variable of the pose edge j: the scaled Jacobian columns of the
// edge's two keyframes times the switch column (W_f, W_t), the switch's
// scaled gradient and J^T J (landmark-style elimination of a 1-dim block).
struct SwitchTerms {
  double W[30];  // W_f (15) | W_t (15)
  double g, h;   // scaled gradient, scaled J^T J (undamped)
};
static SwitchTerms switchTerms(const Problem& p, const Linearization& L, const Scaled& sc, int64_t j) {
  SwitchTerms o{};
  const int q = p.pe_swi[j];
  const int64_t e = p.nimu + j, f = p.e_from[e], t = p.e_to[e];
  const double ss = sc.ssw[q], w = p.sw_w[q], rp = (1.0 - p.sw[q]) * w;
  const double* js = &L.sJ[6 * j];
  double jj = w * w, g = -w * rp;
  for (int k = 0; k < 6; ++k) { jj += js[k] * js[k]; g += js[k] * L.ir[15 * e + k]; }
  o.h = jj * ss * ss;
  o.g = g * ss;
  for (int c = 0; c < 15; ++c) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < 6; ++k) { a += L.iJf[225 * e + 15 * k + c] * js[k]; b += L.iJt[225 * e + 15 * k + c] * js[k]; }
    o.W[c] = a * sc.skf[15 * f + c] * ss;
    o.W[15 + c] = b * sc.skf[15 * t + c] * ss;
  }
  return o;
}

// Solves (J^T J + D^2) d = -J^T r for the scaled Jacobian via Schur
// elimination of the landmarks.
// With dense_A / dense_b set, the reduced system (symmetric, n = 15 N_kf,
// row-major) and its right-hand side are written there and nothing is solved.
static StepResult computeStep(const Problem& p, const Linearization& L, const Scaled& sc,
                              const std::vector<double>& dkf, const std::vector<double>& dlm,
                              const std::vector<double>& dsw, const BlockSystem& pattern, int solver, int max_it,
                              double tol, double* dense_A = nullptr, double* dense_b = nullptr) {
  StepResult out;
  const int64_t N = p.nkf, NB = p.nkf + p.ng;  // keyframe blocks, then global nodes
  BlockSystem S = pattern;  // copies pattern + zeroed blocks
  std::fill(S.blocks.begin(), S.blocks.end(), 0.0);
  std::vector<double> bc(15 * NB, 0.0);  // rhs (-g_c initially)
  std::vector<double> Hll(9 * p.nlm, 0.0), gl(3 * p.nlm, 0.0);
  // Scaled node Jacobians of observation i: block ids (nkf + g) and 2 x 15 rows.
  auto nodeJ = [&](int64_t i, int64_t* nb, double (*Jn)[30]) -> int {
    if (p.ng == 0) return 0;
    int n = 0;
    for (int a = 0; a < 3; ++a) {
      const int g = L.vGn[3 * i + a];
      if (g < 0) continue;
      nb[n] = N + g;
      for (int c = 0; c < 30; ++c) Jn[n][c] = L.vG[90 * i + 30 * a + c] * sc.skf[15 * (N + g) + c % 15];
      ++n;
    }
    return n;
  };
  // Camera-camera terms and gradient.
  double Ja[2 * 15], Jb[2 * 15];
  for (int64_t i = 0; i < p.nobs; ++i) {
    const int l = p.obs_lm[i];
    const double* r = &L.vr[2 * i];
    const double* Jl = &L.vJl[6 * i];
    for (int a = 0; a < 3; ++a) {
      const double s = sc.slm[3 * l + a];
      for (int b = 0; b < 3; ++b)
        Hll[9 * l + 3 * a + b] += (Jl[a] * Jl[b] + Jl[3 + a] * Jl[3 + b]) * s * sc.slm[3 * l + b];
      gl[3 * l + a] += (Jl[a] * r[0] + Jl[3 + a] * r[1]) * s;
    }
    int64_t nb[3];
    double Jn[3][30];
    const int nn = nodeJ(i, nb, Jn);
    for (int a = 0; a < nn; ++a) {
      for (int b = a; b < nn; ++b) addJtJ(&S, nb[a], nb[b], Jn[a], Jn[b], 2, 1.0);
      for (int c = 0; c < 15; ++c) bc[15 * nb[a] + c] -= Jn[a][c] * r[0] + Jn[a][15 + c] * r[1];
    }
    if (p.obs_type[i] == MBA_LOCAL_KEYFRAME) continue;
    const int64_t ks = p.lm_store[l], ko = p.obs_kf[i];
    std::memset(Ja, 0, sizeof(Ja)); std::memset(Jb, 0, sizeof(Jb));
    for (int rr = 0; rr < 2; ++rr)
      for (int c = 0; c < 6; ++c) {
        Ja[15 * rr + c] = L.vJs[12 * i + 6 * rr + c] * sc.skf[15 * ks + c];
        Jb[15 * rr + c] = L.vJo[12 * i + 6 * rr + c] * sc.skf[15 * ko + c];
      }
    addJtJ(&S, ks, ks, Ja, Ja, 2, 1.0);
    addJtJ(&S, ko, ko, Jb, Jb, 2, 1.0);
    addJtJ(&S, ks, ko, Ja, Jb, 2, 1.0);
    for (int a = 0; a < nn; ++a) {
      addJtJ(&S, ks, nb[a], Ja, Jn[a], 2, 1.0);
      addJtJ(&S, ko, nb[a], Jb, Jn[a], 2, 1.0);
    }
    for (int c = 0; c < 6; ++c) {
      bc[15 * ks + c] -= Ja[c] * r[0] + Ja[15 + c] * r[1];
      bc[15 * ko + c] -= Jb[c] * r[0] + Jb[15 + c] * r[1];
    }
  }
  std::vector<double> Jf(225), Jt(225);
  for (int64_t e = 0; e < p.nedge; ++e) {
    const int64_t f = p.e_from[e], t = p.e_to[e];
    for (int rr = 0; rr < 15; ++rr)
      for (int c = 0; c < 15; ++c) {
        Jf[15 * rr + c] = L.iJf[225 * e + 15 * rr + c] * sc.skf[15 * f + c];
        Jt[15 * rr + c] = L.iJt[225 * e + 15 * rr + c] * sc.skf[15 * t + c];
      }
    addJtJ(&S, f, f, Jf.data(), Jf.data(), 15, 1.0);
    addJtJ(&S, t, t, Jt.data(), Jt.data(), 15, 1.0);
    addJtJ(&S, f, t, Jf.data(), Jt.data(), 15, 1.0);
    const double* r = &L.ir[15 * e];
    for (int c = 0; c < 15; ++c) {
      double a = 0.0, b = 0.0;
      for (int rr = 0; rr < 15; ++rr) { a += Jf[15 * rr + c] * r[rr]; b += Jt[15 * rr + c] * r[rr]; }
      bc[15 * f + c] -= a;
      bc[15 * t + c] -= b;
    }
  }
  // LM diagonal on keyframes and global nodes.
  for (int64_t k = 0; k < NB; ++k) {
    double* B = &S.blocks[225 * S.find(k, k)];
    for (int d = 0; d < 15; ++d) B[16 * d] += dkf[15 * k + d];
  }
  // Schur elimination per landmark.
  std::vector<double> Vinv(9 * p.nlm, 0.0);
  std::vector<int64_t> ks, gs;
  std::vector<double> W;   // per touched KF: 3 x 6
  std::vector<double> WG;  // per touched global node: 3 x 15
  for (int64_t l = 0; l < p.nlm; ++l) {
    if (!p.lm_mask[l]) continue;
    double H[9];
    for (int a = 0; a < 9; ++a) H[a] = Hll[9 * l + a];
    for (int a = 0; a < 3; ++a) H[4 * a] += dlm[3 * l + a];
    if (!inv3(H, &Vinv[9 * l])) { out.status = MBA_ERR_NOT_SPD; return out; }
    if (p.ng > 0) {
      // W of the landmark's global nodes: Wn = sum over its observations of J_l^T J_n.
      gs.clear();
      for (int64_t a = p.lm_obs_off[l]; a < p.lm_obs_off[l + 1]; ++a) {
        int64_t g[3];
        const int n = obsNodes(p, p.lm_obs_idx[a], g);
        for (int b = 0; b < n; ++b) gs.push_back(g[b]);
      }
      std::sort(gs.begin(), gs.end());
      gs.erase(std::unique(gs.begin(), gs.end()), gs.end());
      WG.assign(45 * gs.size(), 0.0);
      for (int64_t a = p.lm_obs_off[l]; a < p.lm_obs_off[l + 1]; ++a) {
        const int64_t i = p.lm_obs_idx[a];
        const double* Jl = &L.vJl[6 * i];
        int64_t nb[3];
        double Jn[3][30];
        const int nn = nodeJ(i, nb, Jn);
        for (int b = 0; b < nn; ++b) {
          const size_t pos = std::lower_bound(gs.begin(), gs.end(), nb[b]) - gs.begin();
          for (int x = 0; x < 3; ++x)
            for (int c = 0; c < 15; ++c)
              WG[45 * pos + 15 * x + c] += (Jl[x] * Jn[b][c] + Jl[3 + x] * Jn[b][15 + c]) * sc.slm[3 * l + x];
        }
      }
    }
    ks.clear();
    ks.push_back(p.lm_store[l]);
    for (int64_t a = p.lm_obs_off[l]; a < p.lm_obs_off[l + 1]; ++a) ks.push_back(p.obs_kf[p.lm_obs_idx[a]]);
    std::sort(ks.begin(), ks.end());
    ks.erase(std::unique(ks.begin(), ks.end()), ks.end());
    W.assign(18 * ks.size(), 0.0);
    for (int64_t a = p.lm_obs_off[l]; a < p.lm_obs_off[l + 1]; ++a) {
      const int64_t i = p.lm_obs_idx[a];
      if (p.obs_type[i] == MBA_LOCAL_KEYFRAME) continue;
      const double* Jl = &L.vJl[6 * i];
      const int64_t kk[2] = {p.lm_store[l], p.obs_kf[i]};
      const double* Jc[2] = {&L.vJs[12 * i], &L.vJo[12 * i]};
      for (int s = 0; s < 2; ++s) {
        const size_t pos = std::lower_bound(ks.begin(), ks.end(), kk[s]) - ks.begin();
        for (int x = 0; x < 3; ++x)
          for (int c = 0; c < 6; ++c)
            W[18 * pos + 6 * x + c] += (Jl[x] * Jc[s][c] + Jl[3 + x] * Jc[s][6 + c]) * sc.slm[3 * l + x] *
                                       sc.skf[15 * kk[s] + c];
      }
    }
    const double* Vi = &Vinv[9 * l];
    // VW = Vinv * W_j (3x6); S_ij -= W_i^T VW_j ; rhs_i += W_i^T Vinv g_l
    std::vector<double> VW(18 * ks.size());
    for (size_t j = 0; j < ks.size(); ++j)
      for (int x = 0; x < 3; ++x)
        for (int c = 0; c < 6; ++c)
          VW[18 * j + 6 * x + c] = Vi[3 * x] * W[18 * j + c] + Vi[3 * x + 1] * W[18 * j + 6 + c] + Vi[3 * x + 2] * W[18 * j + 12 + c];
    double Vg[3];
    for (int x = 0; x < 3; ++x) Vg[x] = Vi[3 * x] * gl[3 * l] + Vi[3 * x + 1] * gl[3 * l + 1] + Vi[3 * x + 2] * gl[3 * l + 2];
    for (size_t a = 0; a < ks.size(); ++a) {
      for (int c = 0; c < 6; ++c)
        bc[15 * ks[a] + c] += W[18 * a + c] * Vg[0] + W[18 * a + 6 + c] * Vg[1] + W[18 * a + 12 + c] * Vg[2];
      for (size_t b = a; b < ks.size(); ++b) {
        double* B = &S.blocks[225 * S.find(ks[a], ks[b])];
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c) {
            const double v = W[18 * a + r] * VW[18 * b + c] + W[18 * a + 6 + r] * VW[18 * b + 6 + c] +
                             W[18 * a + 12 + r] * VW[18 * b + 12 + c];
            B[15 * r + c] -= v;  // ks sorted => a<=b => (ks[a], ks[b]) is the stored orientation
          }
      }
    }
    if (!gs.empty()) {
      // Global nodes: VWn = Vinv Wn; S(kf, n) -= W_kf^T VWn, S(n_a, n_b) -= Wn_a^T VWn_b,
      // rhs_n += Wn^T Vinv g_l.  Node blocks come after every keyframe block.
      std::vector<double> VWG(45 * gs.size());
      for (size_t j = 0; j < gs.size(); ++j)
        for (int x = 0; x < 3; ++x)
          for (int c = 0; c < 15; ++c)
            VWG[45 * j + 15 * x + c] = Vi[3 * x] * WG[45 * j + c] + Vi[3 * x + 1] * WG[45 * j + 15 + c] +
                                       Vi[3 * x + 2] * WG[45 * j + 30 + c];
      for (size_t b = 0; b < gs.size(); ++b) {
        for (int c = 0; c < 15; ++c)
          bc[15 * gs[b] + c] += WG[45 * b + c] * Vg[0] + WG[45 * b + 15 + c] * Vg[1] + WG[45 * b + 30 + c] * Vg[2];
        for (size_t a = 0; a < ks.size(); ++a) {
          double* B = &S.blocks[225 * S.find(ks[a], gs[b])];
          for (int r = 0; r < 6; ++r)
            for (int c = 0; c < 15; ++c)
              B[15 * r + c] -= W[18 * a + r] * VWG[45 * b + c] + W[18 * a + 6 + r] * VWG[45 * b + 15 + c] +
                               W[18 * a + 12 + r] * VWG[45 * b + 30 + c];
        }
        for (size_t a = 0; a <= b; ++a) {
          double* B = &S.blocks[225 * S.find(gs[a], gs[b])];
          for (int r = 0; r < 15; ++r)
            for (int c = 0; c < 15; ++c)
              B[15 * r + c] -= WG[45 * a + r] * VWG[45 * b + c] + WG[45 * a + 15 + r] * VWG[45 * b + 15 + c] +
                               WG[45 * a + 30 + r] * VWG[45 * b + 30 + c];
        }
      }
    }
  }
  // Schur elimination of each switch variable: S_ab -= W_a W_b^T / H,
  // rhs_a += W_a g / H for a, b in {from, to}.
  const int64_t npe = p.nedge - p.nimu;
  std::vector<SwitchTerms> swt(npe);
  for (int64_t j = 0; j < npe; ++j) {
    const int q = p.pe_swi[j];
    if (q < 0) continue;
    swt[j] = switchTerms(p, L, sc, j);
    SwitchTerms& w = swt[j];
    w.h += dsw[q];
    const int64_t e = p.nimu + j, f = p.e_from[e], t = p.e_to[e];
    const double hi = 1.0 / w.h;
    addOuter(&S, f, f, w.W, w.W, -hi);
    addOuter(&S, t, t, w.W + 15, w.W + 15, -hi);
    addOuter(&S, f, t, w.W, w.W + 15, -hi);
    for (int c = 0; c < 15; ++c) {
      bc[15 * f + c] += w.W[c] * hi * w.g;
      bc[15 * t + c] += w.W[15 + c] * hi * w.g;
    }
  }
  // Masked keyframe dims: identity rows, zero rhs.
  for (size_t b = 0; b < S.bi.size(); ++b) {
    const int64_t i = S.bi[b], j = S.bj[b];
    double* B = &S.blocks[225 * b];
    for (int r = 0; r < 15; ++r)
      for (int c = 0; c < 15; ++c)
        if (!dimActive(p, i, r) || !dimActive(p, j, c)) B[15 * r + c] = (i == j && r == c) ? 1.0 : 0.0;
  }
  for (int64_t k = 0; k < NB; ++k)
    for (int d = 0; d < 15; ++d)
      if (!dimActive(p, k, d)) bc[15 * k + d] = 0.0;

  if (dense_A) {
    const size_t n = 15 * NB;
    std::fill(dense_A, dense_A + n * n, 0.0);
    for (size_t b = 0; b < S.bi.size(); ++b) {
      const int64_t i = S.bi[b], j = S.bj[b];
      const double* B = &S.blocks[225 * b];
      for (int r = 0; r < 15; ++r)
        for (int c = 0; c < 15; ++c) {
          dense_A[(15 * i + r) * n + 15 * j + c] = B[15 * r + c];
          dense_A[(15 * j + c) * n + 15 * i + r] = B[15 * r + c];
        }
    }
    std::copy(bc.begin(), bc.end(), dense_b);
    return out;
  }
  std::vector<double> x(15 * NB, 0.0);
  if (solver == MBA_LINEAR_SOLVER_DENSE_SCHUR) {
    const int n = (int)(15 * NB);
    std::vector<double> A((size_t)n * n, 0.0);
    for (size_t b = 0; b < S.bi.size(); ++b) {
      const int64_t i = S.bi[b], j = S.bj[b];
      const double* B = &S.blocks[225 * b];
      for (int r = 0; r < 15; ++r)
        for (int c = 0; c < 15; ++c) {
          A[(size_t)(15 * i + r) * n + 15 * j + c] = B[15 * r + c];
          A[(size_t)(15 * j + c) * n + 15 * i + r] = B[15 * r + c];
        }
    }
    if (!cholN(A, n)) { out.status = MBA_ERR_NOT_SPD; return out; }
    x = bc;
    cholSolve(A, n, x.data());
    out.linear_iterations = 1;
  } else {
    // Block-Jacobi PCG on S x = bc.
    std::vector<std::vector<double>> Linv(NB);
    for (int64_t k = 0; k < NB; ++k) {
      std::vector<double> B(S.blocks.begin() + 225 * S.find(k, k), S.blocks.begin() + 225 * S.find(k, k) + 225);
      if (!cholN(B, 15)) { out.status = MBA_ERR_NOT_SPD; return out; }
      Linv[k] = B;
    }
    auto spmv = [&](const std::vector<double>& in, std::vector<double>& o) {
      std::fill(o.begin(), o.end(), 0.0);
      for (size_t b = 0; b < S.bi.size(); ++b) {
        const int64_t i = S.bi[b], j = S.bj[b];
        const double* B = &S.blocks[225 * b];
        for (int r = 0; r < 15; ++r) {
          double a = 0.0;
          for (int c = 0; c < 15; ++c) a += B[15 * r + c] * in[15 * j + c];
          o[15 * i + r] += a;
        }
        if (i != j)
          for (int c = 0; c < 15; ++c) {
            double a = 0.0;
            for (int r = 0; r < 15; ++r) a += B[15 * r + c] * in[15 * i + r];
            o[15 * j + c] += a;
          }
      }
    };
    auto precond = [&](const std::vector<double>& in, std::vector<double>& o) {
      o = in;
      for (int64_t k = 0; k < NB; ++k) cholSolve(Linv[k], 15, &o[15 * k]);
    };
    std::vector<double> r = bc, z(15 * NB), pp(15 * NB), q(15 * NB);
    double bnorm = 0.0;
    for (double v : bc) bnorm += v * v;
    bnorm = std::sqrt(bnorm);
    precond(r, z);
    pp = z;
    double rz = 0.0;
    for (int64_t a = 0; a < 15 * NB; ++a) rz += r[a] * z[a];
    int it = 0;
    if (bnorm > 0.0) {
      for (it = 0; it < max_it; ++it) {
        spmv(pp, q);
        double pq = 0.0;
        for (int64_t a = 0; a < 15 * NB; ++a) pq += pp[a] * q[a];
        const double alpha = rz / pq;
        double rn = 0.0;
        for (int64_t a = 0; a < 15 * NB; ++a) { x[a] += alpha * pp[a]; r[a] -= alpha * q[a]; rn += r[a] * r[a]; }
        if (std::sqrt(rn) <= tol * bnorm) { ++it; break; }
        precond(r, z);
        double rz2 = 0.0;
        for (int64_t a = 0; a < 15 * NB; ++a) rz2 += r[a] * z[a];
        const double beta = rz2 / rz;
        rz = rz2;
        for (int64_t a = 0; a < 15 * NB; ++a) pp[a] = z[a] + beta * pp[a];
      }
    }
    out.linear_iterations = it;
  }
  // Back substitution: dl = Vinv (-g_l - W dc).
  out.dc = x;
  out.dl.assign(3 * p.nlm, 0.0);
  std::vector<double> t(3 * p.nlm, 0.0);
  for (int64_t l = 0; l < p.nlm; ++l) for (int a = 0; a < 3; ++a) t[3 * l + a] = -gl[3 * l + a];
  for (int64_t i = 0; i < p.nobs; ++i) {
    const int l = p.obs_lm[i];
    if (!p.lm_mask[l]) continue;
    const double* Jl = &L.vJl[6 * i];
    double u[2] = {0.0, 0.0};
    if (p.obs_type[i] != MBA_LOCAL_KEYFRAME) {
      const int64_t ks2 = p.lm_store[l], ko = p.obs_kf[i];
      for (int rr = 0; rr < 2; ++rr)
        for (int c = 0; c < 6; ++c)
          u[rr] += L.vJs[12 * i + 6 * rr + c] * sc.skf[15 * ks2 + c] * x[15 * ks2 + c] +
                   L.vJo[12 * i + 6 * rr + c] * sc.skf[15 * ko + c] * x[15 * ko + c];
    }
    int64_t nb[3];
    double Jn[3][30];
    const int nn = nodeJ(i, nb, Jn);
    for (int a = 0; a < nn; ++a)
      for (int rr = 0; rr < 2; ++rr)
        for (int c = 0; c < 15; ++c) u[rr] += Jn[a][15 * rr + c] * x[15 * nb[a] + c];
    for (int a = 0; a < 3; ++a) t[3 * l + a] -= (Jl[a] * u[0] + Jl[3 + a] * u[1]) * sc.slm[3 * l + a];
  }
  for (int64_t l = 0; l < p.nlm; ++l) {
    if (!p.lm_mask[l]) continue;
    const double* Vi = &Vinv[9 * l];
    for (int a = 0; a < 3; ++a)
      out.dl[3 * l + a] = Vi[3 * a] * t[3 * l] + Vi[3 * a + 1] * t[3 * l + 1] + Vi[3 * a + 2] * t[3 * l + 2];
  }
  // Switches: ds = (-g - W_f^T dc_f - W_t^T dc_t) / H.
  out.ds.assign(p.sw.size(), 0.0);
  for (int64_t j = 0; j < npe; ++j) {
    const int q = p.pe_swi[j];
    if (q < 0) continue;
    const int64_t e = p.nimu + j, f = p.e_from[e], te = p.e_to[e];
    double u = -swt[j].g;
    for (int c = 0; c < 15; ++c) u -= swt[j].W[c] * x[15 * f + c] + swt[j].W[15 + c] * x[15 * te + c];
    out.ds[q] = u / swt[j].h;
  }
  return out;
}

// Retraction of the full state by the unscaled tangent step.
static void plusState(const Problem& p, const std::vector<double>& dkf, const std::vector<double>& dlm,
                      std::vector<double>* kx, std::vector<double>* kv, std::vector<double>* kbg,
                      std::vector<double>* kba, std::vector<double>* lp) {
  for (int64_t k = 0; k < p.nkf; ++k) {
    const double* d = &dkf[15 * k];
    const uint8_t* m = &p.kf_mask[15 * k];
    double* x = &(*kx)[7 * k];
    if (p.kf_flags[k] & MBA_KF_GAUGE_ROLL_PITCH) {
      if (m[0] || m[1]) {
        double q[4];
        const double d2[2] = {d[0], d[1]};
        jplRollPitchPlus(&p.mis[7 * p.kf_mis[k]], x, d2, q);
        std::memcpy(x, q, sizeof(q));
      }
    } else if (m[0] || m[1] || m[2]) {
      double q[4];
      jplQuaternionPlus(x, d, q);
      std::memcpy(x, q, sizeof(q));
    }
    for (int i = 0; i < 3; ++i) {
      if (m[3 + i]) x[4 + i] += d[3 + i];
      if (m[6 + i]) (*kv)[3 * k + i] += d[6 + i];
      if (m[9 + i]) (*kbg)[3 * k + i] += d[9 + i];
      if (m[12 + i]) (*kba)[3 * k + i] += d[12 + i];
    }
  }
  for (int64_t l = 0; l < p.nlm; ++l)
    if (p.lm_mask[l])
      for (int i = 0; i < 3; ++i) (*lp)[3 * l + i] += dlm[3 * l + i];
}

// Retraction of the global nodes by the unscaled tangent step (dkf holds the
// keyframe blocks, then the nodes): intrinsics, distortion and p_C_I add,
// q_C_I by JplQuaternionParameterization::Plus; a baseframe by
// JplPoseParameterization or JplYawOnlyPoseParameterization (the yaw Plus of
// quaternion-param-jpl.cc:78-105 and an added position).
static void plusNodes(const Problem& p, const std::vector<double>& dkf, std::vector<mba_camera>* cams,
                      std::vector<double>* mis) {
  for (int64_t g = 0; g < p.ng; ++g) {
    const double* d = &dkf[15 * (p.nkf + g)];
    const uint8_t* m = &p.g_mask[15 * g];
    if (p.node_cam[g] >= 0) {
      mba_camera& c = (*cams)[p.node_cam[g]];
      for (int a = 0; a < 4; ++a) {
        if (m[a]) c.intrinsics[a] += d[a];
        if (m[4 + a]) c.distortion[a] += d[4 + a];
      }
      if (m[8] || m[9] || m[10]) {
        double q[4];
        jplQuaternionPlus(c.q_CI_p_CI, d + 8, q);
        std::memcpy(c.q_CI_p_CI, q, sizeof(q));
      }
      for (int a = 0; a < 3; ++a)
        if (m[11 + a]) c.q_CI_p_CI[4 + a] += d[11 + a];
    } else {
      const int mi = p.node_mis[g];
      double* x = &(*mis)[7 * mi];
      double q[4];
      if (p.mis_flags[mi] == MBA_MIS_BASEFRAME_YAW_POSITION) jplYawPlus(x, d, q);
      else jplQuaternionPlus(x, d, q);
      std::memcpy(x, q, sizeof(q));
      for (int a = 0; a < 3; ++a) x[4 + a] += d[3 + a];
    }
  }
}

// Switch retraction: plain addition projected onto the bounds [0, 1], as
// Ceres applies parameter bounds after Plus.
static void plusSwitches(const std::vector<double>& ds, std::vector<double>* sw) {
  for (size_t q = 0; q < sw->size(); ++q) (*sw)[q] = std::min(1.0, std::max(0.0, (*sw)[q] + ds[q]));
}

// Jacobi scaling 1 / (1 + |column|) and the column norms of the Jacobian.
static void columnNorms(const Problem& p, const Linearization& L, std::vector<double>& nkf, std::vector<double>& nlm,
                        std::vector<double>& nsw) {
  nkf.assign(15 * (p.nkf + p.ng), 0.0);  // keyframe blocks, then the global nodes
  nlm.assign(3 * p.nlm, 0.0);
  nsw.assign(p.sw.size(), 0.0);
  for (int64_t j = 0; j < p.nedge - p.nimu; ++j) {
    const int q = p.pe_swi[j];
    if (q < 0) continue;
    double a = p.sw_w[q] * p.sw_w[q];
    for (int k = 0; k < 6; ++k) a += L.sJ[6 * j + k] * L.sJ[6 * j + k];
    nsw[q] = a;
  }
  for (int64_t i = 0; i < p.nobs; ++i) {
    const int l = p.obs_lm[i];
    for (int a = 0; a < 3; ++a) nlm[3 * l + a] += L.vJl[6 * i + a] * L.vJl[6 * i + a] + L.vJl[6 * i + 3 + a] * L.vJl[6 * i + 3 + a];
    for (int a = 0; a < 3 && p.ng > 0; ++a) {
      const int g = L.vGn[3 * i + a];
      if (g < 0) continue;
      const double* J = &L.vG[90 * i + 30 * a];
      for (int c = 0; c < 15; ++c) nkf[15 * (p.nkf + g) + c] += J[c] * J[c] + J[15 + c] * J[15 + c];
    }
    if (p.obs_type[i] == MBA_LOCAL_KEYFRAME) continue;
    const int64_t ks = p.lm_store[l], ko = p.obs_kf[i];
    for (int c = 0; c < 6; ++c) {
      nkf[15 * ks + c] += L.vJs[12 * i + c] * L.vJs[12 * i + c] + L.vJs[12 * i + 6 + c] * L.vJs[12 * i + 6 + c];
      nkf[15 * ko + c] += L.vJo[12 * i + c] * L.vJo[12 * i + c] + L.vJo[12 * i + 6 + c] * L.vJo[12 * i + 6 + c];
    }
  }
  for (int64_t e = 0; e < p.nedge; ++e)
    for (int c = 0; c < 15; ++c)
      for (int r = 0; r < 15; ++r) {
        nkf[15 * p.e_from[e] + c] += L.iJf[225 * e + 15 * r + c] * L.iJf[225 * e + 15 * r + c];
        nkf[15 * p.e_to[e] + c] += L.iJt[225 * e + 15 * r + c] * L.iJt[225 * e + 15 * r + c];
      }
}

// Max |g| of the robustified gradient g = J^T r over every variable tangent
// dim (keyframes, landmarks, switch variables, global nodes), unscaled.
static double gradientMaxNorm(const Problem& p, const Linearization& L) {
  std::vector<double> gk(15 * (p.nkf + p.ng), 0.0), gl(3 * p.nlm, 0.0), gs(p.sw.size(), 0.0);
  for (int64_t i = 0; i < p.nobs; ++i) {
    const int l = p.obs_lm[i];
    const double* r = &L.vr[2 * i];
    for (int a = 0; a < 3; ++a) gl[3 * l + a] += L.vJl[6 * i + a] * r[0] + L.vJl[6 * i + 3 + a] * r[1];
    if (p.obs_type[i] != MBA_LOCAL_KEYFRAME) {
      const int64_t ks = p.lm_store[l], ko = p.obs_kf[i];
      for (int c = 0; c < 6; ++c) {
        gk[15 * ks + c] += L.vJs[12 * i + c] * r[0] + L.vJs[12 * i + 6 + c] * r[1];
        gk[15 * ko + c] += L.vJo[12 * i + c] * r[0] + L.vJo[12 * i + 6 + c] * r[1];
      }
    }
    for (int a = 0; a < 3 && p.ng > 0; ++a) {
      const int g = L.vGn[3 * i + a];
      if (g < 0) continue;
      const double* J = &L.vG[90 * i + 30 * a];
      for (int c = 0; c < 15; ++c) gk[15 * (p.nkf + g) + c] += J[c] * r[0] + J[15 + c] * r[1];
    }
  }
  for (int64_t e = 0; e < p.nedge; ++e) {
    const double* r = &L.ir[15 * e];
    for (int c = 0; c < 15; ++c)
      for (int rr = 0; rr < 15; ++rr) {
        gk[15 * p.e_from[e] + c] += L.iJf[225 * e + 15 * rr + c] * r[rr];
        gk[15 * p.e_to[e] + c] += L.iJt[225 * e + 15 * rr + c] * r[rr];
      }
    const int q = e >= p.nimu ? p.pe_swi[e - p.nimu] : -1;
    if (q >= 0) {
      const double w = p.sw_w[q];
      double v = -w * (1.0 - p.sw[q]) * w;
      for (int k = 0; k < 6; ++k) v += L.sJ[6 * (e - p.nimu) + k] * r[k];
      gs[q] = v;
    }
  }
  double m = 0.0;
  for (int64_t k = 0; k < p.nkf + p.ng; ++k)
    for (int d = 0; d < 15; ++d)
      if (dimActive(p, k, d)) m = std::max(m, std::fabs(gk[15 * k + d]));
  for (int64_t l = 0; l < p.nlm; ++l)
    if (p.lm_mask[l] && !p.lm_off[l])
      for (int a = 0; a < 3; ++a) m = std::max(m, std::fabs(gl[3 * l + a]));
  for (double v : gs) m = std::max(m, std::fabs(v));
  return m;
}

// findOutlierLandmarks (outlier-rejection-solver.cc:28-103): a landmark is
// an outlier if one of its observations has camera depth <= 0 or, with
// use_reprojection_error, a squared pixel error above the threshold.
// Returns the number of newly rejected landmarks.
static int64_t rejectOutlierLandmarks(Problem& p, const mba_solver_options& o) {
  int64_t n = 0;
  const double max2 = o.outlier_max_reprojection_error_px * o.outlier_max_reprojection_error_px;
  std::vector<uint8_t> out(p.nlm, 0);
  for (int64_t i = 0; i < p.nobs; ++i) {
    const int l = p.obs_lm[i];
    if (p.lm_off[l] || out[l]) continue;
    const double* P[9];
    visualParams(p, i, P);
    double pc[3];
    visualPointInCamera(P, p.obs_type[i], pc);
    bool bad = !(pc[2] > 0.0);
    if (!bad && o.outlier_use_reprojection_error) {
      double kp[2];
      pinholeProject3(p.cams[p.obs_cam[i]], pc, kp, nullptr, nullptr, nullptr);
      const double e0 = kp[0] - p.obs_uv[2 * i], e1 = kp[1] - p.obs_uv[2 * i + 1];
      bad = !(e0 * e0 + e1 * e1 <= max2);
    }
    if (bad) out[l] = 1;
  }
  for (int64_t l = 0; l < p.nlm; ++l)
    if (out[l]) { p.lm_off[l] = 1; ++n; }
  return n;
}

int solve(Problem& p, const mba_solver_options& o, mba_summary* sum) {
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  Linearization L;
  int st = linearize(p, true, &L);
  if (st) return st;
  Scaled sc;
  sc.skf.assign(15 * (p.nkf + p.ng), 1.0);
  sc.slm.assign(3 * p.nlm, 1.0);
  sc.ssw.assign(p.sw.size(), 1.0);
  std::vector<double> nkf, nlm, nsw;
  auto colnorms = [&]() { columnNorms(p, L, nkf, nlm, nsw); };
  auto jacobi = [&]() {
    if (!o.jacobi_scaling) return;
    for (size_t a = 0; a < nkf.size(); ++a) sc.skf[a] = 1.0 / (1.0 + std::sqrt(nkf[a]));
    for (size_t a = 0; a < nlm.size(); ++a) sc.slm[a] = 1.0 / (1.0 + std::sqrt(nlm[a]));
    for (size_t a = 0; a < nsw.size(); ++a) sc.ssw[a] = 1.0 / (1.0 + std::sqrt(nsw[a]));
  };
  colnorms();
  jacobi();
  BlockSystem pattern;
  buildPattern(p, &pattern);
  // Ceres' gradient test (TrustRegionMinimizer): max |J^T r| over the
  // variable tangent dims at or below gradient_tolerance ends the solve, at
  // the start and after each accepted step.
  auto gradient_converged = [&]() {
    if (!o.check_tolerances) return false;
    return gradientMaxNorm(p, L) <= o.gradient_tolerance;
  };

  double cost = L.cost;
  double radius = o.initial_trust_region_radius;
  double decrease_factor = 2.0;
  bool reuse_diag = false;
  std::vector<double> dkf(15 * (p.nkf + p.ng)), dlm(3 * p.nlm), dsw(p.sw.size());
  if (sum) {
    sum->initial_cost = cost;
    sum->num_iterations = 0;
    sum->num_successful_steps = 0;
    sum->termination = 0;
    sum->total_linear_iterations = 0;
    sum->time_to_stop_cost_ms = -1.0;
  }
  auto record = [&](int iter, bool ok, int lin, double c, double dc, double sn, double rd) {
    if (!sum) return;
    if (sum->iterations && iter < sum->max_iterations_capacity) {
      mba_iteration_summary& it = sum->iterations[iter];
      it.iteration = iter; it.step_is_successful = ok; it.linear_solver_iterations = lin;
      it.cost = c; it.cost_change = dc; it.gradient_max_norm = 0.0; it.step_norm = sn;
      it.relative_decrease = rd; it.trust_region_radius = radius;
      it.iteration_time_ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    }
    sum->num_iterations = iter + 1;
  };
  record(0, true, 0, cost, 0.0, 0.0, 0.0);
  if (sum && o.stop_cost > 0 && cost <= o.stop_cost) { sum->termination = 6; sum->time_to_stop_cost_ms = 0.0; }
  bool done = false;
  if (gradient_converged()) {
    if (sum) sum->termination = 2;
    done = true;
  }
  int64_t rejected = 0;
  for (int iter = 1; iter <= o.max_num_iterations && !done; ++iter) {
    if (sum && sum->termination == 6) break;
    // solveWithOutlierRejection (outlier-rejection-solver.cc:199-259): every
    // n iterations the Ceres solve ends, outlier landmarks are removed and a
    // new solve starts from the last trust-region radius (fresh evaluation,
    // Jacobi scaling and decrease factor).
    const int nrej = o.reject_outliers_every_n_iters;
    if (nrej > 0 && iter > 1 && (iter - 1) % nrej == 0) {
      rejected += rejectOutlierLandmarks(p, o);
      st = linearize(p, true, &L);
      if (st) return st;
      cost = L.cost;
      colnorms();
      jacobi();
      decrease_factor = 2.0;
      reuse_diag = false;
    }
    // LM diagonal from the scaled Jacobian column norms.
    if (!reuse_diag) {
      colnorms();
      for (size_t a = 0; a < nkf.size(); ++a) nkf[a] = std::min(std::max(nkf[a] * sc.skf[a] * sc.skf[a], o.min_lm_diagonal), o.max_lm_diagonal);
      for (size_t a = 0; a < nlm.size(); ++a) nlm[a] = std::min(std::max(nlm[a] * sc.slm[a] * sc.slm[a], o.min_lm_diagonal), o.max_lm_diagonal);
      for (size_t a = 0; a < nsw.size(); ++a) nsw[a] = std::min(std::max(nsw[a] * sc.ssw[a] * sc.ssw[a], o.min_lm_diagonal), o.max_lm_diagonal);
    }
    for (size_t a = 0; a < nkf.size(); ++a) dkf[a] = nkf[a] / radius;
    for (size_t a = 0; a < nlm.size(); ++a) dlm[a] = nlm[a] / radius;
    for (size_t a = 0; a < nsw.size(); ++a) dsw[a] = nsw[a] / radius;
    StepResult s = computeStep(p, L, sc, dkf, dlm, dsw, pattern, o.linear_solver, o.max_linear_iterations,
                               o.linear_tolerance);
    if (sum) sum->total_linear_iterations += s.linear_iterations;
    double mcc = 0.0;
    if (s.status == 0) {
      // model_cost_change = -J d . (r + J d / 2)
      for (int64_t i = 0; i < p.nobs; ++i) {
        const int l = p.obs_lm[i];
        double u[2] = {0.0, 0.0};
        for (int rr = 0; rr < 2; ++rr) {
          for (int a = 0; a < 3; ++a) u[rr] += L.vJl[6 * i + 3 * rr + a] * sc.slm[3 * l + a] * s.dl[3 * l + a];
          if (p.obs_type[i] != MBA_LOCAL_KEYFRAME) {
            const int64_t ks = p.lm_store[l], ko = p.obs_kf[i];
            for (int c = 0; c < 6; ++c)
              u[rr] += L.vJs[12 * i + 6 * rr + c] * sc.skf[15 * ks + c] * s.dc[15 * ks + c] +
                       L.vJo[12 * i + 6 * rr + c] * sc.skf[15 * ko + c] * s.dc[15 * ko + c];
          }
          for (int a = 0; a < 3 && p.ng > 0; ++a) {
            const int g = L.vGn[3 * i + a];
            if (g < 0) continue;
            const int64_t b = p.nkf + g;
            for (int c = 0; c < 15; ++c)
              u[rr] += L.vG[90 * i + 30 * a + 15 * rr + c] * sc.skf[15 * b + c] * s.dc[15 * b + c];
          }
        }
        mcc -= u[0] * (L.vr[2 * i] + u[0] / 2.0) + u[1] * (L.vr[2 * i + 1] + u[1] / 2.0);
      }
      for (int64_t e = 0; e < p.nedge; ++e) {
        const int64_t f = p.e_from[e], t = p.e_to[e];
        const int q = e >= p.nimu ? p.pe_swi[e - p.nimu] : -1;
        for (int rr = 0; rr < 15; ++rr) {
          double u = 0.0;
          for (int c = 0; c < 15; ++c)
            u += L.iJf[225 * e + 15 * rr + c] * sc.skf[15 * f + c] * s.dc[15 * f + c] +
                 L.iJt[225 * e + 15 * rr + c] * sc.skf[15 * t + c] * s.dc[15 * t + c];
          if (q >= 0 && rr < 6) u += L.sJ[6 * (e - p.nimu) + rr] * sc.ssw[q] * s.ds[q];
          mcc -= u * (L.ir[15 * e + rr] + u / 2.0);
        }
        if (q >= 0) {  // switch prior: r = (1 - s) w, J = -w
          const double w = p.sw_w[q], u = -w * sc.ssw[q] * s.ds[q];
          mcc -= u * ((1.0 - p.sw[q]) * w + u / 2.0);
        }
      }
    }
    if (s.status != 0 || !(mcc > 0.0) || !std::isfinite(mcc)) {
      radius /= decrease_factor;
      decrease_factor *= 2.0;
      reuse_diag = true;
      record(iter, false, s.linear_iterations, cost, 0.0, 0.0, 0.0);
      if (radius < o.min_trust_region_radius) { if (sum) sum->termination = 4; break; }
      continue;
    }
    // Unscale and retract.
    std::vector<double> ukf(15 * (p.nkf + p.ng)), ulm(3 * p.nlm), usw(p.sw.size());
    for (size_t a = 0; a < ukf.size(); ++a) ukf[a] = s.dc[a] * sc.skf[a];
    for (size_t a = 0; a < ulm.size(); ++a) ulm[a] = s.dl[a] * sc.slm[a];
    for (size_t a = 0; a < usw.size(); ++a) usw[a] = s.ds[a] * sc.ssw[a];
    std::vector<double> kx = p.kf_x, kv = p.kf_v, kbg = p.kf_bg, kba = p.kf_ba, lp = p.lm_p, swv = p.sw;
    std::vector<mba_camera> cams = p.cams;
    std::vector<double> mis = p.mis;
    plusState(p, ukf, ulm, &kx, &kv, &kbg, &kba, &lp);
    plusSwitches(usw, &swv);
    if (p.ng > 0) plusNodes(p, ukf, &cams, &mis);
    auto swap_state = [&]() {
      std::swap(kx, p.kf_x); std::swap(kv, p.kf_v); std::swap(kbg, p.kf_bg); std::swap(kba, p.kf_ba);
      std::swap(lp, p.lm_p); std::swap(swv, p.sw);
      std::swap(cams, p.cams); std::swap(mis, p.mis);
    };
    swap_state();
    Linearization Lc;
    const int cst = linearize(p, false, &Lc);
    const double new_cost = cst ? INFINITY : Lc.cost;
    // parameter tolerance bookkeeping (ambient step norm)
    double step_norm = 0.0, x_norm = 0.0;
    // (Ceres: norms of the ambient step and state over the parameter blocks
    // of the reduced program, i.e. the non-constant blocks)
    auto any = [&](int64_t k, int a0, int a1) {
      for (int a = a0; a < a1; ++a)
        if (p.kf_mask[15 * k + a]) return true;
      return false;
    };
    auto add = [&](const std::vector<double>& now, const std::vector<double>& old, int64_t b, int n) {
      for (int a = 0; a < n; ++a) {
        const double dd = now[n * b + a] - old[n * b + a];
        step_norm += dd * dd;
        x_norm += old[n * b + a] * old[n * b + a];
      }
    };
    for (int64_t k = 0; k < p.nkf; ++k) {
      if (any(k, 0, 6)) add(p.kf_x, kx, k, 7);
      if (any(k, 6, 9)) add(p.kf_v, kv, k, 3);
      if (any(k, 9, 12)) add(p.kf_bg, kbg, k, 3);
      if (any(k, 12, 15)) add(p.kf_ba, kba, k, 3);
    }
    for (int64_t l = 0; l < p.nlm; ++l)
      if (p.lm_mask[l]) add(p.lm_p, lp, l, 3);
    auto addv = [&](const double* now, const double* old, int n) {
      for (int a = 0; a < n; ++a) {
        step_norm += (now[a] - old[a]) * (now[a] - old[a]);
        x_norm += old[a] * old[a];
      }
    };
    for (int64_t g = 0; g < p.ng; ++g) {
      const uint8_t* m = &p.g_mask[15 * g];
      if (p.node_cam[g] >= 0) {
        const int c = p.node_cam[g];
        const mba_camera &now = p.cams[c], &old = cams[c];
        if (m[0]) addv(now.intrinsics, old.intrinsics, 4);
        if (m[4]) addv(now.distortion, old.distortion, distortionParams(old.distortion_type));
        if (m[8]) addv(now.q_CI_p_CI, old.q_CI_p_CI, 4);
        if (m[11]) addv(now.q_CI_p_CI + 4, old.q_CI_p_CI + 4, 3);
      } else {
        addv(&p.mis[7 * p.node_mis[g]], &mis[7 * p.node_mis[g]], 7);
      }
    }
    for (size_t a = 0; a < swv.size(); ++a) { const double dd = p.sw[a] - swv[a]; step_norm += dd * dd; x_norm += swv[a] * swv[a]; }
    step_norm = std::sqrt(step_norm);
    x_norm = std::sqrt(x_norm);
    const double rel = (cost - new_cost) / mcc;
    const bool ok = std::isfinite(new_cost) && rel > o.min_relative_decrease;
    if (o.check_tolerances && step_norm <= o.parameter_tolerance * (x_norm + o.parameter_tolerance)) {
      if (!ok) swap_state();
      record(iter, ok, s.linear_iterations, ok ? new_cost : cost, cost - new_cost, step_norm, rel);
      if (ok) cost = new_cost;
      if (sum) sum->termination = 3;
      break;
    }
    if (o.check_tolerances && std::fabs(cost - new_cost) <= o.function_tolerance * cost) {
      if (!ok) swap_state();
      record(iter, ok, s.linear_iterations, ok ? new_cost : cost, cost - new_cost, step_norm, rel);
      if (ok) cost = new_cost;
      if (sum) sum->termination = 1;
      break;
    }
    if (ok) {
      const double prev = cost;
      cost = new_cost;
      st = linearize(p, true, &L);
      if (st) return st;
      radius = radius / std::max(1.0 / 3.0, 1.0 - std::pow(2.0 * rel - 1.0, 3));
      radius = std::min(radius, o.max_trust_region_radius);
      decrease_factor = 2.0;
      reuse_diag = false;
      if (sum) sum->num_successful_steps++;
      record(iter, true, s.linear_iterations, cost, prev - cost, step_norm, rel);
      if (sum && o.stop_cost > 0 && cost <= o.stop_cost && sum->time_to_stop_cost_ms < 0) {
        sum->time_to_stop_cost_ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
        sum->termination = 6;
      }
      if (gradient_converged()) {
        if (sum) sum->termination = 2;
        break;
      }
    } else {
      swap_state();
      radius /= decrease_factor;
      decrease_factor *= 2.0;
      reuse_diag = true;
      record(iter, false, s.linear_iterations, cost, cost - new_cost, step_norm, rel);
    }
    if (radius < o.min_trust_region_radius) { if (sum) sum->termination = 4; break; }
  }
  if (sum) {
    sum->final_cost = cost;
    sum->total_time_ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    sum->num_rejected_landmarks = (int32_t)rejected;
  }
  return MBA_OK;
}

// The damped, Jacobi-scaled reduced camera system of the first LM iteration
// at trust-region radius `radius` (dense, row-major, n = 15 N_kf).
int reducedSystemDense(Problem& p, const mba_solver_options& o, double radius, double* A, double* b) {
  Linearization L;
  int st = linearize(p, true, &L);
  if (st) return st;
  Scaled sc;
  std::vector<double> nkf, nlm, nsw;
  columnNorms(p, L, nkf, nlm, nsw);
  sc.skf.assign(15 * (p.nkf + p.ng), 1.0);
  sc.slm.assign(3 * p.nlm, 1.0);
  sc.ssw.assign(p.sw.size(), 1.0);
  if (o.jacobi_scaling) {
    for (size_t a = 0; a < nkf.size(); ++a) sc.skf[a] = 1.0 / (1.0 + std::sqrt(nkf[a]));
    for (size_t a = 0; a < nlm.size(); ++a) sc.slm[a] = 1.0 / (1.0 + std::sqrt(nlm[a]));
    for (size_t a = 0; a < nsw.size(); ++a) sc.ssw[a] = 1.0 / (1.0 + std::sqrt(nsw[a]));
  }
  std::vector<double> dkf(15 * (p.nkf + p.ng)), dlm(3 * p.nlm), dsw(p.sw.size());
  for (size_t a = 0; a < nsw.size(); ++a)
    dsw[a] = std::min(std::max(nsw[a] * sc.ssw[a] * sc.ssw[a], o.min_lm_diagonal), o.max_lm_diagonal) / radius;
  for (size_t a = 0; a < nkf.size(); ++a)
    dkf[a] = std::min(std::max(nkf[a] * sc.skf[a] * sc.skf[a], o.min_lm_diagonal), o.max_lm_diagonal) / radius;
  for (size_t a = 0; a < nlm.size(); ++a)
    dlm[a] = std::min(std::max(nlm[a] * sc.slm[a] * sc.slm[a], o.min_lm_diagonal), o.max_lm_diagonal) / radius;
  BlockSystem pattern;
  buildPattern(p, &pattern);
  StepResult r = computeStep(p, L, sc, dkf, dlm, dsw, pattern, MBA_LINEAR_SOLVER_DENSE_SCHUR, 1, 0.0, A, b);
  return r.status;
}

// Relative pose edges at the current state: r [n][6], tangent Jacobians
// [n][36] (rows 0-5 / columns theta, p of the 15x15 edge blocks).
int oracleLinearizePoseEdges(Problem* p, double* r, double* Jf, double* Jt) {
  Linearization L;
  const int st = linearize(*p, true, &L);
  for (int64_t i = p->nimu; i < p->nedge; ++i) {
    const int64_t j = i - p->nimu;
    for (int a = 0; a < 6; ++a) {
      if (r) r[6 * j + a] = L.ir[15 * i + a];
      for (int c = 0; c < 6; ++c) {
        if (Jf) Jf[36 * j + 6 * a + c] = L.iJf[225 * i + 15 * a + c];
        if (Jt) Jt[36 * j + 6 * a + c] = L.iJt[225 * i + 15 * a + c];
      }
    }
  }
  return st;
}

int oracleLinearizeVisual(Problem* p, double* r, double* Jl, double* Js, double* Jo, double* cost) {
  Linearization L;
  const int st = linearize(*p, true, &L);
  if (r) std::memcpy(r, L.vr.data(), L.vr.size() * sizeof(double));
  if (Jl) std::memcpy(Jl, L.vJl.data(), L.vJl.size() * sizeof(double));
  if (Js) std::memcpy(Js, L.vJs.data(), L.vJs.size() * sizeof(double));
  if (Jo) std::memcpy(Jo, L.vJo.data(), L.vJo.size() * sizeof(double));
  if (cost) *cost = L.cost;
  return st;
}

// isVisualLandmarkWellConstrained (map-structure/vi-map/src/
// landmark-quality-metrics.cc:103-166) with the options of
// mba_landmark_quality_options: observer count, signed distance of the
// closest observing camera (negative when the landmark lies behind it),
// maximum disparity angle of the unit incidence rays
// (getMaxDisparityRadAngleOfUnitVectorBundle, maplab-common geometry.cc:30-44)
// and the optional reprojection bound (a projection counts when the point's
// depth exceeds kMinimumDepth = 1e-10).
static void cameraCenterG(const Problem& p, int64_t k, int cam, double* c) {
  const mba_camera& cm = p.cams[cam];
  double RCI[9], RIM[9], RGM[9], pIC[3], pM[3];
  toRotationMatrixJPL(cm.q_CI_p_CI, RCI);
  for (int i = 0; i < 3; ++i)
    pIC[i] = -(RCI[i] * cm.q_CI_p_CI[4] + RCI[3 + i] * cm.q_CI_p_CI[5] + RCI[6 + i] * cm.q_CI_p_CI[6]);
  const double* x = &p.kf_x[7 * k];
  toRotationMatrixJPL(x, RIM);
  for (int i = 0; i < 3; ++i) pM[i] = RIM[i] * pIC[0] + RIM[3 + i] * pIC[1] + RIM[6 + i] * pIC[2] + x[4 + i];
  const double* mg = &p.mis[7 * p.kf_mis[k]];
  toRotationMatrixJPL(mg, RGM);
  for (int i = 0; i < 3; ++i) c[i] = RGM[3 * i] * pM[0] + RGM[3 * i + 1] * pM[1] + RGM[3 * i + 2] * pM[2] + mg[4 + i];
}

int oracleLandmarkQuality(Problem* pp, const mba_landmark_quality_options* o, uint8_t* good) {
  const Problem& p = *pp;
  for (int64_t l = 0; l < p.nlm; ++l) {
    const int64_t a0 = p.lm_obs_off[l], a1 = p.lm_obs_off[l + 1];
    good[l] = 0;
    if (a1 - a0 < o->min_observers || a1 == a0) continue;
    const int64_t st = p.lm_store[l];
    double R[9], pM[3], pG[3];
    toRotationMatrixJPL(&p.kf_x[7 * st], R);
    const double* pB = &p.lm_p[3 * l];
    for (int i = 0; i < 3; ++i) pM[i] = R[i] * pB[0] + R[3 + i] * pB[1] + R[6 + i] * pB[2] + p.kf_x[7 * st + 4 + i];
    const double* mg = &p.mis[7 * p.kf_mis[st]];
    toRotationMatrixJPL(mg, R);
    for (int i = 0; i < 3; ++i) pG[i] = R[3 * i] * pM[0] + R[3 * i + 1] * pM[1] + R[3 * i + 2] * pM[2] + mg[4 + i];
    std::vector<std::array<double, 3>> rays;
    double min_sd = std::numeric_limits<double>::max();
    bool reproj_fail = false;
    for (int64_t a = a0; a < a1; ++a) {
      const int64_t i = p.lm_obs_idx[a];
      double c[3], pC[3];
      cameraCenterG(p, p.obs_kf[i], p.obs_cam[i], c);
      const double* P9[9];
      visualParams(p, i, P9);
      visualPointInCamera(P9, p.obs_type[i], pC);
      const double r[3] = {c[0] - pG[0], c[1] - pG[1], c[2] - pG[2]};
      const double d = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      min_sd = std::min(min_sd, pC[2] < 0.0 ? -d : d);
      if (d > 0) rays.push_back({r[0] / d, r[1] / d, r[2] / d});
      if (o->max_reprojection_error_px > 0.0) {
        double kp[2];
        pinholeProject3(p.cams[p.obs_cam[i]], pC, kp, nullptr, nullptr, nullptr);
        const double e2 = pC[2] > 1e-10 ? (kp[0] - p.obs_uv[2 * i]) * (kp[0] - p.obs_uv[2 * i]) +
                                              (kp[1] - p.obs_uv[2 * i + 1]) * (kp[1] - p.obs_uv[2 * i + 1])
                                        : std::numeric_limits<double>::max();
        if (e2 > o->max_reprojection_error_px * o->max_reprojection_error_px) { reproj_fail = true; break; }
      }
    }
    if (reproj_fail) continue;
    if (min_sd > o->max_distance_from_closest_observer || min_sd < o->min_distance_from_closest_observer) continue;
    double min_cos = 1.0;
    for (size_t x = 0; x < rays.size(); ++x)
      for (size_t y = x + 1; y < rays.size(); ++y)
        min_cos = std::min(min_cos, std::abs(rays[x][0] * rays[y][0] + rays[x][1] * rays[y][1] + rays[x][2] * rays[y][2]));
    const double angle = rays.size() < 2 ? 0.0 : std::acos(min_cos) * (180.0 / M_PI);
    good[l] = angle < o->min_observation_angle_deg ? 0 : 1;
  }
  return 0;
}

// Switch value per pose edge (1 for edges without a switch variable).
int oracleReadSwitches(Problem* p, double* s) {
  for (int64_t j = 0; j < p->nedge - p->nimu; ++j) s[j] = p->pe_swi[j] >= 0 ? p->sw[p->pe_swi[j]] : p->pe_swc[j];
  return 0;
}

int oracleReadState(Problem* p, double* kx, double* kv, double* kbg, double* kba, double* lp) {
  if (kx) std::memcpy(kx, p->kf_x.data(), p->kf_x.size() * sizeof(double));
  if (kv) std::memcpy(kv, p->kf_v.data(), p->kf_v.size() * sizeof(double));
  if (kbg) std::memcpy(kbg, p->kf_bg.data(), p->kf_bg.size() * sizeof(double));
  if (kba) std::memcpy(kba, p->kf_ba.data(), p->kf_ba.size() * sizeof(double));
  if (lp) std::memcpy(lp, p->lm_p.data(), p->lm_p.size() * sizeof(double));
  return 0;
}

// Cameras and mission baseframes of the current state (they move when the
// descriptor leaves calibration or baseframe blocks free).
int oracleReadCalibration(Problem* p, mba_camera* cams, double* mis) {
  if (cams) std::memcpy(cams, p->cams.data(), p->cams.size() * sizeof(mba_camera));
  if (mis) std::memcpy(mis, p->mis.data(), p->mis.size() * sizeof(double));
  return 0;
}

int oracleWriteState(Problem* p, const double* kx, const double* kv, const double* kbg, const double* kba,
                     const double* lp) {
  if (kx) std::memcpy(p->kf_x.data(), kx, p->kf_x.size() * sizeof(double));
  if (kv) std::memcpy(p->kf_v.data(), kv, p->kf_v.size() * sizeof(double));
  if (kbg) std::memcpy(p->kf_bg.data(), kbg, p->kf_bg.size() * sizeof(double));
  if (kba) std::memcpy(p->kf_ba.data(), kba, p->kf_ba.size() * sizeof(double));
  if (lp) std::memcpy(p->lm_p.data(), lp, p->lm_p.size() * sizeof(double));
  return 0;
}

void oracleDestroy(Problem* p) { delete p; }
void oracleSetThreads(Problem* p, int t) { p->threads = std::max(1, t); }

// Robustified tangent linearization of the first `sample` observations on
// `threads` threads, `reps` times; returns mean seconds per pass.  This is the
// same per-observation work as the device evaluation kernel (residual, three
// tangent Jacobian blocks, Huber correction, cost).
double oracleTimeVisual(Problem* p, int threads, int64_t sample, int reps) {
  sample = std::min<int64_t>(sample, p->nobs);
  std::vector<double> out(32 * (size_t)sample);
  std::vector<double> costs(threads, 0.0);
  const auto t0 = std::chrono::steady_clock::now();
  for (int rep = 0; rep < reps; ++rep) {
    std::vector<std::thread> ts;
    const int64_t chunk = (sample + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
      ts.emplace_back([&, t]() {
        const int64_t b = t * chunk, e = std::min<int64_t>(sample, b + chunk);
        double acc = 0.0;
        for (int64_t i = b; i < e; ++i) {
          const double* P[9];
          visualParams(*p, i, P);
          double r[2], Jl[6], Js7[14], Jo7[14], P76[42];
          double* J[9] = {Jl, Js7, nullptr, nullptr, Jo7, nullptr, nullptr, nullptr, nullptr};
          visualEvaluate(P, &p->obs_uv[2 * i], p->obs_sigma[i], p->obs_type[i], p->cams[p->obs_cam[i]], r, J, nullptr);
          const double sq = r[0] * r[0] + r[1] * r[1];
          double rho[3] = {sq, 1.0, 0.0};
          if (p->use_huber) huberLoss(huberA(*p, i), sq, rho);
          acc += 0.5 * rho[0];
          double* o = &out[32 * i];
          double Jst[12] = {0}, Jot[12] = {0};
          if (p->obs_type[i] != MBA_LOCAL_KEYFRAME) {
            poseParam(*p, p->lm_store[p->obs_lm[i]], P76);
            for (int rr = 0; rr < 2; ++rr)
              for (int c = 0; c < 6; ++c) {
                double a = 0.0;
                for (int m = 0; m < 7; ++m) a += Js7[7 * rr + m] * P76[6 * m + c];
                Jst[6 * rr + c] = a;
              }
            poseParam(*p, p->obs_kf[i], P76);
            for (int rr = 0; rr < 2; ++rr)
              for (int c = 0; c < 6; ++c) {
                double a = 0.0;
                for (int m = 0; m < 7; ++m) a += Jo7[7 * rr + m] * P76[6 * m + c];
                Jot[6 * rr + c] = a;
              }
          }
          if (p->use_huber) {
            double* Js_[3] = {Jl, Jst, Jot};
            const int cols[3] = {3, 6, 6};
            applyCorrector(sq, rho, r, Js_, cols, 3);
          }
          std::memcpy(o, r, 2 * sizeof(double));
          std::memcpy(o + 2, Jl, 6 * sizeof(double));
          std::memcpy(o + 8, Jst, 12 * sizeof(double));
          std::memcpy(o + 20, Jot, 12 * sizeof(double));
        }
        costs[t] += acc;
      });
    }
    for (auto& t : ts) t.join();
  }
  const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return s / reps;
}

}  // namespace oracle
