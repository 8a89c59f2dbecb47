// Internal declarations shared by the CUDA translation units of libmaplab_ba.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/maplab_ba.h"
#include "device_math.cuh"

namespace mba {

// Device-resident problem (plain pointers; passed by value to kernels).
// Observations are sorted by landmark (contiguous per landmark).
struct DevProblem {
  int64_t nkf, nlm, nobs, ncam, nmis, nedge, nsamp;
  int64_t nimu;             // edges [0, nimu) are inertial, [nimu, nedge) relative pose edges
  int32_t vis_block;        // threads per block of the evaluation kernel (tuned; 0 = default)
  int32_t vis_minb;         // > 1: register-lean variant of the evaluation kernel (tuned)
  int32_t vis_pipe;         // 1: pipelined persistent variant of the evaluation kernel (tuned)
  int64_t vis_lo, vis_hi;   // observations [vis_lo, vis_hi) of the linearization kernels (vis_hi 0: to nobs)
  // observations
  const double2* obs_uv;
  const double* obs_sinv;   // 1 / sigma
  const double* obs_huber;  // Huber scale a = delta * sigma, 0 = no loss
  const int32_t* obs_lm;
  const int32_t* obs_kf;
  const int32_t* obs_store;
  const uint8_t* obs_cam;
  const uint8_t* obs_type;
  const int64_t* obs_perm;  // sorted index -> caller index
  // landmarks
  double* lm_p;             // [nlm][4] (x, y, z, pad)
  const int64_t* lm_obs_off;// [nlm+1]
  const uint8_t* lm_active;
  int32_t* lm_off;          // [nlm] 1 = rejected as an outlier: its terms are out of the problem
  // keyframes
  double* kf_state;         // [nkf][16] = q(4) p(3) v(3) b_g(3) b_a(3)
  double* kf_rot;           // [nkf][16] = R_I_M (9, row-major), |q|^2, pad: written before each FP64
                            // linearization from kf_state
  const int32_t* kf_mis;
  const uint32_t* kf_flags;
  const uint16_t* kf_mask;  // bit d set = tangent dim d active (theta, p, v, b_g, b_a)
  const double* mis;        // [nmis][8] = q_G_M(4) p_G_M(3) pad
  const DevCamera* cams;
  // inertial edges
  const int32_t* e_from;
  const int32_t* e_to;
  const int64_t* e_off;
  const int64_t* imu_ts;
  const double* imu;        // [nsamp][6]
  double gyro_noise2, gyro_bias2, acc_noise2, acc_bias2, gravity;
  // pose edges (index j = edge - nimu); measurement rotation per kind:
  // relative T_Bk_Bk+1 (Hamilton), loop closure q_AB (JPL), absolute q_S_G
  // (Hamilton, inverse of the measured T_G_S rotation)
  const double* pe_meas;    // [npe][7] q | p
  const double* pe_sqrt;    // [npe][36] row-major M with e_w = e^T M (M = L^-1, cov = L L^T)
  const double* pe_ext;     // [npe][7] q_I_B | p_B_I (relative), q_S_B | p_S_B (absolute)
  const int32_t* pe_type;   // [npe] MBA_POSE_EDGE_*
  const int32_t* pe_swi;    // [npe] switch variable, -1 = none
  const double* pe_swc;     // [npe] switch value of an edge without a variable
  int64_t nsw;              // switch variables (switchable loop closures)
  double* sw;               // [nsw] switch state
  const double* sw_w;       // [nsw] switch prior sqrt information (1 / sigma)
  const int32_t* sw_e;      // [nsw] edge of each switch
  // Inertial scratch: dt per step, end state per edge, RK4 stage inputs
  // (15 values x 4 stages per step, FP64 or FP32).
  double* ine_scratch;
  // FP32 mirrors read by the FP32 evaluation kernel (no FP64 instruction in
  // that kernel: GB300's FP64 pipe is narrow).  The state mirrors are
  // refreshed whenever the FP64 state changes.
  const float2* obs_uv_f;
  const float* obs_sinv_f;
  const float* obs_huber_f;
  float* lm_p_f;            // [nlm][4]
  float* kf_pose_f;         // [nkf][8] = q(4) p(3) pad
  const float* mis_f;       // [nmis][8]
  const DevCameraT<float>* cams_f;
  // Calibration / baseframe variables ("global nodes", FP64 solves): one
  // 15-dim block per camera with a free calibration block (dims: intrinsics
  // 0-3, distortion 4-7, theta_C_I 8-10, p_C_I 11-13) and per mission with a
  // free baseframe (theta 0-2, or yaw 0, and p_G_M 3-5), after the keyframe
  // blocks of the reduced system.  ng = 0: none.
  int64_t ng;
  const int32_t* cam_node;  // [ncam] node of each camera, -1 = constant
  const int32_t* mis_node;  // [nmis]
  const int32_t* node_cam;  // [ng] camera of each node (-1 for a mission node)
  const int32_t* node_mis;  // [ng] mission of each node (-1 for a camera node)
  const uint16_t* g_mask;   // [ng] active dims
  const uint32_t* mis_flags;// [nmis] MBA_MIS_BASEFRAME_*
};

// End of the linearization kernels' observation range.
__host__ __device__ inline int64_t vis_end(const DevProblem& P) { return P.vis_hi > 0 ? P.vis_hi : P.nobs; }

// Typed view of the inputs of the evaluation kernel (FP64 arrays for the
// FP64 kernel, the FP32 mirrors for the FP32 kernel).
template <typename T>
struct VisualInputs {
  const typename Vec2<T>::type* uv;
  const T* sinv;
  const T* huber;
  const T* lm_p;       // stride 4
  const T* kf;         // pose q(4) p(3), stride kf_stride
  int kf_stride;
  const T* mis;        // stride 8
  const DevCameraT<T>* cams;
  const T* kf_rot;     // FP64: per-keyframe R_I_M and |q|^2 (stride 16), else null
};

template <typename T>
struct VisualLin {
  T* r;   // [2][nobs]
  T* Jl;  // [6][nobs]
  T* Js;  // [12][nobs]  store pose tangent (theta, p)
  T* Jo;  // [12][nobs]  observer pose tangent
};

template <typename T>
struct InertialLin {
  T* r;   // [nedge][15]
  T* Jf;  // [nedge][225] from-keyframe tangent (theta, p, v, b_g, b_a)
  T* Jt;  // [nedge][225] to-keyframe tangent
  T* Js;  // [npe][6] d r / d switch of the pose edges (the unswitched residual)
};

// Launchers (kernels_eval.cu).
cudaError_t launch_visual_ambient(const DevProblem& P, double* res, double* const* jac_dev, cudaStream_t s);
template <typename T>
cudaError_t launch_visual_linearize(const DevProblem& P, VisualLin<T> out, double* cost_accum, cudaStream_t s);
cudaError_t launch_visual_cost(const DevProblem& P, const double* kf_state, const double* lm_p, double* cost_accum,
                               int* nonfinite, cudaStream_t s);
// Inertial: full evaluation at `kf_state`; writes tangent linearization (if
// lin.r) and/or the ambient blocks (if amb_res / amb_jac), accumulates cost.
cudaError_t launch_inertial(const DevProblem& P, const double* kf_state, InertialLin<double> lin, double* amb_res,
                            double* const* amb_jac, double* cost_accum, int* status, cudaStream_t s);
template <typename T>
cudaError_t launch_visual_linearize_gated(const DevProblem& P, VisualLin<T> out, double* cost_accum, const int* run_if,
                                          const int* skip_if, cudaStream_t s);
cudaError_t launch_visual_cost_gated(const DevProblem& P, const double* kf_state, const double* lm_p,
                                     double* cost_accum, int* nonfinite, const int* skip_if, cudaStream_t s,
                                     const int* run_if = nullptr);
// Also evaluates the pose edges, with switch state sw_state (NULL: P.sw).
cudaError_t launch_inertial_gated(const DevProblem& P, const double* kf_state, InertialLin<double> lin,
                                  double* cost_accum, int* status, const int* skip_if, cudaStream_t s,
                                  bool f32 = false, const double* sw_state = nullptr);
// obs_inv: caller index -> sorted index (launch_invert_perm).  Destinations
// may be device or mapped page-locked host memory.
template <typename T>
cudaError_t launch_gather_visual(const DevProblem& P, const int64_t* obs_inv, VisualLin<T> v, double* r, double* Jl,
                                 double* Js, double* Jo, cudaStream_t s);
cudaError_t launch_invert_perm(const DevProblem& P, int64_t* inv, cudaStream_t s);
// Caller rows [lo, hi) (inv: caller -> sorted index; null when the SoA buffers
// are in caller order already).
template <typename T>
cudaError_t launch_gather_rows(const DevProblem& P, const int64_t* inv, int64_t lo, int64_t hi, VisualLin<T> v,
                               double* r, double* Jl, double* Js, double* Jo, cudaStream_t s);
// The observation fields the FP64 linearization reads, in the caller's order
// (a DevProblem pointing at them evaluates caller row o as observation o).
struct CallerObs {
  double2* uv;
  double* sinv;
  double* huber;
  int32_t *lm, *kf, *store;
  uint8_t *cam, *type;
};
cudaError_t launch_caller_obs(const DevProblem& P, const int64_t* inv, CallerObs c, cudaStream_t s);
// isVisualLandmarkWellConstrained per landmark at the current state (good [nlm]).
cudaError_t launch_landmark_quality(const DevProblem& P, const mba_landmark_quality_options& o, uint8_t* good,
                                    cudaStream_t s);
// to_device = 1: host-layout device arrays -> kf_state / lm_p; 0: the reverse.
// lp is in the caller's landmark numbering: lm_caller [nlm] maps an internal
// landmark to it (nullptr: the same numbering).
cudaError_t launch_pack_state(const DevProblem& P, const double* kx, const double* kv, const double* kbg,
                              const double* kba, const double* lp, const int32_t* lm_caller, int to_device,
                              cudaStream_t s);
// kernels_inertial.cu: f32_matrices selects FP32 propagation of Phi and Q
// (mixed path); the state, Cholesky, residual and Jacobians stay FP64.
cudaError_t launch_inertial_v2(const DevProblem& P, const double* kf_state, bool f32_matrices, InertialLin<double> lin,
                               double* amb_res, double* const* amb_jac, double* cost_accum, int* status,
                               const int* skip_if, cudaStream_t s);
// Relative pose edges (kernels_pose.cu): residual rows 0-5 and the (theta, p)
// Jacobian columns of edges [nimu, nedge) into lin (if lin.r), cost into
// cost_accum.
cudaError_t launch_pose_edges(const DevProblem& P, const double* kf_state, const double* sw_state,
                              InertialLin<double> lin, double* cost_accum, const int* skip_if, cudaStream_t s);
cudaError_t launch_inertial_f32(const DevProblem& P, const InertialLin<double>& src, InertialLin<float> dst,
                                cudaStream_t s);
// Outlier landmarks at the current state (outlier-rejection-solver.cc:28-103):
// a landmark goes out of the problem when one of its observations has depth
// <= 0 in the observing camera or, if use_reprojection, a reprojection error
// above max_px.  Newly rejected landmarks are counted into *count.  f32:
// the same test on the FP32 copies of the state (mixed path).
cudaError_t launch_find_outliers(const DevProblem& P, int use_reprojection, double max_px, int* count,
                                 const int* run_if, const int* skip_if, cudaStream_t s, bool f32 = false);
// FP32 residuals of the state in FP32 copies (pose q p pad [n][8], landmark
// [n][4]); cost summed in FP64.
cudaError_t launch_visual_cost_f32(const DevProblem& P, const float* kf, const float* lm, double* cost_accum,
                                   int* nonfinite, const int* skip_if, cudaStream_t s, const int* run_if = nullptr);

}  // namespace mba
