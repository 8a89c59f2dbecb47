// CPU ORACLE — test infrastructure only.
//
// Plain C++17 restatement (no Eigen, no Ceres) of maplab's visual-inertial
// bundle-adjustment path, used as the correctness checker of the CUDA
// back-end and as the timed CPU baseline.  Nothing in the product links or
// calls this code; only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg load it (through liboracle.so and ctypes).
//
// Each function cites the reference file:line it restates.  Parity anchors:
//   * the IMU integrator golden vectors of
//     algorithms/imu-integrator-rk4/test/test_imu_integrator_cov_phi_test.cc
//     and the closed-form cases of test_imu_integrator_basic_test.cc
//     (extracted into tests/golden/ by tests/golden/make_golden.py);
//   * numeric-differentiation checks of the JPL parameterizations
//     (test_quaternion_parameterization_test.cc:13-103);
//   * the ground-truth recovery scenarios of test_visual_term_test.cc,
//     test_mission_baseframe_visual_term_test.cc and test_inertial_term_test.cc.
// The Levenberg-Marquardt loop follows Ceres Solver's published trust-region
// algorithm (Ceres is not vendored in the reference): parity of the LM
// trajectory with Ceres itself is unpinned.
#ifndef MBA_ORACLE_H_
#define MBA_ORACLE_H_

#include <cmath>
#include <cstdint>
#include <cstring>

#include "../include/maplab_ba.h"

namespace oracle {

// ---------------------------------------------------------------- 3x3 helpers
// Row-major 3x3 matrices as double[9].
inline void mat3_mul(const double* A, const double* B, double* C) {
  double T[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      T[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
  std::memcpy(C, T, sizeof(T));
}
inline void mat3_transpose(const double* A, double* B) {
  double T[9] = {A[0], A[3], A[6], A[1], A[4], A[7], A[2], A[5], A[8]};
  std::memcpy(B, T, sizeof(T));
}
inline void mat3_vec(const double* A, const double* x, double* y) {
  double t0 = A[0] * x[0] + A[1] * x[1] + A[2] * x[2];
  double t1 = A[3] * x[0] + A[4] * x[1] + A[5] * x[2];
  double t2 = A[6] * x[0] + A[7] * x[1] + A[8] * x[2];
  y[0] = t0; y[1] = t1; y[2] = t2;
}
inline void mat3_scale(double* A, double s) { for (int i = 0; i < 9; ++i) A[i] *= s; }
// common::skew (common/maplab-common/include/maplab-common/geometry.h:15).
inline void skew(const double* v, double* S) {
  S[0] = 0.0;   S[1] = -v[2]; S[2] = v[1];
  S[3] = v[2];  S[4] = 0.0;   S[5] = -v[0];
  S[6] = -v[1]; S[7] = v[0];  S[8] = 0.0;
}

// ------------------------------------------------------ JPL quaternion math
// common::toRotationMatrixJPL (quaternion-math-inl.h:6-27). q = xyzw.
inline void toRotationMatrixJPL(const double* q, double* R) {
  R[0] = 1.0 - 2.0 * (q[1] * q[1] + q[2] * q[2]);
  R[1] = 2.0 * (q[0] * q[1] + q[2] * q[3]);
  R[2] = 2.0 * (q[0] * q[2] - q[1] * q[3]);
  R[3] = 2.0 * (q[0] * q[1] - q[2] * q[3]);
  R[4] = 1.0 - 2.0 * (q[0] * q[0] + q[2] * q[2]);
  R[5] = 2.0 * (q[1] * q[2] + q[0] * q[3]);
  R[6] = 2.0 * (q[0] * q[2] + q[1] * q[3]);
  R[7] = 2.0 * (q[1] * q[2] - q[0] * q[3]);
  R[8] = 1.0 - 2.0 * (q[0] * q[0] + q[1] * q[1]);
}
// Eigen::MatrixBase::normalize(): divide by sqrt(squaredNorm) when > 0.
inline void normalize4(double* q) {
  const double z = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (z > 0.0) {
    const double n = std::sqrt(z);
    q[0] /= n; q[1] /= n; q[2] /= n; q[3] /= n;
  }
}
// common::signedQuaternionProductJPL (quaternion-math-inl.h:112-139):
// L(q1) * q2 with L = [q1w*I - [q1v]x, q1v; -q1v^T, q1w], then normalize.
inline void signedQuaternionProductJPL(const double* q1, const double* q2, double* out) {
  double p[4];
  p[0] = q1[3] * q2[0] + q1[2] * q2[1] - q1[1] * q2[2] + q1[0] * q2[3];
  p[1] = -q1[2] * q2[0] + q1[3] * q2[1] + q1[0] * q2[2] + q1[1] * q2[3];
  p[2] = q1[1] * q2[0] - q1[0] * q2[1] + q1[3] * q2[2] + q1[2] * q2[3];
  p[3] = -q1[0] * q2[0] - q1[1] * q2[1] - q1[2] * q2[2] + q1[3] * q2[3];
  normalize4(p);
  std::memcpy(out, p, sizeof(p));
}
// common::positiveQuaternionProductJPL (quaternion-math-inl.h:141-154).
inline void positiveQuaternionProductJPL(const double* q1, const double* q2, double* out) {
  signedQuaternionProductJPL(q1, q2, out);
  if (out[3] < 0.0) { out[0] = -out[0]; out[1] = -out[1]; out[2] = -out[2]; out[3] = -out[3]; }
}
// common::quaternionInverseJPL (quaternion-math-inl.h:156-163).
inline void quaternionInverseJPL(const double* q, double* out) {
  out[0] = -q[0]; out[1] = -q[1]; out[2] = -q[2]; out[3] = q[3];
}
// common::rotationVectorToQuaternionJPL (quaternion-math-inl.h:94-110).
inline void rotationVectorToQuaternionJPL(const double* v, double* q) {
  const double theta = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (theta < 1e-10) {
    q[0] = q[1] = q[2] = 0.0; q[3] = 1.0;
  } else {
    const double s = std::sin(theta / 2.0);
    q[0] = v[0] / theta * s; q[1] = v[1] / theta * s; q[2] = v[2] / theta * s;
    q[3] = std::cos(theta / 2.0);
  }
}

// ------------------------------------------------------ parameterizations
// get_dQuaternionJpl_dTheta (quaternion-param-jpl.cc:8-32): 4x3 row-major.
void jplQuaternionJacobian(const double* q, double* J43);
// JplQuaternionParameterization::Plus (quaternion-param-jpl.cc:35-68).
void jplQuaternionPlus(const double* q, const double* delta, double* out);
// JplPoseParameterization = Product(JplQuaternion, Identity(3)) (pose-param-jpl.h:11-18).
void jplPosePlus(const double* x7, const double* delta6, double* out7);
// JplYawQuaternionParameterization (quaternion-param-jpl.cc:78-105).
void jplYawPlus(const double* q, const double* delta1, double* out);
void jplYawJacobian(const double* q, double* J41);
// JplRollPitchQuaternionParameterization (quaternion-param-jpl.cc:107-164).
void jplRollPitchPlus(const double* q_GM, const double* q_IM, const double* delta2, double* out);
void jplRollPitchJacobian(const double* q_GM, const double* q_IM, double* J42);

// ------------------------------------------------------ camera + distortion
// aslam::ProjectionResult::Status (aslam_cv_cameras/include/aslam/cameras/camera.h:34-100).
enum ProjectionStatus { KEYPOINT_VISIBLE = 0, KEYPOINT_OUTSIDE_IMAGE_BOX = 1, POINT_BEHIND_CAMERA = 2, PROJECTION_INVALID = 3 };

// RadTanDistortion::distortUsingExternalCoefficients / distortParameterJacobian
// (aslam_cv_cameras/src/distortion-radtan.cc:14-91).
void radtanDistort(const double* k, double* pt, double* J22 /*nullable*/);
void radtanParamJacobian(const double* k, const double* pt, double* J24);
// EquidistantDistortion (aslam_cv_cameras/src/distortion-equidistant.cc:14-142).
void equidistantDistort(const double* k, double* pt, double* J22 /*nullable*/);
void equidistantParamJacobian(const double* k, const double* pt, double* J24);

// PinholeCamera::project3Functional (aslam_cv_cameras/src/camera-pinhole.cc:65-164)
// + evaluateProjectionResult (camera-pinhole-inl.h:47-65).
int pinholeProject3(const mba_camera& cam, const double* p_C, double* kp,
                    double* J_point23 /*nullable*/, double* J_intr24 /*nullable*/,
                    double* J_dist24 /*nullable*/);

// ------------------------------------------------------ visual error term
// VisualReprojectionError<PinholeCamera, D>::Evaluate
// (visual-error-term-inl.h:12-379).  params: 9 pointers in Ceres block order
// (p_B 3, q_B_LM|p_LM_B 7, q_G_LM|p_G_LM 7, q_G_M|p_G_M 7, q_I_M|p_M_I 7,
// q_C_I 4, p_C_I 3, intrinsics 4, distortion 4).  jacobians: 9 nullable
// row-major ambient blocks (2x3, 2x7, 2x7, 2x7, 2x7, 2x4, 2x3, 2x4, 2x4).
// Returns true like Evaluate; *failed tells whether the projection failed.
void visualPointInCamera(const double* const* params, int type, double* p_C);
void poseEdgeEvaluate(const double* xk, const double* xk1, const double* ext, const double* meas, const double* M,
                      double* r, double* Jk, double* Jk1);
bool poseEdgeSqrtInfo(const double* cov, double* M);
// LoopClosureEdgeErrorTerm without the switch factor: residual [6], ambient
// Jacobians [6][7] of the two vertex blocks (may be NULL).
void loopClosureEvaluate(const double* bfA, const double* bfB, const double* xA, const double* xB, const double* meas,
                         const double* M, double* r, double* JA, double* JB);
// BlockPosePriorErrorTermV2: residual [6], ambient Jacobian [6][7] of the
// vertex block (may be NULL).
void absolutePoseEvaluate(const double* bf, const double* x, const double* ext, const double* meas, const double* M,
                          double* r, double* J);
bool visualEvaluate(const double* const* params, const double* measurement, double pixel_sigma,
                    int error_type, const mba_camera& cam, double* residual,
                    double** jacobians, bool* failed);

// ------------------------------------------------------ IMU integrator
struct ImuNoise {
  double gyro_noise_sigma, gyro_bias_sigma, acc_noise_sigma, acc_bias_sigma, gravity;
};
// ImuIntegratorRK4::integrate (imu-integrator-inl.h:17-168).  state16 =
// [q_I_M(4), b_g(3), v_M(3), b_a(3), p_M_I(3)]; readings12 = [acc0, gyro0,
// acc1, gyro1] debiased.  phi/cov 15x15 row-major, both NULL to skip.
void imuIntegrate(const ImuNoise& n, const double* state16, const double* readings12, double dt,
                  double* next16, double* phi, double* cov);

// InertialErrorTerm::IntegrateStateAndCovariance (inertial-error-term.cc:9-75).
// Returns false on unordered timestamps (CHECK in the reference).
bool inertialIntegrate(const ImuNoise& n, const double* begin16, int num_samples,
                       const int64_t* ts_ns, const double* imu6, double* end16,
                       double* phi_accum, double* Q_accum);

// InertialErrorTerm::Evaluate (inertial-error-term.cc:77-286).  params: 8
// pointers (pose_from 7, b_g_from 3, v_from 3, b_a_from 3, pose_to 7, b_g_to,
// v_to, b_a_to).  jacobians: 8 nullable row-major blocks 15x{7,3,3,3,7,3,3,3}.
// Returns 0 on success, MBA_ERR_NOT_SPD when Q_accum is not positive definite,
// MBA_ERR_UNORDERED_IMU on unordered timestamps.
int inertialEvaluate(const ImuNoise& n, const double* const* params, int num_samples,
                     const int64_t* ts_ns, const double* imu6, double* residual15,
                     double** jacobians);

// ceres::HuberLoss::Evaluate (third-party; restated from Ceres' documented
// definition rho(s) = s for s <= a^2, 2 a sqrt(s) - a^2 otherwise).
inline void huberLoss(double a, double s, double* rho) {
  const double b = a * a;
  if (s > b) {
    const double r = std::sqrt(s);
    rho[0] = 2.0 * a * r - b;
    rho[1] = a / r;
    if (rho[1] < 2.2250738585072014e-308) rho[1] = 2.2250738585072014e-308;
    rho[2] = -rho[1] / (2.0 * s);
  } else {
    rho[0] = s; rho[1] = 1.0; rho[2] = 0.0;
  }
}

}  // namespace oracle

#endif  // MBA_ORACLE_H_
