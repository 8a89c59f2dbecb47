// CPU ORACLE — test infrastructure only (see oracle.h).
// Per-term restatements: parameterizations, camera, distortion, visual and
// inertial error terms, RK4 IMU integrator.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "oracle.h"

namespace oracle {

// ---------------------------------------------------------------- params
void jplQuaternionJacobian(const double* q, double* J) {
  // quaternion-param-jpl.cc:8-32
  J[0] = q[3];  J[1] = -q[2]; J[2] = q[1];
  J[3] = q[2];  J[4] = q[3];  J[5] = -q[0];
  J[6] = -q[1]; J[7] = q[0];  J[8] = q[3];
  J[9] = -q[0]; J[10] = -q[1]; J[11] = -q[2];
  for (int i = 0; i < 12; ++i) J[i] *= 0.5;
}

void jplQuaternionPlus(const double* q, const double* d, double* out) {
  // quaternion-param-jpl.cc:35-68
  const double sq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  constexpr double kThr = (0.262 * 2) * (0.262 * 2);
  double qd[4];
  if (sq < kThr) {
    qd[0] = 0.5 * d[0]; qd[1] = 0.5 * d[1]; qd[2] = 0.5 * d[2]; qd[3] = 1.0;
    normalize4(qd);
  } else {
    const double nh = 0.5 * std::sqrt(sq);
    const double s = std::sin(nh);
    qd[0] = 0.5 * d[0] / nh * s; qd[1] = 0.5 * d[1] / nh * s; qd[2] = 0.5 * d[2] / nh * s;
    qd[3] = std::cos(nh);
  }
  positiveQuaternionProductJPL(qd, q, out);
}

void jplPosePlus(const double* x, const double* d, double* out) {
  double q[4];
  jplQuaternionPlus(x, d, q);
  out[0] = q[0]; out[1] = q[1]; out[2] = q[2]; out[3] = q[3];
  out[4] = x[4] + d[3]; out[5] = x[5] + d[4]; out[6] = x[6] + d[5];
}

void jplYawPlus(const double* q, const double* d, double* out) {
  // quaternion-param-jpl.cc:78-93
  const double h = 0.5 * d[0];
  const double qd[4] = {0.0, 0.0, std::sin(h), std::cos(std::fabs(h))};
  positiveQuaternionProductJPL(qd, q, out);
}

void jplYawJacobian(const double* q, double* J) {
  // quaternion-param-jpl.cc:95-105
  J[0] = q[1] * 0.5; J[1] = -q[0] * 0.5; J[2] = q[3] * 0.5; J[3] = -q[2] * 0.5;
}

static void rollPitchRMG(const double* q_GM, double* R_M_G) {
  // JplRollPitchQuaternionParameterization ctor (quaternion-param-jpl.cc:107-111)
  double qi[4];
  quaternionInverseJPL(q_GM, qi);
  toRotationMatrixJPL(qi, R_M_G);
}

void jplRollPitchPlus(const double* q_GM, const double* q_IM, const double* d, double* out) {
  // quaternion-param-jpl.cc:113-142
  double R_M_G[9];
  rollPitchRMG(q_GM, R_M_G);
  const double Gd[3] = {d[0], d[1], 0.0};
  double Md[3];
  mat3_vec(R_M_G, Gd, Md);
  double q_M_Mrp[4], q_inv[4], q_M_I[4];
  rotationVectorToQuaternionJPL(Md, q_M_Mrp);
  quaternionInverseJPL(q_IM, q_inv);
  positiveQuaternionProductJPL(q_M_Mrp, q_inv, q_M_I);
  quaternionInverseJPL(q_M_I, out);
}

void jplRollPitchJacobian(const double* q_GM, const double* q_IM, double* J42) {
  // quaternion-param-jpl.cc:144-164: (-dq/dtheta * R_I_M * R_M_G).leftCols<2>()
  double R_M_G[9], R_I_M[9], A[9], dq[12];
  rollPitchRMG(q_GM, R_M_G);
  jplQuaternionJacobian(q_IM, dq);
  toRotationMatrixJPL(q_IM, R_I_M);
  mat3_mul(R_I_M, R_M_G, A);
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 2; ++c)
      J42[2 * r + c] = -(dq[3 * r] * A[c] + dq[3 * r + 1] * A[3 + c] + dq[3 * r + 2] * A[6 + c]);
}

// ---------------------------------------------------------------- distortion
void radtanDistort(const double* k, double* pt, double* J) {
  // distortion-radtan.cc:14-65
  double& x = pt[0];
  double& y = pt[1];
  const double k1 = k[0], k2 = k[1], p1 = k[2], p2 = k[3];
  const double mx2_u = x * x, my2_u = y * y, mxy_u = x * y;
  const double rho2_u = mx2_u + my2_u;
  const double rad_dist_u = k1 * rho2_u + k2 * rho2_u * rho2_u;
  if (J) {
    J[0] = 1.0 + rad_dist_u + 2.0 * k1 * mx2_u + 4.0 * k2 * rho2_u * mx2_u + 2.0 * p1 * y + 6.0 * p2 * x;
    J[1] = 2.0 * k1 * mxy_u + 4.0 * k2 * rho2_u * mxy_u + 2.0 * p1 * x + 2.0 * p2 * y;
    J[2] = J[1];
    J[3] = 1.0 + rad_dist_u + 2.0 * k1 * my2_u + 4.0 * k2 * rho2_u * my2_u + 2.0 * p2 * x + 6.0 * p1 * y;
  }
  const double nx = x + x * rad_dist_u + 2.0 * p1 * mxy_u + p2 * (rho2_u + 2.0 * mx2_u);
  const double ny = y + y * rad_dist_u + 2.0 * p2 * mxy_u + p1 * (rho2_u + 2.0 * my2_u);
  x = nx;
  y = ny;
}

void radtanParamJacobian(const double*, const double* pt, double* J) {
  // distortion-radtan.cc:67-91
  const double y0 = pt[0], y1 = pt[1];
  const double r2 = y0 * y0 + y1 * y1;
  const double r4 = r2 * r2;
  J[0] = y0 * r2; J[1] = y0 * r4; J[2] = 2.0 * y0 * y1; J[3] = r2 + 2.0 * y0 * y0;
  J[4] = y1 * r2; J[5] = y1 * r4; J[6] = r2 + 2.0 * y1 * y1; J[7] = 2.0 * y0 * y1;
}

void equidistantDistort(const double* k, double* pt, double* J) {
  // distortion-equidistant.cc:14-107
  double& x = pt[0];
  double& y = pt[1];
  const double k1 = k[0], k2 = k[1], k3 = k[2], k4 = k[3];
  const double x2 = x * x, y2 = y * y;
  const double r = std::sqrt(x2 + y2);
  if (r < 1e-10) {
    if (J) J[0] = J[1] = J[2] = J[3] = 0.0;
    return;
  }
  const double theta = std::atan(r);
  const double theta2 = theta * theta, theta4 = theta2 * theta2;
  const double theta6 = theta2 * theta4, theta8 = theta4 * theta4;
  const double thetad = theta * (1 + k1 * theta2 + k2 * theta4 + k3 * theta6 + k4 * theta8);
  if (J) {
    const double theta3 = theta2 * theta, theta5 = theta4 * theta, theta7 = theta6 * theta;
    const double poly = k1 * theta2 + k2 * theta4 + k3 * theta6 + k4 * theta8 + 1.0;
    const double r2 = x2 + y2;
    const double r2p1 = x2 + y2 + 1.0;
    const double p15 = std::pow(x2 + y2, 3.0 / 2.0);
    // The four terms below restate the MATLAB-generated expressions
    // (distortion-equidistant.cc:52-96) with common subexpressions named.
    const double sx = (k2 * x * theta3 * 1.0 / r * 4.0) / r2p1 + (k3 * x * theta5 * 1.0 / r * 6.0) / r2p1 +
                      (k4 * x * theta7 * 1.0 / r * 8.0) / r2p1 + (k1 * x * theta * 1.0 / r * 2.0) / r2p1;
    const double sy = (k2 * y * theta3 * 1.0 / r * 4.0) / r2p1 + (k3 * y * theta5 * 1.0 / r * 6.0) / r2p1 +
                      (k4 * y * theta7 * 1.0 / r * 8.0) / r2p1 + (k1 * y * theta * 1.0 / r * 2.0) / r2p1;
    J[0] = theta * 1.0 / r * poly + x * theta * 1.0 / r * sx + (x2 * poly) / (r2 * r2p1) - x2 * theta * 1.0 / p15 * poly;
    J[1] = x * theta * 1.0 / r * sy + (x * y * poly) / (r2 * r2p1) - x * y * theta * 1.0 / p15 * poly;
    J[2] = y * theta * 1.0 / r * sx + (x * y * poly) / (r2 * r2p1) - x * y * theta * 1.0 / p15 * poly;
    J[3] = theta * 1.0 / r * poly + y * theta * 1.0 / r * sy + (y2 * poly) / (r2 * r2p1) - y2 * theta * 1.0 / p15 * poly;
  }
  const double scaling = (r > 1e-8) ? thetad / r : 1.0;
  x *= scaling;
  y *= scaling;
}

void equidistantParamJacobian(const double*, const double* pt, double* J) {
  // distortion-equidistant.cc:109-142
  const double x = pt[0], y = pt[1];
  const double r = std::sqrt(x * x + y * y);
  const double theta = std::atan(r);
  if (r < 1e-10) {
    for (int i = 0; i < 8; ++i) J[i] = 0.0;
    return;
  }
  J[0] = x * std::pow(theta, 3.0) * 1.0 / r;
  J[1] = x * std::pow(theta, 5.0) * 1.0 / r;
  J[2] = x * std::pow(theta, 7.0) * 1.0 / r;
  J[3] = x * std::pow(theta, 9.0) * 1.0 / r;
  J[4] = y * std::pow(theta, 3.0) * 1.0 / r;
  J[5] = y * std::pow(theta, 5.0) * 1.0 / r;
  J[6] = y * std::pow(theta, 7.0) * 1.0 / r;
  J[7] = y * std::pow(theta, 9.0) * 1.0 / r;
}

void fovDistort(const double* k, double* pt, double* J) {
  // FisheyeDistortion::distortUsingExternalCoefficients (distortion-fisheye.cc:14-80):
  // the FOV model r_d = atan(2 tan(w / 2) r_u) / w with one parameter w.
  const double w = k[0];
  const double u = pt[0], v = pt[1];
  const double r_u = std::sqrt(u * u + v * v);
  const double r_u_cubed = r_u * r_u * r_u;
  const double tanwhalf = std::tan(w / 2.0);
  const double tanwhalfsq = tanwhalf * tanwhalf;
  const double atan_wrd = std::atan(2.0 * tanwhalf * r_u);
  double r_rd;
  if (w * w < 1e-5) r_rd = 1.0;
  else if (r_u * r_u < 1e-5) r_rd = 2.0 * tanwhalf / w;
  else r_rd = atan_wrd / (r_u * w);
  if (J) {
    if (w * w < 1e-5) {
      J[0] = 1.0; J[1] = 0.0; J[2] = 0.0; J[3] = 1.0;
    } else if (r_u * r_u < 1e-5) {
      J[0] = 2.0 * tanwhalf / w; J[1] = 0.0; J[2] = 0.0; J[3] = 2.0 * tanwhalf / w;
    } else {
      const double uv2 = u * u + v * v;
      const double den = w * uv2 * (4 * tanwhalfsq * uv2 + 1);
      J[0] = atan_wrd / (w * r_u) - (u * u * atan_wrd) / (w * r_u_cubed) + (2 * u * u * tanwhalf) / den;
      J[1] = (2 * u * v * tanwhalf) / den - (u * v * atan_wrd) / (w * r_u_cubed);
      J[2] = (2 * u * v * tanwhalf) / den - (u * v * atan_wrd) / (w * r_u_cubed);
      J[3] = atan_wrd / (w * r_u) - (v * v * atan_wrd) / (w * r_u_cubed) + (2 * v * v * tanwhalf) / den;
    }
  }
  pt[0] = u * r_rd;
  pt[1] = v * r_rd;
}

void fovParamJacobian(const double* k, const double* pt, double* J) {
  // FisheyeDistortion::distortParameterJacobian (distortion-fisheye.cc:82-110):
  // 2 x 1 in columns 0 of the 2 x 4 block, the other columns zero.
  const double w = k[0];
  const double tanwhalf = std::tan(w / 2.0);
  const double tanwhalfsq = tanwhalf * tanwhalf;
  const double u = pt[0], v = pt[1];
  const double r_u = std::sqrt(u * u + v * v);
  const double atan_wrd = std::atan(2.0 * tanwhalf * r_u);
  for (int i = 0; i < 8; ++i) J[i] = 0.0;
  if (w * w < 1e-5) return;
  if (r_u * r_u < 1e-5) {
    J[0] = J[4] = (w - std::sin(w)) / (w * w * std::cos(w / 2) * std::cos(w / 2));
    return;
  }
  J[0] = (2 * u * (tanwhalfsq / 2 + 0.5)) / (w * (4 * tanwhalfsq * r_u * r_u + 1)) - (u * atan_wrd) / (w * w * r_u);
  J[4] = (2 * v * (tanwhalfsq / 2 + 0.5)) / (w * (4 * tanwhalfsq * r_u * r_u + 1)) - (v * atan_wrd) / (w * w * r_u);
}

// ---------------------------------------------------------------- camera
int pinholeProject3(const mba_camera& cam, const double* p, double* kp, double* Jp, double* Ji,
                    double* Jd) {
  // camera-pinhole.cc:65-164
  const double fu = cam.intrinsics[0], fv = cam.intrinsics[1];
  const double cu = cam.intrinsics[2], cv = cam.intrinsics[3];
  const double x = p[0], y = p[1], z = p[2];
  const double rz = 1.0 / z;
  kp[0] = x * rz;
  kp[1] = y * rz;
  double Jdist[4] = {1.0, 0.0, 0.0, 1.0};
  if (Jd) {
    if (cam.distortion_type == MBA_DISTORTION_RADTAN) radtanParamJacobian(cam.distortion, kp, Jd);
    else if (cam.distortion_type == MBA_DISTORTION_EQUIDISTANT) equidistantParamJacobian(cam.distortion, kp, Jd);
    else if (cam.distortion_type == MBA_DISTORTION_FOV) fovParamJacobian(cam.distortion, kp, Jd);
    else for (int i = 0; i < 8; ++i) Jd[i] = 0.0;
    for (int i = 0; i < 4; ++i) { Jd[i] *= fu; Jd[4 + i] *= fv; }
  }
  if (cam.distortion_type == MBA_DISTORTION_RADTAN) radtanDistort(cam.distortion, kp, Jp ? Jdist : nullptr);
  else if (cam.distortion_type == MBA_DISTORTION_EQUIDISTANT) equidistantDistort(cam.distortion, kp, Jp ? Jdist : nullptr);
  else if (cam.distortion_type == MBA_DISTORTION_FOV) fovDistort(cam.distortion, kp, Jp ? Jdist : nullptr);
  if (Jp) {
    const double rz2 = rz * rz;
    Jp[0] = fu * Jdist[0] * rz;
    Jp[1] = fu * Jdist[1] * rz;
    Jp[2] = -fu * (x * Jdist[0] + y * Jdist[1]) * rz2;
    Jp[3] = fv * Jdist[2] * rz;
    Jp[4] = fv * Jdist[3] * rz;
    Jp[5] = -fv * (x * Jdist[2] + y * Jdist[3]) * rz2;
  }
  if (Ji) {
    Ji[0] = kp[0]; Ji[1] = 0.0; Ji[2] = 1.0; Ji[3] = 0.0;
    Ji[4] = 0.0; Ji[5] = kp[1]; Ji[6] = 0.0; Ji[7] = 1.0;
  }
  kp[0] = fu * kp[0] + cu;
  kp[1] = fv * kp[1] + cv;
  // camera-pinhole-inl.h:47-65, camera-inl.h:17-25
  constexpr double kMinimumDepth = 1e-10;
  const bool vis = kp[0] >= 0.0 && kp[1] >= 0.0 && kp[0] < (double)cam.width && kp[1] < (double)cam.height;
  if (vis && z > kMinimumDepth) return KEYPOINT_VISIBLE;
  if (!vis && z > kMinimumDepth) return KEYPOINT_OUTSIDE_IMAGE_BOX;
  if (z < 0.0) return POINT_BEHIND_CAMERA;
  return PROJECTION_INVALID;
}

// ---------------------------------------------------------------- visual
// out(2xC) = A(2x3) * B(3xC)
static void mul23(const double* A, const double* B, int C, double* out) {
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < C; ++c)
      out[r * C + c] = A[3 * r] * B[c] + A[3 * r + 1] * B[C + c] + A[3 * r + 2] * B[2 * C + c];
}

// Writes J_kp * J_theta * 4 * Jq^T * s into a 2x7 pose block (cols 0..3) and
// J_kp * J_pos * s into cols 4..6 (visual-error-term-inl.h:246-318).
static void writePoseBlock(const double* Jkp, const double* Jth, const double* Jpos, const double* q,
                           double s, double* out27) {
  double Jq[12], JqT4[12], A[6], B[8], C[6];
  jplQuaternionJacobian(q, Jq);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) JqT4[4 * r + c] = 4.0 * Jq[3 * c + r];
  mul23(Jkp, Jth, 3, A);
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 4; ++c)
      B[4 * r + c] = (A[3 * r] * JqT4[c] + A[3 * r + 1] * JqT4[4 + c] + A[3 * r + 2] * JqT4[8 + c]) * s;
  mul23(Jkp, Jpos, 3, C);
  for (int r = 0; r < 2; ++r) {
    for (int c = 0; c < 4; ++c) out27[7 * r + c] = B[4 * r + c];
    for (int c = 0; c < 3; ++c) out27[7 * r + 4 + c] = C[3 * r + c] * s;
  }
}

// Landmark position in the observing camera frame (VIMap::getLandmark_p_C_fi,
// map-structure/vi-map/src/vi-map.cc, as used by findOutlierLandmarks in
// outlier-rejection-solver.cc:62-63): the frame chain of the visual term.
void visualPointInCamera(const double* const* P, int type, double* p_C) {
  const double* p_B = P[0];
  double R[9], Rt[9], p_I[3], p_M[3], t[3];
  if (type == MBA_LOCAL_KEYFRAME) {
    for (int i = 0; i < 3; ++i) p_I[i] = p_B[i];
  } else {
    toRotationMatrixJPL(P[1], R);
    mat3_transpose(R, Rt);
    double p_LM[3];
    mat3_vec(Rt, p_B, p_LM);
    for (int i = 0; i < 3; ++i) p_LM[i] += P[1][4 + i];
    if (type == MBA_LOCAL_MISSION) {
      for (int i = 0; i < 3; ++i) p_M[i] = p_LM[i];
    } else {
      double p_G[3];
      toRotationMatrixJPL(P[2], R);
      mat3_vec(R, p_LM, p_G);
      for (int i = 0; i < 3; ++i) t[i] = p_G[i] + P[2][4 + i] - P[3][4 + i];
      toRotationMatrixJPL(P[3], R);
      mat3_transpose(R, Rt);
      mat3_vec(Rt, t, p_M);
    }
    toRotationMatrixJPL(P[4], R);
    for (int i = 0; i < 3; ++i) t[i] = p_M[i] - P[4][4 + i];
    mat3_vec(R, t, p_I);
  }
  toRotationMatrixJPL(P[5], R);
  mat3_vec(R, p_I, p_C);
  for (int i = 0; i < 3; ++i) p_C[i] += P[6][i];
}

bool visualEvaluate(const double* const* P, const double* meas, double pixel_sigma, int type,
                    const mba_camera& cam, double* residual, double** jac, bool* failed_out) {
  const double sinv = 1.0 / pixel_sigma;
  const double* p_B = P[0];
  const double* q_B_LM = P[1];
  const double* p_LM_B = P[1] + 4;
  const double* q_G_LM = P[2];
  const double* p_G_LM = P[2] + 4;
  const double* q_G_M = P[3];
  const double* p_G_M = P[3] + 4;
  const double* q_I_M = P[4];
  const double* p_M_I = P[4] + 4;
  const double* q_C_I = P[5];
  const double* p_C_I = P[6];
  mba_camera c = cam;
  if (P[7]) std::memcpy(c.intrinsics, P[7], 4 * sizeof(double));
  if (P[8] && c.distortion_type != MBA_DISTORTION_NONE) std::memcpy(c.distortion, P[8], 4 * sizeof(double));

  double R_B_LM[9], R_LM_B[9], R_G_LM[9], R_G_M[9], R_M_G[9], R_I_M[9], R_C_I[9];
  toRotationMatrixJPL(q_C_I, R_C_I);
  double p_M[3] = {0, 0, 0}, p_G[3] = {0, 0, 0}, p_I[3] = {0, 0, 0}, t[3];
  if (type == MBA_LOCAL_KEYFRAME) {
    p_I[0] = p_B[0]; p_I[1] = p_B[1]; p_I[2] = p_B[2];
  } else {
    toRotationMatrixJPL(q_B_LM, R_B_LM);
    mat3_transpose(R_B_LM, R_LM_B);
    toRotationMatrixJPL(q_I_M, R_I_M);
    if (type == MBA_LOCAL_MISSION) {
      mat3_vec(R_LM_B, p_B, p_M);
      for (int i = 0; i < 3; ++i) { p_M[i] += p_LM_B[i]; t[i] = p_M[i] - p_M_I[i]; }
      mat3_vec(R_I_M, t, p_I);
    } else {
      toRotationMatrixJPL(q_G_LM, R_G_LM);
      toRotationMatrixJPL(q_G_M, R_G_M);
      mat3_transpose(R_G_M, R_M_G);
      double p_LM[3];
      mat3_vec(R_LM_B, p_B, p_LM);
      for (int i = 0; i < 3; ++i) p_LM[i] += p_LM_B[i];
      mat3_vec(R_G_LM, p_LM, p_G);
      for (int i = 0; i < 3; ++i) { p_G[i] += p_G_LM[i]; t[i] = p_G[i] - p_G_M[i]; }
      mat3_vec(R_M_G, t, p_M);
      for (int i = 0; i < 3; ++i) t[i] = p_M[i] - p_M_I[i];
      mat3_vec(R_I_M, t, p_I);
    }
  }
  double p_C[3];
  mat3_vec(R_C_I, p_I, p_C);
  for (int i = 0; i < 3; ++i) p_C[i] += p_C_I[i];

  double kp[2], Jkp[6], Ji[8], Jd[8];
  const bool want_i = jac && jac[7];
  const bool want_d = jac && jac[8] && c.distortion_type != MBA_DISTORTION_NONE;
  const int res = pinholeProject3(c, p_C, kp, jac ? Jkp : nullptr, want_i ? Ji : nullptr, want_d ? Jd : nullptr);
  const bool failed = res == POINT_BEHIND_CAMERA || res == PROJECTION_INVALID || p_C[2] < 0.05 ||
                      (kp[0] * kp[0] + kp[1] * kp[1]) > 1.0e5 * 1.0e5;
  if (failed_out) *failed_out = failed;

  if (jac) {
    double J_pCI[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, J_qCI[9], RCIpI[3];
    mat3_vec(R_C_I, p_I, RCIpI);
    skew(RCIpI, J_qCI);
    double J_pMI[9], J_pGM[9], J_pGLM[9], J_pLMB[9], J_pB[9], J_qBLM[9], J_qGLM[9], J_qGM[9], J_qIM[9], S[9];
    std::memset(J_pMI, 0, sizeof(J_pMI)); std::memset(J_pGM, 0, sizeof(J_pGM));
    std::memset(J_pGLM, 0, sizeof(J_pGLM)); std::memset(J_pLMB, 0, sizeof(J_pLMB));
    std::memset(J_qBLM, 0, sizeof(J_qBLM)); std::memset(J_qGLM, 0, sizeof(J_qGLM));
    std::memset(J_qGM, 0, sizeof(J_qGM)); std::memset(J_qIM, 0, sizeof(J_qIM));
    if (type == MBA_GLOBAL) {
      // visual-error-term-inl.h:188-210
      mat3_mul(R_C_I, R_I_M, J_pMI); mat3_scale(J_pMI, -1.0);
      mat3_mul(J_pMI, R_M_G, J_pGM);
      for (int i = 0; i < 9; ++i) J_pGLM[i] = -J_pGM[i];
      mat3_mul(J_pGLM, R_G_LM, J_pLMB);
      mat3_mul(J_pLMB, R_LM_B, J_pB);
      skew(p_B, S); mat3_mul(J_pB, S, J_qBLM); mat3_scale(J_qBLM, -1.0);
      skew(p_G, S); mat3_mul(J_pGLM, S, J_qGLM);
      mat3_mul(J_pGM, S, J_qGM);
      skew(p_I, S); mat3_mul(R_C_I, S, J_qIM);
    } else if (type == MBA_LOCAL_MISSION) {
      // visual-error-term-inl.h:211-224
      mat3_mul(R_C_I, R_I_M, J_pMI); mat3_scale(J_pMI, -1.0);
      for (int i = 0; i < 9; ++i) J_pLMB[i] = -J_pMI[i];
      skew(p_I, S); mat3_mul(R_C_I, S, J_qIM);
      mat3_mul(J_pLMB, R_LM_B, J_pB);
      skew(p_B, S); mat3_mul(J_pB, S, J_qBLM); mat3_scale(J_qBLM, -1.0);
    } else {
      std::memcpy(J_pB, R_C_I, sizeof(J_pB));
    }
    // Blocks Ceres would receive as nullptr in the maplab problem (dummies and
    // constant blocks) are written as zeros here when requested.
    const bool dummy_base = type == MBA_LOCAL_KEYFRAME;
    const bool dummy_mis = type != MBA_GLOBAL;
    if (jac[0]) {
      if (!failed) { mul23(Jkp, J_pB, 3, jac[0]); for (int i = 0; i < 6; ++i) jac[0][i] *= sinv; }
      else std::memset(jac[0], 0, 6 * sizeof(double));
    }
    if (jac[1]) {
      if (!failed && !dummy_base) writePoseBlock(Jkp, J_qBLM, J_pLMB, q_B_LM, sinv, jac[1]);
      else std::memset(jac[1], 0, 14 * sizeof(double));
    }
    if (jac[2]) {
      if (!failed && !dummy_mis) writePoseBlock(Jkp, J_qGLM, J_pGLM, q_G_LM, sinv, jac[2]);
      else std::memset(jac[2], 0, 14 * sizeof(double));
    }
    if (jac[3]) {
      if (!failed && !dummy_mis) writePoseBlock(Jkp, J_qGM, J_pGM, q_G_M, sinv, jac[3]);
      else std::memset(jac[3], 0, 14 * sizeof(double));
    }
    if (jac[4]) {
      if (!failed && !dummy_base) writePoseBlock(Jkp, J_qIM, J_pMI, q_I_M, sinv, jac[4]);
      else std::memset(jac[4], 0, 14 * sizeof(double));
    }
    if (jac[5]) {
      if (!failed) {
        double Jq[12], A[6];
        jplQuaternionJacobian(q_C_I, Jq);
        mul23(Jkp, J_qCI, 3, A);
        for (int r = 0; r < 2; ++r)
          for (int cc = 0; cc < 4; ++cc)
            jac[5][4 * r + cc] = (A[3 * r] * 4.0 * Jq[3 * cc] + A[3 * r + 1] * 4.0 * Jq[3 * cc + 1] +
                                  A[3 * r + 2] * 4.0 * Jq[3 * cc + 2]) * sinv;
      } else std::memset(jac[5], 0, 8 * sizeof(double));
    }
    if (jac[6]) {
      if (!failed) { mul23(Jkp, J_pCI, 3, jac[6]); for (int i = 0; i < 6; ++i) jac[6][i] *= sinv; }
      else std::memset(jac[6], 0, 6 * sizeof(double));
    }
    if (jac[7]) {
      if (!failed) for (int i = 0; i < 8; ++i) jac[7][i] = Ji[i] * sinv;
      else std::memset(jac[7], 0, 8 * sizeof(double));
    }
    if (jac[8]) {
      if (!failed && want_d) for (int i = 0; i < 8; ++i) jac[8][i] = Jd[i] * sinv;
      else std::memset(jac[8], 0, 8 * sizeof(double));
    }
  }
  if (!failed) {
    residual[0] = (kp[0] - meas[0]) * sinv;
    residual[1] = (kp[1] - meas[1]) * sinv;
  } else {
    residual[0] = residual[1] = 0.0;
  }
  return true;
}

// ---------------------------------------------------------------- IMU RK4
// gyroOmegaJPL (imu-integrator-inl.h:321-334) applied to q: 0.5 * Omega(w) q.
static void qdot(const double* w, const double* q, double* out) {
  out[0] = 0.5 * (w[2] * q[1] - w[1] * q[2] + w[0] * q[3]);
  out[1] = 0.5 * (-w[2] * q[0] + w[0] * q[2] + w[1] * q[3]);
  out[2] = 0.5 * (w[1] * q[0] - w[0] * q[1] + w[2] * q[3]);
  out[3] = 0.5 * (-w[0] * q[0] - w[1] * q[1] - w[2] * q[2]);
}

// getStateDerivativeRungeKutta (imu-integrator-inl.h:170-207).
static void stateDerivative(double g, const double* imu6, const double* s, double* d) {
  double q[4] = {s[0], s[1], s[2], s[3]};
  normalize4(q);
  double B_R_G[9], G_R_B[9];
  toRotationMatrixJPL(q, B_R_G);
  mat3_transpose(B_R_G, G_R_B);
  for (int i = 0; i < 16; ++i) d[i] = 0.0;
  qdot(imu6 + 3, q, d);
  double a[3];
  mat3_vec(G_R_B, imu6, a);
  d[7] = a[0]; d[8] = a[1]; d[9] = a[2] - g;
  d[13] = s[7]; d[14] = s[8]; d[15] = s[9];
}

// getCovarianceTransitionDerivativesRungeKutta (imu-integrator-inl.h:209-296).
static void covTransDerivative(const ImuNoise& n, const double* imu6, const double* s, const double* P,
                               const double* T, double* dP, double* dT) {
  double q[4] = {s[0], s[1], s[2], s[3]};
  normalize4(q);
  double B_R_G[9], G_R_B[9], gs[9], as[9], F00[9], F60[9], F69[9];
  toRotationMatrixJPL(q, B_R_G);
  mat3_transpose(B_R_G, G_R_B);
  skew(imu6 + 3, gs);
  skew(imu6, as);
  for (int i = 0; i < 9; ++i) { F00[i] = -gs[i]; F69[i] = -G_R_B[i]; }
  mat3_mul(G_R_B, as, F60);
  mat3_scale(F60, -1.0);
  // transition derivative rows 0-2, 6-8, 12-14 (others zero)
  for (int i = 0; i < 225; ++i) dT[i] = 0.0;
  double PC[225];
  for (int i = 0; i < 225; ++i) PC[i] = 0.0;
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 15; ++c) {
      dT[r * 15 + c] = F00[3 * r] * T[c] + F00[3 * r + 1] * T[15 + c] + F00[3 * r + 2] * T[30 + c] - T[(3 + r) * 15 + c];
      dT[(6 + r) * 15 + c] = (F60[3 * r] * T[c] + F60[3 * r + 1] * T[15 + c] + F60[3 * r + 2] * T[30 + c]) +
                             (F69[3 * r] * T[135 + c] + F69[3 * r + 1] * T[150 + c] + F69[3 * r + 2] * T[165 + c]);
      dT[(12 + r) * 15 + c] = T[(6 + r) * 15 + c];
      PC[r * 15 + c] = F00[3 * r] * P[c] + F00[3 * r + 1] * P[15 + c] + F00[3 * r + 2] * P[30 + c] - P[(3 + r) * 15 + c];
      PC[(6 + r) * 15 + c] = (F60[3 * r] * P[c] + F60[3 * r + 1] * P[15 + c] + F60[3 * r + 2] * P[30 + c]) +
                             (F69[3 * r] * P[135 + c] + F69[3 * r + 1] * P[150 + c] + F69[3 * r + 2] * P[165 + c]);
      PC[(12 + r) * 15 + c] = P[(6 + r) * 15 + c];
    }
  }
  for (int r = 0; r < 15; ++r)
    for (int c = 0; c < 15; ++c) dP[r * 15 + c] = PC[r * 15 + c] + PC[c * 15 + r];
  const double gn = n.gyro_noise_sigma * n.gyro_noise_sigma;
  const double gb = n.gyro_bias_sigma * n.gyro_bias_sigma;
  const double an = n.acc_noise_sigma * n.acc_noise_sigma;
  const double ab = n.acc_bias_sigma * n.acc_bias_sigma;
  for (int i = 0; i < 3; ++i) {
    dP[i * 16] += gn;
    dP[(3 + i) * 16] += gb;
    dP[(6 + i) * 16] += an;
    dP[(9 + i) * 16] += ab;
  }
}

void imuIntegrate(const ImuNoise& n, const double* s0, const double* rd, double dt, double* next,
                  double* phi, double* cov) {
  // imu-integrator-inl.h:17-168
  const double* k1r = rd;
  double k23r[6];
  // interpolateImuReadings (imu-integrator-inl.h:298-319)
  if (dt < 2.220446049250313e-16) {
    for (int i = 0; i < 6; ++i) k23r[i] = rd[i];
  } else {
    for (int i = 0; i < 6; ++i) k23r[i] = rd[i] + (rd[6 + i] - rd[i]) * ((0.5 * dt) / dt);
  }
  const double* k4r = rd + 6;
  double d1[16], d2[16], d3[16], d4[16], tmp[16];
  stateDerivative(n.gravity, k1r, s0, d1);
  for (int i = 0; i < 16; ++i) tmp[i] = s0[i] + 0.5 * dt * d1[i];
  stateDerivative(n.gravity, k23r, tmp, d2);
  for (int i = 0; i < 16; ++i) tmp[i] = s0[i] + 0.5 * dt * d2[i];
  stateDerivative(n.gravity, k23r, tmp, d3);
  for (int i = 0; i < 16; ++i) tmp[i] = s0[i] + dt * d3[i];
  stateDerivative(n.gravity, k4r, tmp, d4);
  for (int i = 0; i < 16; ++i) next[i] = s0[i] + dt * (d1[i] + 2.0 * d2[i] + 2.0 * d3[i] + d4[i]) / 6.0;
  if (!phi || !cov) return;

  static thread_local double P0[225], T0[225], cd[4][225], td[4][225], Pi[225], Ti[225];
  for (int i = 0; i < 225; ++i) { P0[i] = 0.0; T0[i] = 0.0; }
  for (int i = 0; i < 15; ++i) T0[i * 16] = 1.0;
  covTransDerivative(n, k1r, s0, P0, T0, cd[0], td[0]);
  for (int i = 0; i < 16; ++i) tmp[i] = s0[i] + 0.5 * dt * d1[i];
  for (int i = 0; i < 225; ++i) { Pi[i] = P0[i] + 0.5 * dt * cd[0][i]; Ti[i] = T0[i] + 0.5 * dt * td[0][i]; }
  covTransDerivative(n, k23r, tmp, Pi, Ti, cd[1], td[1]);
  for (int i = 0; i < 16; ++i) tmp[i] = s0[i] + 0.5 * dt * d2[i];
  for (int i = 0; i < 225; ++i) { Pi[i] = P0[i] + 0.5 * dt * cd[1][i]; Ti[i] = T0[i] + 0.5 * dt * td[1][i]; }
  covTransDerivative(n, k23r, tmp, Pi, Ti, cd[2], td[2]);
  for (int i = 0; i < 16; ++i) tmp[i] = s0[i] + dt * d3[i];
  for (int i = 0; i < 225; ++i) { Pi[i] = P0[i] + dt * cd[2][i]; Ti[i] = T0[i] + dt * td[2][i]; }
  covTransDerivative(n, k4r, tmp, Pi, Ti, cd[3], td[3]);
  for (int i = 0; i < 225; ++i)
    cov[i] = P0[i] + dt * (cd[0][i] + 2.0 * cd[1][i] + 2.0 * cd[2][i] + cd[3][i]) / 6.0;
  for (int i = 0; i < 225; ++i) phi[i] = T0[i];
  for (int blk : {0, 6, 12})
    for (int r = blk; r < blk + 3; ++r)
      for (int c = 0; c < 15; ++c) {
        const int k = r * 15 + c;
        phi[k] += dt * (td[0][k] + 2.0 * td[1][k] + 2.0 * td[2][k] + td[3][k]) / 6.0;
      }
}

// C(15x15) = A * B
static void mat15_mul(const double* A, const double* B, double* C) {
  for (int i = 0; i < 15; ++i)
    for (int j = 0; j < 15; ++j) {
      double s = 0.0;
      for (int k = 0; k < 15; ++k) s += A[i * 15 + k] * B[k * 15 + j];
      C[i * 15 + j] = s;
    }
}

bool inertialIntegrate(const ImuNoise& n, const double* begin, int ns, const int64_t* ts,
                       const double* imu, double* end, double* phi_acc, double* Q_acc) {
  // inertial-error-term.cc:9-75
  for (int i = 0; i < 225; ++i) { Q_acc[i] = 0.0; phi_acc[i] = 0.0; }
  for (int i = 0; i < 15; ++i) phi_acc[i * 16] = 1.0;
  double cur[16], nxt[16], rd[12], phi[225], Q[225], t1[225], t2[225];
  std::memcpy(cur, begin, sizeof(cur));
  std::memcpy(nxt, begin, sizeof(nxt));
  for (int i = 0; i < ns - 1; ++i) {
    if (ts[i + 1] < ts[i]) return false;
    for (int k = 0; k < 3; ++k) {
      rd[k] = imu[6 * i + k] - cur[10 + k];
      rd[3 + k] = imu[6 * i + 3 + k] - cur[4 + k];
      rd[6 + k] = imu[6 * (i + 1) + k] - cur[10 + k];
      rd[9 + k] = imu[6 * (i + 1) + 3 + k] - cur[4 + k];
    }
    const double dt = (double)(ts[i + 1] - ts[i]) * 1e-9;
    imuIntegrate(n, cur, rd, dt, nxt, phi, Q);
    std::memcpy(cur, nxt, sizeof(cur));
    // Q_acc = phi Q_acc phi^T + Q ; phi_acc = phi phi_acc
    mat15_mul(phi, Q_acc, t1);
    for (int r = 0; r < 15; ++r)
      for (int c = 0; c < 15; ++c) {
        double s = 0.0;
        for (int k = 0; k < 15; ++k) s += t1[r * 15 + k] * phi[c * 15 + k];
        Q_acc[r * 15 + c] = s + Q[r * 15 + c];
      }
    mat15_mul(phi, phi_acc, t2);
    std::memcpy(phi_acc, t2, sizeof(t2));
  }
  std::memcpy(end, nxt, sizeof(nxt));
  return true;
}

// Eigen::LLT<Matrix15d>::compute restated (the column-by-column in-place
// factorization Eigen uses below 32 rows): L L^T = A, lower triangle.  The
// reference calls compute() and then matrixL() without checking info()
// (inertial-error-term.cc:155-182), so a non-positive pivot does not fail
// the term: the factorization stops at that column j, whose diagonal and
// sub-diagonal keep A's values, as do all later columns of the lower
// triangle; the triangular solves then use that matrix.  Returns false in
// that case (the factor is still written).
static bool cholesky15(const double* A, double* L) {
  for (int i = 0; i < 225; ++i) L[i] = 0.0;
  for (int i = 0; i < 15; ++i)
    for (int k = 0; k <= i; ++k) L[i * 15 + k] = A[i * 15 + k];
  for (int j = 0; j < 15; ++j) {
    double d = A[j * 15 + j];
    for (int k = 0; k < j; ++k) d -= L[j * 15 + k] * L[j * 15 + k];
    if (!(d > 0.0)) return false;
    const double ljj = std::sqrt(d);
    L[j * 15 + j] = ljj;
    for (int i = j + 1; i < 15; ++i) {
      double s = A[i * 15 + j];
      for (int k = 0; k < j; ++k) s -= L[i * 15 + k] * L[j * 15 + k];
      L[i * 15 + j] = s / ljj;
    }
  }
  return true;
}

// In-place forward substitution L X = B for B (15 x cols, row-major).
static void forwardSubst(const double* L, double* B, int cols) {
  for (int c = 0; c < cols; ++c)
    for (int i = 0; i < 15; ++i) {
      double s = B[i * cols + c];
      for (int k = 0; k < i; ++k) s -= L[i * 15 + k] * B[k * cols + c];
      B[i * cols + c] = s / L[i * 15 + i];
    }
}

int inertialEvaluate(const ImuNoise& n, const double* const* P, int ns, const int64_t* ts,
                     const double* imu, double* res, double** jac) {
  // inertial-error-term.cc:77-286
  double begin[16], end[16], phi[225], Q[225], L[225];
  std::memcpy(begin, P[0], 4 * sizeof(double));
  std::memcpy(begin + 4, P[1], 3 * sizeof(double));
  std::memcpy(begin + 7, P[2], 3 * sizeof(double));
  std::memcpy(begin + 10, P[3], 3 * sizeof(double));
  std::memcpy(begin + 13, P[0] + 4, 3 * sizeof(double));
  if (!inertialIntegrate(n, begin, ns, ts, imu, end, phi, Q)) return MBA_ERR_UNORDERED_IMU;
  cholesky15(Q, L);  // a non-positive-definite Q_accum is used as Eigen leaves it (no failure)
  const double* q_to = P[4];
  if (res) {
    // Eigen::Quaterniond::inverse(): conjugate / squaredNorm.
    const double* qi = end;
    const double n2 = qi[0] * qi[0] + qi[1] * qi[1] + qi[2] * qi[2] + qi[3] * qi[3];
    double qinv[4];
    if (n2 > 0.0) { qinv[0] = -qi[0] / n2; qinv[1] = -qi[1] / n2; qinv[2] = -qi[2] / n2; qinv[3] = qi[3] / n2; }
    else { qinv[0] = qinv[1] = qinv[2] = qinv[3] = 0.0; }
    double dq[4];
    positiveQuaternionProductJPL(q_to, qinv, dq);
    res[0] = 2.0 * dq[0]; res[1] = 2.0 * dq[1]; res[2] = 2.0 * dq[2];
    for (int k = 0; k < 3; ++k) {
      res[3 + k] = P[5][k] - end[4 + k];
      res[6 + k] = P[6][k] - end[7 + k];
      res[9 + k] = P[7][k] - end[10 + k];
      res[12 + k] = P[4][4 + k] - end[13 + k];
    }
    forwardSubst(L, res, 1);
  }
  if (jac) {
    double Je[15 * 16], Jb[15 * 16], tl_end[12], tl_begin[12];
    jplQuaternionJacobian(q_to, tl_end);
    jplQuaternionJacobian(P[0], tl_begin);
    for (int i = 0; i < 240; ++i) { Je[i] = 0.0; Jb[i] = 0.0; }
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c) Je[r * 16 + c] = 4.0 * tl_end[c * 3 + r];
    for (int i = 0; i < 12; ++i) Je[(3 + i) * 16 + 4 + i] = 1.0;
    // J_begin (inertial-error-term.cc:215-225)
    for (int r = 0; r < 15; ++r) {
      for (int c = 0; c < 4; ++c) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += phi[r * 15 + k] * tl_begin[c * 3 + k];
        Jb[r * 16 + c] = -4.0 * s;
      }
      for (int c = 0; c < 12; ++c) Jb[r * 16 + 4 + c] = -phi[r * 15 + 3 + c];
    }
    forwardSubst(L, Je, 16);
    forwardSubst(L, Jb, 16);
    // Scatter (inertial-error-term.cc:235-283). State column layout:
    // q 0..3, b_g 4..6, v 7..9, b_a 10..12, p 13..15.
    const double* src[2] = {Jb, Je};
    for (int s = 0; s < 2; ++s) {
      const double* J = src[s];
      double* pose = jac[4 * s + 0];
      double* bg = jac[4 * s + 1];
      double* v = jac[4 * s + 2];
      double* ba = jac[4 * s + 3];
      for (int r = 0; r < 15; ++r) {
        if (pose) {
          for (int c = 0; c < 4; ++c) pose[r * 7 + c] = J[r * 16 + c];
          for (int c = 0; c < 3; ++c) pose[r * 7 + 4 + c] = J[r * 16 + 13 + c];
        }
        if (bg) for (int c = 0; c < 3; ++c) bg[r * 3 + c] = J[r * 16 + 4 + c];
        if (v) for (int c = 0; c < 3; ++c) v[r * 3 + c] = J[r * 16 + 7 + c];
        if (ba) for (int c = 0; c < 3; ++c) ba[r * 3 + c] = J[r * 16 + 10 + c];
      }
    }
  }
  return 0;
}


// ---------------------------------------------------------------- pose edges
// Forward-mode dual number with N derivative components (the role of
// ceres::Jet in the reference's AutoDiffCostFunction).
template <int N>
struct Dual {
  double a = 0.0;
  double d[N] = {};
  Dual() = default;
  Dual(double v) : a(v) {}  // NOLINT
};
template <int N> Dual<N> operator+(const Dual<N>& x, const Dual<N>& y) { Dual<N> r(x.a + y.a); for (int i = 0; i < N; ++i) r.d[i] = x.d[i] + y.d[i]; return r; }
template <int N> Dual<N> operator-(const Dual<N>& x, const Dual<N>& y) { Dual<N> r(x.a - y.a); for (int i = 0; i < N; ++i) r.d[i] = x.d[i] - y.d[i]; return r; }
template <int N> Dual<N> operator-(const Dual<N>& x) { Dual<N> r(-x.a); for (int i = 0; i < N; ++i) r.d[i] = -x.d[i]; return r; }
template <int N> Dual<N> operator*(const Dual<N>& x, const Dual<N>& y) { Dual<N> r(x.a * y.a); for (int i = 0; i < N; ++i) r.d[i] = x.a * y.d[i] + x.d[i] * y.a; return r; }
template <int N> Dual<N> operator/(const Dual<N>& x, const Dual<N>& y) {
  const double inv = 1.0 / y.a, q = x.a * inv;
  Dual<N> r(q);
  for (int i = 0; i < N; ++i) r.d[i] = (x.d[i] - q * y.d[i]) * inv;
  return r;
}
template <int N> Dual<N> sqrtS(const Dual<N>& x) {
  const double v = std::sqrt(x.a), h = 0.5 / v;
  Dual<N> r(v);
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] * h;
  return r;
}
static inline double sqrtS(double x) { return std::sqrt(x); }
template <int N> double valueOf(const Dual<N>& x) { return x.a; }
static inline double valueOf(double x) { return x; }
template <int N> bool isNegative(const Dual<N>& x) { return x.a < 0.0; }

// Hamilton quaternion (x y z w) product, rotation (Eigen's _transformVector
// form), and the transformation algebra of minkindr (x -> R(q) x + p).
template <typename S> static void hqMul(const S* a, const S* b, S* o) {
  o[3] = a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2];
  o[0] = a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1];
  o[1] = a[3] * b[1] - a[0] * b[2] + a[1] * b[3] + a[2] * b[0];
  o[2] = a[3] * b[2] + a[0] * b[1] - a[1] * b[0] + a[2] * b[3];
}
template <typename S> static void hqRot(const S* q, const S* v, S* o) {
  const S two(2.0);
  S uv[3] = {two * (q[1] * v[2] - q[2] * v[1]), two * (q[2] * v[0] - q[0] * v[2]), two * (q[0] * v[1] - q[1] * v[0])};
  o[0] = v[0] + q[3] * uv[0] + (q[1] * uv[2] - q[2] * uv[1]);
  o[1] = v[1] + q[3] * uv[1] + (q[2] * uv[0] - q[0] * uv[2]);
  o[2] = v[2] + q[3] * uv[2] + (q[0] * uv[1] - q[1] * uv[0]);
}
template <typename S> static void htMul(const S* A, const S* B, S* O) {
  hqMul(A, B, O);
  S r[3];
  hqRot(A, B + 4, r);
  for (int i = 0; i < 3; ++i) O[4 + i] = r[i] + A[4 + i];
}
template <typename S> static void htInv(const S* A, S* O) {
  O[0] = -A[0]; O[1] = -A[1]; O[2] = -A[2]; O[3] = A[3];
  S r[3];
  hqRot(O, A + 4, r);
  for (int i = 0; i < 3; ++i) O[4 + i] = -r[i];
}

// SixDoFBlockPoseErrorTermWithExtrinsics::operator()
// (six-dof-block-pose-error-term-with-extrinsics-autodiff-inl.h:6-55):
// T_Bk_Bkp1_est = T_B_I T_G_Ik^-1 T_G_Ikp1 T_B_I^-1 with the keyframe blocks'
// coefficients read as Hamilton quaternions; e = [p_meas - p_est;
// 2 vec(q_meas^-1 q_est) (w >= 0)]; e_w = e^T sqrtinfo (row vector).
template <typename S>
static void poseEdgeResidual(const S* xk, const S* xk1, const double* ext, const double* meas, const double* M, S* ew) {
  S TBI[7] = {S(-ext[0]), S(-ext[1]), S(-ext[2]), S(ext[3]), S(ext[4]), S(ext[5]), S(ext[6])};
  S TkI[7], TBIi[7], X[7], Y[7], Te[7];
  htInv(xk, TkI);
  htInv(TBI, TBIi);
  htMul(TBI, TkI, X);
  htMul(X, xk1, Y);
  htMul(Y, TBIi, Te);
  const S qmi[4] = {S(-meas[0]), S(-meas[1]), S(-meas[2]), S(meas[3])};
  S qe[4];
  hqMul(qmi, Te, qe);
  if (isNegative(qe[3]))
    for (int i = 0; i < 4; ++i) qe[i] = -qe[i];
  S e[6];
  for (int i = 0; i < 3; ++i) e[i] = S(meas[4 + i]) - Te[4 + i];
  for (int i = 0; i < 3; ++i) e[3 + i] = S(2.0) * qe[i];
  for (int j = 0; j < 6; ++j) {
    S acc(0.0);
    for (int i = 0; i < 6; ++i) acc = acc + e[i] * S(M[6 * i + j]);
    ew[j] = acc;
  }
}

// JPL quaternion algebra on any scalar (quaternion-math-inl.h):
// toRotationMatrixJPL (:6-27), quaternionInverseJPL (:156-163) and
// positiveQuaternionProductJPL (:112-154: left-multiplication matrix of q1
// times q2, normalized, sign flipped to w >= 0).
template <typename S> static void jplRotS(const S* q, S* R) {
  const S one(1.0), two(2.0);
  R[0] = one - two * (q[1] * q[1] + q[2] * q[2]);
  R[1] = two * (q[0] * q[1] + q[2] * q[3]);
  R[2] = two * (q[0] * q[2] - q[1] * q[3]);
  R[3] = two * (q[0] * q[1] - q[2] * q[3]);
  R[4] = one - two * (q[0] * q[0] + q[2] * q[2]);
  R[5] = two * (q[1] * q[2] + q[0] * q[3]);
  R[6] = two * (q[0] * q[2] + q[1] * q[3]);
  R[7] = two * (q[1] * q[2] - q[0] * q[3]);
  R[8] = one - two * (q[0] * q[0] + q[1] * q[1]);
}
template <typename S> static void jplInvS(const S* q, S* o) { o[0] = -q[0]; o[1] = -q[1]; o[2] = -q[2]; o[3] = q[3]; }
template <typename S> static void jplProdPosS(const S* a, const S* b, S* o) {
  S p[4];
  p[0] = a[3] * b[0] + a[2] * b[1] - a[1] * b[2] + a[0] * b[3];
  p[1] = -a[2] * b[0] + a[3] * b[1] + a[0] * b[2] + a[1] * b[3];
  p[2] = a[1] * b[0] - a[0] * b[1] + a[3] * b[2] + a[2] * b[3];
  p[3] = -a[0] * b[0] - a[1] * b[1] - a[2] * b[2] + a[3] * b[3];
  const S z = p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3];
  if (valueOf(z) > 0.0) {
    const S n = sqrtS(z);
    for (int i = 0; i < 4; ++i) p[i] = p[i] / n;
  }
  const bool flip = isNegative(p[3]);
  for (int i = 0; i < 4; ++i) o[i] = flip ? -p[i] : p[i];
}
template <typename S> static void mat3MulS(const S* A, const S* B, S* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}
template <typename S> static void mat3VecS(const S* A, const S* v, S* o) {
  for (int i = 0; i < 3; ++i) o[i] = A[3 * i] * v[0] + A[3 * i + 1] * v[1] + A[3 * i + 2] * v[2];
}
template <typename S> static void transpose3S(const S* A, S* B) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) B[3 * j + i] = A[3 * i + j];
}

// Rotation matrix (row-major) to Hamilton quaternion (x y z w), the
// trace / largest-diagonal method (K. Shoemake, "Animating rotation with
// quaternion curves", SIGGRAPH 1985), in the form Eigen's
// Quaternion(const Matrix3&) constructor uses.
template <typename S> static void rotToHamiltonS(const S* m, S* q) {
  const S tr = m[0] + m[4] + m[8];
  if (valueOf(tr) > 0.0) {
    S t = sqrtS(tr + S(1.0));
    q[3] = S(0.5) * t;
    t = S(0.5) / t;
    q[0] = (m[7] - m[5]) * t;
    q[1] = (m[2] - m[6]) * t;
    q[2] = (m[3] - m[1]) * t;
  } else {
    int i = 0;
    if (valueOf(m[4]) > valueOf(m[0])) i = 1;
    if (valueOf(m[8]) > valueOf(m[4 * i])) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    S t = sqrtS(m[4 * i] - m[4 * j] - m[4 * k] + S(1.0));
    q[i] = S(0.5) * t;
    t = S(0.5) / t;
    q[3] = (m[3 * k + j] - m[3 * j + k]) * t;
    q[j] = (m[3 * j + i] + m[3 * i + j]) * t;
    q[k] = (m[3 * k + i] + m[3 * i + k]) * t;
  }
}

template <typename S> static void whiten6(const S* e, const double* M, S* ew) {
  for (int j = 0; j < 6; ++j) {
    S acc(0.0);
    for (int i = 0; i < 6; ++i) acc = acc + e[i] * S(M[6 * i + j]);
    ew[j] = acc;
  }
}

// LoopClosureEdgeErrorTerm::operator() (loop-closure-edge-error-term-inl.h:
// 6-81), without the switch factor: baseframes T_G_MA, T_G_MB (JPL q | p,
// constants; identity for two vertices of one mission, :83-95), vertex
// blocks q_IA_MA | p_MA_IA; measurement q_AB (JPL) | p_AB.
template <typename S>
static void loopClosureResidual(const double* bfA, const double* bfB, const S* xA, const S* xB, const double* meas,
                                const double* M, S* ew) {
  S qGMA[4], qGMB[4], RGMA[9], RGMB[9];
  for (int i = 0; i < 4; ++i) { qGMA[i] = S(bfA[i]); qGMB[i] = S(bfB[i]); }
  jplRotS(qGMA, RGMA);
  jplRotS(qGMB, RGMB);
  S pA[3], pB[3], pGIA[3], pGIB[3];
  mat3VecS(RGMA, xA + 4, pA);
  mat3VecS(RGMB, xB + 4, pB);
  for (int i = 0; i < 3; ++i) { pGIA[i] = S(bfA[4 + i]) + pA[i]; pGIB[i] = S(bfB[4 + i]) + pB[i]; }
  S qi[4], qGIA[4], qGIB[4], qIAIB[4], qlci[4], qerr[4];
  jplInvS(xA, qi);
  jplProdPosS(qGMA, qi, qGIA);
  jplInvS(xB, qi);
  jplProdPosS(qGMB, qi, qGIB);
  jplInvS(qGIA, qi);
  jplProdPosS(qi, qGIB, qIAIB);
  const S qlc[4] = {S(meas[0]), S(meas[1]), S(meas[2]), S(meas[3])};
  jplInvS(qlc, qlci);
  jplProdPosS(qlci, qIAIB, qerr);
  S RIAG[9], d[3], e[6];
  jplInvS(qGIA, qi);
  jplRotS(qi, RIAG);
  for (int i = 0; i < 3; ++i) d[i] = pGIB[i] - pGIA[i];
  mat3VecS(RIAG, d, e);
  for (int i = 0; i < 3; ++i) e[i] = e[i] - S(meas[4 + i]);
  for (int i = 0; i < 3; ++i) e[3 + i] = S(2.0) * qerr[i];
  whiten6(e, M, ew);
}

// BlockPosePriorErrorTermV2::operator() (block-pose-prior-error-term-v2-inl.h:
// 8-60): baseframe q_G_M | p_G_M and sensor extrinsics q_S_B | p_S_B (JPL,
// constants), vertex block q_B_M | p_M_B; measurement q_S_G (Hamilton, the
// inverse of the measured rotation, as the constructor stores it) | p_G_S.
template <typename S>
static void absolutePoseResidual(const double* bf, const S* x, const double* ext, const double* meas, const double* M,
                                 S* ew) {
  S q[4], RGM[9], RBM[9], RMB[9], RSB[9], RBS[9], A[9], RGS[9];
  for (int i = 0; i < 4; ++i) q[i] = S(bf[i]);
  jplRotS(q, RGM);
  jplRotS(x, RBM);
  transpose3S(RBM, RMB);
  for (int i = 0; i < 4; ++i) q[i] = S(ext[i]);
  jplRotS(q, RSB);
  transpose3S(RSB, RBS);
  mat3MulS(RGM, RMB, A);
  mat3MulS(A, RBS, RGS);
  const S pSB[3] = {S(ext[4]), S(ext[5]), S(ext[6])};
  S pBS[3], a[3], b[3], e[6];
  mat3VecS(RBS, pSB, pBS);
  for (int i = 0; i < 3; ++i) pBS[i] = -pBS[i];
  mat3VecS(A, pBS, a);
  mat3VecS(RGM, x + 4, b);
  for (int i = 0; i < 3; ++i) e[i] = a[i] + b[i] + S(bf[4 + i]) - S(meas[4 + i]);
  S qGS[4], qd[4];
  rotToHamiltonS(RGS, qGS);
  const S qSG[4] = {S(meas[0]), S(meas[1]), S(meas[2]), S(meas[3])};
  hqMul(qGS, qSG, qd);
  for (int i = 0; i < 3; ++i) e[3 + i] = S(2.0) * qd[i];
  whiten6(e, M, ew);
}

void loopClosureEvaluate(const double* bfA, const double* bfB, const double* xA, const double* xB, const double* meas,
                         const double* M, double* r, double* JA, double* JB) {
  typedef Dual<14> D;
  D a[7], b[7], ew[6];
  for (int i = 0; i < 7; ++i) { a[i] = D(xA[i]); a[i].d[i] = 1.0; b[i] = D(xB[i]); b[i].d[7 + i] = 1.0; }
  loopClosureResidual(bfA, bfB, a, b, meas, M, ew);
  for (int j = 0; j < 6; ++j) {
    r[j] = ew[j].a;
    for (int c = 0; c < 7; ++c) {
      if (JA) JA[7 * j + c] = ew[j].d[c];
      if (JB) JB[7 * j + c] = ew[j].d[7 + c];
    }
  }
}

void absolutePoseEvaluate(const double* bf, const double* x, const double* ext, const double* meas, const double* M,
                          double* r, double* J) {
  typedef Dual<7> D;
  D a[7], ew[6];
  for (int i = 0; i < 7; ++i) { a[i] = D(x[i]); a[i].d[i] = 1.0; }
  absolutePoseResidual(bf, a, ext, meas, M, ew);
  for (int j = 0; j < 6; ++j) {
    r[j] = ew[j].a;
    if (J) for (int c = 0; c < 7; ++c) J[7 * j + c] = ew[j].d[c];
  }
}

// Residual and ambient Jacobians ([6][7] each, w.r.t. q(4) p(3)) by forward
// differentiation, as AutoDiffCostFunction computes them.
void poseEdgeEvaluate(const double* xk, const double* xk1, const double* ext, const double* meas, const double* M,
                      double* r, double* Jk, double* Jk1) {
  typedef Dual<14> D;
  D a[7], b[7], ew[6];
  for (int i = 0; i < 7; ++i) { a[i] = D(xk[i]); a[i].d[i] = 1.0; b[i] = D(xk1[i]); b[i].d[7 + i] = 1.0; }
  poseEdgeResidual(a, b, ext, meas, M, ew);
  for (int j = 0; j < 6; ++j) {
    r[j] = ew[j].a;
    for (int c = 0; c < 7; ++c) {
      if (Jk) Jk[7 * j + c] = ew[j].d[c];
      if (Jk1) Jk1[7 * j + c] = ew[j].d[7 + c];
    }
  }
}

// Square-root information of a 6x6 covariance: L^-1 with L L^T = cov
// (SixDoFBlockPoseErrorTermWithExtrinsics constructor, Eigen llt + triangular
// solve).  Returns false if cov is not positive definite.
bool poseEdgeSqrtInfo(const double* cov, double* M) {
  double L[36] = {};
  for (int j = 0; j < 6; ++j) {
    double dsum = cov[7 * j];
    for (int k = 0; k < j; ++k) dsum -= L[6 * j + k] * L[6 * j + k];
    if (!(dsum > 0.0)) return false;
    L[7 * j] = std::sqrt(dsum);
    for (int i = j + 1; i < 6; ++i) {
      double v = cov[6 * i + j];
      for (int k = 0; k < j; ++k) v -= L[6 * i + k] * L[6 * j + k];
      L[6 * i + j] = v / L[7 * j];
    }
  }
  for (int c = 0; c < 6; ++c)
    for (int i = 0; i < 6; ++i) {
      double v = (i == c) ? 1.0 : 0.0;
      for (int k = c; k < i; ++k) v -= L[6 * i + k] * M[6 * k + c];
      M[6 * i + c] = (i < c) ? 0.0 : v / L[7 * i];
    }
  return true;
}

}  // namespace oracle
