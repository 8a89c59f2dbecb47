// Device-side math of the VI bundle adjustment: JPL quaternions, pinhole
// projection with radtan / equidistant distortion, and the visual
// reprojection residual with its tangent-space Jacobians.
//
// Restates (same formulas, fused into one pass per observation):
//   common/maplab-common/include/maplab-common/quaternion-math-inl.h:6-163
//   algorithms/ceres-error-terms/src/parameterization/quaternion-param-jpl.cc:8-76
//   aslam_cv2/aslam_cv_cameras/src/camera-pinhole.cc:65-164
//   aslam_cv2/aslam_cv_cameras/include/aslam/cameras/camera-pinhole-inl.h:47-65
//   aslam_cv2/aslam_cv_cameras/src/distortion-radtan.cc:14-91
//   aslam_cv2/aslam_cv_cameras/src/distortion-equidistant.cc:14-142
//   algorithms/ceres-error-terms/include/ceres-error-terms/visual-error-term-inl.h:12-379
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/maplab_ba.h"

namespace mba {

template <typename T>
struct M3 {
  T m[9];
};

template <typename T>
__device__ __forceinline__ void jplR(const T* q, M3<T>& R) {
  // toRotationMatrixJPL (quaternion-math-inl.h:6-27)
  const T one = T(1), two = T(2);
  R.m[0] = one - two * (q[1] * q[1] + q[2] * q[2]);
  R.m[1] = two * (q[0] * q[1] + q[2] * q[3]);
  R.m[2] = two * (q[0] * q[2] - q[1] * q[3]);
  R.m[3] = two * (q[0] * q[1] - q[2] * q[3]);
  R.m[4] = one - two * (q[0] * q[0] + q[2] * q[2]);
  R.m[5] = two * (q[1] * q[2] + q[0] * q[3]);
  R.m[6] = two * (q[0] * q[2] + q[1] * q[3]);
  R.m[7] = two * (q[1] * q[2] - q[0] * q[3]);
  R.m[8] = one - two * (q[0] * q[0] + q[1] * q[1]);
}

template <typename T>
__device__ __forceinline__ void mv3(const M3<T>& A, const T* x, T* y) {
  const T a = A.m[0] * x[0] + A.m[1] * x[1] + A.m[2] * x[2];
  const T b = A.m[3] * x[0] + A.m[4] * x[1] + A.m[5] * x[2];
  const T c = A.m[6] * x[0] + A.m[7] * x[1] + A.m[8] * x[2];
  y[0] = a; y[1] = b; y[2] = c;
}
// y = A^T x
template <typename T>
__device__ __forceinline__ void mtv3(const M3<T>& A, const T* x, T* y) {
  const T a = A.m[0] * x[0] + A.m[3] * x[1] + A.m[6] * x[2];
  const T b = A.m[1] * x[0] + A.m[4] * x[1] + A.m[7] * x[2];
  const T c = A.m[2] * x[0] + A.m[5] * x[1] + A.m[8] * x[2];
  y[0] = a; y[1] = b; y[2] = c;
}
template <typename T>
__device__ __forceinline__ M3<T> mm3(const M3<T>& A, const M3<T>& B) {
  M3<T> C;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C.m[3 * i + j] = A.m[3 * i] * B.m[j] + A.m[3 * i + 1] * B.m[3 + j] + A.m[3 * i + 2] * B.m[6 + j];
  return C;
}
// C = A^T B
template <typename T>
__device__ __forceinline__ M3<T> mtm3(const M3<T>& A, const M3<T>& B) {
  M3<T> C;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C.m[3 * i + j] = A.m[i] * B.m[j] + A.m[3 + i] * B.m[3 + j] + A.m[6 + i] * B.m[6 + j];
  return C;
}
// (2x3) * (3x3) -> 2x3, all row-major.
template <typename T>
__device__ __forceinline__ void m23x33(const T* A, const M3<T>& B, T* C) {
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) C[3 * r + c] = A[3 * r] * B.m[c] + A[3 * r + 1] * B.m[3 + c] + A[3 * r + 2] * B.m[6 + c];
}
// (2x3) * skew(v): row_r x v ... A * [v]x
template <typename T>
__device__ __forceinline__ void m23xskew(const T* A, const T* v, T* C) {
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const T a0 = A[3 * r], a1 = A[3 * r + 1], a2 = A[3 * r + 2];
    // [v]x = [[0,-v2,v1],[v2,0,-v0],[-v1,v0,0]]
    C[3 * r + 0] = a1 * v[2] - a2 * v[1];
    C[3 * r + 1] = -a0 * v[2] + a2 * v[0];
    C[3 * r + 2] = a0 * v[1] - a1 * v[0];
  }
}

// ---------------------------------------------------------------- camera
template <typename S>
struct DevCameraT {
  S intr[4];
  S dist[4];
  int32_t dtype;
  int32_t width, height, pad;
  S q_CI[4];
  S p_CI[3];
  S pad2;
};
using DevCamera = DevCameraT<double>;

template <typename T>
struct Vec2;
template <>
struct Vec2<double> {
  using type = double2;
};
template <>
struct Vec2<float> {
  using type = float2;
};

template <typename T>
__device__ __forceinline__ T dsqrt(T x);
template <>
__device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }
template <>
__device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
template <typename T>
__device__ __forceinline__ T datan(T x);
template <>
__device__ __forceinline__ double datan<double>(double x) { return atan(x); }
template <>
__device__ __forceinline__ float datan<float>(float x) { return atanf(x); }
template <typename T>
__device__ __forceinline__ T dtan(T x);
template <>
__device__ __forceinline__ double dtan<double>(double x) { return tan(x); }
template <>
__device__ __forceinline__ float dtan<float>(float x) { return tanf(x); }
template <typename T>
__device__ __forceinline__ T dpow(T x, T y);
template <>
__device__ __forceinline__ double dpow<double>(double x, double y) { return pow(x, y); }
template <>
__device__ __forceinline__ float dpow<float>(float x, float y) { return powf(x, y); }

// Distortion of the normalized point (in place) and its 2x2 Jacobian.
template <typename T>
__device__ __forceinline__ void distort(int dtype, const T* k, T* pt, T* J) {
  if (dtype == MBA_DISTORTION_RADTAN) {
    // distortion-radtan.cc:14-65
    const T x = pt[0], y = pt[1];
    const T k1 = k[0], k2 = k[1], p1 = k[2], p2 = k[3];
    const T mx2 = x * x, my2 = y * y, mxy = x * y;
    const T rho2 = mx2 + my2;
    const T rad = k1 * rho2 + k2 * rho2 * rho2;
    J[0] = T(1) + rad + T(2) * k1 * mx2 + T(4) * k2 * rho2 * mx2 + T(2) * p1 * y + T(6) * p2 * x;
    J[1] = T(2) * k1 * mxy + T(4) * k2 * rho2 * mxy + T(2) * p1 * x + T(2) * p2 * y;
    J[2] = J[1];
    J[3] = T(1) + rad + T(2) * k1 * my2 + T(4) * k2 * rho2 * my2 + T(2) * p2 * x + T(6) * p1 * y;
    pt[0] = x + x * rad + T(2) * p1 * mxy + p2 * (rho2 + T(2) * mx2);
    pt[1] = y + y * rad + T(2) * p2 * mxy + p1 * (rho2 + T(2) * my2);
  } else if (dtype == MBA_DISTORTION_EQUIDISTANT) {
    // distortion-equidistant.cc:14-107
    const T x = pt[0], y = pt[1];
    const T k1 = k[0], k2 = k[1], k3 = k[2], k4 = k[3];
    const T x2 = x * x, y2 = y * y;
    const T r2 = x2 + y2;
    const T r = dsqrt(r2);
    if (r < T(1e-10)) {
      J[0] = J[1] = J[2] = J[3] = T(0);
      return;
    }
    const T th = datan(r);
    const T th2 = th * th, th4 = th2 * th2, th6 = th2 * th4, th8 = th4 * th4;
    const T th3 = th2 * th, th5 = th4 * th, th7 = th6 * th;
    const T poly = k1 * th2 + k2 * th4 + k3 * th6 + k4 * th8 + T(1);
    const T thetad = th * poly;
    const T r2p1 = r2 + T(1);
    // The reference's generated expression divides each of its eight terms by
    // r^2 + 1 and further terms by r^2 (r^2 + 1) and r^3; here 1 / r and
    // 1 / (r^2 + 1) are formed once and multiplied in (same values up to
    // rounding, two divisions per observation instead of twelve).
    const T ir = T(1) / r, ir2p1 = T(1) / r2p1;
    const T q = (T(4) * k2 * th3 + T(6) * k3 * th5 + T(8) * k4 * th7 + T(2) * k1 * th) * ir * ir2p1;
    const T sx = x * q, sy = y * q;
    const T a = poly * (ir * ir) * ir2p1;     // poly / (r^2 (r^2 + 1))
    const T b = th * (ir * ir * ir) * poly;   // th / r^3 * poly
    J[0] = th * ir * poly + x * th * ir * sx + x2 * a - x2 * b;
    J[1] = x * th * ir * sy + x * y * a - x * y * b;
    J[2] = y * th * ir * sx + x * y * a - x * y * b;
    J[3] = th * ir * poly + y * th * ir * sy + y2 * a - y2 * b;
    const T s = (r > T(1e-8)) ? thetad * ir : T(1);
    pt[0] = x * s;
    pt[1] = y * s;
  } else if (dtype == MBA_DISTORTION_FOV) {
    // FisheyeDistortion (distortion-fisheye.cc:14-80): r_d = atan(2 tan(w/2) r_u) / w.
    const T w = k[0];
    const T u = pt[0], v = pt[1];
    const T uv2 = u * u + v * v;
    const T r_u = dsqrt(uv2);
    const T tanwhalf = dtan(w / T(2));
    const T tanwhalfsq = tanwhalf * tanwhalf;
    const T atan_wrd = datan(T(2) * tanwhalf * r_u);
    T r_rd;
    if (w * w < T(1e-5)) {
      r_rd = T(1);
      J[0] = T(1); J[1] = T(0); J[2] = T(0); J[3] = T(1);
    } else if (r_u * r_u < T(1e-5)) {
      r_rd = T(2) * tanwhalf / w;
      J[0] = r_rd; J[1] = T(0); J[2] = T(0); J[3] = r_rd;
    } else {
      r_rd = atan_wrd / (r_u * w);
      const T r_u_cubed = r_u * r_u * r_u;
      const T den = w * uv2 * (T(4) * tanwhalfsq * uv2 + T(1));
      J[0] = atan_wrd / (w * r_u) - (u * u * atan_wrd) / (w * r_u_cubed) + (T(2) * u * u * tanwhalf) / den;
      J[1] = (T(2) * u * v * tanwhalf) / den - (u * v * atan_wrd) / (w * r_u_cubed);
      J[2] = J[1];
      J[3] = atan_wrd / (w * r_u) - (v * v * atan_wrd) / (w * r_u_cubed) + (T(2) * v * v * tanwhalf) / den;
    }
    pt[0] = u * r_rd;
    pt[1] = v * r_rd;
  } else {
    J[0] = T(1); J[1] = T(0); J[2] = T(0); J[3] = T(1);
  }
}

// Distortion-parameter Jacobian at the undistorted normalized point
// (distortion-radtan.cc:67-91, distortion-equidistant.cc:109-142,
// distortion-fisheye.cc:82-110); k = the model's parameters.
__device__ __forceinline__ void dist_param_jac(int dtype, const double* k, const double* pt, double* J) {
  if (dtype == MBA_DISTORTION_RADTAN) {
    const double y0 = pt[0], y1 = pt[1], r2 = y0 * y0 + y1 * y1, r4 = r2 * r2;
    J[0] = y0 * r2; J[1] = y0 * r4; J[2] = 2.0 * y0 * y1; J[3] = r2 + 2.0 * y0 * y0;
    J[4] = y1 * r2; J[5] = y1 * r4; J[6] = r2 + 2.0 * y1 * y1; J[7] = 2.0 * y0 * y1;
  } else if (dtype == MBA_DISTORTION_EQUIDISTANT) {
    const double x = pt[0], y = pt[1];
    const double r = sqrt(x * x + y * y);
    const double th = atan(r);
    if (r < 1e-10) {
      for (int a = 0; a < 8; ++a) J[a] = 0.0;
      return;
    }
    const double t3 = pow(th, 3.0), t5 = pow(th, 5.0), t7 = pow(th, 7.0), t9 = pow(th, 9.0);
    J[0] = x * t3 / r; J[1] = x * t5 / r; J[2] = x * t7 / r; J[3] = x * t9 / r;
    J[4] = y * t3 / r; J[5] = y * t5 / r; J[6] = y * t7 / r; J[7] = y * t9 / r;
  } else if (dtype == MBA_DISTORTION_FOV) {
    // distortion-fisheye.cc:82-110: d(distorted point) / dw in column 0.
    for (int a = 0; a < 8; ++a) J[a] = 0.0;
    const double w = k[0];
    if (w * w < 1e-5) return;
    const double u = pt[0], v = pt[1];
    const double r_u = sqrt(u * u + v * v);
    const double tanwhalf = tan(w / 2.0), tanwhalfsq = tanwhalf * tanwhalf;
    const double atan_wrd = atan(2.0 * tanwhalf * r_u);
    if (r_u * r_u < 1e-5) {
      J[0] = J[4] = (w - sin(w)) / (w * w * cos(w / 2) * cos(w / 2));
      return;
    }
    J[0] = (2 * u * (tanwhalfsq / 2 + 0.5)) / (w * (4 * tanwhalfsq * r_u * r_u + 1)) - (u * atan_wrd) / (w * w * r_u);
    J[4] = (2 * v * (tanwhalfsq / 2 + 0.5)) / (w * (4 * tanwhalfsq * r_u * r_u + 1)) - (v * atan_wrd) / (w * w * r_u);
  } else {
    for (int a = 0; a < 8; ++a) J[a] = 0.0;
  }
}

// PinholeCamera::project3Functional with point Jacobian; returns true when the
// term fails (visual-error-term-inl.h:159-166): POINT_BEHIND_CAMERA,
// PROJECTION_INVALID (camera-pinhole-inl.h:47-65), depth < 0.05, or
// |kp|^2 > 1e10.  KEYPOINT_OUTSIDE_IMAGE_BOX is not a failure.
template <typename T, typename S>
__device__ __forceinline__ bool project(const DevCameraT<S>& c, const T* p, T* kp, T* Jkp) {
  const T fu = T(c.intr[0]), fv = T(c.intr[1]), cu = T(c.intr[2]), cv = T(c.intr[3]);
  const T x = p[0], y = p[1], z = p[2];
  const T rz = T(1) / z;
  T pt[2] = {x * rz, y * rz};
  T Jd[4];
  T k[4] = {T(c.dist[0]), T(c.dist[1]), T(c.dist[2]), T(c.dist[3])};
  distort<T>(c.dtype, k, pt, Jd);
  if (Jkp) {
    const T rz2 = rz * rz;
    Jkp[0] = fu * Jd[0] * rz;
    Jkp[1] = fu * Jd[1] * rz;
    Jkp[2] = -fu * (x * Jd[0] + y * Jd[1]) * rz2;
    Jkp[3] = fv * Jd[2] * rz;
    Jkp[4] = fv * Jd[3] * rz;
    Jkp[5] = -fv * (x * Jd[2] + y * Jd[3]) * rz2;
  }
  kp[0] = fu * pt[0] + cu;
  kp[1] = fv * pt[1] + cv;
  // evaluateProjectionResult: behind (z < 0 and not z > 1e-10) or invalid
  // (0 <= z <= 1e-10) both fail; those cases are covered by z <= 1e-10.
  const bool bad_depth = !(z > T(1e-10));
  const T n2 = kp[0] * kp[0] + kp[1] * kp[1];
  return bad_depth || z < T(0.05) || n2 > T(1.0e10);
}

// get_dQuaternionJpl_dTheta (quaternion-param-jpl.cc:8-32), 4x3 row-major.
template <typename T>
__device__ __forceinline__ void dqdtheta(const T* q, T* J) {
  J[0] = T(0.5) * q[3];  J[1] = T(-0.5) * q[2]; J[2] = T(0.5) * q[1];
  J[3] = T(0.5) * q[2];  J[4] = T(0.5) * q[3];  J[5] = T(-0.5) * q[0];
  J[6] = T(-0.5) * q[1]; J[7] = T(0.5) * q[0];  J[8] = T(0.5) * q[3];
  J[9] = T(-0.5) * q[0]; J[10] = T(-0.5) * q[1]; J[11] = T(-0.5) * q[2];
}

// Normalize like Eigen (divide by the norm when the squared norm is > 0).
template <typename T>
__device__ __forceinline__ void normalize4(T* q) {
  const T z = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (z > T(0)) {
    const T n = dsqrt(z);
    q[0] /= n; q[1] /= n; q[2] /= n; q[3] /= n;
  }
}

// positiveQuaternionProductJPL (quaternion-math-inl.h:112-154).
__device__ __forceinline__ void qprod_pos(const double* a, const double* b, double* o) {
  double p[4];
  p[0] = a[3] * b[0] + a[2] * b[1] - a[1] * b[2] + a[0] * b[3];
  p[1] = -a[2] * b[0] + a[3] * b[1] + a[0] * b[2] + a[1] * b[3];
  p[2] = a[1] * b[0] - a[0] * b[1] + a[3] * b[2] + a[2] * b[3];
  p[3] = -a[0] * b[0] - a[1] * b[1] - a[2] * b[2] + a[3] * b[3];
  normalize4(p);
  if (p[3] < 0.0) { p[0] = -p[0]; p[1] = -p[1]; p[2] = -p[2]; p[3] = -p[3]; }
  o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; o[3] = p[3];
}

// JplQuaternionParameterization::Plus (quaternion-param-jpl.cc:35-68).
__device__ __forceinline__ void jpl_plus(const double* q, const double* d, double* out) {
  const double sq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  const double thr = (0.262 * 2) * (0.262 * 2);
  double qd[4];
  if (sq < thr) {
    qd[0] = 0.5 * d[0]; qd[1] = 0.5 * d[1]; qd[2] = 0.5 * d[2]; qd[3] = 1.0;
    normalize4(qd);
  } else {
    const double nh = 0.5 * sqrt(sq);
    const double s = sin(nh);
    qd[0] = 0.5 * d[0] / nh * s; qd[1] = 0.5 * d[1] / nh * s; qd[2] = 0.5 * d[2] / nh * s;
    qd[3] = cos(nh);
  }
  qprod_pos(qd, q, out);
}

// JplYawQuaternionParameterization::Plus and ComputeJacobian
// (quaternion-param-jpl.cc:78-105): a rotation about z by the one tangent
// dim, applied on the left; Jacobian 4 x 1.
__device__ __forceinline__ void jpl_yaw_plus(const double* q, const double* d, double* out) {
  const double h = 0.5 * d[0];
  const double qd[4] = {0.0, 0.0, sin(h), cos(fabs(h))};
  qprod_pos(qd, q, out);
}
__device__ __forceinline__ void dqdyaw(const double* q, double* J) {
  J[0] = q[1] * 0.5; J[1] = -q[0] * 0.5; J[2] = q[3] * 0.5; J[3] = -q[2] * 0.5;
}

// JplRollPitchQuaternionParameterization::Plus (quaternion-param-jpl.cc:113-142).
__device__ __forceinline__ void jpl_rollpitch_plus(const double* q_GM, const double* q_IM, const double* d,
                                                   double* out) {
  const double qi[4] = {-q_GM[0], -q_GM[1], -q_GM[2], q_GM[3]};
  M3<double> R_M_G;
  jplR(qi, R_M_G);
  const double Gd[3] = {d[0], d[1], 0.0};
  double Md[3];
  mv3(R_M_G, Gd, Md);
  const double th = sqrt(Md[0] * Md[0] + Md[1] * Md[1] + Md[2] * Md[2]);
  double qm[4];
  if (th < 1e-10) {
    qm[0] = qm[1] = qm[2] = 0.0; qm[3] = 1.0;
  } else {
    const double s = sin(th / 2.0);
    qm[0] = Md[0] / th * s; qm[1] = Md[1] / th * s; qm[2] = Md[2] / th * s; qm[3] = cos(th / 2.0);
  }
  const double qinv[4] = {-q_IM[0], -q_IM[1], -q_IM[2], q_IM[3]};
  double qmi[4];
  qprod_pos(qm, qinv, qmi);
  out[0] = -qmi[0]; out[1] = -qmi[1]; out[2] = -qmi[2]; out[3] = qmi[3];
}

// Huber loss rho(s) with scale a (ceres::HuberLoss) and the Ceres corrector
// factors for a 2-dim residual: r' = rs * r, J' = sq1 * (J - as * r (r^T J)).
template <typename T>
__device__ __forceinline__ void huber_corrector(T a, T s, T* rho0, T* sq1, T* rs, T* as) {
  const T b = a * a;
  T r0, r1, r2;
  if (s > b) {
    const T r = dsqrt(s);
    r0 = T(2) * a * r - b;
    r1 = a / r;
    r2 = -r1 / (T(2) * s);
  } else {
    r0 = s; r1 = T(1); r2 = T(0);
  }
  *rho0 = r0;
  const T sqrt_rho1 = dsqrt(r1);
  if (s == T(0) || r2 <= T(0)) {
    *sq1 = sqrt_rho1; *rs = sqrt_rho1; *as = T(0);
  } else {
    const T D = T(1) + T(2) * s * r2 / r1;
    const T alpha = T(1) - dsqrt(D);
    *sq1 = sqrt_rho1; *rs = sqrt_rho1 / (T(1) - alpha); *as = alpha / s;
  }
}

}  // namespace mba
