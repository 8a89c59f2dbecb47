// Relative 6-DoF pose edges (odometry, wheel odometry):
// SixDoFBlockPoseErrorTermWithExtrinsics
// (algorithms/ceres-error-terms/include/ceres-error-terms/
//  six-dof-block-pose-error-term-with-extrinsics-autodiff-inl.h:6-55).
//
// The reference builds it as an AutoDiffCostFunction over the ambient pose
// blocks; here the ambient Jacobians come from forward-mode dual numbers
// (14 components: q(4) p(3) of both keyframes) and are projected on the
// keyframe tangent by the pose parameterization's Jacobian, as Ceres does.
// Edges are few (at most one per keyframe pair): one thread per edge, FP64.
#include <cuda_runtime.h>

#include "internal.h"

namespace mba {
namespace {

struct D14 {
  double a;
  double d[14];
};

__device__ __forceinline__ D14 cst(double v) {
  D14 r;
  r.a = v;
#pragma unroll
  for (int i = 0; i < 14; ++i) r.d[i] = 0.0;
  return r;
}
__device__ __forceinline__ D14 operator+(const D14& x, const D14& y) {
  D14 r;
  r.a = x.a + y.a;
#pragma unroll
  for (int i = 0; i < 14; ++i) r.d[i] = x.d[i] + y.d[i];
  return r;
}
__device__ __forceinline__ D14 operator-(const D14& x, const D14& y) {
  D14 r;
  r.a = x.a - y.a;
#pragma unroll
  for (int i = 0; i < 14; ++i) r.d[i] = x.d[i] - y.d[i];
  return r;
}
__device__ __forceinline__ D14 operator-(const D14& x) {
  D14 r;
  r.a = -x.a;
#pragma unroll
  for (int i = 0; i < 14; ++i) r.d[i] = -x.d[i];
  return r;
}
__device__ __forceinline__ D14 operator*(const D14& x, const D14& y) {
  D14 r;
  r.a = x.a * y.a;
#pragma unroll
  for (int i = 0; i < 14; ++i) r.d[i] = x.a * y.d[i] + x.d[i] * y.a;
  return r;
}
__device__ __forceinline__ D14 operator*(double s, const D14& x) {
  D14 r;
  r.a = s * x.a;
#pragma unroll
  for (int i = 0; i < 14; ++i) r.d[i] = s * x.d[i];
  return r;
}

// Hamilton quaternions (x y z w) and transformations (q, p): x -> R(q) x + p.
__device__ void hq_mul(const D14* a, const D14* b, D14* o) {
  o[3] = a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2];
  o[0] = a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1];
  o[1] = a[3] * b[1] - a[0] * b[2] + a[1] * b[3] + a[2] * b[0];
  o[2] = a[3] * b[2] + a[0] * b[1] - a[1] * b[0] + a[2] * b[3];
}
__device__ void hq_rot(const D14* q, const D14* v, D14* o) {
  D14 uv[3] = {2.0 * (q[1] * v[2] - q[2] * v[1]), 2.0 * (q[2] * v[0] - q[0] * v[2]), 2.0 * (q[0] * v[1] - q[1] * v[0])};
  o[0] = v[0] + q[3] * uv[0] + (q[1] * uv[2] - q[2] * uv[1]);
  o[1] = v[1] + q[3] * uv[1] + (q[2] * uv[0] - q[0] * uv[2]);
  o[2] = v[2] + q[3] * uv[2] + (q[0] * uv[1] - q[1] * uv[0]);
}
__device__ void ht_mul(const D14* A, const D14* B, D14* O) {
  hq_mul(A, B, O);
  D14 r[3];
  hq_rot(A, B + 4, r);
#pragma unroll
  for (int i = 0; i < 3; ++i) O[4 + i] = r[i] + A[4 + i];
}
__device__ void ht_inv(const D14* A, D14* O) {
  O[0] = -A[0]; O[1] = -A[1]; O[2] = -A[2]; O[3] = A[3];
  D14 r[3];
  hq_rot(O, A + 4, r);
#pragma unroll
  for (int i = 0; i < 3; ++i) O[4 + i] = -r[i];
}

// e_w = e^T M with e = [p_meas - p_est; 2 vec(q_meas^-1 q_est)] (w >= 0) and
// T_est = T_B_I T_Ik^-1 T_Ik+1 T_B_I^-1, keyframe coefficients read as Hamilton.
__device__ void pose_edge_residual(const D14* xk, const D14* xk1, const double* ext, const double* meas,
                                   const double* M, D14* ew) {
  D14 TBI[7] = {cst(-ext[0]), cst(-ext[1]), cst(-ext[2]), cst(ext[3]), cst(ext[4]), cst(ext[5]), cst(ext[6])};
  D14 TkI[7], TBIi[7], X[7], Y[7], Te[7];
  ht_inv(xk, TkI);
  ht_inv(TBI, TBIi);
  ht_mul(TBI, TkI, X);
  ht_mul(X, xk1, Y);
  ht_mul(Y, TBIi, Te);
  const D14 qmi[4] = {cst(-meas[0]), cst(-meas[1]), cst(-meas[2]), cst(meas[3])};
  D14 qe[4];
  hq_mul(qmi, Te, qe);
  if (qe[3].a < 0.0)
#pragma unroll
    for (int i = 0; i < 4; ++i) qe[i] = -qe[i];
  D14 e[6];
#pragma unroll
  for (int i = 0; i < 3; ++i) e[i] = cst(meas[4 + i]) - Te[4 + i];
#pragma unroll
  for (int i = 0; i < 3; ++i) e[3 + i] = 2.0 * qe[i];
  for (int j = 0; j < 6; ++j) {
    D14 acc = cst(0.0);
    for (int i = 0; i < 6; ++i) acc = acc + M[6 * i + j] * e[i];
    ew[j] = acc;
  }
}

// Pose parameterization Jacobian d(q, p) / d(theta, p) [7][6] of keyframe k:
// JplQuaternionParameterization (quaternion-param-jpl.cc:8-32), or the
// roll-pitch gauge form (:144-164), fixed dims zeroed.
__device__ void pose_param(const DevProblem& P, int64_t k, const double* q, double* P76) {
#pragma unroll
  for (int i = 0; i < 42; ++i) P76[i] = 0.0;
  const uint16_t m = P.kf_mask[k];
  double Jq[12];
  dqdtheta(q, Jq);
  if (P.kf_flags[k] & MBA_KF_GAUGE_ROLL_PITCH) {
    M3<double> RIM, RGM;
    jplR(q, RIM);
    jplR(P.mis + 8 * P.kf_mis[k], RGM);
    double A[9];  // R_I_M R_M_G = R_I_M R_G_M^T
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        A[3 * i + j] = RIM.m[3 * i] * RGM.m[3 * j] + RIM.m[3 * i + 1] * RGM.m[3 * j + 1] + RIM.m[3 * i + 2] * RGM.m[3 * j + 2];
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 2; ++c)
        P76[6 * r + c] = -(Jq[3 * r] * A[c] + Jq[3 * r + 1] * A[3 + c] + Jq[3 * r + 2] * A[6 + c]);
  } else {
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 3; ++c) P76[6 * r + c] = ((m >> c) & 1) ? Jq[3 * r + c] : 0.0;
  }
  for (int i = 0; i < 3; ++i) P76[6 * (4 + i) + 3 + i] = ((m >> (3 + i)) & 1) ? 1.0 : 0.0;
}

// One thread per pose edge e = nimu + j: residual (rows 0-5 of the 15-row edge
// residual), tangent Jacobians in the (theta, p) columns of the 15x15 edge
// blocks (if lin.r), cost 0.5 |e_w|^2.
__global__ void __launch_bounds__(128) k_pose_edges(DevProblem P, const double* kf_state, InertialLin<double> lin,
                                                    double* cost_accum, const int* skip_if) {
  if (skip_if && *skip_if) return;
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t npe = P.nedge - P.nimu;
  double c = 0.0;
  if (j < npe) {
    const int64_t e = P.nimu + j, f = P.e_from[e], t = P.e_to[e];
    const double* xf = kf_state + 16 * f;
    const double* xt = kf_state + 16 * t;
    D14 a[7], b[7], ew[6];
    for (int i = 0; i < 7; ++i) {
      a[i] = cst(xf[i]);
      a[i].d[i] = 1.0;
      b[i] = cst(xt[i]);
      b[i].d[7 + i] = 1.0;
    }
    pose_edge_residual(a, b, P.pe_ext + 7 * j, P.pe_meas + 7 * j, P.pe_sqrt + 36 * j, ew);
    for (int r = 0; r < 6; ++r) c += 0.5 * ew[r].a * ew[r].a;
    if (lin.r) {
      double Pf[42], Pt[42];
      pose_param(P, f, xf, Pf);
      pose_param(P, t, xt, Pt);
      double* Rr = lin.r + 15 * e;
      double* Jf = lin.Jf + 225 * e;
      double* Jt = lin.Jt + 225 * e;
      for (int r = 0; r < 15; ++r) Rr[r] = r < 6 ? ew[r].a : 0.0;
      for (int q = 0; q < 225; ++q) { Jf[q] = 0.0; Jt[q] = 0.0; }
      for (int r = 0; r < 6; ++r)
        for (int col = 0; col < 6; ++col) {
          double sf = 0.0, st = 0.0;
          for (int mm = 0; mm < 7; ++mm) {
            sf += ew[r].d[mm] * Pf[6 * mm + col];
            st += ew[r].d[7 + mm] * Pt[6 * mm + col];
          }
          Jf[15 * r + col] = sf;
          Jt[15 * r + col] = st;
        }
    }
  }
  // block sum of the cost
  __shared__ double red[4];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0 && cost_accum) {
    const double s = red[0] + red[1] + red[2] + red[3];
    if (s != 0.0) atomicAdd(cost_accum, s);
  }
}

}  // namespace

cudaError_t launch_pose_edges(const DevProblem& P, const double* kf_state, InertialLin<double> lin,
                              double* cost_accum, const int* skip_if, cudaStream_t s) {
  const int64_t npe = P.nedge - P.nimu;
  if (npe <= 0) return cudaSuccess;
  k_pose_edges<<<(unsigned)((npe + 127) / 128), 128, 0, s>>>(P, kf_state, lin, cost_accum, skip_if);
  return cudaGetLastError();
}

}  // namespace mba
