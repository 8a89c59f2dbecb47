// Pose-graph terms ("pose edges"), in the reference's
// algorithms/ceres-error-terms/include/ceres-error-terms/:
//  - relative odometry: SixDoFBlockPoseErrorTermWithExtrinsics
//    (six-dof-block-pose-error-term-with-extrinsics-autodiff-inl.h:6-55);
//  - loop closure: LoopClosureEdgeErrorTerm (loop-closure-edge-error-term-inl.h:
//    6-95) times a switch variable, whose SwitchPriorErrorTerm
//    (switch-prior-error-term-inl.h) adds ((1 - s) / sigma)^2 / 2;
//  - absolute 6-DoF: BlockPosePriorErrorTermV2 (block-pose-prior-error-term-v2-
//    inl.h:8-60).
//
// The reference builds them as AutoDiffCostFunctions over the ambient pose
// blocks; here the ambient Jacobians come from forward-mode dual numbers
// (14 components: q(4) p(3) of both keyframes) and are projected on the
// keyframe tangent by the pose parameterization's Jacobian, as Ceres does.
// Edges are few (loop closures and measurements, not observations): one
// thread per edge, FP64.
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
__device__ __forceinline__ D14 operator/(const D14& x, const D14& y) {
  const double inv = 1.0 / y.a, q = x.a * inv;
  D14 r;
  r.a = q;
#pragma unroll
  for (int i = 0; i < 14; ++i) r.d[i] = (x.d[i] - q * y.d[i]) * inv;
  return r;
}
__device__ __forceinline__ D14 dsqrt14(const D14& x) {
  const double v = sqrt(x.a), h = 0.5 / v;
  D14 r;
  r.a = v;
#pragma unroll
  for (int i = 0; i < 14; ++i) r.d[i] = x.d[i] * h;
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

__device__ void whiten(const D14* e, const double* M, D14* ew) {
  for (int j = 0; j < 6; ++j) {
    D14 acc = cst(0.0);
    for (int i = 0; i < 6; ++i) acc = acc + M[6 * i + j] * e[i];
    ew[j] = acc;
  }
}

// JPL algebra (quaternion-math-inl.h): toRotationMatrixJPL (:6-27), the
// normalized positive product positiveQuaternionProductJPL (:112-154).
__device__ void jpl_rot(const D14* q, D14* R) {
  R[0] = cst(1.0) - 2.0 * (q[1] * q[1] + q[2] * q[2]);
  R[1] = 2.0 * (q[0] * q[1] + q[2] * q[3]);
  R[2] = 2.0 * (q[0] * q[2] - q[1] * q[3]);
  R[3] = 2.0 * (q[0] * q[1] - q[2] * q[3]);
  R[4] = cst(1.0) - 2.0 * (q[0] * q[0] + q[2] * q[2]);
  R[5] = 2.0 * (q[1] * q[2] + q[0] * q[3]);
  R[6] = 2.0 * (q[0] * q[2] + q[1] * q[3]);
  R[7] = 2.0 * (q[1] * q[2] - q[0] * q[3]);
  R[8] = cst(1.0) - 2.0 * (q[0] * q[0] + q[1] * q[1]);
}
__device__ void jpl_inv(const D14* q, D14* o) { o[0] = -q[0]; o[1] = -q[1]; o[2] = -q[2]; o[3] = q[3]; }
__device__ void jpl_prod_pos(const D14* a, const D14* b, D14* o) {
  D14 p[4];
  p[0] = a[3] * b[0] + a[2] * b[1] - a[1] * b[2] + a[0] * b[3];
  p[1] = -(a[2] * b[0]) + a[3] * b[1] + a[0] * b[2] + a[1] * b[3];
  p[2] = a[1] * b[0] - a[0] * b[1] + a[3] * b[2] + a[2] * b[3];
  p[3] = -(a[0] * b[0]) - a[1] * b[1] - a[2] * b[2] + a[3] * b[3];
  const D14 z = p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3];
  if (z.a > 0.0) {
    const D14 n = dsqrt14(z);
    for (int i = 0; i < 4; ++i) p[i] = p[i] / n;
  }
  const bool flip = p[3].a < 0.0;
  for (int i = 0; i < 4; ++i) o[i] = flip ? -p[i] : p[i];
}
__device__ void mat_vec3(const D14* A, const D14* v, D14* o) {
  for (int i = 0; i < 3; ++i) o[i] = A[3 * i] * v[0] + A[3 * i + 1] * v[1] + A[3 * i + 2] * v[2];
}
__device__ void mat_mul3(const D14* A, const D14* B, D14* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}
__device__ void transpose3(const D14* A, D14* B) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) B[3 * j + i] = A[3 * i + j];
}
// Rotation matrix (row-major) to Hamilton quaternion (x y z w): the trace /
// largest-diagonal method (Shoemake 1985), in the form of Eigen's
// Quaternion(const Matrix3&) constructor.
__device__ void rot_to_hamilton(const D14* m, D14* q) {
  const D14 tr = m[0] + m[4] + m[8];
  if (tr.a > 0.0) {
    D14 t = dsqrt14(tr + cst(1.0));
    q[3] = 0.5 * t;
    t = cst(0.5) / t;
    q[0] = (m[7] - m[5]) * t;
    q[1] = (m[2] - m[6]) * t;
    q[2] = (m[3] - m[1]) * t;
  } else {
    int i = 0;
    if (m[4].a > m[0].a) i = 1;
    if (m[8].a > m[4 * i].a) i = 2;
    const int j = (i + 1) % 3, k = (j + 1) % 3;
    D14 t = dsqrt14(m[4 * i] - m[4 * j] - m[4 * k] + cst(1.0));
    q[i] = 0.5 * t;
    t = cst(0.5) / t;
    q[3] = (m[3 * k + j] - m[3 * j + k]) * t;
    q[j] = (m[3 * j + i] + m[3 * i + j]) * t;
    q[k] = (m[3 * k + i] + m[3 * i + k]) * t;
  }
}

// LoopClosureEdgeErrorTerm without the switch: baseframes bfA, bfB (JPL
// q_G_M | p_G_M; identity within one mission), vertex blocks q_I_M | p_M_I,
// measurement q_AB (JPL) | p_AB.
__device__ void loop_closure_residual(const double* bfA, const double* bfB, const D14* xA, const D14* xB,
                                      const double* meas, const double* M, D14* ew) {
  D14 qGMA[4], qGMB[4], R[9], pA[3], pB[3], pGIA[3], pGIB[3];
  for (int i = 0; i < 4; ++i) { qGMA[i] = cst(bfA[i]); qGMB[i] = cst(bfB[i]); }
  jpl_rot(qGMA, R);
  mat_vec3(R, xA + 4, pA);
  jpl_rot(qGMB, R);
  mat_vec3(R, xB + 4, pB);
  for (int i = 0; i < 3; ++i) { pGIA[i] = cst(bfA[4 + i]) + pA[i]; pGIB[i] = cst(bfB[4 + i]) + pB[i]; }
  D14 qi[4], qGIA[4], qGIB[4], qAB[4], qerr[4];
  jpl_inv(xA, qi);
  jpl_prod_pos(qGMA, qi, qGIA);
  jpl_inv(xB, qi);
  jpl_prod_pos(qGMB, qi, qGIB);
  jpl_inv(qGIA, qi);
  jpl_prod_pos(qi, qGIB, qAB);
  const D14 qlci[4] = {cst(-meas[0]), cst(-meas[1]), cst(-meas[2]), cst(meas[3])};
  jpl_prod_pos(qlci, qAB, qerr);
  D14 d[3], e[6];
  jpl_rot(qi, R);  // R_IA_G
  for (int i = 0; i < 3; ++i) d[i] = pGIB[i] - pGIA[i];
  mat_vec3(R, d, e);
  for (int i = 0; i < 3; ++i) e[i] = e[i] - cst(meas[4 + i]);
  for (int i = 0; i < 3; ++i) e[3 + i] = 2.0 * qerr[i];
  whiten(e, M, ew);
}

// BlockPosePriorErrorTermV2: baseframe q_G_M | p_G_M and sensor extrinsics
// q_S_B | p_S_B (JPL constants), vertex block q_B_M | p_M_B, measurement
// q_S_G (Hamilton) | p_G_S.
__device__ void absolute_pose_residual(const double* bf, const D14* x, const double* ext, const double* meas,
                                       const double* M, D14* ew) {
  D14 q[4], RGM[9], RBM[9], RMB[9], RSB[9], RBS[9], A[9], RGS[9];
  for (int i = 0; i < 4; ++i) q[i] = cst(bf[i]);
  jpl_rot(q, RGM);
  jpl_rot(x, RBM);
  transpose3(RBM, RMB);
  for (int i = 0; i < 4; ++i) q[i] = cst(ext[i]);
  jpl_rot(q, RSB);
  transpose3(RSB, RBS);
  mat_mul3(RGM, RMB, A);
  mat_mul3(A, RBS, RGS);
  const D14 pSB[3] = {cst(ext[4]), cst(ext[5]), cst(ext[6])};
  D14 pBS[3], a[3], b[3], e[6];
  mat_vec3(RBS, pSB, pBS);
  for (int i = 0; i < 3; ++i) pBS[i] = -pBS[i];
  mat_vec3(A, pBS, a);
  mat_vec3(RGM, x + 4, b);
  for (int i = 0; i < 3; ++i) e[i] = a[i] + b[i] + cst(bf[4 + i]) - cst(meas[4 + i]);
  D14 qGS[4], qd[4];
  rot_to_hamilton(RGS, qGS);
  const D14 qSG[4] = {cst(meas[0]), cst(meas[1]), cst(meas[2]), cst(meas[3])};
  hq_mul(qGS, qSG, qd);
  for (int i = 0; i < 3; ++i) e[3 + i] = 2.0 * qd[i];
  whiten(e, M, ew);
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
  whiten(e, M, ew);
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

// One thread per pose edge e = nimu + j: residual s e_w (rows 0-5 of the
// 15-row edge residual), tangent Jacobians in the (theta, p) columns of the
// 15x15 edge blocks and d r / d s = e_w (if lin.r), cost 0.5 |s e_w|^2 plus
// the switch prior's 0.5 ((1 - s) w)^2.
__global__ void __launch_bounds__(128) k_pose_edges(DevProblem P, const double* kf_state, const double* sw_state,
                                                    InertialLin<double> lin, double* cost_accum, const int* skip_if) {
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
    const int type = P.pe_type[j];
    const double* M = P.pe_sqrt + 36 * j;
    if (type == MBA_POSE_EDGE_LOOP_CLOSURE) {
      const double kIdentity[7] = {0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0};
      const bool same = P.kf_mis[f] == P.kf_mis[t];
      loop_closure_residual(same ? kIdentity : P.mis + 8 * P.kf_mis[f], same ? kIdentity : P.mis + 8 * P.kf_mis[t],
                            a, b, P.pe_meas + 7 * j, M, ew);
    } else if (type == MBA_POSE_EDGE_ABSOLUTE) {
      absolute_pose_residual(P.mis + 8 * P.kf_mis[f], a, P.pe_ext + 7 * j, P.pe_meas + 7 * j, M, ew);
    } else {
      pose_edge_residual(a, b, P.pe_ext + 7 * j, P.pe_meas + 7 * j, M, ew);
    }
    const int q = P.pe_swi[j];
    const double sw = q >= 0 ? sw_state[q] : P.pe_swc[j];
    for (int r = 0; r < 6; ++r) c += 0.5 * (sw * ew[r].a) * (sw * ew[r].a);
    if (q >= 0) {
      const double rp = (1.0 - sw) * P.sw_w[q];
      c += 0.5 * rp * rp;
    }
    if (lin.r) {
      double Pf[42], Pt[42];
      pose_param(P, f, xf, Pf);
      pose_param(P, t, xt, Pt);
      double* Rr = lin.r + 15 * e;
      double* Jf = lin.Jf + 225 * e;
      double* Jt = lin.Jt + 225 * e;
      for (int r = 0; r < 15; ++r) Rr[r] = r < 6 ? sw * ew[r].a : 0.0;
      if (lin.Js)
        for (int r = 0; r < 6; ++r) lin.Js[6 * j + r] = ew[r].a;
      for (int k = 0; k < 225; ++k) { Jf[k] = 0.0; Jt[k] = 0.0; }
      const bool unary = type == MBA_POSE_EDGE_ABSOLUTE;  // no to-vertex block
      for (int r = 0; r < 6; ++r)
        for (int col = 0; col < 6; ++col) {
          double sf = 0.0, st = 0.0;
          for (int mm = 0; mm < 7; ++mm) {
            sf += (sw * ew[r].d[mm]) * Pf[6 * mm + col];
            st += (sw * ew[r].d[7 + mm]) * Pt[6 * mm + col];
          }
          Jf[15 * r + col] = sf;
          Jt[15 * r + col] = unary ? 0.0 : st;
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

cudaError_t launch_pose_edges(const DevProblem& P, const double* kf_state, const double* sw_state,
                              InertialLin<double> lin, double* cost_accum, const int* skip_if, cudaStream_t s) {
  const int64_t npe = P.nedge - P.nimu;
  if (npe <= 0) return cudaSuccess;
  k_pose_edges<<<(unsigned)((npe + 127) / 128), 128, 0, s>>>(P, kf_state, sw_state ? sw_state : P.sw, lin,
                                                               cost_accum, skip_if);
  return cudaGetLastError();
}

}  // namespace mba
