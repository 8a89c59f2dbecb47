// Inertial error terms: RK4 preintegration of the IMU samples of every edge,
// the 15x15 transition Phi_acc and covariance Q_acc, and the whitened residual
// and Jacobians.
//
// Restates InertialErrorTerm::IntegrateStateAndCovariance / Evaluate
// (algorithms/ceres-error-terms/src/inertial-error-term.cc:9-286) and
// ImuIntegratorRK4::integrate / getStateDerivativeRungeKutta /
// getCovarianceTransitionDerivativesRungeKutta / interpolateImuReadings
// (algorithms/imu-integrator-rk4/include/imu-integrator/imu-integrator-inl.h:17-319).
//
// Work split (GB300's FP64 pipe is narrow, so FP64 instructions are spent
// only where they are needed):
//   k_inertial_state  one thread per edge, FP64: integrates the 16-dim state
//                     through all samples and records, for every RK4 stage,
//                     the gyro rate, the specific force and G_R_B.
//   k_inertial_mat<TM> one warp per edge: per step, Phi = I + A and Q from
//                     the stage quantities (the transition derivative is only
//                     non-zero in rows 0-2, 6-8, 12-14), then the chain
//                     Q_acc <- Q_acc + A Q_acc + (A Q_acc)^T + A Q_acc A^T + Q,
//                     Phi_acc <- Phi_acc + A Phi_acc, elementwise over the warp
//                     from shared memory (FP64 path); Cholesky, whitening,
//                     residual and Jacobians in FP64 (inertial_tail).
//   k_inertial_mat_cols the same chain in FP32 (mixed path) with one half-warp
//                     per edge and one column per lane, in registers;
//   k_inertial_whiten  its FP64 part (inertial_tail), one warp per edge.
#include <cuda_runtime.h>

#include "internal.h"

namespace mba {

namespace {

constexpr int kStageVals = 15;  // omega(3), a(3), G_R_B(9)

__device__ __forceinline__ bool gated_i(const int* skip_if) { return skip_if && *skip_if; }

// Rotation-tangent basis of keyframe k (same rule as the visual kernels):
// |q|^2 I for JplQuaternionParameterization, -|q|^2 (R_I_M R_M_G)[:, 0:2] for
// the roll/pitch gauge parameterization; masked dims are zero columns.
__device__ __forceinline__ void rot_basis_d(const DevProblem& P, int k, const double* q, const M3<double>& R_I_M,
                                            M3<double>& B) {
  const uint16_t m = P.kf_mask[k];
  const double n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
#pragma unroll
  for (int i = 0; i < 9; ++i) B.m[i] = 0.0;
  if (P.kf_flags[k] & MBA_KF_GAUGE_ROLL_PITCH) {
    M3<double> R_G_M;
    jplR(P.mis + 8 * P.kf_mis[k], R_G_M);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 2; ++j) {
        const double a = R_I_M.m[3 * i] * R_G_M.m[3 * j] + R_I_M.m[3 * i + 1] * R_G_M.m[3 * j + 1] +
                         R_I_M.m[3 * i + 2] * R_G_M.m[3 * j + 2];
        B.m[3 * i + j] = ((m >> j) & 1) ? -n2 * a : 0.0;
      }
  } else {
    B.m[0] = (m & 1) ? n2 : 0.0;
    B.m[4] = (m & 2) ? n2 : 0.0;
    B.m[8] = (m & 4) ? n2 : 0.0;
  }
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// getStateDerivativeRungeKutta (imu-integrator-inl.h:170-207) that also
// returns the normalized B_R_G of the stage state.
__device__ __forceinline__ void state_derivative(double g, const double* rd, const double* s, double* d,
                                                 M3<double>& BRG) {
  double q[4] = {s[0], s[1], s[2], s[3]};
  normalize4(q);
  jplR(q, BRG);
  const double* w = rd + 3;
#pragma unroll
  for (int a = 0; a < 16; ++a) d[a] = 0.0;
  d[0] = 0.5 * (w[2] * q[1] - w[1] * q[2] + w[0] * q[3]);
  d[1] = 0.5 * (-w[2] * q[0] + w[0] * q[2] + w[1] * q[3]);
  d[2] = 0.5 * (w[1] * q[0] - w[0] * q[1] + w[2] * q[3]);
  d[3] = 0.5 * (-w[0] * q[0] - w[1] * q[1] - w[2] * q[2]);
  double a[3];
  mtv3(BRG, rd, a);  // G_R_B * acc
  d[7] = a[0]; d[8] = a[1]; d[9] = a[2] - g;
  d[13] = s[7]; d[14] = s[8]; d[15] = s[9];
}

// One thread per edge: state RK4 (FP64) and the per-stage inputs of the
// covariance / transition derivatives.
template <typename TM>
__global__ void __launch_bounds__(128) k_inertial_state(DevProblem P, const double* kf_state, TM* stage_out,
                                                        double* dt_out, double* end_out, int* status,
                                                        const int* skip_if) {
  if (gated_i(skip_if)) return;
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= P.nimu) return;
  const double* xf = kf_state + 16 * (int64_t)P.e_from[e];
  // integrator layout: q(4) b_g(3) v(3) b_a(3) p(3)
  double s0[16];
  for (int a = 0; a < 4; ++a) s0[a] = xf[a];
  for (int a = 0; a < 3; ++a) {
    s0[4 + a] = xf[10 + a];
    s0[7 + a] = xf[7 + a];
    s0[10 + a] = xf[13 + a];
    s0[13 + a] = xf[4 + a];
  }
  const int64_t o0 = P.e_off[e];
  const int ns = (int)(P.e_off[e + 1] - o0);
  const int64_t step0 = o0 - e;  // global index of this edge's first step
  bool unordered = false;
  for (int k = 0; k + 1 < ns; ++k) {
    const int64_t a0 = o0 + k;
    if (P.imu_ts[a0 + 1] < P.imu_ts[a0]) unordered = true;
    const double dt = (double)(P.imu_ts[a0 + 1] - P.imu_ts[a0]) * 1e-9;
    double rd[12];
    for (int a = 0; a < 3; ++a) {
      rd[a] = P.imu[6 * a0 + a] - s0[10 + a];
      rd[3 + a] = P.imu[6 * a0 + 3 + a] - s0[4 + a];
      rd[6 + a] = P.imu[6 * (a0 + 1) + a] - s0[10 + a];
      rd[9 + a] = P.imu[6 * (a0 + 1) + 3 + a] - s0[4 + a];
    }
    double r23[6];
    if (dt < 2.220446049250313e-16) {
      for (int a = 0; a < 6; ++a) r23[a] = rd[a];
    } else {
      for (int a = 0; a < 6; ++a) r23[a] = rd[a] + (rd[6 + a] - rd[a]) * ((0.5 * dt) / dt);
    }
    const double* rk[4] = {rd, r23, r23, rd + 6};
    const double cst[3] = {0.5, 0.5, 1.0};
    double si[16], d[16], sum[16];
    for (int a = 0; a < 16; ++a) { si[a] = s0[a]; sum[a] = 0.0; }
    TM* so = stage_out + (step0 + k) * 4 * kStageVals;
    for (int stg = 0; stg < 4; ++stg) {
      M3<double> BRG;
      state_derivative(P.gravity, rk[stg], si, d, BRG);
      TM* o = so + stg * kStageVals;
      for (int a = 0; a < 3; ++a) { o[a] = TM(rk[stg][3 + a]); o[3 + a] = TM(rk[stg][a]); }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) o[6 + 3 * i + j] = TM(BRG.m[3 * j + i]);  // G_R_B
      const double wgt = (stg == 0 || stg == 3) ? 1.0 : 2.0;
      for (int a = 0; a < 16; ++a) {
        sum[a] += wgt * d[a];
        if (stg < 3) si[a] = s0[a] + cst[stg] * dt * d[a];
      }
    }
    for (int a = 0; a < 16; ++a) s0[a] = s0[a] + dt * sum[a] / 6.0;
    dt_out[step0 + k] = dt;
  }
  double* eo = end_out + 16 * e;
  for (int a = 0; a < 16; ++a) eo[a] = s0[a];
  if (unordered && status) atomicMax(status, (int)MBA_ERR_UNORDERED_IMU);
}

template <typename TM>
struct MatSmem {
  TM Q[225], Phi[225], D[225], Pm[225], td[225], PC[225], sumtd[225], sumcd[225];
};

struct InertialOutputs {
  double* lin_r;   // [nedge][15] or null
  double* lin_Jf;  // [nedge][225]
  double* lin_Jt;
  double* amb_res;
  double* amb_J[8];
  double* cost;
  int* status;
};

__device__ __forceinline__ bool active_row(int r) { return r < 3 || (r >= 6 && r < 9) || r >= 12; }

// FP64 part of an edge (one full warp): Cholesky of Q_acc, L^-1, residual and
// Jacobians from the accumulated Q_acc and Phi_acc (row-major 15x15 in shared
// memory).  L, X (225 each) and rs (16) are the warp's FP64 scratch.
template <typename TM>
__device__ void inertial_tail(const DevProblem& P, const double* kf_state, const double* end_in,
                              const InertialOutputs& out, int64_t e, const TM* Qa, const TM* Phia, double* L,
                              double* X, double* rs, int lane) {
  // Right-looking Cholesky spread over the warp (Eigen's LLT is a textbook
  // Cholesky; the order of the subtractions differs, the factor agrees to
  // rounding).  Lane `lane` owns the lower-triangle elements t = lane + 32 s
  // (s < 4, t < 120, row-major); each column's pivot square root and
  // reciprocal are computed by every lane from a broadcast read, and the
  // reciprocals replace the divisions of the triangular inverse.
  double* dinv = rs;  // 1 / L_jj until the residual needs rs
  int own_i[4], own_k[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int t = lane + 32 * s;
    int r = 0;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;  // t in row r of the lower triangle
    own_i[s] = t < 120 ? r : -1;
    own_k[s] = t < 120 ? t - r * (r + 1) / 2 : -1;
  }
  for (int a = lane; a < 225; a += 32) L[a] = (double)Qa[a];
  __syncwarp();
  int fail = -1;
  for (int j = 0; j < 15; ++j) {
    const double d = L[j * 16];
    if (!(d > 0.0)) {  // the same value in every lane: a uniform exit
      fail = j;
      break;
    }
    const double ljj = sqrt(d), inv = 1.0 / ljj;
    // Phase 1: scale column j below the pivot (every lane has read the pivot
    // before any lane writes column j).
#pragma unroll
    for (int s = 0; s < 4; ++s)
      if (own_k[s] == j && own_i[s] > j) L[own_i[s] * 15 + j] *= inv;
    if (lane == 0) dinv[j] = inv;
    __syncwarp();
    // Phase 2: the pivot, and the trailing update from the scaled column
    // (which no lane writes in this phase).
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      if (own_k[s] == j && own_i[s] == j) L[j * 16] = ljj;
      if (own_k[s] > j) L[own_i[s] * 15 + own_k[s]] -= L[own_i[s] * 15 + j] * L[own_k[s] * 15 + j];
    }
    __syncwarp();
  }
  if (fail >= 0) {
    // Q_acc not positive definite.  The reference factorizes with Eigen's
    // LLT and never checks info() (inertial-error-term.cc:155-182): Eigen's
    // column-by-column factorization stops at column `fail`, leaving that
    // column (diagonal included) and every later column of the lower
    // triangle at Q's own values, and the triangular solves use that matrix.
    // Columns >= fail are restored from Q here (the right-looking updates
    // above had already touched them).
#pragma unroll
    for (int s = 0; s < 4; ++s)
      if (own_k[s] >= fail) L[own_i[s] * 15 + own_k[s]] = (double)Qa[own_i[s] * 15 + own_k[s]];
    __syncwarp();
    if (lane >= fail && lane < 15) dinv[lane] = 1.0 / L[lane * 16];
    __syncwarp();
  }
  if (lane < 15) {  // X = L^-1, column `lane`
    for (int i = 0; i < 15; ++i) {
      double v = (i == lane) ? 1.0 : 0.0;
      for (int q = 0; q < i; ++q) v -= L[i * 15 + q] * X[q * 15 + lane];
      X[i * 15 + lane] = v * dinv[i];
    }
  }
  __syncwarp();
  // Mx = L^-1 Phi_acc (into L, no longer needed after the next sync)
  double mvals[8];
  for (int j = 0, a = lane; a < 225; a += 32, ++j) {
    const int r = a / 15, c = a % 15;
    double v = 0.0;
    for (int q = 0; q <= r; ++q) v += X[r * 15 + q] * (double)Phia[q * 15 + c];
    mvals[j] = v;
  }
  __syncwarp();
  for (int j = 0, a = lane; a < 225; a += 32, ++j) L[a] = mvals[j];
  const double* xf = kf_state + 16 * (int64_t)P.e_from[e];
  const double* xt = kf_state + 16 * (int64_t)P.e_to[e];
  const double* en = end_in + 16 * e;  // integrator layout
  if (lane == 0) {
    const double n2 = en[0] * en[0] + en[1] * en[1] + en[2] * en[2] + en[3] * en[3];
    double qinv[4] = {0, 0, 0, 0};
    if (n2 > 0.0) { qinv[0] = -en[0] / n2; qinv[1] = -en[1] / n2; qinv[2] = -en[2] / n2; qinv[3] = en[3] / n2; }
    double dq[4];
    qprod_pos(xt, qinv, dq);
    double* rr = rs;
    rr[0] = 2.0 * dq[0]; rr[1] = 2.0 * dq[1]; rr[2] = 2.0 * dq[2];
    for (int a = 0; a < 3; ++a) {
      rr[3 + a] = xt[10 + a] - en[4 + a];
      rr[6 + a] = xt[7 + a] - en[7 + a];
      rr[9 + a] = xt[13 + a] - en[10 + a];
      rr[12 + a] = xt[4 + a] - en[13 + a];
    }
  }
  __syncwarp();
  double rw = 0.0;
  if (lane < 15)
    for (int q = 0; q <= lane; ++q) rw += X[lane * 15 + q] * rs[q];
  __syncwarp();
  if (lane < 15) rs[lane] = rw;
  const double sq = warp_sum_d(lane < 15 ? rw * rw : 0.0);
  if (lane == 0 && out.cost) atomicAdd(out.cost, 0.5 * sq);
  __syncwarp();
  const double* Mx = L;
  const int f = P.e_from[e], t = P.e_to[e];
  if (out.lin_r) {
    if (lane < 15) out.lin_r[15 * e + lane] = rs[lane];
    double qf[4] = {xf[0], xf[1], xf[2], xf[3]}, qt[4] = {xt[0], xt[1], xt[2], xt[3]};
    M3<double> Rf, Rt, Bf, Bt;
    jplR(qf, Rf);
    jplR(qt, Rt);
    rot_basis_d(P, f, qf, Rf, Bf);
    rot_basis_d(P, t, qt, Rt, Bt);
    const uint16_t mf = P.kf_mask[f], mt = P.kf_mask[t];
    const int src[15] = {0, 1, 2, 12, 13, 14, 6, 7, 8, 3, 4, 5, 9, 10, 11};
    for (int a = lane; a < 225; a += 32) {
      const int r = a / 15, c = a % 15;
      double vf, vt;
      if (c < 3) {
        vf = -(Mx[r * 15 + 0] * Bf.m[c] + Mx[r * 15 + 1] * Bf.m[3 + c] + Mx[r * 15 + 2] * Bf.m[6 + c]);
        vt = X[r * 15 + 0] * Bt.m[c] + X[r * 15 + 1] * Bt.m[3 + c] + X[r * 15 + 2] * Bt.m[6 + c];
      } else {
        vf = (mf & (1u << c)) ? -Mx[r * 15 + src[c]] : 0.0;
        vt = (mt & (1u << c)) ? X[r * 15 + src[c]] : 0.0;
      }
      out.lin_Jf[225 * e + a] = vf;
      out.lin_Jt[225 * e + a] = vt;
    }
  }
  if (out.amb_res && lane < 15) out.amb_res[15 * e + lane] = rs[lane];
  if (out.amb_J[0] || out.amb_J[4]) {
    double Jqf[12], Jqt[12];
    dqdtheta(xf, Jqf);
    dqdtheta(xt, Jqt);
    for (int a = lane; a < 105; a += 32) {
      const int r = a / 7, c = a % 7;
      if (out.amb_J[0]) {
        double v;
        if (c < 4) v = -4.0 * (Mx[r * 15] * Jqf[3 * c] + Mx[r * 15 + 1] * Jqf[3 * c + 1] + Mx[r * 15 + 2] * Jqf[3 * c + 2]);
        else v = -Mx[r * 15 + 12 + (c - 4)];
        out.amb_J[0][105 * e + a] = v;
      }
      if (out.amb_J[4]) {
        double v;
        if (c < 4) v = 4.0 * (X[r * 15] * Jqt[3 * c] + X[r * 15 + 1] * Jqt[3 * c + 1] + X[r * 15 + 2] * Jqt[3 * c + 2]);
        else v = X[r * 15 + 12 + (c - 4)];
        out.amb_J[4][105 * e + a] = v;
      }
    }
  }
  for (int b = 0; b < 3; ++b) {
    const int col0 = (b == 0) ? 3 : (b == 1 ? 6 : 9);  // b_g, v, b_a
    for (int a = lane; a < 45; a += 32) {
      const int r = a / 3, c = a % 3;
      if (out.amb_J[1 + b]) out.amb_J[1 + b][45 * e + a] = -Mx[r * 15 + col0 + c];
      if (out.amb_J[5 + b]) out.amb_J[5 + b][45 * e + a] = X[r * 15 + col0 + c];
    }
  }
}

template <typename TM, int kWarps>
__global__ void __launch_bounds__(32 * kWarps) k_inertial_mat(DevProblem P, const double* kf_state,
                                                              const TM* stage_in, const double* dt_in,
                                                              const double* end_in, InertialOutputs out,
                                                              const int* skip_if) {
  if (gated_i(skip_if)) return;
  __shared__ MatSmem<TM> smem[kWarps];
  __shared__ double Ld[kWarps][225], Xd[kWarps][225], rsh[kWarps][16];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t e = blockIdx.x * (int64_t)kWarps + w;
  if (e >= P.nimu) return;
  MatSmem<TM>& S = smem[w];
  const TM gn = TM(P.gyro_noise2), gb = TM(P.gyro_bias2), an = TM(P.acc_noise2), ab = TM(P.acc_bias2);
  for (int a = lane; a < 225; a += 32) {
    S.Q[a] = TM(0);
    S.Phi[a] = (a % 16 == 0) ? TM(1) : TM(0);
    S.td[a] = TM(0);  // rows 3-5 and 9-11 of td / PC stay zero for the whole edge
    S.PC[a] = TM(0);
  }
  __syncwarp();
  const int64_t o0 = P.e_off[e];
  const int ns = (int)(P.e_off[e + 1] - o0);
  const int64_t step0 = o0 - e;
  for (int k = 0; k + 1 < ns; ++k) {
    const TM dt = TM(dt_in[step0 + k]);
    const TM* sk = stage_in + (step0 + k) * 4 * kStageVals;
    // stage 0: D = 0 (T = I), Pm = 0
    for (int a = lane; a < 225; a += 32) {
      S.D[a] = TM(0);
      S.Pm[a] = TM(0);
      S.sumtd[a] = TM(0);
      S.sumcd[a] = TM(0);
    }
    __syncwarp();
    for (int stg = 0; stg < 4; ++stg) {
      const TM* f = sk + stg * kStageVals;
      const TM wx = f[0], wy = f[1], wz = f[2], ax = f[3], ay = f[4], az = f[5];
      // F00 = -[w]x ; F69 = -G_R_B ; F60 = -G_R_B [a]x
      const TM F00[9] = {TM(0), wz, -wy, -wz, TM(0), wx, wy, -wx, TM(0)};
      TM F69[9], F60[9];
#pragma unroll
      for (int a = 0; a < 9; ++a) F69[a] = -f[6 + a];
      const TM axm[9] = {TM(0), -az, ay, az, TM(0), -ax, -ay, ax, TM(0)};
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          F60[3 * i + j] = F69[3 * i] * axm[j] + F69[3 * i + 1] * axm[3 + j] + F69[3 * i + 2] * axm[6 + j];
      // td = F T (T = I + D) and PC = F Pm, rows 0-2, 6-8, 12-14 (the other
      // rows are zero: the 135 active elements are spread over the lanes).
      for (int qa = lane; qa < 135; qa += 32) {
        const int r = 6 * (qa / 45) + (qa % 45) / 15, c = qa % 15, a = 15 * r + c;
        TM t = TM(0), pc = TM(0);
        if (r < 3) {
          t = (c < 3 ? F00[3 * r + c] : TM(0)) + F00[3 * r] * S.D[c] + F00[3 * r + 1] * S.D[15 + c] +
              F00[3 * r + 2] * S.D[30 + c] - (c == 3 + r ? TM(1) : TM(0));
          pc = F00[3 * r] * S.Pm[c] + F00[3 * r + 1] * S.Pm[15 + c] + F00[3 * r + 2] * S.Pm[30 + c] -
               S.Pm[(3 + r) * 15 + c];
        } else if (r >= 6 && r < 9) {
          const int q = r - 6;
          t = (c < 3 ? F60[3 * q + c] : TM(0)) + F60[3 * q] * S.D[c] + F60[3 * q + 1] * S.D[15 + c] +
              F60[3 * q + 2] * S.D[30 + c] + (c >= 9 && c < 12 ? F69[3 * q + c - 9] : TM(0));
          pc = F60[3 * q] * S.Pm[c] + F60[3 * q + 1] * S.Pm[15 + c] + F60[3 * q + 2] * S.Pm[30 + c] +
               F69[3 * q] * S.Pm[135 + c] + F69[3 * q + 1] * S.Pm[150 + c] + F69[3 * q + 2] * S.Pm[165 + c];
        } else if (r >= 12) {
          const int q = r - 12;
          t = (c == 6 + q ? TM(1) : TM(0)) + S.D[(6 + q) * 15 + c];
          pc = S.Pm[(6 + q) * 15 + c];
        }
        S.td[a] = t;
        S.PC[a] = pc;
      }
      __syncwarp();
      const TM wgt = (stg == 0 || stg == 3) ? TM(1) : TM(2);
      const TM cnext = (stg == 2) ? dt : TM(0.5) * dt;
      for (int a = lane; a < 225; a += 32) {
        const int r = a / 15, c = a % 15;
        TM cd = S.PC[a] + S.PC[c * 15 + r];
        if (r == c) cd += (r < 3) ? gn : (r < 6) ? gb : (r < 9) ? an : (r < 12) ? ab : TM(0);
        S.sumtd[a] += wgt * S.td[a];
        S.sumcd[a] += wgt * cd;
        if (stg < 3) {
          S.D[a] = cnext * S.td[a];
          S.Pm[a] = cnext * cd;
        }
      }
      __syncwarp();
    }
    // A = dt/6 sum(td) on rows 0-2, 6-8, 12-14 (into D); Qk = dt/6 sum(cd) (into Pm).
    for (int a = lane; a < 225; a += 32) {
      const int r = a / 15;
      S.D[a] = active_row(r) ? dt * S.sumtd[a] / TM(6) : TM(0);
      S.Pm[a] = dt * S.sumcd[a] / TM(6);
    }
    __syncwarp();
    // M = A Q (td), N = A Phi (PC); only the active rows are non-zero.
    for (int qa = lane; qa < 135; qa += 32) {
      const int r = 6 * (qa / 45) + (qa % 45) / 15, c = qa % 15, a = 15 * r + c;
      TM m = TM(0), n = TM(0);
#pragma unroll
      for (int j = 0; j < 15; ++j) {
        const TM arj = S.D[r * 15 + j];
        m += arj * S.Q[j * 15 + c];
        n += arj * S.Phi[j * 15 + c];
      }
      S.td[a] = m;
      S.PC[a] = n;
    }
    __syncwarp();
    // Q <- Q + M + M^T + M A^T + Qk ; Phi <- Phi + N   (written to sumtd / sumcd first)
    for (int a = lane; a < 225; a += 32) {
      const int r = a / 15, c = a % 15;
      TM q = S.Q[a] + S.td[a] + S.td[c * 15 + r] + S.Pm[a];
      if (active_row(r) && active_row(c)) {
        TM v = TM(0);
#pragma unroll
        for (int j = 0; j < 15; ++j) v += S.td[r * 15 + j] * S.D[c * 15 + j];
        q += v;
      }
      S.sumtd[a] = q;
      S.sumcd[a] = S.Phi[a] + S.PC[a];
    }
    __syncwarp();
    for (int a = lane; a < 225; a += 32) {
      S.Q[a] = S.sumtd[a];
      S.Phi[a] = S.sumcd[a];
    }
    __syncwarp();
  }
  inertial_tail<TM>(P, kf_state, end_in, out, e, S.Q, S.Phi, Ld[w], Xd[w], rsh[w], lane);
}

// The FP32 transition / covariance chain with one half-warp per edge and one
// lane per column: lane c keeps column c of Q_acc, Phi_acc, Pm and the stage
// sums in registers.  Left products by the (row-sparse) RK4 derivative F and
// by A act on columns, so they need no other lane's data; only the
// transposes (PC^T in the stage covariance, M^T and M A^T in the Q update)
// and the rows of A go through shared memory.  Rows of D, td, A and M are
// kept for the active rows 0-2, 6-8, 12-14 only (index i -> row kAct(i)).
// Q_acc and Phi_acc go to qp_out [edge][450] (row-major, Q then Phi) for the
// FP64 whitening kernel.
__device__ __forceinline__ constexpr int kAct(int i) { return i < 3 ? i : (i < 6 ? i + 3 : i + 6); }

template <int kWarps>
__global__ void __launch_bounds__(32 * kWarps, 4) k_inertial_mat_cols(DevProblem P, const float* stage_in,
                                                                   const double* dt_in, float* qp_out,
                                                                   const int* skip_if) {
  if (gated_i(skip_if)) return;
  __shared__ __align__(16) float ex[kWarps][2][512];  // per edge: X [16][16] then Y [16][16]
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, h = lane >> 4, c = lane & 15;
  const int64_t e0 = 2 * (blockIdx.x * (int64_t)kWarps + w);
  if (e0 >= P.nimu) return;  // uniform over the warp
  const int64_t e = e0 + h;
  const unsigned hm = 0xffffu << (16 * h);
  float* X = ex[w][h];
  float* Y = X + 256;
  const bool col = c < 15;
  if (e < P.nimu) {
    const float gn = float(P.gyro_noise2), gb = float(P.gyro_bias2), an = float(P.acc_noise2),
                ab = float(P.acc_bias2);
    const float noise = c < 3 ? gn : c < 6 ? gb : c < 9 ? an : c < 12 ? ab : 0.f;  // diagonal of the stage covariance
    const bool cact = col && active_row(c);
    float Q[15], Phi[15];
#pragma unroll
    for (int r = 0; r < 15; ++r) {
      Q[r] = 0.f;
      Phi[r] = (r == c) ? 1.f : 0.f;
    }
    const int64_t o0 = P.e_off[e];
    const int ns = (int)(P.e_off[e + 1] - o0);
    const int64_t step0 = o0 - e;
    for (int k = 0; k + 1 < ns; ++k) {
      const float dt = float(dt_in[step0 + k]);
      const float* sk = stage_in + (step0 + k) * 4 * kStageVals;
      float D[9], Pm[15], sumtd[9], sumcd[15];
#pragma unroll
      for (int i = 0; i < 9; ++i) { D[i] = 0.f; sumtd[i] = 0.f; }
#pragma unroll
      for (int r = 0; r < 15; ++r) { Pm[r] = 0.f; sumcd[r] = 0.f; }
#pragma unroll 1
      for (int stg = 0; stg < 4; ++stg) {
        const float* f = sk + stg * kStageVals;
        const float wx = f[0], wy = f[1], wz = f[2], ax = f[3], ay = f[4], az = f[5];
        const float F00[9] = {0.f, wz, -wy, -wz, 0.f, wx, wy, -wx, 0.f};
        float F69[9], F60[9];
#pragma unroll
        for (int a = 0; a < 9; ++a) F69[a] = -f[6 + a];
        const float axm[9] = {0.f, -az, ay, az, 0.f, -ax, -ay, ax, 0.f};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j)
            F60[3 * i + j] = F69[3 * i] * axm[j] + F69[3 * i + 1] * axm[3 + j] + F69[3 * i + 2] * axm[6 + j];
        // td = F (I + D) and PC = F Pm, column c, active rows.
        float td[9], pc[9];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          td[q] = (c < 3 ? F00[3 * q + c] : 0.f) + F00[3 * q] * D[0] + F00[3 * q + 1] * D[1] + F00[3 * q + 2] * D[2] -
                  (c == 3 + q ? 1.f : 0.f);
          pc[q] = F00[3 * q] * Pm[0] + F00[3 * q + 1] * Pm[1] + F00[3 * q + 2] * Pm[2] - Pm[3 + q];
          td[3 + q] = (c < 3 ? F60[3 * q + c] : 0.f) + F60[3 * q] * D[0] + F60[3 * q + 1] * D[1] +
                      F60[3 * q + 2] * D[2] + (c >= 9 && c < 12 ? F69[3 * q + c - 9] : 0.f);
          pc[3 + q] = F60[3 * q] * Pm[0] + F60[3 * q + 1] * Pm[1] + F60[3 * q + 2] * Pm[2] + F69[3 * q] * Pm[9] +
                      F69[3 * q + 1] * Pm[10] + F69[3 * q + 2] * Pm[11];
          td[6 + q] = (c == 6 + q ? 1.f : 0.f) + D[3 + q];
          pc[6 + q] = Pm[6 + q];
        }
        if (col)
#pragma unroll
          for (int i = 0; i < 9; ++i) X[16 * kAct(i) + c] = pc[i];
        __syncwarp(hm);
        // cd = PC + PC^T + noise; PC^T's column c is row c of PC (non-zero for active c).
        const float wgt = (stg == 0 || stg == 3) ? 1.f : 2.f;
        const float cnext = (stg == 2) ? dt : 0.5f * dt;
        float cd[15];
#pragma unroll
        for (int r = 0; r < 15; ++r) cd[r] = (cact ? X[16 * c + r] : 0.f) + (r == c ? noise : 0.f);
#pragma unroll
        for (int i = 0; i < 9; ++i) cd[kAct(i)] += pc[i];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          sumtd[i] += wgt * td[i];
          if (stg < 3) D[i] = cnext * td[i];
        }
#pragma unroll
        for (int r = 0; r < 15; ++r) {
          sumcd[r] += wgt * cd[r];
          if (stg < 3) Pm[r] = cnext * cd[r];
        }
        __syncwarp(hm);  // X is rewritten by the next stage
      }
      // A = dt/6 sum(td) (rows of A to X), Qk = dt/6 sum(cd).
      float Acol[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        Acol[i] = dt * sumtd[i] / 6.f;
        if (col) X[16 * kAct(i) + c] = Acol[i];
      }
      __syncwarp(hm);
      // M = A Q, N = A Phi (column c, active rows); M to Y for the transposes.
      float M[9], Nn[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        float m = 0.f, n = 0.f;
#pragma unroll
        for (int j = 0; j < 15; ++j) {
          const float arj = X[16 * kAct(i) + j];
          m += arj * Q[j];
          n += arj * Phi[j];
        }
        M[i] = m;
        Nn[i] = n;
        if (col) Y[16 * kAct(i) + c] = m;
      }
      __syncwarp(hm);
      // Q <- Q + M + M^T + M A^T + Qk ; Phi <- Phi + N
      float Mfull[15];
#pragma unroll
      for (int r = 0; r < 15; ++r) Mfull[r] = 0.f;
#pragma unroll
      for (int i = 0; i < 9; ++i) Mfull[kAct(i)] = M[i];
#pragma unroll
      for (int r = 0; r < 15; ++r) {
        float q = Q[r] + Mfull[r] + (cact ? Y[16 * c + r] : 0.f) + dt * sumcd[r] / 6.f;
        if (cact && active_row(r)) {
          float v = 0.f;
#pragma unroll
          for (int j = 0; j < 15; ++j) v += Y[16 * r + j] * X[16 * c + j];
          q += v;
        }
        Q[r] = q;
      }
#pragma unroll
      for (int i = 0; i < 9; ++i) Phi[kAct(i)] += Nn[i];
      __syncwarp(hm);  // X and Y are rewritten by the next step
    }
    if (col) {
      float* o = qp_out + 450 * e;
#pragma unroll
      for (int r = 0; r < 15; ++r) {
        o[15 * r + c] = Q[r];
        o[225 + 15 * r + c] = Phi[r];
      }
    }
  }
}

// FP64 whitening, residual and Jacobians of the mixed path: one warp per
// edge from the FP32 Q_acc / Phi_acc of k_inertial_mat_cols.
template <int kWarps>
__global__ void __launch_bounds__(32 * kWarps) k_inertial_whiten(DevProblem P, const double* kf_state,
                                                                 const float* qp_in, const double* end_in,
                                                                 InertialOutputs out, const int* skip_if) {
  if (gated_i(skip_if)) return;
  __shared__ float qs[kWarps][450];
  __shared__ double Ld[kWarps][225], Xd[kWarps][225], rsh[kWarps][16];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t e = blockIdx.x * (int64_t)kWarps + w;
  if (e >= P.nimu) return;
  for (int a = lane; a < 450; a += 32) qs[w][a] = qp_in[450 * e + a];
  __syncwarp();
  inertial_tail<float>(P, kf_state, end_in, out, e, qs[w], qs[w] + 225, Ld[w], Xd[w], rsh[w], lane);
}

}  // namespace

cudaError_t launch_inertial_v2(const DevProblem& P, const double* kf_state, bool f32_matrices, InertialLin<double> lin,
                               double* amb_res, double* const* amb_jac, double* cost_accum, int* status,
                               const int* skip_if, cudaStream_t s) {
  if (P.nimu == 0) return cudaSuccess;
  InertialOutputs o;
  o.lin_r = lin.r;
  o.lin_Jf = lin.Jf;
  o.lin_Jt = lin.Jt;
  o.amb_res = amb_res;
  for (int b = 0; b < 8; ++b) o.amb_J[b] = amb_jac ? amb_jac[b] : nullptr;
  o.cost = cost_accum;
  o.status = status;
  const int64_t nsteps = P.nsamp - P.nimu;
  double* dt = P.ine_scratch;
  double* endst = dt + nsteps;
  void* stage = endst + 16 * P.nimu;
  const unsigned gA = (unsigned)((P.nimu + 127) / 128);
  if (f32_matrices) {
    k_inertial_state<float><<<gA, 128, 0, s>>>(P, kf_state, (float*)stage, dt, endst, status, skip_if);
    constexpr int W = 4;  // two edges per warp
    float* qp = reinterpret_cast<float*>(endst + 16 * P.nimu + 60 * nsteps);
    k_inertial_mat_cols<W><<<(unsigned)((P.nimu + 2 * W - 1) / (2 * W)), 32 * W, 0, s>>>(
        P, (const float*)stage, dt, qp, skip_if);
    k_inertial_whiten<W><<<(unsigned)((P.nimu + W - 1) / W), 32 * W, 0, s>>>(P, kf_state, qp, endst, o, skip_if);
  } else {
    k_inertial_state<double><<<gA, 128, 0, s>>>(P, kf_state, (double*)stage, dt, endst, status, skip_if);
    constexpr int W = 1;
    k_inertial_mat<double, W><<<(unsigned)((P.nimu + W - 1) / W), 32 * W, 0, s>>>(P, kf_state, (const double*)stage,
                                                                                    dt, endst, o, skip_if);
  }
  return cudaGetLastError();
}

}  // namespace mba
