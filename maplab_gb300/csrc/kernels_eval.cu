// Evaluation kernels: visual reprojection terms (one thread per observation,
// SoA in/out); the inertial launchers route to kernels_inertial.cu.
//
// Visual: VisualReprojectionError::Evaluate
//   (algorithms/ceres-error-terms/include/ceres-error-terms/visual-error-term-inl.h:12-379)
// Inertial: InertialErrorTerm::Evaluate / IntegrateStateAndCovariance
//   (algorithms/ceres-error-terms/src/inertial-error-term.cc:9-286) with
//   ImuIntegratorRK4::integrate
//   (algorithms/imu-integrator-rk4/include/imu-integrator/imu-integrator-inl.h:17-334).
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"

namespace mba {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of v, one atomicAdd per block into *acc.
__device__ __forceinline__ void block_accumulate(double v, double* acc) {
  __shared__ double red[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    v = warp_sum(v);
    if (lane == 0 && v != 0.0) atomicAdd(acc, v);
  }
}

__device__ __forceinline__ bool gated(const int* run_if, const int* skip_if) {
  if (skip_if && *skip_if) return true;
  if (run_if && !*run_if) return true;
  return false;
}

template <typename T>
__device__ __forceinline__ void load_q(const double* s, T* q) {
  const double2 a = *reinterpret_cast<const double2*>(s);
  const double2 b = *reinterpret_cast<const double2*>(s + 2);
  q[0] = T(a.x); q[1] = T(a.y); q[2] = T(b.x); q[3] = T(b.y);
}

// Rotation-tangent basis of keyframe k: Ceres applies the local
// parameterization Jacobian on top of the ambient 4-column quaternion block;
// with the 4*Jq^T lift of the error terms this gives J_theta * B where
// B = |q|^2 I for JplQuaternionParameterization and
// B = -|q|^2 (R_I_M R_M_G)[:, 0:2] for JplRollPitchQuaternionParameterization
// (quaternion-param-jpl.cc:144-164).  Masked tangent dims are zero columns.
template <typename T, typename S>
__device__ __forceinline__ void rot_basis(const DevProblem& P, const S* mis, int k, const T* q, const M3<T>& R_I_M,
                                          M3<T>& B) {
  const uint16_t m = P.kf_mask[k];
  const T n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  if (P.kf_flags[k] & MBA_KF_GAUGE_ROLL_PITCH) {
    T qg[4];
    const S* mq = mis + 8 * P.kf_mis[k];
    qg[0] = T(mq[0]); qg[1] = T(mq[1]); qg[2] = T(mq[2]); qg[3] = T(mq[3]);
    M3<T> R_G_M;
    jplR(qg, R_G_M);
    // R_I_M * R_M_G = R_I_M * R_G_M^T
    M3<T> A;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        A.m[3 * i + j] = R_I_M.m[3 * i] * R_G_M.m[3 * j] + R_I_M.m[3 * i + 1] * R_G_M.m[3 * j + 1] +
                         R_I_M.m[3 * i + 2] * R_G_M.m[3 * j + 2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      B.m[3 * i + 0] = (m & 1) ? -n2 * A.m[3 * i + 0] : T(0);
      B.m[3 * i + 1] = (m & 2) ? -n2 * A.m[3 * i + 1] : T(0);
      B.m[3 * i + 2] = T(0);
    }
  } else {
#pragma unroll
    for (int i = 0; i < 9; ++i) B.m[i] = T(0);
    B.m[0] = (m & 1) ? n2 : T(0);
    B.m[4] = (m & 2) ? n2 : T(0);
    B.m[8] = (m & 4) ? n2 : T(0);
  }
}

// ------------------------------------------------------------------ visual
// Tangent-space, Huber-corrected linearization of every observation.  kCost
// adds the FP64 cost reduction (FP64 path only): the FP32 instantiation reads
// the FP32 mirrors and executes no FP64 instruction.
//
// The global reads of one observation are split in two stages so that a
// pipelined loop can overlap them with the arithmetic of the previous
// observation: load_obs_stream (the observation's own streamed fields,
// coalesced) and load_obs_gather (landmark and keyframe poses addressed by
// them).  compute_obs holds the arithmetic and the stores.
template <typename T>
struct ObsInputs {
  typename Vec2<T>::type uv;
  T sinv, ha;
  T pB[3];
  T xs[7], xo[7];  // store / observer pose q | p
  int lm, kf, st, type, cam;
  int lm_off, lm_active;
};

template <typename T>
__device__ __forceinline__ void load_obs_stream(const DevProblem& P, const VisualInputs<T>& in, int64_t i,
                                                ObsInputs<T>& o) {
  o.lm = P.obs_lm[i];
  o.kf = P.obs_kf[i];
  o.st = P.obs_store[i];
  o.type = P.obs_type[i];
  o.cam = P.obs_cam[i];
  o.uv = in.uv[i];
  o.sinv = in.sinv[i];
  o.ha = in.huber[i];
}

template <typename T>
__device__ __forceinline__ void load_obs_gather(const DevProblem& P, const VisualInputs<T>& in, ObsInputs<T>& o) {
  const T* lp = in.lm_p + 4 * (int64_t)o.lm;
  o.pB[0] = lp[0]; o.pB[1] = lp[1]; o.pB[2] = lp[2];
  o.lm_off = P.lm_off[o.lm];
  o.lm_active = P.lm_active[o.lm];
  if (o.type != MBA_LOCAL_KEYFRAME) {
    const T* xs = in.kf + (int64_t)in.kf_stride * o.st;
    const T* xo = in.kf + (int64_t)in.kf_stride * o.kf;
#pragma unroll
    for (int a = 0; a < 7; ++a) { o.xs[a] = xs[a]; o.xo[a] = xo[a]; }
  }
}

// Arithmetic and stores of observation i; returns its cost (kCost).
// rci: the camera's R_C_I (9 values, e.g. from the block's shared memory) or
// null; FP64 inputs carry the keyframes' rotation matrices and |q|^2
// (in.kf_rot, written by k_kf_rotations) so that the kernel does not rebuild
// them per observation.
template <typename T, bool kCost>
__device__ __forceinline__ double compute_obs(const DevProblem& P, const VisualInputs<T>& in, const ObsInputs<T>& o,
                                              const VisualLin<T>& out, int64_t i, int64_t N, const T* rci) {
  double cost = 0.0;
  const int kf = o.kf, st = o.st, type = o.type;
  const DevCameraT<T>& cam = in.cams[o.cam];
  const auto uv = o.uv;
  const T sinv = o.sinv;
  const T ha = o.ha;
  const T pB[3] = {o.pB[0], o.pB[1], o.pB[2]};
  M3<T> RCI;
  if (rci) {
#pragma unroll
    for (int a = 0; a < 9; ++a) RCI.m[a] = rci[a];
  } else {
    jplR(cam.q_CI, RCI);
  }
  T pI[3];
  M3<T> RIM, RBLM, RMG, RGLM;
  T qst[4], qob[4], pLMB[3], pMI[3];
  T n2s = T(0), n2o = T(0);  // |q|^2 of the store / observer keyframe
  if (type == MBA_LOCAL_KEYFRAME) {
    pI[0] = pB[0]; pI[1] = pB[1]; pI[2] = pB[2];
  } else {
#pragma unroll
    for (int a = 0; a < 4; ++a) { qst[a] = o.xs[a]; qob[a] = o.xo[a]; }
    pLMB[0] = o.xs[4]; pLMB[1] = o.xs[5]; pLMB[2] = o.xs[6];
    pMI[0] = o.xo[4]; pMI[1] = o.xo[5]; pMI[2] = o.xo[6];
    if (sizeof(T) == 8 && in.kf_rot) {
      const T* ra = in.kf_rot + 16 * (int64_t)st;
      const T* rb = in.kf_rot + 16 * (int64_t)kf;
#pragma unroll
      for (int a = 0; a < 9; ++a) { RBLM.m[a] = ra[a]; RIM.m[a] = rb[a]; }
      n2s = ra[9];
      n2o = rb[9];
    } else {
      jplR(qst, RBLM);
      jplR(qob, RIM);
      n2s = qst[0] * qst[0] + qst[1] * qst[1] + qst[2] * qst[2] + qst[3] * qst[3];
      n2o = qob[0] * qob[0] + qob[1] * qob[1] + qob[2] * qob[2] + qob[3] * qob[3];
    }
    T pM[3];
    mtv3(RBLM, pB, pM);  // R_LM_B p_B
    pM[0] += pLMB[0]; pM[1] += pLMB[1]; pM[2] += pLMB[2];
    if (type == MBA_GLOBAL) {
      const T* ml = in.mis + 8 * P.kf_mis[st];
      const T* mo = in.mis + 8 * P.kf_mis[kf];
      jplR(ml, RGLM);
      M3<T> RGM;
      jplR(mo, RGM);
      T pG[3];
      mv3(RGLM, pM, pG);
      pG[0] += ml[4] - mo[4]; pG[1] += ml[5] - mo[5]; pG[2] += ml[6] - mo[6];
      mtv3(RGM, pG, pM);  // R_M_G (p_G - p_G_M)
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) RMG.m[3 * a + b] = RGM.m[3 * b + a];
    }
    T d[3] = {pM[0] - pMI[0], pM[1] - pMI[1], pM[2] - pMI[2]};
    mv3(RIM, d, pI);
  }
  T pC[3];
  mv3(RCI, pI, pC);
  pC[0] += cam.p_CI[0]; pC[1] += cam.p_CI[1]; pC[2] += cam.p_CI[2];
  T kp[2], Jkp[6];
  const bool failed = project<T>(cam, pC, kp, Jkp) || o.lm_off;
  T r[2], Jl[6], Js[12], Jo[12];
#pragma unroll
  for (int a = 0; a < 12; ++a) { Js[a] = T(0); Jo[a] = T(0); }
  if (failed) {
    r[0] = r[1] = T(0);
#pragma unroll
    for (int a = 0; a < 6; ++a) Jl[a] = T(0);
  } else {
    r[0] = (kp[0] - uv.x) * sinv;
    r[1] = (kp[1] - uv.y) * sinv;
    // Every Jacobian block is linear in the projection Jacobian: scale it by
    // 1 / sigma once instead of each of the 32 outputs.
#pragma unroll
    for (int a = 0; a < 6; ++a) Jkp[a] *= sinv;
    T A[6];
    m23x33(Jkp, RCI, A);  // Jkp * R_C_I / sigma
    if (type == MBA_LOCAL_KEYFRAME) {
#pragma unroll
      for (int a = 0; a < 6; ++a) Jl[a] = A[a];
    } else {
      T B[6], Cp[6];
      m23x33(A, RIM, B);  // Jkp R_C_I R_I_M  (= -J_p_M_I)
      if (type == MBA_LOCAL_MISSION) {
#pragma unroll
        for (int a = 0; a < 6; ++a) Cp[a] = B[a];
      } else {
        T D[6];
        m23x33(B, RMG, D);   // J_p_G_LM
        m23x33(D, RGLM, Cp); // J_p_LM_B
      }
      // J_p_B = J_p_LM_B * R_LM_B  (R_LM_B = R_B_LM^T)
      T JpB[6];
#pragma unroll
      for (int rr = 0; rr < 2; ++rr)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          JpB[3 * rr + c] = Cp[3 * rr] * RBLM.m[3 * c] + Cp[3 * rr + 1] * RBLM.m[3 * c + 1] + Cp[3 * rr + 2] * RBLM.m[3 * c + 2];
      T Jqs[6], Jqo[6];
      m23xskew(JpB, pB, Jqs);  // -J_q_B_LM
      m23xskew(A, pI, Jqo);    // J_q_I_M
      const uint16_t ms = P.kf_mask[st], mo = P.kf_mask[kf];
      // Rotation tangent: J_theta * B.  B = |q|^2 I (masked columns zero) for
      // JplQuaternionParameterization, a full 3 x 2 basis only for the
      // gauge keyframe's roll / pitch parameterization; the scaled identity
      // is applied as a scalar (same products, fewer instructions).
      const bool rps = P.kf_flags[st] & MBA_KF_GAUGE_ROLL_PITCH, rpo = P.kf_flags[kf] & MBA_KF_GAUGE_ROLL_PITCH;
      if (!rps) {
#pragma unroll
        for (int rr = 0; rr < 2; ++rr)
#pragma unroll
          for (int c = 0; c < 3; ++c) Js[6 * rr + c] = (ms & (1u << c)) ? -(Jqs[3 * rr + c] * n2s) : T(0);
      } else {
        M3<T> Bs;
        rot_basis<T>(P, in.mis, st, qst, RBLM, Bs);
#pragma unroll
        for (int rr = 0; rr < 2; ++rr)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            Js[6 * rr + c] = -(Jqs[3 * rr] * Bs.m[c] + Jqs[3 * rr + 1] * Bs.m[3 + c] + Jqs[3 * rr + 2] * Bs.m[6 + c]);
      }
      if (!rpo) {
#pragma unroll
        for (int rr = 0; rr < 2; ++rr)
#pragma unroll
          for (int c = 0; c < 3; ++c) Jo[6 * rr + c] = (mo & (1u << c)) ? (Jqo[3 * rr + c] * n2o) : T(0);
      } else {
        M3<T> Bo;
        rot_basis<T>(P, in.mis, kf, qob, RIM, Bo);
#pragma unroll
        for (int rr = 0; rr < 2; ++rr)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            Jo[6 * rr + c] = (Jqo[3 * rr] * Bo.m[c] + Jqo[3 * rr + 1] * Bo.m[3 + c] + Jqo[3 * rr + 2] * Bo.m[6 + c]);
      }
#pragma unroll
      for (int rr = 0; rr < 2; ++rr) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          Js[6 * rr + 3 + c] = (ms & (8u << c)) ? Cp[3 * rr + c] : T(0);
          Jo[6 * rr + 3 + c] = (mo & (8u << c)) ? -B[3 * rr + c] : T(0);
        }
      }
#pragma unroll
      for (int a = 0; a < 6; ++a) Jl[a] = JpB[a];
    }
    if (!o.lm_active) {
#pragma unroll
      for (int a = 0; a < 6; ++a) Jl[a] = T(0);
    }
  }
  const T s = r[0] * r[0] + r[1] * r[1];
  // Inside the Huber threshold (s <= a^2) the loss is the identity: rho' = 1,
  // rho'' = 0, so the corrector leaves r and J unchanged and the cost is s / 2.
  // Only observations beyond it pay for the correction.
  if (ha > T(0) && s > ha * ha) {
    T rho0, sq1, rs, as;
    huber_corrector<T>(ha, s, &rho0, &sq1, &rs, &as);
    if (kCost) cost = 0.5 * double(rho0);
    // J' = sq1 (J - as r (r^T J)), r' = rs r
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const T t = r[0] * Jl[c] + r[1] * Jl[3 + c];
      Jl[c] = sq1 * (Jl[c] - as * r[0] * t);
      Jl[3 + c] = sq1 * (Jl[3 + c] - as * r[1] * t);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const T t = r[0] * Js[c] + r[1] * Js[6 + c];
      Js[c] = sq1 * (Js[c] - as * r[0] * t);
      Js[6 + c] = sq1 * (Js[6 + c] - as * r[1] * t);
      const T u = r[0] * Jo[c] + r[1] * Jo[6 + c];
      Jo[c] = sq1 * (Jo[c] - as * r[0] * u);
      Jo[6 + c] = sq1 * (Jo[6 + c] - as * r[1] * u);
    }
    r[0] *= rs;
    r[1] *= rs;
  } else if (kCost) {
    cost = 0.5 * double(s);
  }
  out.r[i] = r[0];
  out.r[N + i] = r[1];
#pragma unroll
  for (int a = 0; a < 6; ++a) out.Jl[a * N + i] = Jl[a];
#pragma unroll
  for (int a = 0; a < 12; ++a) out.Js[a * N + i] = Js[a];
#pragma unroll
  for (int a = 0; a < 12; ++a) out.Jo[a * N + i] = Jo[a];
  return cost;
}

// The cameras' R_C_I, built once per block into shared memory (at most
// kCamRot cameras; returns false for more, and compute_obs builds them).
constexpr int kCamRot = 16;
template <typename T>
__device__ __forceinline__ bool stage_camera_rotations(const DevProblem& P, const VisualInputs<T>& in, T* rci) {
  if (P.ncam > kCamRot) return false;
  for (int c = threadIdx.x; c < P.ncam; c += blockDim.x) {
    M3<T> R;
    jplR(in.cams[c].q_CI, R);
#pragma unroll
    for (int a = 0; a < 9; ++a) rci[9 * c + a] = R.m[a];
  }
  __syncthreads();
  return true;
}

// One thread per observation.  kMinBlocks > 1 trades registers (spilled to
// L1) for resident warps; the autotuner picks the variant per problem.
template <typename T, bool kCost, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_visual_linearize(DevProblem P, VisualInputs<T> in, VisualLin<T> out,
                                                             double* cost_accum, const int* run_if,
                                                             const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  __shared__ T rci[9 * kCamRot];
  const bool cam_sm = stage_camera_rotations(P, in, rci);
  const int64_t i = P.vis_lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double cost = 0.0;
  if (i < vis_end(P)) {
    ObsInputs<T> o;
    load_obs_stream(P, in, i, o);
    load_obs_gather(P, in, o);
    cost = compute_obs<T, kCost>(P, in, o, out, i, P.nobs, cam_sm ? rci + 9 * o.cam : nullptr);
  }
  if (kCost) block_accumulate(cost, cost_accum);
}

// Persistent, software-pipelined: a grid of resident blocks strides over the
// observations; while observation i is computed, the gathers of i + stride
// (whose indices arrived during the previous iteration) and the streamed
// fields of i + 2 stride are in flight.  Three observations per thread are in
// the memory system at once instead of one.  kMinBlocks = 2 caps the
// registers (more resident warps, some spilling).
template <typename T, bool kCost, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_visual_linearize_pipe(DevProblem P, VisualInputs<T> in, VisualLin<T> out,
                                                                  double* cost_accum, const int* run_if,
                                                                  const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  __shared__ T rci[9 * kCamRot];
  const bool cam_sm = stage_camera_rotations(P, in, rci);
  // observations [vis_lo, hi) of the component-major outputs of stride N
  const int64_t N = P.nobs, hi = vis_end(P), stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = P.vis_lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double cost = 0.0;
  ObsInputs<T> cur, nxt;
  if (i < hi) {
    load_obs_stream(P, in, i, cur);
    load_obs_gather(P, in, cur);
  }
  if (i + stride < hi) load_obs_stream(P, in, i + stride, nxt);
  for (; i < hi; i += stride) {
    const int64_t j = i + stride;
    if (j < hi) load_obs_gather(P, in, nxt);
    ObsInputs<T> nn;
    if (j + stride < hi) load_obs_stream(P, in, j + stride, nn);
    cost += compute_obs<T, kCost>(P, in, cur, out, i, N, cam_sm ? rci + 9 * cur.cam : nullptr);
    cur = nxt;
    nxt = nn;
  }
  if (kCost) block_accumulate(cost, cost_accum);
}

// FP64 residual-only cost at an arbitrary state (candidate evaluation).
// Landmark of observation i in the observing camera frame (FP64), following
// the frame chain of the visual term for its error type.
__device__ void obs_point_C(const DevProblem& P, const double* kf_state, const double* lm_p, int64_t i, double* pC) {
  const int lm = P.obs_lm[i], kf = P.obs_kf[i], st = P.obs_store[i], type = P.obs_type[i];
  const DevCamera& cam = P.cams[P.obs_cam[i]];
  const double pB[3] = {lm_p[4 * (int64_t)lm], lm_p[4 * (int64_t)lm + 1], lm_p[4 * (int64_t)lm + 2]};
  M3<double> RCI;
  jplR(cam.q_CI, RCI);
  double pI[3];
  if (type == MBA_LOCAL_KEYFRAME) {
    pI[0] = pB[0]; pI[1] = pB[1]; pI[2] = pB[2];
  } else {
    const double* xs = kf_state + 16 * (int64_t)st;
    const double* xo = kf_state + 16 * (int64_t)kf;
    M3<double> RBLM, RIM;
    jplR(xs, RBLM);
    jplR(xo, RIM);
    double pM[3];
    mtv3(RBLM, pB, pM);
    pM[0] += xs[4]; pM[1] += xs[5]; pM[2] += xs[6];
    if (type == MBA_GLOBAL) {
      const double* ml = P.mis + 8 * P.kf_mis[st];
      const double* mo = P.mis + 8 * P.kf_mis[kf];
      M3<double> RGLM, RGM;
      jplR(ml, RGLM);
      jplR(mo, RGM);
      double pG[3];
      mv3(RGLM, pM, pG);
      pG[0] += ml[4] - mo[4]; pG[1] += ml[5] - mo[5]; pG[2] += ml[6] - mo[6];
      mtv3(RGM, pG, pM);
    }
    const double d[3] = {pM[0] - xo[4], pM[1] - xo[5], pM[2] - xo[6]};
    mv3(RIM, d, pI);
  }
  mv3(RCI, pI, pC);
  pC[0] += cam.p_CI[0]; pC[1] += cam.p_CI[1]; pC[2] += cam.p_CI[2];
}

__global__ void __launch_bounds__(kBlock) k_visual_cost(DevProblem P, const double* kf_state, const double* lm_p,
                                                        double* cost_accum, int* nonfinite, const int* run_if,
                                                        const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double cost = 0.0;
  if (i < P.nobs && !P.lm_off[P.obs_lm[i]]) {
    const DevCamera& cam = P.cams[P.obs_cam[i]];
    double pC[3];
    obs_point_C(P, kf_state, lm_p, i, pC);
    double kp[2];
    const bool failed = project<double>(cam, pC, kp, nullptr);
    if (!failed) {
      const double2 uv = P.obs_uv[i];
      const double sinv = P.obs_sinv[i];
      const double r0 = (kp[0] - uv.x) * sinv, r1 = (kp[1] - uv.y) * sinv;
      const double s = r0 * r0 + r1 * r1;
      const double a = P.obs_huber[i];
      if (a > 0.0 && s > a * a) cost = 0.5 * (2.0 * a * sqrt(s) - a * a);
      else cost = 0.5 * s;
      if (!isfinite(cost) && nonfinite) *nonfinite = 1;
    }
  }
  block_accumulate(cost, cost_accum);
}

// FP32 candidate cost (mixed path): the visual term's frame chain and
// projection in FP32 from FP32 copies of the candidate state, robustified
// cost summed in FP64.  No FP64 arithmetic per observation.
// FP32 landmark of observation i in the observing camera frame, from FP32
// copies of the state (pose q p pad [n][8], landmark [n][4]).
__device__ void obs_point_C_f32(const DevProblem& P, const float* kf, const float* lp, int64_t i, float* pC) {
  const int lm = P.obs_lm[i], k = P.obs_kf[i], st = P.obs_store[i], type = P.obs_type[i];
  const DevCameraT<float>& cam = P.cams_f[P.obs_cam[i]];
  const float pB[3] = {lp[4 * (int64_t)lm], lp[4 * (int64_t)lm + 1], lp[4 * (int64_t)lm + 2]};
  M3<float> RCI;
  jplR(cam.q_CI, RCI);
  float pI[3];
  if (type == MBA_LOCAL_KEYFRAME) {
    pI[0] = pB[0]; pI[1] = pB[1]; pI[2] = pB[2];
  } else {
    const float* xs = kf + 8 * (int64_t)st;
    const float* xo = kf + 8 * (int64_t)k;
    M3<float> RBLM, RIM;
    jplR(xs, RBLM);
    jplR(xo, RIM);
    float pM[3];
    mtv3(RBLM, pB, pM);
    pM[0] += xs[4]; pM[1] += xs[5]; pM[2] += xs[6];
    if (type == MBA_GLOBAL) {
      const float* ml = P.mis_f + 8 * P.kf_mis[st];
      const float* mo = P.mis_f + 8 * P.kf_mis[k];
      M3<float> RGLM, RGM;
      jplR(ml, RGLM);
      jplR(mo, RGM);
      float pG[3];
      mv3(RGLM, pM, pG);
      pG[0] += ml[4] - mo[4]; pG[1] += ml[5] - mo[5]; pG[2] += ml[6] - mo[6];
      mtv3(RGM, pG, pM);
    }
    const float d[3] = {pM[0] - xo[4], pM[1] - xo[5], pM[2] - xo[6]};
    mv3(RIM, d, pI);
  }
  mv3(RCI, pI, pC);
  pC[0] += cam.p_CI[0]; pC[1] += cam.p_CI[1]; pC[2] += cam.p_CI[2];
}

__global__ void __launch_bounds__(kBlock) k_visual_cost_f32(DevProblem P, const float* kf, const float* lp,
                                                            double* cost_accum, int* nonfinite, const int* run_if,
                                                            const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double cost = 0.0;
  if (i < P.nobs && !P.lm_off[P.obs_lm[i]]) {
    const DevCameraT<float>& cam = P.cams_f[P.obs_cam[i]];
    float pC[3];
    obs_point_C_f32(P, kf, lp, i, pC);
    float kp[2];
    if (!project<float>(cam, pC, kp, nullptr)) {
      const float2 uv = P.obs_uv_f[i];
      const float sinv = P.obs_sinv_f[i];
      const float r0 = (kp[0] - uv.x) * sinv, r1 = (kp[1] - uv.y) * sinv;
      const double sq = (double)r0 * r0 + (double)r1 * r1;
      const double a = (double)P.obs_huber_f[i];
      cost = (a > 0.0 && sq > a * a) ? 0.5 * (2.0 * a * sqrt(sq) - a * a) : 0.5 * sq;
      if (!isfinite(cost) && nonfinite) *nonfinite = 1;
    }
  }
  block_accumulate(cost, cost_accum);
}

// Outlier test per observation (outlier-rejection-solver.cc:28-103): depth
// p_C.z <= 0, or (optionally) squared reprojection error in pixels above
// max_px^2, marks the landmark.  Landmarks already out are skipped.
__global__ void __launch_bounds__(kBlock) k_find_outliers(DevProblem P, int use_reprojection, double max_px2,
                                                          int* count, const int* run_if, const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.nobs) return;
  const int lm = P.obs_lm[i];
  if (P.lm_off[lm]) return;
  double pC[3];
  obs_point_C(P, P.kf_state, P.lm_p, i, pC);
  bool out = !(pC[2] > 0.0);
  if (!out && use_reprojection) {
    double kp[2];
    project<double>(P.cams[P.obs_cam[i]], pC, kp, nullptr);
    const double2 uv = P.obs_uv[i];
    const double e0 = kp[0] - uv.x, e1 = kp[1] - uv.y;
    out = !(e0 * e0 + e1 * e1 <= max_px2);
  }
  if (out && atomicExch(&P.lm_off[lm], 1) == 0) atomicAdd(count, 1);
}

// The same test on the FP32 copies of the state (mixed path).
__global__ void __launch_bounds__(kBlock) k_find_outliers_f32(DevProblem P, int use_reprojection, float max_px2,
                                                              int* count, const int* run_if, const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.nobs) return;
  const int lm = P.obs_lm[i];
  if (P.lm_off[lm]) return;
  float pC[3];
  obs_point_C_f32(P, P.kf_pose_f, P.lm_p_f, i, pC);
  bool out = !(pC[2] > 0.0f);
  if (!out && use_reprojection) {
    float kp[2];
    project<float>(P.cams_f[P.obs_cam[i]], pC, kp, nullptr);
    const float2 uv = P.obs_uv_f[i];
    const float e0 = kp[0] - uv.x, e1 = kp[1] - uv.y;
    out = !(e0 * e0 + e1 * e1 <= max_px2);
  }
  if (out && atomicExch(&P.lm_off[lm], 1) == 0) atomicAdd(count, 1);
}

// isVisualLandmarkWellConstrained (landmark-quality-metrics.cc:103-166), one
// thread per landmark, FP64.  The observing cameras' global positions and the
// landmark's global position give the incidence rays; the maximum disparity
// angle is acos of the smallest |cos| over all ray pairs
// (getMaxDisparityRadAngleOfUnitVectorBundle, maplab-common geometry.cc:30-44),
// recomputed per pair instead of stored.
__device__ void camera_center_G(const DevProblem& P, int k, int cam, double* pG) {
  const DevCamera& c = P.cams[cam];
  M3<double> RCI, RIM, RGM;
  jplR(c.q_CI, RCI);
  double pIC[3];
  mtv3(RCI, c.p_CI, pIC);  // R_C_I^T p_C_I
  pIC[0] = -pIC[0]; pIC[1] = -pIC[1]; pIC[2] = -pIC[2];
  const double* x = P.kf_state + 16 * (int64_t)k;
  jplR(x, RIM);
  double pM[3];
  mtv3(RIM, pIC, pM);
  pM[0] += x[4]; pM[1] += x[5]; pM[2] += x[6];
  const double* mg = P.mis + 8 * P.kf_mis[k];
  jplR(mg, RGM);
  mv3(RGM, pM, pG);
  pG[0] += mg[4]; pG[1] += mg[5]; pG[2] += mg[6];
}

__global__ void __launch_bounds__(kBlock) k_landmark_quality(DevProblem P, mba_landmark_quality_options o,
                                                             uint8_t* good) {
  const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (l >= P.nlm) return;
  const int64_t i0 = P.lm_obs_off[l], i1 = P.lm_obs_off[l + 1];
  if (i1 - i0 < o.min_observers || i1 == i0) { good[l] = 0; return; }
  // global position of the landmark from its store keyframe
  const int st = P.obs_store[i0];
  const double* xs = P.kf_state + 16 * (int64_t)st;
  M3<double> R;
  jplR(xs, R);
  const double* pB = P.lm_p + 4 * l;
  double pM[3], pG[3];
  mtv3(R, pB, pM);
  pM[0] += xs[4]; pM[1] += xs[5]; pM[2] += xs[6];
  const double* mg = P.mis + 8 * P.kf_mis[st];
  jplR(mg, R);
  mv3(R, pM, pG);
  pG[0] += mg[4]; pG[1] += mg[5]; pG[2] += mg[6];
  const double max_px2 = o.max_reprojection_error_px * o.max_reprojection_error_px;
  double min_sd = 1.79769313486231570e308;
  for (int64_t i = i0; i < i1; ++i) {
    double c[3], pC[3];
    camera_center_G(P, P.obs_kf[i], P.obs_cam[i], c);
    obs_point_C(P, P.kf_state, P.lm_p, i, pC);
    const double rx = c[0] - pG[0], ry = c[1] - pG[1], rz = c[2] - pG[2];
    const double d = sqrt(rx * rx + ry * ry + rz * rz);
    min_sd = fmin(min_sd, pC[2] < 0.0 ? -d : d);
    if (o.max_reprojection_error_px > 0.0) {
      double kp[2];
      project<double>(P.cams[P.obs_cam[i]], pC, kp, nullptr);
      const double2 uv = P.obs_uv[i];
      const double e2 = pC[2] > 1e-10 ? (kp[0] - uv.x) * (kp[0] - uv.x) + (kp[1] - uv.y) * (kp[1] - uv.y)
                                      : 1.79769313486231570e308;
      if (e2 > max_px2) { good[l] = 0; return; }
    }
  }
  if (min_sd > o.max_distance_from_closest_observer || min_sd < o.min_distance_from_closest_observer) {
    good[l] = 0;
    return;
  }
  double min_cos = 1.0;
  int nrays = 0;
  for (int64_t i = i0; i < i1; ++i) {
    double a[3];
    camera_center_G(P, P.obs_kf[i], P.obs_cam[i], a);
    a[0] -= pG[0]; a[1] -= pG[1]; a[2] -= pG[2];
    const double da = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (!(da > 0.0)) continue;
    ++nrays;
    for (int64_t j = i + 1; j < i1; ++j) {
      double b[3];
      camera_center_G(P, P.obs_kf[j], P.obs_cam[j], b);
      b[0] -= pG[0]; b[1] -= pG[1]; b[2] -= pG[2];
      const double db = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
      if (!(db > 0.0)) continue;
      const double dot = (a[0] / da) * (b[0] / db) + (a[1] / da) * (b[1] / db) + (a[2] / da) * (b[2] / db);
      min_cos = fmin(min_cos, fabs(dot));
    }
  }
  const double angle_deg = nrays < 2 ? 0.0 : acos(min_cos) * (180.0 / 3.14159265358979323846);
  good[l] = angle_deg < o.min_observation_angle_deg ? 0 : 1;
}

struct AmbientOut {
  double* res;
  double* J[9];
};

// Writes [A_q * 4 Jq^T * s | A_p * s] as a 2x7 row-major block.
__device__ __forceinline__ void write_pose_block(const double* Aq, const double* Ap, const double* q, double s,
                                                 double* out) {
  double Jq[12];
  dqdtheta(q, Jq);
#pragma unroll
  for (int rr = 0; rr < 2; ++rr) {
#pragma unroll
    for (int c = 0; c < 4; ++c)
      out[7 * rr + c] = (Aq[3 * rr] * 4.0 * Jq[3 * c] + Aq[3 * rr + 1] * 4.0 * Jq[3 * c + 1] + Aq[3 * rr + 2] * 4.0 * Jq[3 * c + 2]) * s;
#pragma unroll
    for (int c = 0; c < 3; ++c) out[7 * rr + 4 + c] = Ap[3 * rr + c] * s;
  }
}

// Ambient (Ceres-facing) evaluation of every observation: residual and all
// nine Jacobian blocks exactly as VisualReprojectionError::Evaluate writes
// them.  Outputs are in the caller's observation order.
__global__ void __launch_bounds__(128) k_visual_ambient(DevProblem P, AmbientOut o) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.nobs) return;
  const int64_t oi = P.obs_perm[i];
  const int lm = P.obs_lm[i], kf = P.obs_kf[i], st = P.obs_store[i], type = P.obs_type[i];
  const DevCamera& cam = P.cams[P.obs_cam[i]];
  const double sinv = P.obs_sinv[i];
  const double* pB = P.lm_p + 4 * (int64_t)lm;
  const double* xs = P.kf_state + 16 * (int64_t)st;
  const double* xo = P.kf_state + 16 * (int64_t)kf;
  const double* ml = P.mis + 8 * P.kf_mis[st];
  const double* mo = P.mis + 8 * P.kf_mis[kf];
  M3<double> RCI, RBLM, RIM, RGLM, RGM, RMG;
  jplR(cam.q_CI, RCI);
  double pI[3], pG[3] = {0, 0, 0};
  if (type == MBA_LOCAL_KEYFRAME) {
    pI[0] = pB[0]; pI[1] = pB[1]; pI[2] = pB[2];
  } else {
    jplR(xs, RBLM);
    jplR(xo, RIM);
    double pM[3];
    mtv3(RBLM, pB, pM);
    pM[0] += xs[4]; pM[1] += xs[5]; pM[2] += xs[6];
    if (type == MBA_GLOBAL) {
      jplR(ml, RGLM);
      jplR(mo, RGM);
      mv3(RGLM, pM, pG);
      pG[0] += ml[4]; pG[1] += ml[5]; pG[2] += ml[6];
      const double d[3] = {pG[0] - mo[4], pG[1] - mo[5], pG[2] - mo[6]};
      mtv3(RGM, d, pM);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) RMG.m[3 * a + b] = RGM.m[3 * b + a];
    }
    const double d[3] = {pM[0] - xo[4], pM[1] - xo[5], pM[2] - xo[6]};
    mv3(RIM, d, pI);
  }
  double pC[3];
  mv3(RCI, pI, pC);
  pC[0] += cam.p_CI[0]; pC[1] += cam.p_CI[1]; pC[2] += cam.p_CI[2];
  double kp[2], Jkp[6];
  const bool failed = project<double>(cam, pC, kp, Jkp);
  double* r = o.res ? o.res + 2 * oi : nullptr;
  if (r) {
    if (failed) { r[0] = r[1] = 0.0; }
    else { const double2 uv = P.obs_uv[i]; r[0] = (kp[0] - uv.x) * sinv; r[1] = (kp[1] - uv.y) * sinv; }
  }
  const int sz[9] = {6, 14, 14, 14, 14, 8, 6, 8, 8};
  if (failed) {
    for (int b = 0; b < 9; ++b)
      if (o.J[b]) for (int a = 0; a < sz[b]; ++a) o.J[b][sz[b] * oi + a] = 0.0;
    return;
  }
  double A[6];
  m23x33(Jkp, RCI, A);  // Jkp * R_C_I
  double JpB[6], JpMI[6] = {0}, JpLMB[6] = {0}, JpGLM[6] = {0}, JpGM[6] = {0};
  double JqBLM[6] = {0}, JqGLM[6] = {0}, JqGM[6] = {0}, JqIM[6] = {0};
  if (type == MBA_LOCAL_KEYFRAME) {
    for (int a = 0; a < 6; ++a) JpB[a] = A[a];
  } else {
    double B[6];
    m23x33(A, RIM, B);
    for (int a = 0; a < 6; ++a) JpMI[a] = -B[a];
    if (type == MBA_LOCAL_MISSION) {
      for (int a = 0; a < 6; ++a) JpLMB[a] = B[a];
    } else {
      double D[6];
      m23x33(JpMI, RMG, D);  // J_p_G_M
      for (int a = 0; a < 6; ++a) { JpGM[a] = D[a]; JpGLM[a] = -D[a]; }
      m23x33(JpGLM, RGLM, JpLMB);
      m23xskew(JpGLM, pG, JqGLM);
      m23xskew(JpGM, pG, JqGM);
    }
    for (int rr = 0; rr < 2; ++rr)
      for (int c = 0; c < 3; ++c)
        JpB[3 * rr + c] = JpLMB[3 * rr] * RBLM.m[3 * c] + JpLMB[3 * rr + 1] * RBLM.m[3 * c + 1] + JpLMB[3 * rr + 2] * RBLM.m[3 * c + 2];
    m23xskew(JpB, pB, JqBLM);
    for (int a = 0; a < 6; ++a) JqBLM[a] = -JqBLM[a];
    m23xskew(A, pI, JqIM);
  }
  if (o.J[0]) for (int a = 0; a < 6; ++a) o.J[0][6 * oi + a] = JpB[a] * sinv;
  const bool dummy_base = type == MBA_LOCAL_KEYFRAME;
  const bool dummy_mis = type != MBA_GLOBAL;
  if (o.J[1]) { if (dummy_base) for (int a = 0; a < 14; ++a) o.J[1][14 * oi + a] = 0.0; else write_pose_block(JqBLM, JpLMB, xs, sinv, o.J[1] + 14 * oi); }
  if (o.J[2]) { if (dummy_mis) for (int a = 0; a < 14; ++a) o.J[2][14 * oi + a] = 0.0; else write_pose_block(JqGLM, JpGLM, ml, sinv, o.J[2] + 14 * oi); }
  if (o.J[3]) { if (dummy_mis) for (int a = 0; a < 14; ++a) o.J[3][14 * oi + a] = 0.0; else write_pose_block(JqGM, JpGM, mo, sinv, o.J[3] + 14 * oi); }
  if (o.J[4]) { if (dummy_base) for (int a = 0; a < 14; ++a) o.J[4][14 * oi + a] = 0.0; else write_pose_block(JqIM, JpMI, xo, sinv, o.J[4] + 14 * oi); }
  if (o.J[5]) {
    double RpI[3], S[6], Jq[12];
    mv3(RCI, pI, RpI);
    // J_p_C_wrt_q_C_I = skew(R_C_I p_I); Jkp * skew(v)
    m23xskew(Jkp, RpI, S);
    dqdtheta(cam.q_CI, Jq);
    for (int rr = 0; rr < 2; ++rr)
      for (int c = 0; c < 4; ++c)
        o.J[5][8 * oi + 4 * rr + c] = (S[3 * rr] * 4.0 * Jq[3 * c] + S[3 * rr + 1] * 4.0 * Jq[3 * c + 1] + S[3 * rr + 2] * 4.0 * Jq[3 * c + 2]) * sinv;
  }
  if (o.J[6]) for (int a = 0; a < 6; ++a) o.J[6][6 * oi + a] = Jkp[a] * sinv;
  if (o.J[7] || o.J[8]) {
    // Distorted normalized point for the intrinsics Jacobian, undistorted one
    // for the distortion-parameter Jacobian (camera-pinhole.cc:98-157).
    const double un[2] = {pC[0] / pC[2], pC[1] / pC[2]};
    double dn[2] = {un[0], un[1]}, Jd[4];
    distort<double>(cam.dtype, cam.dist, dn, Jd);
    if (o.J[7]) {
      double* J = o.J[7] + 8 * oi;
      J[0] = dn[0] * sinv; J[1] = 0.0; J[2] = sinv; J[3] = 0.0;
      J[4] = 0.0; J[5] = dn[1] * sinv; J[6] = 0.0; J[7] = sinv;
    }
    if (o.J[8]) {
      double Jp[8];
      dist_param_jac(cam.dtype, cam.dist, un, Jp);
      for (int a = 0; a < 4; ++a) {
        o.J[8][8 * oi + a] = Jp[a] * cam.intr[0] * sinv;
        o.J[8][8 * oi + 4 + a] = Jp[4 + a] * cam.intr[1] * sinv;
      }
    }
  }
}

__global__ void k_convert_f32(const double* a, float* b, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

}  // namespace

cudaError_t launch_visual_ambient(const DevProblem& P, double* res, double* const* jac_dev, cudaStream_t s) {
  if (P.nobs == 0) return cudaSuccess;
  AmbientOut o;
  o.res = res;
  for (int b = 0; b < 9; ++b) o.J[b] = jac_dev ? jac_dev[b] : nullptr;
  const int64_t blocks = (P.nobs + 127) / 128;
  k_visual_ambient<<<(unsigned)blocks, 128, 0, s>>>(P, o);
  return cudaGetLastError();
}

template <typename T>
VisualInputs<T> visual_inputs(const DevProblem& P) {
  VisualInputs<T> in;
  if constexpr (sizeof(T) == 8) {
    in.uv = P.obs_uv; in.sinv = P.obs_sinv; in.huber = P.obs_huber; in.lm_p = P.lm_p;
    in.kf = P.kf_state; in.kf_stride = 16; in.mis = P.mis; in.cams = P.cams; in.kf_rot = P.kf_rot;
  } else {
    in.uv = P.obs_uv_f; in.sinv = P.obs_sinv_f; in.huber = P.obs_huber_f; in.lm_p = P.lm_p_f;
    in.kf = P.kf_pose_f; in.kf_stride = 8; in.mis = P.mis_f; in.cams = P.cams_f; in.kf_rot = nullptr;
  }
  return in;
}

// Rotation matrix R_I_M and |q|^2 of every keyframe (FP64 linearization):
// built once per keyframe instead of twice per observation.
__global__ void k_kf_rotations(const double* kf_state, int64_t nkf, double* out, const int* run_if,
                               const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nkf) return;
  const double* q = kf_state + 16 * k;
  M3<double> R;
  jplR(q, R);
  double* o = out + 16 * k;
#pragma unroll
  for (int a = 0; a < 9; ++a) o[a] = R.m[a];
  o[9] = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
}

template <typename T>
cudaError_t launch_visual_linearize_gated(const DevProblem& P, VisualLin<T> out, double* cost_accum, const int* run_if,
                                          const int* skip_if, cudaStream_t s) {
  const int64_t n = vis_end(P) - P.vis_lo;
  if (n <= 0) return cudaSuccess;
  // A chunk after the first of a chunked evaluation reuses the rotations.
  if (sizeof(T) == 8 && P.vis_lo == 0)
    k_kf_rotations<<<(unsigned)((P.nkf + 127) / 128), 128, 0, s>>>(P.kf_state, P.nkf, P.kf_rot, run_if, skip_if);
  // Block size: tuned per problem (mba_autotune), at most the launch bound.
  const int bs = (P.vis_block > 0 && P.vis_block <= kBlock) ? P.vis_block : kBlock;
  if (P.vis_pipe) {
    // Pipelined persistent variant: as many blocks as stay resident.
    int per_sm = 0, sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const bool capped = P.vis_minb == 2;
    auto kern = cost_accum ? (capped ? k_visual_linearize_pipe<T, true, 2> : k_visual_linearize_pipe<T, true, 1>)
                           : (capped ? k_visual_linearize_pipe<T, false, 2> : k_visual_linearize_pipe<T, false, 1>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, bs, 0);
    const int64_t need = (n + bs - 1) / bs;
    const int64_t grid = std::min<int64_t>(need, (int64_t)std::max(1, per_sm) * std::max(1, sms));
    kern<<<(unsigned)grid, bs, 0, s>>>(P, visual_inputs<T>(P), out, cost_accum, run_if, skip_if);
    return cudaGetLastError();
  }
  const int64_t blocks = (n + bs - 1) / bs;
  // Register caps: minb 1 none, 3 -> 85 registers, 4 -> 64 registers (more warps per SM, more spills).
  auto kern = cost_accum ? (P.vis_minb >= 4 ? k_visual_linearize<T, true, 4>
                            : P.vis_minb > 1 ? k_visual_linearize<T, true, 3> : k_visual_linearize<T, true, 1>)
                         : (P.vis_minb >= 4 ? k_visual_linearize<T, false, 4>
                            : P.vis_minb > 1 ? k_visual_linearize<T, false, 3> : k_visual_linearize<T, false, 1>);
  kern<<<(unsigned)blocks, bs, 0, s>>>(P, visual_inputs<T>(P), out, cost_accum, run_if, skip_if);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_visual_linearize(const DevProblem& P, VisualLin<T> out, double* cost_accum, cudaStream_t s) {
  return launch_visual_linearize_gated<T>(P, out, cost_accum, nullptr, nullptr, s);
}
template cudaError_t launch_visual_linearize<double>(const DevProblem&, VisualLin<double>, double*, cudaStream_t);
template cudaError_t launch_visual_linearize<float>(const DevProblem&, VisualLin<float>, double*, cudaStream_t);
template cudaError_t launch_visual_linearize_gated<double>(const DevProblem&, VisualLin<double>, double*, const int*,
                                                           const int*, cudaStream_t);
template cudaError_t launch_visual_linearize_gated<float>(const DevProblem&, VisualLin<float>, double*, const int*,
                                                          const int*, cudaStream_t);

cudaError_t launch_find_outliers(const DevProblem& P, int use_reprojection, double max_px, int* count,
                                 const int* run_if, const int* skip_if, cudaStream_t s, bool f32) {
  if (P.nobs == 0) return cudaSuccess;
  const int64_t blocks = (P.nobs + kBlock - 1) / kBlock;
  if (f32)
    k_find_outliers_f32<<<(unsigned)blocks, kBlock, 0, s>>>(P, use_reprojection, (float)(max_px * max_px), count,
                                                             run_if, skip_if);
  else
    k_find_outliers<<<(unsigned)blocks, kBlock, 0, s>>>(P, use_reprojection, max_px * max_px, count, run_if, skip_if);
  return cudaGetLastError();
}

cudaError_t launch_visual_cost_gated(const DevProblem& P, const double* kf_state, const double* lm_p,
                                     double* cost_accum, int* nonfinite, const int* skip_if, cudaStream_t s,
                                     const int* run_if) {
  if (P.nobs == 0) return cudaSuccess;
  const int64_t blocks = (P.nobs + kBlock - 1) / kBlock;
  k_visual_cost<<<(unsigned)blocks, kBlock, 0, s>>>(P, kf_state, lm_p, cost_accum, nonfinite, run_if, skip_if);
  return cudaGetLastError();
}
cudaError_t launch_visual_cost_f32(const DevProblem& P, const float* kf, const float* lm, double* cost_accum,
                                   int* nonfinite, const int* skip_if, cudaStream_t s, const int* run_if) {
  if (P.nobs == 0) return cudaSuccess;
  const int64_t blocks = (P.nobs + kBlock - 1) / kBlock;
  k_visual_cost_f32<<<(unsigned)blocks, kBlock, 0, s>>>(P, kf, lm, cost_accum, nonfinite, run_if, skip_if);
  return cudaGetLastError();
}
cudaError_t launch_visual_cost(const DevProblem& P, const double* kf_state, const double* lm_p, double* cost_accum,
                               int* nonfinite, cudaStream_t s) {
  return launch_visual_cost_gated(P, kf_state, lm_p, cost_accum, nonfinite, nullptr, s);
}

static cudaError_t launch_inertial_impl(const DevProblem& P, const double* kf_state, InertialLin<double> lin,
                                        double* amb_res, double* const* amb_jac, double* cost_accum, int* status,
                                        const int* skip_if, cudaStream_t s, bool f32 = false) {
  return launch_inertial_v2(P, kf_state, f32, lin, amb_res, amb_jac, cost_accum, status, skip_if, s);
}
cudaError_t launch_inertial(const DevProblem& P, const double* kf_state, InertialLin<double> lin, double* amb_res,
                            double* const* amb_jac, double* cost_accum, int* status, cudaStream_t s) {
  return launch_inertial_impl(P, kf_state, lin, amb_res, amb_jac, cost_accum, status, nullptr, s);
}
cudaError_t launch_inertial_gated(const DevProblem& P, const double* kf_state, InertialLin<double> lin,
                                  double* cost_accum, int* status, const int* skip_if, cudaStream_t s, bool f32,
                                  const double* sw_state) {
  cudaError_t e = launch_inertial_impl(P, kf_state, lin, nullptr, nullptr, cost_accum, status, skip_if, s, f32);
  if (e == cudaSuccess) e = launch_pose_edges(P, kf_state, sw_state, lin, cost_accum, skip_if, s);
  return e;
}

cudaError_t launch_inertial_f32(const DevProblem& P, const InertialLin<double>& src, InertialLin<float> dst,
                                cudaStream_t s) {
  if (P.nedge == 0) return cudaSuccess;
  const int64_t n1 = 15 * P.nedge, n2 = 225 * P.nedge;
  k_convert_f32<<<(unsigned)((n1 + 255) / 256), 256, 0, s>>>(src.r, dst.r, n1);
  k_convert_f32<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(src.Jf, dst.Jf, n2);
  k_convert_f32<<<(unsigned)((n2 + 255) / 256), 256, 0, s>>>(src.Jt, dst.Jt, n2);
  const int64_t n3 = 6 * (P.nedge - P.nimu);
  if (n3 > 0 && src.Js && dst.Js) k_convert_f32<<<(unsigned)((n3 + 255) / 256), 256, 0, s>>>(src.Js, dst.Js, n3);
  return cudaGetLastError();
}

namespace {
// Caller-order rows [lo, hi) of the linearization in FP64: r [N][2],
// J_l [N][6], J_s [N][12], J_o [N][12] (each may be null).  A block takes
// kGatherRows consecutive caller indices o, reads sorted index inv[o] (o
// itself when inv is null: SoA buffers already in caller order) from the SoA
// buffers, stages the rows in shared memory (component-major, conflict-free)
// and writes each array's part as one contiguous run, so that the stores
// coalesce also when the destination is page-locked host memory.
constexpr int kGatherRows = 128;
template <typename T>
__global__ void __launch_bounds__(kGatherRows) k_gather_rows(int64_t N, int64_t lo, int64_t hi, const int64_t* inv,
                                                             VisualLin<T> v, double* r, double* Jl, double* Js,
                                                             double* Jo) {
  __shared__ double sh[32 * kGatherRows];
  const int64_t base = lo + (int64_t)blockIdx.x * kGatherRows;
  const int t = threadIdx.x;
  const int cnt = (int)(hi - base < kGatherRows ? hi - base : kGatherRows);
  if (t < cnt) {
    const int64_t i = inv ? inv[base + t] : base + t;
    if (r) for (int c = 0; c < 2; ++c) sh[c * kGatherRows + t] = (double)v.r[c * N + i];
    if (Jl) for (int c = 0; c < 6; ++c) sh[(2 + c) * kGatherRows + t] = (double)v.Jl[c * N + i];
    if (Js) for (int c = 0; c < 12; ++c) sh[(8 + c) * kGatherRows + t] = (double)v.Js[c * N + i];
    if (Jo) for (int c = 0; c < 12; ++c) sh[(20 + c) * kGatherRows + t] = (double)v.Jo[c * N + i];
  }
  __syncthreads();
  double* dst[4] = {r, Jl, Js, Jo};
  const int width[4] = {2, 6, 12, 12}, first[4] = {0, 2, 8, 20};
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    if (!dst[a]) continue;
    const int w = width[a];
    double* out = dst[a] + base * w;
    for (int k = t; k < cnt * w; k += kGatherRows) out[k] = sh[(first[a] + k % w) * kGatherRows + k / w];
  }
}

__global__ void k_pack_state(int64_t NK, int64_t NL, double* kf_state, double* lm_p, float* kf_pose_f, float* lm_p_f,
                             const double* kx, const double* kv, const double* kbg, const double* kba, const double* lp,
                             const int32_t* lm_caller, int to_device) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < NK) {
    double* x = kf_state + 16 * i;
    if (to_device) {
      if (kx)
        for (int a = 0; a < 7; ++a) {
          x[a] = kx[7 * i + a];
          kf_pose_f[8 * i + a] = (float)kx[7 * i + a];
        }
      for (int a = 0; a < 3; ++a) {
        if (kv) x[7 + a] = kv[3 * i + a];
        if (kbg) x[10 + a] = kbg[3 * i + a];
        if (kba) x[13 + a] = kba[3 * i + a];
      }
    } else {
      if (kx) for (int a = 0; a < 7; ++a) const_cast<double*>(kx)[7 * i + a] = x[a];
      for (int a = 0; a < 3; ++a) {
        if (kv) const_cast<double*>(kv)[3 * i + a] = x[7 + a];
        if (kbg) const_cast<double*>(kbg)[3 * i + a] = x[10 + a];
        if (kba) const_cast<double*>(kba)[3 * i + a] = x[13 + a];
      }
    }
  } else if (i < NK + NL && lp) {
    const int64_t l = i - NK, c = lm_caller ? lm_caller[l] : l;
    for (int a = 0; a < 3; ++a) {
      if (to_device) {
        lm_p[4 * l + a] = lp[3 * c + a];
        lm_p_f[4 * l + a] = (float)lp[3 * c + a];
      } else {
        const_cast<double*>(lp)[3 * c + a] = lm_p[4 * l + a];
      }
    }
  }
}
}  // namespace

template <typename T>
cudaError_t launch_gather_visual(const DevProblem& P, const int64_t* obs_inv, VisualLin<T> v, double* r, double* Jl,
                                 double* Js, double* Jo, cudaStream_t s) {
  return launch_gather_rows<T>(P, obs_inv, 0, P.nobs, v, r, Jl, Js, Jo, s);
}

template <typename T>
cudaError_t launch_gather_rows(const DevProblem& P, const int64_t* inv, int64_t lo, int64_t hi, VisualLin<T> v,
                               double* r, double* Jl, double* Js, double* Jo, cudaStream_t s) {
  if (hi <= lo) return cudaSuccess;
  k_gather_rows<T><<<(unsigned)((hi - lo + kGatherRows - 1) / kGatherRows), kGatherRows, 0, s>>>(P.nobs, lo, hi, inv,
                                                                                                   v, r, Jl, Js, Jo);
  return cudaGetLastError();
}
template cudaError_t launch_gather_rows<double>(const DevProblem&, const int64_t*, int64_t, int64_t, VisualLin<double>,
                                                double*, double*, double*, double*, cudaStream_t);
template cudaError_t launch_gather_rows<float>(const DevProblem&, const int64_t*, int64_t, int64_t, VisualLin<float>,
                                               double*, double*, double*, double*, cudaStream_t);
template cudaError_t launch_gather_visual<double>(const DevProblem&, const int64_t*, VisualLin<double>, double*,
                                                  double*, double*, double*, cudaStream_t);
template cudaError_t launch_gather_visual<float>(const DevProblem&, const int64_t*, VisualLin<float>, double*, double*,
                                                 double*, double*, cudaStream_t);

namespace {
__global__ void k_invert_perm(int64_t N, const int64_t* perm, int64_t* inv) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < N) inv[perm[i]] = i;
}

// The FP64 linearization's observation fields in the caller's order.
__global__ void k_caller_obs(DevProblem P, const int64_t* inv, CallerObs c) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= P.nobs) return;
  const int64_t i = inv[o];
  c.uv[o] = P.obs_uv[i];
  c.sinv[o] = P.obs_sinv[i];
  c.huber[o] = P.obs_huber[i];
  c.lm[o] = P.obs_lm[i];
  c.kf[o] = P.obs_kf[i];
  c.store[o] = P.obs_store[i];
  c.cam[o] = P.obs_cam[i];
  c.type[o] = P.obs_type[i];
}
}  // namespace

cudaError_t launch_caller_obs(const DevProblem& P, const int64_t* inv, CallerObs c, cudaStream_t s) {
  if (P.nobs == 0) return cudaSuccess;
  k_caller_obs<<<(unsigned)((P.nobs + 255) / 256), 256, 0, s>>>(P, inv, c);
  return cudaGetLastError();
}

cudaError_t launch_landmark_quality(const DevProblem& P, const mba_landmark_quality_options& o, uint8_t* good,
                                    cudaStream_t s) {
  if (P.nlm == 0) return cudaSuccess;
  k_landmark_quality<<<(unsigned)((P.nlm + kBlock - 1) / kBlock), kBlock, 0, s>>>(P, o, good);
  return cudaGetLastError();
}

cudaError_t launch_invert_perm(const DevProblem& P, int64_t* inv, cudaStream_t s) {
  if (P.nobs == 0) return cudaSuccess;
  k_invert_perm<<<(unsigned)((P.nobs + 255) / 256), 256, 0, s>>>(P.nobs, P.obs_perm, inv);
  return cudaGetLastError();
}

cudaError_t launch_pack_state(const DevProblem& P, const double* kx, const double* kv, const double* kbg,
                              const double* kba, const double* lp, const int32_t* lm_caller, int to_device,
                              cudaStream_t s) {
  const int64_t n = P.nkf + P.nlm;
  k_pack_state<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P.nkf, P.nlm, P.kf_state, P.lm_p, P.kf_pose_f, P.lm_p_f,
                                                            kx, kv, kbg, kba, lp, lm_caller, to_device);
  return cudaGetLastError();
}

}  // namespace mba
