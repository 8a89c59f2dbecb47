// Camera calibration and mission baseframes as variables ("global nodes") in
// the device LM: FP64 solves only.
//
// maplab optimizes the camera intrinsics / distortion and q_C_I / p_C_I
// blocks when ba_fix_ncamera_intrinsics / ba_fix_ncamera_extrinsics_* are
// off (vi-optimization-builder.cc:24-35, optimization-terms-addition.cc:
// 203-234), and mission baseframes when they are not fixed
// (vi-optimization-builder.cc:366-371).  Ceres keeps them in the reduced
// camera system beside the keyframe poses (SPARSE_SCHUR eliminates only the
// landmarks).  Here every camera with a free block and every mission with a
// free baseframe is one 15-dim block after the keyframe blocks: its J^T J
// couplings to the keyframes (pose rows) and to the other nodes are dense,
// and the landmarks are eliminated into them like into the keyframe blocks.
// A problem has a handful of nodes, so these kernels favour simplicity
// (one thread per observation or landmark, FP64, atomics) over throughput.
//
// The node Jacobians of an observation follow VisualReprojectionError::
// Evaluate (visual-error-term-inl.h:184-377): intrinsics and distortion
// additive, q_C_I through JplQuaternionParameterization, a baseframe through
// JplPoseParameterization or JplYawOnlyPoseParameterization; Huber-corrected
// with the observation's raw residual like the other blocks.
#include <cuda_runtime.h>

#include "solver.h"

namespace mba {

namespace {

constexpr int kB = 256;

__device__ __forceinline__ double wsum_b(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void block_add_b(double v, double* acc) {
  __shared__ double red[32];
  v = wsum_b(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    v = wsum_b(v);
    if (lane == 0 && v != 0.0) atomicAdd(acc, v);
  }
}

inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }
inline unsigned gridcap(int64_t n) { return (unsigned)(n <= 0 ? 1 : (n + kB - 1) / kB > 4096 ? 4096 : (n + kB - 1) / kB); }

// Tangent rows (2 x k) of an ambient quaternion block A_q * 4 Jq(q)^T (the
// error term's lift), times the parameterization Jacobian: P = Jq (4 x 3)
// for JplQuaternionParameterization, the yaw column (4 x 1) for
// JplYawQuaternionParameterization.
__device__ __forceinline__ void quat_tangent(const double* Aq, const double* q, bool yaw, double s, double* out,
                                             int stride) {
  double Jq[12];
  dqdtheta(q, Jq);
  double amb[8];  // A_q * 4 Jq^T, 2 x 4
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 4; ++c)
      amb[4 * r + c] = (Aq[3 * r] * 4.0 * Jq[3 * c] + Aq[3 * r + 1] * 4.0 * Jq[3 * c + 1] +
                        Aq[3 * r + 2] * 4.0 * Jq[3 * c + 2]) * s;
  if (yaw) {
    double Jy[4];
    dqdyaw(q, Jy);
    for (int r = 0; r < 2; ++r)
      out[stride * r] = amb[4 * r] * Jy[0] + amb[4 * r + 1] * Jy[1] + amb[4 * r + 2] * Jy[2] + amb[4 * r + 3] * Jy[3];
  } else {
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 3; ++c)
        out[stride * r + c] = amb[4 * r] * Jq[c] + amb[4 * r + 1] * Jq[3 + c] + amb[4 * r + 2] * Jq[6 + c] +
                              amb[4 * r + 3] * Jq[9 + c];
  }
}

}  // namespace

// Robustified tangent Jacobians of observation i (sorted index) with respect
// to its global nodes, at the state (kf, lm, cams, mis): node ids (g) in nid
// and 2 x 15 rows in Jn (masked dims zero).  Returns the node count (0 for a
// failed projection or a rejected landmark).
__device__ int obs_node_jacobians(const DevProblem& P, const DevCamera* cams, const double* mis,
                                  const double* kf_state, const double* lm_p, int64_t i, int32_t* nid,
                                  double (*Jn)[30]) {
  const int cam_i = P.obs_cam[i];
  const int lm = P.obs_lm[i], kf = P.obs_kf[i], st = P.obs_store[i], type = P.obs_type[i];
  const int gc = P.cam_node[cam_i];
  const int gl = type == MBA_GLOBAL ? P.mis_node[P.kf_mis[st]] : -1;
  const int go = type == MBA_GLOBAL ? P.mis_node[P.kf_mis[kf]] : -1;
  if (gc < 0 && gl < 0 && go < 0) return 0;
  if (P.lm_off[lm]) return 0;
  const DevCamera& cam = cams[cam_i];
  const double sinv = P.obs_sinv[i];
  const double* pB = lm_p + 4 * (int64_t)lm;
  const double* xs = kf_state + 16 * (int64_t)st;
  const double* xo = kf_state + 16 * (int64_t)kf;
  const double* ml = mis + 8 * P.kf_mis[st];
  const double* mo = mis + 8 * P.kf_mis[kf];
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
  if (project<double>(cam, pC, kp, Jkp)) return 0;
  const double2 uv = P.obs_uv[i];
  const double r[2] = {(kp[0] - uv.x) * sinv, (kp[1] - uv.y) * sinv};
  int n = 0;
  if (gc >= 0) {
    const uint16_t m = P.g_mask[gc];
    double* J = Jn[n];
    for (int a = 0; a < 30; ++a) J[a] = 0.0;
    // intrinsics at the distorted normalized point, distortion parameters at
    // the undistorted one (camera-pinhole.cc:98-157)
    const double un[2] = {pC[0] / pC[2], pC[1] / pC[2]};
    double dn[2] = {un[0], un[1]}, Jd[4];
    distort<double>(cam.dtype, cam.dist, dn, Jd);
    const double Ji[8] = {dn[0], 0.0, 1.0, 0.0, 0.0, dn[1], 0.0, 1.0};
    double Jp[8];
    dist_param_jac(cam.dtype, cam.dist, un, Jp);
    double RpI[3], S[6];
    mv3(RCI, pI, RpI);
    m23xskew(Jkp, RpI, S);  // J_p_C / J_q_C_I before the lift
    double Jth[6];
    quat_tangent(S, cam.q_CI, false, sinv, Jth, 3);
    for (int rr = 0; rr < 2; ++rr) {
      for (int a = 0; a < 4; ++a) {
        J[15 * rr + a] = ((m >> a) & 1) ? Ji[4 * rr + a] * sinv : 0.0;
        J[15 * rr + 4 + a] = ((m >> (4 + a)) & 1) ? Jp[4 * rr + a] * cam.intr[rr] * sinv : 0.0;
      }
      for (int a = 0; a < 3; ++a) {
        J[15 * rr + 8 + a] = ((m >> (8 + a)) & 1) ? Jth[3 * rr + a] : 0.0;
        J[15 * rr + 11 + a] = ((m >> (11 + a)) & 1) ? Jkp[3 * rr + a] * sinv : 0.0;
      }
    }
    nid[n++] = gc;
  }
  if (gl >= 0 || go >= 0) {
    // kGlobal chain (visual-error-term-inl.h:196-226): J_p_G_M = -J_p_M_I R_M_G,
    // landmark baseframe = -J_p_G_M, rotations through skew(p_G).
    double A[6], B[6], JpMI[6], JpGM[6], JpGLM[6], JqGLM[6], JqGM[6];
    m23x33(Jkp, RCI, A);
    m23x33(A, RIM, B);
    for (int a = 0; a < 6; ++a) JpMI[a] = -B[a];
    m23x33(JpMI, RMG, JpGM);
    for (int a = 0; a < 6; ++a) JpGLM[a] = -JpGM[a];
    m23xskew(JpGLM, pG, JqGLM);
    m23xskew(JpGM, pG, JqGM);
    const int ids[2] = {gl, go};
    const double* Aq[2] = {JqGLM, JqGM};
    const double* Ap[2] = {JpGLM, JpGM};
    const double* q[2] = {ml, mo};
    const int mi[2] = {P.kf_mis[st], P.kf_mis[kf]};
    for (int s = 0; s < 2; ++s) {
      if (ids[s] < 0) continue;
      double* J = Jn[n];
      for (int a = 0; a < 30; ++a) J[a] = 0.0;
      const uint16_t m = P.g_mask[ids[s]];
      const bool yaw = P.mis_flags[mi[s]] == MBA_MIS_BASEFRAME_YAW_POSITION;
      quat_tangent(Aq[s], q[s], yaw, sinv, J, 15);
      for (int rr = 0; rr < 2; ++rr) {
        for (int a = 0; a < 3; ++a) if (!((m >> a) & 1)) J[15 * rr + a] = 0.0;
        for (int a = 0; a < 3; ++a) J[15 * rr + 3 + a] = ((m >> (3 + a)) & 1) ? Ap[s][3 * rr + a] * sinv : 0.0;
      }
      nid[n++] = ids[s];
    }
  }
  const double ha = P.obs_huber[i];
  if (ha > 0.0) {
    double rho0, sq1, rs, as;
    huber_corrector<double>(ha, r[0] * r[0] + r[1] * r[1], &rho0, &sq1, &rs, &as);
    for (int b = 0; b < n; ++b)
      for (int c = 0; c < 15; ++c) {
        const double t = r[0] * Jn[b][c] + r[1] * Jn[b][15 + c];
        Jn[b][c] = sq1 * (Jn[b][c] - as * r[0] * t);
        Jn[b][15 + c] = sq1 * (Jn[b][15 + c] - as * r[1] * t);
      }
  }
  return n;
}

namespace {

// Direct J^T J and J^T r terms of the observations on the nodes (unscaled):
// node-node, keyframe-node (store and observer pose rows), node gradient.
// vis holds the corrected residual and tangent pose Jacobians of the same
// linearization.
__global__ void __launch_bounds__(kB) k_border_assemble(DevProblem P, VisualLin<double> vis, BorderSystem B,
                                                        const int* run_if, const int* skip_if) {
  if ((skip_if && *skip_if) || (run_if && !*run_if)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.nobs) return;
  int32_t nid[3];
  double Jn[3][30];
  const int n = obs_node_jacobians(P, P.cams, P.mis, P.kf_state, P.lm_p, i, nid, Jn);
  if (n == 0) return;
  const int64_t N = P.nobs, G = P.ng;
  const double r0 = vis.r[i], r1 = vis.r[N + i];
  for (int a = 0; a < n; ++a) {
    for (int c = 0; c < 15; ++c) {
      const double g = Jn[a][c] * r0 + Jn[a][15 + c] * r1;
      if (g != 0.0) atomicAdd(&B.gg[15 * nid[a] + c], g);
    }
    for (int b = 0; b < n; ++b) {
      double* blk = B.Gb + 225 * (G * nid[a] + nid[b]);
      for (int rr = 0; rr < 15; ++rr)
        for (int c = 0; c < 15; ++c) {
          const double v = Jn[a][rr] * Jn[b][c] + Jn[a][15 + rr] * Jn[b][15 + c];
          if (v != 0.0) atomicAdd(&blk[15 * rr + c], v);
        }
    }
  }
  if (P.obs_type[i] == MBA_LOCAL_KEYFRAME) return;
  const int64_t ks = P.obs_store[i], ko = P.obs_kf[i];
  for (int s = 0; s < 2; ++s) {
    const int64_t k = s == 0 ? ks : ko;
    const double* Jk = s == 0 ? vis.Js : vis.Jo;
    double Jp[12];
    for (int a = 0; a < 12; ++a) Jp[a] = Jk[a * N + i];
    for (int a = 0; a < n; ++a) {
      double* blk = B.Bb + 90 * (G * k + nid[a]);
      for (int rr = 0; rr < 6; ++rr)
        for (int c = 0; c < 15; ++c) {
          const double v = Jp[rr] * Jn[a][c] + Jp[6 + rr] * Jn[a][15 + c];
          if (v != 0.0) atomicAdd(&blk[15 * rr + c], v);
        }
    }
  }
}

// Jacobi scale of the node dims from the unscaled diagonal (first
// linearization only), into the tails of the FP64 and T scale vectors.
__global__ void k_border_scale(DevProblem P, BorderSystem B, double* skf, double* skf_t, int jacobi,
                               const int* run_if) {
  if (run_if && !*run_if) return;
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= 15 * P.ng) return;
  const int64_t g = j / 15, d = j % 15;
  const double h = B.Gb[225 * (P.ng * g + g) + 16 * d];
  const double s = jacobi ? 1.0 / (1.0 + sqrt(h > 0.0 ? h : 0.0)) : 1.0;
  skf[15 * P.nkf + j] = s;
  skf_t[15 * P.nkf + j] = s;
}

// Scaled, damped node blocks and right-hand side: GS = s Gb s + diag,
// BS = s_kf Bb s_n, rhs_n = -s gg.
__global__ void __launch_bounds__(kB) k_border_build(SolverLaunch<double> s) {
  if (s.ctl->terminated) return;
  const int64_t G = s.P.ng, NK = s.P.nkf;
  const double* sk = s.sc.skf;
  const double* sn = s.sc.skf + 15 * NK;
  const double radius = s.ctl->radius, mn = s.prm.min_lm_diagonal, mx = s.prm.max_lm_diagonal;
  const int64_t n1 = G * G * 225, n2 = n1 + NK * G * 90, n3 = n2 + 15 * G;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n1) {
      const int64_t blk = i / 225, e = i % 225, a = blk / G, b = blk % G, r = e / 15, c = e % 15;
      double v = s.B.Gb[i] * sn[15 * a + r] * sn[15 * b + c];
      if (a == b && r == c) {
        const double d = v < mn ? mn : (v > mx ? mx : v);
        v += d / radius;
      }
      s.B.GS[i] = v;
    } else if (i < n2) {
      const int64_t j = i - n1, k = j / (90 * G), g = (j / 90) % G, e = j % 90, r = e / 15, c = e % 15;
      s.B.BS[j] = s.B.Bb[j] * sk[15 * k + r] * sn[15 * g + c];
    } else {
      const int64_t j = i - n2;
      s.L.rhs[15 * NK + j] = -s.B.gg[j] * sn[j];
    }
  }
}

// Landmark elimination into the node blocks (after V and U = V W are
// known): GS(a, b) -= W_a^T V W_b, BS(k_slot, a) -= U_slot^T W_a,
// rhs_a += W_a^T V g_l, with W_a = sum over the landmark's observations of
// J_l^T J_a (scaled).  One thread per landmark.
constexpr int kMaxLmNodes = 8;

__device__ int landmark_node_W(const SolverLaunch<double>& s, int64_t l, int32_t* ids, double (*W)[45]) {
  const int64_t N = s.P.nobs, NL = s.P.nlm, NK = s.P.nkf;
  const double* sn = s.sc.skf + 15 * NK;
  int nn = 0;
  for (int64_t i = s.P.lm_obs_off[l]; i < s.P.lm_obs_off[l + 1]; ++i) {
    int32_t nid[3];
    double Jn[3][30];
    const int n = obs_node_jacobians(s.P, s.P.cams, s.P.mis, s.P.kf_state, s.P.lm_p, i, nid, Jn);
    double Jl[6];
    for (int a = 0; a < 6; ++a) Jl[a] = s.vis.Jl[a * N + i];
    for (int b = 0; b < n; ++b) {
      int pos = -1;
      for (int q = 0; q < nn; ++q) if (ids[q] == nid[b]) pos = q;
      if (pos < 0) {
        if (nn == kMaxLmNodes) { atomicExch(&s.ctl->status, (int)MBA_ERR_INVALID_ARG); return -1; }
        pos = nn++;
        ids[pos] = nid[b];
        for (int a = 0; a < 45; ++a) W[pos][a] = 0.0;
      }
      for (int x = 0; x < 3; ++x)
        for (int c = 0; c < 15; ++c)
          W[pos][15 * x + c] += (Jl[x] * Jn[b][c] + Jl[3 + x] * Jn[b][15 + c]) * s.sc.slm[x * NL + l] *
                                sn[15 * nid[b] + c];
    }
  }
  return nn;
}

__global__ void __launch_bounds__(64) k_border_schur(SolverLaunch<double> s) {
  if (s.ctl->terminated) return;
  const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (l >= s.P.nlm || !s.P.lm_active[l] || s.P.lm_off[l]) return;
  int32_t ids[kMaxLmNodes];
  double W[kMaxLmNodes][45];
  const int nn = landmark_node_W(s, l, ids, W);
  if (nn <= 0) return;
  const int64_t NL = s.P.nlm, G = s.P.ng, NK = s.P.nkf;
  double V[9];
  for (int a = 0; a < 9; ++a) V[a] = s.L.V[a * NL + l];
  const double g[3] = {s.L.gl[l], s.L.gl[NL + l], s.L.gl[2 * NL + l]};
  double Vg[3];
  for (int x = 0; x < 3; ++x) Vg[x] = V[3 * x] * g[0] + V[3 * x + 1] * g[1] + V[3 * x + 2] * g[2];
  for (int b = 0; b < nn; ++b) {
    double VW[45];
    for (int x = 0; x < 3; ++x)
      for (int c = 0; c < 15; ++c)
        VW[15 * x + c] = V[3 * x] * W[b][c] + V[3 * x + 1] * W[b][15 + c] + V[3 * x + 2] * W[b][30 + c];
    for (int c = 0; c < 15; ++c) {
      const double v = W[b][c] * Vg[0] + W[b][15 + c] * Vg[1] + W[b][30 + c] * Vg[2];
      if (v != 0.0) atomicAdd(&s.L.rhs[15 * (NK + ids[b]) + c], v);
    }
    for (int a = 0; a < nn; ++a) {
      double* blk = s.B.GS + 225 * (G * ids[a] + ids[b]);
      for (int r = 0; r < 15; ++r)
        for (int c = 0; c < 15; ++c) {
          const double v = W[a][r] * VW[c] + W[a][15 + r] * VW[15 + c] + W[a][30 + r] * VW[30 + c];
          if (v != 0.0) atomicAdd(&blk[15 * r + c], -v);
        }
    }
    for (int64_t sl = s.S.lm_slot_off[l]; sl < s.S.lm_slot_end[l]; ++sl) {
      const int64_t k = s.S.slot_kf[sl];
      const double* U = s.L.U + kSlotStride * (int64_t)s.S.w_u[sl];  // V W_slot, 3 x 6
      double* blk = s.B.BS + 90 * (G * k + ids[b]);
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 15; ++c) {
          const double v = U[r] * W[b][c] + U[6 + r] * W[b][15 + c] + U[12 + r] * W[b][30 + c];
          if (v != 0.0) atomicAdd(&blk[15 * r + c], -v);
        }
    }
  }
}

// Masked node dims: identity rows in the diagonal blocks, zero elsewhere and
// in the right-hand side; masked keyframe dims zero in BS.  The diagonal node
// blocks go to SD (block-Jacobi inverse with the keyframe blocks).
__global__ void __launch_bounds__(kB) k_border_finalize(SolverLaunch<double> s) {
  if (s.ctl->terminated) return;
  const int64_t G = s.P.ng, NK = s.P.nkf;
  const int64_t n1 = G * G * 225, n2 = n1 + NK * G * 90, n3 = n2 + 15 * G;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n1) {
      const int64_t blk = i / 225, e = i % 225, a = blk / G, b = blk % G, r = e / 15, c = e % 15;
      double v = s.B.GS[i];
      if (!((s.P.g_mask[a] >> r) & 1) || !((s.P.g_mask[b] >> c) & 1)) v = (a == b && r == c) ? 1.0 : 0.0;
      s.B.GS[i] = v;
      if (a == b) s.L.SD[225 * (NK + a) + e] = v;
    } else if (i < n2) {
      const int64_t j = i - n1, k = j / (90 * G), g = (j / 90) % G, e = j % 90, r = e / 15, c = e % 15;
      if (!((s.P.kf_mask[k] >> r) & 1) || !((s.P.g_mask[g] >> c) & 1)) s.B.BS[j] = 0.0;
    } else {
      const int64_t j = i - n2, g = j / 15, d = j % 15;
      if (!((s.P.g_mask[g] >> d) & 1)) s.L.rhs[15 * NK + j] = 0.0;
    }
  }
}

// PCG product for the node rows: p_new = z + beta p_old on the node rows,
// q_n = sum_k BS(k, n)^T p_new_k + sum_m GS(n, m) p_new_m, pq += p_new.q.
// Runs after k_pcg_spmv (which wrote p_new of the keyframe rows to pb).
// One block per node.
__global__ void __launch_bounds__(128) k_border_spmv(SolverLaunch<double> s, int it, const double* pa, double* pb) {
  LmControl* ctl = s.ctl;
  if (ctl->terminated || ctl->pcg_done || ctl->status || !(ctl->pcg_bnorm2 > 0.0)) return;
  double beta = 0.0;
  if (it > 0) {
    const double rzprev = (it == 1) ? ctl->pcg_rz0 : ctl->pcg_rz[(it + 1) % 3];
    beta = ctl->pcg_rz[(it - 1) % 3] / rzprev;
  }
  const int64_t g = blockIdx.x, G = s.P.ng, NK = s.P.nkf;
  double acc[15];
  for (int c = 0; c < 15; ++c) acc[c] = 0.0;
  for (int64_t k = threadIdx.x; k < NK; k += blockDim.x) {
    const double* B = s.B.BS + 90 * (G * k + g);
    const double* pk = pb + 15 * k;
    for (int r = 0; r < 6; ++r) {
      const double pr = pk[r];
      if (pr == 0.0) continue;
      for (int c = 0; c < 15; ++c) acc[c] += B[15 * r + c] * pr;
    }
  }
  __shared__ double red[15][128];
  for (int c = 0; c < 15; ++c) red[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 15; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  double pq = 0.0;
  if (threadIdx.x < 15) {
    const int c = threadIdx.x;
    double y = red[c][0];
    for (int64_t m = 0; m < G; ++m) {
      const double* Gm = s.B.GS + 225 * (G * g + m);
      const double* zm = s.L.z + 15 * (NK + m);
      const double* pm = pa + 15 * (NK + m);
      for (int d = 0; d < 15; ++d) y += Gm[15 * c + d] * (zm[d] + beta * pm[d]);
    }
    const int64_t row = 15 * (NK + g) + c;
    const double p_new = s.L.z[row] + beta * pa[row];
    pb[row] = p_new;
    s.L.q[row] = y;
    pq = y * p_new;
  }
  if (threadIdx.x < 32) {
    pq = wsum_b(pq);
    if (threadIdx.x == 0 && pq != 0.0) atomicAdd(&ctl->pcg_pq[it % 3], pq);
  }
}

// Back substitution, node part: bl = sum_a W_a^T x_a per landmark (scaled),
// subtracted from -g_l by k_backsub.
__global__ void __launch_bounds__(64) k_border_backsub(SolverLaunch<double> s) {
  if (s.ctl->terminated) return;
  const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t NL = s.P.nlm, NK = s.P.nkf;
  if (l >= NL) return;
  double t[3] = {0.0, 0.0, 0.0};
  if (s.P.lm_active[l] && !s.P.lm_off[l]) {
    int32_t ids[kMaxLmNodes];
    double W[kMaxLmNodes][45];
    const int nn = landmark_node_W(s, l, ids, W);
    for (int b = 0; b < nn; ++b) {
      const double* x = s.L.x + 15 * (NK + ids[b]);
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 15; ++c) t[a] += W[b][15 * a + c] * x[c];
    }
  }
  for (int a = 0; a < 3; ++a) s.B.bl[a * NL + l] = t[a];
}

// Model cost change of the visual terms with the node columns:
// -u.(r + u/2), u = J_l dl + J_s dx_s + J_o dx_o + sum_n J_n dx_n (unscaled J,
// unscaled step).  Replaces k_model_visual when the problem has nodes.
__global__ void __launch_bounds__(kB) k_model_visual_nodes(SolverLaunch<double> s) {
  if (s.ctl->terminated) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t N = s.P.nobs, NL = s.P.nlm, NK = s.P.nkf;
  double m = 0.0;
  if (i < N) {
    const int64_t l = s.P.obs_lm[i];
    double u[2] = {0.0, 0.0};
    for (int rr = 0; rr < 2; ++rr)
      for (int a = 0; a < 3; ++a) u[rr] += s.vis.Jl[(3 * rr + a) * N + i] * s.sc.slm[a * NL + l] * s.L.dl[a * NL + l];
    if (s.P.obs_type[i] != MBA_LOCAL_KEYFRAME) {
      const int64_t ks = s.P.obs_store[i], ko = s.P.obs_kf[i];
      for (int rr = 0; rr < 2; ++rr)
        for (int c = 0; c < 6; ++c)
          u[rr] += s.vis.Js[(6 * rr + c) * N + i] * s.sc.skf[15 * ks + c] * s.L.x[15 * ks + c] +
                   s.vis.Jo[(6 * rr + c) * N + i] * s.sc.skf[15 * ko + c] * s.L.x[15 * ko + c];
    }
    int32_t nid[3];
    double Jn[3][30];
    const int n = obs_node_jacobians(s.P, s.P.cams, s.P.mis, s.P.kf_state, s.P.lm_p, i, nid, Jn);
    for (int b = 0; b < n; ++b) {
      const int64_t row = 15 * (NK + nid[b]);
      for (int rr = 0; rr < 2; ++rr)
        for (int c = 0; c < 15; ++c) u[rr] += Jn[b][15 * rr + c] * s.sc.skf[row + c] * s.L.x[row + c];
    }
    m = -(u[0] * (s.vis.r[i] + u[0] / 2.0) + u[1] * (s.vis.r[N + i] + u[1] / 2.0));
  }
  block_add_b(m, &s.ctl->model_change);
}

// Retraction of the nodes into the candidate cameras / baseframes, with the
// step and state norms of their blocks (ambient, as Ceres measures them).
__global__ void k_border_retract(SolverLaunch<double> s) {
  if (s.ctl->terminated) return;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= s.P.ng) return;
  const int64_t row = 15 * (s.P.nkf + g);
  const uint16_t m = s.P.g_mask[g];
  double d[15];
  for (int a = 0; a < 15; ++a) d[a] = ((m >> a) & 1) ? s.sc.skf[row + a] * s.L.x[row + a] : 0.0;
  double sn = 0.0, xn = 0.0;
  auto acc = [&](const double* now, const double* old, int n) {
    for (int a = 0; a < n; ++a) { sn += (now[a] - old[a]) * (now[a] - old[a]); xn += old[a] * old[a]; }
  };
  if (s.P.node_cam[g] >= 0) {
    const int c = s.P.node_cam[g];
    const DevCamera& o = s.P.cams[c];
    DevCamera& n = s.B.cams_cand[c];
    n = o;
    for (int a = 0; a < 4; ++a) {
      if ((m >> a) & 1) n.intr[a] = o.intr[a] + d[a];
      if ((m >> (4 + a)) & 1) n.dist[a] = o.dist[a] + d[4 + a];
    }
    if ((m >> 8) & 7) jpl_plus(o.q_CI, d + 8, n.q_CI);
    for (int a = 0; a < 3; ++a) if ((m >> (11 + a)) & 1) n.p_CI[a] = o.p_CI[a] + d[11 + a];
    if (m & 0xf) acc(n.intr, o.intr, 4);
    if ((m >> 4) & 0xf) {
      int nd = 0;
      for (int a = 0; a < 4; ++a) nd += (m >> (4 + a)) & 1;
      acc(n.dist, o.dist, nd);
    }
    if ((m >> 8) & 7) acc(n.q_CI, o.q_CI, 4);
    if ((m >> 11) & 7) acc(n.p_CI, o.p_CI, 3);
  } else {
    const int mi = s.P.node_mis[g];
    const double* o = s.P.mis + 8 * mi;
    double* n = s.B.mis_cand + 8 * mi;
    if (s.P.mis_flags[mi] == MBA_MIS_BASEFRAME_YAW_POSITION) jpl_yaw_plus(o, d, n);
    else jpl_plus(o, d, n);
    for (int a = 0; a < 3; ++a) n[4 + a] = o[4 + a] + d[3 + a];
    n[7] = 0.0;
    acc(n, o, 7);
  }
  atomicAdd(&s.ctl->step_norm2, sn);
  atomicAdd(&s.ctl->x_norm2, xn);
}

// Accepted step: the candidate cameras / baseframes become current.
__global__ void k_border_accept(SolverLaunch<double> s) {
  if (!s.ctl->accepted) return;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= s.P.ng) return;
  if (s.P.node_cam[g] >= 0) {
    const int c = s.P.node_cam[g];
    const_cast<DevCamera*>(s.P.cams)[c] = s.B.cams_cand[c];
  } else {
    const int mi = s.P.node_mis[g];
    for (int a = 0; a < 8; ++a) const_cast<double*>(s.P.mis)[8 * mi + a] = s.B.mis_cand[8 * mi + a];
  }
}

}  // namespace

// ---- launchers (called by the solver for problems with nodes, FP64)
cudaError_t border_zero(const SolverLaunch<double>& s, const int* run_if, const int* skip_if, cudaStream_t st);
cudaError_t border_assemble(const SolverLaunch<double>& s, const int* run_if, const int* skip_if, cudaStream_t st) {
  cudaError_t e = border_zero(s, run_if, skip_if, st);
  if (e != cudaSuccess) return e;
  if (s.P.nobs) k_border_assemble<<<nblk(s.P.nobs, kB), kB, 0, st>>>(s.P, s.vis, s.B, run_if, skip_if);
  return cudaGetLastError();
}

namespace {
__global__ void k_border_zero(BorderSystem B, int64_t n_g, int64_t n_b, int64_t n_gg, const int* run_if,
                              const int* skip_if) {
  if ((skip_if && *skip_if) || (run_if && !*run_if)) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_g + n_b + n_gg;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n_g) B.Gb[i] = 0.0;
    else if (i < n_g + n_b) B.Bb[i - n_g] = 0.0;
    else B.gg[i - n_g - n_b] = 0.0;
  }
}
}  // namespace

cudaError_t border_zero(const SolverLaunch<double>& s, const int* run_if, const int* skip_if, cudaStream_t st) {
  const int64_t G = s.P.ng, n_g = 225 * G * G, n_b = 90 * s.P.nkf * G, n_gg = 15 * G;
  k_border_zero<<<gridcap(n_g + n_b + n_gg), kB, 0, st>>>(s.B, n_g, n_b, n_gg, run_if, skip_if);
  return cudaGetLastError();
}

cudaError_t border_scale(const SolverLaunch<double>& s, int jacobi, const int* run_if, cudaStream_t st) {
  k_border_scale<<<nblk(15 * s.P.ng, kB), kB, 0, st>>>(s.P, s.B, s.sc.skf, s.L.skf, jacobi, run_if);
  return cudaGetLastError();
}

cudaError_t border_build(const SolverLaunch<double>& s, cudaStream_t st) {
  const int64_t G = s.P.ng;
  k_border_build<<<gridcap(225 * G * G + 90 * s.P.nkf * G + 15 * G), kB, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t border_schur_and_finalize(const SolverLaunch<double>& s, cudaStream_t st) {
  const int64_t G = s.P.ng;
  if (s.P.nlm) k_border_schur<<<nblk(s.P.nlm, 64), 64, 0, st>>>(s);
  k_border_finalize<<<gridcap(225 * G * G + 90 * s.P.nkf * G + 15 * G), kB, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t border_spmv(const SolverLaunch<double>& s, int it, const double* pa, double* pb, cudaStream_t st) {
  k_border_spmv<<<(unsigned)s.P.ng, 128, 0, st>>>(s, it, pa, pb);
  return cudaGetLastError();
}

cudaError_t border_backsub(const SolverLaunch<double>& s, cudaStream_t st) {
  if (s.P.nlm) k_border_backsub<<<nblk(s.P.nlm, 64), 64, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t border_model_visual(const SolverLaunch<double>& s, cudaStream_t st) {
  if (s.P.nobs) k_model_visual_nodes<<<nblk(s.P.nobs, kB), kB, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t border_retract(const SolverLaunch<double>& s, cudaStream_t st) {
  k_border_retract<<<nblk(s.P.ng, 64), 64, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t border_accept(const SolverLaunch<double>& s, cudaStream_t st) {
  k_border_accept<<<nblk(s.P.ng, 64), 64, 0, st>>>(s);
  return cudaGetLastError();
}

}  // namespace mba
