// Device-resident Levenberg-Marquardt with Schur elimination of the
// landmarks and block-Jacobi PCG on the reduced camera system.
//
// Restates the solver behaviour maplab configures in
// algorithms/map-optimization/include/map-optimization/solver-options.h:26-75
// (Ceres trust-region LM, Jacobi scaling, SPARSE_SCHUR / ITERATIVE_SCHUR
// linear solvers): Jacobi scaling s = 1 / (1 + sqrt(diag(J^T J))) from the
// first Jacobian, LM diagonal clamp(diag, 1e-6, 1e32) / radius, model cost
// change -J d . (r + J d / 2), step acceptance at relative decrease > 1e-3,
// radius update radius / max(1/3, 1 - (2 rho - 1)^3) on success and
// radius / 2^k on failure.  Every per-iteration decision runs on the device
// (one thread), so an LM iteration is a fixed kernel sequence that is
// captured once as a CUDA graph.
#include <cuda_runtime.h>

#include "solver.h"

namespace mba {

namespace {

constexpr int kB = 256;

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void block_add(double v, double* acc) {
  __shared__ double red[32];
  v = wsum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    v = wsum(v);
    if (lane == 0 && v != 0.0) atomicAdd(acc, v);
  }
}

__device__ __forceinline__ bool gated(const int* run_if, const int* skip_if) {
  if (skip_if && *skip_if) return true;
  if (run_if && !*run_if) return true;
  return false;
}

template <typename T>
__device__ __forceinline__ void atomic_add(T* a, T v) {
  atomicAdd(a, v);
}

// Loads the 18 values of one slot (slot-major W or U rows, kSlotStride apart).
__device__ __forceinline__ void load_slot(const float* p, float* v) {
  const float4* q = reinterpret_cast<const float4*>(p);  // 80-byte rows: 16-byte aligned
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 t = q[i];
    v[4 * i] = t.x;
    v[4 * i + 1] = t.y;
    v[4 * i + 2] = t.z;
    v[4 * i + 3] = t.w;
  }
  const float2 t = reinterpret_cast<const float2*>(p)[8];
  v[16] = t.x;
  v[17] = t.y;
}
// Vector stores of one slot row (18 values of a 20-value row).
__device__ __forceinline__ void store_slot(float* p, const float* v) {
  float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
  for (int i = 0; i < 4; ++i) q[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
  reinterpret_cast<float2*>(p)[8] = make_float2(v[16], v[17]);
}
__device__ __forceinline__ void store_slot(double* p, const double* v) {
  double2* q = reinterpret_cast<double2*>(p);
#pragma unroll
  for (int i = 0; i < 9; ++i) q[i] = make_double2(v[2 * i], v[2 * i + 1]);
}

__device__ __forceinline__ void load_slot(const double* p, double* v) {
  const double2* q = reinterpret_cast<const double2*>(p);  // 160-byte rows: 16-byte aligned
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const double2 t = q[i];
    v[2 * i] = t.x;
    v[2 * i + 1] = t.y;
  }
}

// ------------------------------------------------------------ assembly
template <typename T>
__global__ void __launch_bounds__(kB) k_zero(T* a, int64_t n, const int* run_if, const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = T(0);
}

// Upper triangle of a symmetric 6x6 block, row by row: entry t (< 21) is
// (up_row(t), up_col(t)); kPoseUp = 24 floats per keyframe (21 + 3 pad, six
// float4).
constexpr int kPoseUp = 24;
__host__ __device__ constexpr int up_row(int t) { return t < 6 ? 0 : t < 11 ? 1 : t < 15 ? 2 : t < 18 ? 3 : t < 20 ? 4 : 5; }
__host__ __device__ constexpr int up_col(int t) {
  return t < 6 ? t : t < 11 ? t - 5 : t < 15 ? t - 9 : t < 18 ? t - 12 : t < 20 ? t - 14 : t - 15;
}

// One thread per landmark: H_ll, g_l, slot blocks W and the direct
// camera-camera terms of its observations.  The keyframes' 6x6 pose blocks of
// D are symmetric: only their upper triangle is accumulated here (and by the
// inertial assembly); k_mirror_pose_blocks fills the lower one afterwards.
// scaled != 0 (re-linearizations inside the LM loop, whose Jacobi scale is
// fixed): the Jacobian columns are multiplied by the scale as they are read,
// so the assembled blocks come out scaled (no separate scaling pass).
template <typename T>
__global__ void __launch_bounds__(kB, sizeof(T) == 4 ? 2 : 1) k_assemble_lm(DevProblem P, SchurPattern S, VisualLin<T> v,
                                                                            LinearSystem<T> L,
                                                    int scaled, const int* run_if, const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (l >= P.nlm) return;
  const int64_t N = P.nobs, NL = P.nlm;
  const int64_t s0 = S.lm_slot_off[l];
  const int st = S.slot_kf[s0];
  T sl[3], ss[6];
#pragma unroll
  for (int a = 0; a < 3; ++a) sl[a] = scaled ? L.slm[a * NL + l] : T(1);
#pragma unroll
  for (int a = 0; a < 6; ++a) ss[a] = scaled ? L.skf[15 * (int64_t)st + a] : T(1);
  T H[9], g[3], Wst[18], Dst[36], gst[6];
#pragma unroll
  for (int a = 0; a < 9; ++a) H[a] = T(0);
#pragma unroll
  for (int a = 0; a < 3; ++a) g[a] = T(0);
#pragma unroll
  for (int a = 0; a < 18; ++a) Wst[a] = T(0);
#pragma unroll
  for (int a = 0; a < 36; ++a) Dst[a] = T(0);
#pragma unroll
  for (int a = 0; a < 6; ++a) gst[a] = T(0);
  bool any_cam = false;
  for (int64_t i = P.lm_obs_off[l]; i < P.lm_obs_off[l + 1]; ++i) {
    T r[2] = {v.r[i], v.r[N + i]};
    T Jl[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) Jl[a] = v.Jl[a * N + i] * sl[a % 3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
      for (int b = 0; b < 3; ++b) H[3 * a + b] += Jl[a] * Jl[b] + Jl[3 + a] * Jl[3 + b];
      g[a] += Jl[a] * r[0] + Jl[3 + a] * r[1];
    }
    const int slot = S.obs_slot[i];
    if (slot < 0) continue;
    any_cam = true;
    T Js[12], Jo[12];
    const int ob = P.obs_kf[i];
#pragma unroll
    for (int a = 0; a < 12; ++a) {
      Js[a] = v.Js[a * N + i] * ss[a % 6];
      Jo[a] = v.Jo[a * N + i] * (scaled ? L.skf[15 * (int64_t)ob + a % 6] : T(1));
    }
    T Wo[18];
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        Wst[6 * x + c] += Jl[x] * Js[c] + Jl[3 + x] * Js[6 + c];
        Wo[6 * x + c] = Jl[x] * Jo[c] + Jl[3 + x] * Jo[6 + c];
      }
    store_slot(L.Wslot + kSlotStride * (int64_t)slot, Wo);
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      gst[a] += Js[a] * r[0] + Js[6 + a] * r[1];
#pragma unroll
      for (int b = a; b < 6; ++b) Dst[6 * a + b] += Js[a] * Js[b] + Js[6 + a] * Js[6 + b];
    }
    const int blk = S.obs_pblk[i];
    T* Pb = L.Pbase + 36 * (int64_t)blk;
    const T* X = st < ob ? Js : Jo;  // P block rows: the lower keyframe of the pair
    const T* Y = st < ob ? Jo : Js;
    if constexpr (sizeof(T) == 4) {
      // 16-byte vector atomics: the (store, observer) block, the observer's
      // pose block (its 21 upper-triangle values) and its gradient.
      float4* P4 = reinterpret_cast<float4*>(Pb);
      float4* D4 = reinterpret_cast<float4*>(L.Dpose + kPoseUp * (int64_t)ob);
      float4* g4 = reinterpret_cast<float4*>(L.gpose + 8 * (int64_t)ob);
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        float pv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int a = (4 * q + u) / 6, b = (4 * q + u) % 6;
          pv[u] = X[a] * Y[b] + X[6 + a] * Y[6 + b];
        }
        atomicAdd(P4 + q, make_float4(pv[0], pv[1], pv[2], pv[3]));
      }
#pragma unroll
      for (int q = 0; q < kPoseUp / 4; ++q) {
        float dv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = 4 * q + u, a = up_row(t), b = up_col(t);
          dv[u] = t < 21 ? Jo[a] * Jo[b] + Jo[6 + a] * Jo[6 + b] : 0.f;
        }
        atomicAdd(D4 + q, make_float4(dv[0], dv[1], dv[2], dv[3]));
      }
      float gv[6];
#pragma unroll
      for (int a = 0; a < 6; ++a) gv[a] = Jo[a] * r[0] + Jo[6 + a] * r[1];
      atomicAdd(g4, make_float4(gv[0], gv[1], gv[2], gv[3]));
      atomicAdd(g4 + 1, make_float4(gv[4], gv[5], 0.f, 0.f));
    } else {
#pragma unroll
      for (int a = 0; a < 6; ++a) {
        atomic_add(&L.gc[15 * (int64_t)ob + a], Jo[a] * r[0] + Jo[6 + a] * r[1]);
#pragma unroll
        for (int b = a; b < 6; ++b)
          atomic_add(&L.Dbase[225 * (int64_t)ob + 15 * a + b], Jo[a] * Jo[b] + Jo[6 + a] * Jo[6 + b]);
      }
#pragma unroll
      for (int a = 0; a < 6; ++a)
#pragma unroll
        for (int b = 0; b < 6; ++b) atomic_add(&Pb[6 * a + b], X[a] * Y[b] + X[6 + a] * Y[6 + b]);
    }
  }
#pragma unroll
  for (int a = 0; a < 9; ++a) L.Hll[a * NL + l] = H[a];
#pragma unroll
  for (int a = 0; a < 3; ++a) L.gl[a * NL + l] = g[a];
  store_slot(L.Wslot + kSlotStride * s0, Wst);
  if (any_cam) {
    if constexpr (sizeof(T) == 4) {
      float4* D4 = reinterpret_cast<float4*>(L.Dpose + kPoseUp * (int64_t)st);
      float4* g4 = reinterpret_cast<float4*>(L.gpose + 8 * (int64_t)st);
#pragma unroll
      for (int q = 0; q < kPoseUp / 4; ++q) {
        float dv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = 4 * q + u;
          dv[u] = t < 21 ? Dst[6 * up_row(t) + up_col(t)] : 0.f;
        }
        atomicAdd(D4 + q, make_float4(dv[0], dv[1], dv[2], dv[3]));
      }
      atomicAdd(g4, make_float4(gst[0], gst[1], gst[2], gst[3]));
      atomicAdd(g4 + 1, make_float4(gst[4], gst[5], 0.f, 0.f));
    } else {
#pragma unroll
      for (int a = 0; a < 6; ++a) {
        atomic_add(&L.gc[15 * (int64_t)st + a], gst[a]);
#pragma unroll
        for (int b = a; b < 6; ++b) atomic_add(&L.Dbase[225 * (int64_t)st + 15 * a + b], Dst[6 * a + b]);
      }
    }
  }
}

// FP32 path: adds the vector-accumulated visual pose blocks (upper triangle)
// and gradients into D and g_c (before the lower triangles are mirrored).
__global__ void __launch_bounds__(kB) k_merge_pose(int64_t nkf, const float* Dpose, const float* gpose, float* D,
                                                   float* gc, const int* run_if, const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 27 * nkf) return;
  const int64_t k = i / 27;
  const int q = (int)(i % 27);
  if (q < 21) D[225 * k + 15 * up_row(q) + up_col(q)] += Dpose[kPoseUp * k + q];
  else gc[15 * k + q - 21] += gpose[8 * k + q - 21];
}

// One warp per inertial edge.
template <typename T>
__global__ void __launch_bounds__(128) k_assemble_inertial(DevProblem P, InertialLin<T> in, LinearSystem<T> L,
                                                           int scaled, const int* run_if, const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (e >= P.nedge) return;
  const int f = P.e_from[e], t = P.e_to[e];
  const T* Jf = in.Jf + 225 * e;
  const T* Jt = in.Jt + 225 * e;
  const T* r = in.r + 15 * e;
  for (int a = lane; a < 225; a += 32) {
    const int rr = a / 15, c = a % 15;
    T dff = T(0), dtt = T(0), eft = T(0);
#pragma unroll
    for (int m = 0; m < 15; ++m) {
      dff += Jf[15 * m + rr] * Jf[15 * m + c];
      dtt += Jt[15 * m + rr] * Jt[15 * m + c];
      eft += Jf[15 * m + rr] * Jt[15 * m + c];
    }
    if (scaled) {
      const T* sf = L.skf + 15 * (int64_t)f;
      const T* sto = L.skf + 15 * (int64_t)t;
      dff *= sf[rr] * sf[c];
      dtt *= sto[rr] * sto[c];
      eft *= sf[rr] * sto[c];
    }
    const bool pose_lower = rr < 6 && c < rr;  // mirrored from the upper triangle
    if (!pose_lower) {
      atomic_add(&L.Dbase[225 * (int64_t)f + a], dff);
      atomic_add(&L.Dbase[225 * (int64_t)t + a], dtt);
    }
    L.Ebase[225 * e + a] = eft;
  }
  if (lane < 15) {
    T gf = T(0), gt = T(0);
#pragma unroll
    for (int m = 0; m < 15; ++m) { gf += Jf[15 * m + lane] * r[m]; gt += Jt[15 * m + lane] * r[m]; }
    if (scaled) {
      gf *= L.skf[15 * (int64_t)f + lane];
      gt *= L.skf[15 * (int64_t)t + lane];
    }
    atomic_add(&L.gc[15 * (int64_t)f + lane], gf);
    atomic_add(&L.gc[15 * (int64_t)t + lane], gt);
  }
  // Switch variable of a loop closure: its J^T J, gradient (with the prior
  // r = (1 - s) w, J = -w) and the coupling columns W = J_k^T J_s.
  if (e >= P.nimu) {
    const int64_t j = e - P.nimu;
    const int q = P.pe_swi[j];
    if (q >= 0) {
      const T* js = in.Js + 6 * j;
      if (lane < 15) {
        T wf = T(0), wt = T(0);
#pragma unroll
        for (int m = 0; m < 6; ++m) { wf += Jf[15 * m + lane] * js[m]; wt += Jt[15 * m + lane] * js[m]; }
        if (scaled) {
          wf *= L.ssw[q] * L.skf[15 * (int64_t)f + lane];
          wt *= L.ssw[q] * L.skf[15 * (int64_t)t + lane];
        }
        L.swW[30 * q + lane] = wf;
        L.swW[30 * q + 15 + lane] = wt;
      } else if (lane == 15) {
        const double w = P.sw_w[q], rp = (1.0 - P.sw[q]) * w;
        T h = T(w * w), g = T(-w * rp);
#pragma unroll
        for (int m = 0; m < 6; ++m) { h += js[m] * js[m]; g += js[m] * r[m]; }
        if (scaled) {
          h *= L.ssw[q] * L.ssw[q];
          g *= L.ssw[q];
        }
        L.swH[q] = h;
        L.swg[q] = g;
      }
    }
  }
}

// Lower triangle of each keyframe's 6x6 pose block of D from its upper one.
template <typename T>
__global__ void __launch_bounds__(kB) k_mirror_pose_blocks(int64_t nkf, T* D, const int* run_if, const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 15 * nkf) return;
  const int64_t k = i / 15;
  int q = (int)(i % 15), a = 1;  // the 15 strictly-lower entries (a, b), b < a < 6
  while (q >= a) { q -= a; ++a; }
  T* B = D + 225 * k;
  B[15 * a + q] = B[15 * q + a];
}

// Jacobi scaling from the unscaled diagonal of J^T J (first linearization
// only); FP64 and T copies of the scale vectors.
template <typename T>
__global__ void k_scale(DevProblem P, LinearSystem<T> L, ScaleVectors sc, int jacobi, const int* run_if) {
  if (run_if && !*run_if) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nk = 15 * P.nkf, nl = 3 * P.nlm;
  if (i < nk) {
    const int64_t k = i / 15, d = i % 15;
    const double h = (double)L.Dbase[225 * k + 16 * d];
    sc.skf[i] = jacobi ? 1.0 / (1.0 + sqrt(h > 0.0 ? h : 0.0)) : 1.0;
    L.skf[i] = T(sc.skf[i]);
  } else if (i < nk + nl) {
    const int64_t j = i - nk, a = j / P.nlm, l = j % P.nlm;
    const double h = (double)L.Hll[(4 * a) * P.nlm + l];
    sc.slm[j] = jacobi ? 1.0 / (1.0 + sqrt(h > 0.0 ? h : 0.0)) : 1.0;
    L.slm[j] = T(sc.slm[j]);
  } else if (i < nk + nl + P.nsw) {
    const int64_t q = i - nk - nl;
    const double h = (double)L.swH[q];
    sc.ssw[q] = jacobi ? 1.0 / (1.0 + sqrt(h > 0.0 ? h : 0.0)) : 1.0;
    L.ssw[q] = T(sc.ssw[q]);
  }
}

// Applies the Jacobi scaling in place to the assembled normal equations:
// H_ll, g_l, W slots, D, P, E blocks and g_c (J s instead of J).
// W_slot (x, c) *= slm[x] of its landmark * skf[c] of its keyframe; one
// thread per slot row.
template <typename T>
__global__ void __launch_bounds__(kB) k_scale_slots(DevProblem P, SchurPattern S, LinearSystem<T> L,
                                                    const int* run_if, const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t sl = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (sl >= S.nslot) return;
  const int64_t NL = P.nlm, l = S.slot_lm[sl], k = S.slot_kf[sl];
  T w[18], a[3], b[6];
  load_slot(L.Wslot + kSlotStride * sl, w);
#pragma unroll
  for (int x = 0; x < 3; ++x) a[x] = L.slm[x * NL + l];
#pragma unroll
  for (int c = 0; c < 6; ++c) b[c] = L.skf[15 * k + c];
#pragma unroll
  for (int x = 0; x < 3; ++x)
#pragma unroll
    for (int c = 0; c < 6; ++c) w[6 * x + c] *= a[x] * b[c];
  store_slot(L.Wslot + kSlotStride * sl, w);
}

template <typename T>
__global__ void __launch_bounds__(kB) k_scale_inplace(DevProblem P, SchurPattern S, LinearSystem<T> L,
                                                      const int* run_if, const int* skip_if) {
  if (gated(run_if, skip_if)) return;
  const int64_t NL = P.nlm, NK = P.nkf, NE = P.nedge, NPU = S.npu;
  const int64_t n1 = 9 * NL, n2 = n1 + 3 * NL, n3 = n2 /* W slots: k_scale_slots */, n4 = n3 + 225 * NK, n5 = n4 + 36 * NPU,
                n6 = n5 + 225 * NE, n7 = n6 + 15 * NK, n8 = n7 + 2 * P.nsw, n9 = n8 + 30 * P.nsw;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n9; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n1) {
      const int64_t q = i / NL, l = i % NL;
      L.Hll[i] *= L.slm[(q / 3) * NL + l] * L.slm[(q % 3) * NL + l];
    } else if (i < n2) {
      const int64_t j = i - n1, l = j % NL;
      L.gl[j] *= L.slm[j];
      (void)l;
    } else if (i < n4) {
      const int64_t j = i - n3, k = j / 225, e = j % 225;
      L.Dbase[j] *= L.skf[15 * k + e / 15] * L.skf[15 * k + e % 15];
    } else if (i < n5) {
      const int64_t j = i - n4, b = j / 36, e = j % 36;
      L.Pbase[j] *= L.skf[15 * (int64_t)S.pu_i[b] + e / 6] * L.skf[15 * (int64_t)S.pu_j[b] + e % 6];
    } else if (i < n6) {
      const int64_t j = i - n5, ed = j / 225, e = j % 225;
      L.Ebase[j] *= L.skf[15 * (int64_t)P.e_from[ed] + e / 15] * L.skf[15 * (int64_t)P.e_to[ed] + e % 15];
    } else if (i < n7) {
      const int64_t j = i - n6;
      L.gc[j] *= L.skf[j];
    } else if (i < n8) {
      const int64_t j = i - n7, q = j >> 1;
      if (j & 1) L.swg[q] *= L.ssw[q];
      else L.swH[q] *= L.ssw[q] * L.ssw[q];
    } else {
      const int64_t j = i - n8, q = j / 30, c = j % 30, ed = P.sw_e[q];
      const int64_t k = c < 15 ? P.e_from[ed] : P.e_to[ed];
      L.swW[j] *= L.ssw[q] * L.skf[15 * k + c % 15];
    }
  }
}

template <typename T>
__device__ __forceinline__ T lm_damp_t(T h, T mn, T mx, T radius) {
  T d = h < mn ? mn : (h > mx ? mx : h);
  return d / radius;
}

// Damped keyframe system from the scaled blocks: SD = D + diag, SE, SP, rhs = -g.
template <typename T>
__global__ void __launch_bounds__(kB) k_build_system(SolverLaunch<T> s) {
  LmControl* ctl = s.ctl;
  if (ctl->terminated) return;
  const int64_t nkf = s.P.nkf, ne = s.P.nedge, npu = s.S.npu;
  const int64_t n1 = nkf * 225, n2 = n1 + ne * 225, n3 = n2 + npu * 36, n4 = n3 + nkf * 15;
  const T radius = T(ctl->radius);
  const T mn = T(s.prm.min_lm_diagonal), mx = T(s.prm.max_lm_diagonal);
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (tid == 0) {
    ctl->accepted = 0;
    ctl->status = 0;
    ctl->model_change = 0.0;
    ctl->cost_cand = 0.0;
    ctl->cost_cand_ine = 0.0;
    ctl->step_norm2 = 0.0;
    ctl->x_norm2 = 0.0;
    ctl->nonfinite = 0;
    ctl->inertial_status = 0;
    ctl->pcg_done = 0;
    ctl->pcg_iters = 0;
    ctl->chain_failed = 0;
    ctl->pcg_rz0 = 0.0;
    ctl->pcg_bnorm2 = 0.0;
    for (int a = 0; a < 3; ++a) { ctl->pcg_pq[a] = 0.0; ctl->pcg_rr[a] = 0.0; ctl->pcg_rz[a] = 0.0; }
  }
  for (int64_t i = tid; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n1) {
      const int64_t e = i % 225, a = e / 15, b = e % 15;
      const T h = s.L.Dbase[i];
      s.L.SD[i] = (a == b) ? h + lm_damp_t(h, mn, mx, radius) : h;
    } else if (i < n2) {
      s.L.SE[i - n1] = s.L.Ebase[i - n1];
    } else if (i < n3) {
      s.L.SP[i - n2] = s.L.Pbase[i - n2];
    } else {
      s.L.rhs[i - n3] = -s.L.gc[i - n3];
    }
  }
}

template <typename T>
__device__ __forceinline__ bool inv3t(const T* A, T* B) {
  const T c0 = A[4] * A[8] - A[5] * A[7], c1 = A[5] * A[6] - A[3] * A[8], c2 = A[3] * A[7] - A[4] * A[6];
  const T det = A[0] * c0 + A[1] * c1 + A[2] * c2;
  if (!(det != T(0)) || !isfinite((double)det)) return false;
  const T id = T(1) / det;
  B[0] = c0 * id; B[1] = (A[2] * A[7] - A[1] * A[8]) * id; B[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  B[3] = c1 * id; B[4] = (A[0] * A[8] - A[2] * A[6]) * id; B[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  B[6] = c2 * id; B[7] = (A[1] * A[6] - A[0] * A[7]) * id; B[8] = (A[0] * A[4] - A[1] * A[3]) * id;
  return true;
}

// Landmark elimination, part 1: V = (H + D)^-1 and rhs += W^T V g (scaled blocks).
template <typename T>
__global__ void __launch_bounds__(kB) k_schur_lm(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t NL = s.P.nlm;
  if (l >= NL) return;
  T V[9] = {T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
  if (s.P.lm_active[l]) {
    const T radius = T(s.ctl->radius), mn = T(s.prm.min_lm_diagonal), mx = T(s.prm.max_lm_diagonal);
    // The 3x3 inverse runs in FP64 in both paths: poorly constrained landmarks
    // (short baselines) make these blocks ill-conditioned.
    double Hs[9], Vd[9];
#pragma unroll
    for (int a = 0; a < 9; ++a) Hs[a] = (double)s.L.Hll[a * NL + l];
#pragma unroll
    for (int a = 0; a < 3; ++a) Hs[4 * a] += (double)lm_damp_t(T(Hs[4 * a]), mn, mx, radius);
    if (!inv3t(Hs, Vd)) {
      atomicExch(&s.ctl->status, (int)MBA_ERR_NOT_SPD);
#pragma unroll
      for (int a = 0; a < 9; ++a) Vd[a] = 0.0;
    }
#pragma unroll
    for (int a = 0; a < 9; ++a) V[a] = T(Vd[a]);
    T g[3], Vg[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) g[a] = s.L.gl[a * NL + l];
#pragma unroll
    for (int a = 0; a < 3; ++a) Vg[a] = V[3 * a] * g[0] + V[3 * a + 1] * g[1] + V[3 * a + 2] * g[2];
    for (int64_t si = s.S.lm_slot_off[l]; si < s.S.lm_slot_end[l]; ++si) {
      const int64_t k = s.S.slot_kf[si];
      T w[18];
      load_slot(s.L.Wslot + kSlotStride * si, w);
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const T acc = w[c] * Vg[0] + w[6 + c] * Vg[1] + w[12 + c] * Vg[2];
        if (acc != T(0)) atomic_add(&s.L.rhs[15 * k + c], acc);
      }
    }
  }
#pragma unroll
  for (int a = 0; a < 9; ++a) s.L.V[a * NL + l] = V[a];
}

// Landmark elimination, part 2: U = V W per slot, one thread per U row (U
// rows are numbered by store keyframe, W rows by landmark: S.u_w maps).
template <typename T>
__global__ void __launch_bounds__(kB) k_schur_slot(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t NS = s.S.nslot, NL = s.P.nlm;
  if (i >= NS) return;
  const int64_t w = s.S.u_w[i], l = s.S.slot_lm[w];
  T W[18], V[9];
  load_slot(s.L.Wslot + kSlotStride * w, W);
#pragma unroll
  for (int a = 0; a < 9; ++a) V[a] = s.L.V[a * NL + l];
  T U[18];
#pragma unroll
  for (int x = 0; x < 3; ++x)
#pragma unroll
    for (int c = 0; c < 6; ++c) U[6 * x + c] = V[3 * x] * W[c] + V[3 * x + 1] * W[6 + c] + V[3 * x + 2] * W[12 + c];
  store_slot(s.L.U + kSlotStride * i, U);
}

// U row of a pair's b (bitwise-not when b is a itself).
__device__ __forceinline__ int64_t pair_u(int y) { return y < 0 ? ~y : y; }

// Landmark elimination, part 3: S(k_a, k_b) -= W_a^T U_b for every slot pair.
// Pairs are sorted by target block; one thread sums a chunk of one target's
// pairs in registers and writes the block once (plain read-modify-write when
// it owns the whole target, atomics otherwise).  Diagonal targets take
// M + M^T for a != b; upper pairs are oriented so M lands untransposed.
// Chunks are grouped by the target's keyframe row i (k_a = i): one block per
// row stages the row's W slots in shared memory (rows of kSlotStride values,
// if they fit in stage_cap slots), so that only U_b is gathered from global
// memory; the next pair's rows are loaded while a pair is multiplied.
template <typename T>
__global__ void __launch_bounds__(kB, sizeof(T) == 4 ? 2 : 1) k_schur_pairs(SolverLaunch<T> s, int64_t stage_cap) {
  if (s.ctl->terminated) return;
  extern __shared__ __align__(16) unsigned char schur_smem[];
  T* sW = reinterpret_cast<T*>(schur_smem);
  const int64_t i = blockIdx.x;
  const int64_t c0 = s.S.row_chunk_off[i], c1 = s.S.row_chunk_off[i + 1];
  if (c0 == c1) return;
  const int64_t s0 = s.S.kf_slot_off[i], ns = s.S.kf_slot_off[i + 1] - s0;
  const bool staged = ns <= stage_cap;
  if (staged)
    for (int64_t q = threadIdx.x; q < 18 * ns; q += blockDim.x)
      sW[kSlotStride * (q / 18) + q % 18] = s.L.Wslot[kSlotStride * (int64_t)s.S.kf_slot[s0 + q / 18] + q % 18];
  __syncthreads();
  auto wrow = [&](int a) -> const T* {
    return staged ? sW + kSlotStride * (int64_t)a : s.L.Wslot + kSlotStride * (int64_t)s.S.kf_slot[s0 + a];
  };
  for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
    const int32_t raw = s.S.chunk_tgt[c];
    const bool whole = raw >= 0;
    const int64_t tid = whole ? raw : ~raw;
    const bool diag = tid < s.P.nkf;
    T acc[36];
#pragma unroll
    for (int q = 0; q < 36; ++q) acc[q] = T(0);
    const int64_t p0 = s.S.chunk_beg[c], p1 = p0 + s.S.chunk_len[c];
    int2 ab = s.S.pair_rb[p0];
    int2 abn = p0 + 1 < p1 ? s.S.pair_rb[p0 + 1] : ab;  // pair indices run one step ahead of the rows
    T Wa[18], Ub[18];
    load_slot(wrow(ab.x), Wa);
    load_slot(s.L.U + kSlotStride * pair_u(ab.y), Ub);
    for (int64_t p = p0; p < p1; ++p) {
      const bool sym = diag && ab.y >= 0;  // a != b
      T Wn[18], Un[18];
      const int2 abnn = p + 2 < p1 ? s.S.pair_rb[p + 2] : abn;
      if (p + 1 < p1) {
        load_slot(wrow(abn.x), Wn);
        load_slot(s.L.U + kSlotStride * pair_u(abn.y), Un);
      }
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          const T m = Wa[r] * Ub[q] + Wa[6 + r] * Ub[6 + q] + Wa[12 + r] * Ub[12 + q];
          acc[6 * r + q] += m;
          if (sym) acc[6 * q + r] += m;
        }
      if (p + 1 < p1) {
#pragma unroll
        for (int k = 0; k < 18; ++k) { Wa[k] = Wn[k]; Ub[k] = Un[k]; }
        ab = abn;
        abn = abnn;
      }
    }
    T* dst = diag ? s.L.SD + 225 * tid : s.L.SP + 36 * (tid - s.P.nkf);
    const int ld = diag ? 15 : 6;
    if (whole) {
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int q = 0; q < 6; ++q) dst[ld * r + q] -= acc[6 * r + q];
    } else {
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int q = 0; q < 6; ++q) atomic_add(&dst[ld * r + q], -acc[6 * r + q]);
    }
  }
}

// Transposed part of a diagonal target's pair product for the thread that
// owns columns 3H..3H+2: element (q, r) of m^T, q = 3H + qq, goes to this
// thread's acc when column r is its own, else to accT for the partner.
template <int H, typename T>
__device__ __forceinline__ void schur_sym_half(const T (&m)[6][3], T (&acc)[18], T (&accT)[9]) {
#pragma unroll
  for (int r = 0; r < 6; ++r)
#pragma unroll
    for (int qq = 0; qq < 3; ++qq) {
      if (r / 3 == H) acc[3 * (3 * H + qq) + (r - 3 * H)] += m[r][qq];
      else accT[3 * qq + (r - 3 * (1 - H))] += m[r][qq];
    }
}
// The partner's transposed terms: in[3 qq + rr] is element (3 (1 - H) + qq, 3 H + rr).
template <int H, typename T>
__device__ __forceinline__ void schur_sym_merge(const T (&in)[9], T (&acc)[18]) {
#pragma unroll
  for (int qq = 0; qq < 3; ++qq)
#pragma unroll
    for (int rr = 0; rr < 3; ++rr) acc[3 * (3 * (1 - H) + qq) + rr] += in[3 * qq + rr];
}

// k_schur_pairs with two threads per chunk: thread h of a pair owns the
// output columns 3h..3h+2 (18 accumulators instead of 36) and loads only those
// columns of U_b, so a block keeps twice the partner rows in flight at fewer
// registers per thread.  The transposed terms of a diagonal target that land
// in the partner's columns are exchanged once per chunk.
template <typename T>
__global__ void __launch_bounds__(kB, sizeof(T) == 4 ? 3 : 1) k_schur_pairs_split(SolverLaunch<T> s, int64_t stage_cap) {
  if (s.ctl->terminated) return;
  extern __shared__ __align__(16) unsigned char schur_smem[];
  T* sW = reinterpret_cast<T*>(schur_smem);
  const int64_t i = blockIdx.x;
  const int64_t c0 = s.S.row_chunk_off[i], c1 = s.S.row_chunk_off[i + 1];
  if (c0 == c1) return;
  const int64_t s0 = s.S.kf_slot_off[i], ns = s.S.kf_slot_off[i + 1] - s0;
  const bool staged = ns <= stage_cap;
  if (staged)
    for (int64_t q = threadIdx.x; q < 18 * ns; q += blockDim.x)
      sW[kSlotStride * (q / 18) + q % 18] = s.L.Wslot[kSlotStride * (int64_t)s.S.kf_slot[s0 + q / 18] + q % 18];
  __syncthreads();
  const int h = threadIdx.x & 1;
  const unsigned pair_mask = 3u << ((threadIdx.x & 31) & ~1);
  for (int64_t c = c0 + (threadIdx.x >> 1); c < c1; c += blockDim.x >> 1) {
    const int32_t raw = s.S.chunk_tgt[c];
    const bool whole = raw >= 0;
    const int64_t tid = whole ? raw : ~raw;
    const bool diag = tid < s.P.nkf;
    T acc[18], accT[9];
#pragma unroll
    for (int q = 0; q < 18; ++q) acc[q] = T(0);
#pragma unroll
    for (int q = 0; q < 9; ++q) accT[q] = T(0);
    const int64_t p0 = s.S.chunk_beg[c], p1 = p0 + s.S.chunk_len[c];
    int2 ab = s.S.pair_rb[p0];
    int2 abn = p0 + 1 < p1 ? s.S.pair_rb[p0 + 1] : ab;  // pair indices run one step ahead of the rows
    T Ub[9];  // U_b rows 0..2, columns 3h..3h+2
    {
      const T* u = s.L.U + kSlotStride * pair_u(ab.y) + 3 * h;
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) Ub[3 * k + qq] = u[6 * k + qq];
    }
    for (int64_t p = p0; p < p1; ++p) {
      const bool sym = diag && ab.y >= 0;  // a != b
      const T* wa = staged ? sW + kSlotStride * (int64_t)ab.x : s.L.Wslot + kSlotStride * (int64_t)s.S.kf_slot[s0 + ab.x];
      T Un[9];
      const int2 abnn = p + 2 < p1 ? s.S.pair_rb[p + 2] : abn;
      if (p + 1 < p1) {
        const T* u = s.L.U + kSlotStride * pair_u(abn.y) + 3 * h;
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int qq = 0; qq < 3; ++qq) Un[3 * k + qq] = u[6 * k + qq];
      }
      T m[6][3];
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        const T w0 = wa[r], w1 = wa[6 + r], w2 = wa[12 + r];
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) {
          m[r][qq] = w0 * Ub[qq] + w1 * Ub[3 + qq] + w2 * Ub[6 + qq];
          acc[3 * r + qq] += m[r][qq];
        }
      }
      if (sym) {
        if (h) schur_sym_half<1>(m, acc, accT);
        else schur_sym_half<0>(m, acc, accT);
      }
      if (p + 1 < p1) {
#pragma unroll
        for (int k = 0; k < 9; ++k) Ub[k] = Un[k];
        ab = abn;
        abn = abnn;
      }
    }
    if (diag) {
      T in[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) in[q] = __shfl_xor_sync(pair_mask, accT[q], 1);
      if (h) schur_sym_merge<1>(in, acc);
      else schur_sym_merge<0>(in, acc);
    }
    T* dst = diag ? s.L.SD + 225 * tid : s.L.SP + 36 * (tid - s.P.nkf);
    const int ld = diag ? 15 : 6;
    if (whole) {
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) dst[ld * r + 3 * h + qq] -= acc[3 * r + qq];
    } else {
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) atomic_add(&dst[ld * r + 3 * h + qq], -acc[3 * r + qq]);
    }
  }
}

// Shared-memory bytes of k_schur_pairs (a row's staged W slots) and the slot
// count that fits; longer rows read W from global memory.
template <typename T>
int64_t schur_pairs_smem(const SchurPattern& S, bool split, int64_t* cap) {
  // FP32: two blocks per SM (three for the split kernel, whose rows fit in 72 KB)
  const int64_t limit = sizeof(T) == 4 ? (split ? 72 : 96) * 1024 : 200 * 1024;
  const int64_t fit = limit / (kSlotStride * (int64_t)sizeof(T));
  *cap = S.max_row_slots < fit ? S.max_row_slots : fit;
  return *cap * kSlotStride * (int64_t)sizeof(T);
}

// The shared-memory opt-in is set by solver_prepare (outside graph capture).
template <typename T>
cudaError_t launch_schur_pairs(const SolverLaunch<T>& s, cudaStream_t st) {
  if (s.S.nchunk == 0) return cudaSuccess;
  int64_t cap = 0;
  const int64_t bytes = schur_pairs_smem<T>(s.S, s.S.schur_split != 0, &cap);
  if (s.S.schur_split)
    k_schur_pairs_split<T><<<(unsigned)s.P.nkf, kB, (size_t)bytes, st>>>(s, cap);
  else
    k_schur_pairs<T><<<(unsigned)s.P.nkf, kB, (size_t)bytes, st>>>(s, cap);
  return cudaGetLastError();
}

// Switch elimination (one warp per switch variable): H = h + damping,
// SD_ff -= W_f W_f^T / H, SD_tt -= W_t W_t^T / H, SE -= W_f W_t^T / H,
// rhs += W g / H.  H is inverted in FP64.
template <typename T>
__global__ void __launch_bounds__(128) k_schur_switch(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t q = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= s.P.nsw) return;
  const int64_t e = s.P.sw_e[q], f = s.P.e_from[e], t = s.P.e_to[e];
  const T radius = T(s.ctl->radius), mn = T(s.prm.min_lm_diagonal), mx = T(s.prm.max_lm_diagonal);
  const T h = s.L.swH[q];
  const double H = (double)h + (double)lm_damp_t(h, mn, mx, radius);
  const T hi = T(1.0 / H);
  if (lane == 0) s.L.swHi[q] = hi;
  const T* W = s.L.swW + 30 * q;
  const T g = s.L.swg[q];
  for (int a = lane; a < 225; a += 32) {
    const int r = a / 15, c = a % 15;
    const T wff = W[r] * W[c] * hi, wtt = W[15 + r] * W[15 + c] * hi, wft = W[r] * W[15 + c] * hi;
    if (wff != T(0)) atomic_add(&s.L.SD[225 * f + a], -wff);
    if (wtt != T(0)) atomic_add(&s.L.SD[225 * t + a], -wtt);
    s.L.SE[225 * e + a] -= wft;  // one switch per edge: a single writer
  }
  if (lane < 15) {
    atomic_add(&s.L.rhs[15 * f + lane], W[lane] * hi * g);
    atomic_add(&s.L.rhs[15 * t + lane], W[15 + lane] * hi * g);
  }
}

// Masked tangent dims -> identity rows; mirror SP to the lower orientation.
template <typename T>
__global__ void __launch_bounds__(kB) k_finalize_system(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t nkf = s.P.nkf, ne = s.P.nedge, npu = s.S.npu;
  const int64_t n1 = nkf * 225, n2 = n1 + ne * 225, n3 = n2 + npu * 36, n4 = n3 + nkf * 15;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n1) {
      const int64_t k = i / 225, e = i % 225, a = e / 15, b = e % 15;
      const uint16_t m = s.P.kf_mask[k];
      if (!((m >> a) & 1) || !((m >> b) & 1)) s.L.SD[i] = (a == b) ? T(1) : T(0);
    } else if (i < n2) {
      const int64_t j = i - n1, e = j / 225, q = j % 225, a = q / 15, b = q % 15;
      if (!((s.P.kf_mask[s.P.e_from[e]] >> a) & 1) || !((s.P.kf_mask[s.P.e_to[e]] >> b) & 1)) s.L.SE[j] = T(0);
    } else if (i < n3) {
      const int64_t j = i - n2, b = j / 36, q = j % 36, a = q / 6, c = q % 6;
      T v = s.L.SP[j];
      if (!((s.P.kf_mask[s.S.pu_i[b]] >> a) & 1) || !((s.P.kf_mask[s.S.pu_j[b]] >> c) & 1)) {
        v = T(0);
        s.L.SP[j] = v;
      }
      s.L.SP[36 * (npu + b) + 6 * c + a] = v;
    } else {
      const int64_t j = i - n3, k = j / 15, d = j % 15;
      if (!((s.P.kf_mask[k] >> d) & 1)) s.L.rhs[j] = T(0);
    }
  }
}

// Block-Jacobi preconditioner: FP64 Cholesky inverse of each 15x15 SD block.
template <typename T>
__global__ void __launch_bounds__(64) k_block_jacobi(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= s.P.nkf + s.P.ng) return;  // keyframe blocks, then the global nodes' diagonal blocks
  double L[120];  // packed lower triangle
  const T* A = s.L.SD + 225 * k;
  int fail = 0;
  for (int j = 0; j < 15 && !fail; ++j) {
    double d = (double)A[16 * j];
    for (int q = 0; q < j; ++q) d -= L[j * (j + 1) / 2 + q] * L[j * (j + 1) / 2 + q];
    if (!(d > 0.0)) { fail = 1; break; }
    const double ljj = sqrt(d);
    L[j * (j + 1) / 2 + j] = ljj;
    for (int i = j + 1; i < 15; ++i) {
      double v = 0.5 * ((double)A[15 * i + j] + (double)A[15 * j + i]);
      for (int q = 0; q < j; ++q) v -= L[i * (i + 1) / 2 + q] * L[j * (j + 1) / 2 + q];
      L[i * (i + 1) / 2 + j] = v / ljj;
    }
  }
  T* M = s.L.Minv + 225 * k;
  if (fail) {
    atomicExch(&s.ctl->status, (int)MBA_ERR_NOT_SPD);
    for (int a = 0; a < 225; ++a) M[a] = (a % 16 == 0) ? T(1) : T(0);
    return;
  }
  // Linv (lower) in place of a local 15x15, then M = Linv^T Linv.
  double X[225];
  for (int c = 0; c < 15; ++c)
    for (int i = 0; i < 15; ++i) {
      double v = (i == c) ? 1.0 : 0.0;
      for (int q = c; q < i; ++q) v -= L[i * (i + 1) / 2 + q] * X[15 * q + c];
      X[15 * i + c] = (i < c) ? 0.0 : v / L[i * (i + 1) / 2 + i];
    }
  for (int a = 0; a < 15; ++a)
    for (int b = a; b < 15; ++b) {
      double v = 0.0;
      for (int q = b; q < 15; ++q) v += X[15 * q + a] * X[15 * q + b];
      M[15 * a + b] = T(v);
      M[15 * b + a] = T(v);
    }
}

// ------------------------------------------------------------ PCG
// x = 0, r = b, z = M b (block-Jacobi here; the chain sweeps write z and
// rz0 afterwards when the chain preconditioner is active).
template <typename T>
__global__ void __launch_bounds__(kB) k_pcg_init(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t n = 15 * (s.P.nkf + s.P.ng);  // keyframe rows, then the global nodes' rows
  const bool chain = s.precond != MBA_PRECOND_BLOCK_JACOBI && !s.ctl->chain_failed;
  double rz = 0.0, rr = 0.0;
  if (i < n) {
    const int64_t k = i / 15, a = i % 15;
    const double r = (double)s.L.rhs[i];
    double z = 0.0;
    if (!chain || k >= s.P.nkf) {  // node rows: block-Jacobi also under the chain preconditioner
      const T* M = s.L.Minv + 225 * k;
      for (int b = 0; b < 15; ++b) z += (double)M[15 * a + b] * (double)s.L.rhs[15 * k + b];
      rz = r * z;
    }
    s.L.x[i] = T(0);
    s.L.r[i] = T(r);
    s.L.z[i] = T(z);
    s.L.p[i] = T(0);  // read with beta = 0 by the first product; must be finite
    s.L.q[i] = T(0);  // the read-once product accumulates into q
    rr = r * r;
  }
  block_add(rz, &s.ctl->pcg_rz0);
  block_add(rr, &s.ctl->pcg_bnorm2);
}

// Direction update fused into the product: p_new = z + beta p_old (beta = 0
// at it = 0, where p_old = z), q = S p_new, pq += p_new.q.  p is double
// buffered (pa -> pb) because neighbour rows read p_old while each warp writes
// its own p_new.  At it > 0 the convergence test of the previous update runs
// first.  One warp per keyframe row.
template <typename T>
__global__ void __launch_bounds__(128) k_pcg_spmv(SolverLaunch<T> s, int it, const T* pa, T* pb) {
  LmControl* ctl = s.ctl;
  if (ctl->terminated || ctl->pcg_done || ctl->status) return;
  if (!(ctl->pcg_bnorm2 > 0.0)) {
    if (threadIdx.x == 0 && blockIdx.x == 0) { ctl->pcg_done = 1; ctl->pcg_iters = 0; }
    return;
  }
  double beta = 0.0;
  if (it > 0) {
    const double tol = s.prm.linear_tolerance;
    if (ctl->pcg_rr[(it - 1) % 3] <= tol * tol * ctl->pcg_bnorm2) {
      if (threadIdx.x == 0 && blockIdx.x == 0) { ctl->pcg_done = 1; ctl->pcg_iters = it; }
      return;
    }
    const double rzprev = (it == 1) ? ctl->pcg_rz0 : ctl->pcg_rz[(it + 1) % 3];
    beta = ctl->pcg_rz[(it - 1) % 3] / rzprev;
  }
  const T tb = T(beta);
  const T* z = s.L.z;
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  __shared__ T red[4][32];
  double pq = 0.0;
  if (k < s.P.nkf) {
    // Pose-pose blocks of row k: 5 blocks per warp step, 6 lanes per block,
    // lane r of a block owns output row r.  A block below the diagonal is
    // read as the transpose of the stored upper block (column r), so both
    // rows of a co-visible pair read the same bytes and the second read
    // mostly hits L2 (the pair's rows run close together).
    T acc = T(0);
    const int sub = lane / 6, r = lane - 6 * (lane / 6);
    const int64_t npu = s.S.npu;
    if (sub < 5) {
      const int64_t e1 = s.S.row_off[k + 1];
      int64_t e = s.S.row_off[k] + sub;
      int64_t jn = 0, bn = 0;  // the next block's indices, loaded one step ahead
      if (e < e1) { jn = s.S.row_col[e]; bn = s.S.row_blk[e]; }
      for (; e < e1; e += 5) {
        const int64_t j = jn;
        const int64_t blk = bn;
        if (e + 5 < e1) { jn = s.S.row_col[e + 5]; bn = s.S.row_blk[e + 5]; }
        const bool lower = blk >= npu;
        const T* B = lower ? s.L.SP + 36 * (blk - npu) + r : s.L.SP + 36 * blk + 6 * r;
        const int step = lower ? 6 : 1;
        const T* zj = z + 15 * j;
        const T* pj = pa + 15 * j;
#pragma unroll
        for (int c = 0; c < 6; ++c) acc += B[c * step] * (zj[c] + tb * pj[c]);
      }
    }
    red[w][lane] = acc;
    __syncwarp();
    if (lane < 15) {
      const T* D = s.L.SD + 225 * k + 15 * lane;
      const T* zk = z + 15 * k;
      const T* pk_old = pa + 15 * k;
      T y = T(0);
#pragma unroll
      for (int c = 0; c < 15; ++c) y += D[c] * (zk[c] + tb * pk_old[c]);
      if (lane < 6) y += red[w][lane] + red[w][lane + 6] + red[w][lane + 12] + red[w][lane + 18] + red[w][lane + 24];
      if (lane < 6 && s.P.ng > 0) {  // keyframe-node blocks (pose rows) times the nodes' direction
        const int64_t NK = s.P.nkf;
        for (int64_t g = 0; g < s.P.ng; ++g) {
          const double* Bkg = s.B.BS + 90 * (s.P.ng * k + g) + 15 * lane;
          const T* zg = z + 15 * (NK + g);
          const T* pg = pa + 15 * (NK + g);
          for (int c = 0; c < 15; ++c) y += T(Bkg[c]) * (zg[c] + tb * pg[c]);
        }
      }
      for (int64_t e = s.S.kfe_off[k]; e < s.S.kfe_off[k + 1]; ++e) {
        const int code = s.S.kfe[e];
        const bool from = code > 0;
        const int64_t ed = from ? code - 1 : -code - 1;
        const T* E = s.L.SE + 225 * ed;
        const int64_t o = from ? s.P.e_to[ed] : s.P.e_from[ed];
        const T* zo = z + 15 * o;
        const T* po = pa + 15 * o;
        if (from) {
#pragma unroll
          for (int c = 0; c < 15; ++c) y += E[15 * lane + c] * (zo[c] + tb * po[c]);
        } else {
#pragma unroll
          for (int c = 0; c < 15; ++c) y += E[15 * c + lane] * (zo[c] + tb * po[c]);
        }
      }
      const T pk = zk[lane] + tb * pk_old[lane];
      pb[15 * k + lane] = pk;
      s.L.q[15 * k + lane] = y;
      pq = (double)y * (double)pk;
    }
  }
  block_add(pq, &ctl->pcg_pq[it % 3]);
}

// The same product reading each stored pose block once: the warp of row k
// walks the upper blocks (k, j), j > k, adds B v_j to its own row and B^T v_k
// to row j with atomics (lane c of a block owns column c).  q must be zero on
// entry (k_pcg_init, k_pcg_update); p.q comes from k_pcg_pq once every row is
// complete.  Keyframe rows only (no global nodes).
template <typename T>
__global__ void __launch_bounds__(128) k_pcg_spmv_sym(SolverLaunch<T> s, int it, const T* pa, T* pb) {
  LmControl* ctl = s.ctl;
  if (ctl->terminated || ctl->pcg_done || ctl->status) return;
  if (!(ctl->pcg_bnorm2 > 0.0)) {
    if (threadIdx.x == 0 && blockIdx.x == 0) { ctl->pcg_done = 1; ctl->pcg_iters = 0; }
    return;
  }
  double beta = 0.0;
  if (it > 0) {
    const double tol = s.prm.linear_tolerance;
    if (ctl->pcg_rr[(it - 1) % 3] <= tol * tol * ctl->pcg_bnorm2) {
      if (threadIdx.x == 0 && blockIdx.x == 0) { ctl->pcg_done = 1; ctl->pcg_iters = it; }
      return;
    }
    const double rzprev = (it == 1) ? ctl->pcg_rz0 : ctl->pcg_rz[(it + 1) % 3];
    beta = ctl->pcg_rz[(it - 1) % 3] / rzprev;
  }
  const T tb = T(beta);
  const T* z = s.L.z;
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  __shared__ T red[4][32];
  __shared__ T vk[4][16];
  if (k >= s.P.nkf) return;  // whole warps: no block-wide synchronisation below
  if (lane < 15) {
    const T v = z[15 * k + lane] + tb * pa[15 * k + lane];
    pb[15 * k + lane] = v;
    vk[w][lane] = v;
  }
  __syncwarp();
  T acc = T(0);
  const int sub = lane / 6, r = lane - 6 * (lane / 6);
  if (sub < 5) {
    const int64_t e1 = s.S.up_off[k + 1];
    int64_t e = s.S.up_off[k] + sub;
    int64_t jn = 0, bn = 0;  // the next block's indices, loaded one step ahead
    if (e < e1) { jn = s.S.up_col[e]; bn = s.S.up_blk[e]; }
    for (; e < e1; e += 5) {
      const int64_t j = jn;
      const T* B = s.L.SP + 36 * bn;
      if (e + 5 < e1) { jn = s.S.up_col[e + 5]; bn = s.S.up_blk[e + 5]; }
      const T* zj = z + 15 * j;
      const T* pj = pa + 15 * j;
      T t = T(0);
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        acc += B[6 * r + c] * (zj[c] + tb * pj[c]);
        t += B[6 * c + r] * vk[w][c];
      }
      atomic_add(&s.L.q[15 * j + r], t);
    }
  }
  red[w][lane] = acc;
  __syncwarp();
  if (lane < 15) {
    const T* D = s.L.SD + 225 * k + 15 * lane;
    T y = T(0);
#pragma unroll
    for (int c = 0; c < 15; ++c) y += D[c] * vk[w][c];
    if (lane < 6) y += red[w][lane] + red[w][lane + 6] + red[w][lane + 12] + red[w][lane + 18] + red[w][lane + 24];
    for (int64_t e = s.S.kfe_off[k]; e < s.S.kfe_off[k + 1]; ++e) {
      const int code = s.S.kfe[e];
      const bool from = code > 0;
      const int64_t ed = from ? code - 1 : -code - 1;
      const T* E = s.L.SE + 225 * ed;
      const int64_t o = from ? s.P.e_to[ed] : s.P.e_from[ed];
      const T* zo = z + 15 * o;
      const T* po = pa + 15 * o;
      if (from) {
#pragma unroll
        for (int c = 0; c < 15; ++c) y += E[15 * lane + c] * (zo[c] + tb * po[c]);
      } else {
#pragma unroll
        for (int c = 0; c < 15; ++c) y += E[15 * c + lane] * (zo[c] + tb * po[c]);
      }
    }
    atomic_add(&s.L.q[15 * k + lane], y);
  }
}

// p.q of the read-once product.
template <typename T>
__global__ void __launch_bounds__(kB) k_pcg_pq(SolverLaunch<T> s, int it, const T* p) {
  LmControl* ctl = s.ctl;
  if (ctl->terminated || ctl->pcg_done || ctl->status) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double pq = 0.0;
  if (i < 15 * s.P.nkf) pq = (double)p[i] * (double)s.L.q[i];
  block_add(pq, &ctl->pcg_pq[it % 3]);
}

// x += alpha p ; r -= alpha q ; z = M r ; rr, rz dots.  16 threads per keyframe.
template <typename T>
__global__ void __launch_bounds__(kB) k_pcg_update(SolverLaunch<T> s, int it, const T* p, int last) {
  LmControl* ctl = s.ctl;
  if (ctl->terminated || ctl->pcg_done || ctl->status) return;
  __shared__ T rsh[kB];
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 4;
  const int a = threadIdx.x & 15;
  const double rzprev = it == 0 ? ctl->pcg_rz0 : ctl->pcg_rz[(it + 2) % 3];
  const T alpha = T(rzprev / ctl->pcg_pq[it % 3]);
  double rr = 0.0, rz = 0.0;
  T rnew = T(0);
  const bool act = (k < s.P.nkf + s.P.ng) && a < 15;  // keyframe rows, then the global nodes' rows
  // the chain preconditioner covers the keyframe rows; node rows stay block-Jacobi
  const bool chain = s.precond != MBA_PRECOND_BLOCK_JACOBI && !ctl->chain_failed && k < s.P.nkf;
  if (act) {
    const int64_t i = 15 * k + a;
    s.L.x[i] = s.L.x[i] + alpha * p[i];
    rnew = s.L.r[i] - alpha * s.L.q[i];
    s.L.r[i] = rnew;
    if (s.S.spmv_sym) s.L.q[i] = T(0);  // the next read-once product accumulates into q
  }
  rsh[threadIdx.x] = rnew;
  __syncthreads();
  if (act && chain) rr = (double)rnew * (double)rnew;  // z and r.z come from the chain sweeps
  if (act && !chain) {
    const T* M = s.L.Minv + 225 * k + 15 * a;
    const int base = threadIdx.x & ~15;
    T z = T(0);
#pragma unroll
    for (int b = 0; b < 15; ++b) z += M[b] * rsh[base + b];
    s.L.z[15 * k + a] = z;
    rr = (double)rnew * (double)rnew;
    rz = (double)rnew * (double)z;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->pcg_pq[(it + 1) % 3] = 0.0;
    ctl->pcg_rr[(it + 1) % 3] = 0.0;
    ctl->pcg_rz[(it + 1) % 3] = 0.0;
    if (last) ctl->pcg_iters = it + 1;
  }
  block_add(rr, &ctl->pcg_rr[it % 3]);
  block_add(rz, &ctl->pcg_rz[it % 3]);
}

// ------------------------------------------------------------ step
// Back substitution: dl = V (-g - sum_a W_a x_{k_a}) (scaled system).
template <typename T>
__global__ void __launch_bounds__(kB) k_backsub(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t NL = s.P.nlm, NS = s.S.nslot;
  if (l >= NL) return;
  T t[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) t[a] = -s.L.gl[a * NL + l];
  if (s.P.ng > 0)  // W_n^T x_n of the global nodes (k_border_backsub)
    for (int a = 0; a < 3; ++a) t[a] -= T(s.B.bl[a * NL + l]);
  for (int64_t i = s.S.lm_slot_off[l]; i < s.S.lm_slot_end[l]; ++i) {
    const T* xk = s.L.x + 15 * (int64_t)s.S.slot_kf[i];
    T xv[6], w[18];
#pragma unroll
    for (int c = 0; c < 6; ++c) xv[c] = xk[c];
    load_slot(s.L.Wslot + kSlotStride * i, w);
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      T acc = T(0);
#pragma unroll
      for (int c = 0; c < 6; ++c) acc += w[6 * x + c] * xv[c];
      t[x] -= acc;
    }
  }
  const bool act = s.P.lm_active[l];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    T v = T(0);
#pragma unroll
    for (int b = 0; b < 3; ++b) v += s.L.V[(3 * a + b) * NL + l] * t[b];
    s.L.dl[a * NL + l] = act ? (double)v : 0.0;
  }
}

// Switch back substitution: ds = (-g - W_f^T x_f - W_t^T x_t) / H.
template <typename T>
__global__ void __launch_bounds__(kB) k_backsub_switch(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= s.P.nsw) return;
  const int64_t e = s.P.sw_e[q], f = s.P.e_from[e], t = s.P.e_to[e];
  const T* W = s.L.swW + 30 * q;
  T u = -s.L.swg[q];
#pragma unroll
  for (int c = 0; c < 15; ++c) u -= W[c] * s.L.x[15 * f + c] + W[15 + c] * s.L.x[15 * t + c];
  s.L.swx[q] = (double)(u * s.L.swHi[q]);
}

// Model cost change -u.(r + u/2) with u = J du (unscaled J, du = s dx);
// u in T, the reduction in FP64.
template <typename T>
__global__ void __launch_bounds__(kB) k_model_visual(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t N = s.P.nobs, NL = s.P.nlm;
  double m = 0.0;
  if (i < N) {
    const int64_t l = s.P.obs_lm[i];
    T dl[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) dl[a] = s.L.slm[a * NL + l] * T(s.L.dl[a * NL + l]);
    T u[2] = {T(0), T(0)};
#pragma unroll
    for (int rr = 0; rr < 2; ++rr)
#pragma unroll
      for (int a = 0; a < 3; ++a) u[rr] += s.vis.Jl[(3 * rr + a) * N + i] * dl[a];
    if (s.P.obs_type[i] != MBA_LOCAL_KEYFRAME) {
      const int64_t ks = s.P.obs_store[i], ko = s.P.obs_kf[i];
      T xs[6], xo[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        xs[c] = s.L.skf[15 * ks + c] * s.L.x[15 * ks + c];
        xo[c] = s.L.skf[15 * ko + c] * s.L.x[15 * ko + c];
      }
#pragma unroll
      for (int rr = 0; rr < 2; ++rr)
#pragma unroll
        for (int c = 0; c < 6; ++c)
          u[rr] += s.vis.Js[(6 * rr + c) * N + i] * xs[c] + s.vis.Jo[(6 * rr + c) * N + i] * xo[c];
    }
    const double u0 = (double)u[0], u1 = (double)u[1];
    m = -(u0 * ((double)s.vis.r[i] + u0 / 2.0) + u1 * ((double)s.vis.r[N + i] + u1 / 2.0));
  }
  block_add(m, &s.ctl->model_change);
}

template <typename T>
__global__ void __launch_bounds__(128) k_model_inertial(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  double m = 0.0;
  const int q = (e < s.P.nedge && e >= s.P.nimu) ? s.P.pe_swi[e - s.P.nimu] : -1;
  if (e < s.P.nedge && lane < 15) {
    const int64_t f = s.P.e_from[e], t = s.P.e_to[e];
    T u = T(0);
#pragma unroll
    for (int c = 0; c < 15; ++c)
      u += s.ine.Jf[225 * e + 15 * lane + c] * s.L.skf[15 * f + c] * s.L.x[15 * f + c] +
           s.ine.Jt[225 * e + 15 * lane + c] * s.L.skf[15 * t + c] * s.L.x[15 * t + c];
    if (q >= 0 && lane < 6) u += s.ine.Js[6 * (e - s.P.nimu) + lane] * s.L.ssw[q] * T(s.L.swx[q]);
    const double ud = (double)u;
    m = -ud * ((double)s.ine.r[15 * e + lane] + ud / 2.0);
  } else if (q >= 0 && lane == 15) {  // switch prior: r = (1 - s) w, J = -w
    const double w = s.P.sw_w[q], ud = -w * s.sc.ssw[q] * s.L.swx[q];
    m = -ud * ((1.0 - s.P.sw[q]) * w + ud / 2.0);
  }
  block_add(m, &s.ctl->model_change);
}

// Retraction x_cand = Plus(x, s * dx) in FP64 (JplPoseParameterization,
// JplRollPitchQuaternionParameterization for the gauge keyframe).
template <typename T>
__global__ void __launch_bounds__(kB) k_retract(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double sn = 0.0, xn = 0.0;
  if (i < s.P.nkf) {
    const int64_t k = i;
    const uint16_t m = s.P.kf_mask[k];
    const double* x = s.P.kf_state + 16 * k;
    double* o = s.kf_cand + 16 * k;
    double d[15];
    for (int a = 0; a < 15; ++a) d[a] = ((m >> a) & 1) ? s.sc.skf[15 * k + a] * (double)s.L.x[15 * k + a] : 0.0;
    double q[4] = {x[0], x[1], x[2], x[3]};
    if (s.P.kf_flags[k] & MBA_KF_GAUGE_ROLL_PITCH) {
      if (m & 3) jpl_rollpitch_plus(s.P.mis + 8 * s.P.kf_mis[k], x, d, q);
    } else if (m & 7) {
      jpl_plus(x, d, q);
    }
    for (int a = 0; a < 4; ++a) o[a] = q[a];
    for (int a = 0; a < 12; ++a) o[4 + a] = x[4 + a] + d[3 + a];
    if (s.kf_cand_f)
      for (int a = 0; a < 7; ++a) s.kf_cand_f[8 * k + a] = (float)o[a];
    const bool pose_var = (m & 0x3f) != 0;
    if (pose_var)
      for (int a = 0; a < 7; ++a) { sn += (o[a] - x[a]) * (o[a] - x[a]); xn += x[a] * x[a]; }
    for (int blk = 0; blk < 3; ++blk)
      if ((m >> (6 + 3 * blk)) & 7)
        for (int a = 0; a < 3; ++a) { const double dd = o[7 + 3 * blk + a] - x[7 + 3 * blk + a]; sn += dd * dd; xn += x[7 + 3 * blk + a] * x[7 + 3 * blk + a]; }
  } else if (i < s.P.nkf + s.P.nlm) {
    const int64_t l = i - s.P.nkf, NL = s.P.nlm;
    const double* x = s.P.lm_p + 4 * l;
    double* o = s.lm_cand + 4 * l;
    const bool act = s.P.lm_active[l];
    for (int a = 0; a < 3; ++a) {
      const double d = act ? s.sc.slm[a * NL + l] * s.L.dl[a * NL + l] : 0.0;
      o[a] = x[a] + d;
      if (s.lm_cand_f) s.lm_cand_f[4 * l + a] = (float)o[a];
      if (act) { sn += d * d; xn += x[a] * x[a]; }
    }
    o[3] = 0.0;
  } else if (i < s.P.nkf + s.P.nlm + s.P.nsw) {
    // Switch: plain addition projected onto its bounds [0, 1].
    const int64_t q = i - s.P.nkf - s.P.nlm;
    const double x = s.P.sw[q], v = fmin(1.0, fmax(0.0, x + s.sc.ssw[q] * s.L.swx[q]));
    s.sw_cand[q] = v;
    sn += (v - x) * (v - x);
    xn += x * x;
  }
  block_add(sn, &s.ctl->step_norm2);
  block_add(xn, &s.ctl->x_norm2);
}

// The LM decision (single thread).
__global__ void k_decide(LmControl* ctl, LmParams prm, mba_iteration_summary* log) {
  if (ctl->terminated) return;
  if (ctl->fatal) {  // a bounded wait in a device pipeline ran out: stop (the host reports MBA_ERR_TIMEOUT)
    ctl->terminated = 1;
    ctl->termination = 7;
    return;
  }
  const int it = ++ctl->iteration;
  const double mcc = ctl->model_change;
  const double cost = ctl->cost;
  double new_cost = ctl->cost_cand + ctl->cost_cand_ine;
  if (ctl->nonfinite || ctl->inertial_status || !isfinite(new_cost)) new_cost = INFINITY;
  const bool valid = ctl->status == 0 && mcc > 0.0 && isfinite(mcc);
  int ok = 0;
  double rel = 0.0;
  const double step_norm = sqrt(ctl->step_norm2), x_norm = sqrt(ctl->x_norm2);
  if (valid) {
    rel = (cost - new_cost) / mcc;
    ok = isfinite(new_cost) && rel > prm.min_relative_decrease;
    if (prm.check_tolerances && step_norm <= prm.parameter_tolerance * (x_norm + prm.parameter_tolerance)) {
      ctl->terminated = 1;
      ctl->termination = 3;
    } else if (prm.check_tolerances && fabs(cost - new_cost) <= prm.function_tolerance * cost) {
      ctl->terminated = 1;
      ctl->termination = 1;
    }
  }
  if (ok) {
    ctl->cost = new_cost;
    ctl->cost_ine = ctl->cost_cand_ine;
    ctl->num_successful++;
    if (!ctl->terminated) {
      double r = ctl->radius / fmax(1.0 / 3.0, 1.0 - pow(2.0 * rel - 1.0, 3.0));
      ctl->radius = fmin(r, prm.max_radius);
      ctl->decrease_factor = 2.0;
    }
  } else if (!ctl->terminated) {
    ctl->radius /= ctl->decrease_factor;
    ctl->decrease_factor *= 2.0;
  }
  ctl->accepted = ok;
  ctl->total_pcg += ctl->pcg_iters;
  if (prm.stop_cost > 0.0 && ctl->cost <= prm.stop_cost && ctl->stop_iteration < 0) {
    ctl->stop_iteration = it;
    if (!ctl->terminated) { ctl->terminated = 1; ctl->termination = 6; }
  }
  if (!ctl->terminated && ctl->radius < prm.min_radius) { ctl->terminated = 1; ctl->termination = 4; }
  if (!ctl->terminated && it >= prm.max_num_iterations) { ctl->terminated = 1; ctl->termination = 0; }
  // maplab's outlier-rejection solve restarts every n iterations (not after the last one).
  ctl->restart_now = !ctl->terminated && prm.reject_every > 0 && it % prm.reject_every == 0;
  if (log && it <= prm.max_num_iterations) {
    mba_iteration_summary& e = log[it];
    e.iteration = it;
    e.step_is_successful = ok;
    e.linear_solver_iterations = ctl->pcg_iters;
    e.cost = ctl->cost;
    e.cost_change = valid ? cost - new_cost : 0.0;
    e.gradient_max_norm = 0.0;
    e.step_norm = step_norm;
    e.relative_decrease = rel;
    e.trust_region_radius = ctl->radius;
    unsigned long long now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    e.iteration_time_ms = ctl->t0_ns ? (double)(now - ctl->t0_ns) * 1e-6 : 0.0;
  }
}

// Accepted step: candidate state and inertial linearization become current.
template <typename T>
__global__ void __launch_bounds__(kB) k_accept(SolverLaunch<T> s, InertialLin<double> cand, InertialLin<double> cur) {
  if (!s.ctl->accepted) return;
  const int64_t nk = 16 * s.P.nkf, nl = 4 * s.P.nlm, ne1 = 15 * s.P.nedge, ne2 = 225 * s.P.nedge;
  const int64_t total = nk + nl + ne1 + 2 * ne2;
  const int64_t ns = s.P.nsw, nj = 6 * (s.P.nedge - s.P.nimu);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total + ns + nj;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i >= total) {
      const int64_t j = i - total;
      if (j < ns) {
        s.P.sw[j] = s.sw_cand[j];
      } else if (cand.Js) {
        cur.Js[j - ns] = cand.Js[j - ns];
        s.ine.Js[j - ns] = T(cand.Js[j - ns]);
      }
      continue;
    }
    if (i < nk) {
      const double v = s.kf_cand[i];
      s.P.kf_state[i] = v;
      if ((i & 15) < 7) s.P.kf_pose_f[8 * (i >> 4) + (i & 15)] = (float)v;  // FP32 mirror
    } else if (i < nk + nl) {
      const double v = s.lm_cand[i - nk];
      s.P.lm_p[i - nk] = v;
      s.P.lm_p_f[i - nk] = (float)v;
    } else if (i < nk + nl + ne1) {
      const int64_t j = i - nk - nl;
      cur.r[j] = cand.r[j];
      s.ine.r[j] = T(cand.r[j]);
    } else if (i < nk + nl + ne1 + ne2) {
      const int64_t j = i - nk - nl - ne1;
      cur.Jf[j] = cand.Jf[j];
      s.ine.Jf[j] = T(cand.Jf[j]);
    } else {
      const int64_t j = i - nk - nl - ne1 - ne2;
      cur.Jt[j] = cand.Jt[j];
      s.ine.Jt[j] = T(cand.Jt[j]);
    }
  }
}

__global__ void k_init_control(LmControl* ctl, double radius) {
  ctl->radius = radius;
  ctl->decrease_factor = 2.0;
  ctl->accepted = 0;
  ctl->terminated = 0;
  ctl->termination = 0;
  ctl->iteration = 0;
  ctl->num_successful = 0;
  ctl->total_pcg = 0;
  ctl->status = 0;
  ctl->stop_iteration = -1;
  ctl->rejected = 0;
  ctl->reject_count = 0;
  ctl->cost_ine = 0.0;
  ctl->cost_cand_ine = 0.0;
  ctl->fatal = 0;
}

__global__ void k_add_inertial_cost(LmControl* ctl) { ctl->cost += ctl->cost_ine; }

template <typename T>
__global__ void k_copy_cast(const double* a, T* b, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = T(a[i]);
}

inline unsigned nblk(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }
inline unsigned gridcap(int64_t n) {
  const int64_t b = (n + kB - 1) / kB;
  return (unsigned)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

}  // namespace

cudaError_t solver_init_control(LmControl* ctl, double radius, cudaStream_t st) {
  k_init_control<<<1, 1, 0, st>>>(ctl, radius);
  return cudaGetLastError();
}

cudaError_t solver_add_inertial_cost(LmControl* ctl, cudaStream_t st) {
  k_add_inertial_cost<<<1, 1, 0, st>>>(ctl);
  return cudaGetLastError();
}

template <typename T>
cudaError_t solver_assemble(const SolverLaunch<T>& s, const int* gate, cudaStream_t st) {
  const int* skip = gate ? &s.ctl->terminated : nullptr;
  k_zero<T><<<gridcap(225 * s.P.nkf), kB, 0, st>>>(s.L.Dbase, 225 * s.P.nkf, gate, skip);
  k_zero<T><<<gridcap(15 * s.P.nkf), kB, 0, st>>>(s.L.gc, 15 * s.P.nkf, gate, skip);
  if (s.S.npu) k_zero<T><<<gridcap(36 * s.S.npu), kB, 0, st>>>(s.L.Pbase, 36 * s.S.npu, gate, skip);
  if constexpr (sizeof(T) == 4) {
    k_zero<float><<<gridcap(kPoseUp * s.P.nkf), kB, 0, st>>>(s.L.Dpose, kPoseUp * s.P.nkf, gate, skip);
    k_zero<float><<<gridcap(8 * s.P.nkf), kB, 0, st>>>(s.L.gpose, 8 * s.P.nkf, gate, skip);
  }
  // Relinearizations inside the LM loop (gate set) assemble with the fixed
  // Jacobi scale applied; the first assembly is scaled by solver_compute_scale.
  const int scaled = gate ? 1 : 0;
  if (s.P.nlm) k_assemble_lm<T><<<nblk(s.P.nlm, kB), kB, 0, st>>>(s.P, s.S, s.vis, s.L, scaled, gate, skip);
  if (s.P.nedge)
    k_assemble_inertial<T><<<nblk(32 * s.P.nedge, 128), 128, 0, st>>>(s.P, s.ine, s.L, scaled, gate, skip);
  if constexpr (sizeof(T) == 4)
    k_merge_pose<<<nblk(27 * s.P.nkf, kB), kB, 0, st>>>(s.P.nkf, s.L.Dpose, s.L.gpose, s.L.Dbase, s.L.gc, gate, skip);
  k_mirror_pose_blocks<T><<<nblk(15 * s.P.nkf, kB), kB, 0, st>>>(s.P.nkf, s.L.Dbase, gate, skip);
  if constexpr (sizeof(T) == 8)
    if (s.P.ng > 0) {
      const cudaError_t e = border_assemble(s, gate, skip, st);
      if (e != cudaSuccess) return e;
    }
  return cudaGetLastError();
}

template <typename T>
cudaError_t solver_compute_scale(const SolverLaunch<T>& s, int jacobi, cudaStream_t st) {
  const int64_t n = 15 * s.P.nkf + 3 * s.P.nlm + s.P.nsw;
  k_scale<T><<<nblk(n, kB), kB, 0, st>>>(s.P, s.L, s.sc, jacobi, nullptr);
  const int64_t m = 12 * s.P.nlm + 240 * s.P.nkf + 36 * s.S.npu + 225 * s.P.nedge + 32 * s.P.nsw;
  k_scale_inplace<T><<<gridcap(m), kB, 0, st>>>(s.P, s.S, s.L, nullptr, nullptr);
  if (s.S.nslot) k_scale_slots<T><<<nblk(s.S.nslot, kB), kB, 0, st>>>(s.P, s.S, s.L, nullptr, nullptr);
  if constexpr (sizeof(T) == 8)
    if (s.P.ng > 0) {
      const cudaError_t e = border_scale(s, jacobi, nullptr, st);
      if (e != cudaSuccess) return e;
    }
  return cudaGetLastError();
}

// Max |J^T r| of the current assembly (unscaled: the assembled gradients are
// scaled by the Jacobi scale) over the variable dims: keyframes, landmarks,
// switch variables and global nodes (whose gradient is kept unscaled).
template <typename T>
__global__ void __launch_bounds__(kB) k_gradient_max(SolverLaunch<T> s, const int* run_if) {
  if (s.ctl->terminated || (run_if && !*run_if)) return;
  const int64_t NK = s.P.nkf, NL = s.P.nlm, nk = 15 * NK, nl = 3 * NL, nn = 15 * s.P.ng;
  double m = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk + nl + s.P.nsw + nn;
       i += (int64_t)gridDim.x * blockDim.x) {
    double g = 0.0;
    if (i < nk) {
      if ((s.P.kf_mask[i / 15] >> (i % 15)) & 1) g = (double)s.L.gc[i] / s.sc.skf[i];
    } else if (i < nk + nl) {
      const int64_t j = i - nk, l = j % NL;
      if (s.P.lm_active[l] && !s.P.lm_off[l]) g = (double)s.L.gl[j] / s.sc.slm[j];
    } else if (i < nk + nl + s.P.nsw) {
      const int64_t q = i - nk - nl;
      g = (double)s.L.swg[q] / s.sc.ssw[q];
    } else {
      const int64_t j = i - nk - nl - s.P.nsw;
      if ((s.P.g_mask[j / 15] >> (j % 15)) & 1) g = s.B.gg[j];
    }
    m = fmax(m, fabs(g));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(&s.ctl->grad_max_bits, (unsigned long long)__double_as_longlong(m));
}

__global__ void k_gradient_reset(LmControl* ctl, const int* run_if) {
  if (run_if && !*run_if) return;
  ctl->grad_max_bits = 0ull;
}

__global__ void k_gradient_decide(LmControl* ctl, LmParams prm, const int* run_if) {
  if (ctl->terminated || (run_if && !*run_if) || !prm.check_tolerances) return;
  if (__longlong_as_double((long long)ctl->grad_max_bits) <= prm.gradient_tolerance) {
    ctl->terminated = 1;
    ctl->termination = 2;
  }
}

template <typename T>
cudaError_t solver_gradient_check(const SolverLaunch<T>& s, const int* run_if, cudaStream_t st) {
  k_gradient_reset<<<1, 1, 0, st>>>(s.ctl, run_if);
  const int64_t n = 15 * s.P.nkf + 3 * s.P.nlm + s.P.nsw + 15 * s.P.ng;
  k_gradient_max<T><<<gridcap(n), kB, 0, st>>>(s, run_if);
  k_gradient_decide<<<1, 1, 0, st>>>(s.ctl, s.prm, run_if);
  return cudaGetLastError();
}

template <typename T>
cudaError_t solver_build_reduced(const SolverLaunch<T>& s, cudaStream_t st) {
  const int64_t nsys = 225 * s.P.nkf + 225 * s.P.nedge + 36 * s.S.npu + 15 * s.P.nkf;
  k_build_system<T><<<gridcap(nsys), kB, 0, st>>>(s);
  if constexpr (sizeof(T) == 8)
    if (s.P.ng > 0) {
      const cudaError_t e = border_build(s, st);
      if (e != cudaSuccess) return e;
    }
  if (s.P.nlm) k_schur_lm<T><<<nblk(s.P.nlm, kB), kB, 0, st>>>(s);
  if (s.S.nslot) k_schur_slot<T><<<nblk(s.S.nslot, kB), kB, 0, st>>>(s);
  if (s.S.nchunk) {
    const cudaError_t e = launch_schur_pairs<T>(s, st);
    if (e != cudaSuccess) return e;
  }
  if (s.P.nsw) k_schur_switch<T><<<nblk(32 * s.P.nsw, 128), 128, 0, st>>>(s);
  k_finalize_system<T><<<gridcap(nsys), kB, 0, st>>>(s);
  if constexpr (sizeof(T) == 8)
    if (s.P.ng > 0) {
      const cudaError_t e = border_schur_and_finalize(s, st);
      if (e != cudaSuccess) return e;
    }
  // Block-Jacobi inverses of the keyframe blocks and of the global nodes' diagonal blocks.
  k_block_jacobi<T><<<nblk(s.P.nkf + s.P.ng, 64), 64, 0, st>>>(s);
  if (s.precond != MBA_PRECOND_BLOCK_JACOBI) {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && s.precond == MBA_PRECOND_LEARNED) e = gnn_forward<T>(s, s.gg, s.gp, s.gw, st);
    if (e != cudaSuccess) return e;
    return chain_factor<T>(s, st);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t solver_prepare(const SchurPattern& S) {
  int64_t cap = 0;
  const int64_t bytes = schur_pairs_smem<T>(S, false, &cap);  // the larger of the two kernels' sizes
  cudaError_t e = chain_prepare<T>();
  if (e != cudaSuccess || bytes <= 48 * 1024) return e;
  // both Schur pair kernels, at the larger of their shared-memory sizes
  e = cudaFuncSetAttribute(k_schur_pairs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_schur_pairs_split<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return e;
}

template <typename T>
cudaError_t solver_schur_pairs(const SolverLaunch<T>& s, cudaStream_t st) {
  return launch_schur_pairs<T>(s, st);
}

// One PCG product (after the PCG start) on the current reduced system, for
// timing the two product kernels.
template <typename T>
cudaError_t solver_product(const SolverLaunch<T>& s, bool sym, cudaStream_t st) {
  k_pcg_init<T><<<nblk(15 * (s.P.nkf + s.P.ng), kB), kB, 0, st>>>(s);
  if (sym) {
    k_pcg_spmv_sym<T><<<nblk(32 * s.P.nkf, 128), 128, 0, st>>>(s, 0, s.L.p, s.L.q2);
    k_pcg_pq<T><<<nblk(15 * s.P.nkf, kB), kB, 0, st>>>(s, 0, s.L.q2);
  } else {
    k_pcg_spmv<T><<<nblk(32 * s.P.nkf, 128), 128, 0, st>>>(s, 0, s.L.p, s.L.q2);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t solver_step(const SolverLaunch<T>& s, cudaStream_t st) {
  cudaError_t e = solver_build_reduced<T>(s, st);
  if (e != cudaSuccess) return e;
  const int64_t nb = s.P.nkf + s.P.ng;  // keyframe blocks, then the global nodes
  const int64_t n = 15 * nb;
  k_pcg_init<T><<<nblk(n, kB), kB, 0, st>>>(s);
  const bool chain = s.precond != MBA_PRECOND_BLOCK_JACOBI;
  if (chain) {
    e = chain_apply<T>(s, s.L.r, s.L.z, &s.ctl->pcg_rz0, st);
    if (e != cudaSuccess) return e;
  }
  const int maxit = s.prm.max_linear_iterations;
  for (int it = 0; it < maxit; ++it) {
    T* pa = (it & 1) ? s.L.q2 : s.L.p;
    T* pb = (it & 1) ? s.L.p : s.L.q2;
    if (s.S.spmv_sym && s.P.ng == 0) {
      k_pcg_spmv_sym<T><<<nblk(32 * s.P.nkf, 128), 128, 0, st>>>(s, it, pa, pb);
      k_pcg_pq<T><<<nblk(15 * s.P.nkf, kB), kB, 0, st>>>(s, it, pb);
    } else {
      k_pcg_spmv<T><<<nblk(32 * s.P.nkf, 128), 128, 0, st>>>(s, it, pa, pb);
    }
    if constexpr (sizeof(T) == 8)
      if (s.P.ng > 0) {
        e = border_spmv(s, it, pa, pb, st);
        if (e != cudaSuccess) return e;
      }
    k_pcg_update<T><<<nblk(16 * nb, kB), kB, 0, st>>>(s, it, pb, it == maxit - 1);
    if (chain) {
      e = chain_apply<T>(s, s.L.r, s.L.z, &s.ctl->pcg_rz[it % 3], st);
      if (e != cudaSuccess) return e;
    }
  }
  if constexpr (sizeof(T) == 8)
    if (s.P.ng > 0) {
      e = border_backsub(s, st);
      if (e != cudaSuccess) return e;
    }
  if (s.P.nlm) k_backsub<T><<<nblk(s.P.nlm, kB), kB, 0, st>>>(s);
  if (s.P.nsw) k_backsub_switch<T><<<nblk(s.P.nsw, kB), kB, 0, st>>>(s);
  bool model_done = false;
  if constexpr (sizeof(T) == 8)
    if (s.P.ng > 0) {
      e = border_model_visual(s, st);
      if (e != cudaSuccess) return e;
      model_done = true;
    }
  if (s.P.nobs && !model_done) k_model_visual<T><<<nblk(s.P.nobs, kB), kB, 0, st>>>(s);
  if (s.P.nedge) k_model_inertial<T><<<nblk(32 * s.P.nedge, 128), 128, 0, st>>>(s);
  k_retract<T><<<nblk(s.P.nkf + s.P.nlm + s.P.nsw, kB), kB, 0, st>>>(s);
  if constexpr (sizeof(T) == 8)
    if (s.P.ng > 0) {
      e = border_retract(s, st);
      if (e != cudaSuccess) return e;
    }
  return cudaGetLastError();
}

template <typename T>
cudaError_t solver_evaluate_candidate(const SolverLaunch<T>& s, InertialLin<double> ine_cand, cudaStream_t st) {
  // Global nodes: the candidate cameras and baseframes.
  DevProblem Pc = s.P;
  if (s.P.ng > 0) {
    Pc.cams = s.B.cams_cand;
    Pc.mis = s.B.mis_cand;
  }
  // Mixed path: FP32 residuals from FP32 copies of the candidate, FP64 sum.
  cudaError_t e = (sizeof(T) == 4 && s.kf_cand_f)
                      ? launch_visual_cost_f32(s.P, s.kf_cand_f, s.lm_cand_f, &s.ctl->cost_cand, &s.ctl->nonfinite,
                                               &s.ctl->terminated, st)
                      : launch_visual_cost_gated(Pc, s.kf_cand, s.lm_cand, &s.ctl->cost_cand, &s.ctl->nonfinite,
                                                 &s.ctl->terminated, st);
  if (e != cudaSuccess) return e;
  // Mixed path: Phi / Q propagated in FP32 (state, Cholesky, residual FP64).
  return launch_inertial_gated(s.P, s.kf_cand, ine_cand, &s.ctl->cost_cand_ine, &s.ctl->inertial_status,
                               &s.ctl->terminated, st, sizeof(T) == 4, s.sw_cand);
}

template <typename T>
cudaError_t solver_decide_and_accept(const SolverLaunch<T>& s, InertialLin<double> ine_cand,
                                     InertialLin<double> ine_cur, cudaStream_t st) {
  k_decide<<<1, 1, 0, st>>>(s.ctl, s.prm, s.log);
  const int64_t total = 16 * s.P.nkf + 4 * s.P.nlm + 465 * s.P.nedge + s.P.nsw + 6 * (s.P.nedge - s.P.nimu);
  k_accept<T><<<gridcap(total), kB, 0, st>>>(s, ine_cand, ine_cur);
  if constexpr (sizeof(T) == 8)
    if (s.P.ng > 0) {
      const cudaError_t e = border_accept(s, st);
      if (e != cudaSuccess) return e;
    }
  return cudaGetLastError();
}

template <typename T>
cudaError_t solver_relinearize(const SolverLaunch<T>& s, const InertialLin<double>& ine_cur, cudaStream_t st) {
  (void)ine_cur;
  cudaError_t e = launch_visual_linearize_gated<T>(s.P, s.vis, nullptr, &s.ctl->accepted, &s.ctl->terminated, st);
  if (e != cudaSuccess) return e;
  e = solver_assemble<T>(s, &s.ctl->accepted, st);
  if (e != cudaSuccess) return e;
  // Ceres' gradient test after an accepted step.
  return solver_gradient_check<T>(s, &s.ctl->accepted, st);
}

// Outlier rejection + restart, run when ctl->restart_now (set by k_decide).
__global__ void k_restart_begin(LmControl* ctl) {
  if (!ctl->restart_now) return;
  ctl->cost = 0.0;
  ctl->reject_count = 0;
}

__global__ void k_restart_end(LmControl* ctl) {
  if (!ctl->restart_now) return;
  ctl->cost += ctl->cost_ine;
  ctl->decrease_factor = 2.0;
  ctl->rejected += ctl->reject_count;
}

template <typename T>
cudaError_t solver_reject_and_restart(const SolverLaunch<T>& s, int use_reprojection, double max_px, int jacobi,
                                      cudaStream_t st) {
  LmControl* c = s.ctl;
  const int* run = &c->restart_now;
  k_restart_begin<<<1, 1, 0, st>>>(c);
  // The mixed path tests and costs in FP32 from the state's FP32 copies, as
  // its candidates are costed (one precision on both sides of the gain ratio).
  constexpr bool f32 = sizeof(T) == 4;
  cudaError_t e = launch_find_outliers(s.P, use_reprojection, max_px, &c->reject_count, run, nullptr, st, f32);
  if (e == cudaSuccess)
    e = f32 ? launch_visual_cost_f32(s.P, s.P.kf_pose_f, s.P.lm_p_f, &c->cost, nullptr, nullptr, st, run)
            : launch_visual_cost_gated(s.P, s.P.kf_state, s.P.lm_p, &c->cost, nullptr, nullptr, st, run);
  if (e != cudaSuccess) return e;
  k_restart_end<<<1, 1, 0, st>>>(c);
  e = launch_visual_linearize_gated<T>(s.P, s.vis, nullptr, run, nullptr, st);
  if (e != cudaSuccess) return e;
  // Fresh assembly and Jacobi scaling (the restarted Ceres solve rescales).
  k_zero<T><<<gridcap(225 * s.P.nkf), kB, 0, st>>>(s.L.Dbase, 225 * s.P.nkf, run, nullptr);
  k_zero<T><<<gridcap(15 * s.P.nkf), kB, 0, st>>>(s.L.gc, 15 * s.P.nkf, run, nullptr);
  if (s.S.npu) k_zero<T><<<gridcap(36 * s.S.npu), kB, 0, st>>>(s.L.Pbase, 36 * s.S.npu, run, nullptr);
  if constexpr (sizeof(T) == 4) {
    k_zero<float><<<gridcap(kPoseUp * s.P.nkf), kB, 0, st>>>(s.L.Dpose, kPoseUp * s.P.nkf, run, nullptr);
    k_zero<float><<<gridcap(8 * s.P.nkf), kB, 0, st>>>(s.L.gpose, 8 * s.P.nkf, run, nullptr);
  }
  if (s.P.nlm) k_assemble_lm<T><<<nblk(s.P.nlm, kB), kB, 0, st>>>(s.P, s.S, s.vis, s.L, 0, run, nullptr);
  if (s.P.nedge) k_assemble_inertial<T><<<nblk(32 * s.P.nedge, 128), 128, 0, st>>>(s.P, s.ine, s.L, 0, run, nullptr);
  if constexpr (sizeof(T) == 4)
    k_merge_pose<<<nblk(27 * s.P.nkf, kB), kB, 0, st>>>(s.P.nkf, s.L.Dpose, s.L.gpose, s.L.Dbase, s.L.gc, run,
                                                        nullptr);
  k_mirror_pose_blocks<T><<<nblk(15 * s.P.nkf, kB), kB, 0, st>>>(s.P.nkf, s.L.Dbase, run, nullptr);
  const int64_t n = 15 * s.P.nkf + 3 * s.P.nlm + s.P.nsw;
  k_scale<T><<<nblk(n, kB), kB, 0, st>>>(s.P, s.L, s.sc, jacobi, run);
  const int64_t m = 12 * s.P.nlm + 240 * s.P.nkf + 36 * s.S.npu + 225 * s.P.nedge + 32 * s.P.nsw;
  k_scale_inplace<T><<<gridcap(m), kB, 0, st>>>(s.P, s.S, s.L, run, nullptr);
  if (s.S.nslot) k_scale_slots<T><<<nblk(s.S.nslot, kB), kB, 0, st>>>(s.P, s.S, s.L, run, nullptr);
  if constexpr (sizeof(T) == 8)
    if (s.P.ng > 0) {
      e = border_assemble(s, run, nullptr, st);
      if (e == cudaSuccess) e = border_scale(s, jacobi, run, st);
      if (e != cudaSuccess) return e;
    }
  return cudaGetLastError();
}

__global__ void k_loop_start(LmControl* ctl) {
  unsigned long long now;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
  ctl->t0_ns = now;
}

__global__ void k_loop_control(LmControl* ctl, cudaGraphConditionalHandle handle, const volatile int* cancel) {
  if (!ctl->terminated && cancel && *cancel) {
    ctl->terminated = 1;
    ctl->termination = 5;
  }
  ctl->loop_active = !ctl->terminated;
  cudaGraphSetConditional(handle, ctl->terminated ? 0u : 1u);
}

cudaError_t solver_loop_start(LmControl* ctl, cudaStream_t st) {
  k_loop_start<<<1, 1, 0, st>>>(ctl);
  return cudaGetLastError();
}

cudaError_t solver_loop_control(LmControl* ctl, cudaGraphConditionalHandle handle, const volatile int* cancel,
                                cudaStream_t st) {
  k_loop_control<<<1, 1, 0, st>>>(ctl, handle, cancel);
  return cudaGetLastError();
}

template cudaError_t solver_assemble<double>(const SolverLaunch<double>&, const int*, cudaStream_t);
template cudaError_t solver_assemble<float>(const SolverLaunch<float>&, const int*, cudaStream_t);
template cudaError_t solver_compute_scale<double>(const SolverLaunch<double>&, int, cudaStream_t);
template cudaError_t solver_compute_scale<float>(const SolverLaunch<float>&, int, cudaStream_t);
template cudaError_t solver_build_reduced<double>(const SolverLaunch<double>&, cudaStream_t);
template cudaError_t solver_build_reduced<float>(const SolverLaunch<float>&, cudaStream_t);
template cudaError_t solver_prepare<double>(const SchurPattern&);
template cudaError_t solver_prepare<float>(const SchurPattern&);
template cudaError_t solver_schur_pairs<double>(const SolverLaunch<double>&, cudaStream_t);
template cudaError_t solver_schur_pairs<float>(const SolverLaunch<float>&, cudaStream_t);
template cudaError_t solver_step<double>(const SolverLaunch<double>&, cudaStream_t);
template cudaError_t solver_product<double>(const SolverLaunch<double>&, bool, cudaStream_t);
template cudaError_t solver_product<float>(const SolverLaunch<float>&, bool, cudaStream_t);
template cudaError_t solver_step<float>(const SolverLaunch<float>&, cudaStream_t);
template cudaError_t solver_evaluate_candidate<double>(const SolverLaunch<double>&, InertialLin<double>, cudaStream_t);
template cudaError_t solver_evaluate_candidate<float>(const SolverLaunch<float>&, InertialLin<double>, cudaStream_t);
template cudaError_t solver_decide_and_accept<double>(const SolverLaunch<double>&, InertialLin<double>,
                                                      InertialLin<double>, cudaStream_t);
template cudaError_t solver_decide_and_accept<float>(const SolverLaunch<float>&, InertialLin<double>,
                                                     InertialLin<double>, cudaStream_t);
template cudaError_t solver_relinearize<double>(const SolverLaunch<double>&, const InertialLin<double>&, cudaStream_t);
template cudaError_t solver_relinearize<float>(const SolverLaunch<float>&, const InertialLin<double>&, cudaStream_t);
template cudaError_t solver_reject_and_restart<double>(const SolverLaunch<double>&, int, double, int, cudaStream_t);
template cudaError_t solver_reject_and_restart<float>(const SolverLaunch<float>&, int, double, int, cudaStream_t);
template cudaError_t solver_gradient_check<double>(const SolverLaunch<double>&, const int*, cudaStream_t);
template cudaError_t solver_gradient_check<float>(const SolverLaunch<float>&, const int*, cudaStream_t);

}  // namespace mba
