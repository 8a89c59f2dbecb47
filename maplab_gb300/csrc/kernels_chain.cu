// Chain preconditioner: block cyclic reduction of the block-tridiagonal
// matrix T formed by the keyframe chains of the reduced camera system.
//
// Chain positions p = 0..n-1 (all chains end to end, no coupling across chain
// ends).  Level l (stride s = 2^l) eliminates positions p = s (mod 2s) and
// keeps p = 0 (mod 2s); position 0 is the last survivor.  Elimination of p
// stores F = T_l(p,p)^-1 (FP64 Cholesky), the couplings CL = T_l(p, p-s),
// CR = T_l(p, p+s) and the products XL = T_l(p-s, p) F, XR = T_l(p+s, p) F;
// the survivors q take T(q,q) -= XR(q-s) CR(q-s) + XL(q+s) CL(q+s) and the
// new coupling T(q, q-2s) = -XR(q-s) CL(q-s).
//
// Solve T z = r: forward sweep w(q) -= XR(q-s) w(q-s) + XL(q+s) w(q+s) level
// by level, z(0) = F(0) w(0), back sweep z(p) = F(p) (w(p) - CL(p) z(p-s) -
// CR(p) z(p+s)).  The levels with at most kTailNodes active positions run in
// one block (one launch) instead of one launch per level.
//
// Segmented sweeps (chain_seg = m > 0): block j owns positions
// [j 2^m, (j+1) 2^m) and runs the forward levels 0..m-1 in shared memory.
// The first position q of a segment is a survivor of all those levels and
// nobody reads its w before level m, so its left-neighbour terms
// sum_l XR(q - 2^l) w(q - 2^l) (positions of the previous segment, final once
// that segment is swept) are left in lc and subtracted by the tail, which runs
// levels m.. in one block.  The back sweep of levels m-1..0 again runs per
// segment.  Three launches per apply instead of one per level.
#include <cuda_runtime.h>

#include "solver.h"

namespace mba {
namespace {

constexpr int kCW = 4;           // warps per block in the factorization kernels
constexpr int kTailThreads = 1024;

__device__ __forceinline__ double wsum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void block_add_d(double v, double* acc) {
  __shared__ double red[32];
  v = wsum_d(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    v = wsum_d(v);
    if (lane == 0 && v != 0.0) atomicAdd(acc, v);
  }
}

__device__ __forceinline__ bool apply_gate(const LmControl* c) {
  return c->terminated || c->pcg_done || c->status || c->chain_failed;
}

// ---- warp-level 15x15 FP64 helpers (row-major blocks in shared memory)

// C = alpha op(A) op(B) (+ C if acc).  C must not alias A or B.
__device__ void w_gemm(const double* A, bool ta, const double* B, bool tb, double* C, double alpha, bool acc) {
  const int lane = threadIdx.x & 31;
  for (int idx = lane; idx < 225; idx += 32) {
    const int r = idx / 15, c = idx - 15 * (idx / 15);
    double v = 0.0;
#pragma unroll
    for (int q = 0; q < 15; ++q) v += (ta ? A[15 * q + r] : A[15 * r + q]) * (tb ? B[15 * c + q] : B[15 * q + c]);
    C[idx] = acc ? C[idx] + alpha * v : alpha * v;
  }
  __syncwarp();
}

__device__ void w_load(const double* g, double* sm, bool transpose = false) {
  const int lane = threadIdx.x & 31;
  for (int idx = lane; idx < 225; idx += 32) {
    const int r = idx / 15, c = idx - 15 * (idx / 15);
    sm[idx] = transpose ? g[15 * c + r] : g[idx];
  }
  __syncwarp();
}

template <typename T>
__device__ void w_store(const double* sm, double* g64, T* gt) {
  const int lane = threadIdx.x & 31;
  for (int idx = lane; idx < 225; idx += 32) {
    g64[idx] = sm[idx];
    if ((void*)gt != (void*)g64) gt[idx] = T(sm[idx]);
  }
}

__device__ void w_zero(double* sm) {
  const int lane = threadIdx.x & 31;
  for (int idx = lane; idx < 225; idx += 32) sm[idx] = 0.0;
  __syncwarp();
}

// F = A^-1 for SPD A (symmetrized); A and X are scratch.  Returns false if a
// pivot is not positive (F is then the identity).
__device__ bool w_spd_inverse(double* A, double* X, double* F) {
  const int lane = threadIdx.x & 31;
  bool ok = true;
  // Lower triangle <- (A + A^T) / 2; the factorization reads only that.
  for (int idx = lane; idx < 225; idx += 32) {
    const int i = idx / 15, k = idx - 15 * (idx / 15);
    if (k < i) X[idx] = 0.5 * (A[idx] + A[15 * k + i]);
  }
  __syncwarp();
  for (int idx = lane; idx < 225; idx += 32) {
    const int i = idx / 15, k = idx - 15 * (idx / 15);
    if (k < i) A[idx] = X[idx];
  }
  __syncwarp();
  for (int j = 0; j < 15; ++j) {
    const double d = A[16 * j];
    if (!(d > 0.0) || !isfinite(d)) ok = false;
    const double ljj = ok ? sqrt(d) : 1.0;
    __syncwarp();
    if (lane > j && lane < 15) A[15 * lane + j] /= ljj;
    __syncwarp();
    if (lane == 0) A[16 * j] = ljj;
    for (int idx = lane; idx < 225; idx += 32) {
      const int i = idx / 15, k = idx - 15 * (idx / 15);
      if (i > j && k > j && k <= i) A[idx] -= A[15 * i + j] * A[15 * k + j];
    }
    __syncwarp();
  }
  if (!ok) {
    for (int idx = lane; idx < 225; idx += 32) F[idx] = (idx % 16 == 0) ? 1.0 : 0.0;
    __syncwarp();
    return false;
  }
  // X = L^-1 (lower), one column per lane.
  if (lane < 15) {
    const int c = lane;
    for (int i = 0; i < 15; ++i) {
      double v = (i == c) ? 1.0 : 0.0;
      for (int q = c; q < i; ++q) v -= A[15 * i + q] * X[15 * q + c];
      X[15 * i + c] = (i < c) ? 0.0 : v / A[16 * i];
    }
  }
  __syncwarp();
  // F = X^T X.
  for (int idx = lane; idx < 225; idx += 32) {
    const int a = idx / 15, b = idx - 15 * (idx / 15);
    double v = 0.0;
    for (int q = (a > b ? a : b); q < 15; ++q) v += X[15 * q + a] * X[15 * q + b];
    F[idx] = v;
  }
  __syncwarp();
  return true;
}

// ---- factorization

// T's level-0 blocks.  One warp per position.
template <typename T>
__global__ void __launch_bounds__(32 * kCW) k_chain_init(SolverLaunch<T> s) {
  if (s.ctl->terminated) return;
  const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t n = s.P.nkf;
  if (p >= n) return;
  const int64_t k = s.S.chain_perm[p];
  const double ge = s.C.coef[3 * p], gv = s.C.coef[3 * p + 1], al = s.C.coef[3 * p + 2];
  double* A = s.C.A + 225 * p;
  double* B = s.C.B + 225 * p;
  const T* D = s.L.SD + 225 * k;
  for (int idx = lane; idx < 225; idx += 32) A[idx] = (double)D[idx];
  // Diagonal compensation: alpha * sum of |S| over the off-chain pose blocks of row k.
  // Only the learned coefficients use it (alpha = 0 and no gradient for the
  // fixed chain), so the fixed chain skips the pass over the row's blocks.
  if (s.precond == MBA_PRECOND_LEARNED) {
    const bool ll = p > 0 && (s.S.link_edge[p] >= 0 || s.S.link_blk[p] >= 0);
    const bool lr = p + 1 < n && (s.S.link_edge[p + 1] >= 0 || s.S.link_blk[p + 1] >= 0);
    const int64_t kl = ll ? s.S.chain_perm[p - 1] : -1, kr = lr ? s.S.chain_perm[p + 1] : -1;
    double c = 0.0;
    const int r = lane / 5, part = lane - 5 * (lane / 5);  // 6 rows x 5 lanes
    if (r < 6) {
      for (int64_t e = s.S.row_off[k] + part; e < s.S.row_off[k + 1]; e += 5) {
        const int64_t j = s.S.row_col[e];
        if (j == kl || j == kr) continue;
        const T* Bk = s.L.SP + 36 * (int64_t)s.S.row_blk[e] + 6 * r;
#pragma unroll
        for (int q = 0; q < 6; ++q) c += fabs((double)Bk[q]);
      }
    }
#pragma unroll
    for (int o = 1; o < 5; o <<= 1) {
      const double t = __shfl_down_sync(0xffffffffu, c, o);
      if (part + o < 5) c += t;
    }
    __syncwarp();
    if (r < 6 && part == 0) {
      s.C.comp[6 * p + r] = c;
      if (al != 0.0 && ((s.P.kf_mask[k] >> r) & 1)) A[16 * r] += al * c;
    }
  }
  const int32_t le = p > 0 ? s.S.link_edge[p] : -1, lb = p > 0 ? s.S.link_blk[p] : -1;
  for (int idx = lane; idx < 225; idx += 32) {
    const int r = idx / 15, c = idx - 15 * (idx / 15);
    double v = 0.0;
    if (le >= 0) v += ge * (double)s.L.SE[225 * (int64_t)le + 15 * c + r];  // SE is (kf(p-1), kf(p)): transpose
    if (lb >= 0 && r < 6 && c < 6) v += gv * (double)s.L.SP[36 * (int64_t)lb + 6 * r + c];
    B[idx] = v;
  }
}

// FP32 product of 15x15 blocks in shared memory, C = op(A) op(B) (C must not
// alias A or B): the mixed path's factorization products.
__device__ void w_gemm_f(const float* A, bool ta, const float* B, bool tb, float* C) {
  const int lane = threadIdx.x & 31;
  for (int idx = lane; idx < 225; idx += 32) {
    const int r = idx / 15, c = idx - 15 * (idx / 15);
    float v = 0.f;
#pragma unroll
    for (int q = 0; q < 15; ++q) v += (ta ? A[15 * q + r] : A[15 * r + q]) * (tb ? B[15 * c + q] : B[15 * q + c]);
    C[idx] = v;
  }
  __syncwarp();
}

// Eliminates the positions of level l (or position 0 when top).  The pivot
// block's Cholesky inverse is FP64 in both paths; the mixed path forms the
// coupling products XL = CL^T F, XR = CR^T F in FP32 (the sweeps read them in
// FP32) and keeps no FP64 copies of the factors.
template <typename T>
__global__ void __launch_bounds__(32 * kCW) k_chain_elim(SolverLaunch<T> s, int l, int top) {
  if (s.ctl->terminated) return;
  __shared__ double sm[kCW][5][225];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t n = s.P.nkf, st = (int64_t)1 << l;
  const int64_t p = top ? (j == 0 ? 0 : n) : st + 2 * st * j;
  if (p >= n) return;
  double *sA = sm[w][0], *sX = sm[w][1], *sF = sm[w][2], *sL = sm[w][3], *sR = sm[w][4];
  w_load(s.C.A + 225 * p, sA);
  const bool ok = w_spd_inverse(sA, sX, sF);
  if (!ok && lane == 0) atomicExch(&s.ctl->chain_failed, 1);
  if constexpr (sizeof(T) == 8) {
    w_store(sF, s.C.F64 + 225 * p, s.C.F + 225 * p);
    if (top) return;
    w_load(s.C.B + 225 * p, sL);  // T(p, p-s)
    if (p + st < n) w_load(s.C.B + 225 * (p + st), sR, true);  // T(p, p+s) = T(p+s, p)^T
    else w_zero(sR);
    w_store(sL, s.C.CL64 + 225 * p, s.C.CL + 225 * p);
    w_store(sR, s.C.CR64 + 225 * p, s.C.CR + 225 * p);
    __syncwarp();
    w_gemm(sL, true, sF, false, sA, 1.0, false);  // XL = CL^T F
    w_store(sA, s.C.XL64 + 225 * p, s.C.XL + 225 * p);
    w_gemm(sR, true, sF, false, sX, 1.0, false);  // XR = CR^T F
    w_store(sX, s.C.XR64 + 225 * p, s.C.XR + 225 * p);
  } else {
    // FP32 working copies in the (now free) A and X buffers: 3 x 225 floats fit in 2 x 225 doubles.
    float* fF = reinterpret_cast<float*>(sA);
    float* fL = fF + 225;
    float* fR = reinterpret_cast<float*>(sX);
    float* fP = fR + 225;
    __syncwarp();
    for (int idx = lane; idx < 225; idx += 32) {
      fF[idx] = float(sF[idx]);
      s.C.F[225 * p + idx] = fF[idx];
    }
    if (top) return;
    const double* B1 = s.C.B + 225 * p;                                // T(p, p-s)
    const double* B2 = p + st < n ? s.C.B + 225 * (p + st) : nullptr;  // T(p+s, p): CR = its transpose
    for (int idx = lane; idx < 225; idx += 32) {
      const int r = idx / 15, c = idx - 15 * (idx / 15);
      fL[idx] = float(B1[idx]);
      fR[idx] = B2 ? float(B2[15 * c + r]) : 0.f;
      s.C.CL[225 * p + idx] = fL[idx];
      s.C.CR[225 * p + idx] = fR[idx];
    }
    __syncwarp();
    w_gemm_f(fL, true, fF, false, fP);  // XL = CL^T F
    for (int idx = lane; idx < 225; idx += 32) s.C.XL[225 * p + idx] = fP[idx];
    __syncwarp();
    w_gemm_f(fR, true, fF, false, fP);  // XR = CR^T F
    for (int idx = lane; idx < 225; idx += 32) s.C.XR[225 * p + idx] = fP[idx];
  }
}

// Survivors of level l absorb their eliminated neighbours (the mixed path
// forms the products in FP32 from the FP32 factors and subtracts them from the
// FP64 blocks).
template <typename T>
__global__ void __launch_bounds__(32 * kCW) k_chain_merge(SolverLaunch<T> s, int l) {
  if (s.ctl->terminated) return;
  __shared__ double sm[kCW][4][225];
  const int w = threadIdx.x >> 5;
  const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t n = s.P.nkf, st = (int64_t)1 << l;
  const int64_t q = 2 * st * j;
  if (q >= n) return;
  const int lane = threadIdx.x & 31;
  double *sD = sm[w][0], *s1 = sm[w][1], *s2 = sm[w][2], *sB = sm[w][3];
  w_load(s.C.A + 225 * q, sD);
  w_zero(sB);
  if constexpr (sizeof(T) == 8) {
    if (q >= st) {
      const int64_t a = q - st;
      w_load(s.C.XR64 + 225 * a, s1);
      w_load(s.C.CR64 + 225 * a, s2);
      w_gemm(s1, false, s2, false, sD, -1.0, true);
      w_load(s.C.CL64 + 225 * a, s2);
      w_gemm(s1, false, s2, false, sB, -1.0, false);
    }
    if (q + st < n) {
      const int64_t b = q + st;
      w_load(s.C.XL64 + 225 * b, s1);
      w_load(s.C.CL64 + 225 * b, s2);
      w_gemm(s1, false, s2, false, sD, -1.0, true);
    }
  } else {
    float* fX = reinterpret_cast<float*>(s1);
    float* fC = fX + 225;
    float* fP = reinterpret_cast<float*>(s2);
    auto load_f = [&](const float* g, float* d) {
      for (int idx = lane; idx < 225; idx += 32) d[idx] = g[idx];
      __syncwarp();
    };
    if (q >= st) {
      const int64_t a = q - st;
      load_f(s.C.XR + 225 * a, fX);
      load_f(s.C.CR + 225 * a, fC);
      w_gemm_f(fX, false, fC, false, fP);
      for (int idx = lane; idx < 225; idx += 32) sD[idx] -= double(fP[idx]);
      __syncwarp();
      load_f(s.C.CL + 225 * a, fC);
      w_gemm_f(fX, false, fC, false, fP);
      for (int idx = lane; idx < 225; idx += 32) sB[idx] = -double(fP[idx]);
      __syncwarp();
    }
    if (q + st < n) {
      const int64_t b = q + st;
      load_f(s.C.XL + 225 * b, fX);
      load_f(s.C.CL + 225 * b, fC);
      w_gemm_f(fX, false, fC, false, fP);
      for (int idx = lane; idx < 225; idx += 32) sD[idx] -= double(fP[idx]);
      __syncwarp();
    }
  }
  for (int idx = lane; idx < 225; idx += 32) {
    s.C.A[225 * q + idx] = sD[idx];
    s.C.B[225 * q + idx] = sB[idx];
  }
}

// ---- sweeps (16 threads per position, thread r owns row r)

template <typename T>
__device__ __forceinline__ T row_dot(const T* M, int r, const T* v) {
  T a = T(0);
#pragma unroll
  for (int c = 0; c < 15; ++c) a += M[15 * r + c] * v[c];
  return a;
}

// Forward sweep of level l >= 1 for survivor index j.
template <typename T>
__device__ __forceinline__ void fwd_node(const SolverLaunch<T>& s, int64_t st, int64_t j, int r) {
  const int64_t n = s.P.nkf, q = 2 * st * j;
  if (q >= n || r >= 15) return;
  T v = s.C.w[15 * q + r];
  if (q >= st) v -= row_dot(s.C.XR + 225 * (q - st), r, s.C.w + 15 * (q - st));
  if (q + st < n) v -= row_dot(s.C.XL + 225 * (q + st), r, s.C.w + 15 * (q + st));
  s.C.w[15 * q + r] = v;
}

// Back sweep of level l for eliminated index j; t is 16 values of scratch
// shared by the node's 16 threads.  Returns r.z of the row.
template <typename T>
__device__ __forceinline__ double bwd_node(const SolverLaunch<T>& s, int64_t st, int64_t j, int r, const T* rv, T* z,
                                           T* t, unsigned mask) {
  const int64_t n = s.P.nkf, p = st + 2 * st * j;
  const bool act = p < n && r < 15;
  if (act) {
    T v = s.C.w[15 * p + r];
    v -= row_dot(s.C.CL + 225 * p, r, z + 15 * (int64_t)s.S.chain_perm[p - st]);
    if (p + st < n) v -= row_dot(s.C.CR + 225 * p, r, z + 15 * (int64_t)s.S.chain_perm[p + st]);
    t[r] = v;
  }
  __syncwarp(mask);
  double rz = 0.0;
  if (act) {
    const int64_t k = s.S.chain_perm[p];
    const T zr = row_dot(s.C.F + 225 * p, r, t);
    z[15 * k + r] = zr;
    rz = (double)rv[15 * k + r] * (double)zr;
  }
  __syncwarp(mask);
  return rz;
}

// Level 0 forward: w(p) = r(p) for odd p; survivors subtract their neighbours.
template <typename T>
__global__ void __launch_bounds__(128) k_chain_fwd0(SolverLaunch<T> s, const T* rv) {
  if (apply_gate(s.ctl)) return;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t p = g >> 4, n = s.P.nkf;
  const int r = (int)(g & 15);
  if (p >= n || r >= 15) return;
  const T* rp = rv + 15 * (int64_t)s.S.chain_perm[p];
  T v = rp[r];
  if (!(p & 1)) {
    if (p >= 1) v -= row_dot(s.C.XR + 225 * (p - 1), r, rv + 15 * (int64_t)s.S.chain_perm[p - 1]);
    if (p + 1 < n) v -= row_dot(s.C.XL + 225 * (p + 1), r, rv + 15 * (int64_t)s.S.chain_perm[p + 1]);
  }
  s.C.w[15 * p + r] = v;
}

template <typename T>
__global__ void __launch_bounds__(128) k_chain_fwd(SolverLaunch<T> s, int l) {
  if (apply_gate(s.ctl)) return;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  fwd_node(s, (int64_t)1 << l, g >> 4, (int)(g & 15));
}

template <typename T>
__global__ void __launch_bounds__(128) k_chain_bwd(SolverLaunch<T> s, int l, const T* rv, T* z, double* rz) {
  if (apply_gate(s.ctl)) return;
  __shared__ T tsh[128];
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int r = (int)(g & 15);
  const unsigned mask = 0xffffu << (threadIdx.x & 16);
  const double v = bwd_node(s, (int64_t)1 << l, g >> 4, r, rv, z, tsh + (threadIdx.x & ~15), mask);
  block_add_d(v, rz);
}

// Levels l0.. in one block: forward sweeps, the last survivor, back sweeps.
// seg > 0: the segments' first positions take their left-neighbour terms from
// lc first (segmented sweeps, l0 = seg).
template <typename T>
__global__ void __launch_bounds__(kTailThreads) k_chain_tail(SolverLaunch<T> s, int l0, int seg, const T* rv, T* z,
                                                             double* rz) {
  if (apply_gate(s.ctl)) return;
  __shared__ T tsh[kTailThreads];
  const int64_t n = s.P.nkf;
  const int L = s.S.chain_levels;
  const int grp = threadIdx.x >> 4, r = threadIdx.x & 15;
  const int ngrp = kTailThreads / 16;
  const unsigned mask = 0xffffu << (threadIdx.x & 16);
  if (seg > 0) {
    for (int64_t j = 1 + grp; (j << seg) < n; j += ngrp)
      if (r < 15) s.C.w[15 * (j << seg) + r] -= s.C.lc[15 * j + r];
    __syncthreads();
  }
  for (int l = l0; l < L; ++l) {
    const int64_t st = (int64_t)1 << l, cnt = (n + 2 * st - 1) / (2 * st);
    for (int64_t j = grp; j < cnt; j += ngrp) fwd_node(s, st, j, r);
    __syncthreads();
  }
  double acc = 0.0;
  if (grp == 0) {
    if (r < 15) tsh[r] = s.C.w[r];
    __syncwarp(mask);
    if (r < 15) {
      const int64_t k = s.S.chain_perm[0];
      const T zr = row_dot(s.C.F, r, tsh);
      z[15 * k + r] = zr;
      acc += (double)rv[15 * k + r] * (double)zr;
    }
  }
  __syncthreads();
  for (int l = L - 1; l >= l0; --l) {
    const int64_t st = (int64_t)1 << l, cnt = n > st ? (n - st + 2 * st - 1) / (2 * st) : 0;
    const int64_t passes = (cnt + ngrp - 1) / ngrp;
    for (int64_t q = 0; q < passes; ++q) acc += bwd_node(s, st, grp + q * ngrp, r, rv, z, tsh + 16 * grp, mask);
    __syncthreads();
  }
  block_add_d(acc, rz);
}

// The same levels with the survivors' w and z in shared memory (tail index
// j = position >> l0): only the factor rows come from global memory.  Used
// when 2 ceil(n / 2^l0) x 16 values fit in kTailSmem bytes.
constexpr int kTailSmem = 96 * 1024;
template <typename T>
__global__ void __launch_bounds__(kTailThreads) k_chain_tail_sm(SolverLaunch<T> s, int l0, int seg, const T* rv, T* z,
                                                                double* rz) {
  if (apply_gate(s.ctl)) return;
  extern __shared__ __align__(16) unsigned char tail_smem[];
  const int64_t n = s.P.nkf;
  const int L = s.S.chain_levels;
  const int ns0 = (int)((n + ((int64_t)1 << l0) - 1) >> l0);
  T* ws = reinterpret_cast<T*>(tail_smem);  // [ns0][16] w, then the solve's right-hand side
  T* zs = ws + 16 * ns0;                    // [ns0][16] z
  const int grp = threadIdx.x >> 4, r = threadIdx.x & 15, ngrp = kTailThreads / 16;
  const unsigned mask = 0xffffu << (threadIdx.x & 16);
  for (int i = threadIdx.x; i < 16 * ns0; i += kTailThreads) {
    const int j = i >> 4, c = i & 15;
    T v = T(0);
    if (c < 15) {
      v = s.C.w[15 * ((int64_t)j << l0) + c];
      if (seg > 0 && j > 0) v -= s.C.lc[15 * (int64_t)j + c];
    }
    ws[i] = v;
  }
  __syncthreads();
  for (int l = l0; l < L; ++l) {
    const int st = 1 << (l - l0), cnt = (ns0 + 2 * st - 1) / (2 * st);
    for (int j = grp; j < cnt; j += ngrp) {
      const int q = 2 * st * j;
      if (r < 15) {
        T v = ws[16 * q + r];
        if (q >= st) v -= row_dot(s.C.XR + 225 * ((int64_t)(q - st) << l0), r, ws + 16 * (q - st));
        if (q + st < ns0) v -= row_dot(s.C.XL + 225 * ((int64_t)(q + st) << l0), r, ws + 16 * (q + st));
        ws[16 * q + r] = v;
      }
    }
    __syncthreads();
  }
  double acc = 0.0;
  if (grp == 0 && r < 15) {
    const T zr = row_dot(s.C.F, r, ws);
    zs[r] = zr;
    const int64_t k = s.S.chain_perm[0];
    z[15 * k + r] = zr;
    acc += (double)rv[15 * k + r] * (double)zr;
  }
  __syncthreads();
  for (int l = L - 1; l >= l0; --l) {
    const int st = 1 << (l - l0), cnt = ns0 > st ? (ns0 - st + 2 * st - 1) / (2 * st) : 0;
    const int passes = (cnt + ngrp - 1) / ngrp;
    for (int qq = 0; qq < passes; ++qq) {
      const int p = st + 2 * st * (grp + qq * ngrp);
      const bool act = p < ns0 && r < 15;
      const int64_t gp = (int64_t)p << l0;
      if (act) {
        T v = ws[16 * p + r];
        v -= row_dot(s.C.CL + 225 * gp, r, zs + 16 * (p - st));
        if (p + st < ns0) v -= row_dot(s.C.CR + 225 * gp, r, zs + 16 * (p + st));
        ws[16 * p + r] = v;
      }
      __syncwarp(mask);
      if (act) {
        const T zr = row_dot(s.C.F + 225 * gp, r, ws + 16 * p);
        zs[16 * p + r] = zr;
        const int64_t k = s.S.chain_perm[gp];
        z[15 * k + r] = zr;
        acc += (double)rv[15 * k + r] * (double)zr;
      }
      __syncwarp(mask);
    }
    __syncthreads();
  }
  block_add_d(acc, rz);
}

// One-block tail from level l0 (seg > 0: segmented sweeps).
template <typename T>
void launch_tail(const SolverLaunch<T>& s, int l0, int seg, const T* r, T* z, double* rz, cudaStream_t st) {
  const int64_t ns0 = (s.P.nkf + ((int64_t)1 << l0) - 1) >> l0;
  const int64_t bytes = 2 * 16 * ns0 * (int64_t)sizeof(T);
  if (s.S.chain_tail_sm && bytes <= kTailSmem)
    k_chain_tail_sm<T><<<1, kTailThreads, (size_t)bytes, st>>>(s, l0, seg, r, z, rz);
  else
    k_chain_tail<T><<<1, kTailThreads, 0, st>>>(s, l0, seg, r, z, rz);
}

constexpr int kSegThreads = 256;  // 16 positions at a time, thread r of a position owns row r

// Segmented forward sweep: block j runs levels 0..m-1 on positions
// [j 2^m, (j+1) 2^m) in shared memory (16 values per position), writes w and
// the next segment's left-neighbour terms lc[j + 1].
template <typename T>
__global__ void __launch_bounds__(kSegThreads) k_chain_seg_fwd(SolverLaunch<T> s, int m, const T* rv) {
  if (apply_gate(s.ctl)) return;
  extern __shared__ __align__(16) unsigned char seg_smem[];
  T* ws = reinterpret_cast<T*>(seg_smem);  // [2^m][16]
  const int64_t n = s.P.nkf, base = (int64_t)blockIdx.x << m;
  const int64_t left = n - base;
  const int cnt = left < ((int64_t)1 << m) ? (int)left : (1 << m);
  const int grp = threadIdx.x >> 4, r = threadIdx.x & 15, ngrp = kSegThreads / 16;
  for (int i = threadIdx.x; i < 16 * cnt; i += kSegThreads) {
    const int p = i >> 4, c = i & 15;
    ws[i] = c < 15 ? rv[15 * (int64_t)s.S.chain_perm[base + p] + c] : T(0);
  }
  __syncthreads();
  for (int l = 0; l < m; ++l) {
    const int st = 1 << l, ns = (cnt + 2 * st - 1) / (2 * st);
    for (int j = grp; j < ns; j += ngrp) {
      const int q = 2 * st * j;  // survivor; q - st and q + st were eliminated at level l
      if (r < 15) {
        T v = ws[16 * q + r];
        if (q >= st) v -= row_dot(s.C.XR + 225 * (base + q - st), r, ws + 16 * (q - st));
        if (q + st < cnt) v -= row_dot(s.C.XL + 225 * (base + q + st), r, ws + 16 * (q + st));
        ws[16 * q + r] = v;
      }
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < 16 * cnt; i += kSegThreads)
    if ((i & 15) < 15) s.C.w[15 * base + 15 * (i >> 4) + (i & 15)] = ws[i];
  // Terms of the next segment's first position q' = base + 2^m from this
  // segment's positions q' - 2^l (eliminated at level l, final now).
  if (grp == 0 && r < 15 && cnt == (1 << m) && base + cnt < n) {
    T v = T(0);
    for (int l = 0; l < m; ++l) {
      const int p = cnt - (1 << l);
      v += row_dot(s.C.XR + 225 * (base + p), r, ws + 16 * p);
    }
    s.C.lc[15 * ((int64_t)blockIdx.x + 1) + r] = v;
  }
}

// Segmented back sweep: block j runs levels m-1..0 on its segment; the
// segment's first position and the next segment's first position were solved
// by the tail.  Writes z of the eliminated positions and adds their r.z.
template <typename T>
__global__ void __launch_bounds__(kSegThreads) k_chain_seg_bwd(SolverLaunch<T> s, int m, const T* rv, T* z,
                                                               double* rz) {
  if (apply_gate(s.ctl)) return;
  extern __shared__ __align__(16) unsigned char seg_smem[];
  const int seg = 1 << m;
  T* ws = reinterpret_cast<T*>(seg_smem);  // [2^m][16] w, then the solve's right-hand side
  T* zs = ws + 16 * seg;                   // [2^m + 1][16] z in position order
  const int64_t n = s.P.nkf, base = (int64_t)blockIdx.x << m;
  const int64_t left = n - base;
  const int cnt = left < (int64_t)seg ? (int)left : seg;
  const int grp = threadIdx.x >> 4, r = threadIdx.x & 15, ngrp = kSegThreads / 16;
  const unsigned mask = 0xffffu << (threadIdx.x & 16);
  for (int i = threadIdx.x; i < 16 * cnt; i += kSegThreads)
    ws[i] = (i & 15) < 15 ? s.C.w[15 * base + 15 * (i >> 4) + (i & 15)] : T(0);
  if (threadIdx.x < 15) zs[threadIdx.x] = z[15 * (int64_t)s.S.chain_perm[base] + threadIdx.x];
  if (threadIdx.x >= 16 && threadIdx.x < 31 && base + seg < n)
    zs[16 * seg + threadIdx.x - 16] = z[15 * (int64_t)s.S.chain_perm[base + seg] + threadIdx.x - 16];
  __syncthreads();
  double acc = 0.0;
  for (int l = m - 1; l >= 0; --l) {
    const int st = 1 << l, ne = cnt > st ? (cnt - st + 2 * st - 1) / (2 * st) : 0;
    const int passes = (ne + ngrp - 1) / ngrp;
    for (int q = 0; q < passes; ++q) {
      const int p = st + 2 * st * (grp + q * ngrp);
      const bool act = p < cnt && r < 15;
      if (act) {
        T v = ws[16 * p + r];
        v -= row_dot(s.C.CL + 225 * (base + p), r, zs + 16 * (p - st));
        if (base + p + st < n) v -= row_dot(s.C.CR + 225 * (base + p), r, zs + 16 * (p + st));
        ws[16 * p + r] = v;
      }
      __syncwarp(mask);
      if (act) {
        const T zr = row_dot(s.C.F + 225 * (base + p), r, ws + 16 * p);
        zs[16 * p + r] = zr;
        const int64_t k = s.S.chain_perm[base + p];
        z[15 * k + r] = zr;
        acc += (double)rv[15 * k + r] * (double)zr;
      }
      __syncwarp(mask);
    }
    __syncthreads();
  }
  block_add_d(acc, rz);
}

__global__ void k_chain_coef(double* coef, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    coef[3 * i] = 1.0;
    coef[3 * i + 1] = 1.0;
    coef[3 * i + 2] = 0.0;
  }
}

inline unsigned nb(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

cudaError_t chain_default_coef(double* coef, int64_t n, cudaStream_t st) {
  if (n) k_chain_coef<<<nb(n, 256), 256, 0, st>>>(coef, n);
  return cudaGetLastError();
}

template <typename T>
cudaError_t chain_factor(const SolverLaunch<T>& s, cudaStream_t st) {
  const int64_t n = s.P.nkf;
  if (!n) return cudaSuccess;
  k_chain_init<T><<<nb(32 * n, 32 * kCW), 32 * kCW, 0, st>>>(s);
  for (int l = 0; l < s.S.chain_levels; ++l) {
    const int64_t sd = (int64_t)1 << l;
    const int64_t ne = n > sd ? (n - sd + 2 * sd - 1) / (2 * sd) : 0, ns = (n + 2 * sd - 1) / (2 * sd);
    if (ne) k_chain_elim<T><<<nb(32 * ne, 32 * kCW), 32 * kCW, 0, st>>>(s, l, 0);
    k_chain_merge<T><<<nb(32 * ns, 32 * kCW), 32 * kCW, 0, st>>>(s, l);
  }
  k_chain_elim<T><<<1, 32 * kCW, 0, st>>>(s, 0, 1);
  return cudaGetLastError();
}

template <typename T>
cudaError_t chain_apply(const SolverLaunch<T>& s, const T* r, T* z, double* rz, cudaStream_t st) {
  const int64_t n = s.P.nkf;
  if (!n) return cudaSuccess;
  const int L = s.S.chain_levels, l0 = s.S.chain_tail;
  if (s.S.chain_seg > 0) {
    const int m = s.S.chain_seg;
    const unsigned blocks = nb(n, 1 << m);
    const size_t sm = sizeof(T) * 16 * (size_t)(1 << m);
    k_chain_seg_fwd<T><<<blocks, kSegThreads, sm, st>>>(s, m, r);
    launch_tail<T>(s, m, m, r, z, rz, st);
    k_chain_seg_bwd<T><<<blocks, kSegThreads, 2 * sm + sizeof(T) * 16, st>>>(s, m, r, z, rz);
    return cudaGetLastError();
  }
  k_chain_fwd0<T><<<nb(16 * n, 128), 128, 0, st>>>(s, r);
  for (int l = 1; l < l0; ++l) {
    const int64_t sd = (int64_t)1 << l, ns = (n + 2 * sd - 1) / (2 * sd);
    k_chain_fwd<T><<<nb(16 * ns, 128), 128, 0, st>>>(s, l);
  }
  launch_tail<T>(s, l0 < 1 ? 1 : l0, 0, r, z, rz, st);
  for (int l = (l0 < 1 ? 1 : l0) - 1; l >= 0; --l) {
    const int64_t sd = (int64_t)1 << l, ne = n > sd ? (n - sd + 2 * sd - 1) / (2 * sd) : 0;
    if (ne) k_chain_bwd<T><<<nb(16 * ne, 128), 128, 0, st>>>(s, l, r, z, rz);
  }
  (void)L;
  return cudaGetLastError();
}

// Shared-memory opt-in of the tail kernel (outside graph capture).
template <typename T>
cudaError_t chain_prepare() {
  cudaError_t e = cudaFuncSetAttribute(k_chain_tail_sm<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmem);
  // segments of up to 256 positions: 2 x 256 x 16 values (+ one position) in the back sweep
  const int seg_bytes = (int)(sizeof(T) * 16 * (2 * 256 + 1));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_chain_seg_fwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, seg_bytes);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_chain_seg_bwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, seg_bytes);
  return e;
}

template cudaError_t chain_prepare<double>();
template cudaError_t chain_prepare<float>();
template cudaError_t chain_factor<double>(const SolverLaunch<double>&, cudaStream_t);
template cudaError_t chain_factor<float>(const SolverLaunch<float>&, cudaStream_t);
template cudaError_t chain_apply<double>(const SolverLaunch<double>&, const double*, double*, double*, cudaStream_t);
template cudaError_t chain_apply<float>(const SolverLaunch<float>&, const float*, float*, double*, cudaStream_t);

}  // namespace mba
