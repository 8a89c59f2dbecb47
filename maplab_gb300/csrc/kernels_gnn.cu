// Graph network for the learned chain-preconditioner coefficients: features,
// forward pass (the node updates are BF16 products with FP32 accumulation on
// the tcgen05 tensor cores, kernels_gnn_tc.cu), probe loss with adjoint chain
// solves, backward pass and Adam.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "solver.h"

namespace mba {
namespace {

typedef __nv_bfloat16 bf16;

inline unsigned nb(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

__device__ __forceinline__ float sigm(float x) { return 1.f / (1.f + __expf(-x)); }

// ---- graph features

template <typename T>
__device__ __forceinline__ float frob(const T* B, int n) {
  float s = 0.f;
  for (int q = 0; q < n; ++q) s += (float)B[q] * (float)B[q];
  return sqrtf(s);
}

// Node norms |S_kk|_F.
template <typename T>
__global__ void k_gnn_norms(SolverLaunch<T> s, float* nrm) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < s.P.nkf) nrm[k] = fmaxf(frob(s.L.SD + 225 * k, 225), 1e-30f);
}

// Edge couplings c_kj and their sums d_k.
template <typename T>
__global__ void k_gnn_edges(SolverLaunch<T> s, GnnGraph g, const float* nrm, float* wgt, float* deg) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= s.P.nkf) return;
  float d = 0.f;
  for (int64_t e = g.nbr_off[k]; e < g.nbr_off[k + 1]; ++e) {
    const int32_t b = g.nbr_blk[e];
    const float f = b >= 0 ? frob(s.L.SP + 36 * (int64_t)b, 36) : frob(s.L.SE + 225 * (int64_t)(-b - 1), 225);
    const float c = f / sqrtf(nrm[k] * nrm[g.nbr[e]]);
    wgt[e] = c;
    d += c;
  }
  deg[k] = d;
}

__device__ __forceinline__ float coupling_to(const GnnGraph& g, const float* wgt, int64_t k, int64_t j) {
  if (j < 0) return 0.f;
  float c = 0.f;
  for (int64_t e = g.nbr_off[k]; e < g.nbr_off[k + 1]; ++e)
    if (g.nbr[e] == j) c += wgt[e];
  return c;
}

__device__ __forceinline__ bool linked(const SchurPattern& S, int64_t p) {
  return p > 0 && (S.link_edge[p] >= 0 || S.link_blk[p] >= 0);
}

// Input features per chain position (written at the node's keyframe row).
template <typename T>
__global__ void k_gnn_features(SolverLaunch<T> s, GnnGraph g, const float* wgt, const float* deg, bf16* x) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t n = s.P.nkf;
  if (p >= n) return;
  const int64_t k = s.S.chain_perm[p];
  const int64_t kp = linked(s.S, p) ? s.S.chain_perm[p - 1] : -1;
  const int64_t kn = (p + 1 < n && linked(s.S, p + 1)) ? s.S.chain_perm[p + 1] : -1;
  float f[kGnnIn];
#pragma unroll
  for (int a = 0; a < kGnnIn; ++a) f[a] = 0.f;
  const T* D = s.L.SD + 225 * k;
#pragma unroll
  for (int a = 0; a < 15; ++a) f[a] = log10f(fmaxf((float)D[16 * a], 1e-12f)) * 0.1f;
  const float cp = coupling_to(g, wgt, k, kp), cn = coupling_to(g, wgt, k, kn);
  f[15] = log2f(1.f + (float)(g.nbr_off[k + 1] - g.nbr_off[k])) * 0.125f;
  f[16] = deg[k] - cp - cn;
  f[17] = cp;
  f[18] = cn;
  f[19] = 1.f;
#pragma unroll
  for (int a = 0; a < kGnnIn; ++a) x[k * kGnnIn + a] = __float2bfloat16_rn(f[a]);
}

// m_k = bf16(sum_j c_kj h_j / d_k); one warp per node, lanes over features.
template <int K>
__global__ void k_gnn_aggregate(int64_t n, GnnGraph g, const float* wgt, const float* deg, const bf16* h, bf16* m) {
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= n) return;
  float a0 = 0.f, a1 = 0.f;
  for (int64_t e = g.nbr_off[k]; e < g.nbr_off[k + 1]; ++e) {
    const float c = wgt[e];
    const bf16* hj = h + (int64_t)g.nbr[e] * K;
    a0 += c * __bfloat162float(hj[lane]);
    if (K > 32) a1 += c * __bfloat162float(hj[lane + 32]);
  }
  const float inv = deg[k] > 0.f ? 1.f / deg[k] : 0.f;
  m[k * K + lane] = __float2bfloat16_rn(a0 * inv);
  if (K > 32) m[k * K + lane + 32] = __float2bfloat16_rn(a1 * inv);
}

// dh_j += sum_i c_ij dm_i / d_i (transpose of the aggregation).
template <int K>
__global__ void k_gnn_aggregate_bwd(int64_t n, GnnGraph g, const float* wgt, const float* deg, const float* dm,
                                    float* dh) {
  const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= n) return;
  float a0 = 0.f, a1 = 0.f;
  for (int64_t e = g.nbr_off[j]; e < g.nbr_off[j + 1]; ++e) {
    const int64_t i = g.nbr[e];
    const float c = deg[i] > 0.f ? wgt[e] / deg[i] : 0.f;
    a0 += c * dm[i * K + lane];
    if (K > 32) a1 += c * dm[i * K + lane + 32];
  }
  dh[j * K + lane] += a0;
  if (K > 32) dh[j * K + lane + 32] += a1;
}

// Head per chain position; writes the chain coefficients.
template <typename T>
__global__ void k_gnn_head(SolverLaunch<T> s, GnnParams prm, const bf16* h3, float* o) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= s.P.nkf) return;
  const GnnLayout L = GnnLayout::make();
  const int64_t k = s.S.chain_perm[p];
  const int64_t kp = linked(s.S, p) ? s.S.chain_perm[p - 1] : -1;
  float out[kGnnOut];
#pragma unroll
  for (int q = 0; q < kGnnOut; ++q) {
    const bf16* wr = prm.wb + L.wh + q * kGnnHeadIn;
    float a = prm.w[L.bh + q];
    for (int c = 0; c < kGnnHidden; ++c) a += __bfloat162float(wr[c]) * __bfloat162float(h3[k * kGnnHidden + c]);
    if (kp >= 0)
      for (int c = 0; c < kGnnHidden; ++c)
        a += __bfloat162float(wr[kGnnHidden + c]) * __bfloat162float(h3[kp * kGnnHidden + c]);
    out[q] = a;
    o[p * kGnnOut + q] = a;
  }
  s.C.coef[3 * p] = sigm(out[0]);
  s.C.coef[3 * p + 1] = sigm(out[1]);
  s.C.coef[3 * p + 2] = kGnnAlphaMax * sigm(out[2]);
}

// ---- loss and gradients

__device__ __forceinline__ uint64_t smix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void k_gnn_probe(int64_t n, uint64_t seed, float* w) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t a = smix(seed * 0x100000001B3ull + 2 * i), b = smix(seed * 0x100000001B3ull + 2 * i + 1);
  const float u1 = ((a >> 40) + 1.f) * (1.f / 16777217.f), u2 = (b >> 40) * (1.f / 16777216.f);
  w[i] = sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
}

// y = S x (all blocks of the damped, masked reduced system); warp per row.
template <typename T>
__global__ void __launch_bounds__(128) k_gnn_spmv(SolverLaunch<T> s, const float* x, float* y) {
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= s.P.nkf) return;
  float acc = 0.f;
  if (lane < 15) {
    const T* D = s.L.SD + 225 * k + 15 * lane;
    for (int c = 0; c < 15; ++c) acc += (float)D[c] * x[15 * k + c];
    for (int64_t e = s.S.kfe_off[k]; e < s.S.kfe_off[k + 1]; ++e) {
      const int code = s.S.kfe[e];
      const bool from = code > 0;
      const int64_t ed = from ? code - 1 : -code - 1;
      const T* E = s.L.SE + 225 * ed;
      const int64_t o = from ? s.P.e_to[ed] : s.P.e_from[ed];
      for (int c = 0; c < 15; ++c) acc += (float)(from ? E[15 * lane + c] : E[15 * c + lane]) * x[15 * o + c];
    }
    if (lane < 6)
      for (int64_t e = s.S.row_off[k]; e < s.S.row_off[k + 1]; ++e) {
        const T* B = s.L.SP + 36 * (int64_t)s.S.row_blk[e] + 6 * lane;
        const float* xj = x + 15 * (int64_t)s.S.row_col[e];
        for (int c = 0; c < 6; ++c) acc += (float)B[c] * xj[c];
      }
    y[15 * k + lane] = acc;
  }
}

// e = y - w; loss += |e|^2 * scale; r = 2 e * scale.
__global__ void k_gnn_resid(int64_t n, const float* y, const float* w, float* r, float scale, double* loss) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float v = 0.f;
  if (i < n) {
    const float e = y[i] - w[i];
    r[i] = 2.f * e * scale;
    v = e * e * scale;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v != 0.f) atomicAdd(loss, (double)v);
}

// dL/dcoef += -lambda^T dT y per chain position (T = chain matrix).
template <typename T>
__global__ void k_gnn_coef_grad(SolverLaunch<T> s, const float* y, const float* lam, float* dcoef) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t n = s.P.nkf;
  if (p >= n) return;
  const int64_t k = s.S.chain_perm[p];
  const float* yk = y + 15 * k;
  const float* lk = lam + 15 * k;
  float ga = 0.f;
  const double* comp = s.C.comp + 6 * p;
  for (int r = 0; r < 6; ++r)
    if ((s.P.kf_mask[k] >> r) & 1) ga -= lk[r] * (float)comp[r] * yk[r];
  float ge = 0.f, gv = 0.f;
  if (p > 0) {
    const int64_t kq = s.S.chain_perm[p - 1];
    const float* yq = y + 15 * kq;
    const float* lq = lam + 15 * kq;
    const int32_t le = s.S.link_edge[p], lb = s.S.link_blk[p];
    // B = T(p, p-1) part: lambda_p^T B y_{p-1} + lambda_{p-1}^T B^T y_p.
    if (le >= 0) {
      const T* E = s.L.SE + 225 * (int64_t)le;  // (kf(p-1), kf(p)) block: B = E^T
      for (int r = 0; r < 15; ++r)
        for (int c = 0; c < 15; ++c) {
          const float b = (float)E[15 * c + r];
          ge -= lk[r] * b * yq[c] + lq[c] * b * yk[r];
        }
    }
    if (lb >= 0) {
      const T* B = s.L.SP + 36 * (int64_t)lb;
      for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) {
          const float b = (float)B[6 * r + c];
          gv -= lk[r] * b * yq[c] + lq[c] * b * yk[r];
        }
    }
  }
  dcoef[3 * p] += ge;
  dcoef[3 * p + 1] += gv;
  dcoef[3 * p + 2] += ga;
}

// Head backward: do = dcoef * sig', weight / bias gradients, dh3.
template <typename T>
__global__ void k_gnn_head_bwd(SolverLaunch<T> s, GnnParams prm, const bf16* h3, const float* o, const float* dcoef,
                               float* dh) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= s.P.nkf) return;
  const GnnLayout L = GnnLayout::make();
  const int64_t k = s.S.chain_perm[p];
  const int64_t kp = linked(s.S, p) ? s.S.chain_perm[p - 1] : -1;
  float d[kGnnOut];
  for (int q = 0; q < kGnnOut; ++q) {
    const float sg = sigm(o[p * kGnnOut + q]);
    d[q] = dcoef[3 * p + q] * sg * (1.f - sg) * (q == 2 ? kGnnAlphaMax : 1.f);
  }
  for (int q = 0; q < kGnnOut; ++q) {
    if (d[q] == 0.f) continue;
    atomicAdd(&prm.g[L.bh + q], d[q]);
    for (int c = 0; c < kGnnHidden; ++c) {
      atomicAdd(&prm.g[L.wh + q * kGnnHeadIn + c], d[q] * __bfloat162float(h3[k * kGnnHidden + c]));
      if (kp >= 0)
        atomicAdd(&prm.g[L.wh + q * kGnnHeadIn + kGnnHidden + c], d[q] * __bfloat162float(h3[kp * kGnnHidden + c]));
    }
  }
  for (int c = 0; c < kGnnHidden; ++c) {
    float a = 0.f, b = 0.f;
    for (int q = 0; q < kGnnOut; ++q) {
      a += d[q] * __bfloat162float(prm.wb[L.wh + q * kGnnHeadIn + c]);
      b += d[q] * __bfloat162float(prm.wb[L.wh + q * kGnnHeadIn + kGnnHidden + c]);
    }
    atomicAdd(&dh[k * kGnnHidden + c], a);
    if (kp >= 0) atomicAdd(&dh[kp * kGnnHidden + c], b);
  }
}

// dz = bf16(dh * (z > 0)); bias gradient.
__global__ void k_gnn_relu_bwd(int64_t n, const float* dh, const float* z, bf16* dzb, float* gb) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * kGnnHidden) return;
  const float v = z[i] > 0.f ? dh[i] : 0.f;
  const bf16 vb = __float2bfloat16_rn(v);
  dzb[i] = vb;
  const float vr = __bfloat162float(vb);
  if (vr != 0.f) atomicAdd(&gb[i % kGnnHidden], vr);
}

// gW[o][c] += sum_i dz[i][o] a[i][c] over a chunk of 64 nodes per block.
template <int K>
__global__ void __launch_bounds__(256) k_gnn_wgrad(int64_t n, const bf16* dz, const bf16* a, float* gw) {
  __shared__ float sdz[64][kGnnHidden + 1];
  __shared__ float sa[64][K + 1];
  const int64_t i0 = (int64_t)blockIdx.x * 64;
  for (int t = threadIdx.x; t < 64 * kGnnHidden; t += blockDim.x) {
    const int r = t / kGnnHidden, c = t % kGnnHidden;
    sdz[r][c] = i0 + r < n ? __bfloat162float(dz[(i0 + r) * kGnnHidden + c]) : 0.f;
  }
  for (int t = threadIdx.x; t < 64 * K; t += blockDim.x) {
    const int r = t / K, c = t % K;
    sa[r][c] = i0 + r < n ? __bfloat162float(a[(i0 + r) * K + c]) : 0.f;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kGnnHidden * K; t += blockDim.x) {
    const int o = t / K, c = t % K;
    float acc = 0.f;
    for (int r = 0; r < 64; ++r) acc += sdz[r][o] * sa[r][c];
    if (acc != 0.f) atomicAdd(&gw[t], acc);
  }
}

__global__ void k_gnn_adam(GnnParams p, int64_t total, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= total) return;
  const float g = p.g[i];
  const float m = b1 * p.m[i] + (1.f - b1) * g, v = b2 * p.v[i] + (1.f - b2) * g * g;
  p.m[i] = m;
  p.v[i] = v;
  p.w[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

// BF16 copies: row-major and transposed per weight matrix.
__global__ void k_gnn_sync(GnnParams p) {
  const GnnLayout L = GnnLayout::make();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L.total) return;
  p.wb[i] = __float2bfloat16_rn(p.w[i]);
  // transposed copy for W1 / W2 of each layer ([out][in] -> [in][out])
  for (int l = 0; l < kGnnLayers; ++l) {
    const int64_t K = L.k[l];
    for (int which = 0; which < 2; ++which) {
      const int64_t base = which ? L.w2[l] : L.w1[l];
      if (i >= base && i < base + kGnnHidden * K) {
        const int64_t j = i - base, o = j / K, c = j % K;
        p.wt[base + c * kGnnHidden + o] = __float2bfloat16_rn(p.w[i]);
      }
    }
  }
}

// Uniform(-a, a) with a = sqrt(6 / (fan_in + fan_out)); head bias 3, 3, -4
// (gamma ~ 0.95, alpha ~ 0.002: the untrained net starts near the plain chain).
__global__ void k_gnn_init(GnnParams p, uint64_t seed) {
  const GnnLayout L = GnnLayout::make();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= L.total) return;
  float a = 0.f, val = 0.f;
  for (int l = 0; l < kGnnLayers; ++l) {
    if ((i >= L.w1[l] && i < L.w1[l] + kGnnHidden * L.k[l]) || (i >= L.w2[l] && i < L.w2[l] + kGnnHidden * L.k[l]))
      a = sqrtf(6.f / (float)(L.k[l] + kGnnHidden));
  }
  if (i >= L.wh && i < L.wh + kGnnOut * kGnnHeadIn) a = 0.1f * sqrtf(6.f / (float)(kGnnHeadIn + kGnnOut));
  if (a > 0.f) {
    const uint64_t r = smix(seed ^ (0xA5A5A5A5ull + (uint64_t)i));
    val = a * (2.f * ((r >> 40) * (1.f / 16777216.f)) - 1.f);
  }
  if (i == L.bh) val = 3.f;
  if (i == L.bh + 1) val = 3.f;
  if (i == L.bh + 2) val = -4.f;
  p.w[i] = val;
  p.m[i] = 0.f;
  p.v[i] = 0.f;
  p.g[i] = 0.f;
}

// The forward node update runs on the tcgen05 tensor cores (kernels_gnn_tc.cu).
template <int K>
cudaError_t launch_gemm_fwd(int64_t n, const bf16* A, const bf16* W, const bf16* A2, const bf16* W2, const float* bias,
                            float* Z, bf16* H, int* fatal, cudaStream_t st) {
  return gnn_gemm_tc(n, K, A, W, A2, W2, bias, Z, H, fatal, st);
}

}  // namespace

cudaError_t gnn_init_params(GnnParams p, uint64_t seed, cudaStream_t st) {
  const GnnLayout L = GnnLayout::make();
  k_gnn_init<<<nb(L.total, 256), 256, 0, st>>>(p, seed);
  return gnn_sync_bf16(p, st);
}

cudaError_t gnn_sync_bf16(GnnParams p, cudaStream_t st) {
  const GnnLayout L = GnnLayout::make();
  k_gnn_sync<<<nb(L.total, 256), 256, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t gnn_adam(GnnParams p, float lr, cudaStream_t st) {
  const GnnLayout L = GnnLayout::make();
  const float b1 = 0.9f, b2 = 0.999f;
  const double t = (double)p.step;
  const float c1 = (float)(1.0 - pow(0.9, t)), c2 = (float)(1.0 - pow(0.999, t));
  k_gnn_adam<<<nb(L.total, 256), 256, 0, st>>>(p, L.total, lr, b1, b2, 1e-8f, c1, c2);
  return gnn_sync_bf16(p, st);
}

template <typename T>
cudaError_t gnn_forward(const SolverLaunch<T>& s, GnnGraph g, GnnParams p, GnnWork w, cudaStream_t st) {
  const int64_t n = s.P.nkf;
  if (!n) return cudaSuccess;
  const GnnLayout L = GnnLayout::make();
  float* nrm = w.dm;  // scratch: node norms (dm is free during the forward pass)
  k_gnn_norms<T><<<nb(n, 256), 256, 0, st>>>(s, nrm);
  k_gnn_edges<T><<<nb(n, 128), 128, 0, st>>>(s, g, nrm, w.wgt, w.deg);
  k_gnn_features<T><<<nb(n, 128), 128, 0, st>>>(s, g, w.wgt, w.deg, w.h[0]);
  for (int l = 0; l < kGnnLayers; ++l) {
    if (l == 0) {
      k_gnn_aggregate<kGnnIn><<<nb(32 * n, 128), 128, 0, st>>>(n, g, w.wgt, w.deg, w.h[0], w.m[0]);
      launch_gemm_fwd<kGnnIn>(n, w.h[0], p.wb + L.w1[0], w.m[0], p.wb + L.w2[0], p.w + L.b[0], w.z[0], w.h[1], &s.ctl->fatal, st);
    } else {
      k_gnn_aggregate<kGnnHidden><<<nb(32 * n, 128), 128, 0, st>>>(n, g, w.wgt, w.deg, w.h[l], w.m[l]);
      launch_gemm_fwd<kGnnHidden>(n, w.h[l], p.wb + L.w1[l], w.m[l], p.wb + L.w2[l], p.w + L.b[l], w.z[l],
                                  w.h[l + 1], &s.ctl->fatal, st);
    }
  }
  k_gnn_head<T><<<nb(n, 128), 128, 0, st>>>(s, p, w.h[kGnnLayers], w.o);
  return cudaGetLastError();
}

template <typename T>
cudaError_t gnn_loss_backward(const SolverLaunch<T>& s, GnnGraph g, GnnParams p, GnnWork w, int nprobe,
                              const float* probes, uint64_t seed, cudaStream_t st) {
  const int64_t n = s.P.nkf, n15 = 15 * n;
  const GnnLayout L = GnnLayout::make();
  cudaError_t e = cudaMemsetAsync(w.loss, 0, sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.dcoef, 0, sizeof(float) * 3 * n, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(p.g, 0, sizeof(float) * L.total, st);
  if (e != cudaSuccess) return e;
  float *pw = w.vec, *u = w.vec + n15, *y = w.vec + 2 * n15, *r = w.vec + 3 * n15, *lam = w.vec + 4 * n15;
  double* rz = w.loss + 1;  // scratch for the sweeps' r.z
  const float scale = 1.f / ((float)nprobe * (float)n15);
  for (int q = 0; q < nprobe; ++q) {
    if (probes) e = cudaMemcpyAsync(pw, probes + q * n15, sizeof(float) * n15, cudaMemcpyDeviceToDevice, st);
    else k_gnn_probe<<<nb(n15, 256), 256, 0, st>>>(n15, seed + 7919ull * q, pw);
    if (e != cudaSuccess) return e;
    k_gnn_spmv<T><<<nb(32 * n, 128), 128, 0, st>>>(s, pw, u);
    e = chain_apply<T>(s, (const T*)u, (T*)y, rz, st);
    if (e != cudaSuccess) return e;
    k_gnn_resid<<<nb(n15, 256), 256, 0, st>>>(n15, y, pw, r, scale, w.loss);
    e = chain_apply<T>(s, (const T*)r, (T*)lam, rz, st);
    if (e != cudaSuccess) return e;
    k_gnn_coef_grad<T><<<nb(n, 128), 128, 0, st>>>(s, y, lam, w.dcoef);
  }
  // Backward through the head and the layers.
  e = cudaMemsetAsync(w.dh, 0, sizeof(float) * n * kGnnHidden, st);
  if (e != cudaSuccess) return e;
  k_gnn_head_bwd<T><<<nb(n, 128), 128, 0, st>>>(s, p, w.h[kGnnLayers], w.o, w.dcoef, w.dh);
  for (int l = kGnnLayers - 1; l >= 0; --l) {
    const int K = (int)L.k[l];
    k_gnn_relu_bwd<<<nb(n * kGnnHidden, 256), 256, 0, st>>>(n, w.dh, w.z[l], w.dzb, p.g + L.b[l]);
    if (K == kGnnIn) {
      k_gnn_wgrad<kGnnIn><<<nb(n, 64), 256, 0, st>>>(n, w.dzb, w.h[l], p.g + L.w1[l]);
      k_gnn_wgrad<kGnnIn><<<nb(n, 64), 256, 0, st>>>(n, w.dzb, w.m[l], p.g + L.w2[l]);
    } else {
      k_gnn_wgrad<kGnnHidden><<<nb(n, 64), 256, 0, st>>>(n, w.dzb, w.h[l], p.g + L.w1[l]);
      k_gnn_wgrad<kGnnHidden><<<nb(n, 64), 256, 0, st>>>(n, w.dzb, w.m[l], p.g + L.w2[l]);
    }
    if (l == 0) break;
    // dh_l = dz W1 + aggregation^T (dz W2); the W^T products on the tcgen05 tensor cores.
    cudaError_t e2 = gnn_gemm_tc(n, kGnnHidden, w.dzb, p.wt + L.w1[l], nullptr, nullptr, nullptr, w.dh, nullptr,
                                 &s.ctl->fatal, st);
    if (e2 == cudaSuccess)
      e2 = gnn_gemm_tc(n, kGnnHidden, w.dzb, p.wt + L.w2[l], nullptr, nullptr, nullptr, w.dm, nullptr, &s.ctl->fatal,
                       st);
    if (e2 != cudaSuccess) return e2;
    k_gnn_aggregate_bwd<kGnnHidden><<<nb(32 * n, 128), 128, 0, st>>>(n, g, w.wgt, w.deg, w.dm, w.dh);
  }
  return cudaGetLastError();
}

template cudaError_t gnn_forward<float>(const SolverLaunch<float>&, GnnGraph, GnnParams, GnnWork, cudaStream_t);
template cudaError_t gnn_forward<double>(const SolverLaunch<double>&, GnnGraph, GnnParams, GnnWork, cudaStream_t);
template cudaError_t gnn_loss_backward<float>(const SolverLaunch<float>&, GnnGraph, GnnParams, GnnWork, int,
                                              const float*, uint64_t, cudaStream_t);

}  // namespace mba
