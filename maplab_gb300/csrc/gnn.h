// Learned chain-preconditioner coefficients: a message-passing network over
// the keyframe co-visibility graph of the reduced camera system.
//
// Nodes are keyframes; edges are the pose-pose blocks of S (co-visibility)
// and the inertial blocks.  Node input (kGnnIn values): log10 of the 15
// diagonal entries of the damped, scaled S_kk; log2 of the degree; the summed
// coupling of off-chain neighbours; the couplings to the previous and next
// chain keyframe.  Coupling of an edge: c_ij = |S_ij|_F / sqrt(|S_ii|_F |S_jj|_F).
//
// Layer l (3 layers, hidden kGnnHidden):
//   m_i = bf16( sum_j c_ij h_j / sum_j c_ij )
//   z_i = W1 h_i + W2 m_i + b            (BF16 operands, FP32 accumulation)
//   h'_i = bf16( relu(z_i) )
// Head per chain position p (node k, previous chain node k'):
//   o = Wh [h_k ; h_k'] + bh  ->  gamma_ine = sig(o0), gamma_vis = sig(o1),
//   alpha = kGnnAlphaMax sig(o2).
// These are the coefficients of the chain matrix T (ChainSystem.coef).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace mba {

constexpr int kGnnIn = 32;       // padded input width (20 used)
constexpr int kGnnHidden = 64;
constexpr int kGnnLayers = 3;
constexpr int kGnnHeadIn = 2 * kGnnHidden;
constexpr int kGnnOut = 3;
constexpr float kGnnAlphaMax = 0.1f;

// Parameter tensor offsets in the flat FP32 parameter vector.
struct GnnLayout {
  int64_t w1[kGnnLayers], w2[kGnnLayers], b[kGnnLayers], k[kGnnLayers];
  int64_t wh, bh, total;
  __host__ __device__ static GnnLayout make() {
    GnnLayout L{};
    int64_t o = 0;
    for (int l = 0; l < kGnnLayers; ++l) {
      L.k[l] = l == 0 ? kGnnIn : kGnnHidden;
      L.w1[l] = o; o += kGnnHidden * L.k[l];
      L.w2[l] = o; o += kGnnHidden * L.k[l];
      L.b[l] = o; o += kGnnHidden;
    }
    L.wh = o; o += kGnnOut * kGnnHeadIn;
    L.bh = o; o += kGnnOut;
    L.total = o;
    return L;
  }
};

// Model parameters and optimizer state (device).
struct GnnParams {
  float* w;            // [total] FP32 master copy
  __nv_bfloat16* wb;   // [total] BF16 copy used by the kernels (row-major W: [out][in])
  __nv_bfloat16* wt;   // [total] BF16 transposed weight matrices ([in][out]) for the backward product
  float* g;            // [total] gradient
  float* m;            // [total] Adam first moment
  float* v;            // [total] Adam second moment
  int64_t step;
};

// Per-problem activations and scratch (device), sized for nkf nodes.
struct GnnWork {
  int64_t n = 0;
  float* wgt;                     // [2 npu + 2 nedge] edge couplings in CSR order of nbr_off
  float* deg;                     // [n] sum of couplings
  __nv_bfloat16* x;               // [n][kGnnIn] input
  __nv_bfloat16* h[kGnnLayers + 1];  // h[0] = x, h[l+1] = layer l output [n][kGnnHidden]
  __nv_bfloat16* m[kGnnLayers];   // aggregated inputs [n][k_l]
  float* z[kGnnLayers];           // pre-activations [n][kGnnHidden]
  float* o;                       // [n][kGnnOut] head outputs per chain position
  float* dh;                      // [n][kGnnHidden] gradient of the current layer output
  float* dm;                      // [n][kGnnHidden]
  __nv_bfloat16* dzb;             // [n][kGnnHidden] BF16 gradient of pre-activations
  float* dcoef;                   // [n][3] dL / dcoef
  float* vec;                     // [5][15 n] probe, S w, y, e, lambda (working precision float)
  double* loss;                   // [1]
};

// Neighbour lists of the co-visibility + inertial graph (built on the host).
struct GnnGraph {
  int64_t* nbr_off;   // [n+1]
  int32_t* nbr;       // [nnz] neighbour keyframe
  int32_t* nbr_blk;   // [nnz] >= 0: SP block index (row kf, col nbr); < 0: -(e+1) inertial edge
};

// Tensor-core node update (kernels_gnn_tc.cu): Z = A W^T (+ A2 W2^T) + bias,
// H = bf16(relu(Z)); K = 32 or 64, 64 outputs.  `fatal` is raised if a
// bounded wait of the tensor-core pipeline runs out.
cudaError_t gnn_gemm_tc_prepare();
// The same kernel with its operand copies left out and a short wait limit:
// the load barrier is never signalled, the wait runs out, `fatal` is raised
// and the kernel returns with its tensor memory freed (K = 64, A / W valid).
cudaError_t gnn_gemm_tc_wait_check(int64_t n, const __nv_bfloat16* A, const __nv_bfloat16* W, float* Z, int* fatal,
                                   cudaStream_t st);
cudaError_t gnn_gemm_tc(int64_t n, int K, const __nv_bfloat16* A, const __nv_bfloat16* W, const __nv_bfloat16* A2,
                        const __nv_bfloat16* W2, const float* bias, float* Z, __nv_bfloat16* H, int* fatal,
                        cudaStream_t st);

}  // namespace mba
