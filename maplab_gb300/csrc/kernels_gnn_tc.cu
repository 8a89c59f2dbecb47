// Node-update GEMM of the learned preconditioner's message passing on the
// 5th-generation tensor cores:
//
//   Z[n][64] = A[n][K] W[64][K]^T + A2[n][K] W2[64][K]^T + bias,
//   H = bf16(relu(Z))
//
// (z_i = W1 h_i + W2 m_i + b of each layer; BF16 operands, FP32
// accumulation).  One CTA per 128-row tile:
//   - one thread issues the TMA loads of the A / A2 tiles (128 x K) and of
//     W / W2 (64 x K) into shared memory, 128B swizzle for K = 64 (64B for
//     K = 32), completing on an mbarrier;
//   - the same thread issues K/16 tcgen05.mma (kind::f16, M = 128, N = 64,
//     both operands K-major) per operand pair into a 64-column FP32
//     accumulator in tensor memory, then tcgen05.commit to a second mbarrier;
//   - each warp reads its 32 accumulator lanes with tcgen05.ld (one row per
//     thread), adds the bias and writes Z (FP32) and H (BF16).
// Every wait is bounded: on timeout the kernel raises `fatal`, waits (again
// bounded) for what it started, frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstring>

#include "gnn.h"

namespace mba {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kTileM = 128;
constexpr int kTileN = kGnnHidden;  // 64
constexpr int kTmemCols = 64;       // power of two >= 32
constexpr long kWaitLimit = 1L << 22;  // try_wait polls before a wait counts as run out

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long limit) {
  for (long i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Shared-memory matrix descriptor (tcgen05): start address, leading-byte
// offset (unused by swizzled K-major layouts), stride-byte offset between
// 8-row groups, descriptor version 1, swizzle mode.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t sbo, uint32_t swizzle) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1u << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)swizzle << 61;
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 64, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTileN >> 3) << 17) |
                            ((uint32_t)(kTileM >> 4) << 24);

template <int K>
struct TcSmem {
  static constexpr int kA = kTileM * K * 2;  // bytes of one A tile
  static constexpr int kW = kTileN * K * 2;  // bytes of one W tile
  static constexpr int kSwizzle = K == 64 ? 2 : 4;     // 128B : 64B
  static constexpr int kSbo = 8 * K * 2;               // 8 rows of K bf16
  static constexpr int kBytes = 2 * kA + 2 * kW + 1024;  // + alignment slack
};

template <int K>
__global__ void __launch_bounds__(128) k_gnn_gemm_tc(int64_t n, const __grid_constant__ CUtensorMap tA,
                                                     const __grid_constant__ CUtensorMap tW,
                                                     const __grid_constant__ CUtensorMap tA2,
                                                     const __grid_constant__ CUtensorMap tW2, int has2,
                                                     const float* __restrict__ bias, float* __restrict__ Z,
                                                     bf16* __restrict__ H, int* fatal, long wait_limit,
                                                     int skip_loads) {
  using L = TcSmem<K>;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int state;  // 0 ok, 1 load timeout, 2 mma timeout
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA[2] = {base, base + L::kA};
  uint8_t* sW[2] = {base + 2 * L::kA, base + 2 * L::kA + L::kW};
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = blockIdx.x * kTileM;
  const uint32_t bar_load = smem_u32(&bars[0]), bar_mma = smem_u32(&bars[1]);

  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_load));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_mma));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    state = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (threadIdx.x == 0) {
    const int pairs = has2 ? 2 : 1;
    const uint32_t bytes = (uint32_t)(pairs * (L::kA + L::kW));
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_load), "r"(bytes) : "memory");
    // skip_loads (the wait-timeout check only): no copy is issued, so the
    // load barrier never completes and the bounded wait below runs out.
    for (int p = 0; p < (skip_loads ? 0 : pairs); ++p) {
      const CUtensorMap* ta = p ? &tA2 : &tA;
      const CUtensorMap* tw = p ? &tW2 : &tW;
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
              "r"(smem_u32(sA[p])),
          "l"((uint64_t)ta), "r"(0), "r"(row0), "r"(bar_load)
          : "memory");
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
              "r"(smem_u32(sW[p])),
          "l"((uint64_t)tw), "r"(0), "r"(0), "r"(bar_load)
          : "memory");
    }
    if (!mbar_wait(bar_load, 0, wait_limit)) {
      state = 1;
      // The copies may still land in this CTA's shared memory: wait eight
      // times as long again before the tile is given up.  If even that runs
      // out, copies can outlive the CTA; the host then refuses further solves
      // on the handle and the caller must treat the context as unusable.
      mbar_wait(bar_load, 0, 8 * wait_limit);
    } else {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      int first = 1;
      for (int p = 0; p < pairs; ++p) {
#pragma unroll
        for (int k = 0; k < K / 16; ++k) {  // 16 bf16 = 32 bytes of K per instruction
          const uint64_t da = smem_desc(smem_u32(sA[p]) + 32 * k, L::kSbo, L::kSwizzle);
          const uint64_t db = smem_desc(smem_u32(sW[p]) + 32 * k, L::kSbo, L::kSwizzle);
          const uint32_t acc = first ? 0u : 1u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(da), "l"(db), "r"(kIdesc), "r"(acc));
          first = 0;
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_mma)
                   : "memory");
    }
  }
  __syncthreads();
  if (state == 0) {
    if (!mbar_wait(bar_mma, 0, wait_limit)) {
      state = 2;  // every thread that sees the timeout records it (same value)
      mbar_wait(bar_mma, 0, 8 * wait_limit);  // MMAs in flight: wait longer before the tensor memory is freed
    }
  }
  __syncthreads();
  if (state == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int64_t row = (int64_t)row0 + warp * 32 + lane;
    float acc[kTileN];
#pragma unroll
    for (int c = 0; c < kTileN; c += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 16; ++j) acc[c + j] = __uint_as_float(r[j]);
    }
    if (row < n) {
      float4* z4 = reinterpret_cast<float4*>(Z + row * kTileN);
#pragma unroll
      for (int c = 0; c < kTileN; c += 4) {
        const float4 b = bias ? *reinterpret_cast<const float4*>(bias + c) : make_float4(0.f, 0.f, 0.f, 0.f);
        z4[c / 4] = make_float4(acc[c] + b.x, acc[c + 1] + b.y, acc[c + 2] + b.z, acc[c + 3] + b.w);
        acc[c] += b.x; acc[c + 1] += b.y; acc[c + 2] += b.z; acc[c + 3] += b.w;
      }
      if (H) {
        uint4* h4 = reinterpret_cast<uint4*>(H + row * kTileN);
#pragma unroll
        for (int c = 0; c < kTileN; c += 8) {
          __nv_bfloat162 v[4];
#pragma unroll
          for (int j = 0; j < 4; ++j)
            v[j] = __floats2bfloat162_rn(fmaxf(acc[c + 2 * j], 0.f), fmaxf(acc[c + 2 * j + 1], 0.f));
          uint4 u;
          std::memcpy(&u, v, sizeof(u));
          h4[c / 8] = u;
        }
      }
    }
  } else if (threadIdx.x == 0 && fatal) {
    atomicExch(fatal, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// Row-major [rows][K] bf16 matrix, boxes of box_rows x K.
bool tensor_map(CUtensorMap* m, const bf16* ptr, int64_t rows, int K, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc || ((uintptr_t)ptr & 15) || rows <= 0) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  const cuuint32_t box[2] = {(cuuint32_t)K, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUtensorMapSwizzle sw = K == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int K>
cudaError_t launch_tc(int64_t n, const bf16* A, const bf16* W, const bf16* A2, const bf16* W2, const float* bias,
                      float* Z, bf16* H, int* fatal, cudaStream_t st, long wait_limit = kWaitLimit,
                      int skip_loads = 0) {
  CUtensorMap tA, tW, tA2, tW2;
  const bool two = A2 && W2;
  if (!tensor_map(&tA, A, n, K, kTileM) || !tensor_map(&tW, W, kTileN, K, kTileN)) return cudaErrorInvalidValue;
  if (two) {
    if (!tensor_map(&tA2, A2, n, K, kTileM) || !tensor_map(&tW2, W2, kTileN, K, kTileN)) return cudaErrorInvalidValue;
  } else {
    tA2 = tA;
    tW2 = tW;
  }
  if (((uintptr_t)Z & 15) || ((uintptr_t)H & 15) || ((uintptr_t)bias & 15)) return cudaErrorInvalidValue;
  const unsigned grid = (unsigned)((n + kTileM - 1) / kTileM);
  k_gnn_gemm_tc<K><<<grid, 128, TcSmem<K>::kBytes, st>>>(n, tA, tW, tA2, tW2, two ? 1 : 0, bias, Z, H, fatal,
                                                          wait_limit, skip_loads);
  return cudaGetLastError();
}

}  // namespace

cudaError_t gnn_gemm_tc_prepare() {
  cudaError_t e = cudaFuncSetAttribute(k_gnn_gemm_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       TcSmem<64>::kBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_gnn_gemm_tc<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcSmem<32>::kBytes);
  return e;
}

cudaError_t gnn_gemm_tc_wait_check(int64_t n, const bf16* A, const bf16* W, float* Z, int* fatal, cudaStream_t st) {
  if (n <= 0) return cudaErrorInvalidValue;
  return launch_tc<64>(n, A, W, nullptr, nullptr, nullptr, Z, nullptr, fatal, st, 1L << 14, 1);
}

cudaError_t gnn_gemm_tc(int64_t n, int K, const bf16* A, const bf16* W, const bf16* A2, const bf16* W2,
                        const float* bias, float* Z, bf16* H, int* fatal, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (K == 64) return launch_tc<64>(n, A, W, A2, W2, bias, Z, H, fatal, st);
  if (K == 32) return launch_tc<32>(n, A, W, A2, W2, bias, Z, H, fatal, st);
  return cudaErrorInvalidValue;
}

}  // namespace mba
