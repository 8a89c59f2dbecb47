// Measured FP64 arithmetic peak of the device (mba_measure_fp64_peak in
// include/maplab_ba.h): the denominator of the FP64 evaluation kernel's
// roofline.  GB300's FP64 pipe is narrow, so the FP64 kernels of this library
// are bound by it rather than by HBM; the peak is measured rather than taken
// from a data sheet.
//
// Every thread runs kChains independent dependent-FMA chains
// (x <- x * b + c, b < 1, so the values stay near c / (1 - b) and never
// overflow or turn subnormal) for `iters` steps; one FMA counts as two FLOPs.
#include <cuda_runtime.h>

#include <vector>

#include "../../include/maplab_ba.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fp64_fma_loop(int iters, double b, double c, double* out) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = fma(x[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  // The sum is written only under a condition the host never makes true, so
  // the loop cannot be removed and nothing is stored in a normal run.
  if (s == -1.0) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" mba_status mba_measure_fp64_peak(int32_t device, double* tflops) {
  if (!tflops) return MBA_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MBA_ERR_NO_DEVICE;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
    return MBA_ERR_CUDA;
  const int blocks = sms * 8, iters = 4096;
  cudaStream_t st = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  const int reps = 5;
  for (int w = 0; w < 2 && e == cudaSuccess; ++w) {
    k_fp64_fma_loop<<<blocks, kThreads, 0, st>>>(iters, 0.999999, 1e-6, nullptr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(a, st);
  for (int r = 0; r < reps && e == cudaSuccess; ++r) {
    k_fp64_fma_loop<<<blocks, kThreads, 0, st>>>(iters, 0.999999, 1e-6, nullptr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(b, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess || !(ms > 0.f)) return MBA_ERR_CUDA;
  const double flops = 2.0 * kChains * (double)iters * blocks * kThreads * reps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return MBA_OK;
}
