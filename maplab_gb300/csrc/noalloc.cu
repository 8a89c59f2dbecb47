// Allocation-free evaluation of the robustified visual cost
// (mba_visual_cost_noalloc in include/maplab_ba.h).
//
// Intended for callers that may not allocate device memory while they run: a
// real-time visual-inertial estimator thread that must not stall on the
// device-wide synchronization of cudaMalloc / cudaFree or fail on an
// out-of-memory error mid-mission, or an application whose device memory is
// owned by another allocator (a framework's caching pool) that foreign
// cudaMalloc calls would fragment.  The caller passes its own device arrays
// for inputs and the output; every intermediate lives in the file-scope
// scratch array below, which each GPU that loads this library holds until the
// process exits.
//
// Per call: kernel 1 clears the flags, kernel 2 writes one FP64 partial cost
// per 256-observation block into the scratch array, kernel 3 sums the partials
// in a fixed order (deterministic) and writes the cost to the caller's output.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/maplab_ba.h"
#include "device_math.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 65536;  // => at most 16,777,216 observations per call
constexpr int kFlagBadIndex = kMaxBlocks;
constexpr int kFlagNonFinite = kMaxBlocks + 1;

// 65,538 doubles = 512 KiB + 16 B of device memory per GPU.
static __device__ __align__(256) double g_noalloc_scratch[kMaxBlocks + 2];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// Host code cannot use &g_noalloc_scratch (a host-side stand-in); the device
// address is looked up once per device, with that device current.
mba_status scratch_for_device(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return MBA_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return MBA_ERR_CUDA;
    g_scratch_ptr[device] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[device];
  return MBA_OK;
}

__global__ void k_noalloc_clear(double* scratch) {
  scratch[kFlagBadIndex] = 0.0;
  scratch[kFlagNonFinite] = 0.0;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(kThreads) k_noalloc_visual_cost(mba_visual_batch_device b, double* scratch) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double cost = 0.0;
  if (i < b.num_observations) {
    const int l = b.obs_landmark[i], k = b.obs_keyframe[i], c = b.obs_camera[i];
    bool bad = l < 0 || l >= b.num_landmarks || k < 0 || k >= b.num_keyframes || c < 0 || c >= b.num_cameras;
    const int s = bad ? 0 : b.lm_store_keyframe[l];
    bad = bad || s < 0 || s >= b.num_keyframes;
    const int ms = bad ? 0 : b.kf_mission[s], mo = bad ? 0 : b.kf_mission[k];
    bad = bad || ms < 0 || ms >= b.num_missions || mo < 0 || mo >= b.num_missions;
    if (bad) {
      atomicAdd(&scratch[kFlagBadIndex], 1.0);
    } else {
      using namespace mba;
      const mba_camera& cam = b.cameras[c];
      const int type = (k == s) ? MBA_LOCAL_KEYFRAME : (ms == mo ? MBA_LOCAL_MISSION : MBA_GLOBAL);
      const double* pB = b.lm_p_B + 3 * (int64_t)l;
      M3<double> RCI;
      jplR(cam.q_CI_p_CI, RCI);
      double pI[3];
      if (type == MBA_LOCAL_KEYFRAME) {
        pI[0] = pB[0]; pI[1] = pB[1]; pI[2] = pB[2];
      } else {
        const double* xs = b.kf_q_IM_p_MI + 7 * (int64_t)s;
        const double* xo = b.kf_q_IM_p_MI + 7 * (int64_t)k;
        M3<double> RBLM, RIM;
        jplR(xs, RBLM);
        jplR(xo, RIM);
        double pM[3];
        mtv3(RBLM, pB, pM);
        pM[0] += xs[4]; pM[1] += xs[5]; pM[2] += xs[6];
        if (type == MBA_GLOBAL) {
          const double* ml = b.mission_q_GM_p_GM + 7 * (int64_t)ms;
          const double* mo7 = b.mission_q_GM_p_GM + 7 * (int64_t)mo;
          M3<double> RGLM, RGM;
          jplR(ml, RGLM);
          jplR(mo7, RGM);
          double pG[3];
          mv3(RGLM, pM, pG);
          pG[0] += ml[4] - mo7[4]; pG[1] += ml[5] - mo7[5]; pG[2] += ml[6] - mo7[6];
          mtv3(RGM, pG, pM);
        }
        const double d[3] = {pM[0] - xo[4], pM[1] - xo[5], pM[2] - xo[6]};
        mv3(RIM, d, pI);
      }
      double pC[3];
      mv3(RCI, pI, pC);
      pC[0] += cam.q_CI_p_CI[4]; pC[1] += cam.q_CI_p_CI[5]; pC[2] += cam.q_CI_p_CI[6];
      DevCamera dc;
      for (int a = 0; a < 4; ++a) { dc.intr[a] = cam.intrinsics[a]; dc.dist[a] = cam.distortion[a]; }
      dc.dtype = cam.distortion_type;
      dc.width = cam.width;
      dc.height = cam.height;
      double kp[2];
      const bool failed = project<double>(dc, pC, kp, nullptr);
      if (!failed) {
        const double sigma = b.obs_sigma[i];
        const double r0 = (kp[0] - b.obs_uv[2 * i]) / sigma, r1 = (kp[1] - b.obs_uv[2 * i + 1]) / sigma;
        const double sq = r0 * r0 + r1 * r1;
        const double a = b.use_huber ? (type == MBA_GLOBAL ? b.huber_delta_global : b.huber_delta_local) * sigma : 0.0;
        cost = (a > 0.0 && sq > a * a) ? 0.5 * (2.0 * a * sqrt(sq) - a * a) : 0.5 * sq;
        if (!isfinite(cost)) {
          atomicAdd(&scratch[kFlagNonFinite], 1.0);
          cost = 0.0;
        }
      }
    }
  }
  __shared__ double red[kThreads / 32];
  cost = warp_sum(cost);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cost;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) s += red[w];
    scratch[blockIdx.x] = s;  // every partial slot used by this call is written
  }
}

__global__ void __launch_bounds__(kThreads) k_noalloc_reduce(const double* scratch, int nblocks, double* out) {
  __shared__ double red[kThreads];
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += kThreads) s += scratch[b];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

}  // namespace

extern "C" mba_status mba_visual_cost_noalloc(const mba_visual_batch_device* batch, int32_t device, void* stream,
                                              double* cost_out_device) {
  if (!batch || !cost_out_device) return MBA_ERR_INVALID_ARG;
  const int64_t n = batch->num_observations;
  if (n < 0 || n > (int64_t)kMaxBlocks * kThreads) return MBA_ERR_INVALID_ARG;
  if (batch->num_keyframes <= 0 || batch->num_missions <= 0 || batch->num_cameras <= 0 || batch->num_landmarks < 0)
    return MBA_ERR_INVALID_ARG;
  if (n > 0 && (!batch->obs_uv || !batch->obs_sigma || !batch->obs_landmark || !batch->obs_keyframe ||
                !batch->obs_camera || !batch->lm_store_keyframe || !batch->lm_p_B || !batch->kf_q_IM_p_MI ||
                !batch->kf_mission || !batch->mission_q_GM_p_GM || !batch->cameras))
    return MBA_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MBA_ERR_NO_DEVICE;
  // An error the caller's own work left pending is not this call's to clear:
  // report it without launching and leave it for the caller to read.
  if (cudaPeekAtLastError() != cudaSuccess) return MBA_ERR_CUDA;
  double* scratch = nullptr;
  mba_status st = scratch_for_device(device, &scratch);
  if (st != MBA_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblocks = (int)((n + kThreads - 1) / kThreads);
  // Nothing was pending on entry, so an error read here comes from these launches.
  k_noalloc_clear<<<1, 1, 0, s>>>(scratch);
  if (cudaGetLastError() != cudaSuccess) return MBA_ERR_CUDA;
  if (nblocks > 0) {
    k_noalloc_visual_cost<<<nblocks, kThreads, 0, s>>>(*batch, scratch);
    if (cudaGetLastError() != cudaSuccess) return MBA_ERR_CUDA;
  }
  k_noalloc_reduce<<<1, kThreads, 0, s>>>(scratch, nblocks, cost_out_device);
  if (cudaGetLastError() != cudaSuccess) return MBA_ERR_CUDA;
  double flags[2] = {0.0, 0.0};
  if (cudaMemcpyAsync(flags, scratch + kFlagBadIndex, sizeof(flags), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return MBA_ERR_CUDA;
  if (flags[0] > 0.0) return MBA_ERR_OUT_OF_RANGE_INDEX;
  if (flags[1] > 0.0) return MBA_ERR_NON_FINITE;
  return MBA_OK;
}
