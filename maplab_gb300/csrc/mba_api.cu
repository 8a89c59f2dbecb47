// C ABI of the GB300 VI bundle-adjustment back-end (include/maplab_ba.h).
//
// mba_create restates the parts of map_optimization::constructOptimizationProblem
// (algorithms/map-optimization/src/vi-optimization-builder.cc:154-374) and
// OptimizationStateBuffer::importStatesOfMissions
// (src/optimization-state-buffer.cc:153-264) that decide which blocks exist,
// which are constant and which local parameterization they carry; the input
// descriptor already holds the JPL state arrays.  mba_solve replaces
// map_optimization::solve (src/solver.cc:14-44), i.e. ceres::Solve with the
// options of include/map-optimization/solver-options.h:26-75.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "../../include/maplab_ba.h"
#include "solver.h"

using namespace mba;

namespace {

struct DeviceArena {
  std::vector<void*> ptrs;
  int64_t bytes = 0;
  cudaError_t err = cudaSuccess;
  template <typename T>
  T* alloc(int64_t n) {
    if (n <= 0) n = 1;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, sizeof(T) * (size_t)n);
    if (e != cudaSuccess) { err = e; return nullptr; }
    ptrs.push_back(p);
    bytes += (int64_t)sizeof(T) * n;
    return static_cast<T*>(p);
  }
  template <typename T>
  T* upload(const std::vector<T>& v, cudaStream_t s) {
    T* d = alloc<T>((int64_t)v.size());
    if (d && !v.empty()) {
      cudaError_t e = cudaMemcpyAsync(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) err = e;
    }
    return d;
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
    bytes = 0;
  }
};

// Open-addressing map (i, j) -> block index for the pose-pose pattern.
struct PairMap {
  std::vector<uint64_t> keys;
  std::vector<int32_t> vals;
  uint64_t mask = 0;
  int32_t count = 0;
  std::vector<int32_t> bi, bj;
  explicit PairMap(int64_t expected) {
    uint64_t cap = 1024;
    while (cap < (uint64_t)(expected * 2 + 16)) cap <<= 1;
    keys.assign(cap, ~0ull);
    vals.assign(cap, -1);
    mask = cap - 1;
  }
  void grow() {
    std::vector<uint64_t> ok = std::move(keys);
    std::vector<int32_t> ov = std::move(vals);
    const uint64_t cap = (mask + 1) * 2;
    keys.assign(cap, ~0ull);
    vals.assign(cap, -1);
    mask = cap - 1;
    for (size_t a = 0; a < ok.size(); ++a)
      if (ok[a] != ~0ull) place(ok[a], ov[a]);
  }
  void place(uint64_t key, int32_t v) {
    uint64_t h = (key * 0x9E3779B97F4A7C15ull) & mask;
    while (keys[h] != ~0ull) h = (h + 1) & mask;
    keys[h] = key;
    vals[h] = v;
  }
  int32_t get(int32_t i, int32_t j) {
    if (i > j) std::swap(i, j);
    const uint64_t key = ((uint64_t)(uint32_t)i << 32) | (uint32_t)j;
    uint64_t h = (key * 0x9E3779B97F4A7C15ull) & mask;
    while (keys[h] != ~0ull) {
      if (keys[h] == key) return vals[h];
      h = (h + 1) & mask;
    }
    if ((uint64_t)(count + 1) * 2 > mask) {
      grow();
      return get(i, j);
    }
    keys[h] = key;
    vals[h] = count;
    bi.push_back(i);
    bj.push_back(j);
    return count++;
  }
  // Index of the (i, j) block, -1 if absent (no insertion).
  int32_t find(int32_t i, int32_t j) const {
    if (i > j) std::swap(i, j);
    const uint64_t key = ((uint64_t)(uint32_t)i << 32) | (uint32_t)j;
    uint64_t h = (key * 0x9E3779B97F4A7C15ull) & mask;
    while (keys[h] != ~0ull) {
      if (keys[h] == key) return vals[h];
      h = (h + 1) & mask;
    }
    return -1;
  }
};

template <typename T>
struct SolverBuffers {
  bool ready = false;
  bool chain_ready = false;
  ChainSystem<T> C{};
  VisualLin<T> vis{};
  InertialLin<T> ine{};
  LinearSystem<T> L{};
};

}  // namespace

// Learned-preconditioner model: parameters and Adam state on one device.
struct mba_gnn {
  int device = 0;
  DeviceArena arena;
  GnnParams p{};
};

constexpr int kLinChunks = 8;  // chunks of the FP64 linearization into page-locked host memory

struct mba_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy = nullptr;             // device-to-host copies overlapping the next chunk's evaluation
  cudaEvent_t chunk_ev[kLinChunks] = {};
  DeviceArena arena;
  DevProblem P{};
  SchurPattern S{};
  std::atomic<int> cancel{0};
  // host copies used by the API
  std::vector<int64_t> perm;  // sorted -> caller observation index
  std::vector<int32_t> lm_caller;  // internal -> caller landmark index (empty: the same)
  int32_t* lm_caller_dev = nullptr;
  // solver state (lazily allocated)
  bool solver_ready = false;
  SolverBuffers<double> b64;
  SolverBuffers<float> b32;
  InertialLin<double> ine_cur{}, ine_cand{};
  ScaleVectors sc{};
  LmControl* ctl = nullptr;
  mba_iteration_summary* log = nullptr;
  int log_capacity = 0;
  double* kf_cand = nullptr;
  double* lm_cand = nullptr;
  float* kf_cand_f = nullptr;
  float* lm_cand_f = nullptr;
  double* sw_cand = nullptr;  // [nsw] candidate switch variables
  double* scratch = nullptr;  // [4] cost accumulators
  int* iscratch = nullptr;    // [4] flags
  // staging in the caller's layout (lazily allocated)
  double* stage_state = nullptr;  // 16 NK + 3 NL
  double* stage_lin = nullptr;    // 32 N
  int64_t* obs_inv = nullptr;     // [N] caller observation index -> sorted index
  CallerObs cobs{};               // observation fields in caller order (chunked host linearization)
  char* l2_flush = nullptr;       // buffer larger than L2 for timing hygiene
  // learned preconditioner
  GnnGraph gg{};
  GnnWork gw{};
  bool gw_ready = false;
  mba_gnn* model = nullptr;
  // options of the running solve read while recording the iteration graph
  int outlier_reproj = 0;
  double outlier_max_px = 50.0;
  int jacobi = 1;
  // cancellation seen by the device-driven loop (mapped pinned host memory)
  volatile int* cancel_host = nullptr;
  const volatile int* cancel_dev = nullptr;
  // Schur pair targets in kernel order (pair range per target) for re-cutting
  // the chunks under a tuned chunk size
  std::vector<int64_t> tgt_off, tgt_order;
  std::vector<int32_t> tgt_row;  // keyframe row of each target in tgt_order
  mba_tuning tuning{};
  // Set when a bounded device wait ran out during a solve or a training call
  // (MBA_ERR_TIMEOUT): the work that wait guarded may still be in flight, so
  // later solves and training calls on this handle are refused.
  bool poisoned = false;
  // Global nodes (calibration / baseframe variables) of the reduced system.
  BorderSystem border{};
};

namespace {

// Cuts each target's contiguous pair range [off[r], off[r+1]) into chunks of
// at most `chunk` pairs (one thread each); a target spanning several chunks
// is marked by the bitwise-not of its id.  Chunks are then grouped by the
// target's keyframe row (row_of[r], rows ascending; one block per row) and,
// within a row, ordered by length (longest first, stable) so that the 32
// lanes of a warp loop over similar pair counts.  row_chunk_off [nkf + 1]
// receives each row's chunk range.
void cut_chunks(const std::vector<int64_t>& off, const std::vector<int64_t>& order,
                const std::vector<int32_t>& row_of, int64_t nkf, int64_t chunk, std::vector<int32_t>* tgt,
                std::vector<int64_t>* beg, std::vector<int32_t>* len, std::vector<int64_t>* row_chunk_off) {
  std::vector<int32_t> t, n, rw;
  std::vector<int64_t> b;
  const int64_t ntgt = (int64_t)order.size();
  for (int64_t r = 0; r < ntgt; ++r) {
    const int64_t b0 = off[r], b1 = off[r + 1];
    if (b1 == b0) continue;
    const bool whole = b1 - b0 <= chunk;
    for (int64_t c0 = b0; c0 < b1; c0 += chunk) {
      t.push_back(whole ? (int32_t)order[r] : ~(int32_t)order[r]);
      b.push_back(c0);
      n.push_back((int32_t)(std::min(b1, c0 + chunk) - c0));
      rw.push_back(row_of[r]);
    }
  }
  std::vector<int64_t> idx(t.size());
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int64_t x, int64_t y) {
    return rw[x] != rw[y] ? rw[x] < rw[y] : n[x] > n[y];
  });
  row_chunk_off->assign(nkf + 1, 0);
  for (int32_t r : rw) (*row_chunk_off)[r + 1]++;
  for (int64_t k = 0; k < nkf; ++k) (*row_chunk_off)[k + 1] += (*row_chunk_off)[k];
  tgt->resize(t.size());
  beg->resize(t.size());
  len->resize(t.size());
  for (size_t q = 0; q < idx.size(); ++q) {
    (*tgt)[q] = t[idx[q]];
    (*beg)[q] = b[idx[q]];
    (*len)[q] = n[idx[q]];
  }
}

mba_status cuda_status(cudaError_t e) { return e == cudaSuccess ? MBA_OK : MBA_ERR_CUDA; }

bool quat_ok(const double* q) {
  const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  return std::isfinite(n) && std::fabs(n - 1.0) < 1e-5;  // assertValidQuaternion (optimization-state-buffer.h:63-80)
}

// Square-root information M = L^-1 (row-major, lower triangular) of a 6x6
// covariance with cov = L L^T, so that the whitened residual is e^T M
// (SixDoFBlockPoseErrorTermWithExtrinsics constructor: Cholesky of the
// covariance, then the inverse of its factor).  False if not positive definite.
bool pose_edge_sqrt_information(const double* cov, double* M) {
  double L[36] = {};
  for (int j = 0; j < 6; ++j) {
    double diag = cov[7 * j];
    for (int k = 0; k < j; ++k) diag -= L[6 * j + k] * L[6 * j + k];
    if (!(diag > 0.0)) return false;
    L[7 * j] = std::sqrt(diag);
    for (int i = j + 1; i < 6; ++i) {
      double v = cov[6 * i + j];
      for (int k = 0; k < j; ++k) v -= L[6 * i + k] * L[6 * j + k];
      L[6 * i + j] = v / L[7 * j];
    }
  }
  // forward substitution, one column of L^-1 at a time
  for (int c = 0; c < 6; ++c)
    for (int i = 0; i < 6; ++i) {
      if (i < c) { M[6 * i + c] = 0.0; continue; }
      double v = (i == c) ? 1.0 : 0.0;
      for (int k = c; k < i; ++k) v -= L[6 * i + k] * M[6 * k + c];
      M[6 * i + c] = v / L[7 * i];
    }
  return true;
}

template <typename T>
mba_status ensure_solver_buffers(mba_handle* h, SolverBuffers<T>& b) {
  if (b.ready) return MBA_OK;
  const DevProblem& P = h->P;
  DeviceArena& A = h->arena;
  const int64_t N = P.nobs, NL = P.nlm, NK = P.nkf, NE = P.nedge, NS = h->S.nslot, NPU = h->S.npu;
  const int64_t NB = NK + P.ng;  // PCG blocks: keyframes, then the global nodes
  b.vis.r = A.alloc<T>(2 * N);
  b.vis.Jl = A.alloc<T>(6 * N);
  b.vis.Js = A.alloc<T>(12 * N);
  b.vis.Jo = A.alloc<T>(12 * N);
  if constexpr (sizeof(T) == 4) {  // FP64: the handle's current linearization (make_launch)
    b.ine.r = A.alloc<T>(15 * NE);
    b.ine.Jf = A.alloc<T>(225 * NE);
    b.ine.Jt = A.alloc<T>(225 * NE);
    b.ine.Js = A.alloc<T>(6 * (NE - P.nimu));
  }
  LinearSystem<T>& L = b.L;
  L.Hll = A.alloc<T>(9 * NL);
  L.gl = A.alloc<T>(3 * NL);
  L.Wslot = A.alloc<T>(kSlotStride * NS);
  L.Dbase = A.alloc<T>(225 * NK);
  L.Pbase = A.alloc<T>(36 * NPU);
  L.Ebase = A.alloc<T>(225 * NE);
  L.gc = A.alloc<T>(15 * NK);
  L.SD = A.alloc<T>(225 * NB);
  L.SP = A.alloc<T>(72 * NPU);
  L.SE = A.alloc<T>(225 * NE);
  L.rhs = A.alloc<T>(15 * NB);
  L.V = A.alloc<T>(9 * NL);
  L.U = A.alloc<T>(kSlotStride * NS);
  L.Minv = A.alloc<T>(225 * NB);
  L.x = A.alloc<T>(15 * NB);
  L.r = A.alloc<T>(15 * NB);
  L.z = A.alloc<T>(15 * NB);
  L.p = A.alloc<T>(15 * NB);
  L.q = A.alloc<T>(15 * NB);
  L.q2 = A.alloc<T>(15 * NB);
  L.dl = A.alloc<double>(3 * NL);
  L.skf = A.alloc<T>(15 * NB);
  L.slm = A.alloc<T>(3 * NL);
  L.Dpose = A.alloc<float>(sizeof(T) == 4 ? 24 * NK : 1);
  L.gpose = A.alloc<float>(sizeof(T) == 4 ? 8 * NK : 1);
  L.swH = A.alloc<T>(P.nsw);
  L.swg = A.alloc<T>(P.nsw);
  L.swW = A.alloc<T>(30 * P.nsw);
  L.swHi = A.alloc<T>(P.nsw);
  L.swx = A.alloc<double>(P.nsw);
  L.ssw = A.alloc<T>(P.nsw);
  if (A.err != cudaSuccess) return MBA_ERR_CUDA;
  if (solver_prepare<T>(h->S) != cudaSuccess) return MBA_ERR_CUDA;
  b.ready = true;
  return MBA_OK;
}

// Chain-preconditioner factors (allocated on first use).  The FP64 arrays
// double as the working-precision copies when T = double.
template <typename T>
mba_status ensure_chain_buffers(mba_handle* h, SolverBuffers<T>& b) {
  if (b.chain_ready) return MBA_OK;
  DeviceArena& A = h->arena;
  const int64_t n = h->P.nkf;
  ChainSystem<T>& C = b.C;
  C.A = A.alloc<double>(225 * n);
  C.B = A.alloc<double>(225 * n);
  if constexpr (sizeof(T) == 8) {
    C.F64 = A.alloc<double>(225 * n);
    C.CL64 = A.alloc<double>(225 * n);
    C.CR64 = A.alloc<double>(225 * n);
    C.XL64 = A.alloc<double>(225 * n);
    C.XR64 = A.alloc<double>(225 * n);
    C.F = C.F64; C.CL = C.CL64; C.CR = C.CR64; C.XL = C.XL64; C.XR = C.XR64;
  } else {  // the mixed path keeps the factors in FP32 only
    C.F64 = C.CL64 = C.CR64 = C.XL64 = C.XR64 = nullptr;
    C.F = A.alloc<T>(225 * n);
    C.CL = A.alloc<T>(225 * n);
    C.CR = A.alloc<T>(225 * n);
    C.XL = A.alloc<T>(225 * n);
    C.XR = A.alloc<T>(225 * n);
  }
  C.w = A.alloc<T>(15 * n);
  C.lc = A.alloc<T>(15 * n + 15);
  C.coef = A.alloc<double>(3 * n);
  C.comp = A.alloc<double>(6 * n);
  if (A.err != cudaSuccess) return MBA_ERR_CUDA;
  if (chain_default_coef(C.coef, n, h->stream) != cudaSuccess) return MBA_ERR_CUDA;
  b.chain_ready = true;
  return MBA_OK;
}

mba_status ensure_gnn_work(mba_handle* h) {
  if (h->gw_ready) return MBA_OK;
  DeviceArena& A = h->arena;
  const int64_t n = h->P.nkf, nnz = 2 * h->S.npu + 2 * h->P.nedge;
  GnnWork& w = h->gw;
  w.n = n;
  w.wgt = A.alloc<float>(nnz + 1);
  w.deg = A.alloc<float>(n);
  w.h[0] = w.x = A.alloc<__nv_bfloat16>(n * kGnnIn);
  for (int l = 0; l < kGnnLayers; ++l) {
    w.h[l + 1] = A.alloc<__nv_bfloat16>(n * kGnnHidden);
    w.m[l] = A.alloc<__nv_bfloat16>(n * (l == 0 ? kGnnIn : kGnnHidden));
    w.z[l] = A.alloc<float>(n * kGnnHidden);
  }
  w.o = A.alloc<float>(n * kGnnOut);
  w.dh = A.alloc<float>(n * kGnnHidden);
  w.dm = A.alloc<float>(n * kGnnHidden);
  w.dzb = A.alloc<__nv_bfloat16>(n * kGnnHidden);
  w.dcoef = A.alloc<float>(3 * n);
  w.vec = A.alloc<float>(5 * 15 * n);
  w.loss = A.alloc<double>(2);
  if (A.err != cudaSuccess) return MBA_ERR_CUDA;
  if (gnn_gemm_tc_prepare() != cudaSuccess) return MBA_ERR_CUDA;  // shared-memory opt-in, outside graph capture
  h->gw_ready = true;
  return MBA_OK;
}

mba_status ensure_common_solver(mba_handle* h, int capacity) {
  DeviceArena& A = h->arena;
  const DevProblem& P = h->P;
  if (!h->solver_ready) {
    const int64_t NE = P.nedge;
    h->ine_cur.r = A.alloc<double>(15 * NE);
    h->ine_cur.Jf = A.alloc<double>(225 * NE);
    h->ine_cur.Jt = A.alloc<double>(225 * NE);
    h->ine_cand.r = A.alloc<double>(15 * NE);
    h->ine_cand.Jf = A.alloc<double>(225 * NE);
    h->ine_cand.Jt = A.alloc<double>(225 * NE);
    h->ine_cur.Js = A.alloc<double>(6 * (NE - P.nimu));
    h->ine_cand.Js = A.alloc<double>(6 * (NE - P.nimu));
    h->sc.skf = A.alloc<double>(15 * (P.nkf + P.ng));
    if (P.ng > 0) {
      BorderSystem& B = h->border;
      const int64_t G = P.ng;
      B.Gb = A.alloc<double>(225 * G * G);
      B.Bb = A.alloc<double>(90 * P.nkf * G);
      B.gg = A.alloc<double>(15 * G);
      B.GS = A.alloc<double>(225 * G * G);
      B.BS = A.alloc<double>(90 * P.nkf * G);
      B.bl = A.alloc<double>(3 * P.nlm);
      B.cams_cand = A.alloc<DevCamera>(P.ncam);
      B.mis_cand = A.alloc<double>(8 * P.nmis);
    }
    h->sc.slm = A.alloc<double>(3 * P.nlm);
    h->sc.ssw = A.alloc<double>(P.nsw);
    h->sw_cand = A.alloc<double>(P.nsw);
    h->ctl = A.alloc<LmControl>(1);
    h->kf_cand = A.alloc<double>(16 * P.nkf);
    h->lm_cand = A.alloc<double>(4 * P.nlm);
    h->kf_cand_f = A.alloc<float>(8 * P.nkf);
    h->lm_cand_f = A.alloc<float>(4 * P.nlm);
    if (A.err != cudaSuccess) return MBA_ERR_CUDA;
    h->solver_ready = true;
  }
  if (capacity > h->log_capacity) {
    h->log = A.alloc<mba_iteration_summary>(capacity);
    if (A.err != cudaSuccess) return MBA_ERR_CUDA;
    h->log_capacity = capacity;
  }
  return MBA_OK;
}

template <typename T>
SolverBuffers<T>& buffers_of(mba_handle* h) {
  if constexpr (sizeof(T) == 8) return h->b64; else return h->b32;
}

template <typename T>
SolverLaunch<T> make_launch(mba_handle* h, SolverBuffers<T>& b, const mba_solver_options& o) {
  // FP64 path: the solver reads the current inertial linearization directly.
  // Set before any graph capture records the pointer.
  if constexpr (sizeof(T) == 8) b.ine = h->ine_cur;
  SolverLaunch<T> s;
  s.P = h->P;
  s.S = h->S;
  s.L = b.L;
  s.vis = b.vis;
  s.ine = b.ine;
  s.sc = h->sc;
  s.ctl = h->ctl;
  s.prm.max_num_iterations = o.max_num_iterations;
  s.prm.max_linear_iterations = std::max(1, o.max_linear_iterations);
  s.prm.check_tolerances = o.check_tolerances;
  s.prm.reject_every = std::max(0, o.reject_outliers_every_n_iters);
  h->outlier_reproj = o.outlier_use_reprojection_error;
  h->outlier_max_px = o.outlier_max_reprojection_error_px;
  h->jacobi = o.jacobi_scaling;
  s.prm.max_radius = o.max_trust_region_radius;
  s.prm.min_radius = o.min_trust_region_radius;
  s.prm.function_tolerance = o.function_tolerance;
  s.prm.parameter_tolerance = o.parameter_tolerance;
  s.prm.min_relative_decrease = o.min_relative_decrease;
  s.prm.min_lm_diagonal = o.min_lm_diagonal;
  s.prm.max_lm_diagonal = o.max_lm_diagonal;
  s.prm.linear_tolerance = o.linear_tolerance;
  s.prm.stop_cost = o.stop_cost;
  s.prm.gradient_tolerance = o.gradient_tolerance;
  s.log = h->log;
  s.kf_cand = h->kf_cand;
  s.lm_cand = h->lm_cand;
  s.kf_cand_f = sizeof(T) == 4 ? h->kf_cand_f : nullptr;
  s.lm_cand_f = sizeof(T) == 4 ? h->lm_cand_f : nullptr;
  s.sw_cand = h->sw_cand;
  s.C = b.C;
  s.precond = (o.preconditioner == MBA_PRECOND_CHAIN || o.preconditioner == MBA_PRECOND_LEARNED) && b.chain_ready
                  ? o.preconditioner : MBA_PRECOND_BLOCK_JACOBI;
  if (s.precond == MBA_PRECOND_LEARNED && !(h->model && h->gw_ready)) s.precond = MBA_PRECOND_CHAIN;
  s.gg = h->gg;
  s.gw = h->gw;
  if (h->model) s.gp = h->model->p;
  s.B = h->border;
  return s;
}

// Cost, inertial and visual linearization at the current state, assembly and
// Jacobi scaling (the work before the first LM iteration).
template <typename T>
cudaError_t linearize_current(mba_handle* h, SolverBuffers<T>& b, SolverLaunch<T>& s, int jacobi, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(&h->ctl->cost, 0, sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(&h->ctl->cost_ine, 0, sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->iscratch, 0, 2 * sizeof(int), st);
  // Mixed path: FP32 residuals from the FP32 state copies, FP64 sum (as its
  // candidates are costed).
  if (e == cudaSuccess)
    e = sizeof(T) == 4 ? launch_visual_cost_f32(h->P, h->P.kf_pose_f, h->P.lm_p_f, &h->ctl->cost, h->iscratch, nullptr, st)
                       : launch_visual_cost(h->P, h->P.kf_state, h->P.lm_p, &h->ctl->cost, h->iscratch, st);
  if (e == cudaSuccess)
    e = launch_inertial_gated(h->P, h->P.kf_state, h->ine_cur, &h->ctl->cost_ine, h->iscratch + 1, nullptr, st,
                              sizeof(T) == 4);
  if (e == cudaSuccess) e = solver_add_inertial_cost(h->ctl, st);
  if constexpr (sizeof(T) == 4) {
    if (e == cudaSuccess) e = launch_inertial_f32(h->P, h->ine_cur, b.ine, st);
  }
  if (e == cudaSuccess) e = launch_visual_linearize<T>(h->P, b.vis, nullptr, st);
  if (e == cudaSuccess) e = solver_assemble<T>(s, nullptr, st);
  if (e == cudaSuccess) e = solver_compute_scale<T>(s, jacobi, st);
  return e;
}

// Records one LM iteration (graph body) on the stream.
template <typename T>
cudaError_t record_iteration(mba_handle* h, const SolverLaunch<T>& s) {
  cudaStream_t st = h->stream;
  cudaError_t e = solver_step<T>(s, st);
  if (e == cudaSuccess) e = solver_evaluate_candidate<T>(s, h->ine_cand, st);
  if (e == cudaSuccess) e = solver_decide_and_accept<T>(s, h->ine_cand, h->ine_cur, st);
  if (e == cudaSuccess) e = solver_relinearize<T>(s, h->ine_cur, st);
  if (e == cudaSuccess && s.prm.reject_every > 0)
    e = solver_reject_and_restart<T>(s, h->outlier_reproj, h->outlier_max_px, h->jacobi, st);
  return e;
}

template <typename T>
mba_status run_solve(mba_handle* h, const mba_solver_options& o, mba_summary* sum) {
  mba_status ms = ensure_common_solver(h, o.max_num_iterations + 2);
  if (ms != MBA_OK) return ms;
  SolverBuffers<T>& b = buffers_of<T>(h);
  ms = ensure_solver_buffers<T>(h, b);
  if (ms != MBA_OK) return ms;
  if (o.preconditioner == MBA_PRECOND_LEARNED) {
    if (!h->model || h->model->device != h->device) return MBA_ERR_INVALID_ARG;
    ms = ensure_gnn_work(h);
    if (ms != MBA_OK) return ms;
  }
  if (o.preconditioner == MBA_PRECOND_CHAIN || o.preconditioner == MBA_PRECOND_LEARNED) {
    ms = ensure_chain_buffers<T>(h, b);
    if (ms != MBA_OK) return ms;
    if (o.preconditioner == MBA_PRECOND_CHAIN && chain_default_coef(b.C.coef, h->P.nkf, h->stream) != cudaSuccess)
      return MBA_ERR_CUDA;
  }
  SolverLaunch<T> s = make_launch<T>(h, b, o);
  cudaStream_t st = h->stream;
  cudaError_t e = cudaSuccess;
  // Graphs first (host work outside the timed region): the whole LM loop as
  // one graph with a device-evaluated while condition, or one iteration per
  // graph launched from the host.
  cudaGraphExec_t exec = nullptr;
  bool device_loop = false;
  if (o.use_cuda_graph == 2) {
    cudaGraph_t graph = nullptr;
    cudaGraphConditionalHandle cond;
    e = cudaGraphCreate(&graph, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault);
    // cudaGraphNodeParams (a union of node parameter types) is zero-initialised storage.
    alignas(cudaGraphNodeParams) unsigned char np_raw[sizeof(cudaGraphNodeParams)];
    std::memset(np_raw, 0, sizeof(np_raw));
    cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(np_raw);
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
    if (e == cudaSuccess) {
      cudaGraph_t body = np.conditional.phGraph_out[0];
      e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t e2 = record_iteration<T>(h, s);
        if (e2 == cudaSuccess) e2 = solver_loop_control(h->ctl, cond, h->cancel_dev, st);
        e = cudaStreamEndCapture(st, &body);
        if (e2 != cudaSuccess) e = e2;
      }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e == cudaSuccess) {
      device_loop = true;
    } else {  // no conditional nodes here: fall back to one graph per iteration
      if (exec) cudaGraphExecDestroy(exec);
      exec = nullptr;
      cudaGetLastError();
      e = cudaSuccess;
    }
  }
  if (!exec && o.use_cuda_graph) {
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      cudaError_t e2 = record_iteration<T>(h, s);
      e = cudaStreamEndCapture(st, &graph);
      if (e2 != cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      if (exec) cudaGraphExecDestroy(exec);
      return MBA_ERR_CUDA;
    }
  }
  if (h->cancel_host) *h->cancel_host = 0;
  cudaEvent_t ev0;
  cudaEventCreate(&ev0);
  std::vector<cudaEvent_t> evs(device_loop ? 0 : o.max_num_iterations);
  for (auto& ev : evs) cudaEventCreate(&ev);
  const auto t0 = std::chrono::steady_clock::now();
  cudaEventRecord(ev0, st);
  // Initial evaluation: FP64 cost, inertial linearization, visual linearization, assembly, scaling.
  e = solver_init_control(h->ctl, o.initial_trust_region_radius, st);
  if (e == cudaSuccess) e = solver_loop_start(h->ctl, st);
  if (e == cudaSuccess && h->P.ng > 0) {  // candidate cameras / baseframes start as the current ones
    e = cudaMemcpyAsync(h->border.cams_cand, h->P.cams, sizeof(DevCamera) * h->P.ncam, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->border.mis_cand, h->P.mis, sizeof(double) * 8 * h->P.nmis, cudaMemcpyDeviceToDevice, st);
  }
  if (e == cudaSuccess) e = linearize_current<T>(h, b, s, o.jacobi_scaling, st);
  // Ceres' gradient test at the start of the solve.
  if (e == cudaSuccess) e = solver_gradient_check<T>(s, nullptr, st);
  double initial_cost = 0.0;
  int flags[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&initial_cost, &h->ctl->cost, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(flags, h->iscratch, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  mba_status result = MBA_OK;
  if (e != cudaSuccess) result = MBA_ERR_CUDA;
  else if (flags[1]) result = (mba_status)flags[1];
  else if (flags[0] || !std::isfinite(initial_cost)) result = MBA_ERR_NON_FINITE;
  int launched = 0;
  if (result == MBA_OK && device_loop) {
    e = cudaGraphLaunch(exec, st);
    launched = o.max_num_iterations;
  } else if (result == MBA_OK) {
    for (int it = 0; it < o.max_num_iterations; ++it) {
      if (h->cancel.load()) { result = MBA_ERR_CANCELLED; break; }
      e = exec ? cudaGraphLaunch(exec, st) : record_iteration<T>(h, s);
      if (e != cudaSuccess) break;
      cudaEventRecord(evs[it], st);
      ++launched;
      // Poll for early termination every few iterations without stalling the queue.
      if ((it & 3) == 3) {
        int term = 0;
        cudaMemcpyAsync(&term, &h->ctl->terminated, sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        if (term) break;
      }
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  const double wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (exec) cudaGraphExecDestroy(exec);
  if (e != cudaSuccess) result = MBA_ERR_CUDA;
  LmControl c;
  std::memset(&c, 0, sizeof(c));
  if (result == MBA_OK || result == MBA_ERR_CANCELLED) cudaMemcpy(&c, h->ctl, sizeof(c), cudaMemcpyDeviceToHost);
  if (device_loop && c.termination == 5) result = MBA_ERR_CANCELLED;
  if (c.fatal) {
    result = MBA_ERR_TIMEOUT;
    h->poisoned = true;
  }
  std::vector<mba_iteration_summary> log(o.max_num_iterations + 1);
  cudaMemcpy(log.data(), h->log, sizeof(mba_iteration_summary) * log.size(), cudaMemcpyDeviceToHost);
  if (sum && (result == MBA_OK || result == MBA_ERR_CANCELLED)) {
    sum->initial_cost = initial_cost;
    sum->final_cost = c.cost;
    sum->num_iterations = c.iteration + 1;
    sum->num_successful_steps = c.num_successful;
    sum->termination = (result == MBA_ERR_CANCELLED) ? 5 : c.termination;
    sum->total_linear_iterations = c.total_pcg;
    sum->total_time_ms = wall_ms;
    sum->time_to_stop_cost_ms = -1.0;
    sum->num_rejected_landmarks = c.rejected;
    // Times from the first launch of the solve: device global timer (device
    // loop) or events after each iteration (host loop).
    auto iter_ms = [&](int it) -> double {
      if (device_loop) return log[it].iteration_time_ms;
      float ms = 0.f;
      if (it - 1 < launched) cudaEventElapsedTime(&ms, ev0, evs[it - 1]);
      return ms;
    };
    if (c.stop_iteration > 0 && c.stop_iteration <= launched) sum->time_to_stop_cost_ms = iter_ms(c.stop_iteration);
    if (sum->iterations && sum->max_iterations_capacity > 0) {
      mba_iteration_summary& z = sum->iterations[0];
      std::memset(&z, 0, sizeof(z));
      z.step_is_successful = 1;
      z.cost = initial_cost;
      z.trust_region_radius = o.initial_trust_region_radius;
      for (int it = 1; it <= c.iteration && it < sum->max_iterations_capacity; ++it) {
        sum->iterations[it] = log[it];
        sum->iterations[it].iteration_time_ms = iter_ms(it);
      }
    }
  }
  for (auto& ev : evs) cudaEventDestroy(ev);
  cudaEventDestroy(ev0);
  return result;
}


template <typename T>
static cudaError_t copy_out(double* dst, const T* src, int64_t n, cudaStream_t st) {
  if (!dst || n == 0) return cudaSuccess;
  std::vector<T> tmp(n);
  cudaError_t e = cudaMemcpyAsync(tmp.data(), src, sizeof(T) * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  for (int64_t i = 0; i < n && e == cudaSuccess; ++i) dst[i] = (double)tmp[i];
  return e;
}

template <typename T>
mba_status reduced_system(mba_handle* h, double radius, double* diag, int32_t* upper_ij, double* upper,
                          double* inertial, double* rhs) {
  mba_status ms = ensure_common_solver(h, 2);
  if (ms != MBA_OK) return ms;
  SolverBuffers<T>& b = buffers_of<T>(h);
  ms = ensure_solver_buffers<T>(h, b);
  if (ms != MBA_OK) return ms;
  mba_solver_options o;
  mba_default_solver_options(&o);
  SolverLaunch<T> s = make_launch<T>(h, b, o);
  cudaStream_t st = h->stream;
  cudaError_t e = solver_init_control(h->ctl, radius, st);
  if (e == cudaSuccess) e = linearize_current<T>(h, b, s, o.jacobi_scaling, st);
  if (e == cudaSuccess) e = solver_build_reduced<T>(s, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  const int64_t NK = h->P.nkf, NE = h->P.nedge, NPU = h->S.npu;
  if (e == cudaSuccess) e = copy_out<T>(diag, b.L.SD, 225 * NK, st);
  if (e == cudaSuccess) e = copy_out<T>(upper, b.L.SP, 36 * NPU, st);
  if (e == cudaSuccess) e = copy_out<T>(inertial, b.L.SE, 225 * NE, st);
  if (e == cudaSuccess) e = copy_out<T>(rhs, b.L.rhs, 15 * NK, st);
  if (e == cudaSuccess && upper_ij && NPU) {
    std::vector<int32_t> bi(NPU), bj(NPU);
    e = cudaMemcpy(bi.data(), h->S.pu_i, sizeof(int32_t) * NPU, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(bj.data(), h->S.pu_j, sizeof(int32_t) * NPU, cudaMemcpyDeviceToHost);
    for (int64_t q = 0; q < NPU && e == cudaSuccess; ++q) { upper_ij[2 * q] = bi[q]; upper_ij[2 * q + 1] = bj[q]; }
  }
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  int status = 0;
  cudaMemcpy(&status, &h->ctl->status, sizeof(int), cudaMemcpyDeviceToHost);
  return status ? (mba_status)status : MBA_OK;
}

// z = T^-1 r with the exact chain matrix T (gamma = 1, alpha = 0) of the
// reduced system at the current state, through the configured sweeps.
template <typename T>
mba_status chain_apply_host(mba_handle* h, double radius, const double* r, double* z) {
  mba_status ms = ensure_common_solver(h, 2);
  if (ms != MBA_OK) return ms;
  SolverBuffers<T>& b = buffers_of<T>(h);
  if ((ms = ensure_solver_buffers<T>(h, b)) != MBA_OK) return ms;
  if ((ms = ensure_chain_buffers<T>(h, b)) != MBA_OK) return ms;
  mba_solver_options o;
  mba_default_solver_options(&o);
  o.preconditioner = MBA_PRECOND_CHAIN;
  SolverLaunch<T> s = make_launch<T>(h, b, o);
  cudaStream_t st = h->stream;
  const int64_t n = 15 * h->P.nkf;
  std::vector<T> rt(n);
  for (int64_t i = 0; i < n; ++i) rt[i] = T(r[i]);
  cudaError_t e = chain_default_coef(b.C.coef, h->P.nkf, st);
  if (e == cudaSuccess) e = solver_init_control(h->ctl, radius, st);
  if (e == cudaSuccess) e = linearize_current<T>(h, b, s, o.jacobi_scaling, st);
  if (e == cudaSuccess) e = solver_build_reduced<T>(s, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b.L.r, rt.data(), sizeof(T) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = chain_apply<T>(s, b.L.r, b.L.z, &h->ctl->pcg_rz0, st);
  if (e == cudaSuccess) e = copy_out<T>(z, b.L.z, n, st);
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  int failed = 0;
  if (cudaMemcpy(&failed, &h->ctl->chain_failed, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return MBA_ERR_CUDA;
  return failed ? MBA_ERR_NOT_SPD : MBA_OK;
}

// Device address of a page-locked host range [p, p + bytes) of one mapping,
// or null (pageable or unknown memory, or a range that leaves the mapping).
void* mapped_host_range(void* p, size_t bytes) {
  if (!p || bytes == 0) return nullptr;
  cudaPointerAttributes a{}, z{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  char* last = static_cast<char*>(p) + bytes - 1;
  if (cudaPointerGetAttributes(&z, last) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  if (z.type != cudaMemoryTypeHost || z.devicePointer != static_cast<char*>(a.devicePointer) + bytes - 1) return nullptr;
  return a.devicePointer;
}

// FP64 rows into page-locked host memory in kLinChunks chunks of caller rows.
// Chunk c is evaluated from caller-ordered copies of the observation fields
// (so that its rows depend on no other chunk), transposed into the device
// staging rows, and copied to the host by the copy engine on a second stream
// while chunk c + 1 is evaluated.
mba_status linearize_visual_chunked(mba_handle* h, SolverBuffers<double>& b, double* const* out) {
  const int64_t N = h->P.nobs;
  cudaStream_t st = h->stream;
  cudaError_t e = cudaSuccess;
  DeviceArena& A = h->arena;
  if (!h->cobs.uv) {
    CallerObs c{};
    c.uv = A.alloc<double2>(N);
    c.sinv = A.alloc<double>(N);
    c.huber = A.alloc<double>(N);
    c.lm = A.alloc<int32_t>(N);
    c.kf = A.alloc<int32_t>(N);
    c.store = A.alloc<int32_t>(N);
    c.cam = A.alloc<uint8_t>(N);
    c.type = A.alloc<uint8_t>(N);
    if (A.err != cudaSuccess || launch_caller_obs(h->P, h->obs_inv, c, st) != cudaSuccess) return MBA_ERR_CUDA;
    h->cobs = c;
  }
  if (!h->stage_lin) {
    h->stage_lin = A.alloc<double>(32 * N);
    if (A.err != cudaSuccess) return MBA_ERR_CUDA;
  }
  if (!h->copy) e = cudaStreamCreateWithFlags(&h->copy, cudaStreamNonBlocking);
  for (int c = 0; c < kLinChunks && e == cudaSuccess; ++c)
    if (!h->chunk_ev[c]) e = cudaEventCreateWithFlags(&h->chunk_ev[c], cudaEventDisableTiming);
  DevProblem Pc = h->P;
  Pc.obs_uv = h->cobs.uv;
  Pc.obs_sinv = h->cobs.sinv;
  Pc.obs_huber = h->cobs.huber;
  Pc.obs_lm = h->cobs.lm;
  Pc.obs_kf = h->cobs.kf;
  Pc.obs_store = h->cobs.store;
  Pc.obs_cam = h->cobs.cam;
  Pc.obs_type = h->cobs.type;
  const int64_t width[4] = {2, 6, 12, 12}, first[4] = {0, 2, 8, 20};
  double* rows[4];
  for (int a = 0; a < 4; ++a) rows[a] = out[a] ? h->stage_lin + first[a] * N : nullptr;
  for (int c = 0; c < kLinChunks && e == cudaSuccess; ++c) {
    const int64_t lo = N * c / kLinChunks, hi = N * (c + 1) / kLinChunks;
    Pc.vis_lo = lo;
    Pc.vis_hi = hi;
    e = launch_visual_linearize<double>(Pc, b.vis, nullptr, st);
    if (e == cudaSuccess) e = launch_gather_rows<double>(Pc, nullptr, lo, hi, b.vis, rows[0], rows[1], rows[2], rows[3], st);
    if (e == cudaSuccess) e = cudaEventRecord(h->chunk_ev[c], st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->copy, h->chunk_ev[c], 0);
    for (int a = 0; a < 4 && e == cudaSuccess; ++a)
      if (out[a])
        e = cudaMemcpyAsync(out[a] + width[a] * lo, rows[a] + width[a] * lo, sizeof(double) * width[a] * (hi - lo),
                            cudaMemcpyDeviceToHost, h->copy);
  }
  if (h->copy) {
    const cudaError_t e2 = cudaStreamSynchronize(h->copy);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return cuda_status(e);
}

template <typename T>
mba_status linearize_visual_host(mba_handle* h, double* r, double* Jl, double* Js, double* Jo) {
  SolverBuffers<T>& b = buffers_of<T>(h);
  mba_status ms = ensure_solver_buffers<T>(h, b);
  if (ms != MBA_OK) return ms;
  const int64_t N = h->P.nobs;
  cudaStream_t st = h->stream;
  if (!h->obs_inv) {
    h->obs_inv = h->arena.alloc<int64_t>(N);
    if (h->arena.err != cudaSuccess) return MBA_ERR_CUDA;
    if (launch_invert_perm(h->P, h->obs_inv, st) != cudaSuccess) return MBA_ERR_CUDA;
  }
  // Page-locked host destinations are written by the gather kernel over the
  // host link directly (one pass, no HBM staging, no separate copies).
  double* out[4] = {r, Jl, Js, Jo};
  const int64_t width[4] = {2, 6, 12, 12};
  double* mapped[4] = {nullptr, nullptr, nullptr, nullptr};
  bool direct = true;
  for (int a = 0; a < 4; ++a) {
    if (!out[a]) continue;
    mapped[a] = static_cast<double*>(mapped_host_range(out[a], sizeof(double) * width[a] * N));
    direct = direct && mapped[a];
  }
  if constexpr (sizeof(T) == 8)
    if (direct && N >= 4096 * kLinChunks) return linearize_visual_chunked(h, b, out);
  cudaError_t e = launch_visual_linearize<T>(h->P, b.vis, nullptr, st);
  if (direct) {
    if (e == cudaSuccess) e = launch_gather_visual<T>(h->P, h->obs_inv, b.vis, mapped[0], mapped[1], mapped[2], mapped[3], st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_status(e);
  }
  if (!h->stage_lin) {
    h->stage_lin = h->arena.alloc<double>(32 * N);
    if (h->arena.err != cudaSuccess) return MBA_ERR_CUDA;
  }
  double* dr = h->stage_lin;
  double* dJl = dr + 2 * N;
  double* dJs = dJl + 6 * N;
  double* dJo = dJs + 12 * N;
  if (e == cudaSuccess)
    e = launch_gather_visual<T>(h->P, h->obs_inv, b.vis, r ? dr : nullptr, Jl ? dJl : nullptr, Js ? dJs : nullptr,
                                Jo ? dJo : nullptr, st);
  if (e == cudaSuccess && r) e = cudaMemcpyAsync(r, dr, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && Jl) e = cudaMemcpyAsync(Jl, dJl, sizeof(double) * 6 * N, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && Js) e = cudaMemcpyAsync(Js, dJs, sizeof(double) * 12 * N, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && Jo) e = cudaMemcpyAsync(Jo, dJo, sizeof(double) * 12 * N, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return cuda_status(e);
}

mba_status ensure_stage_state(mba_handle* h) {
  if (!h->stage_state) {
    h->stage_state = h->arena.alloc<double>(16 * h->P.nkf + 3 * h->P.nlm);
    if (h->arena.err != cudaSuccess) return MBA_ERR_CUDA;
  }
  return MBA_OK;
}

}  // namespace

extern "C" {

int32_t mba_abi_version(void) { return MBA_ABI_VERSION; }

void mba_default_solver_options(mba_solver_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->max_num_iterations = 30;
  o->jacobi_scaling = 1;
  o->initial_trust_region_radius = 1e5;
  o->max_trust_region_radius = 1e20;
  o->min_trust_region_radius = 1e-32;
  o->function_tolerance = 1e-12;
  o->gradient_tolerance = 1e-10;
  o->parameter_tolerance = 1e-8;
  o->min_relative_decrease = 1e-3;
  o->min_lm_diagonal = 1e-6;
  o->max_lm_diagonal = 1e32;
  o->linear_solver = MBA_LINEAR_SOLVER_PCG;
  o->max_linear_iterations = 100;
  o->linear_tolerance = 1e-6;
  o->precision = MBA_PRECISION_FP64;
  o->preconditioner = MBA_PRECOND_BLOCK_JACOBI;
  o->use_cuda_graph = 1;
  o->check_tolerances = 1;
  o->stop_cost = 0.0;
  o->reject_outliers_every_n_iters = 3;
  o->outlier_use_reprojection_error = 0;
  o->outlier_max_reprojection_error_px = 50.0;
}

const char* mba_status_string(mba_status s) {
  switch (s) {
    case MBA_OK: return "ok";
    case MBA_ERR_INVALID_ARG: return "invalid argument";
    case MBA_ERR_OUT_OF_RANGE_INDEX: return "index out of range";
    case MBA_ERR_NON_FINITE: return "non-finite value";
    case MBA_ERR_NOT_SPD: return "matrix not positive definite";
    case MBA_ERR_CUDA: return "CUDA error";
    case MBA_ERR_TIMEOUT: return "device wait timed out";
    case MBA_ERR_CANCELLED: return "cancelled";
    case MBA_ERR_NO_DEVICE: return "no CUDA device";
    case MBA_ERR_UNORDERED_IMU: return "IMU measurements not properly ordered";
  }
  return "unknown status";
}

mba_status mba_create(const mba_problem_desc* d, int32_t device, mba_handle** out) {
  if (!d || !out) return MBA_ERR_INVALID_ARG;
  *out = nullptr;
  const int64_t NK = d->num_keyframes, NL = d->num_landmarks, N = d->num_observations, NC = d->num_cameras,
                NM = d->num_missions, NIMU = d->num_imu_edges, NPE = d->num_pose_edges,
                NE = NIMU + NPE, NSMP = d->num_imu_samples;
  if (NK <= 0 || NL < 0 || N < 0 || NC <= 0 || NC > 255 || NM <= 0 || NIMU < 0 || NPE < 0 || NSMP < 0)
    return MBA_ERR_INVALID_ARG;
  if (NK >= (1ll << 31) || NL >= (1ll << 31) || N >= (1ll << 31)) return MBA_ERR_INVALID_ARG;
  if (!d->kf_q_IM_p_MI || !d->kf_v_M || !d->kf_b_g || !d->kf_b_a || !d->kf_mission || !d->mission_q_GM_p_GM || !d->cameras)
    return MBA_ERR_INVALID_ARG;
  if (N > 0 && (!d->obs_uv || !d->obs_sigma || !d->obs_landmark || !d->obs_keyframe || !d->obs_camera)) return MBA_ERR_INVALID_ARG;
  if (NL > 0 && (!d->lm_p_B || !d->lm_store_keyframe)) return MBA_ERR_INVALID_ARG;
  if (NIMU > 0 && (!d->edge_from || !d->edge_to || !d->edge_sample_offset || !d->imu_timestamp_ns || !d->imu_acc_gyro))
    return MBA_ERR_INVALID_ARG;
  if (NPE > 0 && (!d->pose_edge_from || !d->pose_edge_to || !d->pose_edge_T_Bk_Bkp1 || !d->pose_edge_covariance ||
                  !d->pose_edge_q_I_B_p_B_I))
    return MBA_ERR_INVALID_ARG;
  // ---- validation (host)
  for (int64_t k = 0; k < NK; ++k) {
    if (d->kf_mission[k] < 0 || d->kf_mission[k] >= NM) return MBA_ERR_OUT_OF_RANGE_INDEX;
    if (!quat_ok(d->kf_q_IM_p_MI + 7 * k)) return MBA_ERR_INVALID_ARG;
    for (int a = 0; a < 7; ++a) if (!std::isfinite(d->kf_q_IM_p_MI[7 * k + a])) return MBA_ERR_NON_FINITE;
    for (int a = 0; a < 3; ++a)
      if (!std::isfinite(d->kf_v_M[3 * k + a]) || !std::isfinite(d->kf_b_g[3 * k + a]) || !std::isfinite(d->kf_b_a[3 * k + a]))
        return MBA_ERR_NON_FINITE;
  }
  for (int64_t m = 0; m < NM; ++m) if (!quat_ok(d->mission_q_GM_p_GM + 7 * m)) return MBA_ERR_INVALID_ARG;
  for (int64_t c = 0; c < NC; ++c) {
    const mba_camera& cam = d->cameras[c];
    if (!quat_ok(cam.q_CI_p_CI)) return MBA_ERR_INVALID_ARG;
    if (cam.distortion_type < MBA_DISTORTION_NONE || cam.distortion_type > MBA_DISTORTION_FOV) return MBA_ERR_INVALID_ARG;
    if (d->camera_flags && (d->camera_flags[c] & ~0xfu)) return MBA_ERR_INVALID_ARG;
  }
  for (int64_t m = 0; m < NM && d->mission_flags; ++m) {
    const uint32_t f = d->mission_flags[m];
    if (f != 0 && f != MBA_MIS_BASEFRAME_YAW_POSITION && f != MBA_MIS_BASEFRAME_POSE) return MBA_ERR_INVALID_ARG;
  }
  for (int64_t l = 0; l < NL; ++l) {
    if (d->lm_store_keyframe[l] < 0 || d->lm_store_keyframe[l] >= NK) return MBA_ERR_OUT_OF_RANGE_INDEX;
    for (int a = 0; a < 3; ++a) if (!std::isfinite(d->lm_p_B[3 * l + a])) return MBA_ERR_NON_FINITE;
  }
  for (int64_t i = 0; i < N; ++i) {
    if (d->obs_landmark[i] < 0 || d->obs_landmark[i] >= NL || d->obs_keyframe[i] < 0 || d->obs_keyframe[i] >= NK ||
        d->obs_camera[i] < 0 || d->obs_camera[i] >= NC)
      return MBA_ERR_OUT_OF_RANGE_INDEX;
    if (!(d->obs_sigma[i] > 0.0)) return MBA_ERR_INVALID_ARG;
    if (!std::isfinite(d->obs_uv[2 * i]) || !std::isfinite(d->obs_uv[2 * i + 1])) return MBA_ERR_NON_FINITE;
  }
  if (NIMU > 0) {
    if (d->edge_sample_offset[0] < 0 || d->edge_sample_offset[NIMU] > NSMP) return MBA_ERR_OUT_OF_RANGE_INDEX;
    if (!(d->gyro_noise_sigma > 0 && d->gyro_bias_sigma > 0 && d->acc_noise_sigma > 0 && d->acc_bias_sigma > 0))
      return MBA_ERR_INVALID_ARG;
    for (int64_t e = 0; e < NIMU; ++e) {
      if (d->edge_from[e] < 0 || d->edge_from[e] >= NK || d->edge_to[e] < 0 || d->edge_to[e] >= NK ||
          d->edge_from[e] == d->edge_to[e])
        return MBA_ERR_OUT_OF_RANGE_INDEX;
      const int64_t a = d->edge_sample_offset[e], b = d->edge_sample_offset[e + 1];
      if (b <= a) return MBA_ERR_INVALID_ARG;
      for (int64_t j = a; j + 1 < b; ++j) if (d->imu_timestamp_ns[j + 1] < d->imu_timestamp_ns[j]) return MBA_ERR_UNORDERED_IMU;
      for (int64_t j = 6 * a; j < 6 * b; ++j) if (!std::isfinite(d->imu_acc_gyro[j])) return MBA_ERR_NON_FINITE;
    }
  }
  // Edges: the IMU edges, then the pose edges (square-root information of
  // each covariance computed here, as the error terms' constructors do).
  // Loop closures keep the measured rotation as JPL coefficients (the
  // Hamilton inverse, augment-loopclosure.cc:44-49), absolute terms the
  // inverse measured rotation q_S_G (block-pose-prior-error-term-v2.cc:13-16);
  // both inverses as Eigen computes them (conjugate / squared norm).  An
  // absolute term is stored as an edge from its keyframe to itself with a
  // zero to-block.
  std::vector<int32_t> e_from(NE), e_to(NE), pe_type(NPE), pe_swi(NPE, -1), sw_e;
  std::vector<double> pe_meas(7 * NPE), pe_sqrt(36 * NPE), pe_ext(7 * NPE), pe_swc(NPE, 1.0), sw0, sw_w;
  if (NIMU > 0) {
    std::copy(d->edge_from, d->edge_from + NIMU, e_from.begin());
    std::copy(d->edge_to, d->edge_to + NIMU, e_to.begin());
  }
  for (int64_t j = 0; j < NPE; ++j) {
    const int32_t type = d->pose_edge_type ? d->pose_edge_type[j] : MBA_POSE_EDGE_RELATIVE;
    if (type < MBA_POSE_EDGE_RELATIVE || type > MBA_POSE_EDGE_ABSOLUTE) return MBA_ERR_INVALID_ARG;
    const int32_t f = d->pose_edge_from[j];
    const int32_t t = type == MBA_POSE_EDGE_ABSOLUTE ? f : d->pose_edge_to[j];
    if (f < 0 || f >= NK || t < 0 || t >= NK) return MBA_ERR_OUT_OF_RANGE_INDEX;
    if (type != MBA_POSE_EDGE_ABSOLUTE && f == t) return MBA_ERR_OUT_OF_RANGE_INDEX;
    const double* T = d->pose_edge_T_Bk_Bkp1 + 7 * j;
    const double* X = d->pose_edge_q_I_B_p_B_I + 7 * j;
    const double* C = d->pose_edge_covariance + 36 * j;
    for (int a = 0; a < 7; ++a) if (!std::isfinite(T[a]) || !std::isfinite(X[a])) return MBA_ERR_NON_FINITE;
    for (int a = 0; a < 36; ++a) if (!std::isfinite(C[a])) return MBA_ERR_NON_FINITE;
    if (!quat_ok(T)) return MBA_ERR_INVALID_ARG;
    if (type != MBA_POSE_EDGE_LOOP_CLOSURE && !quat_ok(X)) return MBA_ERR_INVALID_ARG;
    if (!pose_edge_sqrt_information(C, &pe_sqrt[36 * j])) return MBA_ERR_NOT_SPD;
    std::copy(T, T + 7, &pe_meas[7 * j]);
    if (type != MBA_POSE_EDGE_RELATIVE) {
      const double n2 = T[0] * T[0] + T[1] * T[1] + T[2] * T[2] + T[3] * T[3];
      for (int a = 0; a < 3; ++a) pe_meas[7 * j + a] = -T[a] / n2;
      pe_meas[7 * j + 3] = T[3] / n2;
    }
    std::copy(X, X + 7, &pe_ext[7 * j]);
    pe_type[j] = type;
    if (type == MBA_POSE_EDGE_LOOP_CLOSURE) {
      const double s0 = d->pose_edge_switch ? d->pose_edge_switch[j] : 1.0;
      const double var = d->pose_edge_switch_variance ? d->pose_edge_switch_variance[j] : 0.0;
      if (!std::isfinite(s0) || !std::isfinite(var)) return MBA_ERR_NON_FINITE;
      if (s0 < 0.0 || s0 > 1.0 || var < 0.0) return MBA_ERR_INVALID_ARG;  // SwitchPriorErrorTerm CHECKs
      pe_swc[j] = s0;
      if (var > 0.0) {
        pe_swi[j] = (int32_t)sw0.size();
        sw0.push_back(s0);
        sw_w.push_back(std::sqrt(1.0 / var));
        sw_e.push_back((int32_t)(NIMU + j));
      }
    }
    e_from[NIMU + j] = f;
    e_to[NIMU + j] = t;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) { cudaGetLastError(); return MBA_ERR_NO_DEVICE; }
  if (device < 0 || device >= ndev) return MBA_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MBA_ERR_CUDA;

  mba_handle* h = new (std::nothrow) mba_handle();
  if (!h) return MBA_ERR_CUDA;
  h->device = device;
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) { delete h; return MBA_ERR_CUDA; }
  {
    void* hp = nullptr;
    void* dp = nullptr;
    if (cudaHostAlloc(&hp, sizeof(int), cudaHostAllocMapped) == cudaSuccess &&
        cudaHostGetDevicePointer(&dp, hp, 0) == cudaSuccess) {
      h->cancel_host = static_cast<volatile int*>(hp);
      *h->cancel_host = 0;
      h->cancel_dev = static_cast<const volatile int*>(dp);
    } else if (hp) {
      cudaFreeHost(hp);
    }
    cudaGetLastError();
  }
  cudaStream_t st = h->stream;

  // ---- internal landmark numbering.  Internal landmark i is the caller's
  // landmark (i * A) mod N_lm, A coprime to N_lm and near 0.618 N_lm: a
  // scattering permutation, so that neighbouring landmarks (neighbouring
  // lanes of the landmark kernels) come from unrelated parts of the map
  // whatever the caller's order (a map's vertices hold their landmarks, so a
  // caller may well list them by store keyframe).  Lanes on landmarks of one
  // store keyframe add into the same blocks at the same time (their atomics
  // serialize); with neighbours on consecutive store keyframes the assembly
  // read five times more from DRAM.  Observations are sorted by internal
  // landmark below, contiguous per lane.  The slots' U
  // rows are numbered by store keyframe (slot_order: internal landmarks by
  // store keyframe, longer tracks first), so that the partner rows a Schur
  // target gathers lie close together.  The state, rejection and quality
  // entry points translate to the caller's numbering (h->lm_caller:
  // internal -> caller index).
  mba_problem_desc dint;
  std::vector<int32_t> lm_rank, int_store, int_obs_lm, slot_order(NL);
  std::vector<double> int_lm_p;
  std::vector<uint8_t> int_lm_const;
  {
    std::vector<int64_t> cnt(NL, 0), end(NK + 1, 0);
    for (int64_t i = 0; i < N; ++i) cnt[d->obs_landmark[i]]++;
    for (int64_t l = 0; l < NL; ++l) end[d->lm_store_keyframe[l] + 1]++;
    for (int64_t k = 0; k < NK; ++k) end[k + 1] += end[k];
    std::vector<int32_t> by_kf(NL);
    std::vector<int64_t> fill(end.begin(), end.end() - 1);
    for (int64_t l = 0; l < NL; ++l) by_kf[fill[d->lm_store_keyframe[l]]++] = (int32_t)l;
    for (int64_t k = 0; k < NK; ++k)
      std::stable_sort(by_kf.begin() + end[k], by_kf.begin() + end[k + 1],
                       [&](int32_t x, int32_t y) { return cnt[x] > cnt[y]; });
    int64_t A = std::max<int64_t>(1, (int64_t)(0.6180339887498949 * (double)NL));
    while (std::gcd(A, std::max<int64_t>(NL, 1)) != 1) ++A;
    h->lm_caller.resize(NL);
    for (int64_t l = 0; l < NL; ++l) h->lm_caller[l] = (int32_t)((l * A) % NL);
    lm_rank.resize(NL);
    for (int64_t l = 0; l < NL; ++l) lm_rank[h->lm_caller[l]] = (int32_t)l;
    for (int64_t q = 0; q < NL; ++q) slot_order[q] = lm_rank[by_kf[q]];
    bool identity = true;
    for (int64_t l = 0; l < NL && identity; ++l) identity = h->lm_caller[l] == l;
    if (identity) {
      h->lm_caller.clear();
    } else {
      int_store.resize(NL);
      int_lm_p.resize(3 * NL);
      for (int64_t l = 0; l < NL; ++l) {
        const int32_t c = h->lm_caller[l];
        int_store[l] = d->lm_store_keyframe[c];
        for (int a = 0; a < 3; ++a) int_lm_p[3 * l + a] = d->lm_p_B[3 * c + a];
      }
      if (d->lm_constant) {
        int_lm_const.resize(NL);
        for (int64_t l = 0; l < NL; ++l) int_lm_const[l] = d->lm_constant[h->lm_caller[l]];
      }
      int_obs_lm.resize(N);
      for (int64_t i = 0; i < N; ++i) int_obs_lm[i] = lm_rank[d->obs_landmark[i]];
      dint = *d;
      dint.lm_store_keyframe = int_store.data();
      dint.lm_p_B = int_lm_p.data();
      dint.lm_constant = d->lm_constant ? int_lm_const.data() : nullptr;
      dint.obs_landmark = int_obs_lm.data();
      d = &dint;
    }
  }

  // ---- observation types and landmark-sorted order
  std::vector<uint8_t> type(N);
  for (int64_t i = 0; i < N; ++i) {
    const int l = d->obs_landmark[i], k = d->obs_keyframe[i], s = d->lm_store_keyframe[l];
    type[i] = (k == s) ? MBA_LOCAL_KEYFRAME : (d->kf_mission[k] == d->kf_mission[s] ? MBA_LOCAL_MISSION : MBA_GLOBAL);
  }
  std::vector<int64_t> off(NL + 1, 0);
  for (int64_t i = 0; i < N; ++i) off[d->obs_landmark[i] + 1]++;
  for (int64_t l = 0; l < NL; ++l) off[l + 1] += off[l];
  h->perm.resize(N);
  {
    std::vector<int64_t> fill(off.begin(), off.end() - 1);
    for (int64_t i = 0; i < N; ++i) h->perm[fill[d->obs_landmark[i]]++] = i;
  }
  std::vector<double> uv(2 * N), sinv(N), hub(N);
  std::vector<int32_t> olm(N), okf(N), ost(N);
  std::vector<uint8_t> ocam(N), otype(N);
  for (int64_t s = 0; s < N; ++s) {
    const int64_t i = h->perm[s];
    uv[2 * s] = d->obs_uv[2 * i];
    uv[2 * s + 1] = d->obs_uv[2 * i + 1];
    sinv[s] = 1.0 / d->obs_sigma[i];
    const double delta = type[i] == MBA_GLOBAL ? d->huber_delta_global : d->huber_delta_local;
    hub[s] = d->use_huber ? delta * d->obs_sigma[i] : 0.0;
    olm[s] = d->obs_landmark[i];
    okf[s] = d->obs_keyframe[i];
    ost[s] = d->lm_store_keyframe[olm[s]];
    ocam[s] = (uint8_t)d->obs_camera[i];
    otype[s] = type[i];
  }
  // ---- keyframe tangent masks (active dims), landmark activity
  std::vector<uint8_t> in_inertial(NK, 0), in_visual(NK, 0);
  for (int64_t e = 0; e < NIMU; ++e) { in_inertial[e_from[e]] = 1; in_inertial[e_to[e]] = 1; }
  // a pose edge makes the pose blocks of its keyframes active, not v / b_g / b_a
  for (int64_t e = NIMU; e < NE; ++e) { in_visual[e_from[e]] = 1; in_visual[e_to[e]] = 1; }
  for (int64_t s = 0; s < N; ++s)
    if (otype[s] != MBA_LOCAL_KEYFRAME) { in_visual[okf[s]] = 1; in_visual[ost[s]] = 1; }
  std::vector<uint16_t> mask(NK);
  std::vector<uint32_t> flags(NK, 0u);
  for (int64_t k = 0; k < NK; ++k) {
    uint32_t m = 0x7fff;
    const uint32_t f = d->kf_flags ? d->kf_flags[k] : 0u;
    flags[k] = f;
    if (!in_inertial[k] && !in_visual[k]) m &= ~0x3fu;
    if (!in_inertial[k]) m &= 0x3fu;
    if (f & (MBA_KF_POSE_CONSTANT | MBA_KF_ROTATION_CONSTANT)) m &= ~0x3fu;
    if (f & MBA_KF_POSITION_CONSTANT) m &= ~0x38u;
    if (f & MBA_KF_GAUGE_ROLL_PITCH) m &= ~0x3cu;
    if (f & MBA_KF_VELOCITY_CONSTANT) m &= ~(7u << 6);
    if (f & MBA_KF_GYRO_BIAS_CONSTANT) m &= ~(7u << 9);
    if (f & MBA_KF_ACCEL_BIAS_CONSTANT) m &= ~(7u << 12);
    mask[k] = (uint16_t)m;
  }
  std::vector<uint8_t> lm_active(NL, 1);
  for (int64_t l = 0; l < NL; ++l)
    if ((d->lm_constant && d->lm_constant[l]) || off[l + 1] == off[l]) lm_active[l] = 0;

  // ---- Schur pattern
  std::vector<int64_t> slot_off(NL, 0), slot_end(NL, 0);
  std::vector<int32_t> slot_kf, slot_lm, obs_slot(N, -1), obs_pblk(N, -1);
  slot_kf.reserve(NL + N);
  slot_lm.reserve(NL + N);
  int64_t npair_est = 0;
  for (int64_t l = 0; l < NL; ++l) {
    slot_off[l] = (int64_t)slot_kf.size();
    slot_kf.push_back(d->lm_store_keyframe[l]);
    slot_lm.push_back((int32_t)l);
    for (int64_t s = off[l]; s < off[l + 1]; ++s) {
      if (otype[s] == MBA_LOCAL_KEYFRAME) continue;
      obs_slot[s] = (int32_t)slot_kf.size();
      slot_kf.push_back(okf[s]);
      slot_lm.push_back((int32_t)l);
    }
    slot_end[l] = (int64_t)slot_kf.size();
    const int64_t m = slot_end[l] - slot_off[l];
    if (lm_active[l]) npair_est += m * (m + 1) / 2;
  }
  // U rows: the slots again, numbered by store keyframe (slot_order).
  std::vector<int32_t> w_u(slot_kf.size()), u_w(slot_kf.size());
  {
    int32_t u = 0;
    for (int64_t q = 0; q < NL; ++q) {
      const int64_t l = slot_order[q];
      for (int64_t x = slot_off[l]; x < slot_end[l]; ++x) {
        w_u[x] = u;
        u_w[u++] = (int32_t)x;
      }
    }
  }
  PairMap pm(std::max<int64_t>(1024, N + NE));
  for (int64_t s = 0; s < N; ++s)
    if (otype[s] != MBA_LOCAL_KEYFRAME) obs_pblk[s] = pm.get(ost[s], okf[s]);
  // Slot pairs, sorted by the S block they update.  Targets are diagonal
  // blocks (kf, kf) -> id kf, and upper blocks (i < j) -> id NK + block; an
  // upper pair is oriented so slot_kf[a] < slot_kf[b] (W_a^T V W_b is
  // transposed by swapping a and b, V being symmetric).  Targets are ordered
  // by (i, j) so consecutive targets touch landmarks of nearby keyframes, and
  // each target's pairs are cut into chunks of at most kSchurChunk pairs,
  // one chunk per thread.
  // A pair stores a as its position in its row's keyframe-major slot list (the
  // row's W slots are staged in shared memory) and b as a global slot.
  std::vector<int2> prb;
  std::vector<int32_t> chunk_tgt, kf_slot, tgt_row;
  std::vector<int64_t> chunk_beg, row_chunk_off, kf_slot_off(NK + 1, 0);
  std::vector<int32_t> chunk_len;
  int64_t max_row_slots = 0;
  {
    std::vector<int32_t> ta, tb;
    std::vector<int64_t> tt;
    ta.reserve(npair_est); tb.reserve(npair_est); tt.reserve(npair_est);
    for (int64_t l = 0; l < NL; ++l) {
      if (!lm_active[l]) continue;
      for (int64_t x = slot_off[l]; x < slot_end[l]; ++x)
        for (int64_t y = x; y < slot_end[l]; ++y) {
          const int32_t kx = slot_kf[x], ky = slot_kf[y];
          if (kx == ky) {
            ta.push_back((int32_t)x); tb.push_back((int32_t)y); tt.push_back(kx);
          } else {
            const int32_t blk = pm.get(kx, ky);
            if (kx < ky) { ta.push_back((int32_t)x); tb.push_back((int32_t)y); }
            else { ta.push_back((int32_t)y); tb.push_back((int32_t)x); }
            tt.push_back(NK + blk);
          }
        }
    }
    // Target order by (i, j); rank[target id] = position.
    const int64_t ntgt = NK + pm.count;
    std::vector<int64_t> order(ntgt);
    std::iota(order.begin(), order.end(), 0);
    auto key = [&](int64_t t) -> int64_t {
      if (t < NK) return t * NK + t;
      return (int64_t)pm.bi[t - NK] * NK + pm.bj[t - NK];
    };
    std::sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return key(x) < key(y); });
    std::vector<int64_t> rank(ntgt), cnt(ntgt + 1, 0);
    for (int64_t r = 0; r < ntgt; ++r) rank[order[r]] = r;
    for (int64_t t : tt) cnt[rank[t] + 1]++;
    for (int64_t r = 0; r < ntgt; ++r) cnt[r + 1] += cnt[r];
    const int64_t np = (int64_t)tt.size();
    const int64_t nsl = (int64_t)slot_kf.size();
    for (int64_t x = 0; x < nsl; ++x) kf_slot_off[slot_kf[x] + 1]++;
    for (int64_t k = 0; k < NK; ++k) {
      max_row_slots = std::max(max_row_slots, kf_slot_off[k + 1]);
      kf_slot_off[k + 1] += kf_slot_off[k];
    }
    kf_slot.resize(nsl);
    std::vector<int32_t> kpos(nsl);
    {
      std::vector<int64_t> fill(kf_slot_off.begin(), kf_slot_off.end() - 1);
      for (int64_t x = 0; x < nsl; ++x) {
        const int64_t at = fill[slot_kf[x]]++;
        kf_slot[at] = (int32_t)x;
        kpos[x] = (int32_t)(at - kf_slot_off[slot_kf[x]]);
      }
    }
    prb.resize(np);
    {
      std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
      for (int64_t q = 0; q < np; ++q) {
        const int64_t dst = fill[rank[tt[q]]]++;
        prb[dst] = make_int2(kpos[ta[q]], ta[q] == tb[q] ? ~w_u[tb[q]] : w_u[tb[q]]);
      }
    }
    tgt_row.resize(ntgt);
    for (int64_t r = 0; r < ntgt; ++r) {
      const int64_t t = order[r];
      tgt_row[r] = (int32_t)(t < NK ? t : pm.bi[t - NK]);
    }
    cut_chunks(cnt, order, tgt_row, NK, kSchurChunk, &chunk_tgt, &chunk_beg, &chunk_len, &row_chunk_off);
    h->tgt_off = std::move(cnt);
    h->tgt_order = std::move(order);
    h->tgt_row = std::move(tgt_row);
  }
  const int64_t npu = pm.count;
  std::vector<int64_t> row_off(NK + 1, 0);
  for (int64_t b = 0; b < npu; ++b) { row_off[pm.bi[b] + 1]++; row_off[pm.bj[b] + 1]++; }
  for (int64_t k = 0; k < NK; ++k) row_off[k + 1] += row_off[k];
  std::vector<int32_t> row_col(2 * npu), row_blk(2 * npu);
  {
    std::vector<int64_t> fill(row_off.begin(), row_off.end() - 1);
    for (int64_t b = 0; b < npu; ++b) {
      const int32_t i = pm.bi[b], j = pm.bj[b];
      row_col[fill[i]] = j; row_blk[fill[i]++] = (int32_t)b;
      row_col[fill[j]] = i; row_blk[fill[j]++] = (int32_t)(npu + b);
    }
  }
  // Upper blocks by their row i (i < j), for the product that reads each block once.
  std::vector<int64_t> up_off(NK + 1, 0);
  for (int64_t b = 0; b < npu; ++b) up_off[pm.bi[b] + 1]++;
  for (int64_t k = 0; k < NK; ++k) up_off[k + 1] += up_off[k];
  std::vector<int32_t> up_col(npu), up_blk(npu);
  {
    std::vector<int64_t> fill(up_off.begin(), up_off.end() - 1);
    for (int64_t b = 0; b < npu; ++b) {
      up_col[fill[pm.bi[b]]] = pm.bj[b];
      up_blk[fill[pm.bi[b]]++] = (int32_t)b;
    }
  }
  std::vector<int64_t> kfe_off(NK + 1, 0);
  // Per-keyframe edge lists (couplings; an absolute term couples nothing).
  for (int64_t e = 0; e < NE; ++e)
    if (e_from[e] != e_to[e]) { kfe_off[e_from[e] + 1]++; kfe_off[e_to[e] + 1]++; }
  for (int64_t k = 0; k < NK; ++k) kfe_off[k + 1] += kfe_off[k];
  std::vector<int32_t> kfe(kfe_off[NK]);
  {
    std::vector<int64_t> fill(kfe_off.begin(), kfe_off.end() - 1);
    for (int64_t e = 0; e < NE; ++e) {
      if (e_from[e] == e_to[e]) continue;
      kfe[fill[e_from[e]]++] = (int32_t)(e + 1);
      kfe[fill[e_to[e]]++] = (int32_t)(-(e + 1));
    }
  }

  // ---- neighbour lists of the co-visibility + inertial graph (learned
  // preconditioner): per keyframe its pose-pose blocks, then its inertial edges.
  std::vector<int64_t> nbr_off(NK + 1, 0);
  std::vector<int32_t> nbr, nbr_blk;
  nbr.reserve(row_col.size() + 2 * NE);
  nbr_blk.reserve(row_col.size() + 2 * NE);
  for (int64_t k = 0; k < NK; ++k) {
    for (int64_t e = row_off[k]; e < row_off[k + 1]; ++e) { nbr.push_back(row_col[e]); nbr_blk.push_back(row_blk[e]); }
    for (int64_t e = kfe_off[k]; e < kfe_off[k + 1]; ++e) {
      const int32_t code = kfe[e];
      const int64_t ed = code > 0 ? code - 1 : -code - 1;
      nbr.push_back(code > 0 ? e_to[ed] : e_from[ed]);
      nbr_blk.push_back((int32_t)(-(ed + 1)));
    }
    nbr_off[k + 1] = (int64_t)nbr.size();
  }

  // ---- keyframe chains (chain preconditioner).  With edges that couple two
  // keyframes (IMU, odometry, loop closures) a chain follows from -> to, the
  // first such edge of a keyframe; without, the keyframes of a mission in
  // index order.
  // All chains are laid end to end in one sequence of positions; position p
  // couples to p - 1 only inside a chain (link_edge / link_blk give the
  // blocks of that coupling, -1 where absent).
  std::vector<int32_t> chain_perm, link_edge(NK, -1), link_blk(NK, -1);
  chain_perm.reserve(NK);
  {
    std::vector<int32_t> next(NK, -1), next_e(NK, -1);
    std::vector<char> has_prev(NK, 0), seen(NK, 0), start(NK, 0);
    for (int64_t e = 0; e < NE; ++e) {
      const int32_t f = e_from[e], t = e_to[e];
      if (f == t) continue;
      if (next[f] < 0 && !has_prev[t]) { next[f] = t; next_e[f] = (int32_t)e; has_prev[t] = 1; }
    }
    auto follow = [&](int32_t k) {
      start[k] = 1;
      while (k >= 0 && !seen[k]) {
        seen[k] = 1;
        chain_perm.push_back(k);
        k = next[k];
      }
    };
    if (kfe_off[NK] > 0) {
      for (int32_t k = 0; k < NK; ++k) if (!has_prev[k] && !seen[k]) follow(k);
      for (int32_t k = 0; k < NK; ++k) if (!seen[k]) follow(k);
    } else {
      std::vector<int32_t> ord(NK);
      std::iota(ord.begin(), ord.end(), 0);
      std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t b) { return d->kf_mission[a] < d->kf_mission[b]; });
      for (int64_t q = 0; q < NK; ++q) {
        const int32_t k = ord[q];
        start[k] = (q == 0 || d->kf_mission[ord[q - 1]] != d->kf_mission[k]);
        chain_perm.push_back(k);
      }
    }
    for (int64_t q = 1; q < NK; ++q) {
      const int32_t a = chain_perm[q - 1], b = chain_perm[q];
      if (start[b]) continue;
      if (next[a] == b) link_edge[q] = next_e[a];  // SE[e] is the (a, b) block
      const int32_t blk = pm.find(a, b);
      if (blk >= 0) link_blk[q] = (b < a) ? blk : (int32_t)(npu + blk);  // SP block with rows b, columns a
    }
  }

  // ---- state and constants
  std::vector<double> kf_state(16 * NK), lm_p(4 * NL, 0.0), mis(8 * NM, 0.0);
  for (int64_t k = 0; k < NK; ++k) {
    for (int a = 0; a < 7; ++a) kf_state[16 * k + a] = d->kf_q_IM_p_MI[7 * k + a];
    for (int a = 0; a < 3; ++a) {
      kf_state[16 * k + 7 + a] = d->kf_v_M[3 * k + a];
      kf_state[16 * k + 10 + a] = d->kf_b_g[3 * k + a];
      kf_state[16 * k + 13 + a] = d->kf_b_a[3 * k + a];
    }
  }
  for (int64_t l = 0; l < NL; ++l) for (int a = 0; a < 3; ++a) lm_p[4 * l + a] = d->lm_p_B[3 * l + a];
  for (int64_t m = 0; m < NM; ++m) for (int a = 0; a < 7; ++a) mis[8 * m + a] = d->mission_q_GM_p_GM[7 * m + a];
  std::vector<DevCamera> cams(NC);
  for (int64_t c = 0; c < NC; ++c) {
    const mba_camera& s = d->cameras[c];
    DevCamera& o = cams[c];
    std::memset(&o, 0, sizeof(o));
    for (int a = 0; a < 4; ++a) { o.intr[a] = s.intrinsics[a]; o.dist[a] = s.distortion[a]; o.q_CI[a] = s.q_CI_p_CI[a]; }
    for (int a = 0; a < 3; ++a) o.p_CI[a] = s.q_CI_p_CI[4 + a];
    o.dtype = s.distortion_type;
    o.width = s.width;
    o.height = s.height;
  }
  std::vector<int32_t> kfm(NK);
  std::vector<int64_t> e_off(NIMU + 1, 0), ts;
  std::vector<double> imu;
  if (NIMU > 0) {
    e_off.assign(d->edge_sample_offset, d->edge_sample_offset + NIMU + 1);
    ts.assign(d->imu_timestamp_ns, d->imu_timestamp_ns + NSMP);
    imu.assign(d->imu_acc_gyro, d->imu_acc_gyro + 6 * NSMP);
  }
  kfm.assign(d->kf_mission, d->kf_mission + NK);
  // ---- global nodes: cameras with a free calibration block, missions with a
  // free baseframe (15-dim blocks after the keyframes; active dims as bits).
  std::vector<int32_t> cam_node(NC, -1), mis_node(NM, -1), node_cam, node_mis;
  std::vector<uint16_t> g_mask;
  std::vector<uint32_t> mflags(NM, 0u);
  for (int64_t c = 0; c < NC; ++c) {
    const uint32_t f = d->camera_flags ? d->camera_flags[c] : 0u;
    if (!f) continue;
    const int dt = d->cameras[c].distortion_type;
    const int nd = (dt == MBA_DISTORTION_RADTAN || dt == MBA_DISTORTION_EQUIDISTANT) ? 4 : (dt == MBA_DISTORTION_FOV ? 1 : 0);
    uint32_t m = 0;
    if (f & MBA_CAM_INTRINSICS_FREE) m |= 0xfu;
    if (f & MBA_CAM_DISTORTION_FREE) m |= ((1u << nd) - 1u) << 4;
    if (f & MBA_CAM_ROTATION_FREE) m |= 7u << 8;
    if (f & MBA_CAM_TRANSLATION_FREE) m |= 7u << 11;
    cam_node[c] = (int32_t)node_cam.size();
    node_cam.push_back((int32_t)c);
    node_mis.push_back(-1);
    g_mask.push_back((uint16_t)m);
  }
  for (int64_t m = 0; m < NM; ++m) {
    const uint32_t f = d->mission_flags ? d->mission_flags[m] : 0u;
    mflags[m] = f;
    if (!f) continue;
    mis_node[m] = (int32_t)node_cam.size();
    node_cam.push_back(-1);
    node_mis.push_back((int32_t)m);
    g_mask.push_back((uint16_t)(f == MBA_MIS_BASEFRAME_POSE ? 0x3fu : 0x39u));
  }
  // A free baseframe enters the visual terms only: absolute 6-DoF terms and
  // cross-mission loop closures need their baseframes constant.
  for (int64_t j = 0; j < NPE; ++j) {
    const int mf = d->kf_mission[e_from[NIMU + j]], mt = d->kf_mission[e_to[NIMU + j]];
    const bool uses_bf = pe_type[j] == MBA_POSE_EDGE_ABSOLUTE || (pe_type[j] == MBA_POSE_EDGE_LOOP_CLOSURE && mf != mt);
    if (uses_bf && (mis_node[mf] >= 0 || mis_node[mt] >= 0)) {
      mba_destroy(h);
      return MBA_ERR_INVALID_ARG;
    }
  }

  // ---- upload
  DeviceArena& A = h->arena;
  DevProblem& P = h->P;
  P.nkf = NK; P.nlm = NL; P.nobs = N; P.ncam = NC; P.nmis = NM; P.nedge = NE; P.nimu = NIMU; P.nsamp = NSMP;
  P.obs_uv = reinterpret_cast<const double2*>(A.upload(uv, st));
  P.obs_sinv = A.upload(sinv, st);
  P.obs_huber = A.upload(hub, st);
  P.obs_lm = A.upload(olm, st);
  P.obs_kf = A.upload(okf, st);
  P.obs_store = A.upload(ost, st);
  P.obs_cam = A.upload(ocam, st);
  P.obs_type = A.upload(otype, st);
  P.obs_perm = A.upload(h->perm, st);
  P.lm_p = A.upload(lm_p, st);
  P.lm_obs_off = A.upload(off, st);
  P.lm_active = A.upload(lm_active, st);
  P.lm_off = A.alloc<int32_t>(NL);
  if (NL && P.lm_off) cudaMemsetAsync(P.lm_off, 0, sizeof(int32_t) * NL, st);
  if (!h->lm_caller.empty()) h->lm_caller_dev = A.upload(h->lm_caller, st);
  P.kf_state = A.upload(kf_state, st);
  P.kf_rot = A.alloc<double>(16 * NK + 16);
  P.kf_mis = A.upload(kfm, st);
  P.kf_flags = A.upload(flags, st);
  P.kf_mask = A.upload(mask, st);
  P.mis = A.upload(mis, st);
  P.cams = A.upload(cams, st);
  P.ng = (int64_t)node_cam.size();
  if (P.ng > 0) {
    P.cam_node = A.upload(cam_node, st);
    P.mis_node = A.upload(mis_node, st);
    P.node_cam = A.upload(node_cam, st);
    P.node_mis = A.upload(node_mis, st);
    P.g_mask = A.upload(g_mask, st);
    P.mis_flags = A.upload(mflags, st);
  }
  P.e_from = A.upload(e_from, st);
  P.e_to = A.upload(e_to, st);
  P.e_off = A.upload(e_off, st);
  P.imu_ts = A.upload(ts, st);
  P.imu = A.upload(imu, st);
  P.pe_meas = A.upload(pe_meas, st);
  P.pe_sqrt = A.upload(pe_sqrt, st);
  P.pe_ext = A.upload(pe_ext, st);
  P.pe_type = A.upload(pe_type, st);
  P.pe_swi = A.upload(pe_swi, st);
  P.pe_swc = A.upload(pe_swc, st);
  P.nsw = (int64_t)sw0.size();
  P.sw = A.upload(sw0, st);
  P.sw_w = A.upload(sw_w, st);
  P.sw_e = A.upload(sw_e, st);
  {
    // FP32 mirrors for the FP32 evaluation kernel.
    std::vector<float> uvf(2 * N), sinvf(N), hubf(N), lmf(4 * NL, 0.f), kff(8 * NK, 0.f), misf(8 * NM, 0.f);
    for (int64_t a = 0; a < 2 * N; ++a) uvf[a] = (float)uv[a];
    for (int64_t a = 0; a < N; ++a) { sinvf[a] = (float)sinv[a]; hubf[a] = (float)hub[a]; }
    for (int64_t a = 0; a < 4 * NL; ++a) lmf[a] = (float)lm_p[a];
    for (int64_t k = 0; k < NK; ++k) for (int a = 0; a < 7; ++a) kff[8 * k + a] = (float)kf_state[16 * k + a];
    for (int64_t a = 0; a < 8 * NM; ++a) misf[a] = (float)mis[a];
    std::vector<DevCameraT<float>> camf(NC);
    for (int64_t c = 0; c < NC; ++c) {
      DevCameraT<float>& o = camf[c];
      std::memset(&o, 0, sizeof(o));
      for (int a = 0; a < 4; ++a) {
        o.intr[a] = (float)cams[c].intr[a];
        o.dist[a] = (float)cams[c].dist[a];
        o.q_CI[a] = (float)cams[c].q_CI[a];
      }
      for (int a = 0; a < 3; ++a) o.p_CI[a] = (float)cams[c].p_CI[a];
      o.dtype = cams[c].dtype;
      o.width = cams[c].width;
      o.height = cams[c].height;
    }
    P.obs_uv_f = reinterpret_cast<const float2*>(A.upload(uvf, st));
    P.obs_sinv_f = A.upload(sinvf, st);
    P.obs_huber_f = A.upload(hubf, st);
    P.lm_p_f = A.upload(lmf, st);
    P.kf_pose_f = A.upload(kff, st);
    P.mis_f = A.upload(misf, st);
    P.cams_f = A.upload(camf, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) A.err = cudaErrorUnknown;  // host vectors die here
  }
  P.gyro_noise2 = d->gyro_noise_sigma * d->gyro_noise_sigma;
  P.gyro_bias2 = d->gyro_bias_sigma * d->gyro_bias_sigma;
  P.acc_noise2 = d->acc_noise_sigma * d->acc_noise_sigma;
  P.acc_bias2 = d->acc_bias_sigma * d->acc_bias_sigma;
  P.gravity = d->gravity_magnitude;
  SchurPattern& S = h->S;
  S.nslot = (int64_t)slot_kf.size();
  S.npu = npu;
  S.npair = (int64_t)prb.size();
  S.lm_slot_off = A.upload(slot_off, st);
  S.lm_slot_end = A.upload(slot_end, st);
  S.w_u = A.upload(w_u, st);
  S.u_w = A.upload(u_w, st);
  S.slot_kf = A.upload(slot_kf, st);
  S.slot_lm = A.upload(slot_lm, st);
  S.obs_slot = A.upload(obs_slot, st);
  S.obs_pblk = A.upload(obs_pblk, st);
  S.pair_rb = A.upload(prb, st);
  S.kf_slot_off = A.upload(kf_slot_off, st);
  S.kf_slot = A.upload(kf_slot, st);
  S.max_row_slots = max_row_slots;
  S.row_chunk_off = A.upload(row_chunk_off, st);
  S.nchunk = (int64_t)chunk_tgt.size();
  S.chunk_tgt = A.upload(chunk_tgt, st);
  S.chunk_beg = A.upload(chunk_beg, st);
  S.chunk_len = A.upload(chunk_len, st);
  S.pu_i = A.upload(pm.bi, st);
  S.pu_j = A.upload(pm.bj, st);
  S.row_off = A.upload(row_off, st);
  S.row_col = A.upload(row_col, st);
  S.row_blk = A.upload(row_blk, st);
  S.up_off = A.upload(up_off, st);
  S.up_col = A.upload(up_col, st);
  S.up_blk = A.upload(up_blk, st);
  S.kfe_off = A.upload(kfe_off, st);
  S.kfe = A.upload(kfe, st);
  h->gg.nbr_off = A.upload(nbr_off, st);
  h->gg.nbr = A.upload(nbr, st);
  h->gg.nbr_blk = A.upload(nbr_blk, st);
  S.chain_perm = A.upload(chain_perm, st);
  S.link_edge = A.upload(link_edge, st);
  S.link_blk = A.upload(link_blk, st);
  S.chain_levels = 0;
  while (((int64_t)1 << S.chain_levels) < NK) ++S.chain_levels;
  S.chain_tail = 0;
  while (S.chain_tail < S.chain_levels && ((NK + ((int64_t)1 << S.chain_tail) - 1) >> S.chain_tail) > 128)
    ++S.chain_tail;
  h->tuning.visual_block = 256;
  h->tuning.visual_min_blocks = 1;
  h->tuning.visual_pipelined = 2;
  h->tuning.schur_chunk = (int32_t)kSchurChunk;
  h->tuning.chain_tail_nodes = 128;
  h->tuning.chain_segment = 1;
  h->tuning.chain_tail_smem = 2;
  h->tuning.pcg_product = 2;
  h->tuning.schur_split = 2;
  // Inertial scratch (kernels_inertial.cu): dt per step, end state per edge,
  // 4 RK4 stages x 15 values per step, FP32 Q_acc | Phi_acc per edge.
  P.ine_scratch = A.alloc<double>((NSMP - NIMU) + 16 * NIMU + 60 * (NSMP - NIMU) + 225 * NIMU + 1);
  h->scratch = A.alloc<double>(4);
  h->iscratch = A.alloc<int>(4);
  if (A.err != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
    mba_destroy(h);
    return MBA_ERR_CUDA;
  }
  *out = h;
  return MBA_OK;
}

void mba_destroy(mba_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->copy) cudaStreamSynchronize(h->copy);
  h->arena.release();
  if (h->cancel_host) cudaFreeHost((void*)h->cancel_host);
  for (cudaEvent_t& ev : h->chunk_ev)
    if (ev) cudaEventDestroy(ev);
  if (h->copy) cudaStreamDestroy(h->copy);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

mba_status mba_evaluate_visual(mba_handle* h, double* residuals, double* const* jacobians) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t N = h->P.nobs;
  if (N == 0) return MBA_OK;
  static const int sz[9] = {6, 14, 14, 14, 14, 8, 6, 8, 8};
  DeviceArena tmp;
  double* dres = residuals ? tmp.alloc<double>(2 * N) : nullptr;
  double* dj[9] = {nullptr};
  for (int b = 0; b < 9; ++b)
    if (jacobians && jacobians[b]) dj[b] = tmp.alloc<double>(sz[b] * N);
  cudaError_t e = tmp.err;
  if (e == cudaSuccess) e = launch_visual_ambient(h->P, dres, dj, h->stream);
  if (e == cudaSuccess && dres) e = cudaMemcpyAsync(residuals, dres, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, h->stream);
  for (int b = 0; b < 9 && e == cudaSuccess; ++b)
    if (dj[b]) e = cudaMemcpyAsync(jacobians[b], dj[b], sizeof(double) * sz[b] * N, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  tmp.release();
  return cuda_status(e);
}

mba_status mba_evaluate_inertial(mba_handle* h, double* residuals, double* const* jacobians) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t NE = h->P.nimu;
  if (NE == 0) return MBA_OK;
  static const int sz[8] = {105, 45, 45, 45, 105, 45, 45, 45};
  DeviceArena tmp;
  double* dres = tmp.alloc<double>(15 * NE);
  double* dj[8] = {nullptr};
  for (int b = 0; b < 8; ++b)
    if (jacobians && jacobians[b]) dj[b] = tmp.alloc<double>(sz[b] * NE);
  int* dstatus = tmp.alloc<int>(1);
  cudaError_t e = tmp.err;
  if (e == cudaSuccess) e = cudaMemsetAsync(dstatus, 0, sizeof(int), h->stream);
  InertialLin<double> none{};
  if (e == cudaSuccess) e = launch_inertial(h->P, h->P.kf_state, none, dres, dj, nullptr, dstatus, h->stream);
  int status = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, dstatus, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && residuals) e = cudaMemcpyAsync(residuals, dres, sizeof(double) * 15 * NE, cudaMemcpyDeviceToHost, h->stream);
  for (int b = 0; b < 8 && e == cudaSuccess; ++b)
    if (dj[b]) e = cudaMemcpyAsync(jacobians[b], dj[b], sizeof(double) * sz[b] * NE, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  tmp.release();
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  return (mba_status)status;
}

mba_status mba_linearize_pose_edges(mba_handle* h, double* r, double* J_from, double* J_to) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t NIMU = h->P.nimu, NPE = h->P.nedge - NIMU;
  if (NPE == 0) return MBA_OK;
  // The kernel writes rows of the full 15x15 edge blocks; a scratch copy of
  // the linearization keeps the solver's buffers untouched.
  DeviceArena tmp;
  InertialLin<double> lin{};
  lin.r = tmp.alloc<double>(15 * h->P.nedge);
  lin.Jf = tmp.alloc<double>(225 * h->P.nedge);
  lin.Jt = tmp.alloc<double>(225 * h->P.nedge);
  cudaError_t e = tmp.err;
  if (e == cudaSuccess) e = launch_pose_edges(h->P, h->P.kf_state, nullptr, lin, nullptr, nullptr, h->stream);
  std::vector<double> hr(15 * NPE), hf(225 * NPE), ht(225 * NPE);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(hr.data(), lin.r + 15 * NIMU, sizeof(double) * 15 * NPE, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && J_from)
    e = cudaMemcpyAsync(hf.data(), lin.Jf + 225 * NIMU, sizeof(double) * 225 * NPE, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && J_to)
    e = cudaMemcpyAsync(ht.data(), lin.Jt + 225 * NIMU, sizeof(double) * 225 * NPE, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  tmp.release();
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  for (int64_t j = 0; j < NPE; ++j)
    for (int a = 0; a < 6; ++a) {
      if (r) r[6 * j + a] = hr[15 * j + a];
      for (int c = 0; c < 6; ++c) {
        if (J_from) J_from[36 * j + 6 * a + c] = hf[225 * j + 15 * a + c];
        if (J_to) J_to[36 * j + 6 * a + c] = ht[225 * j + 15 * a + c];
      }
    }
  return MBA_OK;
}

mba_status mba_relaxation_flags(const mba_problem_desc* d, uint32_t* kf_flags_out, uint8_t* lm_constant_out) {
  if (!d || !kf_flags_out || (d->num_landmarks > 0 && !lm_constant_out) || d->num_keyframes <= 0 ||
      d->num_landmarks < 0)
    return MBA_ERR_INVALID_ARG;
  // options.fix_velocity / fix_gyro_bias / fix_accel_bias / fix_landmark_positions = true
  const uint32_t fixes = MBA_KF_VELOCITY_CONSTANT | MBA_KF_GYRO_BIAS_CONSTANT | MBA_KF_ACCEL_BIAS_CONSTANT;
  for (int64_t k = 0; k < d->num_keyframes; ++k) kf_flags_out[k] = (d->kf_flags ? d->kf_flags[k] : 0u) | fixes;
  for (int64_t l = 0; l < d->num_landmarks; ++l) lm_constant_out[l] = 1;
  return MBA_OK;
}

mba_status mba_gauge_fixes(const mba_problem_desc* d, uint32_t* kf_flags_out, uint8_t* lm_constant_out,
                           int32_t* num_clusters) {
  if (!d || d->num_keyframes <= 0 || d->num_missions <= 0 || d->num_landmarks < 0 || !d->kf_mission) return MBA_ERR_INVALID_ARG;
  const int64_t NK = d->num_keyframes, NL = d->num_landmarks, N = d->num_observations, NM = d->num_missions;
  const int64_t NI = d->num_imu_edges, NPE = d->num_pose_edges;
  if ((N > 0 && (!d->obs_landmark || !d->obs_keyframe)) || (NL > 0 && !d->lm_store_keyframe)) return MBA_ERR_INVALID_ARG;
  for (int64_t k = 0; k < NK; ++k)
    if (d->kf_mission[k] < 0 || d->kf_mission[k] >= NM) return MBA_ERR_OUT_OF_RANGE_INDEX;
  // mission clusters: co-observed landmarks and loop closures (union-find)
  std::vector<int64_t> parent(NM);
  std::iota(parent.begin(), parent.end(), 0);
  auto find = [&](int64_t a) {
    while (parent[a] != a) a = parent[a] = parent[parent[a]];
    return a;
  };
  auto unite = [&](int64_t a, int64_t b) {
    a = find(a); b = find(b);
    if (a != b) parent[std::max(a, b)] = std::min(a, b);
  };
  std::vector<char> kf_in(NK, 0), mis_visual(NM, 0), mis_imu(NM, 0), mis_odo(NM, 0);
  std::vector<int64_t> mis_abs(NM, 0);
  for (int64_t i = 0; i < N; ++i) {
    const int64_t l = d->obs_landmark[i], k = d->obs_keyframe[i];
    if (l < 0 || l >= NL || k < 0 || k >= NK) return MBA_ERR_OUT_OF_RANGE_INDEX;
    const int64_t st = d->lm_store_keyframe[l];
    if (st < 0 || st >= NK) return MBA_ERR_OUT_OF_RANGE_INDEX;
    unite(d->kf_mission[k], d->kf_mission[st]);
    kf_in[k] = kf_in[st] = 1;
    mis_visual[d->kf_mission[k]] = 1;
  }
  for (int64_t e = 0; e < NI; ++e) {
    const int64_t f = d->edge_from[e], t = d->edge_to[e];
    if (f < 0 || f >= NK || t < 0 || t >= NK) return MBA_ERR_OUT_OF_RANGE_INDEX;
    kf_in[f] = kf_in[t] = 1;
    mis_imu[d->kf_mission[f]] = 1;
  }
  for (int64_t j = 0; j < NPE; ++j) {
    const int type = d->pose_edge_type ? d->pose_edge_type[j] : MBA_POSE_EDGE_RELATIVE;
    const int64_t f = d->pose_edge_from[j], t = type == MBA_POSE_EDGE_ABSOLUTE ? f : d->pose_edge_to[j];
    if (f < 0 || f >= NK || t < 0 || t >= NK) return MBA_ERR_OUT_OF_RANGE_INDEX;
    kf_in[f] = kf_in[t] = 1;
    if (type == MBA_POSE_EDGE_LOOP_CLOSURE) unite(d->kf_mission[f], d->kf_mission[t]);
    else if (type == MBA_POSE_EDGE_ABSOLUTE) mis_abs[d->kf_mission[f]]++;
    else mis_odo[d->kf_mission[f]] = 1;
  }
  if (kf_flags_out)
    for (int64_t k = 0; k < NK; ++k) kf_flags_out[k] = d->kf_flags ? d->kf_flags[k] : 0u;
  if (lm_constant_out)
    for (int64_t l = 0; l < NL; ++l) lm_constant_out[l] = d->lm_constant ? d->lm_constant[l] : 0;
  int32_t clusters = 0;
  for (int64_t root = 0; root < NM; ++root) {
    if (find(root) != root) continue;  // root = lowest mission index of its cluster ("first mission")
    ++clusters;
    bool all_imu = true, all_visual = true, all_odo = true;
    int64_t n_abs = 0;
    for (int64_t m = 0; m < NM; ++m) {
      if (find(m) != root) continue;
      all_imu = all_imu && mis_imu[m];
      all_visual = all_visual && mis_visual[m];
      all_odo = all_odo && mis_odo[m];
      n_abs += mis_abs[m];
    }
    const bool scale_obs = all_imu || all_odo || (all_visual && n_abs > 1);
    const bool pos_obs = n_abs > 0, yaw_obs = n_abs > 0, rp_obs = n_abs > 0 || all_imu;
    // first keyframe of the first mission that is part of the problem
    int64_t K = -1;
    for (int64_t k = 0; k < NK && K < 0; ++k)
      if (d->kf_mission[k] == root && kf_in[k]) K = k;
    if (K < 0) continue;
    if (kf_flags_out) {
      uint32_t& f = kf_flags_out[K];
      if (!rp_obs) f |= MBA_KF_POSE_CONSTANT;                 // rotation kAll: the pose block is constant
      else if (!yaw_obs) f |= MBA_KF_GAUGE_ROLL_PITCH;        // kYaw
      if (!pos_obs) f |= MBA_KF_POSITION_CONSTANT;
    }
    if (!scale_obs && lm_constant_out)
      for (int64_t l = 0; l < NL; ++l)
        if (d->lm_store_keyframe[l] == K) { lm_constant_out[l] = 1; break; }
  }
  if (num_clusters) *num_clusters = clusters;
  return MBA_OK;
}

void mba_default_landmark_quality_options(mba_landmark_quality_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->min_observers = 4;
  o->min_observation_angle_deg = 5.0;
  o->max_distance_from_closest_observer = 40.0;
  o->min_distance_from_closest_observer = 0.05;
  o->max_reprojection_error_px = -1.0;
}

mba_status mba_landmark_quality(mba_handle* h, const mba_landmark_quality_options* o, uint8_t* well_constrained) {
  if (!h || !o || (h->P.nlm > 0 && !well_constrained)) return MBA_ERR_INVALID_ARG;
  if (o->min_observers < 0) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t NL = h->P.nlm;
  if (NL == 0) return MBA_OK;
  DeviceArena tmp;
  uint8_t* d = tmp.alloc<uint8_t>(NL);
  cudaError_t e = tmp.err;
  std::vector<uint8_t> good(h->lm_caller.empty() ? 0 : NL);
  uint8_t* host = h->lm_caller.empty() ? well_constrained : good.data();
  if (e == cudaSuccess) e = launch_landmark_quality(h->P, *o, d, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, d, NL, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  tmp.release();
  if (e == cudaSuccess && !h->lm_caller.empty())
    for (int64_t l = 0; l < NL; ++l) well_constrained[h->lm_caller[l]] = good[l];
  return e == cudaSuccess ? MBA_OK : MBA_ERR_CUDA;
}

mba_status mba_read_switch_variables(mba_handle* h, double* s) {
  if (!h || !s) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t NPE = h->P.nedge - h->P.nimu;
  if (NPE == 0) return MBA_OK;
  std::vector<int32_t> swi(NPE);
  std::vector<double> swc(NPE), sw(h->P.nsw);
  cudaError_t e = cudaMemcpyAsync(swi.data(), h->P.pe_swi, sizeof(int32_t) * NPE, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(swc.data(), h->P.pe_swc, sizeof(double) * NPE, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess && h->P.nsw)
    e = cudaMemcpyAsync(sw.data(), h->P.sw, sizeof(double) * h->P.nsw, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  for (int64_t j = 0; j < NPE; ++j) s[j] = swi[j] >= 0 ? sw[swi[j]] : swc[j];
  return MBA_OK;
}

mba_status mba_write_switch_variables(mba_handle* h, const double* s) {
  if (!h || !s) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t NPE = h->P.nedge - h->P.nimu;
  if (NPE == 0) return MBA_OK;
  for (int64_t j = 0; j < NPE; ++j)
    if (!(s[j] >= 0.0 && s[j] <= 1.0)) return MBA_ERR_INVALID_ARG;
  std::vector<int32_t> swi(NPE);
  cudaError_t e = cudaMemcpyAsync(swi.data(), h->P.pe_swi, sizeof(int32_t) * NPE, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  std::vector<double> sw(h->P.nsw), swc(NPE);
  for (int64_t j = 0; j < NPE; ++j) {
    swc[j] = s[j];
    if (swi[j] >= 0) sw[swi[j]] = s[j];
  }
  // pe_swc is read-only for the kernels; it is device memory owned by the handle.
  e = cudaMemcpyAsync(const_cast<double*>(h->P.pe_swc), swc.data(), sizeof(double) * NPE, cudaMemcpyHostToDevice,
                      h->stream);
  if (e == cudaSuccess && h->P.nsw)
    e = cudaMemcpyAsync(h->P.sw, sw.data(), sizeof(double) * h->P.nsw, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  return e == cudaSuccess ? MBA_OK : MBA_ERR_CUDA;
}

mba_status mba_linearize_visual(mba_handle* h, int32_t precision, double* r, double* Jl, double* Js, double* Jo) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  if (h->P.nobs == 0) return MBA_OK;
  if (precision == MBA_PRECISION_FP64) return linearize_visual_host<double>(h, r, Jl, Js, Jo);
  if (precision == MBA_PRECISION_MIXED) return linearize_visual_host<float>(h, r, Jl, Js, Jo);
  return MBA_ERR_INVALID_ARG;
}

mba_status mba_cost(mba_handle* h, int32_t precision, double* cost) {
  if (!h || !cost) return MBA_ERR_INVALID_ARG;
  (void)precision;  // the cost is always reduced in FP64
  cudaSetDevice(h->device);
  cudaStream_t st = h->stream;
  cudaError_t e = cudaMemsetAsync(h->scratch, 0, sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->iscratch, 0, 2 * sizeof(int), st);
  if (e == cudaSuccess) e = launch_visual_cost(h->P, h->P.kf_state, h->P.lm_p, h->scratch, h->iscratch, st);
  InertialLin<double> none{};
  if (e == cudaSuccess) e = launch_inertial(h->P, h->P.kf_state, none, nullptr, nullptr, h->scratch, h->iscratch + 1, st);
  if (e == cudaSuccess) e = launch_pose_edges(h->P, h->P.kf_state, nullptr, none, h->scratch, nullptr, st);
  int flags[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(cost, h->scratch, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(flags, h->iscratch, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  if (flags[1]) return (mba_status)flags[1];
  return flags[0] ? MBA_ERR_NON_FINITE : MBA_OK;
}

mba_status mba_solve(mba_handle* h, const mba_solver_options* opts, mba_summary* summary) {
  if (!h) return MBA_ERR_INVALID_ARG;
  mba_solver_options o;
  if (opts) o = *opts; else mba_default_solver_options(&o);
  if (o.max_num_iterations < 0 || !(o.initial_trust_region_radius > 0)) return MBA_ERR_INVALID_ARG;
  if (h->poisoned) return MBA_ERR_TIMEOUT;
  // Calibration / baseframe variables: FP64 solves with block-Jacobi or chain preconditioning.
  if (h->P.ng > 0 && (o.precision != MBA_PRECISION_FP64 || o.preconditioner == MBA_PRECOND_LEARNED))
    return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  h->cancel.store(0);
  if (o.max_num_iterations == 0) {
    double c = 0;
    mba_status st = mba_cost(h, o.precision, &c);
    if (summary) { summary->initial_cost = summary->final_cost = c; summary->num_iterations = 1; }
    return st;
  }
  if (o.precision == MBA_PRECISION_MIXED) return run_solve<float>(h, o, summary);
  const mba_status st = run_solve<double>(h, o, summary);
  if (h->P.ng > 0 && (st == MBA_OK || st == MBA_ERR_CANCELLED)) {
    // The solve moved cameras / baseframes on the device: refresh their FP32 mirrors.
    std::vector<mba_camera> cams(h->P.ncam);
    std::vector<double> mis(7 * h->P.nmis);
    mba_status r = mba_read_calibration(h, cams.data(), mis.data());
    if (r == MBA_OK) r = mba_write_calibration(h, cams.data(), mis.data());
    if (r != MBA_OK) return r;
  }
  return st;
}

mba_status mba_read_state(mba_handle* h, double* kx, double* kv, double* kbg, double* kba, double* lp) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  if (ensure_stage_state(h) != MBA_OK) return MBA_ERR_CUDA;
  const int64_t NK = h->P.nkf, NL = h->P.nlm;
  double* sx = h->stage_state;
  double* sv = sx + 7 * NK;
  double* sg = sv + 3 * NK;
  double* sa = sg + 3 * NK;
  double* sl = sa + 3 * NK;
  cudaStream_t st = h->stream;
  cudaError_t e = launch_pack_state(h->P, kx ? sx : nullptr, kv ? sv : nullptr, kbg ? sg : nullptr,
                                    kba ? sa : nullptr, lp ? sl : nullptr, h->lm_caller_dev, 0, st);
  if (e == cudaSuccess && kx) e = cudaMemcpyAsync(kx, sx, sizeof(double) * 7 * NK, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && kv) e = cudaMemcpyAsync(kv, sv, sizeof(double) * 3 * NK, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && kbg) e = cudaMemcpyAsync(kbg, sg, sizeof(double) * 3 * NK, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && kba) e = cudaMemcpyAsync(kba, sa, sizeof(double) * 3 * NK, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && lp && NL) e = cudaMemcpyAsync(lp, sl, sizeof(double) * 3 * NL, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return cuda_status(e);
}

mba_status mba_write_state(mba_handle* h, const double* kx, const double* kv, const double* kbg, const double* kba,
                           const double* lp) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t NK = h->P.nkf, NL = h->P.nlm;
  if (kx)
    for (int64_t k = 0; k < NK; ++k)
      if (!quat_ok(kx + 7 * k)) return MBA_ERR_INVALID_ARG;
  if (ensure_stage_state(h) != MBA_OK) return MBA_ERR_CUDA;
  double* sx = h->stage_state;
  double* sv = sx + 7 * NK;
  double* sg = sv + 3 * NK;
  double* sa = sg + 3 * NK;
  double* sl = sa + 3 * NK;
  cudaStream_t st = h->stream;
  cudaError_t e = cudaSuccess;
  if (kx) e = cudaMemcpyAsync(sx, kx, sizeof(double) * 7 * NK, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && kv) e = cudaMemcpyAsync(sv, kv, sizeof(double) * 3 * NK, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && kbg) e = cudaMemcpyAsync(sg, kbg, sizeof(double) * 3 * NK, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && kba) e = cudaMemcpyAsync(sa, kba, sizeof(double) * 3 * NK, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && lp && NL) e = cudaMemcpyAsync(sl, lp, sizeof(double) * 3 * NL, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = launch_pack_state(h->P, kx ? sx : nullptr, kv ? sv : nullptr, kbg ? sg : nullptr, kba ? sa : nullptr,
                          (lp && NL) ? sl : nullptr, h->lm_caller_dev, 1, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return cuda_status(e);
}

mba_status mba_read_calibration(mba_handle* h, mba_camera* cameras, double* mission_q_GM_p_GM) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t NC = h->P.ncam, NM = h->P.nmis;
  std::vector<DevCamera> dc(NC);
  std::vector<double> dm(8 * NM);
  cudaStream_t st = h->stream;
  cudaError_t e = cudaMemcpyAsync(dc.data(), h->P.cams, sizeof(DevCamera) * NC, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dm.data(), h->P.mis, sizeof(double) * 8 * NM, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  for (int64_t c = 0; c < NC && cameras; ++c) {
    mba_camera& o = cameras[c];
    std::memset(&o, 0, sizeof(o));
    for (int a = 0; a < 4; ++a) { o.intrinsics[a] = dc[c].intr[a]; o.distortion[a] = dc[c].dist[a]; o.q_CI_p_CI[a] = dc[c].q_CI[a]; }
    for (int a = 0; a < 3; ++a) o.q_CI_p_CI[4 + a] = dc[c].p_CI[a];
    o.distortion_type = dc[c].dtype;
    o.width = dc[c].width;
    o.height = dc[c].height;
  }
  for (int64_t m = 0; m < NM && mission_q_GM_p_GM; ++m)
    for (int a = 0; a < 7; ++a) mission_q_GM_p_GM[7 * m + a] = dm[8 * m + a];
  return MBA_OK;
}

mba_status mba_write_calibration(mba_handle* h, const mba_camera* cameras, const double* mission_q_GM_p_GM) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t NC = h->P.ncam, NM = h->P.nmis;
  std::vector<DevCamera> dc(NC);
  std::vector<double> dm(8 * NM);
  cudaStream_t st = h->stream;
  cudaError_t e = cudaMemcpyAsync(dc.data(), h->P.cams, sizeof(DevCamera) * NC, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dm.data(), h->P.mis, sizeof(double) * 8 * NM, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  for (int64_t c = 0; c < NC && cameras; ++c) {
    const mba_camera& s = cameras[c];
    if (!quat_ok(s.q_CI_p_CI)) return MBA_ERR_INVALID_ARG;
    if (s.distortion_type != dc[c].dtype || s.width != dc[c].width || s.height != dc[c].height) return MBA_ERR_INVALID_ARG;
    for (int a = 0; a < 4; ++a)
      if (!std::isfinite(s.intrinsics[a]) || !std::isfinite(s.distortion[a])) return MBA_ERR_NON_FINITE;
    for (int a = 0; a < 7; ++a) if (!std::isfinite(s.q_CI_p_CI[a])) return MBA_ERR_NON_FINITE;
    for (int a = 0; a < 4; ++a) { dc[c].intr[a] = s.intrinsics[a]; dc[c].dist[a] = s.distortion[a]; dc[c].q_CI[a] = s.q_CI_p_CI[a]; }
    for (int a = 0; a < 3; ++a) dc[c].p_CI[a] = s.q_CI_p_CI[4 + a];
  }
  for (int64_t m = 0; m < NM && mission_q_GM_p_GM; ++m) {
    if (!quat_ok(mission_q_GM_p_GM + 7 * m)) return MBA_ERR_INVALID_ARG;
    for (int a = 0; a < 7; ++a) {
      if (!std::isfinite(mission_q_GM_p_GM[7 * m + a])) return MBA_ERR_NON_FINITE;
      dm[8 * m + a] = mission_q_GM_p_GM[7 * m + a];
    }
  }
  // FP32 mirrors of the mixed path
  std::vector<DevCameraT<float>> fc(NC);
  std::vector<float> fm(8 * NM, 0.f);
  for (int64_t c = 0; c < NC; ++c) {
    DevCameraT<float>& o = fc[c];
    std::memset(&o, 0, sizeof(o));
    for (int a = 0; a < 4; ++a) { o.intr[a] = (float)dc[c].intr[a]; o.dist[a] = (float)dc[c].dist[a]; o.q_CI[a] = (float)dc[c].q_CI[a]; }
    for (int a = 0; a < 3; ++a) o.p_CI[a] = (float)dc[c].p_CI[a];
    o.dtype = dc[c].dtype;
    o.width = dc[c].width;
    o.height = dc[c].height;
  }
  for (int64_t m = 0; m < 8 * NM; ++m) fm[m] = (float)dm[m];
  e = cudaMemcpyAsync(const_cast<DevCamera*>(h->P.cams), dc.data(), sizeof(DevCamera) * NC, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(const_cast<double*>(h->P.mis), dm.data(), sizeof(double) * 8 * NM, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && h->P.cams_f)
    e = cudaMemcpyAsync(const_cast<DevCameraT<float>*>(h->P.cams_f), fc.data(), sizeof(DevCameraT<float>) * NC,
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && h->P.mis_f)
    e = cudaMemcpyAsync(const_cast<float*>(h->P.mis_f), fm.data(), sizeof(float) * 8 * NM, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return cuda_status(e);
}

void mba_cancel(mba_handle* h) {
  if (!h) return;
  h->cancel.store(1);
  if (h->cancel_host) *h->cancel_host = 1;  // seen by the device-driven loop
}

mba_status mba_time_visual_kernel(mba_handle* h, int32_t mode, int32_t iters, double* ms_per_launch) {
  if (!h || !ms_per_launch || iters <= 0 || (mode != 0 && mode != 1)) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  mba_status ms = (mode == 0) ? ensure_solver_buffers<double>(h, h->b64) : ensure_solver_buffers<float>(h, h->b32);
  if (ms != MBA_OK) return ms;
  // Between timed launches a 256 MiB buffer (larger than the 129 MB L2) is
  // written so every launch starts with a cold L2.
  const size_t flush_bytes = 256ull << 20;
  if (!h->l2_flush) {
    h->l2_flush = h->arena.alloc<char>((int64_t)flush_bytes);
    if (h->arena.err != cudaSuccess) return MBA_ERR_CUDA;
  }
  cudaStream_t st = h->stream;
  auto launch = [&]() {
    return mode == 0 ? launch_visual_linearize<double>(h->P, h->b64.vis, nullptr, st)
                     : launch_visual_linearize<float>(h->P, h->b32.vis, nullptr, st);
  };
  cudaError_t e = cudaSuccess;
  for (int w = 0; w < 3 && e == cudaSuccess; ++w) e = launch();
  std::vector<cudaEvent_t> ev(2 * iters);
  for (auto& x : ev) cudaEventCreate(&x);
  for (int it = 0; it < iters && e == cudaSuccess; ++it) {
    e = cudaMemsetAsync(h->l2_flush, it & 0xff, flush_bytes, st);
    if (e != cudaSuccess) break;
    cudaEventRecord(ev[2 * it], st);
    e = launch();
    cudaEventRecord(ev[2 * it + 1], st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  double total = 0.0;
  for (int it = 0; it < iters && e == cudaSuccess; ++it) {
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[2 * it], ev[2 * it + 1]);
    total += t;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  *ms_per_launch = total / iters;
  return cuda_status(e);
}

mba_status mba_reduced_system(mba_handle* h, int32_t precision, double radius, double* diag, int32_t* upper_ij,
                              double* upper, double* inertial, double* rhs) {
  if (!h || !(radius > 0.0)) return MBA_ERR_INVALID_ARG;
  if (precision != MBA_PRECISION_FP64 && precision != MBA_PRECISION_MIXED) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  if (precision == MBA_PRECISION_MIXED) return reduced_system<float>(h, radius, diag, upper_ij, upper, inertial, rhs);
  return reduced_system<double>(h, radius, diag, upper_ij, upper, inertial, rhs);
}

mba_status mba_chain_apply(mba_handle* h, int32_t precision, double radius, const double* r, double* z) {
  if (!h || !r || !z || !(radius > 0.0)) return MBA_ERR_INVALID_ARG;
  if (precision != MBA_PRECISION_FP64 && precision != MBA_PRECISION_MIXED) return MBA_ERR_INVALID_ARG;
  if (h->P.nkf == 0) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  if (precision == MBA_PRECISION_MIXED) return chain_apply_host<float>(h, radius, r, z);
  return chain_apply_host<double>(h, radius, r, z);
}

mba_status mba_rejected_landmarks(mba_handle* h, uint8_t* flags, int64_t* count) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t NL = h->P.nlm;
  std::vector<int32_t> off(NL);
  if (NL && cudaMemcpy(off.data(), h->P.lm_off, sizeof(int32_t) * NL, cudaMemcpyDeviceToHost) != cudaSuccess)
    return MBA_ERR_CUDA;
  int64_t c = 0;
  for (int64_t l = 0; l < NL; ++l) {
    c += off[l] != 0;
    if (flags) flags[h->lm_caller.empty() ? l : h->lm_caller[l]] = off[l] != 0;
  }
  if (count) *count = c;
  return MBA_OK;
}

mba_status mba_get_stats(mba_handle* h, mba_problem_stats* s) {
  if (!h || !s) return MBA_ERR_INVALID_ARG;
  s->num_keyframes = h->P.nkf;
  s->num_landmarks = h->P.nlm;
  s->num_observations = h->P.nobs;
  s->num_imu_edges = h->P.nimu;
  s->num_schur_pose_blocks = 2 * h->S.npu;
  s->device_bytes = h->arena.bytes;
  s->num_pose_edges = h->P.nedge - h->P.nimu;
  return MBA_OK;
}

}  // extern "C"

// ---- learned preconditioner model

namespace {

// Reduced system of the current state (mixed precision) with the model's
// coefficients and their chain factorization, ready for the probe loss.
mba_status gnn_prepare(mba_handle* h, mba_gnn* m, double radius, SolverLaunch<float>* out) {
  mba_status ms = ensure_common_solver(h, 2);
  if (ms != MBA_OK) return ms;
  SolverBuffers<float>& b = h->b32;
  if ((ms = ensure_solver_buffers<float>(h, b)) != MBA_OK) return ms;
  if ((ms = ensure_chain_buffers<float>(h, b)) != MBA_OK) return ms;
  if ((ms = ensure_gnn_work(h)) != MBA_OK) return ms;
  mba_solver_options o;
  mba_default_solver_options(&o);
  o.precision = MBA_PRECISION_MIXED;
  o.preconditioner = MBA_PRECOND_LEARNED;
  mba_gnn* keep = h->model;
  h->model = m;
  SolverLaunch<float> s = make_launch<float>(h, b, o);
  h->model = keep;
  cudaStream_t st = h->stream;
  cudaError_t e = solver_init_control(h->ctl, radius, st);
  if (e == cudaSuccess) e = linearize_current<float>(h, b, s, o.jacobi_scaling, st);
  if (e == cudaSuccess) e = solver_build_reduced<float>(s, st);
  LmControl c;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&c, h->ctl, sizeof(c), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  if (c.status) return (mba_status)c.status;
  if (c.chain_failed) return MBA_ERR_NOT_SPD;
  *out = s;
  return MBA_OK;
}

// Coefficients and chain factorization after a parameter update.
cudaError_t gnn_refresh(mba_handle* h, const SolverLaunch<float>& s) {
  cudaStream_t st = h->stream;
  cudaError_t e = cudaMemsetAsync(&h->ctl->chain_failed, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) e = gnn_forward<float>(s, s.gg, s.gp, s.gw, st);
  if (e == cudaSuccess) e = chain_factor<float>(s, st);
  return e;
}

}  // namespace

extern "C" {

int64_t mba_gnn_num_parameters(void) { return GnnLayout::make().total; }

mba_status mba_gnn_create(int32_t device, uint64_t seed, mba_gnn** out) {
  if (!out) return MBA_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MBA_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(device);
  mba_gnn* m = new (std::nothrow) mba_gnn();
  if (!m) return MBA_ERR_CUDA;
  m->device = device;
  const int64_t n = GnnLayout::make().total;
  DeviceArena& A = m->arena;
  m->p.w = A.alloc<float>(n);
  m->p.wb = A.alloc<__nv_bfloat16>(n);
  m->p.wt = A.alloc<__nv_bfloat16>(n);
  m->p.g = A.alloc<float>(n);
  m->p.m = A.alloc<float>(n);
  m->p.v = A.alloc<float>(n);
  m->p.step = 0;
  cudaError_t e = A.err;
  if (e == cudaSuccess) e = gnn_init_params(m->p, seed, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    A.release();
    delete m;
    return MBA_ERR_CUDA;
  }
  *out = m;
  return MBA_OK;
}

void mba_gnn_destroy(mba_gnn* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  m->arena.release();
  delete m;
}

mba_status mba_gnn_get_parameters(mba_gnn* m, float* params) {
  if (!m || !params) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(m->device);
  return cuda_status(cudaMemcpy(params, m->p.w, sizeof(float) * GnnLayout::make().total, cudaMemcpyDeviceToHost));
}

mba_status mba_gnn_set_parameters(mba_gnn* m, const float* params) {
  if (!m || !params) return MBA_ERR_INVALID_ARG;
  const int64_t n = GnnLayout::make().total;
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(params[i])) return MBA_ERR_NON_FINITE;
  cudaSetDevice(m->device);
  cudaError_t e = cudaMemcpy(m->p.w, params, sizeof(float) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->p.m, 0, sizeof(float) * n);
  if (e == cudaSuccess) e = cudaMemset(m->p.v, 0, sizeof(float) * n);
  m->p.step = 0;
  if (e == cudaSuccess) e = gnn_sync_bf16(m->p, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return cuda_status(e);
}

mba_status mba_set_preconditioner_model(mba_handle* h, mba_gnn* m) {
  if (!h) return MBA_ERR_INVALID_ARG;
  if (m && m->device != h->device) return MBA_ERR_INVALID_ARG;
  h->model = m;
  return MBA_OK;
}

mba_status mba_gnn_train(mba_handle* h, mba_gnn* m, double radius, int32_t nprobe, int32_t steps, float lr,
                         uint64_t seed, double* losses) {
  if (!h || !m || m->device != h->device || nprobe < 1 || steps < 0 || !(radius > 0.0) || !(lr >= 0.f))
    return MBA_ERR_INVALID_ARG;
  if (h->poisoned) return MBA_ERR_TIMEOUT;
  cudaSetDevice(h->device);
  SolverLaunch<float> s;
  mba_status ms = gnn_prepare(h, m, radius, &s);
  if (ms != MBA_OK) return ms;
  cudaStream_t st = h->stream;
  for (int32_t k = 0; k < steps; ++k) {
    cudaError_t e = cudaMemsetAsync(&h->ctl->fatal, 0, sizeof(int32_t), st);
    if (e == cudaSuccess) e = gnn_loss_backward<float>(s, s.gg, m->p, s.gw, nprobe, nullptr, seed + 104729ull * k, st);
    double loss = 0.0;
    int32_t fatal = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&loss, s.gw.loss, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&fatal, &h->ctl->fatal, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return MBA_ERR_CUDA;
    if (fatal) {
      h->poisoned = true;
      return MBA_ERR_TIMEOUT;
    }
    if (losses) losses[k] = loss;
    if (!std::isfinite(loss)) return MBA_ERR_NON_FINITE;
    if (lr > 0.f) {
      m->p.step++;
      e = gnn_adam(m->p, lr, st);
      s.gp = m->p;
      if (e == cudaSuccess) e = gnn_refresh(h, s);
      int32_t failed = 0;
      if (e == cudaSuccess) e = cudaMemcpyAsync(&failed, &h->ctl->chain_failed, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return MBA_ERR_CUDA;
      if (failed) return MBA_ERR_NOT_SPD;
    }
  }
  return MBA_OK;
}

mba_status mba_gnn_gradient(mba_handle* h, mba_gnn* m, double radius, int32_t nprobe, const float* probes,
                            uint64_t seed, float* grad, double* loss, double* coef) {
  if (!h || !m || m->device != h->device || nprobe < 1 || !(radius > 0.0)) return MBA_ERR_INVALID_ARG;
  if (h->poisoned) return MBA_ERR_TIMEOUT;
  cudaSetDevice(h->device);
  SolverLaunch<float> s;
  mba_status ms = gnn_prepare(h, m, radius, &s);
  if (ms != MBA_OK) return ms;
  cudaStream_t st = h->stream;
  const int64_t n15 = 15 * h->P.nkf, np = GnnLayout::make().total;
  float* dprobe = nullptr;
  cudaError_t e = cudaSuccess;
  if (probes) {
    e = cudaMalloc(&dprobe, sizeof(float) * n15 * nprobe);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dprobe, probes, sizeof(float) * n15 * nprobe, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(&h->ctl->fatal, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) e = gnn_loss_backward<float>(s, s.gg, m->p, s.gw, nprobe, dprobe, seed, st);
  int32_t fatal = 0;
  if (e == cudaSuccess && grad) e = cudaMemcpyAsync(grad, m->p.g, sizeof(float) * np, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, s.gw.loss, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && coef) e = cudaMemcpyAsync(coef, s.C.coef, sizeof(double) * 3 * h->P.nkf, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&fatal, &h->ctl->fatal, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (dprobe) cudaFree(dprobe);
  if (e == cudaSuccess && fatal) {
    h->poisoned = true;
    return MBA_ERR_TIMEOUT;
  }
  return cuda_status(e);
}

mba_status mba_chain_structure(mba_handle* h, int32_t* perm, int32_t* link_edge, int32_t* link_blk) {
  if (!h) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  const int64_t n = h->P.nkf;
  cudaError_t e = cudaSuccess;
  if (perm) e = cudaMemcpy(perm, h->S.chain_perm, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && link_edge) e = cudaMemcpy(link_edge, h->S.link_edge, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && link_blk) e = cudaMemcpy(link_blk, h->S.link_blk, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
  return cuda_status(e);
}

}  // extern "C"

// ---- autotuning

namespace {

int chain_tail_level(int64_t n, int levels, int64_t nodes) {
  int l = 0;
  while (l < levels && ((n + ((int64_t)1 << l) - 1) >> l) > nodes) ++l;
  return l;
}

// Segment of the chain sweeps (positions per block, a power of two up to 256)
// -> its level; 1 -> 0 (one launch per level).
int chain_segment_level(int seg) {
  int m = 0;
  while ((1 << m) < seg) ++m;
  return m;
}

mba_status apply_schur_chunk(mba_handle* h, int chunk) {
  std::vector<int32_t> tgt, len;
  std::vector<int64_t> beg, rco;
  cut_chunks(h->tgt_off, h->tgt_order, h->tgt_row, h->P.nkf, chunk, &tgt, &beg, &len, &rco);
  int32_t* dt = h->arena.upload(tgt, h->stream);
  int64_t* db = h->arena.upload(beg, h->stream);
  int32_t* dl = h->arena.upload(len, h->stream);
  int64_t* dr = h->arena.upload(rco, h->stream);
  if (h->arena.err != cudaSuccess || cudaStreamSynchronize(h->stream) != cudaSuccess) return MBA_ERR_CUDA;
  h->S.chunk_tgt = dt;
  h->S.chunk_beg = db;
  h->S.chunk_len = dl;
  h->S.row_chunk_off = dr;
  h->S.nchunk = (int64_t)tgt.size();
  h->tuning.schur_chunk = chunk;
  return MBA_OK;
}

// Mean milliseconds per call of fn over `reps` calls after `warm` calls.
template <typename F>
double time_ms(cudaStream_t st, int warm, int reps, F fn) {
  for (int i = 0; i < warm; ++i) fn();
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, st);
  for (int i = 0; i < reps; ++i) fn();
  cudaEventRecord(b, st);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}

template <typename T>
mba_status autotune(mba_handle* h, mba_tuning* out) {
  mba_status ms = ensure_common_solver(h, 2);
  if (ms != MBA_OK) return ms;
  SolverBuffers<T>& b = buffers_of<T>(h);
  if ((ms = ensure_solver_buffers<T>(h, b)) != MBA_OK) return ms;
  if ((ms = ensure_chain_buffers<T>(h, b)) != MBA_OK) return ms;
  mba_solver_options o;
  mba_default_solver_options(&o);
  o.preconditioner = MBA_PRECOND_CHAIN;
  cudaStream_t st = h->stream;
  if (chain_default_coef(b.C.coef, h->P.nkf, st) != cudaSuccess) return MBA_ERR_CUDA;
  SolverLaunch<T> s = make_launch<T>(h, b, o);
  cudaError_t e = solver_init_control(h->ctl, o.initial_trust_region_radius, st);
  if (e == cudaSuccess) e = linearize_current<T>(h, b, s, o.jacobi_scaling, st);
  if (e == cudaSuccess) e = solver_build_reduced<T>(s, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  mba_tuning best = h->tuning;
  // evaluation kernel: one thread per observation (plain or register-lean)
  // or the pipelined persistent loop, and the block size
  double tbest = 1e30;
  for (int pipe : {0, 1})
    for (int minb : {1, 2, 3, 4}) {
      if (pipe ? minb >= 3 : minb == 2) continue;  // one-per-thread: 1, 3 or 4 blocks; pipelined: 1 or 2
      for (int bs : {64, 128, 256}) {
        DevProblem P = h->P;
        P.vis_block = bs;
        P.vis_minb = minb;
        P.vis_pipe = pipe;
        const double t = time_ms(st, 1, 3, [&]() { launch_visual_linearize<T>(P, b.vis, nullptr, st); });
        if (t < tbest) {
          tbest = t;
          best.visual_block = bs;
          best.visual_min_blocks = minb;
          best.visual_pipelined = pipe ? 1 : 2;
          best.visual_ms = t;
        }
      }
    }
  h->P.vis_block = best.visual_block;
  h->P.vis_minb = best.visual_min_blocks;
  h->P.vis_pipe = best.visual_pipelined == 1;
  // Schur pairs per thread (each candidate re-cuts the pair chunks on the
  // host; chunks below 16 pairs have not won on any map measured)
  tbest = 1e30;
  for (int chunk : {16, 32, 64}) {
    if (chunk != h->tuning.schur_chunk && (ms = apply_schur_chunk(h, chunk)) != MBA_OK) return ms;
    for (int split : {2, 1}) {  // one or two threads per chunk
      h->S.schur_split = split == 1;
      SolverLaunch<T> sc = make_launch<T>(h, b, o);
      const double t = time_ms(st, 1, 2, [&]() { solver_schur_pairs<T>(sc, st); });
      if (t < tbest) { tbest = t; best.schur_chunk = chunk; best.schur_split = split; best.schur_ms = t; }
    }
  }
  h->S.schur_split = best.schur_split == 1;
  if (best.schur_chunk != h->tuning.schur_chunk && (ms = apply_schur_chunk(h, best.schur_chunk)) != MBA_OK) return ms;
  // single-block tail of the chain sweeps (the factorization from the build is reused)
  tbest = 1e30;
  const int levels = h->S.chain_levels;
  h->S.chain_seg = 0;
  h->S.chain_tail_sm = 0;
  for (int nodes : {32, 64, 128, 256, 512}) {
    h->S.chain_tail = chain_tail_level(h->P.nkf, levels, nodes);
    SolverLaunch<T> sc = make_launch<T>(h, b, o);
    const double t = time_ms(st, 2, 10, [&]() { chain_apply<T>(sc, sc.L.rhs, sc.L.z, &h->ctl->pcg_rz0, st); });
    if (t < tbest) {
      tbest = t;
      best.chain_tail_nodes = nodes;
      best.chain_segment = 1;
      best.chain_tail_smem = 2;
      best.chain_apply_ms = t;
    }
  }
  // segmented sweeps: positions per block; the tail's vectors in shared or global memory
  for (int seg : {16, 32, 64, 128, 256})
    for (int tsm : {1, 2}) {
      h->S.chain_seg = chain_segment_level(seg);
      h->S.chain_tail_sm = tsm == 1;
      SolverLaunch<T> sc = make_launch<T>(h, b, o);
      const double t = time_ms(st, 2, 10, [&]() { chain_apply<T>(sc, sc.L.rhs, sc.L.z, &h->ctl->pcg_rz0, st); });
      if (t < tbest) { tbest = t; best.chain_segment = seg; best.chain_tail_smem = tsm; best.chain_apply_ms = t; }
    }
  h->S.chain_tail = chain_tail_level(h->P.nkf, levels, best.chain_tail_nodes);
  h->S.chain_seg = chain_segment_level(best.chain_segment);
  h->S.chain_tail_sm = best.chain_tail_smem == 1;
  // PCG product: pose blocks read once (atomics) or from both rows
  tbest = 1e30;
  for (int prod : {2, 1}) {
    h->S.spmv_sym = prod == 1;
    SolverLaunch<T> sc = make_launch<T>(h, b, o);
    const double t = time_ms(st, 2, 10, [&]() { solver_product<T>(sc, prod == 1, st); });
    if (t < tbest) { tbest = t; best.pcg_product = prod; }
  }
  h->S.spmv_sym = best.pcg_product == 1;
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return MBA_ERR_CUDA;
  h->tuning = best;
  if (out) *out = best;
  return MBA_OK;
}

}  // namespace

extern "C" {

mba_status mba_autotune(mba_handle* h, int32_t precision, mba_tuning* out) {
  if (!h) return MBA_ERR_INVALID_ARG;
  if (precision != MBA_PRECISION_FP64 && precision != MBA_PRECISION_MIXED) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  if (h->P.nkf == 0) return MBA_ERR_INVALID_ARG;
  return precision == MBA_PRECISION_MIXED ? autotune<float>(h, out) : autotune<double>(h, out);
}

mba_status mba_set_tuning(mba_handle* h, const mba_tuning* t) {
  if (!h || !t) return MBA_ERR_INVALID_ARG;
  if (t->visual_block && (t->visual_block < 32 || t->visual_block > 256 || t->visual_block % 32)) return MBA_ERR_INVALID_ARG;
  if (t->schur_chunk < 0 || t->chain_tail_nodes < 0) return MBA_ERR_INVALID_ARG;
  if (t->chain_segment && (t->chain_segment > 256 || (t->chain_segment & (t->chain_segment - 1))))
    return MBA_ERR_INVALID_ARG;
  if (t->chain_tail_smem < 0 || t->chain_tail_smem > 2) return MBA_ERR_INVALID_ARG;
  if (t->pcg_product < 0 || t->pcg_product > 2) return MBA_ERR_INVALID_ARG;
  if (t->schur_split < 0 || t->schur_split > 2) return MBA_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  if (t->visual_block) { h->P.vis_block = t->visual_block; h->tuning.visual_block = t->visual_block; }
  if (t->visual_min_blocks) {
    if (t->visual_min_blocks < 1 || t->visual_min_blocks > 4) return MBA_ERR_INVALID_ARG;
    h->P.vis_minb = t->visual_min_blocks;
    h->tuning.visual_min_blocks = t->visual_min_blocks;
  }
  if (t->visual_pipelined) {
    if (t->visual_pipelined != 1 && t->visual_pipelined != 2) return MBA_ERR_INVALID_ARG;
    h->P.vis_pipe = t->visual_pipelined == 1;
    h->tuning.visual_pipelined = t->visual_pipelined;
  }
  if (t->schur_chunk && t->schur_chunk != h->tuning.schur_chunk) {
    mba_status ms = apply_schur_chunk(h, t->schur_chunk);
    if (ms != MBA_OK) return ms;
  }
  if (t->chain_tail_nodes) {
    h->S.chain_tail = chain_tail_level(h->P.nkf, h->S.chain_levels, t->chain_tail_nodes);
    h->tuning.chain_tail_nodes = t->chain_tail_nodes;
  }
  if (t->chain_segment) {
    h->S.chain_seg = chain_segment_level(t->chain_segment);
    h->tuning.chain_segment = t->chain_segment;
  }
  if (t->chain_tail_smem) {
    h->S.chain_tail_sm = t->chain_tail_smem == 1;
    h->tuning.chain_tail_smem = t->chain_tail_smem;
  }
  if (t->pcg_product) {
    h->S.spmv_sym = t->pcg_product == 1;
    h->tuning.pcg_product = t->pcg_product;
  }
  if (t->schur_split) {
    h->S.schur_split = t->schur_split == 1;
    h->tuning.schur_split = t->schur_split;
  }
  return MBA_OK;
}

mba_status mba_gnn_gemm_wait_check(int32_t device) {
  if (cudaSetDevice(device) != cudaSuccess) return MBA_ERR_NO_DEVICE;
  if (gnn_gemm_tc_prepare() != cudaSuccess) return MBA_ERR_CUDA;
  const int64_t n = 128;
  void *dA = nullptr, *dW = nullptr, *dZ = nullptr, *df = nullptr;
  cudaError_t e = cudaMalloc(&dA, sizeof(uint16_t) * n * 64);
  if (e == cudaSuccess) e = cudaMalloc(&dW, sizeof(uint16_t) * 64 * 64);
  if (e == cudaSuccess) e = cudaMalloc(&dZ, sizeof(float) * n * 64);
  if (e == cudaSuccess) e = cudaMalloc(&df, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(df, 0, sizeof(int));
  if (e == cudaSuccess)
    e = gnn_gemm_tc_wait_check(n, (const __nv_bfloat16*)dA, (const __nv_bfloat16*)dW, (float*)dZ, (int*)df, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int fatal = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&fatal, df, sizeof(int), cudaMemcpyDeviceToHost);
  for (void* p : {dA, dW, dZ, df})
    if (p) cudaFree(p);
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  return fatal ? MBA_ERR_TIMEOUT : MBA_OK;
}

mba_status mba_gnn_gemm(int32_t device, int64_t n, int32_t k, const uint16_t* A, const uint16_t* W,
                        const uint16_t* A2, const uint16_t* W2, const float* bias, float* Z, uint16_t* H) {
  if (n <= 0 || (k != 32 && k != 64) || !A || !W || !Z || (!A2) != (!W2)) return MBA_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MBA_ERR_NO_DEVICE;
  if (gnn_gemm_tc_prepare() != cudaSuccess) return MBA_ERR_CUDA;
  const size_t na = sizeof(uint16_t) * (size_t)n * k, nw = sizeof(uint16_t) * 64 * (size_t)k;
  void *dA = nullptr, *dW = nullptr, *dA2 = nullptr, *dW2 = nullptr, *db = nullptr, *dZ = nullptr, *dH = nullptr,
       *df = nullptr;
  cudaError_t e = cudaMalloc(&dA, na);
  if (e == cudaSuccess) e = cudaMalloc(&dW, nw);
  if (e == cudaSuccess && A2) e = cudaMalloc(&dA2, na);
  if (e == cudaSuccess && W2) e = cudaMalloc(&dW2, nw);
  if (e == cudaSuccess && bias) e = cudaMalloc(&db, 64 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dZ, sizeof(float) * 64 * (size_t)n);
  if (e == cudaSuccess && H) e = cudaMalloc(&dH, sizeof(uint16_t) * 64 * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&df, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dA, A, na, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dW, W, nw, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && A2) e = cudaMemcpy(dA2, A2, na, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && W2) e = cudaMemcpy(dW2, W2, nw, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && bias) e = cudaMemcpy(db, bias, 64 * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(df, 0, sizeof(int));
  if (e == cudaSuccess)
    e = gnn_gemm_tc(n, k, (const __nv_bfloat16*)dA, (const __nv_bfloat16*)dW, (const __nv_bfloat16*)dA2,
                    (const __nv_bfloat16*)dW2, (const float*)db, (float*)dZ, (__nv_bfloat16*)dH, (int*)df, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int fatal = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&fatal, df, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(Z, dZ, sizeof(float) * 64 * (size_t)n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && H) e = cudaMemcpy(H, dH, sizeof(uint16_t) * 64 * (size_t)n, cudaMemcpyDeviceToHost);
  for (void* p : {dA, dW, dA2, dW2, db, dZ, dH, df})
    if (p) cudaFree(p);
  if (e == cudaErrorInvalidValue) return MBA_ERR_INVALID_ARG;
  if (e != cudaSuccess) return MBA_ERR_CUDA;
  return fatal ? MBA_ERR_TIMEOUT : MBA_OK;
}

}  // extern "C"
