// Device-resident Levenberg-Marquardt solver state (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace mba {

// Slot pairs per thread of the Schur pair kernel (a target with more pairs
// is split into several chunks that add atomically).
constexpr int64_t kSchurChunk = 16;

// Static sparsity of the reduced camera system, built on the host at create.
struct SchurPattern {
  int64_t nslot = 0;      // landmark slots: slot 0 = store keyframe, then one per non-keyframe observation
  int64_t npu = 0;        // upper (i < j) pose-pose 6x6 blocks
  int64_t npair = 0;      // Schur slot pairs (a <= b) within a landmark
  int64_t* lm_slot_off;   // [nlm+1]
  int32_t* slot_kf;       // [nslot]
  int32_t* slot_lm;       // [nslot]
  int32_t* obs_slot;      // [nobs] slot of the observer, -1 for kLocalKeyframe
  int32_t* obs_pblk;      // [nobs] upper block of (store, observer), -1 for kLocalKeyframe
  int64_t nchunk = 0;     // pair chunks (contiguous pair ranges of one target)
  int32_t* pair_a;        // [npair] global slot ids, sorted by target; slot_kf[a] <= slot_kf[b]
  int32_t* pair_b;
  int32_t* chunk_tgt;     // [nchunk] target id (kf for diagonal, nkf + upper block);
                          //   bitwise-not of it when the target spans several chunks
  int64_t* chunk_off;     // [nchunk+1] pair range of each chunk
  int32_t* pu_i;          // [npu]
  int32_t* pu_j;
  int64_t* row_off;       // [nkf+1] full (both orientations) pose-pose rows
  int32_t* row_col;       // [2 npu]
  int32_t* row_blk;       // [2 npu] block index into SP (upper b -> b, lower -> npu + b)
  int64_t* kfe_off;       // [nkf+1] incident inertial edges
  int32_t* kfe;           // +(e+1): keyframe is 'from' ; -(e+1): keyframe is 'to'
};

// Device control block of the LM loop (all scalars live on the device).
struct LmControl {
  double cost;
  double cost_cand;
  double model_change;
  double radius;
  double decrease_factor;
  double step_norm2;
  double x_norm2;
  double pcg_rz0;
  double pcg_bnorm2;
  double pcg_pq[3];
  double pcg_rr[3];
  double pcg_rz[3];
  int32_t accepted;
  int32_t terminated;
  int32_t termination;
  int32_t iteration;
  int32_t num_successful;
  int32_t pcg_done;
  int32_t pcg_iters;
  int32_t total_pcg;
  int32_t status;          // linear-solve failure of the current step
  int32_t nonfinite;
  int32_t inertial_status;
  int32_t stop_iteration;  // iteration at which cost <= stop_cost (or -1)
  int32_t pad_[2];
};

struct LmParams {
  int32_t max_num_iterations;
  int32_t max_linear_iterations;
  int32_t check_tolerances;
  int32_t pad_;
  double max_radius, min_radius;
  double function_tolerance, parameter_tolerance, min_relative_decrease;
  double min_lm_diagonal, max_lm_diagonal;
  double linear_tolerance;
  double stop_cost;
};

template <typename T>
struct LinearSystem {
  T* Hll;    // [9][nlm]
  T* gl;     // [3][nlm]
  T* Wslot;  // [nslot][18] slot-major
  T* Dbase;  // [nkf][225]
  T* Pbase;  // [npu][36]
  T* Ebase;  // [nedge][225]
  T* gc;     // [nkf][15]
  T* SD;     // [nkf][225]
  T* SP;     // [2 npu][36]
  T* SE;     // [nedge][225]
  T* rhs;    // [nkf*15]
  T* V;      // [9][nlm]
  T* U;      // [nslot][18] slot-major
  T* Minv;       // [nkf][225] block-Jacobi inverses (factorized and inverted in FP64)
  T *x, *r, *z, *p, *q, *q2;  // [nkf*15]; p and q2 double-buffer the PCG direction
  double* dl;    // [3][nlm] scaled landmark step
  T* skf;        // [nkf*15] Jacobi scale (T copy)
  T* slm;        // [3][nlm]
};

struct ScaleVectors {
  double* skf;  // [nkf*15]
  double* slm;  // [3][nlm]
};

template <typename T>
struct SolverLaunch {
  DevProblem P;
  SchurPattern S;
  LinearSystem<T> L;
  VisualLin<T> vis;
  InertialLin<T> ine;
  ScaleVectors sc;
  LmControl* ctl;
  LmParams prm;
  mba_iteration_summary* log;  // device [max_num_iterations + 1]
  double* kf_cand;             // [nkf][16]
  double* lm_cand;             // [nlm][4]
};

// kernels_solver.cu
template <typename T>
cudaError_t solver_assemble(const SolverLaunch<T>& s, const int* gate, cudaStream_t st);
template <typename T>
cudaError_t solver_compute_scale(const SolverLaunch<T>& s, int jacobi, cudaStream_t st);
template <typename T>
cudaError_t solver_step(const SolverLaunch<T>& s, cudaStream_t st);
template <typename T>
cudaError_t solver_evaluate_candidate(const SolverLaunch<T>& s, InertialLin<double> ine_cand, cudaStream_t st);
template <typename T>
cudaError_t solver_decide_and_accept(const SolverLaunch<T>& s, InertialLin<double> ine_cand,
                                     InertialLin<double> ine_cur, cudaStream_t st);
template <typename T>
cudaError_t solver_relinearize(const SolverLaunch<T>& s, const InertialLin<double>& ine_cur, cudaStream_t st);
cudaError_t solver_init_control(LmControl* ctl, double radius, cudaStream_t st);

}  // namespace mba
