// Device-resident Levenberg-Marquardt solver state (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gnn.h"
#include "internal.h"

namespace mba {

// Slot pairs per thread of the Schur pair kernel (a target with more pairs
// is split into several chunks that add atomically).
constexpr int64_t kSchurChunk = 16;

// Static sparsity of the reduced camera system, built on the host at create.
// Landmark slot rows (W and U, 18 values: 3 x 6) are padded to 20 values so
// that every row starts on a 16-byte boundary (vector loads).
constexpr int kSlotStride = 20;

struct SchurPattern {
  int64_t nslot = 0;      // landmark slots: slot 0 = store keyframe, then one per non-keyframe observation
  int64_t npu = 0;        // upper (i < j) pose-pose 6x6 blocks
  int64_t npair = 0;      // Schur slot pairs (a <= b) within a landmark
  int64_t* lm_slot_off;   // [nlm] first W slot of each landmark (W rows numbered by landmark)
  int64_t* lm_slot_end;   // [nlm] one past its last W slot
  int32_t* w_u;           // [nslot] U row of each W slot (U rows numbered by store keyframe)
  int32_t* u_w;           // [nslot] W slot of each U row
  int32_t* slot_kf;       // [nslot]
  int32_t* slot_lm;       // [nslot]
  int32_t* obs_slot;      // [nobs] slot of the observer, -1 for kLocalKeyframe
  int32_t* obs_pblk;      // [nobs] upper block of (store, observer), -1 for kLocalKeyframe
  int64_t nchunk = 0;     // pair chunks (contiguous pair ranges of one target)
  int2* pair_rb;          // [npair] (a as position in its row's W slot list, b as U row, bitwise-not
                          //   of it when b is a itself), sorted by target; slot_kf[a] <= slot_kf[b]
  int64_t* kf_slot_off;   // [nkf+1] keyframe-major slot lists (a row's W slots are staged from them)
  int32_t* kf_slot;       // [nslot]
  int64_t max_row_slots = 0;
  int64_t* row_chunk_off; // [nkf+1] chunks of the targets of keyframe row i
  int32_t* chunk_tgt;     // [nchunk] target id (kf for diagonal, nkf + upper block);
                          //   bitwise-not of it when the target spans several chunks
  int64_t* chunk_beg;     // [nchunk] first pair of each chunk (grouped by row; by length within a row)
  int32_t* chunk_len;     // [nchunk] pairs in the chunk
  int32_t* pu_i;          // [npu]
  int32_t* pu_j;
  int64_t* row_off;       // [nkf+1] full (both orientations) pose-pose rows
  int32_t* row_col;       // [2 npu]
  int32_t* row_blk;       // [2 npu] block index into SP (upper b -> b, lower -> npu + b)
  int64_t* up_off;        // [nkf+1] upper pose-pose blocks (i < j) by row i
  int32_t* up_col;        // [npu] j
  int32_t* up_blk;        // [npu] block index into SP
  int64_t* kfe_off;       // [nkf+1] incident inertial edges
  int32_t* kfe;           // +(e+1): keyframe is 'from' ; -(e+1): keyframe is 'to'
  // Keyframe chains laid end to end (chain preconditioner): position -> kf,
  // and the blocks coupling position p to p - 1 (-1 where absent):
  // link_edge = inertial edge whose SE block is (kf(p-1), kf(p)); link_blk =
  // SP block with rows kf(p), columns kf(p-1).
  int32_t* chain_perm;    // [nkf]
  int32_t* link_edge;     // [nkf]
  int32_t* link_blk;      // [nkf]
  int32_t chain_levels = 0;  // cyclic-reduction levels, 2^levels >= nkf
  int32_t chain_tail = 0;    // first level handled by the single-block tail sweep
  int32_t chain_seg = 0;     // segmented sweeps: log2 of the positions one block sweeps through the
                             // levels below it (0: one launch per level)
  int32_t chain_tail_sm = 0;  // 1: one-block tail with the survivors' vectors in shared memory
  int32_t spmv_sym = 0;       // 1: PCG product reads each stored pose block once (transposed part by atomics)
  int32_t schur_split = 0;    // 1: Schur pair kernel with two threads per chunk
};

// Device control block of the LM loop (all scalars live on the device).
struct LmControl {
  double cost;
  double cost_cand;        // visual part of the candidate cost
  double cost_ine;         // inertial part of `cost`
  double cost_cand_ine;    // inertial part of the candidate cost
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
  int32_t chain_failed;    // chain factorization hit a non-SPD pivot: PCG falls back to block-Jacobi
  int32_t rejected;        // landmarks rejected as outliers during this solve
  int32_t reject_count;    // landmarks rejected by the last outlier pass
  int32_t restart_now;     // set by the LM decision: outlier rejection + restart after this iteration
  int32_t loop_active;     // device-driven LM loop: 1 while another iteration follows
  int32_t fatal;           // a bounded device wait ran out (tensor-core pipeline): the solve fails with MBA_ERR_TIMEOUT
  unsigned long long grad_max_bits;  // max |J^T r| over the variable dims (bits of a non-negative double)
  unsigned long long t0_ns;  // device global timer at the start of the solve
};

struct LmParams {
  int32_t max_num_iterations;
  int32_t max_linear_iterations;
  int32_t check_tolerances;
  int32_t reject_every;    // outlier rejection + restart every n iterations (0: off)
  double max_radius, min_radius;
  double function_tolerance, parameter_tolerance, min_relative_decrease;
  double min_lm_diagonal, max_lm_diagonal;
  double linear_tolerance;
  double stop_cost;
  double gradient_tolerance;  // with check_tolerances: stop once max |J^T r| <= it
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
  // Switch variables, eliminated like landmarks (1-dim blocks, each touching
  // one edge's two keyframes): J^T J and gradient (scaled in place), W_f | W_t
  // (scaled Jacobian columns of the keyframes times the switch column), the
  // damped inverse, the scaled step.
  // FP32 path: the visual terms' 6x6 pose blocks of D and their gradient,
  // accumulated with 16-byte vector atomics and merged into Dbase / gc.
  float* Dpose;  // [nkf][24]: upper triangle of the visual pose block (21 used)
  float* gpose;  // [nkf][8] (6 used)
  T* swH;        // [nsw]
  T* swg;        // [nsw]
  T* swW;        // [nsw][30]
  T* swHi;       // [nsw]
  double* swx;   // [nsw]
  T* ssw;        // [nsw] Jacobi scale (T copy)
};

// Block cyclic reduction of the chain matrix T (block-tridiagonal in chain
// positions): T_pp = S_kk + alpha_p diag(off-chain |S| row sums, pose rows),
// T_{p,p-1} = gamma_ine,p E + gamma_vis,p P (inertial / visual coupling).
// Position p (> 0) is eliminated at level ctz(p); position 0 last.
template <typename T>
struct ChainSystem {
  double* A;     // [n][225] diagonal blocks of the current level
  double* B;     // [n][225] coupling to the left neighbour of the current level
  double* F64;   // [n][225] inverse of the eliminated diagonal block
  double* CL64;  // [n][225] T(p, p - s) at elimination
  double* CR64;  // [n][225] T(p, p + s)
  double* XL64;  // [n][225] T(p - s, p) F(p)
  double* XR64;  // [n][225] T(p + s, p) F(p)
  T *F, *CL, *CR, *XL, *XR;  // working-precision copies read by the sweeps
  T* w;          // [n*15] forward-sweep vector (position order)
  T* lc;         // [n*15] segmented sweeps: left-neighbour terms of each segment's first position
  double* coef;  // [n][3] gamma_ine, gamma_vis (link p -> p-1), alpha (node p)
  double* comp;  // [n][6] off-chain |S| row sums of the pose rows (alpha's direction)
};

struct ScaleVectors {
  double* skf;  // [(nkf + ng)*15]: keyframe dims, then the global nodes' dims
  double* slm;  // [3][nlm]
  double* ssw;  // [nsw]
};

// Reduced-system blocks of the global nodes (calibration / baseframe
// variables; FP64 solves only).  Node g is block nkf + g of the PCG vectors
// and of SD / Minv; its couplings are stored dense.
struct BorderSystem {
  double* Gb;            // [ng][ng][225] node-node J^T J (unscaled, both orientations)
  double* Bb;            // [nkf][ng][90] keyframe pose rows (6) x node dims (15), J^T J (unscaled)
  double* gg;            // [ng][15] node gradient J^T r (unscaled)
  double* GS;            // [ng][ng][225] scaled, damped, landmark-reduced node blocks
  double* BS;            // [nkf][ng][90] scaled, landmark-reduced keyframe-node blocks
  double* bl;            // [3][nlm] W_n^T x_n per landmark (back substitution)
  DevCamera* cams_cand;  // [ncam] candidate cameras (retraction)
  double* mis_cand;      // [nmis][8] candidate baseframes
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
  float* kf_cand_f;            // [nkf][8] FP32 pose copies of the candidate (mixed path)
  float* lm_cand_f;            // [nlm][4]
  double* sw_cand;             // [nsw] candidate switch variables
  ChainSystem<T> C;
  int32_t precond = 0;         // MBA_PRECOND_*
  GnnGraph gg{};               // learned preconditioner (precond == MBA_PRECOND_LEARNED)
  GnnParams gp{};
  GnnWork gw{};
  BorderSystem B{};            // global nodes (P.ng > 0, FP64 only)
};

// kernels_solver.cu
template <typename T>
cudaError_t solver_assemble(const SolverLaunch<T>& s, const int* gate, cudaStream_t st);
template <typename T>
cudaError_t solver_compute_scale(const SolverLaunch<T>& s, int jacobi, cudaStream_t st);
// Damped reduced camera system (build + Schur + masks) and the block-Jacobi
// inverses, at the radius held in the control block.
template <typename T>
cudaError_t solver_build_reduced(const SolverLaunch<T>& s, cudaStream_t st);
// Per-problem launch preparation (shared-memory opt-in of the Schur pair
// kernel); call before the solver's kernels are launched or captured.
template <typename T>
cudaError_t solver_prepare(const SchurPattern& S);
template <typename T>
cudaError_t chain_prepare();
template <typename T>
cudaError_t solver_product(const SolverLaunch<T>& s, bool sym, cudaStream_t st);
// The Schur pair kernel alone (autotuning).
template <typename T>
cudaError_t solver_schur_pairs(const SolverLaunch<T>& s, cudaStream_t st);
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
// cost += cost_ine (after the initial visual and inertial evaluations).
cudaError_t solver_add_inertial_cost(LmControl* ctl, cudaStream_t st);
// Outlier rejection and restart at the current state (the Ceres solve that
// maplab restarts every n iterations): rejects outlier landmarks, recomputes
// the cost, the visual linearization, the assembly and the Jacobi scaling;
// keeps the trust-region radius and resets the decrease factor.
template <typename T>
cudaError_t solver_reject_and_restart(const SolverLaunch<T>& s, int use_reprojection, double max_px, int jacobi,
                                      cudaStream_t st);
// Device-driven loop: records the solve's start time; ends the loop (and
// reports cancellation) through the conditional handle.
cudaError_t solver_loop_start(LmControl* ctl, cudaStream_t st);
cudaError_t solver_loop_control(LmControl* ctl, cudaGraphConditionalHandle handle, const volatile int* cancel,
                                cudaStream_t st);

// Max |J^T r| over the variable dims (after an assembly) into ctl->grad_max_bits;
// with check_tolerances, a value at or below gradient_tolerance ends the solve
// (termination 2) when `run_if` is set (NULL: always).
template <typename T>
cudaError_t solver_gradient_check(const SolverLaunch<T>& s, const int* run_if, cudaStream_t st);

// kernels_border.cu: the global nodes (calibration / baseframe variables) of
// FP64 solves.  border_assemble zeroes and re-assembles the direct node
// terms of the current linearization; border_scale sets the nodes' Jacobi
// scale (first linearization); border_build / border_schur_and_finalize
// form the node blocks of the reduced system around the landmark
// elimination; border_spmv is the node rows' PCG product (after
// k_pcg_spmv); border_backsub the node part of the landmark back
// substitution; border_model_visual the visual model cost change with the
// node columns; border_retract / border_accept move the candidate cameras and
// baseframes.
cudaError_t border_assemble(const SolverLaunch<double>& s, const int* run_if, const int* skip_if, cudaStream_t st);
cudaError_t border_scale(const SolverLaunch<double>& s, int jacobi, const int* run_if, cudaStream_t st);
cudaError_t border_build(const SolverLaunch<double>& s, cudaStream_t st);
cudaError_t border_schur_and_finalize(const SolverLaunch<double>& s, cudaStream_t st);
cudaError_t border_spmv(const SolverLaunch<double>& s, int it, const double* pa, double* pb, cudaStream_t st);
cudaError_t border_backsub(const SolverLaunch<double>& s, cudaStream_t st);
cudaError_t border_model_visual(const SolverLaunch<double>& s, cudaStream_t st);
cudaError_t border_retract(const SolverLaunch<double>& s, cudaStream_t st);
cudaError_t border_accept(const SolverLaunch<double>& s, cudaStream_t st);

// kernels_chain.cu: factorization of the chain matrix (after the reduced
// system is built) and z = T^-1 r with the r.z dot added to *rz.
template <typename T>
cudaError_t chain_factor(const SolverLaunch<T>& s, cudaStream_t st);
template <typename T>
cudaError_t chain_apply(const SolverLaunch<T>& s, const T* r, T* z, double* rz, cudaStream_t st);
// Fixed coefficients of the untrained chain preconditioner (gamma = 1, alpha = 0).
cudaError_t chain_default_coef(double* coef, int64_t n, cudaStream_t st);

// kernels_gnn.cu: the coefficient network.
cudaError_t gnn_init_params(GnnParams p, uint64_t seed, cudaStream_t st);
cudaError_t gnn_sync_bf16(GnnParams p, cudaStream_t st);
// Features, forward pass and chain coefficients (s.C.coef) for the reduced
// system held in s.L.
template <typename T>
cudaError_t gnn_forward(const SolverLaunch<T>& s, GnnGraph g, GnnParams p, GnnWork w, cudaStream_t st);
// Probe loss mean |T^-1 S w - w|^2 over nprobe probes (device `probes`
// [nprobe][15 n] if given, else seeded normal draws) into w.loss, and its
// gradient into p.g.  Needs the chain factorization of the current coef.
template <typename T>
cudaError_t gnn_loss_backward(const SolverLaunch<T>& s, GnnGraph g, GnnParams p, GnnWork w, int nprobe,
                              const float* probes, uint64_t seed, cudaStream_t st);
cudaError_t gnn_adam(GnnParams p, float lr, cudaStream_t st);

}  // namespace mba
