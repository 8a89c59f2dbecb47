// CPU ORACLE — test infrastructure only (see oracle.h).
// extern "C" surface loaded by tests/ and bench.py (CPU baseline) via ctypes.
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle.h"

namespace oracle {
struct Problem;
int createProblem(const mba_problem_desc* d, Problem** out);
void evaluateVisualAmbient(const Problem& p, double* res, double* const* jac);
int evaluateInertialAmbient(const Problem& p, double* res, double* const* jac);
struct Linearization;
int solve(Problem& p, const mba_solver_options& o, mba_summary* sum);
int reducedSystemDense(Problem& p, const mba_solver_options& o, double radius, double* A, double* b);
}  // namespace oracle

// Access helpers defined in solver.cc's translation unit are kept private; the
// problem object is opaque to callers.
namespace oracle {
int oracleLinearizeVisual(Problem* p, double* r, double* Jl, double* Js, double* Jo, double* cost);
int oracleLinearizePoseEdges(Problem* p, double* r, double* Jf, double* Jt);
int oracleReadState(Problem* p, double* kx, double* kv, double* kbg, double* kba, double* lp);
int oracleReadCalibration(Problem* p, mba_camera* cams, double* mis);
int oracleReadSwitches(Problem* p, double* s);
int oracleLandmarkQuality(Problem* p, const mba_landmark_quality_options* o, uint8_t* good);
int oracleWriteState(Problem* p, const double* kx, const double* kv, const double* kbg, const double* kba, const double* lp);
void oracleDestroy(Problem* p);
void oracleSetThreads(Problem* p, int t);
double oracleTimeVisual(Problem* p, int threads, int64_t sample, int reps);
}  // namespace oracle

extern "C" {

int oracle_create(const mba_problem_desc* d, void** out) {
  oracle::Problem* p = nullptr;
  const int st = oracle::createProblem(d, &p);
  *out = p;
  return st;
}
void oracle_destroy(void* h) { oracle::oracleDestroy((oracle::Problem*)h); }
void oracle_set_threads(void* h, int t) { oracle::oracleSetThreads((oracle::Problem*)h, t); }

int oracle_evaluate_visual(void* h, double* res, double* const* jac) {
  oracle::evaluateVisualAmbient(*(oracle::Problem*)h, res, jac);
  return 0;
}
int oracle_evaluate_inertial(void* h, double* res, double* const* jac) {
  return oracle::evaluateInertialAmbient(*(oracle::Problem*)h, res, jac);
}
int oracle_linearize_visual(void* h, double* r, double* Jl, double* Js, double* Jo, double* cost) {
  return oracle::oracleLinearizeVisual((oracle::Problem*)h, r, Jl, Js, Jo, cost);
}
int oracle_solve(void* h, const mba_solver_options* o, mba_summary* s) {
  return oracle::solve(*(oracle::Problem*)h, *o, s);
}
int oracle_reduced_system(void* h, const mba_solver_options* o, double radius, double* A, double* b) {
  return oracle::reducedSystemDense(*(oracle::Problem*)h, *o, radius, A, b);
}
int oracle_linearize_pose_edges(void* h, double* r, double* Jf, double* Jt) {
  return oracle::oracleLinearizePoseEdges((oracle::Problem*)h, r, Jf, Jt);
}
// One relative pose term: residual [6] and ambient Jacobians [6][7] (q, p) of
// both keyframe blocks; cov [36] (p, q order).  Returns 0, or 1 if cov is not
// positive definite.
int oracle_pose_edge(const double* xk, const double* xk1, const double* ext, const double* meas, const double* cov,
                     double* r, double* Jk, double* Jk1) {
  double M[36];
  if (!oracle::poseEdgeSqrtInfo(cov, M)) return 1;
  oracle::poseEdgeEvaluate(xk, xk1, ext, meas, M, r, Jk, Jk1);
  return 0;
}
int oracle_read_switches(void* h, double* s) { return oracle::oracleReadSwitches((oracle::Problem*)h, s); }
int oracle_landmark_quality(void* h, const mba_landmark_quality_options* o, uint8_t* good) {
  return oracle::oracleLandmarkQuality((oracle::Problem*)h, o, good);
}
// One loop-closure term without its switch (baseframes, vertex blocks,
// measurement q_AB JPL | p_AB, covariance): residual [6], ambient Jacobians.
int oracle_loop_closure(const double* bfA, const double* bfB, const double* xA, const double* xB, const double* meas,
                        const double* cov, double* r, double* JA, double* JB) {
  double M[36];
  if (!oracle::poseEdgeSqrtInfo(cov, M)) return 1;
  oracle::loopClosureEvaluate(bfA, bfB, xA, xB, meas, M, r, JA, JB);
  return 0;
}
// One absolute pose term (baseframe, vertex block, sensor extrinsics q_S_B |
// p_S_B, measurement q_S_G Hamilton | p_G_S, covariance).
int oracle_absolute_pose(const double* bf, const double* x, const double* ext, const double* meas, const double* cov,
                         double* r, double* J) {
  double M[36];
  if (!oracle::poseEdgeSqrtInfo(cov, M)) return 1;
  oracle::absolutePoseEvaluate(bf, x, ext, meas, M, r, J);
  return 0;
}
int oracle_read_state(void* h, double* kx, double* kv, double* kbg, double* kba, double* lp) {
  return oracle::oracleReadState((oracle::Problem*)h, kx, kv, kbg, kba, lp);
}
int oracle_read_calibration(void* h, mba_camera* cams, double* mis) {
  return oracle::oracleReadCalibration((oracle::Problem*)h, cams, mis);
}
int oracle_write_state(void* h, const double* kx, const double* kv, const double* kbg, const double* kba,
                       const double* lp) {
  return oracle::oracleWriteState((oracle::Problem*)h, kx, kv, kbg, kba, lp);
}
// Mean seconds per pass of the robustified tangent linearization of `sample`
// visual observations on `threads` host threads (CPU baseline).
double oracle_time_visual(void* h, int threads, int64_t sample, int reps) {
  return oracle::oracleTimeVisual((oracle::Problem*)h, threads, sample, reps);
}

// ---- single-term entry points (golden / known-answer tests)
void oracle_imu_integrate(const double* noise5, const double* state16, const double* readings12, double dt,
                          double* next16, double* phi, double* cov) {
  const oracle::ImuNoise n{noise5[0], noise5[1], noise5[2], noise5[3], noise5[4]};
  oracle::imuIntegrate(n, state16, readings12, dt, next16, phi, cov);
}
void oracle_quat_jacobian(const double* q, double* J43) { oracle::jplQuaternionJacobian(q, J43); }
void oracle_quat_plus(const double* q, const double* d, double* out) { oracle::jplQuaternionPlus(q, d, out); }
void oracle_yaw_plus(const double* q, const double* d, double* out) { oracle::jplYawPlus(q, d, out); }
void oracle_yaw_jacobian(const double* q, double* J) { oracle::jplYawJacobian(q, J); }
void oracle_rollpitch_plus(const double* qGM, const double* q, const double* d, double* out) {
  oracle::jplRollPitchPlus(qGM, q, d, out);
}
void oracle_rollpitch_jacobian(const double* qGM, const double* q, double* J) {
  oracle::jplRollPitchJacobian(qGM, q, J);
}
void oracle_rotation_matrix(const double* q, double* R) { oracle::toRotationMatrixJPL(q, R); }
int oracle_visual_term(const double* const* params, const double* meas, double sigma, int type,
                       const mba_camera* cam, double* residual, double** jac, int* failed) {
  bool f = false;
  oracle::visualEvaluate(params, meas, sigma, type, *cam, residual, jac, &f);
  if (failed) *failed = f ? 1 : 0;
  return 0;
}
int oracle_inertial_term(const double* noise5, const double* const* params, int ns, const int64_t* ts,
                         const double* imu6, double* res, double** jac) {
  const oracle::ImuNoise n{noise5[0], noise5[1], noise5[2], noise5[3], noise5[4]};
  return oracle::inertialEvaluate(n, params, ns, ts, imu6, res, jac);
}
int oracle_project(const mba_camera* cam, const double* p_C, double* kp, double* Jp, double* Ji, double* Jd) {
  return oracle::pinholeProject3(*cam, p_C, kp, Jp, Ji, Jd);
}

}  // extern "C"
