// Seeded synthetic visual-inertial maps (host C++, no CUDA).  See
// include/maplab_ba_synth.h for the reference recipe this restates.
#include <algorithm>
#include <array>
#include <functional>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <random>
#include <vector>

#include "../../include/maplab_ba_synth.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

// Deterministic across x86_64 and aarch64: mt19937 words -> Box-Muller.
struct Rng {
  std::mt19937 mt;
  bool has_spare = false;
  double spare = 0.0;
  explicit Rng(uint64_t seed) : mt(static_cast<uint32_t>(seed ^ (seed >> 32))) {}
  double uniform() { return (static_cast<double>(mt()) + 0.5) * (1.0 / 4294967296.0); }
  double normal() {
    if (has_spare) { has_spare = false; return spare; }
    const double u1 = uniform(), u2 = uniform();
    const double r = std::sqrt(-2.0 * std::log(u1));
    spare = r * std::sin(2.0 * kPi * u2);
    has_spare = true;
    return r * std::cos(2.0 * kPi * u2);
  }
  int64_t below(int64_t n) { return std::min<int64_t>(n - 1, static_cast<int64_t>(uniform() * n)); }
};

struct Mat3 { double m[9]; };
Mat3 mul(const Mat3& a, const Mat3& b) {
  Mat3 c;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) c.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
  return c;
}
Mat3 tr(const Mat3& a) { return Mat3{{a.m[0], a.m[3], a.m[6], a.m[1], a.m[4], a.m[7], a.m[2], a.m[5], a.m[8]}}; }
void mv(const Mat3& a, const double* x, double* y) {
  const double t0 = a.m[0] * x[0] + a.m[1] * x[1] + a.m[2] * x[2];
  const double t1 = a.m[3] * x[0] + a.m[4] * x[1] + a.m[5] * x[2];
  const double t2 = a.m[6] * x[0] + a.m[7] * x[1] + a.m[8] * x[2];
  y[0] = t0; y[1] = t1; y[2] = t2;
}
Mat3 rotX(double a) { const double c = std::cos(a), s = std::sin(a); return Mat3{{1, 0, 0, 0, c, -s, 0, s, c}}; }
Mat3 rotY(double a) { const double c = std::cos(a), s = std::sin(a); return Mat3{{c, 0, s, 0, 1, 0, -s, 0, c}}; }
Mat3 rotZ(double a) { const double c = std::cos(a), s = std::sin(a); return Mat3{{c, -s, 0, s, c, 0, 0, 0, 1}}; }

// JPL rotation matrix of q (xyzw), R = toRotationMatrixJPL(q).
Mat3 jplR(const double* q) {
  return Mat3{{1.0 - 2.0 * (q[1] * q[1] + q[2] * q[2]), 2.0 * (q[0] * q[1] + q[2] * q[3]), 2.0 * (q[0] * q[2] - q[1] * q[3]),
               2.0 * (q[0] * q[1] - q[2] * q[3]), 1.0 - 2.0 * (q[0] * q[0] + q[2] * q[2]), 2.0 * (q[1] * q[2] + q[0] * q[3]),
               2.0 * (q[0] * q[2] + q[1] * q[3]), 2.0 * (q[1] * q[2] - q[0] * q[3]), 1.0 - 2.0 * (q[0] * q[0] + q[1] * q[1])}};
}
// Quaternion q (xyzw, w >= 0) with jplR(q) == R (Shepperd's method on R^T,
// i.e. the Hamilton quaternion of R^T stored in JPL layout).
void quatFromJplR(const Mat3& R, double* q) {
  const Mat3 A = tr(R);  // Hamilton rotation matrix of the same coefficients
  const double t = A.m[0] + A.m[4] + A.m[8];
  double w, x, y, z;
  if (t > 0.0) {
    const double s = std::sqrt(t + 1.0) * 2.0;
    w = 0.25 * s; x = (A.m[7] - A.m[5]) / s; y = (A.m[2] - A.m[6]) / s; z = (A.m[3] - A.m[1]) / s;
  } else if (A.m[0] > A.m[4] && A.m[0] > A.m[8]) {
    const double s = std::sqrt(1.0 + A.m[0] - A.m[4] - A.m[8]) * 2.0;
    w = (A.m[7] - A.m[5]) / s; x = 0.25 * s; y = (A.m[1] + A.m[3]) / s; z = (A.m[2] + A.m[6]) / s;
  } else if (A.m[4] > A.m[8]) {
    const double s = std::sqrt(1.0 + A.m[4] - A.m[0] - A.m[8]) * 2.0;
    w = (A.m[2] - A.m[6]) / s; x = (A.m[1] + A.m[3]) / s; y = 0.25 * s; z = (A.m[5] + A.m[7]) / s;
  } else {
    const double s = std::sqrt(1.0 + A.m[8] - A.m[0] - A.m[4]) * 2.0;
    w = (A.m[3] - A.m[1]) / s; x = (A.m[2] + A.m[6]) / s; y = (A.m[5] + A.m[7]) / s; z = 0.25 * s;
  }
  if (w < 0.0) { w = -w; x = -x; y = -y; z = -z; }
  const double n = std::sqrt(w * w + x * x + y * y + z * z);
  q[0] = x / n; q[1] = y / n; q[2] = z / n; q[3] = w / n;
}

// Hamilton quaternion (x y z w) algebra for the odometry measurement model.
void hMul(const double* a, const double* b, double* o) {
  o[3] = a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2];
  o[0] = a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1];
  o[1] = a[3] * b[1] - a[0] * b[2] + a[1] * b[3] + a[2] * b[0];
  o[2] = a[3] * b[2] + a[0] * b[1] - a[1] * b[0] + a[2] * b[3];
}
void hRot(const double* q, const double* v, double* o) {
  double uv[3] = {2 * (q[1] * v[2] - q[2] * v[1]), 2 * (q[2] * v[0] - q[0] * v[2]), 2 * (q[0] * v[1] - q[1] * v[0])};
  o[0] = v[0] + q[3] * uv[0] + (q[1] * uv[2] - q[2] * uv[1]);
  o[1] = v[1] + q[3] * uv[1] + (q[2] * uv[0] - q[0] * uv[2]);
  o[2] = v[2] + q[3] * uv[2] + (q[0] * uv[1] - q[1] * uv[0]);
}
// Transformations (q, p): x -> R(q) x + p.
void tMul(const double* A, const double* B, double* O) {
  hMul(A, B, O);
  double r[3];
  hRot(A, B + 4, r);
  for (int i = 0; i < 3; ++i) O[4 + i] = r[i] + A[4 + i];
}
void tInv(const double* A, double* O) {
  O[0] = -A[0]; O[1] = -A[1]; O[2] = -A[2]; O[3] = A[3];
  double r[3];
  hRot(O, A + 4, r);
  for (int i = 0; i < 3; ++i) O[4 + i] = -r[i];
}
void odometryFromStates(const double* xa, const double* xb, const double* ext, double* T) {
  const double TBI[7] = {-ext[0], -ext[1], -ext[2], ext[3], ext[4], ext[5], ext[6]};
  double TaI[7], TBIi[7], X[7], Y[7];
  tInv(xa, TaI);
  tInv(TBI, TBIi);
  tMul(TBI, TaI, X);
  tMul(X, xb, Y);
  tMul(Y, TBIi, T);
}
void hamiltonPerturb(double* T, const double* d) {
  const double th = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const double s = th > 0 ? std::sin(0.5 * th) / th : 0.5;
  const double dq[4] = {s * d[0], s * d[1], s * d[2], std::cos(0.5 * th)};
  double q[4];
  hMul(T, dq, q);
  for (int i = 0; i < 4; ++i) T[i] = q[i];
}
// JPL quaternion product (left-multiplication matrix of a times b),
// normalized with w >= 0.
void jplProd(const double* a, const double* b, double* o) {
  double p[4];
  p[0] = a[3] * b[0] + a[2] * b[1] - a[1] * b[2] + a[0] * b[3];
  p[1] = -a[2] * b[0] + a[3] * b[1] + a[0] * b[2] + a[1] * b[3];
  p[2] = a[1] * b[0] - a[0] * b[1] + a[3] * b[2] + a[2] * b[3];
  p[3] = -a[0] * b[0] - a[1] * b[1] - a[2] * b[2] + a[3] * b[3];
  const double n = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3]);
  const double sgn = p[3] < 0 ? -1.0 : 1.0;
  for (int i = 0; i < 4; ++i) o[i] = sgn * p[i] / n;
}
// Relative pose T_A_B (Hamilton q | p) of vertex blocks xa, xb (q_I_M JPL |
// p_M_I) in missions with baseframes ba, bb (q_G_M JPL | p_G_M): the
// measurement model of LoopClosureEdgeErrorTerm.
void loopClosureFromStates(const double* ba, const double* xa, const double* bb, const double* xb, double* T) {
  double qi[4], qGA[4], qGB[4], qAB[4], pGA[3], pGB[3];
  qi[0] = -xa[0]; qi[1] = -xa[1]; qi[2] = -xa[2]; qi[3] = xa[3];
  jplProd(ba, qi, qGA);
  qi[0] = -xb[0]; qi[1] = -xb[1]; qi[2] = -xb[2]; qi[3] = xb[3];
  jplProd(bb, qi, qGB);
  mv(jplR(ba), xa + 4, pGA);
  mv(jplR(bb), xb + 4, pGB);
  for (int i = 0; i < 3; ++i) { pGA[i] += ba[4 + i]; pGB[i] += bb[4 + i]; }
  qi[0] = -qGA[0]; qi[1] = -qGA[1]; qi[2] = -qGA[2]; qi[3] = qGA[3];
  jplProd(qi, qGB, qAB);
  const double d[3] = {pGB[0] - pGA[0], pGB[1] - pGA[1], pGB[2] - pGA[2]};
  mv(jplR(qi), d, T + 4);
  T[0] = -qAB[0]; T[1] = -qAB[1]; T[2] = -qAB[2]; T[3] = qAB[3];  // Hamilton coefficients
}
// Sensor pose T_G_S (Hamilton q | p) of vertex block x in a mission with
// baseframe b, sensor extrinsics ext = q_S_B (JPL) | p_S_B: the measurement
// model of BlockPosePriorErrorTermV2.
void absolutePoseFromState(const double* b, const double* x, const double* ext, double* T) {
  const Mat3 RGM = jplR(b), RMB = tr(jplR(x)), RBS = tr(jplR(ext));
  const Mat3 A = mul(RGM, RMB), RGS = mul(A, RBS);
  double pBS[3], a[3], c[3];
  mv(RBS, ext + 4, pBS);
  for (int i = 0; i < 3; ++i) pBS[i] = -pBS[i];
  mv(A, pBS, a);
  mv(RGM, x + 4, c);
  for (int i = 0; i < 3; ++i) T[4 + i] = a[i] + c[i] + b[4 + i];
  quatFromJplR(tr(RGS), T);  // Hamilton quaternion of R_G_S
}
// JPL box-plus used only to perturb initial orientations.
void jplPlus(const double* q, const double* d, double* out) {
  const double th = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  double dq[4] = {0, 0, 0, 1};
  if (th > 1e-12) {
    const double s = std::sin(0.5 * th) / th;
    dq[0] = d[0] * s; dq[1] = d[1] * s; dq[2] = d[2] * s; dq[3] = std::cos(0.5 * th);
  }
  double p[4];
  p[0] = dq[3] * q[0] + dq[2] * q[1] - dq[1] * q[2] + dq[0] * q[3];
  p[1] = -dq[2] * q[0] + dq[3] * q[1] + dq[0] * q[2] + dq[1] * q[3];
  p[2] = dq[1] * q[0] - dq[0] * q[1] + dq[3] * q[2] + dq[2] * q[3];
  p[3] = -dq[0] * q[0] - dq[1] * q[1] - dq[2] * q[2] + dq[3] * q[3];
  const double n = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3]);
  const double sgn = p[3] < 0 ? -1.0 : 1.0;
  for (int i = 0; i < 4; ++i) out[i] = sgn * p[i] / n;
}

// Forward projection (pinhole + distortion) used for visibility and measurements.
bool project(const mba_camera& c, const double* pC, double* kp) {
  if (pC[2] < 0.5) return false;
  double x = pC[0] / pC[2], y = pC[1] / pC[2];
  if (c.distortion_type == MBA_DISTORTION_RADTAN) {
    const double* k = c.distortion;
    const double mx2 = x * x, my2 = y * y, mxy = x * y, r2 = mx2 + my2;
    const double rd = k[0] * r2 + k[1] * r2 * r2;
    const double nx = x + x * rd + 2.0 * k[2] * mxy + k[3] * (r2 + 2.0 * mx2);
    const double ny = y + y * rd + 2.0 * k[3] * mxy + k[2] * (r2 + 2.0 * my2);
    x = nx; y = ny;
  } else if (c.distortion_type == MBA_DISTORTION_EQUIDISTANT) {
    const double* k = c.distortion;
    const double r = std::sqrt(x * x + y * y);
    if (r > 1e-8) {
      const double th = std::atan(r), t2 = th * th;
      const double thd = th * (1 + k[0] * t2 + k[1] * t2 * t2 + k[2] * t2 * t2 * t2 + k[3] * t2 * t2 * t2 * t2);
      x *= thd / r; y *= thd / r;
    }
  }
  kp[0] = c.intrinsics[0] * x + c.intrinsics[2];
  kp[1] = c.intrinsics[1] * y + c.intrinsics[3];
  const double margin = 2.0;
  return kp[0] >= margin && kp[1] >= margin && kp[0] < c.width - margin && kp[1] < c.height - margin;
}

}  // namespace

struct mba_synth_map {
  mba_synth_config cfg{};
  int64_t nkf = 0, nlm = 0, nobs = 0, nmis = 0, ncam = 0, nedge = 0, nsamp = 0;
  std::vector<double> obs_uv, obs_sigma;
  std::vector<int32_t> obs_lm, obs_kf, obs_cam;
  std::vector<double> lm_p, lm_p_true;
  std::vector<int32_t> lm_store;
  std::vector<uint8_t> lm_const;
  std::vector<double> kf_x, kf_v, kf_bg, kf_ba, kf_x_true, kf_v_true, kf_bg_true, kf_ba_true;
  std::vector<int32_t> kf_mis;
  std::vector<uint32_t> kf_flags;
  std::vector<double> mis;
  std::vector<mba_camera> cams;
  std::vector<int32_t> e_from, e_to;
  std::vector<int64_t> e_off, ts;
  std::vector<double> imu;
  std::vector<int32_t> pe_from, pe_to, pe_type;
  std::vector<double> pe_meas, pe_cov, pe_ext, pe_sw, pe_swvar;
  double gravity = 9.81;
};

extern "C" {

void mba_synth_default_config(mba_synth_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->seed = 1;
  c->num_missions = 1;
  c->keyframes_per_mission = 100;
  c->num_landmarks = 2000;
  c->landmark_mode = MBA_SYNTH_LANDMARKS_BOX;
  c->track_model = MBA_SYNTH_TRACK_UNIFORM;
  c->track_min = 2; c->track_max = 8;
  c->track_mean = 8.0; c->track_alpha = 2.2;
  c->num_cameras = 1;
  c->camera0_distortion = MBA_DISTORTION_RADTAN;
  c->camera1_distortion = MBA_DISTORTION_EQUIDISTANT;
  c->radius_m = 20.0;
  c->box_half_xy = 15.0; c->box_half_z = 2.5;
  c->keyframes_per_lap = 100.0;
  c->kf_rate_hz = 10.0; c->imu_rate_hz = 200.0;
  c->pixel_sigma = 1.0;
  c->acc_noise = 0.02; c->gyro_noise = 0.002;
  c->acc_bias_rw = 0.002; c->gyro_bias_rw = 0.0002;
  c->rot_perturb = 0.05; c->pos_perturb = 0.1; c->lm_perturb = 0.2; c->vel_perturb = 0.05;
  c->pose_edges = 0;
  c->pose_edge_sigma_p = 0.02;
  c->pose_edge_sigma_q = 0.005;
  c->loop_closure_sigma_p = 0.05;
  c->loop_closure_sigma_q = 0.01;
  c->loop_closure_switch_variance = 1e-2;
  c->absolute_pose_sigma_p = 0.1;
  c->absolute_pose_sigma_q = 0.02;
  c->include_inertial = 1;
  c->co_registered = 1;
}

mba_status mba_synth_generate(const mba_synth_config* cfg, mba_synth_map** out) {
  if (!cfg || !out || cfg->num_missions <= 0 || cfg->num_cameras < 1 || cfg->num_cameras > 2) return MBA_ERR_INVALID_ARG;
  std::unique_ptr<mba_synth_map> M(new mba_synth_map());
  M->cfg = *cfg;
  Rng rng(cfg->seed);
  const int nm = cfg->num_missions;
  // Keyframes per mission.
  std::vector<int> nk(nm);
  for (int m = 0; m < nm; ++m) {
    if (cfg->kf_min > 0) {
      const double lo = std::log((double)cfg->kf_min), hi = std::log((double)cfg->kf_max);
      nk[m] = std::max(2, (int)std::lround(std::exp(lo + (hi - lo) * rng.uniform())));
    } else {
      nk[m] = cfg->keyframes_per_mission;
    }
    if (nk[m] < 2) return MBA_ERR_INVALID_ARG;
  }
  std::vector<int64_t> kf0(nm + 1, 0);
  for (int m = 0; m < nm; ++m) kf0[m + 1] = kf0[m] + nk[m];
  const int64_t NK = kf0[nm];
  M->nkf = NK; M->nmis = nm;

  // Gravity (common::GravityProvider, Zurich).
  {
    const double phi = 47.22 * kPi / 180.0;
    const double s2 = std::sin(phi) * std::sin(phi), s22 = std::sin(2 * phi) * std::sin(2 * phi);
    M->gravity = 9.780327 * (1 + 0.0053024 * s2 - 0.0000058 * s22) - 3.155 * 1e-7 * 392.0;
  }
  const double g = M->gravity;

  // Cameras: pinhole 752x480, fu=fv=460; camera 1 yawed 25 deg left.
  M->ncam = cfg->num_cameras;
  for (int c = 0; c < cfg->num_cameras; ++c) {
    mba_camera cam;
    std::memset(&cam, 0, sizeof(cam));
    cam.intrinsics[0] = 460.0; cam.intrinsics[1] = 460.0; cam.intrinsics[2] = 376.0; cam.intrinsics[3] = 240.0;
    cam.width = 752; cam.height = 480;
    cam.distortion_type = c == 0 ? cfg->camera0_distortion : cfg->camera1_distortion;
    if (cam.distortion_type == MBA_DISTORTION_RADTAN) {
      cam.distortion[0] = -0.28; cam.distortion[1] = 0.07; cam.distortion[2] = 0.0; cam.distortion[3] = 0.0;
    } else if (cam.distortion_type == MBA_DISTORTION_EQUIDISTANT) {
      cam.distortion[0] = -0.01; cam.distortion[1] = 0.005; cam.distortion[2] = -0.001; cam.distortion[3] = 0.0001;
    }
    // R_I_C: optical axis along I_x, image x along -I_y, image y along -I_z.
    const Mat3 RIC0{{0, 0, 1, -1, 0, 0, 0, -1, 0}};
    const Mat3 RIC = mul(rotZ(c == 0 ? 0.0 : 25.0 * kPi / 180.0), RIC0);
    const Mat3 RCI = tr(RIC);
    quatFromJplR(RCI, cam.q_CI_p_CI);
    const double pIC[3] = {0.1, c == 0 ? 0.0 : 0.05, 0.05};
    double t[3];
    mv(RCI, pIC, t);
    cam.q_CI_p_CI[4] = -t[0]; cam.q_CI_p_CI[5] = -t[1]; cam.q_CI_p_CI[6] = -t[2];
    M->cams.push_back(cam);
  }

  // Baseframes T_G_M: yaw-only (gravity aligned).
  M->mis.resize(7 * nm);
  std::vector<Mat3> R_G_M(nm);
  std::vector<std::array<double, 3>> p_G_M(nm);
  for (int m = 0; m < nm; ++m) {
    const double yaw = 0.1 * m;
    R_G_M[m] = rotZ(yaw);
    p_G_M[m] = {0.5 * m, -0.25 * m, 0.0};
    // q_G_M (JPL) with jplR(q) = R_G_M as used by the visual error term.
    quatFromJplR(R_G_M[m], &M->mis[7 * m]);
    for (int i = 0; i < 3; ++i) M->mis[7 * m + 4 + i] = p_G_M[m][i];
  }

  // Trajectories: IMU pose in G at time t for mission m.
  const double omega = 2.0 * kPi / (cfg->keyframes_per_lap / cfg->kf_rate_hz);
  const double R = cfg->radius_m;
  std::vector<double> phase(nm), zoff(nm);
  for (int m = 0; m < nm; ++m) {
    phase[m] = cfg->co_registered ? 2.0 * kPi * rng.uniform() : 0.0;
    zoff[m] = cfg->co_registered ? 0.3 * (rng.uniform() - 0.5) : 0.0;
  }
  auto poseG = [&](int m, double t, Mat3* RGI, double* p, double* v, double* a) {
    const double psi = omega * t + phase[m];
    const double az = 0.5, wz = 1.3 * omega;
    p[0] = R * std::cos(psi); p[1] = R * std::sin(psi); p[2] = zoff[m] + az * std::sin(wz * t);
    if (v) { v[0] = -R * omega * std::sin(psi); v[1] = R * omega * std::cos(psi); v[2] = az * wz * std::cos(wz * t); }
    if (a) { a[0] = -R * omega * omega * std::cos(psi); a[1] = -R * omega * omega * std::sin(psi); a[2] = -az * wz * wz * std::sin(wz * t); }
    const double yaw = psi + kPi;
    const double roll = 0.05 * std::sin(2.1 * omega * t), pitch = 0.05 * std::sin(1.7 * omega * t + 0.3);
    *RGI = mul(rotZ(yaw), mul(rotY(pitch), rotX(roll)));
  };
  const int spk = (int)std::lround(cfg->imu_rate_hz / cfg->kf_rate_hz);  // IMU intervals per keyframe
  const double dt = 1.0 / cfg->imu_rate_hz;
  const int64_t dt_ns = (int64_t)std::llround(1e9 / cfg->imu_rate_hz);

  M->kf_x.resize(7 * NK); M->kf_v.resize(3 * NK); M->kf_bg.resize(3 * NK); M->kf_ba.resize(3 * NK);
  M->kf_mis.resize(NK); M->kf_flags.assign(NK, 0u);
  std::vector<Mat3> kf_RGI(NK);
  std::vector<std::array<double, 3>> kf_pG(NK);
  for (int m = 0; m < nm; ++m) {
    const Mat3 RMG = tr(R_G_M[m]);
    double bg[3] = {0, 0, 0}, ba[3] = {0, 0, 0};
    const int64_t nsamp_m = (int64_t)(nk[m] - 1) * spk + 1;
    std::vector<double> imu_m(6 * nsamp_m);
    std::vector<double> bg_at(3 * nsamp_m), ba_at(3 * nsamp_m);
    for (int64_t j = 0; j < nsamp_m; ++j) {
      const double t = j * dt;
      Mat3 RGI, Rp, Rm, Rp2, Rm2;
      double p[3], v[3], a[3], tmp[3];
      poseG(m, t, &RGI, p, v, a);
      // Body rates from a 4th-order central difference of R_G_I.
      const double h = 1e-3;
      poseG(m, t + h, &Rp, tmp, nullptr, nullptr);
      poseG(m, t - h, &Rm, tmp, nullptr, nullptr);
      poseG(m, t + 2 * h, &Rp2, tmp, nullptr, nullptr);
      poseG(m, t - 2 * h, &Rm2, tmp, nullptr, nullptr);
      Mat3 Rd;
      for (int i = 0; i < 9; ++i) Rd.m[i] = (-Rp2.m[i] + 8.0 * Rp.m[i] - 8.0 * Rm.m[i] + Rm2.m[i]) / (12.0 * h);
      const Mat3 W = mul(tr(RGI), Rd);
      const double w[3] = {0.5 * (W.m[7] - W.m[5]), 0.5 * (W.m[2] - W.m[6]), 0.5 * (W.m[3] - W.m[1])};
      // Specific force in I (accelerometer): R_I_G (a_G + g e_z).
      const double f[3] = {a[0], a[1], a[2] + g};
      double aI[3];
      mv(tr(RGI), f, aI);
      for (int i = 0; i < 3; ++i) {
        bg_at[3 * j + i] = bg[i];
        ba_at[3 * j + i] = ba[i];
      }
      // 6dof-test-trajectory-gen.cc:180-215: white noise sigma/sqrt(dt), bias walk sigma*sqrt(dt).
      double ng[3], na[3];
      for (int i = 0; i < 3; ++i) ng[i] = rng.normal();
      for (int i = 0; i < 3; ++i) na[i] = rng.normal();
      for (int i = 0; i < 3; ++i) {
        imu_m[6 * j + i] = aI[i] + ba[i] + na[i] * cfg->acc_noise / std::sqrt(dt);
        imu_m[6 * j + 3 + i] = w[i] + bg[i] + ng[i] * cfg->gyro_noise / std::sqrt(dt);
      }
      double wg[3], wa[3];
      for (int i = 0; i < 3; ++i) wg[i] = rng.normal();
      for (int i = 0; i < 3; ++i) wa[i] = rng.normal();
      for (int i = 0; i < 3; ++i) {
        bg[i] += wg[i] * cfg->gyro_bias_rw * std::sqrt(dt);
        ba[i] += wa[i] * cfg->acc_bias_rw * std::sqrt(dt);
      }
    }
    for (int k = 0; k < nk[m]; ++k) {
      const int64_t K = kf0[m] + k;
      const int64_t j = (int64_t)k * spk;
      Mat3 RGI;
      double p[3], v[3], a[3];
      poseG(m, j * dt, &RGI, p, v, a);
      kf_RGI[K] = RGI;
      kf_pG[K] = {p[0], p[1], p[2]};
      const Mat3 RMI = mul(RMG, RGI);
      double* x = &M->kf_x[7 * K];
      quatFromJplR(tr(RMI), x);  // jplR(q) = R_I_M
      double d[3] = {p[0] - p_G_M[m][0], p[1] - p_G_M[m][1], p[2] - p_G_M[m][2]};
      mv(RMG, d, x + 4);
      mv(RMG, v, &M->kf_v[3 * K]);
      for (int i = 0; i < 3; ++i) { M->kf_bg[3 * K + i] = bg_at[3 * j + i]; M->kf_ba[3 * K + i] = ba_at[3 * j + i]; }
      M->kf_mis[K] = m;
    }
    if (cfg->include_inertial) {
      for (int k = 0; k + 1 < nk[m]; ++k) {
        M->e_from.push_back((int32_t)(kf0[m] + k));
        M->e_to.push_back((int32_t)(kf0[m] + k + 1));
        M->e_off.push_back(M->nsamp);
        for (int j = k * spk; j <= (k + 1) * spk; ++j) {
          M->ts.push_back((int64_t)j * dt_ns);
          for (int i = 0; i < 6; ++i) M->imu.push_back(imu_m[6 * j + i]);
          M->nsamp++;
        }
      }
    }
  }
  M->nedge = (int64_t)M->e_from.size();
  M->e_off.push_back(M->nsamp);

  // Camera pose of keyframe K, camera c, in G: p_C = R_C_G (p_G - p_G_C).
  auto camOf = [&](int64_t K, int c, Mat3* RCG, double* pGC) {
    const mba_camera& cam = M->cams[c];
    const Mat3 RCI = jplR(cam.q_CI_p_CI);
    *RCG = mul(RCI, tr(kf_RGI[K]));
    // p_I_C = -R_I_C p_C_I
    double pIC[3];
    mv(tr(RCI), cam.q_CI_p_CI + 4, pIC);
    for (int i = 0; i < 3; ++i) pIC[i] = -pIC[i];
    double t[3];
    mv(kf_RGI[K], pIC, t);
    for (int i = 0; i < 3; ++i) pGC[i] = kf_pG[K][i] + t[i];
  };
  auto visibleIn = [&](int64_t K, int c, const double* pG, double* kp) {
    Mat3 RCG;
    double pGC[3], d[3], pC[3];
    camOf(K, c, &RCG, pGC);
    for (int i = 0; i < 3; ++i) d[i] = pG[i] - pGC[i];
    mv(RCG, d, pC);
    return project(M->cams[c], pC, kp);
  };

  // Track-length sampler.
  std::vector<double> plcdf;
  if (cfg->track_model == MBA_SYNTH_TRACK_POWER_LAW) {
    // p(L) ~ L^-alpha on [max(2, track_min), track_max]
    for (int k = std::max(2, cfg->track_min); k <= cfg->track_max; ++k)
      plcdf.push_back(std::pow((double)k, -cfg->track_alpha));
    std::partial_sum(plcdf.begin(), plcdf.end(), plcdf.begin());
    for (double& v : plcdf) v /= plcdf.back();
  }
  auto sampleTrack = [&]() -> int {
    if (cfg->track_model == MBA_SYNTH_TRACK_UNIFORM)
      return cfg->track_min + (int)rng.below(cfg->track_max - cfg->track_min + 1);
    if (cfg->track_model == MBA_SYNTH_TRACK_GEOMETRIC) {
      const double p = 1.0 / cfg->track_mean;
      const int L = 1 + (int)std::floor(std::log(rng.uniform()) / std::log(1.0 - p));
      return std::min(std::max(L, 2), cfg->track_max);
    }
    const double u = rng.uniform();
    return std::max(2, cfg->track_min) + (int)(std::lower_bound(plcdf.begin(), plcdf.end(), u) - plcdf.begin());
  };

  const int64_t NL = cfg->landmarks_per_keyframe > 0 ? (int64_t)cfg->landmarks_per_keyframe * NK : cfg->num_landmarks;
  M->lm_p.reserve(3 * NL); M->lm_store.reserve(NL);
  std::vector<int32_t> track;
  std::vector<std::array<double, 2>> kps;
  std::vector<int> vis;
  int64_t lm = 0;
  int64_t attempts = 0;
  while (lm < NL && attempts < 50 * NL + 1000) {
    ++attempts;
    double pG[3];
    int m = 0, c = 0;
    track.clear(); kps.clear();
    const int L = sampleTrack();
    if (cfg->landmark_mode == MBA_SYNTH_LANDMARKS_BOX) {
      m = (int)rng.below(nm);
      c = cfg->camera_per_mission ? m % cfg->num_cameras : (int)rng.below(cfg->num_cameras);
      pG[0] = cfg->box_half_xy * (2 * rng.uniform() - 1);
      pG[1] = cfg->box_half_xy * (2 * rng.uniform() - 1);
      pG[2] = cfg->box_half_z * (2 * rng.uniform() - 1);
      vis.clear();
      for (int k = 0; k < nk[m]; ++k) {
        double kp[2];
        if (visibleIn(kf0[m] + k, c, pG, kp)) vis.push_back(k);
      }
      if ((int)vis.size() < 2) continue;
      const int n = std::min<int>(L, (int)vis.size());
      const int s = (int)rng.below((int)vis.size() - n + 1);
      for (int a = 0; a < n; ++a) track.push_back((int32_t)(kf0[m] + vis[s + a]));
    } else {
      // Pick a keyframe uniformly, a camera, a point in its frustum.
      const int64_t K = rng.below(NK);
      m = M->kf_mis[K];
      c = cfg->camera_per_mission ? m % cfg->num_cameras : (int)rng.below(cfg->num_cameras);
      const double depth = 4.0 + 26.0 * rng.uniform();
      const double u = 0.8 * (2 * rng.uniform() - 1), v = 0.5 * (2 * rng.uniform() - 1);
      const double pC[3] = {u * depth, v * depth, depth};
      Mat3 RCG;
      double pGC[3], t[3];
      camOf(K, c, &RCG, pGC);
      mv(tr(RCG), pC, t);
      for (int i = 0; i < 3; ++i) pG[i] = pGC[i] + t[i];
      for (int64_t k = K; k < kf0[m + 1] && (int)track.size() < L; ++k) {
        double kp[2];
        if (!visibleIn(k, c, pG, kp)) break;
        track.push_back((int32_t)k);
      }
      if ((int)track.size() < 2) continue;
    }
    // Measurements.
    const int64_t store = track[0];
    for (int32_t K : track) {
      double kp[2];
      visibleIn(K, c, pG, kp);
      M->obs_uv.push_back(kp[0] + cfg->pixel_sigma * rng.normal());
      M->obs_uv.push_back(kp[1] + cfg->pixel_sigma * rng.normal());
      M->obs_sigma.push_back(cfg->pixel_sigma);
      M->obs_lm.push_back((int32_t)lm);
      M->obs_kf.push_back(K);
      M->obs_cam.push_back(c);
    }
    // Loop-closure landmarks shared with another co-registered mission.  The
    // missions re-traverse the same path; mission m overlaps its ring
    // neighbours m-1 and m+1, and the landmark is re-observed from the
    // keyframes of that mission closest to the store keyframe within the same
    // lap, so loop closures link corresponding trajectory segments.
    if (nm > 1 && cfg->co_registered && cfg->shared_landmark_fraction > 0 && rng.uniform() < cfg->shared_landmark_fraction) {
      const int m2 = nm == 2 ? 1 - m : (rng.below(2) ? (m + 1) % nm : (m + nm - 1) % nm);
      const int c2 = cfg->camera_per_mission ? m2 % cfg->num_cameras : c;
      const int64_t Kbest = [&]() {
        const int64_t lap = (int64_t)std::llround(cfg->keyframes_per_lap);
        const int64_t local = store - kf0[m];
        const int64_t lo = std::max<int64_t>(0, local - lap / 2), hi = std::min<int64_t>(nk[m2], local + lap / 2 + 1);
        int64_t best = -1;
        double bd = 1e30;
        for (int64_t k = lo; k < hi; ++k) {
          const int64_t K = kf0[m2] + k;
          double d = 0.0;
          for (int i = 0; i < 3; ++i) d += (kf_pG[K][i] - kf_pG[store][i]) * (kf_pG[K][i] - kf_pG[store][i]);
          if (d < bd) { bd = d; best = K; }
        }
        return best;
      }();
      int added = 0;
      for (int64_t k = Kbest; k >= 0 && k < kf0[m2 + 1] && added < L; ++k) {
        double kp[2];
        if (!visibleIn(k, c2, pG, kp)) break;
        M->obs_uv.push_back(kp[0] + cfg->pixel_sigma * rng.normal());
        M->obs_uv.push_back(kp[1] + cfg->pixel_sigma * rng.normal());
        M->obs_sigma.push_back(cfg->pixel_sigma);
        M->obs_lm.push_back((int32_t)lm);
        M->obs_kf.push_back((int32_t)k);
        M->obs_cam.push_back(c2);
        ++added;
      }
    }
    // p_B in the store keyframe's IMU frame.
    const int ms = M->kf_mis[store];
    double d[3] = {pG[0] - kf_pG[store][0], pG[1] - kf_pG[store][1], pG[2] - kf_pG[store][2]};
    double pB[3];
    mv(tr(kf_RGI[store]), d, pB);
    (void)ms;
    for (int i = 0; i < 3; ++i) M->lm_p.push_back(pB[i]);
    M->lm_store.push_back((int32_t)store);
    ++lm;
  }
  M->nlm = lm;
  M->nobs = (int64_t)M->obs_lm.size();
  M->lm_const.assign(M->nlm, 0);

  // Mission clusters by shared landmarks (union-find), gauge fixes per cluster.
  std::vector<int> parent(nm);
  std::iota(parent.begin(), parent.end(), 0);
  std::function<int(int)> find = [&](int a) { return parent[a] == a ? a : parent[a] = find(parent[a]); };
  for (int64_t i = 0; i < M->nobs; ++i) {
    const int a = find(M->kf_mis[M->obs_kf[i]]), b = find(M->kf_mis[M->lm_store[M->obs_lm[i]]]);
    if (a != b) parent[std::max(a, b)] = std::min(a, b);
  }
  for (int m = 0; m < nm; ++m) {
    if (find(m) != m) continue;  // first mission of its cluster
    const int64_t K = kf0[m];
    if (cfg->include_inertial) {
      M->kf_flags[K] |= MBA_KF_GAUGE_ROLL_PITCH | MBA_KF_POSITION_CONSTANT;
    } else {
      M->kf_flags[K] |= MBA_KF_POSE_CONSTANT;
      for (int64_t l = 0; l < M->nlm; ++l)
        if (M->lm_store[l] == K) { M->lm_const[l] = 1; break; }
    }
  }

  // Ground truth copies, then perturb the initial state (first keyframe of
  // each mission untouched, 6dof-pose-graph-gen.cc:337-340).
  M->kf_x_true = M->kf_x; M->kf_v_true = M->kf_v; M->kf_bg_true = M->kf_bg; M->kf_ba_true = M->kf_ba;
  M->lm_p_true = M->lm_p;
  for (int m = 0; m < nm; ++m) {
    for (int k = 1; k < nk[m]; ++k) {
      const int64_t K = kf0[m] + k;
      double d[3] = {cfg->rot_perturb * rng.normal(), cfg->rot_perturb * rng.normal(), cfg->rot_perturb * rng.normal()};
      double q[4];
      jplPlus(&M->kf_x[7 * K], d, q);
      for (int i = 0; i < 4; ++i) M->kf_x[7 * K + i] = q[i];
      for (int i = 0; i < 3; ++i) M->kf_x[7 * K + 4 + i] += cfg->pos_perturb * rng.normal();
      for (int i = 0; i < 3; ++i) M->kf_v[3 * K + i] += cfg->vel_perturb * rng.normal();
    }
    for (int k = 0; k < nk[m]; ++k) {
      const int64_t K = kf0[m] + k;
      for (int i = 0; i < 3; ++i) { M->kf_bg[3 * K + i] = 0.0; M->kf_ba[3 * K + i] = 0.0; }
    }
  }
  for (int64_t l = 0; l < M->nlm; ++l)
    if (!M->lm_const[l])
      for (int i = 0; i < 3; ++i) M->lm_p[3 * l + i] += cfg->lm_perturb * rng.normal();
  // Odometry edges between consecutive keyframes: the relative pose
  // T_B_I T_M_Ik^-1 T_M_Ik+1 T_B_I^-1 of the true state (the measurement model
  // of SixDoFBlockPoseErrorTermWithExtrinsics; Hamilton quaternions on the
  // state's JPL coefficients), perturbed by the stated noise.  Drawn last so
  // that maps without them keep their random stream.
  if (cfg->pose_edges) {
    const double ext[7] = {0.0, 0.0, std::sin(0.05), std::cos(0.05), 0.10, -0.02, 0.05};  // q_I_B | p_B_I
    for (int m = 0; m < nm; ++m)
      for (int k = 0; k + 1 < nk[m]; ++k) {
        const int64_t a = kf0[m] + k, b = a + 1;
        double T[7];
        odometryFromStates(&M->kf_x_true[7 * a], &M->kf_x_true[7 * b], ext, T);
        const double dq[3] = {cfg->pose_edge_sigma_q * rng.normal(), cfg->pose_edge_sigma_q * rng.normal(),
                              cfg->pose_edge_sigma_q * rng.normal()};
        hamiltonPerturb(T, dq);
        for (int i = 0; i < 3; ++i) T[4 + i] += cfg->pose_edge_sigma_p * rng.normal();
        M->pe_from.push_back((int32_t)a);
        M->pe_to.push_back((int32_t)b);
        for (int i = 0; i < 7; ++i) M->pe_meas.push_back(T[i]);
        for (int i = 0; i < 7; ++i) M->pe_ext.push_back(ext[i]);
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c) {
            const double sg = r < 3 ? cfg->pose_edge_sigma_p : cfg->pose_edge_sigma_q;
            M->pe_cov.push_back(r == c ? sg * sg : 0.0);
          }
        M->pe_type.push_back(MBA_POSE_EDGE_RELATIVE);
        M->pe_sw.push_back(1.0);
        M->pe_swvar.push_back(0.0);
      }
  }
  auto push_measurement = [&](int64_t a, int64_t b, int type, double* T, double sp, double sq, double nsp, double nsq,
                              const double* ext) {
    const double dq[3] = {nsq * rng.normal(), nsq * rng.normal(), nsq * rng.normal()};
    hamiltonPerturb(T, dq);
    for (int i = 0; i < 3; ++i) T[4 + i] += nsp * rng.normal();
    M->pe_from.push_back((int32_t)a);
    M->pe_to.push_back((int32_t)b);
    for (int i = 0; i < 7; ++i) M->pe_meas.push_back(T[i]);
    for (int i = 0; i < 7; ++i) M->pe_ext.push_back(ext[i]);
    for (int r = 0; r < 6; ++r)
      for (int c = 0; c < 6; ++c) {
        const double sg = r < 3 ? sp : sq;
        M->pe_cov.push_back(r == c ? sg * sg : 0.0);
      }
    M->pe_type.push_back(type);
    M->pe_sw.push_back(1.0);
    M->pe_swvar.push_back(type == MBA_POSE_EDGE_LOOP_CLOSURE ? cfg->loop_closure_switch_variance : 0.0);
  };
  // Loop closures (true relative pose plus noise; a fraction replaced by a
  // grossly wrong transform) and absolute 6-DoF measurements.
  if (cfg->loop_closure_stride > 0) {
    static const double kNone[7] = {0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0};
    const int64_t lap = std::max<int64_t>(1, std::llround(cfg->keyframes_per_lap));
    auto add_lc = [&](int64_t a, int64_t b) {
      const bool same = M->kf_mis[a] == M->kf_mis[b];
      const double* ba = same ? kNone : &M->mis[7 * M->kf_mis[a]];
      const double* bb = same ? kNone : &M->mis[7 * M->kf_mis[b]];
      double T[7];
      loopClosureFromStates(ba, &M->kf_x_true[7 * a], bb, &M->kf_x_true[7 * b], T);
      const bool outlier = rng.uniform() < cfg->loop_closure_outlier_fraction;
      push_measurement(a, b, MBA_POSE_EDGE_LOOP_CLOSURE, T, cfg->loop_closure_sigma_p, cfg->loop_closure_sigma_q,
                       outlier ? 3.0 : cfg->loop_closure_sigma_p, outlier ? 0.5 : cfg->loop_closure_sigma_q, kNone);
    };
    for (int m = 0; m < nm; ++m)
      for (int64_t k = 0; k + lap < nk[m]; k += cfg->loop_closure_stride) add_lc(kf0[m] + k, kf0[m] + k + lap);
    for (int m = 0; m + 1 < nm; ++m)
      for (int64_t k = 0; k < std::min<int64_t>(nk[m], nk[m + 1]); k += cfg->loop_closure_stride)
        add_lc(kf0[m] + k, kf0[m + 1] + k);
  }
  if (cfg->absolute_pose_stride > 0) {
    const double ext[7] = {std::sin(0.05), 0.0, 0.0, std::cos(0.05), 0.2, 0.0, -0.1};  // q_S_B | p_S_B
    for (int m = 0; m < nm; ++m)
      for (int64_t k = 0; k < nk[m]; k += cfg->absolute_pose_stride) {
        const int64_t K = kf0[m] + k;
        double T[7];
        absolutePoseFromState(&M->mis[7 * m], &M->kf_x_true[7 * K], ext, T);
        push_measurement(K, K, MBA_POSE_EDGE_ABSOLUTE, T, cfg->absolute_pose_sigma_p, cfg->absolute_pose_sigma_q,
                         cfg->absolute_pose_sigma_p, cfg->absolute_pose_sigma_q, ext);
      }
  }
  *out = M.release();
  return MBA_OK;
}

void mba_synth_free(mba_synth_map* map) { delete map; }

mba_status mba_synth_describe(const mba_synth_map* M, mba_problem_desc* d) {
  if (!M || !d) return MBA_ERR_INVALID_ARG;
  std::memset(d, 0, sizeof(*d));
  d->num_keyframes = M->nkf; d->num_landmarks = M->nlm; d->num_observations = M->nobs;
  d->num_cameras = M->ncam; d->num_missions = M->nmis; d->num_imu_edges = M->nedge; d->num_imu_samples = M->nsamp;
  d->obs_uv = M->obs_uv.data(); d->obs_sigma = M->obs_sigma.data(); d->obs_landmark = M->obs_lm.data();
  d->obs_keyframe = M->obs_kf.data(); d->obs_camera = M->obs_cam.data();
  d->lm_p_B = M->lm_p.data(); d->lm_store_keyframe = M->lm_store.data(); d->lm_constant = M->lm_const.data();
  d->kf_q_IM_p_MI = M->kf_x.data(); d->kf_v_M = M->kf_v.data(); d->kf_b_g = M->kf_bg.data(); d->kf_b_a = M->kf_ba.data();
  d->kf_mission = M->kf_mis.data(); d->kf_flags = M->kf_flags.data();
  d->mission_q_GM_p_GM = M->mis.data(); d->cameras = M->cams.data();
  d->edge_from = M->e_from.data(); d->edge_to = M->e_to.data(); d->edge_sample_offset = M->e_off.data();
  d->imu_timestamp_ns = M->ts.data(); d->imu_acc_gyro = M->imu.data();
  d->num_pose_edges = (int64_t)M->pe_from.size();
  d->pose_edge_from = M->pe_from.data(); d->pose_edge_to = M->pe_to.data();
  d->pose_edge_T_Bk_Bkp1 = M->pe_meas.data(); d->pose_edge_covariance = M->pe_cov.data();
  d->pose_edge_q_I_B_p_B_I = M->pe_ext.data();
  d->pose_edge_type = M->pe_type.data();
  d->pose_edge_switch = M->pe_sw.data();
  d->pose_edge_switch_variance = M->pe_swvar.data();
  d->gyro_noise_sigma = M->cfg.gyro_noise; d->gyro_bias_sigma = M->cfg.gyro_bias_rw;
  d->acc_noise_sigma = M->cfg.acc_noise; d->acc_bias_sigma = M->cfg.acc_bias_rw;
  d->gravity_magnitude = M->gravity;
  d->use_huber = 1; d->huber_delta_local = 3.0; d->huber_delta_global = 10.0;
  return MBA_OK;
}

mba_status mba_synth_ground_truth(const mba_synth_map* M, double* kx, double* kv, double* kbg, double* kba, double* lp) {
  if (!M) return MBA_ERR_INVALID_ARG;
  if (kx) std::memcpy(kx, M->kf_x_true.data(), M->kf_x_true.size() * sizeof(double));
  if (kv) std::memcpy(kv, M->kf_v_true.data(), M->kf_v_true.size() * sizeof(double));
  if (kbg) std::memcpy(kbg, M->kf_bg_true.data(), M->kf_bg_true.size() * sizeof(double));
  if (kba) std::memcpy(kba, M->kf_ba_true.data(), M->kf_ba_true.size() * sizeof(double));
  if (lp) std::memcpy(lp, M->lm_p_true.data(), M->lm_p_true.size() * sizeof(double));
  return MBA_OK;
}

}  // extern "C"
