"""The reference's own cost-term test scenarios (tests/golden/
error_term_scenarios.json, extracted from algorithms/ceres-error-terms/test/
by tests/golden/make_golden.py) as problem descriptors of include/maplab_ba.h,
and the reference's assertions checked on a solved state.

Mapping of a scenario onto the descriptor:
* visual files: every pose block passed as landmark_base_pose or imu_pose is
  a keyframe; a landmark's store keyframe is its base pose.  In
  test_visual_term_test.cc (kLocalMission) all keyframes share one mission
  with the identity baseframe (the constant dummy blocks); in
  test_mission_baseframe_visual_term_test.cc (kGlobal) base poses belong to
  the mission of landmark_mission_baseframe_ and observers to the mission of
  keyframe_mission_baseframe_, so every term is kGlobal.  The camera is the
  fixture's PinholeCamera (640 x 480) with FisheyeDistortion(w): w = 0 is the
  identity map (the w^2 < 1e-5 branch of distortion-fisheye.cc), i.e. no
  distortion.  No loss function (the tests pass NULL).
* inertial files: pose_k / velocity_k / gyro_bias_k / accel_bias_k of
  keyframe k, one InertialErrorTerm per consecutive pair with the fixture's
  samples, sigmas 1 and Zurich gravity; the 3-keyframe file's ground truth is
  integrated with the oracle's RK4 integrator (itself pinned to the
  reference's integrator vectors) exactly as its SetUp does.
Solver settings: the tests' ceres::Solver::Options (tolerances 1e-50,
default trust region: initial radius 1e4, maximum 1e16).
"""
import ctypes
import json
import math
import os

import numpy as np

from maplab_gb300 import _native as N
from problem_util import OwnedDesc, camera

GOLDEN = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                     "error_term_scenarios.json")))

FAMILIES = ["visual_local_mission", "visual_global", "inertial_two_keyframes", "inertial_three_keyframes"]


def all_scenarios():
    return [(fam, sc) for fam in FAMILIES for sc in GOLDEN[fam]["scenarios"]]


def scenario_id(item):
    fam, sc = item
    return f"{fam}:{sc['name']}"


class Built:
    """A descriptor plus where each named block of the scenario lives."""

    def __init__(self, owned, where, requires):
        self.owned = owned
        self.desc = owned.desc
        self.where = where        # block name -> ("kf", k) | ("lm", l) | ("v"|"bg"|"ba", k) | ("cam", part) | ("mis", m)
        self.requires = requires  # calibration / baseframe blocks the scenario leaves free


def _integrate(state16, readings, dt, gravity):
    import oracle_lib as O
    nxt = np.zeros(16)
    O.load().oracle_imu_integrate(N.ptr(O.arr([0, 0, 0, 0, gravity])), N.ptr(O.arr(state16)),
                                  N.ptr(O.arr(readings)), ctypes.c_double(dt), N.ptr(nxt), None, None)
    return nxt


def _normalized(q):
    q = np.asarray(q, dtype=np.float64)
    return q / np.linalg.norm(q)


def build(fam, sc):
    if fam.startswith("visual"):
        return _build_visual(fam, sc)
    return _build_inertial(fam, sc)


def _build_visual(fam, sc):
    B = sc["blocks"]
    res = sc["residuals"]
    const = set(sc["constant"])
    kfs, lms = [], []
    for r in res:
        for k in (r["landmark_base_pose"], r["imu_pose"]):
            if k not in kfs:
                kfs.append(k)
        if r["landmark"] not in lms:
            lms.append(r["landmark"])
    base_of = {}
    for r in res:
        assert base_of.setdefault(r["landmark"], r["landmark_base_pose"]) == r["landmark_base_pose"]
    bases = {r["landmark_base_pose"] for r in res}
    observers = {r["imu_pose"] for r in res}
    assert not (bases & observers), "a keyframe is both a landmark base and an observer"

    def block(name):
        if "[" in name:
            base, i = name[:-1].split("[")
            return B[base][int(i)]
        return B[name]

    if fam == "visual_global":
        mission_names = ["landmark_mission_baseframe_", "keyframe_mission_baseframe_"]
        kf_mission = [0 if k in bases else 1 for k in kfs]
    else:
        mission_names = ["dummy_7d_0_"]
        kf_mission = [0] * len(kfs)
    missions = [B[m] for m in mission_names]
    qci, pci = res[0]["q_CI"], res[0]["p_CI"]
    assert all(r["q_CI"] == qci and r["p_CI"] == pci for r in res)
    cam = sc["camera"]
    # The camera's blocks the test leaves free become variables; baseframes
    # free in the test use the 6-dof JplPoseParameterization it sets.
    cam_flags = 0
    for name, bit in (("intrinsics", N.MBA_CAM_INTRINSICS_FREE), ("distortion", N.MBA_CAM_DISTORTION_FREE),
                      (qci, N.MBA_CAM_ROTATION_FREE), (pci, N.MBA_CAM_TRANSLATION_FREE)):
        if name not in const:
            cam_flags |= bit
    mis_flags = [0 if m in const else N.MBA_MIS_BASEFRAME_POSE for m in mission_names]
    w = cam["fisheye_w"]
    c = camera(fu=cam["intrinsics"][0], fv=cam["intrinsics"][1], cu=cam["intrinsics"][2], cv=cam["intrinsics"][3],
               w=int(cam["width"]), h=int(cam["height"]), dtype=N.MBA_DISTORTION_FOV, dist=(w, 0, 0, 0),
               q_CI=B[qci], p_CI=B[pci])
    # the fixture's quaternion block is used as given (a unit quaternion)
    for i in range(4):
        c.q_CI_p_CI[i] = B[qci][i]
    flags = [N.MBA_KF_POSE_CONSTANT if k in const else 0 for k in kfs]
    od = OwnedDesc(obs_uv=[r["keypoint"] for r in res], obs_sigma=[r["sigma"] for r in res],
                   obs_landmark=[lms.index(r["landmark"]) for r in res],
                   obs_keyframe=[kfs.index(r["imu_pose"]) for r in res], obs_camera=[0] * len(res),
                   lm_p_B=[block(l) for l in lms], lm_store_keyframe=[kfs.index(base_of[l]) for l in lms],
                   lm_constant=[1 if l in const else 0 for l in lms], kf_q_IM_p_MI=[B[k] for k in kfs],
                   kf_mission=kf_mission, kf_flags=flags, mission_q_GM_p_GM=missions, cameras=[c], use_huber=0,
                   camera_flags=[cam_flags], mission_flags=mis_flags)
    where = {k: ("kf", i) for i, k in enumerate(kfs)}
    where.update({l: ("lm", i) for i, l in enumerate(lms)})
    where.update({"intrinsics": ("cam", "intrinsics"), "distortion": ("cam", "distortion"), qci: ("cam", "q_CI"),
                  pci: ("cam", "p_CI")})
    where.update({m: ("mis", i) for i, m in enumerate(mission_names)})
    return Built(od, where, [])


def _build_inertial(fam, sc):
    B = {k: list(v) for k, v in sc["blocks"].items()}
    const = set(sc["constant"])
    if fam == "inertial_three_keyframes":
        gt = GOLDEN[fam]["ground_truth"]
        s0 = np.zeros(16)
        s0[0:4] = gt["rot0"]
        s0[7:10] = gt["velocity0"]
        s0[13:16] = gt["pos0"]
        s1 = _integrate(s0, gt["readings"], gt["dt"], gt["gravity"])
        s2 = _integrate(s1, gt["readings"], gt["dt"], gt["gravity"])
        field = {"Orientation": slice(0, 4), "Velocity": slice(7, 10), "Position": slice(13, 16)}
        truth = {}
        for name, t in gt["states_from_integration"].items():
            v = (s1 if t["integration"] == 1 else s2)[field[t["field"]]].tolist()
            B[name] = list(v)
            truth[name] = list(v)
        for op in sc["ops"]:
            if op["op"] == "add":
                B[op["block"]] = [a + b for a, b in zip(B[op["block"]], op["value"])]
            elif op["op"] == "normalize":
                B[op["block"]] = _normalized(B[op["block"]]).tolist()
        sc = dict(sc, truth=truth)
        nk = 3
        stamps = [gt["imu_timestamps_01_ns"], gt["imu_timestamps_12_ns"]]
        datas = [gt["imu_data_01_row_major_6xn"], gt["imu_data_12_row_major_6xn"]]
        gravity = gt["gravity"]
    else:
        nk = 2
        stamps = [sc["imu_timestamps_ns"]]
        datas = [sc["imu_data_row_major_6xn"]]
        gravity = sc["gravity"]
    poses, flags = [], []
    for k in range(nk):
        poses.append(list(_normalized(B[f"rot{k}_"])) + list(B[f"pos{k}_"]))  # addResidual normalizes
        f = 0
        f |= N.MBA_KF_POSE_CONSTANT if f"pose{k}_" in const else 0
        f |= N.MBA_KF_VELOCITY_CONSTANT if f"velocity{k}_" in const else 0
        f |= N.MBA_KF_GYRO_BIAS_CONSTANT if f"gyro_bias{k}_" in const else 0
        f |= N.MBA_KF_ACCEL_BIAS_CONSTANT if f"accel_bias{k}_" in const else 0
        flags.append(f)
    ts, imu, off = [], [], [0]
    for st, dat in zip(stamps, datas):
        n = len(st)
        D = np.asarray(dat, dtype=np.float64).reshape(6, n)
        ts += [int(round(t)) for t in st]
        imu += [D[:, j].tolist() for j in range(n)]
        off.append(off[-1] + n)
    od = OwnedDesc(obs_uv=np.zeros((0, 2)), obs_sigma=[], obs_landmark=[], obs_keyframe=[], obs_camera=[],
                   lm_p_B=np.zeros((0, 3)), lm_store_keyframe=[], kf_q_IM_p_MI=poses,
                   kf_v_M=[B[f"velocity{k}_"] for k in range(nk)], kf_b_g=[B[f"gyro_bias{k}_"] for k in range(nk)],
                   kf_b_a=[B[f"accel_bias{k}_"] for k in range(nk)], kf_flags=flags, cameras=[camera()],
                   edge_from=list(range(nk - 1)), edge_to=list(range(1, nk)), edge_sample_offset=off,
                   imu_timestamp_ns=ts, imu_acc_gyro=imu, imu_sigmas=(1.0, 1.0, 1.0, 1.0), gravity=gravity)
    where = {}
    for k in range(nk):
        where[f"pose{k}_"] = ("kf", k)
        where[f"velocity{k}_"] = ("v", k)
        where[f"gyro_bias{k}_"] = ("bg", k)
        where[f"accel_bias{k}_"] = ("ba", k)
    b = Built(od, where, [])
    b.truth = sc.get("truth", {})
    return b


def solver_options(lib_default, device):
    """The tests' ceres::Solver::Options: tolerances 1e-50, Ceres' default
    trust region (initial radius 1e4, maximum 1e16), no outlier rejection
    (plain ceres::Solve).  Device: PCG run to a tight tolerance (the tests
    solve DENSE_SCHUR)."""
    o = lib_default()
    o.max_num_iterations = 500
    o.function_tolerance = 1e-50
    o.gradient_tolerance = 1e-50
    o.parameter_tolerance = 1e-50
    o.initial_trust_region_radius = 1e4
    o.max_trust_region_radius = 1e16
    o.check_tolerances = 1
    o.reject_outliers_every_n_iters = 0
    if device:
        o.linear_solver = N.MBA_LINEAR_SOLVER_PCG
        o.linear_tolerance = 1e-14
        o.max_linear_iterations = 1000
    else:
        o.linear_solver = N.MBA_LINEAR_SOLVER_DENSE_SCHUR
    return o


def _disparity_angle(qa, qb):
    """Rotation angle between two unit quaternions (kindr getDisparityAngle)."""
    qa = _normalized(qa)
    qb = _normalized(qb)
    d = abs(float(np.dot(qa, qb)))
    # angle of qa * qb^-1 = 2 acos(|<qa, qb>|), written with atan2 for accuracy near 0
    s = math.sqrt(max(0.0, 1.0 - d * d))
    return 2.0 * math.atan2(s, d)


def check(built, sc, summary, state, calibration=None):
    """The scenario's assertions on a solved state; returns failure strings.
    state: read_state() dict; calibration: optional dict with 'intrinsics',
    'q_CI', 'p_CI', 'distortion' and 'baseframes' after the solve."""
    fails = []

    def value(name):
        kind, i = built.where[name]
        if kind == "kf":
            return np.asarray(state["kf_q_IM_p_MI"][i])
        if kind == "lm":
            return np.asarray(state["lm_p_B"][i])
        if kind in ("v", "bg", "ba"):
            key = {"v": "kf_v_M", "bg": "kf_b_g", "ba": "kf_b_a"}[kind]
            return np.asarray(state[key][i])
        if calibration is None:
            raise KeyError(name)
        if kind == "cam":  # the scenarios have one camera
            return np.asarray(calibration[i][0])
        return np.asarray(calibration["baseframes"][i])

    for e in sc["expect"]:
        k = e["kind"]
        if k == "final_cost_eq":
            if summary["final_cost"] != e["value"]:
                fails.append(f"final cost {summary['final_cost']!r} != {e['value']}")
        elif k == "final_cost_lt":
            if not summary["final_cost"] < e["value"]:
                fails.append(f"final cost {summary['final_cost']!r} !< {e['value']}")
        elif k == "iterations_eq":
            if summary["num_iterations"] != int(e["value"]):
                fails.append(f"iterations {summary['num_iterations']} != {int(e['value'])}")
        elif k == "near":
            v = value(e["block"])
            end = e["end"] if e.get("end") is not None else len(v)
            a = v[e["begin"]:end]
            if "other_block" in e:
                b = value(e["other_block"])[e["begin"]:end]
            elif "truth" in e:
                b = np.asarray(built.truth[e["truth"]])
            elif e["value"] == "zeros":
                b = np.zeros_like(a)
            else:
                b = np.asarray(e["value"])
            err = float(np.abs(a - b).max())
            if not err <= e["tol"]:
                fails.append(f"{e['block']}[{e['begin']}:{end}] = {a.tolist()} vs {b.tolist()}: {err:.3e} > {e['tol']}")
        elif k == "quat":
            ang = _disparity_angle(value(e["block"])[:4], e["value"])
            if not ang <= e["tol"]:
                fails.append(f"{e['block']} disparity angle {ang:.3e} > {e['tol']}")
        elif k == "quat_norm":
            n = float(np.linalg.norm(value(e["block"])[:4]))
            if not abs(n - e["value"]) <= e["tol"]:
                fails.append(f"{e['block']} norm {n!r} vs {e['value']} (tol {e['tol']})")
        else:
            fails.append(f"unknown assertion {k}")
    return fails
