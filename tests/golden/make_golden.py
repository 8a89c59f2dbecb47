"""Extracts golden vectors from the reference's own unit tests (read as text).

Run where the maplab source tree is available (its root as the argument or
in the MAPLAB_REFERENCE_ROOT environment variable):

    python tests/golden/make_golden.py /path/to/maplab

It writes tests/golden/imu_integrator.json with the known-answer cases of
algorithms/imu-integrator-rk4/test/test_imu_integrator_cov_phi_test.cc
(ImuIntegratorPhiTest, ImuIntegratorCovarianceTest: expected 16-dim state,
15x15 transition and 15x15 covariance at 1e-12) and the closed-form cases of
test_imu_integrator_basic_test.cc (restated as inputs + expected outputs).
The numbers are copied verbatim from the reference tests; nothing is
recomputed here.  It also writes reference_sensors.json (maplab's own
calibration files), error_term_scenarios.json (the visual and inertial
cost-term tests, via error_term_scenarios.py), pose_extrinsics_scenarios.json
(the relative pose term with extrinsics), pose_parameterization_scenario.json
(JplPoseParameterization's minimization test), camera_scenarios.json
(aslam's pinhole camera and distortion tests) and quaternion_math.json
(maplab-common's JPL rotation-matrix known answer).
"""
import json
import math
import os
import re
import sys


def _numbers_after(text, marker, count):
    i = text.index(marker)
    j = text.index("<<", i) + 2
    k = text.index(";", j)
    nums = re.findall(r"[-+]?\d+(?:\.\d*)?(?:[eE][-+]?\d+)?", text[j:k])
    vals = [float(x) for x in nums]
    assert len(vals) == count, (marker, len(vals))
    return vals


def _test_body(text, name):
    i = text.index(name)
    j = text.index("TEST_F", i + len(name)) if "TEST_F" in text[i + len(name):] else len(text)
    return text[i:j]


def main(root, here=None):
    """Writes every fixture into `here` (default: this file's directory)."""
    here = here or os.path.dirname(os.path.abspath(__file__))
    base = os.path.join(root, "algorithms", "imu-integrator-rk4", "test")
    src = open(os.path.join(base, "test_imu_integrator_cov_phi_test.cc")).read()
    phi_body = _test_body(src, "ImuIntegratorPhiTest")
    cov_body = _test_body(src, "ImuIntegratorCovarianceTest")
    s2 = math.sqrt(2.0) / 2.0
    # Common inputs of both tests (cov_phi_test.cc:14-40 and :94-121).
    readings = [0.3, 0.0, 9.81, 0.0, 0.2, 0.0, 0.3, 0.0, 9.81, 0.0, 0.2, 0.0]
    state = [0.0, 0.0, -s2, s2, 0, 0, 0, 0.0, 2.5, 0.0, 0, 0, 0, 0, 0, 0]
    cases = [
        {
            "name": "ImuIntegratorPhiTest",
            "source": "algorithms/imu-integrator-rk4/test/test_imu_integrator_cov_phi_test.cc:13-90",
            "gravity": 9.81, "sigmas": [0.0, 0.0, 0.0, 0.0], "dt": 1.2,
            "state": state, "readings": readings, "tol": 1e-12,
            "expected_state": _numbers_after(phi_body, "expected_state", 16),
            "expected_phi": _numbers_after(phi_body, "expected_phi", 225),
        },
        {
            "name": "ImuIntegratorCovarianceTest",
            "source": "algorithms/imu-integrator-rk4/test/test_imu_integrator_cov_phi_test.cc:92-178",
            "gravity": 9.81, "sigmas": [0.1, 0.2, 0.3, 0.4], "dt": 1.2,
            "state": state, "readings": readings, "tol": 1e-12,
            "expected_state": _numbers_after(cov_body, "expected_state", 16),
            "expected_cov": _numbers_after(cov_body, "expected_cov", 225),
        },
    ]
    # Closed-form cases of test_imu_integrator_basic_test.cc (inputs and the
    # expected values stated by those tests).
    a, v = 0.3, 2.5
    basic = []
    basic.append({"name": "ZeroReadingsZeroBiases", "source": "test_imu_integrator_basic_test.cc:13-28",
                  "gravity": 0.0, "dt": 1.0, "state": [0, 0, 0, 1] + [0] * 12, "readings": [0.0] * 12,
                  "expected_state": [0, 0, 0, 1] + [0] * 12, "tol": 1e-15, "cov_zero": True})
    basic.append({"name": "JustNonzeroGravity", "source": "test_imu_integrator_basic_test.cc:30-60",
                  "gravity": 1.0, "dt": 1.0, "state": [0, 0, 0, 1] + [0] * 12, "readings": [0.0] * 12,
                  "expected_state": [0, 0, 0, 1, 0, 0, 0, 0, 0, -1.0, 0, 0, 0, 0, 0, -0.5], "tol": 1e-15,
                  "cov_zero": True})
    basic.append({"name": "ConstantForwardAcceleration", "source": "test_imu_integrator_basic_test.cc:62-95",
                  "gravity": 9.81, "dt": 1.0, "state": [0, 0, 0, 1] + [0] * 12,
                  "readings": [a, 0, 9.81, 0, 0, 0, a, 0, 9.81, 0, 0, 0],
                  "expected_state": [0, 0, 0, 1, 0, 0, 0, a, 0, 0, 0, 0, 0, a / 2, 0, 0], "tol": 1e-15,
                  "cov_zero": True})
    dt = 1.8
    basic.append({"name": "ConstForwardAccelInitialVelocity", "source": "test_imu_integrator_basic_test.cc:97-136",
                  "gravity": 9.81, "dt": dt, "state": [0, 0, 0, 1, 0, 0, 0, v, 0, 0, 0, 0, 0, 0, 0, 0],
                  "readings": [a, 0, 9.81, 0, 0, 0, a, 0, 9.81, 0, 0, 0],
                  "expected_state": [0, 0, 0, 1, 0, 0, 0, v + a * dt, 0, 0, 0, 0, 0,
                                     v * dt + a * dt * dt / 2, 0, 0], "tol": 1e-15, "cov_zero": True})
    dt = 1.2
    basic.append({"name": "ConstAccelAndVelocityWhenRotated", "source": "test_imu_integrator_basic_test.cc:138-181",
                  "gravity": 9.81, "dt": dt, "state": [0, 0, s2, s2, 0, 0, 0, 0, v, 0, 0, 0, 0, 0, 0, 0],
                  "readings": [a, 0, 9.81, 0, 0, 0, a, 0, 9.81, 0, 0, 0],
                  "expected_state": [0, 0, s2, s2, 0, 0, 0, 0, v + a * dt, 0, 0, 0, 0, 0,
                                     v * dt + a * dt * dt / 2, 0], "tol": 1e-15, "cov_zero": True})
    w = math.pi / 180.0
    basic.append({"name": "ConstantAngularVelocity", "source": "test_imu_integrator_basic_test.cc:183-226",
                  "gravity": 9.81, "dt": 1.0, "state": [0, 0, 0, 1] + [0] * 12,
                  "readings": [0, 0, 9.81, 0, 0, w, 0, 0, 9.81, 0, 0, w],
                  "expected_quat": [0, 0, math.sin(w / 2), math.cos(w / 2)], "quat_tol": 1e-10})
    basic.append({"name": "AngularVelocitySlope", "source": "test_imu_integrator_basic_test.cc:228-256",
                  "gravity": 0.0, "dt": 1.0, "state": [0, 0, 0, 1] + [0] * 12,
                  "readings": [0, 0, 0, 0, 0, w, 0, 0, 0, 0, 0, 0],
                  "expected_quat": [0, 0, math.sin(w / 4), math.cos(w / 4)], "quat_tol": 1e-8})
    dt = 3.0
    basic.append({"name": "LinearAccelerationSlope", "source": "test_imu_integrator_basic_test.cc:258-288",
                  "gravity": 9.81, "dt": dt, "state": [0, 0, 0, 1] + [0] * 12,
                  "readings": [0.5, 0, 9.81, 0, 0, 0, 0, 0, 9.81, 0, 0, 0],
                  "expected_velocity": [0.5 * dt / 2, 0, 0],
                  "expected_position": [0.5 * dt * dt / 3, 0, 0], "tol": 1e-15})
    out = {"generator": "tests/golden/make_golden.py", "cases": cases, "basic": basic}
    with open(os.path.join(here, "imu_integrator.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(here, "imu_integrator.json"))
    sensor_files(root, here)
    pose_extrinsics_scenarios(root, here)
    pose_parameterization_scenario(root, here)
    camera_scenarios(root, here)
    quaternion_math_cases(root, here)
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import error_term_scenarios
    with open(os.path.join(here, "error_term_scenarios.json"), "w") as f:
        json.dump(error_term_scenarios.extract(root), f, indent=1)
    print("wrote", os.path.join(here, "error_term_scenarios.json"))


# maplab's own calibration files: the map reader's sensors.yaml parser is
# checked against them (tests/test_vimap_io.py: test_reference_sensor_files).
SENSOR_FILES = [
    "maplab-launch/config/alphasense-dev-kit/calib/alphasense-dev-kit-sensors.yaml",
    "maplab-launch/config/lidarstick/calib/lidarstick-150-deg-cams-sensors.yaml",
]


def sensor_files(root, here):
    out = {"generator": "tests/golden/make_golden.py",
           "files": {name: open(os.path.join(root, name)).read() for name in SENSOR_FILES}}
    with open(os.path.join(here, "reference_sensors.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(here, "reference_sensors.json"))


# The relative pose term with extrinsics (SixDoFBlockPoseErrorTermWithExtrinsics,
# the odometry term of the optimization builder) has its own unit test; its
# enabled cases are read here: the fixture's SetUp values and, per test, the
# measurement, the blocks held constant and the asserted outcomes.
POSE_EXTRINSICS_TEST = "algorithms/ceres-error-terms/test/test_six_dof_block_transformation_error_term_with_extrinsics.cc"


def _eval_list(expr):
    """Comma-separated numeric expressions of a comma initializer: numbers,
    + - * / and sqrt(...), nothing else."""
    import ast

    def ev(n):
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return float(n.value)
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, (ast.USub, ast.UAdd)):
            v = ev(n.operand)
            return -v if isinstance(n.op, ast.USub) else v
        if isinstance(n, ast.BinOp) and isinstance(n.op, (ast.Add, ast.Sub, ast.Mult, ast.Div)):
            a, b = ev(n.left), ev(n.right)
            return {ast.Add: a + b, ast.Sub: a - b, ast.Mult: a * b, ast.Div: a / b}[type(n.op)]
        if (isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id == "sqrt" and len(n.args) == 1):
            return math.sqrt(ev(n.args[0]))
        raise ValueError("unsupported expression: " + ast.dump(n))

    return [ev(ast.parse(part.strip(), mode="eval").body) for part in expr.split(",")]


def pose_extrinsics_scenarios(root, here):
    text = re.sub(r"//[^\n]*", "", open(os.path.join(root, POSE_EXTRINSICS_TEST)).read())
    setup = text[text.index("virtual void SetUp()"):text.index("void addPriorOn_T_B_I")]
    values = {}
    for m in re.finditer(r"(prior_\w+)(\.coeffs\(\))?\s*<<\s*([^;]+);", setup):
        values[m.group(1)] = _eval_list(m.group(3))
    # The parameter blocks are built from those values (SetUp): the keyframe
    # blocks as q_G_I coefficients | p_G_I, the extrinsics block as the
    # coefficients of q_B_I's inverse | p_B_I.
    assert "pose_G_Ik_ << prior_orientation_G_Ik_.coeffs(), prior_position_G_Ik_" in " ".join(setup.split())
    assert "orientation_B_I_ << prior_orientation_B_I_.inverse().coeffs()" in " ".join(setup.split())
    normalized = set(re.findall(r"(\w+)\.coeffs\(\)\.normalize\(\);", setup))
    for name in normalized:
        v = values[name]
        n = math.sqrt(sum(x * x for x in v))
        values[name] = [x / n for x in v]
    fixture = {
        "p_G_Ik": values["prior_position_G_Ik_"], "p_G_Ikp1": values["prior_position_G_Ikp1_"],
        "p_B_I": values["prior_position_B_I_"],
        "q_G_Ik": values["prior_orientation_G_Ik_"], "q_G_Ikp1": values["prior_orientation_G_Ikp1_"],
        "q_B_I": values["prior_orientation_B_I_"],
        "quaternions": "Hamilton, x y z w (Eigen coeffs)",
        "covariance": "identity" if "T_Bk_Bkp1_measurement_covariance_matrix_.setIdentity()" in setup else None,
    }
    assert fixture["covariance"] == "identity"
    getters = {"get_T_G_Ik()": "T_G_Ik", "get_T_G_Ikp1()": "T_G_Ikp1", "get_T_B_I()": "T_B_I"}
    tests = []
    for m in re.finditer(r"TEST_F\(\s*\w+,\s*(\w+)\)\s*\{", text):
        name = m.group(1)
        depth, i = 0, m.end() - 1
        for j in range(i, len(text)):
            depth += {"{": 1, "}": -1}.get(text[j], 0)
            if depth == 0:
                break
        body = text[i + 1:j]
        if name.startswith("DISABLED_"):
            tests.append({"name": name, "skipped": "disabled in the reference"})
            continue
        case = {"name": name, "fixed": [], "expect": []}
        local = {}
        for stmt in [s.strip() for s in body.split(";") if s.strip()]:
            stmt = " ".join(stmt.split())
            mm = re.fullmatch(r"const aslam::Transformation (\w+) = (.+)", stmt)
            if mm:
                factors = []
                for f in mm.group(2).split(" * "):
                    inv = f.endswith(".inverse()")
                    g = f[:-len(".inverse()")] if inv else f
                    factors.append([getters[g], -1 if inv else 1])
                local[mm.group(1)] = factors
                continue
            mm = re.fullmatch(r"add_T_Bk_Bkp1_Measurement\((.+)\)", stmt)
            if mm:
                arg = mm.group(1)
                case["measurement"] = [] if arg == "aslam::Transformation()" else local[arg]
                continue
            mm = re.fullmatch(r"fix_(T_\w+)\(\)", stmt)
            if mm:
                case["fixed"].append(mm.group(1))
                continue
            if stmt == "solve()":
                continue
            mm = re.fullmatch(r"EXPECT_NEAR\(summary_\.(initial_cost|final_cost), ([-+.\deE]+), ([-+.\deE]+)\)", stmt)
            if mm:
                case["expect"].append({"what": mm.group(1), "value": float(mm.group(2)), "tol": float(mm.group(3))})
                continue
            mm = re.fullmatch(r"EXPECT_TRUE\( EIGEN_MATRIX_NEAR\( (get_T_\w+\(\))\.getTransformationMatrix\(\), "
                              r"(get_T_\w+\(\))\.getTransformationMatrix\(\), ([-+.\deE]+)\)\)", stmt)
            if mm:
                case["expect"].append({"what": "same_transform", "a": getters[mm.group(1)],
                                       "b": getters[mm.group(2)], "tol": float(mm.group(3))})
                continue
            raise ValueError(f"{name}: unsupported statement: {stmt}")
        tests.append(case)
    out = {"generator": "tests/golden/make_golden.py", "source": POSE_EXTRINSICS_TEST,
           "fixture": fixture, "tests": tests}
    with open(os.path.join(here, "pose_extrinsics_scenarios.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(here, "pose_extrinsics_scenarios.json"))


# JplPoseParameterization's own test: a pose block pulled onto a reference
# transformation by a 6-dim error (2 vec(q (x) q_ref^-1) | p - p_ref) under the
# pose parameterization, with Ceres' default options.
POSE_PARAM_TEST = "algorithms/ceres-error-terms/test/test_pose_parameterization_test.cc"


def pose_parameterization_scenario(root, here):
    text = re.sub(r"//[^\n]*", "", open(os.path.join(root, POSE_PARAM_TEST)).read())
    body = text[text.index("TEST(JplPoseParameterization, SimpleMinimization)"):]
    vals = {}
    for m in re.finditer(r"pose::(Quaternion|Position3D) ((?:x|reference)_(?:rot|pos))\(([^;]*)\);", body):
        vals[m.group(2)] = _eval_list(m.group(3))
    wxyz = lambda q: [q[1], q[2], q[3], q[0]]  # kindr (w, x, y, z) -> Eigen coeffs (x, y, z, w)
    flat = " ".join(body.split())
    assert "x_pose << x_rot.toImplementation().coeffs(), x_pos" in flat
    assert "pose::Transformation reference(reference_pos, reference_rot)" in flat
    assert "ceres::Solver::Options options; options.minimizer_progress_to_stdout = false; ceres::Solver::Summary" in flat
    tol_q = float(re.search(r"EXPECT_NEAR_KINDR_QUATERNION\(out_rot, reference_rot, ([-+.\deE]+)\)", flat).group(1))
    tol_p = float(re.search(r"EXPECT_NEAR_EIGEN\(out_pos, reference_pos, ([-+.\deE]+)\)", flat).group(1))
    out = {"generator": "tests/golden/make_golden.py", "source": POSE_PARAM_TEST,
           "name": "JplPoseParameterization.SimpleMinimization",
           "quaternions": "Hamilton, x y z w (Eigen coeffs)",
           "x_q": wxyz(vals["x_rot"]), "x_p": vals["x_pos"],
           "reference_q": wxyz(vals["reference_rot"]), "reference_p": vals["reference_pos"],
           "options": "Ceres defaults", "tol_rotation": tol_q, "tol_position": tol_p}
    with open(os.path.join(here, "pose_parameterization_scenario.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(here, "pose_parameterization_scenario.json"))


# aslam's camera and distortion tests for the models the visual term uses
# (pinhole with radtan, equidistant, fisheye = FOV, or no distortion): the
# test objects' parameters (createTestDistortion, createTestCamera), the
# Jacobian checks' points, finite-difference steps and tolerances, the manual
# projection and the projection-status cases.
CAMERA_DIR = "aslam_cv2/aslam_cv_cameras"


def camera_scenarios(root, here):
    inc = os.path.join(root, CAMERA_DIR, "include", "aslam", "cameras")
    dist = {}
    for name, header, n in (("radtan", "distortion-radtan.h", 4), ("equidistant", "distortion-equidistant.h", 4),
                            ("fov", "distortion-fisheye.h", 1)):
        text = open(os.path.join(inc, header)).read()
        body = text[text.index("createTestDistortion()"):]
        m = re.search(r"Eigen::VectorXd params\((\d+)\);\s*params\s*<<\s*([^;]+);", body)
        assert int(m.group(1)) == n
        dist[name] = _eval_list(m.group(2))
    pin_h = " ".join(open(os.path.join(inc, "camera-pinhole.h")).read().split())
    m = re.search(r"createTestCameraUnique\(\) \{ Distortion::UniquePtr distortion = DistortionType::createTestDistortion\(\); "
                  r"PinholeCamera::UniquePtr camera\( new PinholeCamera\(([^)]*), distortion\)\);", pin_h)
    test_camera = _eval_list(m.group(1))
    pin_cc = " ".join(open(os.path.join(root, CAMERA_DIR, "src", "camera-pinhole.cc")).read().split())
    m = re.search(r"PinholeCamera::Ptr PinholeCamera::createTestCamera\(\) \{ PinholeCamera::Ptr camera\(new PinholeCamera\(([^)]*)\)\);",
                  pin_cc)
    plain_camera = _eval_list(m.group(1))
    tdist = " ".join(re.sub(r"//[^\n]*", "", open(os.path.join(root, CAMERA_DIR, "test", "test-distortions.cc")).read()).split())
    jk = re.search(r"TYPED_TEST\(TestDistortions, JacobianWrtKeypoint\) \{ Eigen::Vector2d keypoint\(([^)]*)\);.*?"
                   r"TEST_JACOBIAN_FINITE_DIFFERENCE\(Point3dJacobianFunctor, keypoint, ([^,]+), ([^,]+),", tdist)
    jd = re.search(r"TYPED_TEST\(TestDistortionsNotNull, JacobianWrtDistortion\) \{ Eigen::Vector2d keypoint\(([^)]*)\);.*?"
                   r"TEST_JACOBIAN_FINITE_DIFFERENCE\(DistortionJacobianFunctor<TypeParam::parameterCount\(\)>, "
                   r"dist_coeffs, ([^,]+), ([^,]+),", tdist)
    tcam = " ".join(re.sub(r"//[^\n]*", "", open(os.path.join(root, CAMERA_DIR, "test", "test-cameras.cc")).read()).split())
    jp = re.search(r"TYPED_TEST\(TestCameras, JacobianWrtPoint3d\) \{ for \(int i=0; i<(\d+); i\+\+\) \{ "
                   r"Eigen::Vector3d x = this->camera_->createRandomVisiblePoint\(([^)]*)\); "
                   r"TEST_JACOBIAN_FINITE_DIFFERENCE\(Point3dFunctor, x, ([^,]+), ([^,]+),", tcam)
    ji = re.search(r"TYPED_TEST\(TestCameras, JacobianWrtIntrinsics\) \{.*?createRandomVisiblePoint\(([^)]*)\);.*?"
                   r"TEST_JACOBIAN_FINITE_DIFFERENCE\(IntrinsicJacobianFunctor<[^>]*>, intrinsics, ([^,]+), ([^,]+),", tcam)
    jdc = re.search(r"TYPED_TEST\(TestCameras, JacobianWrtDistortion\) \{.*?createRandomVisiblePoint\(([^)]*)\);.*?"
                    r"TEST_JACOBIAN_FINITE_DIFFERENCE\(DistortionJacobianFunctor<[^>]*>, dist_coeffs, ([^,]+), ([^,]+) ?,", tcam)
    mp = re.search(r"TEST\(TestCameraPinhole, ManualProjectionWithoutDistortion\) \{.*?double kx = ([^,]+), ky = ([^,]+), "
                   r"kz = ([^;]+);.*?EXPECT_TRUE\(EIGEN_MATRIX_NEAR\(keypoint_manual, keypoint, ([^)]+)\)\);", tcam)
    pr_body = tcam[tcam.index("TEST(TestCameraPinhole, ProjectionResult)"):tcam.index("TEST(CameraComparison, TestEquality)")]
    status = []
    for m in re.finditer(r"ret = cam->project3\(Eigen::Vector3d\(([^)]*)\), &keypoint\); "
                         r"EXPECT_EQ\(ret.getDetailedStatus\(\), aslam::ProjectionResult::Status::(\w+)\);", pr_body):
        status.append({"point": _eval_list(m.group(1)), "status": m.group(2)})
    assert len(status) == 4, status
    f = lambda s: float(s.strip())
    out = {"generator": "tests/golden/make_golden.py", "source": CAMERA_DIR + "/test/test-cameras.cc, test-distortions.cc",
           "distortions": dist,
           "test_camera": {"fu": test_camera[0], "fv": test_camera[1], "cu": test_camera[2], "cv": test_camera[3],
                           "width": test_camera[4], "height": test_camera[5]},
           "plain_camera": {"fu": plain_camera[0], "fv": plain_camera[1], "cu": plain_camera[2], "cv": plain_camera[3],
                            "width": plain_camera[4], "height": plain_camera[5]},
           "numdiff": "five-point central stencil, h = sqrt(step) |x_j| (sqrt(step) where x_j = 0)",
           "distortion_jacobian_wrt_keypoint": {"keypoint": _eval_list(jk.group(1)), "step": f(jk.group(2)),
                                                "tol": f(jk.group(3))},
           "distortion_jacobian_wrt_parameters": {"keypoint": _eval_list(jd.group(1)), "step": f(jd.group(2)),
                                                  "tol": f(jd.group(3))},
           "camera_jacobian_wrt_point": {"points": int(jp.group(1)), "depth": f(jp.group(2)), "step": f(jp.group(3)),
                                         "tol": f(jp.group(4))},
           "camera_jacobian_wrt_intrinsics": {"depth": f(ji.group(1)), "step": f(ji.group(2)), "tol": f(ji.group(3))},
           "camera_jacobian_wrt_distortion": {"depth": f(jdc.group(1)), "step": f(jdc.group(2)), "tol": f(jdc.group(3))},
           "manual_projection": {"point": [f(mp.group(1)), f(mp.group(2)), f(mp.group(3))], "tol": f(mp.group(4))},
           "projection_status": status}
    with open(os.path.join(here, "camera_scenarios.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", os.path.join(here, "camera_scenarios.json"))


# maplab-common's JPL rotation-matrix known answer (the only case of
# test-quaternion-math.cc on the visual and inertial terms' path; the others
# test the inverse map, axis-angle and yaw helpers, which the path does not use).
QUAT_TEST = "common/maplab-common/test/test-quaternion-math.cc"


def quaternion_math_cases(root, here):
    text = " ".join(re.sub(r"//[^\n]*", "", open(os.path.join(root, QUAT_TEST)).read()).split())
    m = re.search(r"TEST\(QuaternionMath, toRotationMatrixJPL\) \{ Eigen::Vector4d quat_coeff_xyzw; "
                  r"quat_coeff_xyzw << ([^;]+); Eigen::Matrix3d expected_rotation_matrix; "
                  r"expected_rotation_matrix << ([^;]+); Eigen::Matrix3d rotation_matrix; "
                  r"common::toRotationMatrixJPL\(quat_coeff_xyzw, &rotation_matrix\); "
                  r"EXPECT_NEAR_EIGEN\(expected_rotation_matrix, rotation_matrix, ([^)]+)\);", text)
    out = {"generator": "tests/golden/make_golden.py", "source": QUAT_TEST,
           "toRotationMatrixJPL": {"q_xyzw": _eval_list(m.group(1)), "R_row_major": _eval_list(m.group(2)),
                                   "tol": float(m.group(3))}}
    with open(os.path.join(here, "quaternion_math.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", os.path.join(here, "quaternion_math.json"))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MAPLAB_REFERENCE_ROOT")
    if not root or not os.path.isdir(root):
        sys.exit("usage: make_golden.py <maplab source root> (or set MAPLAB_REFERENCE_ROOT)")
    main(root)
