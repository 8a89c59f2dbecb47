"""Reads the ground-truth recovery scenarios of the reference's cost-term unit
tests (as text) into a JSON fixture; called by make_golden.py.

Each TEST_F body of

  algorithms/ceres-error-terms/test/test_visual_term_test.cc
  algorithms/ceres-error-terms/test/test_mission_baseframe_visual_term_test.cc
  algorithms/ceres-error-terms/test/test_inertial_term_test.cc
  algorithms/ceres-error-terms/test/test_3keyframe_inertial_term_test.cc

(and the fixture's SetUp) is executed statement by statement by a small
interpreter that knows exactly the statement forms those files use: Eigen
vector / quaternion declarations and comma initializers, the fixture's
scalar members, constructCamera / the intrinsics map, addResidual,
SetParameterBlockConstant, and the EXPECT_* assertions.  Any statement it does
not recognise stops the extraction, so nothing is silently dropped.  Numbers
are taken from the sources; nothing is re-derived except what the sources
compute themselves (sqrt, M_PI, the AngleAxis quaternion, the gravity
formula of common::GravityProvider, normalize()).

Output per scenario: the parameter blocks with their values at the time of
the solve, the residual blocks in the order they were added, the blocks set
constant, the camera, and the assertions with their tolerances.  For the
3-keyframe inertial file, whose ground truth comes from the RK4 integrator,
the integrator inputs are recorded and the perturbations are kept as
operations applied to the integrated states.
"""
import math
import re

# Gravity magnitude of common::GravityProvider(kAltitudeZurichMeters,
# kLatitudeZurichDegrees) (maplab-common/src/gravity-provider.cc:10-23; the
# location constants in gravity-provider.h:9-12).
ZURICH_ALTITUDE_M = 392.0
ZURICH_LATITUDE_DEG = 47.22


def gravity_magnitude(alt=ZURICH_ALTITUDE_M, lat=ZURICH_LATITUDE_DEG):
    phi = lat * math.pi / 180.0
    s2 = math.sin(phi) ** 2
    s22 = math.sin(2 * phi) ** 2
    return 9.780327 * (1 + 0.0053024 * s2 - 0.0000058 * s22) - 3.155 * 1e-7 * alt


class Unsupported(RuntimeError):
    pass


def _strip_comments(text):
    return re.sub(r"//[^\n]*", "", text)


def _bodies(text):
    """[(name, body)] of the TEST_F blocks plus ("SetUp", body)."""
    text = _strip_comments(text)
    out = []
    m = re.search(r"virtual void SetUp\(\)\s*\{", text)
    if m:
        out.append(("SetUp", _block(text, m.end() - 1)))
    for m in re.finditer(r"TEST_F\(\s*\w+,\s*(\w+)\)\s*\{", text):
        out.append((m.group(1), _block(text, m.end() - 1)))
    return out


def _block(text, i):
    """Text between the brace at i and its match."""
    assert text[i] == "{"
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[i + 1:j]
    raise ValueError("unbalanced braces")


def _statements(body):
    """Statements split at top-level semicolons; a for loop over .cols() is
    unrolled (its body repeated with the index substituted)."""
    body = " ".join(body.split())
    body = re.sub(r"\(\s+", "(", re.sub(r"\s+\)", ")", body))
    out = []
    i = 0
    while i < len(body):
        m = re.match(r"\s*for \(unsigned int (\w+) = 0; \1 < (\w+)\.cols\(\); \+\+\1\) \{", body[i:])
        if m:
            start = i + m.end() - 1
            inner = _block(body, start)
            out.append(("for", m.group(1), m.group(2), _statements(inner)))
            i = start + len(inner) + 2
            continue
        depth = 0
        j = i
        while j < len(body):
            c = body[j]
            if c in "([{":
                depth += 1
            elif c in ")]}":
                depth -= 1
            elif c == ";" and depth == 0:
                break
            j += 1
        s = body[i:j].strip()
        if s:
            out.append(s)
        i = j + 1
    return out


def _split_args(s):
    parts, depth, cur = [], 0, ""
    for c in s:
        if c in "([{":
            depth += 1
        elif c in ")]}":
            depth -= 1
        if c == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += c
    if cur.strip():
        parts.append(cur.strip())
    return parts


class Interp:
    """Executes the statements of one fixture + test body."""

    def __init__(self, kind, setup_env=None):
        self.kind = kind  # "visual" | "inertial" | "inertial3"
        self.env = dict(setup_env or {})
        self.residuals = []
        self.constant = []
        self.expect = []
        self.solved = False
        self.ops = []          # inertial3: perturbations of the integrated states
        self.truth_refs = {}   # inertial3: name -> ("state", block) copies of ground truth
        self.intrinsics_alias = False

    # ---- expressions
    def _scalar_env(self):
        env = {k: v for k, v in self.env.items() if isinstance(v, (int, float))}
        env.update({"sqrt": math.sqrt, "M_PI": math.pi, "cos": math.cos, "sin": math.sin})
        return env

    def scalar(self, expr):
        e = expr.strip()
        if not re.fullmatch(r"[\w\s\.\+\-\*/\(\)eE]+", e):
            raise Unsupported(f"expression {expr!r}")
        return float(eval(e, {"__builtins__": {}}, self._scalar_env()))

    def value(self, expr):
        """A scalar or a list (vector / quaternion coefficients)."""
        e = expr.strip()
        m = re.fullmatch(r"(\w+)\.coeffs\(\)", e)
        if m:
            return list(self.env[m.group(1)])
        m = re.fullmatch(r"Eigen::Vector(\d)d\((.*)\)", e)
        if m:
            v = [self.scalar(a) for a in _split_args(m.group(2))]
            assert len(v) == int(m.group(1))
            return v
        if re.fullmatch(r"\w+", e) and isinstance(self.env.get(e), list):
            return list(self.env[e])
        return self.scalar(e)

    def block_ref(self, expr):
        """Name of the parameter block an argument points at."""
        e = expr.strip()
        for pat in (r"(\w+)\.coeffs\(\)\.data\(\)", r"(\w+)\.data\(\)"):
            m = re.fullmatch(pat, e)
            if m:
                return m.group(1)
        m = re.fullmatch(r"(\w+)\.col\((\w+)\)\.data\(\)", e)
        if m:
            return f"{m.group(1)}[{int(self.scalar(m.group(2)))}]"
        if e == "camera_->getParametersMutable()":
            return "intrinsics"
        if e == "camera_->getDistortionMutable()->getParametersMutable()":
            return "distortion"
        raise Unsupported(f"block reference {expr!r}")

    def vec_ref(self, expr):
        e = expr.strip()
        m = re.fullmatch(r"(\w+)\.col\((\w+)\)", e)
        if m:
            return list(self.env[m.group(1)][int(self.scalar(m.group(2)))])
        return list(self.env[e])

    # ---- statements
    def run(self, stmts):
        for s in stmts:
            if isinstance(s, tuple):
                _, var, mat, inner = s
                for i in range(len(self.env[mat])):
                    self.env[var] = i
                    self.run(inner)
                continue
            self.stmt(s)

    def stmt(self, s):
        env = self.env
        if self.kind == "inertial3" and self._integrator_stmt(s):
            return
        m = re.fullmatch(r"Eigen::Quaterniond (\w+)\(Eigen::AngleAxisd\((.*), Eigen::Vector3d::Unit([XYZ])\(\)\)\)", s)
        if m:  # Hamilton quaternion of an angle-axis rotation, coefficients xyzw
            a = self.scalar(m.group(2))
            ax = {"X": 0, "Y": 1, "Z": 2}[m.group(3)]
            q = [0.0, 0.0, 0.0, math.cos(a / 2)]
            q[ax] = math.sin(a / 2)
            env[m.group(1)] = q
            return
        m = re.fullmatch(r"Eigen::Quaterniond (\w+)\((.*)\)", s)
        if m:  # Eigen's (w, x, y, z) constructor; stored as coeffs() = x y z w
            w, x, y, z = (self.scalar(a) for a in _split_args(m.group(2)))
            env[m.group(1)] = [x, y, z, w]
            return
        m = re.fullmatch(r"Eigen::Vector(\d)d (\w+)\((.*)\)", s)
        if m:
            v = [self.scalar(a) for a in _split_args(m.group(3))]
            assert len(v) == int(m.group(1))
            env[m.group(2)] = v
            return
        m = re.fullmatch(r"Eigen::Vector3d (\w+) = (\w+)", s)
        if m:  # a copy of a ground-truth vector (3-keyframe inertial file)
            env[m.group(1)] = list(env[m.group(2)])
            self.truth_refs[m.group(1)] = m.group(2)
            return
        m = re.fullmatch(r"Eigen::Vector4d (\w+) = (\w+)\.coeffs\(\)", s)
        if m:
            env[m.group(1)] = list(env[m.group(2)])
            self.truth_refs[m.group(1)] = m.group(2)
            return
        if re.fullmatch(r"Eigen::Matrix<double, 7, 1> \w+", s) or re.fullmatch(r"Eigen::Vector4d intrinsics", s):
            env[s.split()[-1]] = None
            return
        m = re.fullmatch(r"Eigen::Matrix3d (\w+)", s)
        if m:
            env[m.group(1)] = [[0.0] * 3 for _ in range(3)]
            return
        m = re.fullmatch(r"Eigen::Matrix<double, 2, 3> (\w+)", s)
        if m:
            env[m.group(1)] = [[0.0] * 2 for _ in range(3)]
            return
        if s == "Eigen::Map<Eigen::Vector4d> intrinsics(camera_->getParametersMutable())":
            self.intrinsics_alias = True
            env["intrinsics"] = list(env["camera"]["intrinsics"])
            return
        m = re.fullmatch(r"(\w+)\.col\((\d)\) = Eigen::Vector(\d)d\((.*)\)", s)
        if m:
            env[m.group(1)][int(m.group(2))] = [self.scalar(a) for a in _split_args(m.group(4))]
            return
        m = re.fullmatch(r"const double (\w+) = (.*)", s)
        if m:
            env[m.group(1)] = self.scalar(m.group(2))
            return
        m = re.fullmatch(r"(\w+)\.coeffs\(\) (\+?)= (.*)", s)
        if m:
            name, add, rhs = m.groups()
            if rhs.strip().startswith("next_state"):
                raise Unsupported(s)
            v = self.value(rhs) if rhs.strip().startswith("Eigen::") else [self.scalar(a) for a in _split_args(rhs)]
            if add:
                self.ops.append({"op": "add", "block": name, "value": v})
                env[name] = [a + b for a, b in zip(env[name], v)]
            else:
                env[name] = v
            return
        m = re.fullmatch(r"(\w+)\.coeffs\(\) << (.*)", s)
        if m:
            env[m.group(1)] = [self.scalar(a) for a in _split_args(m.group(2))]
            return
        m = re.fullmatch(r"(\w+) \+= (Eigen::Vector3d\(.*\))", s)
        if m:
            v = self.value(m.group(2))
            self.ops.append({"op": "add", "block": m.group(1), "value": v})
            env[m.group(1)] = [a + b for a, b in zip(env[m.group(1)], v)]
            return
        m = re.fullmatch(r"(\w+) << (.*)", s)
        if m:
            name = m.group(1)
            vals = []
            for a in _split_args(m.group(2)):
                v = self.value(a)
                vals += v if isinstance(v, list) else [v]
            if name == "intrinsics":
                assert len(vals) == 4
                env["intrinsics"] = vals
                if self.intrinsics_alias:
                    env["camera"]["intrinsics"] = list(vals)
            else:
                env[name] = vals  # imu_data_*: row-major 6 x n (Eigen comma initializer)
            return
        m = re.fullmatch(r"(\w+) = (.*)", s)
        if m and m.group(1).endswith("_"):
            rhs = m.group(2).strip()
            if rhs == "gravity_provider.getGravityMagnitude()":
                env[m.group(1)] = gravity_magnitude()
            else:
                env[m.group(1)] = self.scalar(rhs)
            return
        m = re.fullmatch(r"(\w+)\.(setZero|setIdentity)\(\)", s)
        if m:
            env[m.group(1)] = [0.0, 0.0, 0.0, 1.0] if m.group(2) == "setIdentity" else [0.0, 0.0, 0.0]
            return
        m = re.fullmatch(r"(\w+)\.normalize\(\)", s)
        if m:
            q = env[m.group(1)]
            n = math.sqrt(sum(x * x for x in q))
            env[m.group(1)] = [x / n for x in q]
            if self.kind == "inertial3":
                self.ops.append({"op": "normalize", "block": m.group(1)})
            return
        if s == "constructCamera()":
            env["camera"] = {"intrinsics": [env["fu_"], env["fv_"], env["cu_"], env["cv_"]],
                             "width": env["res_u_"], "height": env["res_v_"],
                             "fisheye_w": env["distortion_param_"]}
            return
        if s == "camera_->setParameters(intrinsics)":
            env["camera"]["intrinsics"] = list(env["intrinsics"])
            return
        m = re.fullmatch(r"addResidual\((.*)\)", s)
        if m:
            args = _split_args(m.group(1))
            if self.kind == "visual":
                kp, sigma, base, imu, qci, pci, lm = args
                self.residuals.append({
                    "keypoint": self.vec_ref(kp), "sigma": self.scalar(sigma),
                    "landmark_base_pose": self.block_ref(base), "imu_pose": self.block_ref(imu),
                    "q_CI": self.block_ref(qci), "p_CI": self.block_ref(pci), "landmark": self.block_ref(lm)})
            else:
                assert not args
                self.residuals.append({"inertial": True})
            self._snapshot()
            return
        m = re.fullmatch(r"problem_\.SetParameterBlockConstant\((.*)\)", s)
        if m:
            self.constant.append(self.block_ref(m.group(1)))
            return
        if s in ("solveProblem()", "solve()"):
            self.solved = True
            self._snapshot()
            return
        if s.startswith("EXPECT_"):
            self.expect.append(self.expectation(s))
            return
        if s.startswith("common::GravityProvider gravity_provider("):
            return  # the magnitude is read by getGravityMagnitude() below
        raise Unsupported(s)

    def _integrator_stmt(self, s):
        """The 3-keyframe fixture's ground-truth integration: the integrator
        calls are recorded (the fixture JSON carries their inputs) and the
        states they produce are marked as integrator output (NaN here)."""
        if (s.startswith("imu_integrator::ImuIntegratorRK4 integrator(") or s.startswith("current_state")
                or re.fullmatch(r"Eigen::Matrix<double, [^>]*> (current_state|debiased_imu_readings|next_state|"
                                r"next_phi|next_cov)", s)):
            return True
        if s.startswith("integrator.integrate("):
            self.integrations = getattr(self, "integrations", 0) + 1
            return True
        m = re.fullmatch(r"(\w+)(\.coeffs\(\))? = next_state\.block<(\d), 1>\(imu_integrator::kState(\w+)Offset, 0\)", s)
        if m:
            name, n, field = m.group(1), int(m.group(3)), m.group(4)
            self.env[name] = [float("nan")] * n
            self.truth_of = getattr(self, "truth_of", {})
            self.truth_of[name] = {"integration": self.integrations, "field": field}
            return True
        return False

    def _snapshot(self):
        """Block values as they stand (the last snapshot before solve wins)."""
        blocks = {}
        for k, v in self.env.items():
            if isinstance(v, list) and not k.startswith(("imu_data", "imu_timestamps")):
                blocks[k] = v
        self.blocks = blocks

    def expectation(self, s):
        m = re.fullmatch(r"EXPECT_(EQ|LT)\(summary_\.(final_cost|iterations\.size\(\)), (.*)\)", s)
        if m:
            what = "final_cost" if m.group(2) == "final_cost" else "iterations"
            return {"kind": f"{what}_{m.group(1).lower()}", "value": self.scalar(m.group(3).rstrip("u"))}
        m = re.fullmatch(r"EXPECT_NEAR_EIGEN\((.*)\)", s)
        if m:
            a, b, tol = _split_args(m.group(1))
            out = {"kind": "near", "tol": self.scalar(tol)}
            out.update(self._slice(a))
            bref = b.strip()
            if re.fullmatch(r"\w+", bref) and (bref in self.truth_refs or bref.endswith("_")):
                if bref in self.truth_refs:
                    out["truth"] = self.truth_refs[bref]
                elif bref.endswith("_baseframe_"):
                    out["other_block"] = bref  # both sides read after the solve
                else:
                    out["value"] = list(self.env[bref])
            else:
                out["value"] = self.value(bref)
            return out
        m = re.fullmatch(r"EXPECT_ZERO_EIGEN\((.*)\)", s)
        if m:
            a, tol = _split_args(m.group(1))
            out = {"kind": "near", "tol": self.scalar(tol)}
            out.update(self._slice(a))
            out["value"] = [0.0] * (out["end"] - out["begin"]) if "end" in out else "zeros"
            return out
        m = re.fullmatch(r"EXPECT_NEAR\((\w+)\.head\(4\)\.norm\(\), (.*), (.*)\)", s)
        if m:
            return {"kind": "quat_norm", "block": m.group(1), "value": self.scalar(m.group(2)),
                    "tol": self.scalar(m.group(3))}
        m = re.fullmatch(r"EXPECT_NEAR\(\*\(camera_->getDistortionMutable\(\)->getParametersMutable\(\)\), (.*), (.*)\)", s)
        if m:
            return {"kind": "near", "block": "distortion", "begin": 0, "end": 1,
                    "value": [self.scalar(m.group(1))], "tol": self.scalar(m.group(2))}
        m = re.fullmatch(r"EXPECT_NEAR_KINDR_QUATERNION\((.*)\)", s)
        if m:
            a, b, tol = _split_args(m.group(1))
            ma = re.fullmatch(r"pose::Quaternion\((.*)\)", a)
            mb = re.fullmatch(r"pose::Quaternion\((.*)\)", b)
            if not (ma and mb):
                raise Unsupported(s)
            inner = ma.group(1).strip()
            mm = re.fullmatch(r"Eigen::Map<Eigen::Quaternion<double>>\((\w+)\.head\(4\)\.data\(\)\)", inner)
            name = mm.group(1) if mm else inner
            if not re.fullmatch(r"\w+", name):
                raise Unsupported(s)
            w, x, y, z = (self.scalar(v) for v in _split_args(mb.group(1)))
            return {"kind": "quat", "block": name, "value": [x, y, z, w], "tol": self.scalar(tol)}
        raise Unsupported(s)

    def _slice(self, a):
        a = a.strip()
        m = re.fullmatch(r"(\w+)\.(head|tail)\((\d)\)", a)
        if m:
            name, which, n = m.group(1), m.group(2), int(m.group(3))
            size = 7 if name.endswith("pose") or name.endswith("pose_") or re.fullmatch(r"pose\d_", name) else 3
            if re.fullmatch(r"pose\d_", name) or name.endswith("_pose") or name.endswith("pose"):
                size = 7
            return {"block": name, "begin": 0 if which == "head" else size - n, "end": n if which == "head" else size}
        if re.fullmatch(r"\w+", a):
            v = self.env.get(a)
            return {"block": a, "begin": 0, "end": len(v) if isinstance(v, list) else None}
        raise Unsupported(a)


def _fixture_constants(text):
    """Blocks the fixture's addResidual method sets constant for every test."""
    text = _strip_comments(text)
    m = re.search(r"void PosegraphErrorTerms::addResidual\([^)]*\)\s*\{", text)
    body = _block(text, m.end() - 1)
    return re.findall(r"SetParameterBlockConstant\(\s*(\w+)\.data\(\)\s*\)", body)


def _run_file(path, kind):
    text = open(path).read()
    fixture_constant = _fixture_constants(text)
    bodies = _bodies(text)
    setup = Interp(kind)
    out = []
    for name, body in bodies:
        if name == "SetUp":
            setup.run(_statements(body))
            continue
        it = Interp(kind, setup_env=setup.env)
        it.env = {k: (list(v) if isinstance(v, list) else (dict(v) if isinstance(v, dict) else v))
                  for k, v in setup.env.items()}
        it.run(_statements(body))
        assert it.solved, name
        sc = {"name": name, "blocks": it.blocks, "residuals": it.residuals,
              "constant": sorted(set(it.constant) | set(fixture_constant)), "expect": it.expect}
        if "camera" in it.env:
            sc["camera"] = it.env["camera"]
        if kind != "visual":
            sc["gravity"] = it.env["gravity_magnitude_"]
        if kind == "inertial":
            sc["imu_timestamps_ns"] = it.env["imu_timestamps_"]
            sc["imu_data_row_major_6xn"] = it.env["imu_data_"]
        if kind == "inertial3":
            sc["ops"] = it.ops
        out.append(sc)
    return out, setup.env, getattr(setup, "truth_of", {})


def extract(root):
    base = f"{root}/algorithms/ceres-error-terms/test"
    scen = {"generator": "tests/golden/make_golden.py (tests/golden/error_term_scenarios.py)"}
    v, _, _ = _run_file(f"{base}/test_visual_term_test.cc", "visual")
    scen["visual_local_mission"] = {"source": "algorithms/ceres-error-terms/test/test_visual_term_test.cc",
                                    "error_type": "kLocalMission", "scenarios": v}
    b, _, _ = _run_file(f"{base}/test_mission_baseframe_visual_term_test.cc", "visual")
    scen["visual_global"] = {"source": "algorithms/ceres-error-terms/test/test_mission_baseframe_visual_term_test.cc",
                             "error_type": "kGlobal", "scenarios": b}
    i, _, _ = _run_file(f"{base}/test_inertial_term_test.cc", "inertial")
    scen["inertial_two_keyframes"] = {"source": "algorithms/ceres-error-terms/test/test_inertial_term_test.cc",
                                      "scenarios": i}
    i3, env3, truth_of = _run_file(f"{base}/test_3keyframe_inertial_term_test.cc", "inertial3")
    # The 3-keyframe fixture integrates its ground truth with the RK4
    # integrator (test_3keyframe_inertial_term_test.cc:20-75): one step of
    # delta_time_seconds from (rot0_, velocity0_, pos0_) with the debiased
    # readings, then a second step from the result.
    text = _strip_comments(open(f"{base}/test_3keyframe_inertial_term_test.cc").read())
    rd = re.search(r"debiased_imu_readings << (.*?);", " ".join(text.split())).group(1)
    env = dict(env3)
    it = Interp("inertial3", env)
    readings = [it.scalar(a) for a in _split_args(rd)]
    dt = it.scalar(re.search(r"const double delta_time_seconds = (.*?);", text).group(1))
    scen["inertial_three_keyframes"] = {
        "source": "algorithms/ceres-error-terms/test/test_3keyframe_inertial_term_test.cc",
        "ground_truth": {"rot0": env3["rot0_"], "velocity0": env3["velocity0_"], "pos0": env3["pos0_"],
                         "readings": readings, "dt": dt, "gravity": env3["gravity_magnitude_"],
                         "imu_timestamps_01_ns": env3["imu_timestamps_01_"],
                         "imu_timestamps_12_ns": env3["imu_timestamps_12_"],
                         "imu_data_01_row_major_6xn": env3["imu_data_01_"],
                         "imu_data_12_row_major_6xn": env3["imu_data_12_"],
                         "states_from_integration": truth_of},
        "scenarios": i3}
    return scen
