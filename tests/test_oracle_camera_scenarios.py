"""The oracle's camera model against aslam's own camera and distortion tests
(aslam_cv2/aslam_cv_cameras/test/test-cameras.cc, test-distortions.cc), for
the models the visual term uses: pinhole with radtan, equidistant, fisheye
(FOV) or no distortion.  tests/golden/camera_scenarios.json holds the tests'
parameters (createTestDistortion, createTestCamera), points, steps and
tolerances (written by tests/golden/make_golden.py).

The Jacobian checks difference the oracle's projection numerically with the
tests' scheme (a five-point central stencil, step sqrt(step) |x_j|) and
compare element by element at the tests' tolerances.  A distortion alone is
the projection with unit focal lengths, zero principal point and depth 1.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle_lib as O
import problem_util as U
from maplab_gb300 import _native as N

HERE = os.path.dirname(os.path.abspath(__file__))
CAM = json.load(open(os.path.join(HERE, "golden", "camera_scenarios.json")))
DTYPES = {"radtan": N.MBA_DISTORTION_RADTAN, "equidistant": N.MBA_DISTORTION_EQUIDISTANT,
          "fov": N.MBA_DISTORTION_FOV}
STATUS = {"KEYPOINT_VISIBLE": 0, "KEYPOINT_OUTSIDE_IMAGE_BOX": 1, "POINT_BEHIND_CAMERA": 2, "PROJECTION_INVALID": 3}


def _camera(spec, name):
    params = CAM["distortions"][name] if name else []
    c = U.camera(fu=spec["fu"], fv=spec["fv"], cu=spec["cu"], cv=spec["cv"], w=int(spec["width"]),
                 h=int(spec["height"]), dtype=DTYPES[name] if name else N.MBA_DISTORTION_NONE,
                 dist=tuple(params) + (0.0,) * (4 - len(params)))
    return c


def _unit_camera(name):
    return _camera({"fu": 1.0, "fv": 1.0, "cu": 0.0, "cv": 0.0, "width": 1e9, "height": 1e9}, name)


def _project(cam, p):
    kp = np.zeros(2); Jp = np.zeros(6); Ji = np.zeros(8); Jd = np.zeros(8)
    st = O.load().oracle_project(ctypes.byref(cam), N.ptr(np.ascontiguousarray(p, dtype=np.float64)), N.ptr(kp),
                                 N.ptr(Jp), N.ptr(Ji), N.ptr(Jd))
    return st, kp, Jp.reshape(2, 3), Ji.reshape(2, 4), Jd.reshape(2, 4)


def _numdiff(f, x, step):
    """Five-point central stencil with h = sqrt(step) |x_j| (sqrt(step) where x_j = 0)."""
    eps = np.sqrt(max(step, np.finfo(float).eps))
    x = np.asarray(x, dtype=np.float64)
    cols = []
    for j in range(len(x)):
        h = eps * abs(x[j]) or eps
        e = np.zeros_like(x)
        e[j] = h
        cols.append((8 * f(x + e) + f(x - 2 * e) - f(x + 2 * e) - 8 * f(x - e)) / (12 * h))
    return np.stack(cols, axis=1)


@pytest.mark.parametrize("name", sorted(DTYPES))
def test_distortion_jacobian_wrt_keypoint(name):
    spec = CAM["distortion_jacobian_wrt_keypoint"]
    cam = _unit_camera(name)
    k = np.asarray(spec["keypoint"])
    _, _, Jp, _, _ = _project(cam, [k[0], k[1], 1.0])
    Jn = _numdiff(lambda kk: _project(cam, [kk[0], kk[1], 1.0])[1], k, spec["step"])
    assert np.abs(Jn - Jp[:, :2]).max() <= spec["tol"]


@pytest.mark.parametrize("name", sorted(DTYPES))
def test_distortion_jacobian_wrt_parameters(name):
    spec = CAM["distortion_jacobian_wrt_parameters"]
    params = np.asarray(CAM["distortions"][name])
    k = spec["keypoint"]

    def f(prm):
        c = _unit_camera(name)
        for i, v in enumerate(prm):
            c.distortion[i] = v
        return _project(c, [k[0], k[1], 1.0])[1]

    _, _, _, _, Jd = _project(_unit_camera(name), [k[0], k[1], 1.0])
    Jn = _numdiff(f, params, spec["step"])
    assert np.abs(Jn - Jd[:, :len(params)]).max() <= spec["tol"]


def _visible_points(cam, depth, n, seed):
    """Points at the given depth whose projection is in the image."""
    rng = np.random.default_rng(seed)
    spec = CAM["test_camera"]
    out = []
    while len(out) < n:
        u, v = rng.uniform(0, spec["width"]), rng.uniform(0, spec["height"])
        p = np.array([(u - spec["cu"]) / spec["fu"], (v - spec["cv"]) / spec["fv"], 1.0]) * depth
        if _project(cam, p)[0] == STATUS["KEYPOINT_VISIBLE"]:
            out.append(p)
    return out


@pytest.mark.parametrize("name", sorted(DTYPES) + [None], ids=lambda n: n or "none")
def test_camera_jacobian_wrt_point(name):
    spec = CAM["camera_jacobian_wrt_point"]
    cam = _camera(CAM["test_camera"], name)
    for p in _visible_points(cam, spec["depth"], spec["points"], seed=1):
        _, _, Jp, _, _ = _project(cam, p)
        Jn = _numdiff(lambda x: _project(cam, x)[1], p, spec["step"])
        assert np.abs(Jn - Jp).max() <= spec["tol"]


@pytest.mark.parametrize("name", sorted(DTYPES) + [None], ids=lambda n: n or "none")
def test_camera_jacobian_wrt_intrinsics(name):
    spec = CAM["camera_jacobian_wrt_intrinsics"]
    base = CAM["test_camera"]
    p = _visible_points(_camera(base, name), spec["depth"], 1, seed=2)[0]

    def f(intr):
        return _project(_camera(dict(base, fu=intr[0], fv=intr[1], cu=intr[2], cv=intr[3]), name), p)[1]

    intr = np.array([base["fu"], base["fv"], base["cu"], base["cv"]])
    _, _, _, Ji, _ = _project(_camera(base, name), p)
    assert np.abs(_numdiff(f, intr, spec["step"]) - Ji).max() <= spec["tol"]


@pytest.mark.parametrize("name", sorted(DTYPES))
def test_camera_jacobian_wrt_distortion(name):
    spec = CAM["camera_jacobian_wrt_distortion"]
    base = CAM["test_camera"]
    params = np.asarray(CAM["distortions"][name])
    p = _visible_points(_camera(base, name), spec["depth"], 1, seed=3)[0]

    def f(prm):
        c = _camera(base, name)
        for i, v in enumerate(prm):
            c.distortion[i] = v
        return _project(c, p)[1]

    _, _, _, _, Jd = _project(_camera(base, name), p)
    assert np.abs(_numdiff(f, params, spec["step"]) - Jd[:, :len(params)]).max() <= spec["tol"]


def test_manual_projection_without_distortion():
    spec = CAM["manual_projection"]
    c = CAM["plain_camera"]
    kx, ky, kz = spec["point"]
    st, kp, _, _, _ = _project(_camera(c, None), [kx, ky, kz])
    assert st == STATUS["KEYPOINT_VISIBLE"]
    manual = np.array([c["fu"] * (kx / kz) + c["cu"], c["fv"] * (ky / kz) + c["cv"]])
    assert np.abs(kp - manual).max() <= spec["tol"]


@pytest.mark.parametrize("case", CAM["projection_status"], ids=lambda c: c["status"])
def test_projection_status(case):
    st = _project(_camera(CAM["plain_camera"], None), case["point"])[0]
    assert st == STATUS[case["status"]]
