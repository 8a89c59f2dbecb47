"""The CPU oracle against the reference's own known-answer vectors.

Golden values come from algorithms/imu-integrator-rk4/test/*.cc (extracted
verbatim by tests/golden/make_golden.py) and are checked at the tolerances
those tests use.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "imu_integrator.json")))


def _integrate(noise5, state, readings, dt):
    lib = O.load()
    nxt = np.zeros(16); phi = np.zeros(225); cov = np.zeros(225)
    n = O.arr(noise5); s = O.arr(state); r = O.arr(readings)
    lib.oracle_imu_integrate(N.ptr(n), N.ptr(s), N.ptr(r), ctypes.c_double(dt), N.ptr(nxt), N.ptr(phi), N.ptr(cov))
    return nxt, phi.reshape(15, 15), cov.reshape(15, 15)


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=lambda c: c["name"])
def test_rk4_phi_cov_golden(case):
    nxt, phi, cov = _integrate(case["sigmas"] + [case["gravity"]], case["state"], case["readings"], case["dt"])
    tol = case["tol"]
    np.testing.assert_allclose(nxt, case["expected_state"], rtol=0, atol=tol)
    if "expected_phi" in case:
        np.testing.assert_allclose(phi.ravel(), case["expected_phi"], rtol=0, atol=tol)
    if "expected_cov" in case:
        np.testing.assert_allclose(cov.ravel(), case["expected_cov"], rtol=0, atol=tol)


@pytest.mark.parametrize("case", GOLDEN["basic"], ids=lambda c: c["name"])
def test_rk4_basic_golden(case):
    nxt, phi, cov = _integrate([0, 0, 0, 0, case["gravity"]], case["state"], case["readings"], case["dt"])
    if "expected_state" in case:
        np.testing.assert_allclose(nxt, case["expected_state"], rtol=0, atol=case["tol"])
    if case.get("cov_zero"):
        assert np.abs(cov).max() <= 1e-15
    if "expected_quat" in case:
        np.testing.assert_allclose(nxt[:4], case["expected_quat"], rtol=0, atol=case["quat_tol"])
    if "expected_velocity" in case:
        np.testing.assert_allclose(nxt[7:10], case["expected_velocity"], rtol=0, atol=case["tol"])
        np.testing.assert_allclose(nxt[13:16], case["expected_position"], rtol=0, atol=case["tol"])


QUAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "quaternion_math.json")))


def test_jpl_rotation_matrix_golden():
    """maplab-common's toRotationMatrixJPL known answer
    (common/maplab-common/test/test-quaternion-math.cc)."""
    case = QUAT["toRotationMatrixJPL"]
    R = np.zeros(9)
    O.load().oracle_rotation_matrix(N.ptr(O.arr(case["q_xyzw"])), N.ptr(R))
    assert np.abs(R - np.asarray(case["R_row_major"])).max() <= case["tol"]
