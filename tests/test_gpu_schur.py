"""Reduced camera system (Schur complement of the landmarks) on the device
against the oracle's dense restatement.

The oracle forms S = (J_c^T J_c + D_c) - W V^-1 W^T block by block in FP64
following Ceres's SchurEliminator (the reference's SPARSE_SCHUR path), with
the same Jacobi scaling and LM damping as the first LM iteration.  Bar: FP64
device system within 1e-9 relative (Frobenius, whole matrix) of the oracle;
the FP32 (mixed) system within 1e-4 relative.
"""
import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu


def _dense(sysd, nk):
    """Assembles the device export (diag, upper pose blocks, inertial blocks)
    into one dense symmetric matrix."""
    n = 15 * nk
    A = np.zeros((n, n))
    for k in range(nk):
        A[15 * k:15 * k + 15, 15 * k:15 * k + 15] = sysd["diag"][k]
    for (i, j), B in zip(sysd["upper_ij"], sysd["upper"]):
        A[15 * i:15 * i + 6, 15 * j:15 * j + 6] += B
        A[15 * j:15 * j + 6, 15 * i:15 * i + 6] += B.T
    for f, t, E in zip(sysd["edge_from"], sysd["edge_to"], sysd["inertial"]):
        A[15 * f:15 * f + 15, 15 * t:15 * t + 15] += E
        A[15 * t:15 * t + 15, 15 * f:15 * f + 15] += E.T
    return A


@pytest.fixture(scope="module", params=[2, 1], ids=["one_thread_per_chunk", "two_threads_per_chunk"])
def c1_systems(request):
    """The system built by either Schur pair kernel (schur_split 2 / 1)."""
    m = synth.generate("c1")
    o = O.OracleProblem(m.desc)
    radius = 1e4
    Ao, bo = o.reduced_system(N.default_solver_options(), radius)
    with ba.BundleAdjuster(m.desc) as g:
        g.set_tuning(schur_split=request.param)
        s64 = g.reduced_system(N.MBA_PRECISION_FP64, radius)
        s32 = g.reduced_system(N.MBA_PRECISION_MIXED, radius)
    return m.desc.num_keyframes, Ao, bo, s64, s32


@pytest.mark.parametrize("chunk", [4, 64])
def test_split_schur_kernel_matches_single(chunk):
    """Two-mission map with shared landmarks (off-diagonal and multi-chunk
    targets with atomics, diagonal targets with transposed terms): both Schur
    pair kernels give the same FP64 system to 1e-12."""
    m = synth.generate("c4", num_missions=2, keyframes_per_mission=60, num_landmarks=3000,
                       shared_landmark_fraction=0.3)
    out = []
    for split in (2, 1):
        with ba.BundleAdjuster(m.desc) as g:
            g.set_tuning(schur_split=split, schur_chunk=chunk)
            out.append(_dense(g.reduced_system(N.MBA_PRECISION_FP64, 1e4), m.desc.num_keyframes))
    rel = np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[1])
    assert rel <= 1e-12, rel


def test_reduced_system_fp64_matches_oracle(c1_systems):
    nk, Ao, bo, s64, _ = c1_systems
    A = _dense(s64, nk)
    rel = np.linalg.norm(A - Ao) / np.linalg.norm(Ao)
    assert rel <= 1e-9, rel
    relb = np.linalg.norm(s64["rhs"].ravel() - bo) / np.linalg.norm(bo)
    assert relb <= 1e-9, relb


def test_reduced_system_mixed_error_vs_fp64(c1_systems):
    nk, Ao, bo, _, s32 = c1_systems
    A = _dense(s32, nk)
    rel = np.linalg.norm(A - Ao) / np.linalg.norm(Ao)
    assert rel <= 1e-4, rel
    relb = np.linalg.norm(s32["rhs"].ravel() - bo) / np.linalg.norm(bo)
    assert relb <= 1e-3, relb


def test_reduced_system_rejects_bad_radius():
    m = synth.generate("c1")
    with ba.BundleAdjuster(m.desc) as g:
        with pytest.raises(ba.BAError):
            g.reduced_system(N.MBA_PRECISION_FP64, -1.0)
