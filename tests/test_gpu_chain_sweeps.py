"""The chain preconditioner's sweeps against a dense solve.

T is the block-tridiagonal matrix of the keyframe chains (gamma = 1,
alpha = 0): the reduced system's diagonal blocks, and between consecutive
keyframes of a chain the inertial block plus the pose-pose block.  numpy
assembles T from mba_reduced_system and mba_chain_structure and solves it
densely; the device applies T^-1 by block cyclic reduction, once with one
launch per level and once per segment size of the segmented sweeps, each
with the one-block tail's vectors in shared and in global memory.  The map
has 450 keyframes in three missions, so every segment size leaves a partial
last segment and chain ends fall inside segments.
"""
import numpy as np
import pytest

from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth

pytestmark = pytest.mark.gpu

SEGMENTS = (1, 16, 32, 64, 128, 256)


def _dense_chain(g, precision, radius):
    sys = g.reduced_system(precision=precision, radius=radius)
    perm, le, lb = g.chain_structure()
    n = len(perm)
    D, U, E, ij = sys["diag"], sys["upper"], sys["inertial"], sys["upper_ij"]
    npu = len(U)
    T = np.zeros((15 * n, 15 * n))
    for k in range(n):
        T[15 * k:15 * k + 15, 15 * k:15 * k + 15] = D[k]
    for p in range(1, n):
        k, kl = perm[p], perm[p - 1]
        C = np.zeros((15, 15))  # rows kf(p), columns kf(p - 1)
        if le[p] >= 0:
            C += E[le[p]].T
        if lb[p] >= 0:
            if lb[p] < npu:
                assert tuple(ij[lb[p]]) == (k, kl)
                C[:6, :6] += U[lb[p]]
            else:
                assert tuple(ij[lb[p] - npu]) == (kl, k)
                C[:6, :6] += U[lb[p] - npu].T
        T[15 * k:15 * k + 15, 15 * kl:15 * kl + 15] = C
        T[15 * kl:15 * kl + 15, 15 * k:15 * k + 15] = C.T
    return T


@pytest.fixture(scope="module")
def chain_map():
    return synth.generate("c4", num_missions=3, keyframes_per_mission=150, num_landmarks=6000,
                          shared_landmark_fraction=0.2)


@pytest.mark.parametrize("precision,tol", [(N.MBA_PRECISION_FP64, 1e-9), (N.MBA_PRECISION_MIXED, 2e-3)])
def test_sweeps_match_dense_solve(chain_map, precision, tol):
    m = chain_map
    radius = 1e4
    rng = np.random.default_rng(5)
    with ba.BundleAdjuster(m.desc) as g:
        T = _dense_chain(g, precision, radius)
        r = rng.standard_normal((m.desc.num_keyframes, 15))
        z_ref = np.linalg.solve(T, r.reshape(-1)).reshape(r.shape)
        out = {}
        for seg in SEGMENTS:
            for tsm in (1, 2):  # the tail's vectors in shared / global memory
                g.set_tuning(chain_segment=seg, chain_tail_smem=tsm)
                out[(seg, tsm)] = g.chain_apply(r, precision=precision, radius=radius)
    for seg, z in out.items():
        err = np.linalg.norm(z - z_ref) / np.linalg.norm(z_ref)
        assert err <= tol, (seg, err)
    if precision == N.MBA_PRECISION_FP64:
        ref = out[(1, 2)]
        for key, z in out.items():
            np.testing.assert_allclose(z, ref, rtol=0, atol=1e-9 * np.abs(ref).max(), err_msg=str(key))


def test_segment_setting_is_validated(chain_map):
    with ba.BundleAdjuster(chain_map.desc) as g:
        for bad in (3, 512, -4):
            with pytest.raises(ba.BAError):
                g.set_tuning(chain_segment=bad)
