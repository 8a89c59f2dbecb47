"""Landmark quality filter (isVisualLandmarkWellConstrained) in the CPU
oracle, checked against an independent numpy computation of the same metric
(camera centres and landmark positions in the global frame from the JPL state
conventions, signed distance of the closest observer, maximum disparity angle
of the incidence rays), and the elq_* defaults through the C ABI."""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth


def jpl_R(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)],
                     [2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w)],
                     [2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)]])


def numpy_quality(m, min_obs=4, min_angle=5.0, max_d=40.0, min_d=0.05):
    d = m.desc
    kx = m.array("kf_q_IM_p_MI"); kmis = m.array("kf_mission"); mis = m.array("mission_q_GM_p_GM")
    lp = m.array("lm_p_B"); store = m.array("lm_store_keyframe")
    olm, okf, ocam = m.array("obs_landmark"), m.array("obs_keyframe"), m.array("obs_camera")
    cams = [d.cameras[c] for c in range(d.num_cameras)]
    RIM = np.array([jpl_R(q[:4]) for q in kx]); RGM = np.array([jpl_R(q[:4]) for q in mis])
    RCI = np.array([jpl_R(np.array(c.q_CI_p_CI[:4])) for c in cams]); pCI = np.array([c.q_CI_p_CI[4:7] for c in cams])

    def to_G(k, p_M):
        return RGM[kmis[k]] @ p_M + mis[kmis[k], 4:]

    def to_M(k, p_G):
        return RGM[kmis[k]].T @ (p_G - mis[kmis[k], 4:])

    good = np.zeros(d.num_landmarks, dtype=bool)
    by_lm = [[] for _ in range(d.num_landmarks)]
    for i, l in enumerate(olm):
        by_lm[l].append(i)
    for l in range(d.num_landmarks):
        obs = by_lm[l]
        if len(obs) < min_obs or not obs:
            continue
        st = store[l]
        pG = to_G(st, RIM[st].T @ lp[l] + kx[st, 4:])
        rays, sd = [], np.inf
        for i in obs:
            k, c = okf[i], ocam[i]
            pIC = -RCI[c].T @ pCI[c]
            cG = to_G(k, RIM[k].T @ pIC + kx[k, 4:])
            pC = RCI[c] @ (RIM[k] @ (to_M(k, pG) - kx[k, 4:])) + pCI[c]
            r = cG - pG
            dist = np.linalg.norm(r)
            sd = min(sd, -dist if pC[2] < 0 else dist)
            if dist > 0:
                rays.append(r / dist)
        if sd > max_d or sd < min_d:
            continue
        if len(rays) < 2:
            angle = 0.0
        else:
            R = np.array(rays)
            C = np.abs(R @ R.T)
            iu = np.triu_indices(len(rays), 1)
            angle = np.degrees(np.arccos(min(1.0, C[iu].min())))
        good[l] = angle >= min_angle
    return good


@pytest.fixture(scope="module", params=["c1", "multi"])
def qmap(request):
    if request.param == "c1":
        return synth.generate("c1")
    return synth.generate("c4", num_missions=3, keyframes_per_mission=60, num_landmarks=1500,
                          shared_landmark_fraction=0.3)


def test_oracle_matches_numpy_restatement(qmap):
    o = O.OracleProblem(qmap.desc)
    opts = ba.default_landmark_quality_options()
    got = o.landmark_quality(opts)
    ref = numpy_quality(qmap)
    # Both sides use FP64 and the same thresholds; a flip needs a metric within
    # rounding of a threshold.
    assert (got != ref).sum() == 0, np.flatnonzero(got != ref)[:10]
    assert 0 < got.sum() < len(got)  # the filter keeps some landmarks and drops others


def test_options_change_the_verdict(qmap):
    o = O.OracleProblem(qmap.desc)
    base = o.landmark_quality(ba.default_landmark_quality_options())
    none = o.landmark_quality(ba.default_landmark_quality_options(min_observation_angle_deg=181.0))
    assert not none.any()
    loose = o.landmark_quality(ba.default_landmark_quality_options(
        min_observers=0, min_observation_angle_deg=-1.0, max_distance_from_closest_observer=1e30,
        min_distance_from_closest_observer=-1e30))
    counts = np.bincount(qmap.array("obs_landmark"), minlength=qmap.desc.num_landmarks)
    np.testing.assert_array_equal(loose, counts > 0)
    fewer = o.landmark_quality(ba.default_landmark_quality_options(min_observers=6))
    assert not (fewer & ~base).any() and fewer.sum() <= base.sum()
    # a tight reprojection bound removes landmarks with a noisy observation
    tight = o.landmark_quality(ba.default_landmark_quality_options(max_reprojection_error_px=0.5))
    assert not (tight & ~base).any() and tight.sum() < base.sum()


def test_defaults_are_the_elq_flags():
    o = ba.default_landmark_quality_options()
    assert (o.min_observers, o.min_observation_angle_deg, o.max_distance_from_closest_observer,
            o.min_distance_from_closest_observer, o.max_reprojection_error_px) == (4, 5.0, 40.0, 0.05, -1.0)
