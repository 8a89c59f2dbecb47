"""VIMap map folders (include/maplab_vimap.h) on the host: maps written by
tests/vimap_writer.py from synthetic maps are read back, exported as the BA
problem and compared with the synthetic problem itself; the landmark
selection rules, mission selection, the reference's own sensors.yaml files,
malformed input, and the optimized-state write-back with a lossless save."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle_lib as O
from maplab_gb300 import _native as N
from maplab_gb300 import ba, synth, vimap
from vimap_writer import T_inverse, from_jpl_block, make_id, quat_R, write_map

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def arr(desc, name, shape, dtype=np.float64):
    p = getattr(desc, name)
    n = int(np.prod(shape))
    if n == 0 or not p:
        return np.zeros(shape, dtype=dtype)
    return np.ctypeslib.as_array(p, shape=(n,)).reshape(shape)


def synth_index(ids):
    """Writer ids -> synthetic-map row index."""
    return (ids[:, 0] & ((1 << 48) - 1)).astype(np.int64) - 1


CASES = {
    "vi": dict(preset="c1"),
    "visual_odometry": dict(preset="c1", include_inertial=0, pose_edges=1),
    "multi_mission_graph": dict(preset="c4", num_missions=3, keyframes_per_mission=50, num_landmarks=1200,
                                shared_landmark_fraction=0.3, pose_edges=1, loop_closure_stride=7,
                                absolute_pose_stride=15),
}
ALL_TERMS = dict(landmark_selection=N.MBA_VIMAP_LANDMARKS_ALL, add_6dof_odometry_constraints=1,
                 add_absolute_pose_constraints=1, add_loop_closure_edges=1)


@pytest.fixture(scope="module", params=list(CASES))
def written(request, tmp_path_factory):
    kw = dict(CASES[request.param])
    m = synth.generate(kw.pop("preset"), **kw)
    folder = str(tmp_path_factory.mktemp(request.param) / "map")
    ids = write_map(m, folder)
    return m, folder, ids


def test_export_reproduces_the_synthetic_problem(written):
    m, folder, _ = written
    s = m.desc
    with vimap.VIMap(folder) as vm:
        info = vm.info()
        assert info["num_vertices"] == s.num_keyframes and info["num_landmarks"] == s.num_landmarks
        d = vm.export(**ALL_TERMS)
        ids = vm.export_ids()
        NK, NL, NO = s.num_keyframes, s.num_landmarks, s.num_observations
        assert (d.num_keyframes, d.num_landmarks, d.num_observations) == (NK, NL, NO)
        assert (d.num_missions, d.num_cameras, d.num_imu_edges, d.num_imu_samples) == (
            s.num_missions, s.num_cameras, s.num_imu_edges, s.num_imu_samples)
        # keyframes: the backbone order is the synthetic order
        np.testing.assert_array_equal(synth_index(ids["keyframes"]), np.arange(NK))
        for name, w in (("kf_q_IM_p_MI", 7), ("kf_v_M", 3), ("kf_b_g", 3), ("kf_b_a", 3)):
            np.testing.assert_array_equal(arr(d, name, (NK, w)), m.array(name))
        np.testing.assert_array_equal(arr(d, "kf_mission", (NK,), np.int32), m.array("kf_mission"))
        np.testing.assert_allclose(arr(d, "mission_q_GM_p_GM", (s.num_missions, 7)), m.array("mission_q_GM_p_GM"),
                                   rtol=0, atol=1e-15)
        for c in range(s.num_cameras):
            a, b = d.cameras[c], s.cameras[c]
            assert list(a.intrinsics) == list(b.intrinsics) and list(a.distortion) == list(b.distortion)
            assert (a.distortion_type, a.width, a.height) == (b.distortion_type, b.width, b.height)
            np.testing.assert_allclose(list(a.q_CI_p_CI), list(b.q_CI_p_CI), rtol=0, atol=1e-12)
        # landmarks by id
        li = synth_index(ids["landmarks"])
        assert sorted(li) == list(range(NL))
        np.testing.assert_array_equal(arr(d, "lm_p_B", (NL, 3)), m.array("lm_p_B")[li])
        np.testing.assert_array_equal(arr(d, "lm_store_keyframe", (NL,), np.int32), m.array("lm_store_keyframe")[li])
        # observations: by observer keyframe, camera, then the synthetic order
        perm = np.lexsort((np.arange(NO), m.array("obs_camera"), m.array("obs_keyframe")))
        np.testing.assert_array_equal(arr(d, "obs_uv", (NO, 2)), m.array("obs_uv")[perm])
        np.testing.assert_array_equal(arr(d, "obs_sigma", (NO,)), m.array("obs_sigma")[perm])
        np.testing.assert_array_equal(arr(d, "obs_keyframe", (NO,), np.int32), m.array("obs_keyframe")[perm])
        np.testing.assert_array_equal(arr(d, "obs_camera", (NO,), np.int32), m.array("obs_camera")[perm])
        np.testing.assert_array_equal(li[arr(d, "obs_landmark", (NO,), np.int32)], m.array("obs_landmark")[perm])
        # inertial edges and samples
        for name in ("edge_from", "edge_to", "edge_sample_offset", "imu_timestamp_ns", "imu_acc_gyro"):
            shape = m.array(name).shape
            dt = m.array(name).dtype
            np.testing.assert_array_equal(arr(d, name, shape, dt), m.array(name))
        if s.num_imu_edges:
            assert (d.gyro_noise_sigma, d.gyro_bias_sigma, d.acc_noise_sigma, d.acc_bias_sigma) == (
                s.gyro_noise_sigma, s.gyro_bias_sigma, s.acc_noise_sigma, s.acc_bias_sigma)
        assert d.gravity_magnitude == s.gravity_magnitude
        # pose edges: relative, absolute, loop closures (each group in the synthetic order)
        NP = s.num_pose_edges
        assert d.num_pose_edges == NP
        if NP:
            sty = m.array("pose_edge_type")
            order = np.concatenate([np.flatnonzero(sty == t) for t in
                                    (N.MBA_POSE_EDGE_RELATIVE, N.MBA_POSE_EDGE_ABSOLUTE,
                                     N.MBA_POSE_EDGE_LOOP_CLOSURE)])
            abs_rows = np.flatnonzero(sty[order] == N.MBA_POSE_EDGE_ABSOLUTE)
            # absolute terms follow the keyframe order
            order[abs_rows] = order[abs_rows][np.argsort(m.array("pose_edge_from")[order[abs_rows]], kind="stable")]
            np.testing.assert_array_equal(arr(d, "pose_edge_type", (NP,), np.int32), sty[order])
            for name, w in (("pose_edge_from", None), ("pose_edge_T_Bk_Bkp1", 7), ("pose_edge_covariance", 36),
                            ("pose_edge_switch", None), ("pose_edge_switch_variance", None)):
                shape = (NP,) if w is None else (NP, w)
                dt = np.int32 if name == "pose_edge_from" else np.float64
                np.testing.assert_array_equal(arr(d, name, shape, dt), m.array(name)[order], err_msg=name)
            rel = sty[order] != N.MBA_POSE_EDGE_LOOP_CLOSURE
            np.testing.assert_allclose(arr(d, "pose_edge_q_I_B_p_B_I", (NP, 7))[rel],
                                       m.array("pose_edge_q_I_B_p_B_I")[order][rel], rtol=0, atol=1e-12)
            to = arr(d, "pose_edge_to", (NP,), np.int32)
            keep = sty[order] != N.MBA_POSE_EDGE_ABSOLUTE
            np.testing.assert_array_equal(to[keep], m.array("pose_edge_to")[order][keep])
        # gauge fixes: mba_gauge_fixes of the synthetic problem
        from test_gauge_fixes import fixes
        kf0, lm0, _ = fixes(m)
        np.testing.assert_array_equal(arr(d, "kf_flags", (NK,), np.uint32), kf0)
        np.testing.assert_array_equal(arr(d, "lm_constant", (NL,), np.uint8), lm0[li])


def test_exported_cost_equals_synthetic_cost(written):
    """The oracle's cost of the exported problem equals that of the synthetic
    problem (same terms in another order)."""
    m, folder, _ = written
    with vimap.VIMap(folder) as vm:
        d = vm.export(**ALL_TERMS)
        c = O.OracleProblem(d).cost()
    c0 = O.OracleProblem(m.desc).cost()
    assert abs(c - c0) <= 1e-12 * c0, (c, c0)


def _quality_case(tmp_path, quality):
    m = synth.generate("c1")
    folder = str(tmp_path / "map")
    write_map(m, folder, quality=quality)
    return m, folder


def test_unknown_quality_is_evaluated_like_the_oracle(tmp_path):
    m, folder = _quality_case(tmp_path, 0)
    good = O.OracleProblem(m.desc).landmark_quality(ba.default_landmark_quality_options())
    assert 0 < good.sum() < len(good)
    with vimap.VIMap(folder) as vm:
        d = vm.export()
        kept = np.zeros(m.desc.num_landmarks, dtype=bool)
        kept[synth_index(vm.export_ids()["landmarks"])] = True
    np.testing.assert_array_equal(kept, good)
    assert d.num_observations == int(np.isin(m.array("obs_landmark"), np.flatnonzero(good)).sum())


@pytest.mark.parametrize("max_px", [0.8, 2.5])
def test_unknown_quality_with_the_reprojection_test(tmp_path, max_px):
    """elq_max_reprojection_error_px > 0: the host metric projects every
    observation (pinhole + distortion) like the oracle does."""
    m, folder = _quality_case(tmp_path, 0)
    q = ba.default_landmark_quality_options(max_reprojection_error_px=max_px)
    good = O.OracleProblem(m.desc).landmark_quality(q)
    base = O.OracleProblem(m.desc).landmark_quality(ba.default_landmark_quality_options())
    assert good.sum() < base.sum()  # the bound removes landmarks
    with vimap.VIMap(folder) as vm:
        vm.export(quality=dict(max_reprojection_error_px=max_px))
        kept = np.zeros(m.desc.num_landmarks, dtype=bool)
        kept[synth_index(vm.export_ids()["landmarks"])] = True
    np.testing.assert_array_equal(kept, good)


def test_quality_flags_decide_without_evaluation(tmp_path):
    q = np.where(np.arange(2000) % 3 == 0, 1, 2)  # every third landmark kBad, the rest kGood
    m, folder = _quality_case(tmp_path, q)
    with vimap.VIMap(folder) as vm:
        vm.export()
        li = synth_index(vm.export_ids()["landmarks"])
    assert set(li) == set(np.flatnonzero(q == 2))


def test_landmark_mask_and_min_landmarks_per_frame(tmp_path):
    m, folder = _quality_case(tmp_path, 2)
    with vimap.VIMap(folder) as vm:
        order = synth_index(vm.landmark_ids())
        keep = (order % 2 == 0).astype(np.uint8)
        d = vm.export(landmark_keep=keep)
        li = synth_index(vm.export_ids()["landmarks"])
        assert set(li) == set(order[keep == 1])
        # a frame count threshold above every frame's landmark count drops all visual terms
        d = vm.export(min_landmarks_per_frame=10 ** 6)
        assert d.num_observations == 0 and d.num_landmarks == 0
        # feature type: all landmarks are kBinary; asking for another type keeps none
        d = vm.export(feature_type=1)
        assert d.num_observations == 0


def test_mission_selection(tmp_path):
    m = synth.generate("c4", num_missions=3, keyframes_per_mission=40, num_landmarks=900, shared_landmark_fraction=0.3)
    folder = str(tmp_path / "map")
    write_map(m, folder)
    kmis = m.array("kf_mission")
    with vimap.VIMap(folder) as vm:
        d = vm.export(missions=[2], landmark_selection=N.MBA_VIMAP_LANDMARKS_ALL)
        ids = vm.export_ids()
        ks = synth_index(ids["keyframes"])
        np.testing.assert_array_equal(ks, np.flatnonzero(kmis == 2))
        li = synth_index(ids["landmarks"])
        assert np.all(kmis[m.array("lm_store_keyframe")[li]] == 2)
        okf, olm = m.array("obs_keyframe"), m.array("obs_landmark")
        lst = m.array("lm_store_keyframe")
        expect = int(((kmis[okf] == 2) & (kmis[lst[olm]] == 2)).sum())
        assert d.num_observations == expect
        assert d.num_missions == 1
        np.testing.assert_array_equal(synth_index(ids["missions"]), [2])
        with pytest.raises(ba.BAError) as e:
            vm.export(missions=[3])
        assert e.value.status == N.MBA_ERR_OUT_OF_RANGE_INDEX


def _sensors_only_map(folder, yaml_text, ncamera_hex, num_frames):
    """A map with one mission and one vertex whose frames carry no keypoints,
    under the given sensors.yaml."""
    from vimap_writer import f_bytes, f_doubles, f_id, f_varint
    w = bytes.fromhex(ncamera_hex)
    nc = (int.from_bytes(w[:8], "little"), int.from_bytes(w[8:], "little"))
    vid, mid, bid = make_id("vertex", 0), make_id("mission", 0), make_id("baseframe", 0)
    os.makedirs(os.path.join(folder, "vi_map"))
    frames = b"".join(f_bytes(2, f_id(1, make_id("frame", c))) for c in range(num_frames))
    vertex = (f_doubles(3, [0, 0, 0, 1, 0, 0, 0]) + f_doubles(4, [0] * 3) + f_doubles(5, [0] * 3) +
              f_doubles(6, [0] * 3) + f_bytes(7, frames) + f_bytes(8, b"") + f_id(14, mid))
    files = {
        "missions": f_id(5, mid) + f_bytes(6, f_id(1, bid) + f_id(2, vid) + f_id(8, nc)) + f_id(7, bid) +
                    f_bytes(8, f_doubles(1, [0, 0, 0, 1, 0, 0, 0])),
        "vertices0": f_id(1, vid) + f_bytes(2, vertex),
    }
    for n, b in files.items():
        with open(os.path.join(folder, "vi_map", n), "wb") as f:
            f.write(b)
    with open(os.path.join(folder, "vi_map", "vi_map_metadata"), "w") as f:
        f.write('files {\n  file_type: 0\n  path: "missions"\n}\nfiles {\n  file_type: 1\n  path: "vertices0"\n}\n')
    with open(os.path.join(folder, "vi_map", "sensors.yaml"), "w") as f:
        f.write(yaml_text)


@pytest.mark.parametrize("name, ncam", [
    ("maplab-launch/config/alphasense-dev-kit/calib/alphasense-dev-kit-sensors.yaml", 5),
    ("maplab-launch/config/lidarstick/calib/lidarstick-150-deg-cams-sensors.yaml", None),
])
def test_reference_sensor_files(tmp_path, name, ncam):
    """maplab's own calibration files (copied into tests/golden/ by
    tests/golden/make_golden.py) parse; the cameras' intrinsics and T_B_C
    come out as written there."""
    import json
    text = json.load(open(os.path.join(GOLDEN, "reference_sensors.json")))["files"][name]
    ncam_hex = re.search(r"id: ([0-9a-f]{32})\s+sensor_type: NCAMERA", text).group(1)
    block = text[text.index(ncam_hex):]
    fus = [float(x) for x in re.findall(r"intrinsics:\s+rows: 4\s+cols: 1\s+data:\s+- ([-0-9.e]+)", block)]
    n = ncam if ncam is not None else len(fus)
    _sensors_only_map(str(tmp_path / "m"), text, ncam_hex, n)
    with vimap.VIMap(str(tmp_path / "m")) as vm:
        info = vm.info()
        assert info["num_cameras"] >= n
        d = vm.export(add_inertial_constraints=0)
        assert d.num_cameras == n and d.num_observations == 0
        got = [d.cameras[c].intrinsics[0] for c in range(n)]
        b = np.array(d.cameras[0].q_CI_p_CI[:7])  # the descriptor's memory lives as long as the map
    assert got == fus[:n]
    # the first camera's T_B_C rows, against the exported JPL block
    rows = re.search(r"T_B_C:\s+rows: 4\s+cols: 4\s+data:\s+- \[([^\]]*)\]\s+- \[([^\]]*)\]\s+- \[([^\]]*)\]", block)
    M = np.array([[float(x) for x in rows.group(i).split(",")] for i in (1, 2, 3)])
    T_B_C = T_inverse(from_jpl_block(b))
    np.testing.assert_allclose(quat_R(T_B_C[:4]), M[:, :3], atol=1e-6)
    np.testing.assert_allclose(T_B_C[4:], M[:, 3], atol=1e-9)


def test_absolute_measurement_timestamp_must_match_the_vertex(tmp_path):
    """addAbsolutePoseConstraintTermsForVertices CHECKs that a measurement
    carries its vertex's timestamp; the export refuses a mismatch."""
    from vimap_writer import f_varint
    m = synth.generate("c1", absolute_pose_stride=25)
    folder = tmp_path / "map"
    write_map(m, str(folder))
    k = int(m.array("pose_edge_from")[m.array("pose_edge_type") == N.MBA_POSE_EDGE_ABSOLUTE][0])
    with vimap.VIMap(str(folder)) as vm:
        d = vm.export(add_absolute_pose_constraints=1)
        assert d.num_pose_edges > 0
    # the measurement of vertex k is stamped 1000 k: give it another time
    f = next(p for p in sorted((folder / "vi_map").iterdir()) if p.name.startswith("vertices") and
             f_varint(1, 1000 * k) + bytes([0x12]) in p.read_bytes())
    b = f.read_bytes()
    old_ts = f_varint(1, 1000 * k) + bytes([0x12])
    f.write_bytes(b.replace(old_ts, f_varint(1, 1000 * k + 1) + bytes([0x12]), 1))
    with vimap.VIMap(str(folder)) as vm:
        with pytest.raises(ba.BAError) as e:
            vm.export(add_absolute_pose_constraints=1)
        assert e.value.status == N.MBA_ERR_INVALID_ARG
        vm.export()  # without absolute terms the map exports


def test_legacy_landmark_index_ids_are_rewritten(tmp_path):
    """Legacy maps (landmark_index_ids present): the frames' landmark ids are
    replaced by those of the landmarks' back-links
    (vi-map-serialization.cc:194-212); the export equals the modern map's."""
    m = synth.generate("c1", keyframes_per_mission=40, num_landmarks=500)
    write_map(m, str(tmp_path / "new"))
    write_map(m, str(tmp_path / "old"), legacy_ids=True)
    with vimap.VIMap(str(tmp_path / "new")) as a, vimap.VIMap(str(tmp_path / "old")) as b:
        da = a.export(landmark_selection=N.MBA_VIMAP_LANDMARKS_ALL)
        db = b.export(landmark_selection=N.MBA_VIMAP_LANDMARKS_ALL)
        assert da.num_observations == db.num_observations == m.desc.num_observations
        for name, shape, dt in (("obs_landmark", (da.num_observations,), np.int32),
                                ("obs_uv", (da.num_observations, 2), np.float64),
                                ("lm_p_B", (da.num_landmarks, 3), np.float64)):
            np.testing.assert_array_equal(arr(da, name, shape, dt), arr(db, name, shape, dt))


def test_packed_encoding_reads_the_same(tmp_path):
    m = synth.generate("c1", include_inertial=0, pose_edges=1)
    for packed in (False, True):
        write_map(m, str(tmp_path / f"p{int(packed)}"), packed=packed)
    with vimap.VIMap(str(tmp_path / "p0")) as a, vimap.VIMap(str(tmp_path / "p1")) as b:
        da, db = a.export(**ALL_TERMS), b.export(**ALL_TERMS)
        for name, shape in (("obs_uv", (da.num_observations, 2)), ("lm_p_B", (da.num_landmarks, 3)),
                            ("kf_q_IM_p_MI", (da.num_keyframes, 7)), ("pose_edge_covariance", (da.num_pose_edges, 36))):
            np.testing.assert_array_equal(arr(da, name, shape), arr(db, name, shape))


def _status(folder):
    h = ctypes.c_void_p()
    st = ba.lib().mba_vimap_load(str(folder).encode(), ctypes.byref(h))
    if h.value:
        ba.lib().mba_vimap_destroy(h)
    return st


def test_malformed_maps_are_refused(tmp_path):
    m = synth.generate("c1", keyframes_per_mission=30, num_landmarks=300)
    base = tmp_path / "base"
    write_map(m, str(base))
    assert _status(base) == N.MBA_OK
    assert _status(tmp_path / "missing") == N.MBA_ERR_INVALID_ARG

    def variant(name, edit):
        import shutil
        dst = tmp_path / name
        shutil.copytree(base, dst)
        edit(dst / "vi_map")
        return _status(dst)

    def truncate(d):
        p = d / "vertices0"
        p.write_bytes(p.read_bytes()[:-5])

    def bad_meta(d):
        (d / "vi_map_metadata").write_text('files {\n  file_type: 7\n  path: "x"\n}\n')

    def escape_meta(d):
        (d / "vi_map_metadata").write_text('files {\n  file_type: 1\n  path: "../x"\n}\n')

    def bad_yaml(d):
        (d / "sensors.yaml").write_text("sensors:\n  - id: zz\n    sensor_type: IMU\n")

    def dangling_index(d):
        from vimap_writer import f_bytes, f_id
        p = d / "landmark_index"
        p.write_bytes(p.read_bytes() + f_bytes(10, f_id(1, make_id("vertex", 999)) + f_id(2, make_id("landmark", 5000))))

    def unordered_imu(d):
        from vimap_writer import f_varint
        p = d / "edges0"
        b = p.read_bytes()
        # first viwls edge: swap the encodings of its first two timestamps
        t0, t1 = (f_varint(3, int(t)) for t in m.array("imu_timestamp_ns")[:2])
        i = b.index(t0 + t1)
        p.write_bytes(b[:i] + t1 + t0 + b[i + len(t0) + len(t1):])

    def deep_yaml(d):
        (d / "sensors.yaml").write_text("".join(" " * i + "a:\n" for i in range(200)) + " " * 200 + "b: 1\n")

    def dangling_outgoing(d):
        from vimap_writer import f_bytes, f_id, make_id
        # vertices0's first vertex names an edge that does not exist
        p = d / "vertices0"
        b = p.read_bytes()
        vid = f_id(1, make_id("vertex", 0))
        assert b.startswith(vid)
        # the vertex message follows the id: prepend an outgoing edge id to its body
        rest = b[len(vid):]
        assert rest[0] == 0x12  # field 2, length-delimited
        from vimap_writer import _varint
        i, n, shift = 1, 0, 0
        while True:
            byte = rest[i]
            n |= (byte & 0x7F) << shift
            i += 1
            shift += 7
            if not byte & 0x80:
                break
        body = f_id(2, make_id("edge", 99999)) + rest[i:i + n]
        p.write_bytes(vid + f_bytes(2, body) + rest[i + n:])

    assert variant("deep", deep_yaml) == N.MBA_ERR_INVALID_ARG
    assert variant("outgoing", dangling_outgoing) == N.MBA_ERR_OUT_OF_RANGE_INDEX
    assert variant("trunc", truncate) == N.MBA_ERR_INVALID_ARG
    assert variant("meta", bad_meta) == N.MBA_ERR_INVALID_ARG
    assert variant("escape", escape_meta) == N.MBA_ERR_INVALID_ARG
    assert variant("yaml", bad_yaml) == N.MBA_ERR_INVALID_ARG
    assert variant("index", dangling_index) == N.MBA_ERR_OUT_OF_RANGE_INDEX
    assert variant("imu", unordered_imu) == N.MBA_ERR_UNORDERED_IMU


def test_state_write_back_and_lossless_save(tmp_path):
    m = synth.generate("c4", num_missions=2, keyframes_per_mission=40, num_landmarks=800, shared_landmark_fraction=0.3,
                       pose_edges=1, loop_closure_stride=6)
    src = tmp_path / "src"
    write_map(m, str(src))
    with vimap.VIMap(str(src)) as vm:
        d = vm.export(**ALL_TERMS)
        # unchanged state: every file is written back byte for byte
        st = {k: arr(d, k, (n, w)).copy() for k, n, w in (
            ("kf_q_IM_p_MI", d.num_keyframes, 7), ("kf_v_M", d.num_keyframes, 3), ("kf_b_g", d.num_keyframes, 3),
            ("kf_b_a", d.num_keyframes, 3), ("lm_p_B", d.num_landmarks, 3))}
        sw = arr(d, "pose_edge_switch", (d.num_pose_edges,)).copy()
        vm.import_state(st, sw)
        vm.save(str(tmp_path / "same"))
        for f in os.listdir(src / "vi_map"):
            assert (src / "vi_map" / f).read_bytes() == (tmp_path / "same" / "vi_map" / f).read_bytes(), f
        # a changed state round-trips
        rng = np.random.default_rng(1)
        st2 = {k: v + rng.normal(scale=1e-3, size=v.shape) for k, v in st.items()}
        q = st2["kf_q_IM_p_MI"][:, :4]
        st2["kf_q_IM_p_MI"][:, :4] = q / np.linalg.norm(q, axis=1, keepdims=True)
        lc = arr(d, "pose_edge_type", (d.num_pose_edges,), np.int32) == N.MBA_POSE_EDGE_LOOP_CLOSURE
        assert lc.any()
        sw2 = sw.copy()
        sw2[lc] = rng.uniform(0, 1, lc.sum())
        vm.import_state(st2, sw2)
        vm.save(str(tmp_path / "new"))
        with pytest.raises(ba.BAError):
            vm.save(str(tmp_path / "new"))  # no overwrite
        bad = dict(st2)
        bad["kf_q_IM_p_MI"] = st2["kf_q_IM_p_MI"] * 2.0  # not unit quaternions
        with pytest.raises(ba.BAError):
            vm.import_state(bad)
    with vimap.VIMap(str(tmp_path / "new")) as vm:
        d = vm.export(**ALL_TERMS)
        for k, v in st2.items():
            np.testing.assert_array_equal(arr(d, k, v.shape), v, err_msg=k)
        np.testing.assert_array_equal(arr(d, "pose_edge_switch", sw2.shape)[lc], sw2[lc])
        # untouched files stay identical
        for f in ("missions", "landmark_index", "sensors.yaml", "vi_map_metadata"):
            assert (src / "vi_map" / f).read_bytes() == (tmp_path / "new" / "vi_map" / f).read_bytes(), f
