"""Writes a synthetic map (maplab_gb300.synth) as a maplab map folder, the
input of the VIMap reader tests:

    <folder>/vi_map/vi_map_metadata   text-format VIMapMetadata
    <folder>/vi_map/missions, vertices<i>, edges<i>, landmark_index
                                      binary vi_map.proto VIMap messages
    <folder>/vi_map/sensors.yaml      SensorManager YAML

Test infrastructure with its own protobuf wire-format encoder (independent of
the library's decoder).  Field numbers follow
map-structure/vi-map/proto/vi-map/vi_map.proto,
common/aslam-serialization/proto/aslam-serialization/visual-frame.proto and
aslam_cv2/aslam_cv_common/proto/aslam/common/id.proto; transformations are
stored as the Eigen quaternion x y z w (Hamilton) then p, matrices
column-major (maplab-common eigen-proto-inl.h).  The state conventions are
those of OptimizationStateBuffer (optimization-state-buffer.cc:153-300): a
vertex's q_M_I has the coefficients of the JPL q_IM; baseframes, cameras and
other sensors store the inverse of the JPL block's rotation.
"""
import os
import struct

import numpy as np

from maplab_gb300 import _native as N

# ---------------------------------------------------------------- wire format


def _varint(v):
    v &= (1 << 64) - 1
    out = bytearray()
    while v >= 0x80:
        out.append((v & 0x7F) | 0x80)
        v >>= 7
    out.append(v)
    return bytes(out)


def _key(field, wt):
    return _varint((field << 3) | wt)


def f_varint(field, v):
    return _key(field, 0) + _varint(int(v))


def f_double(field, x):
    return _key(field, 1) + struct.pack("<d", float(x))


def f_doubles(field, xs, packed=False):
    xs = [float(x) for x in np.asarray(xs).ravel()]
    if packed:
        return f_bytes(field, b"".join(struct.pack("<d", x) for x in xs))
    return b"".join(f_double(field, x) for x in xs)


def f_bytes(field, b):
    return _key(field, 2) + _varint(len(b)) + b


def id_msg(w):
    return f_varint(1, w[0]) + f_varint(1, w[1])


def f_id(field, w):
    return f_bytes(field, id_msg(w))


def hex_id(w):
    return (int(w[0]).to_bytes(8, "little") + int(w[1]).to_bytes(8, "little")).hex()


# ---------------------------------------------------------------- rotations


def quat_R(q):
    """Hamilton q (x y z w) -> active rotation matrix."""
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def conj(q):
    return np.array([-q[0], -q[1], -q[2], q[3]])


def T_inverse(T):
    q = conj(T[:4])
    return np.concatenate([q, -quat_R(T[:4]).T @ T[4:]])


def T_matrix(T):
    M = np.eye(4)
    M[:3, :3] = quat_R(T[:4])
    M[:3, 3] = T[4:]
    return M


def from_jpl_block(b):
    """JPL extrinsics block (q_XB, p_XB) -> Hamilton T_X_B."""
    return np.concatenate([conj(b[:4]), b[4:]])


# ---------------------------------------------------------------- ids

KIND = dict(vertex=1, edge=2, mission=3, baseframe=4, landmark=5, frame=6, nframe=7, sensor=8, camera=9)


def make_id(kind, i):
    return (KIND[kind] << 48 | (i + 1), 0x5EED0000 + KIND[kind])


# ---------------------------------------------------------------- writer


def _yaml_matrix(M, indent):
    pad = " " * indent
    rows = "\n".join(pad + "  - [" + ", ".join(repr(float(x)) for x in row) + "]" for row in M)
    return f"{pad}rows: {M.shape[0]}\n{pad}cols: {M.shape[1]}\n{pad}data:\n{rows}\n"


def _yaml_vector(v, indent):
    pad = " " * indent
    data = "\n".join(pad + "  - " + repr(float(x)) for x in v)
    return f"{pad}rows: {len(v)}\n{pad}cols: 1\n{pad}data:\n{data}\n"


def write_map(m, folder, quality=2, vertices_per_file=40, edges_per_file=60, packed=False, legacy_ids=False):
    """Writes synthetic map `m` to `folder`.  quality: landmark quality for all
    landmarks (0 kUnknown, 1 kBad, 2 kGood) or an array per landmark.
    legacy_ids: the frames name landmarks by separate "global" ids listed in
    landmark_index_ids (the legacy map layout).  Returns the ids used."""
    d = m.desc
    NK, NL, NO, NC, NM = d.num_keyframes, d.num_landmarks, d.num_observations, d.num_cameras, d.num_missions
    kx, kv, kbg, kba = m.array("kf_q_IM_p_MI"), m.array("kf_v_M"), m.array("kf_b_g"), m.array("kf_b_a")
    kmis = m.array("kf_mission")
    lp, lst = m.array("lm_p_B"), m.array("lm_store_keyframe")
    ouv, osig, olm, okf, ocam = (m.array(n) for n in ("obs_uv", "obs_sigma", "obs_landmark", "obs_keyframe",
                                                      "obs_camera"))
    mis = m.array("mission_q_GM_p_GM")
    NE = d.num_imu_edges
    ef, et, eoff = m.array("edge_from"), m.array("edge_to"), m.array("edge_sample_offset")
    ts, imu = m.array("imu_timestamp_ns"), m.array("imu_acc_gyro")
    NP = d.num_pose_edges
    pty = m.array("pose_edge_type") if NP and d.pose_edge_type else np.zeros(NP, dtype=np.int32)
    pf, pt, pT = m.array("pose_edge_from"), m.array("pose_edge_to"), m.array("pose_edge_T_Bk_Bkp1")
    pcov, pext = m.array("pose_edge_covariance"), m.array("pose_edge_q_I_B_p_B_I")
    psw = m.array("pose_edge_switch") if NP and d.pose_edge_switch else np.ones(NP)
    psv = m.array("pose_edge_switch_variance") if NP and d.pose_edge_switch_variance else np.zeros(NP)
    qual = np.broadcast_to(np.asarray(quality), (NL,))

    vid = [make_id("vertex", k) for k in range(NK)]
    lid = [make_id("landmark", l) for l in range(NL)]
    gid = [(w0, w1 ^ 0xABCD00) for (w0, w1) in lid] if legacy_ids else lid  # ids the frames carry
    mid = [make_id("mission", q) for q in range(NM)]
    bid = [make_id("baseframe", q) for q in range(NM)]
    imu_sensor, ncam_sensor = make_id("sensor", 0), make_id("sensor", 1)
    odo_sensor = [make_id("sensor", 10 + q) for q in range(NM)]
    abs_sensor = [make_id("sensor", 100 + q) for q in range(NM)]

    # ---- edges: IMU (viwls), relative (odometry), loop closures; backbone
    edges = []  # (id, from, to, body, kind)
    rel = [j for j in range(NP) if pty[j] == N.MBA_POSE_EDGE_RELATIVE]
    lcs = [j for j in range(NP) if pty[j] == N.MBA_POSE_EDGE_LOOP_CLOSURE]
    absj = [j for j in range(NP) if pty[j] == N.MBA_POSE_EDGE_ABSOLUTE]
    backbone = 0 if NE > 0 or not rel else 1
    for e in range(NE):
        a, b = int(eoff[e]), int(eoff[e + 1])
        body = (f_id(1, vid[ef[e]]) + f_id(2, vid[et[e]]) +
                b"".join(f_varint(3, int(t)) for t in ts[a:b]) + f_doubles(4, imu[a:b], packed) +
                f_id(5, mid[kmis[ef[e]]]))
        edges.append((int(ef[e]), int(et[e]), f_bytes(1, body)))
    if NE == 0 and not rel:  # a backbone to walk: viwls edges without samples
        for k in range(NK - 1):
            if kmis[k] == kmis[k + 1]:
                edges.append((k, k + 1, f_bytes(1, f_id(1, vid[k]) + f_id(2, vid[k + 1]) + f_id(5, mid[kmis[k]]))))
    odo_ext = {}
    for j in rel:
        q = int(kmis[pf[j]])
        odo_ext.setdefault(q, pext[j].copy())
        assert np.array_equal(odo_ext[q], pext[j]), "one odometry sensor per mission"
        body = (f_id(1, vid[pf[j]]) + f_id(2, vid[pt[j]]) + f_id(3, mid[q]) + f_doubles(4, pT[j], packed) +
                f_doubles(5, pcov[j].reshape(6, 6).T, packed) + f_id(6, odo_sensor[q]))
        edges.append((int(pf[j]), int(pt[j]), f_bytes(2, body)))
    for j in lcs:
        body = (f_id(1, vid[pf[j]]) + f_id(2, vid[pt[j]]) + f_id(3, mid[kmis[pf[j]]]) +
                f_doubles(4, pT[j], packed) + f_doubles(5, pcov[j].reshape(6, 6).T, packed) +
                f_double(6, psw[j]) + f_double(7, psv[j]))
        edges.append((int(pf[j]), int(pt[j]), f_bytes(3, body)))
    eid = [make_id("edge", i) for i in range(len(edges))]
    out_e = [[] for _ in range(NK)]
    in_e = [[] for _ in range(NK)]
    for i, (a, b, _) in enumerate(edges):
        out_e[a].append(eid[i])
        in_e[b].append(eid[i])
    abs_ext = {}
    abs_of = [[] for _ in range(NK)]
    for j in absj:
        q = int(kmis[pf[j]])
        abs_ext.setdefault(q, pext[j].copy())
        assert np.array_equal(abs_ext[q], pext[j]), "one absolute sensor per mission"
        abs_of[pf[j]].append(j)

    # ---- frames and landmark stores
    by_frame = {}
    for i in range(NO):
        by_frame.setdefault((int(okf[i]), int(ocam[i])), []).append(i)
    kp_index = np.zeros(NO, dtype=np.int64)
    for lst_i in by_frame.values():
        for r, i in enumerate(lst_i):
            kp_index[i] = r
    obs_of_lm = [[] for _ in range(NL)]
    for i in range(NO):
        obs_of_lm[olm[i]].append(i)
    store_of = [[] for _ in range(NK)]
    for l in range(NL):
        store_of[lst[l]].append(l)

    def vertex_msg(k):
        frames = b""
        for c in range(NC):
            obs = by_frame.get((k, c), [])
            fb = (f_id(1, make_id("frame", k * 64 + c)) + f_varint(2, 1000 * k) +
                  f_doubles(3, ouv[obs] if obs else [], packed) + f_doubles(4, osig[obs] if obs else [], packed) +
                  b"".join(f_id(7, gid[olm[i]]) for i in obs) + f_bytes(5, b"") + f_varint(9, 1))
            frames += f_bytes(2, fb)
        nframe = f_id(1, make_id("nframe", k)) + frames
        store = b""
        for l in store_of[k]:
            ob = obs_of_lm[l]
            lb = (f_id(1, lid[l]) + f_doubles(2, lp[l], packed) + b"".join(f_id(4, vid[okf[i]]) for i in ob) +
                  b"".join(f_varint(5, kp_index[i]) for i in ob) + b"".join(f_varint(6, ocam[i]) for i in ob) +
                  f_varint(7, int(qual[l])) + f_varint(9, 0))
            store += f_bytes(1, lb)
        absb = b""
        for j in abs_of[k]:
            ab = (f_varint(1, 1000 * k) + f_id(2, abs_sensor[int(kmis[k])]) + f_doubles(3, pT[j], packed) +
                  f_doubles(4, pcov[j].reshape(6, 6).T, packed))
            absb += f_bytes(15, ab)
        return (b"".join(f_id(1, e) for e in in_e[k]) + b"".join(f_id(2, e) for e in out_e[k]) +
                f_doubles(3, kx[k], packed) + f_doubles(4, kv[k], packed) + f_doubles(5, kba[k], packed) +
                f_doubles(6, kbg[k], packed) + f_bytes(7, nframe) + f_bytes(8, store) + f_id(14, mid[kmis[k]]) +
                absb)

    vi_dir = os.path.join(folder, "vi_map")
    os.makedirs(vi_dir)
    files = []

    def put(name, ftype, data):
        with open(os.path.join(vi_dir, name), "wb") as f:
            f.write(data)
        files.append((ftype, name))

    # missions and baseframes
    mb = b""
    for q in range(NM):
        root = int(np.flatnonzero(kmis == q)[0])
        msg = (f_id(1, bid[q]) + f_id(2, vid[root]) + f_varint(3, backbone) + f_id(8, ncam_sensor) +
               (f_id(9, imu_sensor) if NE else b"") + (f_id(11, odo_sensor[q]) if q in odo_ext else b"") +
               (f_id(13, abs_sensor[q]) if q in abs_ext else b""))
        mb += f_id(5, mid[q]) + f_bytes(6, msg)
    for q in range(NM):
        T_G_M = np.concatenate([conj(mis[q, :4]), mis[q, 4:]])
        mb += f_id(7, bid[q]) + f_bytes(8, f_doubles(1, T_G_M, packed) + f_doubles(2, np.eye(6), packed) +
                                        f_varint(3, 1))
    put("missions", 0, mb)
    for fi, a in enumerate(range(0, NK, vertices_per_file)):
        data = b"".join(f_id(1, vid[k]) + f_bytes(2, vertex_msg(k)) for k in range(a, min(NK, a + vertices_per_file)))
        put(f"vertices{fi}", 1, data)
    for fi, a in enumerate(range(0, max(len(edges), 1), edges_per_file)):
        data = b"".join(f_id(3, eid[i]) + f_bytes(4, edges[i][2]) for i in range(a, min(len(edges), a + edges_per_file)))
        put(f"edges{fi}", 2, data)
    put("landmark_index", 3, b"".join(f_bytes(10, f_id(1, vid[lst[l]]) + f_id(2, lid[l])) for l in range(NL)) +
        (b"".join(f_id(9, gid[l]) for l in range(NL)) if legacy_ids else b""))

    meta = "".join(f'files {{\n  file_type: {t}\n  path: "{n}"\n}}\n' for t, n in files)
    with open(os.path.join(vi_dir, "vi_map_metadata"), "w") as f:
        f.write(meta)

    # sensors.yaml
    y = ["sensors:"]
    y.append(f"  - id: {hex_id(imu_sensor)}\n    sensor_type: IMU\n    description: \"synthetic IMU\"\n    sigmas:\n"
             f"      acc_bias_random_walk_noise_density: {d.acc_bias_sigma!r}\n"
             f"      acc_noise_density: {d.acc_noise_sigma!r}\n"
             f"      gyro_bias_random_walk_noise_density: {d.gyro_bias_sigma!r}\n"
             f"      gyro_noise_density: {d.gyro_noise_sigma!r}\n"
             f"    gravity_magnitude_mps2: {d.gravity_magnitude!r}")
    cams = ""
    for c in range(NC):
        cam = d.cameras[c]
        dist = {N.MBA_DISTORTION_RADTAN: "radial-tangential", N.MBA_DISTORTION_EQUIDISTANT: "equidistant"}.get(
            cam.distortion_type, "none")
        blk = np.array(cam.q_CI_p_CI[:7])
        T_B_C = T_inverse(from_jpl_block(blk))
        cams += (f"      - camera:\n          id: {hex_id(make_id('camera', c))}\n          sensor_type: CAMERA\n"
                 f"          line-delay-nanoseconds: 0\n          image_height: {cam.height}\n"
                 f"          image_width: {cam.width}\n          type: pinhole\n          intrinsics:\n"
                 + _yaml_vector(cam.intrinsics[:4], 12) +
                 f"          distortion:\n            type: {dist}\n            parameters:\n"
                 + _yaml_vector(cam.distortion[:4], 14) +
                 "        T_B_C:\n" + _yaml_matrix(T_matrix(T_B_C), 10))
    y.append(f"  - id: {hex_id(ncam_sensor)}\n    sensor_type: NCAMERA\n    description: \"synthetic rig\"  # comment\n"
             f"    cameras:\n" + cams.rstrip("\n"))
    ext = [(imu_sensor, np.eye(4)), (ncam_sensor, np.eye(4))]
    for q, b in odo_ext.items():
        y.append(f"  - id: {hex_id(odo_sensor[q])}\n    sensor_type: ODOMETRY_6DOF\n    topic: /odometry")
        ext.append((odo_sensor[q], T_matrix(T_inverse(from_jpl_block(b)))))
    for q, b in abs_ext.items():
        y.append(f"  - id: {hex_id(abs_sensor[q])}\n    sensor_type: ABSOLUTE_6DOF\n    topic: /absolute")
        ext.append((abs_sensor[q], T_matrix(T_inverse(from_jpl_block(b)))))
    y.append("\nextrinsics:")
    for sid, M in ext:
        y.append(f"  - sensor_id: {hex_id(sid)}\n    base_sensor_id: {hex_id(imu_sensor)}\n    T_B_S:\n"
                 + _yaml_matrix(M, 6).rstrip("\n"))
    with open(os.path.join(vi_dir, "sensors.yaml"), "w") as f:
        f.write("\n".join(y) + "\n")
    return dict(vertex=vid, landmark=lid, mission=mid, edges=eid, kp_index=kp_index)
