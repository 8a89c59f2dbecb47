"""The C ABI: every symbol declared in include/*.h is exported, the ctypes
mirrors match the C layouts, and host-side validation works without a GPU."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from maplab_gb300 import _native as N
from problem_util import OwnedDesc, camera

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*[\s\*]+(mba_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def _exported(lib_path):
    out = subprocess.check_output(["nm", "-D", "--defined-only", lib_path]).decode()
    return {l.split()[-1] for l in out.splitlines() if l.strip()}


def test_ba_library_exports_every_declared_symbol():
    path = os.path.join(N.BUILD_DIR, "libmaplab_ba.so")
    decl = _declared("maplab_ba.h")
    assert len(decl) >= 15, decl
    missing = [d for d in decl if d not in _exported(path)]
    assert not missing, missing
    N.load_ba()  # loads (resolves libcudart) without touching a device


def test_vimap_entry_points_are_exported():
    """include/maplab_vimap.h is served by libmaplab_ba.so (host code)."""
    path = os.path.join(N.BUILD_DIR, "libmaplab_ba.so")
    decl = _declared("maplab_vimap.h")
    assert len(decl) >= 10, decl
    missing = [d for d in decl if d not in _exported(path)]
    assert not missing, missing


def test_synth_library_exports_every_declared_symbol():
    path = os.path.join(N.BUILD_DIR, "libmba_synth.so")
    decl = _declared("maplab_ba_synth.h")
    missing = [d for d in decl if d not in _exported(path)]
    assert not missing, missing


STRUCTS = {
    "mba_camera": N.Camera, "mba_problem_desc": N.ProblemDesc, "mba_solver_options": N.SolverOptions,
    "mba_iteration_summary": N.IterationSummary, "mba_summary": N.Summary, "mba_problem_stats": N.ProblemStats,
    "mba_synth_config": N.SynthConfig, "mba_visual_batch_device": N.VisualBatchDevice,
    "mba_vimap_info": N.VimapInfo, "mba_vimap_export_options": N.VimapExportOptions,
}


def test_ctypes_layouts_match_c():
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "maplab_ba_synth.h"',
             '#include "maplab_vimap.h"', 'int main(void) {']
    for cname, cls in STRUCTS.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        open(c, "w").write("\n".join(lines))
        exe = os.path.join(d, "l")
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split("\n")
    got = {}
    for l in out:
        if l:
            s, f, v = l.split()
            got[(s, f)] = int(v)
    for cname, cls in STRUCTS.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def _tiny(**over):
    cam = camera()
    kw = dict(obs_uv=[[300.0, 200.0]], obs_sigma=[1.0], obs_landmark=[0], obs_keyframe=[0], obs_camera=[0],
              lm_p_B=[[5.0, 0.1, 0.2]], lm_store_keyframe=[0], kf_q_IM_p_MI=[[0, 0, 0, 1, 0, 0, 0]], cameras=[cam])
    kw.update(over)
    return OwnedDesc(**kw)


@pytest.mark.parametrize("over,status", [
    (dict(obs_landmark=[3]), N.MBA_ERR_OUT_OF_RANGE_INDEX),
    (dict(obs_keyframe=[-1]), N.MBA_ERR_OUT_OF_RANGE_INDEX),
    (dict(obs_sigma=[0.0]), N.MBA_ERR_INVALID_ARG),
    (dict(obs_uv=[[np.nan, 1.0]]), N.MBA_ERR_NON_FINITE),
    (dict(kf_q_IM_p_MI=[[0, 0, 0, 2, 0, 0, 0]]), N.MBA_ERR_INVALID_ARG),
    (dict(lm_store_keyframe=[5]), N.MBA_ERR_OUT_OF_RANGE_INDEX),
])
def test_create_rejects_invalid_input_on_host(over, status):
    lib = N.load_ba()
    od = _tiny(**over)
    h = ctypes.c_void_p()
    assert lib.mba_create(ctypes.byref(od.desc), 0, ctypes.byref(h)) == status
    assert not h.value


def test_create_rejects_unordered_imu_on_host():
    lib = N.load_ba()
    od = _tiny(kf_q_IM_p_MI=[[0, 0, 0, 1, 0, 0, 0], [0, 0, 0, 1, 1, 0, 0]], edge_from=[0], edge_to=[1],
               edge_sample_offset=[0, 3], imu_timestamp_ns=[0, 10, 5], imu_acc_gyro=np.zeros((3, 6)))
    h = ctypes.c_void_p()
    assert lib.mba_create(ctypes.byref(od.desc), 0, ctypes.byref(h)) == N.MBA_ERR_UNORDERED_IMU


def test_status_strings_and_defaults():
    lib = N.load_ba()
    assert lib.mba_status_string(N.MBA_ERR_NOT_SPD) == b"matrix not positive definite"
    assert lib.mba_abi_version() == 2
    o = N.SolverOptions()
    lib.mba_default_solver_options(ctypes.byref(o))
    ref = N.default_solver_options()
    for f, _ in o._fields_:
        assert getattr(o, f) == getattr(ref, f), f
