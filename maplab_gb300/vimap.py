"""maplab map folders for the BA path (include/maplab_vimap.h).

    with VIMap("/maps/run1") as vm:
        desc = vm.export()                      # constructOptimizationProblem
        with BundleAdjuster(desc) as ba:
            summary = ba.solve(opts)
            vm.import_state(ba.read_state(), ba.read_switch_variables())
        vm.save("/maps/run1_optimized")         # saveMapToFolder

`optimize` does the same in one call, the counterpart of
VIMapOptimizer::optimize (algorithms/map-optimization/src/vi-map-optimizer.cc)
followed by saving the map.
"""
import ctypes

import numpy as np

from . import _native as N
from .ba import BAError, BundleAdjuster, _check, default_options, lib


def default_export_options(**kw):
    """ViProblemOptions as maplab's flag defaults set them; keyword
    arguments override fields of mba_vimap_export_options."""
    o = N.VimapExportOptions()
    lib().mba_vimap_default_export_options(ctypes.byref(o))
    for k, v in kw.items():
        if k == "quality":
            for qk, qv in v.items():
                setattr(o.quality, qk, qv)
        else:
            setattr(o, k, v)
    return o


def _ids(buf):
    return buf.reshape(-1, 2)


class VIMap:
    """A loaded map folder (<folder>/vi_map/...)."""

    def __init__(self, folder):
        self._lib = lib()
        h = ctypes.c_void_p()
        _check(self._lib.mba_vimap_load(str(folder).encode(), ctypes.byref(h)), "mba_vimap_load")
        self._h = h
        self._keep = None
        self.desc = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mba_vimap_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self):
        i = N.VimapInfo()
        _check(self._lib.mba_vimap_get_info(self._h, ctypes.byref(i)), "mba_vimap_get_info")
        return {name: getattr(i, name) for name, _ in N.VimapInfo._fields_}

    def mission_ids(self):
        n = self.info()["num_missions"]
        ids = np.zeros(2 * n, dtype=np.uint64)
        _check(self._lib.mba_vimap_mission_ids(self._h, N.ptr(ids, ctypes.c_uint64)), "mba_vimap_mission_ids")
        return _ids(ids)

    def landmark_ids(self):
        """Ids in map landmark order (the order of a landmark_keep mask)."""
        n = self.info()["num_landmarks"]
        ids = np.zeros(2 * max(n, 1), dtype=np.uint64)
        _check(self._lib.mba_vimap_landmark_ids(self._h, N.ptr(ids, ctypes.c_uint64)), "mba_vimap_landmark_ids")
        return _ids(ids)[:n]

    def export(self, missions=None, landmark_keep=None, **options):
        """The SoA problem of `missions` (indices in the missions file order;
        None = all).  The returned descriptor points into memory owned by
        this object, valid until the next export or close."""
        o = default_export_options(**options)
        keep = []
        if missions is not None:
            m = np.ascontiguousarray(missions, dtype=np.int32)
            keep.append(m)
            o.num_missions = len(m)
            o.missions = N.ptr(m, ctypes.c_int32)
        if landmark_keep is not None:
            k = np.ascontiguousarray(landmark_keep, dtype=np.uint8)
            keep.append(k)
            o.landmark_keep = N.ptr(k, ctypes.c_uint8)
            o.landmark_selection = N.MBA_VIMAP_LANDMARKS_MASK
        d = N.ProblemDesc()
        _check(self._lib.mba_vimap_export(self._h, ctypes.byref(o), ctypes.byref(d)), "mba_vimap_export")
        self._keep = keep
        self.desc = d
        return d

    def export_ids(self):
        """Ids of the last export's keyframes, landmarks, missions and pose
        edges (edge ids; the vertex id for absolute terms), [n, 2] uint64."""
        d = self.desc
        bufs = [np.zeros(2 * max(n, 1), dtype=np.uint64)
                for n in (d.num_keyframes, d.num_landmarks, d.num_missions, d.num_pose_edges)]
        _check(self._lib.mba_vimap_export_ids(self._h, *[N.ptr(b, ctypes.c_uint64) for b in bufs]),
               "mba_vimap_export_ids")
        n = (d.num_keyframes, d.num_landmarks, d.num_missions, d.num_pose_edges)
        return dict(zip(("keyframes", "landmarks", "missions", "pose_edges"),
                        (_ids(b)[:k] for b, k in zip(bufs, n))))

    def import_state(self, state, switches=None):
        """Writes a BundleAdjuster.read_state() dict (and the pose edges'
        switch variables) of the last export into the map."""
        arr = [np.ascontiguousarray(state[k], dtype=np.float64) if state.get(k) is not None else None
               for k in ("kf_q_IM_p_MI", "kf_v_M", "kf_b_g", "kf_b_a", "lm_p_B")]
        sw = np.ascontiguousarray(switches, dtype=np.float64) if switches is not None else None
        _check(self._lib.mba_vimap_import_state(self._h, *[N.ptr(a) for a in arr], N.ptr(sw)),
               "mba_vimap_import_state")

    def save(self, folder):
        _check(self._lib.mba_vimap_save(self._h, str(folder).encode()), "mba_vimap_save")


def optimize(map_folder, out_folder, solver_options=None, missions=None, device=0, **export_options):
    """Loads a map, builds the problem of `missions`, solves it on the GPU,
    writes the optimized state back and saves the map to `out_folder`.
    Returns the solver summary."""
    with VIMap(map_folder) as vm:
        desc = vm.export(missions=missions, **export_options)
        with BundleAdjuster(desc, device) as ba:
            summary = ba.solve(solver_options if solver_options is not None else default_options())
            vm.import_state(ba.read_state(), ba.read_switch_variables() if desc.num_pose_edges else None)
        vm.save(out_folder)
    return summary


__all__ = ["VIMap", "default_export_options", "optimize", "BAError"]
