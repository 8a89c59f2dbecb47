"""Python front-end over the C ABI (libmaplab_ba.so).

``BundleAdjuster`` mirrors the reference's optimizer entry points: create from
a problem description (constructOptimizationProblem + state import), evaluate
the cost terms like ceres::CostFunction::Evaluate, solve like
VIMapOptimizer::optimize / map_optimization::solve, and read the state back
like OptimizationStateBuffer::copyAllStatesBackToMap.  Every call goes through
the CUDA library; there is no CPU fallback.
"""
import ctypes

import numpy as np

from . import _native as N


class BAError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__(f"{what} failed: status {status}")


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = N.load_ba()
    return _LIB


def _check(st, what):
    if st != N.MBA_OK:
        raise BAError(st, what)


VISUAL_BLOCK_SIZES = [6, 14, 14, 14, 14, 8, 6, 8, 8]
INERTIAL_BLOCK_SIZES = [105, 45, 45, 45, 105, 45, 45, 45]


def default_options(**kw):
    o = N.SolverOptions()
    lib().mba_default_solver_options(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def measure_fp64_peak(device=0):
    """Measured FP64 rate of the device in TFLOP/s (mba_measure_fp64_peak)."""
    t = ctypes.c_double()
    _check(lib().mba_measure_fp64_peak(device, ctypes.byref(t)), "mba_measure_fp64_peak")
    return t.value


def default_landmark_quality_options(**kw):
    o = N.LandmarkQualityOptions()
    lib().mba_default_landmark_quality_options(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class PreconditionerModel:
    """Learned chain-preconditioner network (mba_gnn): FP32 master weights on
    one device, BF16 copies used by the kernels."""

    def __init__(self, device=0, seed=0):
        self._lib = lib()
        h = ctypes.c_void_p()
        _check(self._lib.mba_gnn_create(device, seed, ctypes.byref(h)), "mba_gnn_create")
        self._h = h
        self.device = device

    @staticmethod
    def num_parameters():
        return int(lib().mba_gnn_num_parameters())

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            self._lib.mba_gnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def parameters(self):
        w = np.zeros(self.num_parameters(), dtype=np.float32)
        _check(self._lib.mba_gnn_get_parameters(self._h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
               "mba_gnn_get_parameters")
        return w

    def set_parameters(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.num_parameters()
        _check(self._lib.mba_gnn_set_parameters(self._h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
               "mba_gnn_set_parameters")

    def save(self, path):
        np.save(path, self.parameters())

    @classmethod
    def load(cls, path, device=0):
        m = cls(device=device)
        m.set_parameters(np.load(path))
        return m


class BundleAdjuster:
    def __init__(self, desc, device=0):
        self._lib = lib()
        self.desc = desc
        h = ctypes.c_void_p()
        _check(self._lib.mba_create(ctypes.byref(desc), device, ctypes.byref(h)), "mba_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mba_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def evaluate_visual(self, blocks=range(9)):
        n = self.desc.num_observations
        r = np.zeros((n, 2))
        J = [np.zeros((n, VISUAL_BLOCK_SIZES[b])) if b in blocks else None for b in range(9)]
        arr = (N.c_double_p * 9)(*[N.ptr(j) if j is not None else None for j in J])
        _check(self._lib.mba_evaluate_visual(self._h, N.ptr(r), arr), "mba_evaluate_visual")
        return r, J

    def evaluate_inertial(self, blocks=range(8)):
        n = self.desc.num_imu_edges
        r = np.zeros((n, 15))
        J = [np.zeros((n, INERTIAL_BLOCK_SIZES[b])) if b in blocks else None for b in range(8)]
        arr = (N.c_double_p * 8)(*[N.ptr(j) if j is not None else None for j in J])
        _check(self._lib.mba_evaluate_inertial(self._h, N.ptr(r), arr), "mba_evaluate_inertial")
        return r, J

    def linearize_visual(self, precision=N.MBA_PRECISION_FP64):
        n = self.desc.num_observations
        r = np.zeros((n, 2)); Jl = np.zeros((n, 6)); Js = np.zeros((n, 12)); Jo = np.zeros((n, 12))
        _check(self._lib.mba_linearize_visual(self._h, precision, N.ptr(r), N.ptr(Jl), N.ptr(Js), N.ptr(Jo)),
               "mba_linearize_visual")
        return r, Jl, Js, Jo

    def linearize_pose_edges(self):
        """Relative pose edges at the current state: whitened residual
        [N_pe, 6] and (theta, p) tangent Jacobians [N_pe, 36] of the from and
        to keyframes."""
        n = self.desc.num_pose_edges
        r = np.zeros((n, 6)); Jf = np.zeros((n, 36)); Jt = np.zeros((n, 36))
        _check(self._lib.mba_linearize_pose_edges(self._h, N.ptr(r), N.ptr(Jf), N.ptr(Jt)),
               "mba_linearize_pose_edges")
        return r, Jf, Jt

    def cost(self):
        c = ctypes.c_double()
        _check(self._lib.mba_cost(self._h, 0, ctypes.byref(c)), "mba_cost")
        return c.value

    def solve(self, opts=None, capacity=256):
        if opts is None:
            opts = default_options()
        s = N.make_summary(capacity)
        _check(self._lib.mba_solve(self._h, ctypes.byref(opts), ctypes.byref(s)), "mba_solve")
        return N.summary_dict(s)

    def read_state(self):
        d = self.desc
        kx = np.zeros((d.num_keyframes, 7)); kv = np.zeros((d.num_keyframes, 3))
        kbg = np.zeros((d.num_keyframes, 3)); kba = np.zeros((d.num_keyframes, 3))
        lp = np.zeros((d.num_landmarks, 3))
        _check(self._lib.mba_read_state(self._h, N.ptr(kx), N.ptr(kv), N.ptr(kbg), N.ptr(kba), N.ptr(lp)),
               "mba_read_state")
        return dict(kf_q_IM_p_MI=kx, kf_v_M=kv, kf_b_g=kbg, kf_b_a=kba, lm_p_B=lp)

    def write_state(self, st):
        g = lambda k: N.ptr(np.ascontiguousarray(st[k], dtype=np.float64)) if st.get(k) is not None else None
        keep = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in st.items() if v is not None}
        _check(self._lib.mba_write_state(self._h, *[N.ptr(keep[k]) if k in keep else None for k in
                                                      ("kf_q_IM_p_MI", "kf_v_M", "kf_b_g", "kf_b_a", "lm_p_B")]),
               "mba_write_state")

    def read_calibration(self):
        """Cameras and mission baseframes of the current state
        (mba_read_calibration) as arrays (see _native.calibration_dict)."""
        d = self.desc
        cams = (N.Camera * d.num_cameras)()
        mis = np.zeros((d.num_missions, 7))
        _check(self._lib.mba_read_calibration(self._h, cams, N.ptr(mis)), "mba_read_calibration")
        return N.calibration_dict(cams, mis)

    def time_visual_kernel(self, mode=1, iters=20):
        ms = ctypes.c_double()
        _check(self._lib.mba_time_visual_kernel(self._h, mode, iters, ctypes.byref(ms)), "mba_time_visual_kernel")
        return ms.value

    def stats(self):
        s = N.ProblemStats()
        _check(self._lib.mba_get_stats(self._h, ctypes.byref(s)), "mba_get_stats")
        return {f: getattr(s, f) for f, _ in s._fields_}

    def reduced_system(self, precision=N.MBA_PRECISION_FP64, radius=1e5):
        """Damped, Jacobi-scaled reduced camera system at the current state:
        dict of diag [N_kf,15,15], upper_ij [N_pu,2], upper [N_pu,6,6],
        inertial [N_e,15,15] (with edge_from / edge_to) and rhs [N_kf,15]."""
        st = self.stats()
        nk, npu = st["num_keyframes"], st["num_schur_pose_blocks"] // 2
        ni, npe = st["num_imu_edges"], st["num_pose_edges"]
        ne = ni + npe
        D = np.zeros((nk, 15, 15)); ij = np.zeros((npu, 2), dtype=np.int32); U = np.zeros((npu, 6, 6))
        E = np.zeros((ne, 15, 15)); b = np.zeros((nk, 15))
        _check(self._lib.mba_reduced_system(self._h, precision, radius, N.ptr(D),
                                            ij.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), N.ptr(U), N.ptr(E),
                                            N.ptr(b)), "mba_reduced_system")
        d = self.desc
        part = lambda p, n: np.ctypeslib.as_array(p, (n,)).copy() if n else np.zeros(0, np.int32)
        ef = np.concatenate([part(d.edge_from, ni), part(d.pose_edge_from, npe)]).astype(np.int32)
        et = np.concatenate([part(d.edge_to, ni), part(d.pose_edge_to, npe)]).astype(np.int32)
        if npe and d.pose_edge_type:  # an absolute term is a (zero) block of its own keyframe
            ty = np.ctypeslib.as_array(d.pose_edge_type, (npe,))
            et[ni:][ty == N.MBA_POSE_EDGE_ABSOLUTE] = ef[ni:][ty == N.MBA_POSE_EDGE_ABSOLUTE]
        return dict(diag=D, upper_ij=ij, upper=U, inertial=E, edge_from=ef, edge_to=et, rhs=b)

    def rejected_landmarks(self):
        """(flags [N_lm] bool, count) of the landmarks rejected as outliers."""
        flags = np.zeros(self.desc.num_landmarks, dtype=np.uint8)
        c = ctypes.c_int64()
        _check(self._lib.mba_rejected_landmarks(self._h, flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                                ctypes.byref(c)), "mba_rejected_landmarks")
        return flags.astype(bool), c.value

    def set_preconditioner_model(self, model):
        _check(self._lib.mba_set_preconditioner_model(self._h, model.handle if model is not None else None),
               "mba_set_preconditioner_model")
        self._model = model

    def train_preconditioner(self, model, radius=1e5, nprobe=4, steps=1, lr=1e-3, seed=0):
        """Adam steps of the coefficient network on this state's reduced system;
        returns the loss before each step."""
        losses = np.zeros(max(steps, 1))
        _check(self._lib.mba_gnn_train(self._h, model.handle, radius, nprobe, steps, lr, seed, N.ptr(losses)),
               "mba_gnn_train")
        return losses[:steps]

    def preconditioner_gradient(self, model, radius=1e5, probes=None, nprobe=2, seed=0):
        """(loss, gradient [num_parameters], coef [N_kf, 3] per chain position)."""
        npar = model.num_parameters()
        grad = np.zeros(npar, dtype=np.float32)
        coef = np.zeros((self.desc.num_keyframes, 3))
        loss = ctypes.c_double()
        pr = None
        if probes is not None:
            probes = np.ascontiguousarray(probes, dtype=np.float32)
            nprobe = probes.shape[0]
            pr = probes.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        _check(self._lib.mba_gnn_gradient(self._h, model.handle, radius, nprobe, pr, seed,
                                          grad.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(loss),
                                          N.ptr(coef)), "mba_gnn_gradient")
        return loss.value, grad, coef

    def autotune(self, precision=N.MBA_PRECISION_MIXED):
        """Times launch / schedule candidates on this problem and keeps the fastest."""
        t = N.Tuning()
        _check(self._lib.mba_autotune(self._h, precision, ctypes.byref(t)), "mba_autotune")
        return {f: getattr(t, f) for f, _ in t._fields_}

    def set_tuning(self, **kw):
        t = N.Tuning()
        for k, v in kw.items():
            setattr(t, k, v)
        _check(self._lib.mba_set_tuning(self._h, ctypes.byref(t)), "mba_set_tuning")

    def chain_structure(self):
        n = self.desc.num_keyframes
        perm = np.zeros(n, dtype=np.int32); le = np.zeros(n, dtype=np.int32); lb = np.zeros(n, dtype=np.int32)
        p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        _check(self._lib.mba_chain_structure(self._h, p(perm), p(le), p(lb)), "mba_chain_structure")
        return perm, le, lb

    def chain_apply(self, r, precision=N.MBA_PRECISION_FP64, radius=1e5):
        """z = T^-1 r with the exact chain matrix of the current reduced system."""
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(self.desc.num_keyframes, 15)
        z = np.zeros_like(r)
        _check(self._lib.mba_chain_apply(self._h, precision, radius, N.ptr(r), N.ptr(z)), "mba_chain_apply")
        return z

    def cancel(self):
        self._lib.mba_cancel(self._h)

    def landmark_quality(self, **kw):
        """isVisualLandmarkWellConstrained per landmark at the current state
        (bool [N_lm]); keyword arguments override the elq_* defaults."""
        o = default_landmark_quality_options(**kw)
        good = np.zeros(max(1, self.desc.num_landmarks), dtype=np.uint8)
        _check(self._lib.mba_landmark_quality(self._h, ctypes.byref(o), good.ctypes.data_as(N.c_uint8_p)),
               "mba_landmark_quality")
        return good[:self.desc.num_landmarks].astype(bool)

    def read_switch_variables(self):
        """Switch value per pose edge [N_pe] (1 where an edge has none)."""
        sw = np.zeros(self.desc.num_pose_edges)
        _check(self._lib.mba_read_switch_variables(self._h, N.ptr(sw)), "mba_read_switch_variables")
        return sw

    def write_switch_variables(self, sw):
        sw = np.ascontiguousarray(sw, dtype=np.float64)
        _check(self._lib.mba_write_switch_variables(self._h, N.ptr(sw)), "mba_write_switch_variables")


class RelaxationProblem:
    """The descriptor of a pose-graph relaxation (VIMapRelaxation::
    solveRelaxation, vi-map-relaxation.cc:97-151): a copy of `desc` with
    velocities, biases and landmark positions fixed; the arrays it points at
    live as long as this object."""

    def __init__(self, desc):
        self.desc = N.ProblemDesc()
        ctypes.memmove(ctypes.byref(self.desc), ctypes.byref(desc), ctypes.sizeof(desc))
        self.kf_flags = np.zeros(desc.num_keyframes, dtype=np.uint32)
        self.lm_constant = np.zeros(max(1, desc.num_landmarks), dtype=np.uint8)
        _check(lib().mba_relaxation_flags(ctypes.byref(desc),
                                          self.kf_flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                          self.lm_constant.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))),
               "mba_relaxation_flags")
        self.desc.kf_flags = self.kf_flags.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        self.desc.lm_constant = self.lm_constant.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def relax(desc, opts=None, device=0):
    """Runs the relaxation solve on the device; returns (summary, state,
    switch variables)."""
    rp = RelaxationProblem(desc)
    with BundleAdjuster(rp.desc, device) as g:
        s = g.solve(opts)
        return s, g.read_state(), g.read_switch_variables()
