"""ctypes binding of libredgb (include/redgb.h) and a Python mirror of the
pp_disk / integrator seam for tests and benchmarks.

Every call goes through the C ABI; there is no fallback: if libredgb.so
cannot be loaded, or the device is missing, the calls raise.
"""
import ctypes as C
import os

import numpy as np

from .types import BMD, EVENT, PARAM, VAR4, System

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libredgb.so")

RED_OK = 0
ERRORS = {1: "RED_ERR_ARG", 2: "RED_ERR_CUDA", 3: "RED_ERR_EVENT_OVERFLOW", 4: "RED_ERR_TIMEOUT",
          5: "RED_ERR_NONFINITE", 6: "RED_ERR_NOT_IMPLEMENTED", 7: "RED_ERR_SUPERPLANETESIMAL",
          8: "RED_ERR_NO_DEVICE"}
PRECISION = {"mixed": 0, "fp64": 1, "fp64_exact": 2, "fp32": 3}
INTEGRATOR = {"euler": 0, "e": 0, "rk2": 1, "rk4": 2, "rkf78": 4, "rkf8": 4}

EXPORTS = ["red_create", "red_destroy", "red_step", "red_launch_tries", "red_synchronize",
           "red_handle_events", "red_check_for_collision", "red_check_for_ejection_hit_centrum",
           "red_calc_dydx", "red_calc_integral", "red_calc_energy_interacting", "red_get_state",
           "red_set_state", "red_get_states", "red_set_states", "red_get_system_info", "red_set_dt_next", "red_rebuild_vectors",
           "red_autotune", "red_get_plan_info", "red_profile_try", "red_interactions_per_eval", "red_kernel_launches", "red_n_systems",
           "red_n_bodies",
           "red_calc_accel_noalloc", "red_mlp_param_count", "red_mlp_predict", "red_mlp_grad", "red_mlp_adam",
           "red_set_step_proposer", "red_clear_step_proposer", "red_log_features", "red_get_feature_log",
           "red_populate_disks",
           "red_last_error", "red_version"]


class RedError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code


class GasParams(C.Structure):
    _fields_ = [("rho", C.c_double * 2), ("sch", C.c_double * 2), ("eta", C.c_double * 2),
                ("tau", C.c_double * 2), ("mfp", C.c_double * 2), ("temp", C.c_double * 2),
                ("c_vth", C.c_double), ("gas_decrease", C.c_int32), ("t0", C.c_double), ("t1", C.c_double),
                ("e_folding_time", C.c_double), ("alpha", C.c_double), ("mean_molecular_weight", C.c_double),
                ("particle_diameter", C.c_double)]


class Config(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("adaptive", C.c_int32), ("tolerance", C.c_double),
                ("error_check_for_tp", C.c_int32), ("precision", C.c_int32), ("stage_exact", C.c_int32),
                ("threshold", C.c_double * 3), ("output_interval", C.c_double), ("length", C.c_double),
                ("gas_disk", C.c_int32), ("gas", GasParams), ("event_capacity", C.c_uint32),
                ("device", C.c_int32), ("stream", C.c_void_p)]


class SystemInfo(C.Structure):
    _fields_ = [("t", C.c_double), ("dt_try", C.c_double), ("dt_did", C.c_double), ("dt_next", C.c_double),
                ("n_tried", C.c_uint64), ("n_passed", C.c_uint64), ("n_failed", C.c_uint64),
                ("playing", C.c_uint32 * 7), ("inactive", C.c_uint32 * 7), ("removed", C.c_uint32 * 7),
                ("n_total", C.c_uint32), ("active", C.c_int32), ("halted", C.c_int32), ("status", C.c_int32),
                ("n_collision", C.c_uint32 * 3), ("n_ejection", C.c_uint32 * 3),
                ("n_hit_centrum", C.c_uint32 * 3), ("n_event", C.c_uint32 * 3)]


class AccelArgs(C.Structure):
    """red_accel_args_t: device pointers of the allocation-free gravity entry point."""
    _fields_ = [("playing", C.c_uint32 * 7), ("r", C.c_void_p), ("v", C.c_void_p), ("mass", C.c_void_p),
                ("radius", C.c_void_p), ("density", C.c_void_p), ("cd", C.c_void_p), ("id", C.c_void_p),
                ("accel", C.c_void_p), ("precision", C.c_int32), ("gas_disk", C.c_int32), ("gas", GasParams),
                ("t", C.c_double), ("device", C.c_int32), ("stream", C.c_void_p)]


NOALLOC_MAX_BODIES = 32768


class PlanInfo(C.Structure):
    """red_plan_info_t: the launch plan in use and the last autotune's timings."""
    _fields_ = [("chunk", C.c_int32), ("lanes_cap", C.c_int32), ("cluster", C.c_int32), ("packed", C.c_int32),
                ("n_items", C.c_int32),
                ("candidates", C.c_int32), ("ms_per_try", C.c_float), ("ms_per_try_default", C.c_float)]


class DiskSpec(C.Structure):
    """red_disk_spec_t: one disk of red_populate_disks."""
    _fields_ = [("n_pp", C.c_uint32), ("n_pl", C.c_uint32), ("m_star", C.c_double), ("star_radius", C.c_double),
                ("pp_mass", C.c_double), ("pp_a0", C.c_double), ("pp_da", C.c_double), ("pp_hill", C.c_double),
                ("pl_a_min", C.c_double), ("pl_a_max", C.c_double), ("pl_a_log", C.c_int32), ("pad", C.c_int32),
                ("pl_mass_total", C.c_double), ("pl_mass_exp", C.c_double), ("sigma_e_pp", C.c_double),
                ("sigma_i_pp", C.c_double), ("sigma_e", C.c_double), ("sigma_i", C.c_double), ("e_max", C.c_double),
                ("density", C.c_double), ("cd", C.c_double), ("seed", C.c_uint64)]


class MlpNorm(C.Structure):
    """red_mlp_norm_t: normalisation of the proposer's features and target."""
    _fields_ = [("x_mean", C.c_float * 12), ("x_std", C.c_float * 12), ("y_mean", C.c_float), ("y_std", C.c_float)]


MLP_NFEAT = 12


class Integral(C.Structure):
    _fields_ = [("R", C.c_double * 4), ("V", C.c_double * 4), ("C", C.c_double * 4), ("E", C.c_double)]


_lib = None


def load(path=LIB_PATH):
    """Loads libredgb.so (built by build.py); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libredgb.so not built (%s); run __graft_entry__.build()" % path)
    L = C.CDLL(path)
    P = C.c_void_p
    u32p = C.POINTER(C.c_uint32)
    L.red_create.argtypes = [C.POINTER(Config), C.c_uint32, u32p, P, P, P, P, P, P, C.POINTER(C.c_void_p)]
    L.red_destroy.argtypes = [P]
    L.red_step.argtypes = [P, C.POINTER(C.c_double)]
    L.red_launch_tries.argtypes = [P, C.c_uint32]
    L.red_synchronize.argtypes = [P, u32p, u32p]
    L.red_handle_events.argtypes = [P, P, C.c_uint32, u32p]
    L.red_check_for_collision.argtypes = [P, P, C.c_uint32, u32p]
    L.red_check_for_ejection_hit_centrum.argtypes = [P, P, C.c_uint32, u32p]
    L.red_calc_dydx.argtypes = [P, C.c_uint32, C.c_int32, C.c_double, P]
    L.red_calc_integral.argtypes = [P, C.c_uint32, C.POINTER(Integral)]
    L.red_calc_energy_interacting.argtypes = [P, C.c_uint32, P]
    L.red_get_state.argtypes = [P, C.c_uint32, P, P, P, P]
    L.red_set_state.argtypes = [P, C.c_uint32, P, P, P, P]
    L.red_get_states.argtypes = [P, C.c_uint32, C.c_uint32, P, P, P, P]
    L.red_set_states.argtypes = [P, C.c_uint32, C.c_uint32, P, P, P, P]
    L.red_get_system_info.argtypes = [P, C.c_uint32, C.POINTER(SystemInfo)]
    L.red_set_dt_next.argtypes = [P, C.c_uint32, C.c_double]
    L.red_rebuild_vectors.argtypes = [P]
    L.red_autotune.argtypes = [P]
    L.red_get_plan_info.argtypes = [P, C.POINTER(PlanInfo)]
    L.red_profile_try.argtypes = [P, P, P, C.c_uint32, u32p]
    L.red_interactions_per_eval.argtypes = [P]
    L.red_interactions_per_eval.restype = C.c_uint64
    L.red_kernel_launches.argtypes = [P]
    L.red_kernel_launches.restype = C.c_uint64
    L.red_n_systems.argtypes = [P]
    L.red_n_systems.restype = C.c_uint32
    L.red_n_bodies.argtypes = [P, C.c_uint32]
    L.red_n_bodies.restype = C.c_uint32
    L.red_calc_accel_noalloc.argtypes = [C.POINTER(AccelArgs)]
    L.red_populate_disks.argtypes = [C.POINTER(DiskSpec), C.c_uint32, C.c_int32, P, P, P, P, P]
    L.red_mlp_param_count.restype = C.c_uint32
    L.red_mlp_predict.argtypes = [P, C.POINTER(MlpNorm), P, P, C.c_uint32, P]
    L.red_mlp_grad.argtypes = [P, P, P, C.c_uint32, P, P, P]
    L.red_mlp_adam.argtypes = [P, P, P, P, P, C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float, P]
    L.red_set_step_proposer.argtypes = [P, P, C.POINTER(MlpNorm), C.c_double, C.c_double, C.c_double]
    L.red_clear_step_proposer.argtypes = [P]
    L.red_log_features.argtypes = [P, C.c_uint32]
    L.red_get_feature_log.argtypes = [P, P, C.c_uint32, u32p, C.c_int32]
    L.red_last_error.restype = C.c_char_p
    L.red_version.restype = C.c_char_p
    _lib = L
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _addr(a):
    """The address of a numpy array's data, for a c_void_p argument (cheaper
    than a ctypes pointer object on the per-step state calls)."""
    return a.ctypes.data


def _check_out(a, dtype, n):
    """An array the library writes n records of `dtype` into: contiguous, of
    that exact layout (a packed copy of a padded record would be overrun)."""
    if not a.flags.c_contiguous or len(a) != n or not (a.dtype is dtype or (a.dtype == dtype and
                                                                            a.dtype.itemsize == dtype.itemsize)):
        raise ValueError("out arrays must be contiguous with %d records of %s" % (n, dtype))


def _check(rc):
    if rc != RED_OK:
        raise RedError(rc, load().red_last_error().decode())


def calc_accel_noalloc(args):
    """Calls red_calc_accel_noalloc with a filled AccelArgs; raises on error."""
    _check(load().red_calc_accel_noalloc(C.byref(args)))


def populate_disks(specs, device=0):
    """red_populate_disks: the disks of `specs` (DiskSpec list) generated on the
    GPU; returns one System per spec."""
    from .types import BMD, PARAM, VAR4, System
    arr = (DiskSpec * len(specs))(*specs)
    ns = [1 + s.n_pp + s.n_pl for s in specs]
    tot = sum(ns)
    r, v, p, md = np.zeros(tot, VAR4), np.zeros(tot, VAR4), np.zeros(tot, PARAM), np.zeros(tot, BMD)
    playing = np.zeros((len(specs), 7), np.uint32)
    _check(load().red_populate_disks(arr, len(specs), device, _p(playing), _p(r), _p(v), _p(p), _p(md)))
    out, o = [], 0
    for k, n in enumerate(ns):
        sl = slice(o, o + n)
        names = ["star"] + ["pp%d" % i for i in range(specs[k].n_pp)] + ["pl%d" % i for i in range(specs[k].n_pl)]
        out.append(System(r[sl].copy(), v[sl].copy(), p[sl].copy(), md[sl].copy(), playing[k].copy(), names))
        o += n
    return out


def mlp_param_count():
    return int(load().red_mlp_param_count())


def mlp_predict(w_ptr, norm, x_ptr, out_ptr, n, stream=None):
    """Device pointers: BF16 weights, n x 12 raw features -> n predicted log|dt|."""
    _check(load().red_mlp_predict(w_ptr, C.byref(norm), x_ptr, out_ptr, n, stream))


def mlp_grad(w_ptr, xn_ptr, tn_ptr, n, grad_ptr, loss_ptr, stream=None):
    _check(load().red_mlp_grad(w_ptr, xn_ptr, tn_ptr, n, grad_ptr, loss_ptr, stream))


def mlp_adam(master_ptr, w_ptr, m_ptr, v_ptr, grad_ptr, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
    _check(load().red_mlp_adam(master_ptr, w_ptr, m_ptr, v_ptr, grad_ptr, step, lr, beta1, beta2, eps, stream))


def gas_struct(gas_record):
    """numpy GAS record (types.GAS) -> GasParams."""
    g = GasParams()
    C.memmove(C.addressof(g), np.ascontiguousarray(gas_record).tobytes(), C.sizeof(GasParams))
    return g


class Sim:
    """One handle of libredgb holding one or more systems."""

    def __init__(self, systems, *, integrator="rkf78", adaptive=True, tolerance=1e-10, dt=None,
                 precision="mixed", stage_exact=False, collision_factor=0.0, ejection=0.0,
                 hit_centrum=0.0, gas=None, output_interval=0.0, length=0.0, error_check_for_tp=False,
                 event_capacity=0, device=0, stream=None, t0=None, gas_model=None):
        L = load()
        if isinstance(systems, System):
            systems = [systems]
        self.systems_n = [s.n for s in systems]
        cfg = Config()
        cfg.integrator = INTEGRATOR[integrator] if isinstance(integrator, str) else int(integrator)
        cfg.adaptive = int(adaptive)
        cfg.tolerance = tolerance
        cfg.error_check_for_tp = int(error_check_for_tp)
        cfg.precision = PRECISION[precision] if isinstance(precision, str) else int(precision)
        cfg.stage_exact = int(stage_exact)
        cfg.threshold[0] = hit_centrum
        cfg.threshold[1] = ejection
        cfg.threshold[2] = collision_factor
        cfg.output_interval = output_interval
        cfg.length = length
        if gas is not None:
            cfg.gas_disk = 1
            cfg.gas = gas_struct(gas)
        if gas_model is not None:   # red's g_disk_model: 0 none, 1 analytic, 2 FARGO (refused)
            cfg.gas_disk = int(gas_model)
        cfg.event_capacity = event_capacity
        cfg.device = device
        cfg.stream = stream
        self.cfg = cfg
        playing = np.concatenate([s.playing for s in systems]).astype(np.uint32)
        # np.concatenate packs structured dtypes (a 20-byte metadata record); keep red's layout
        r = np.concatenate([s.r for s in systems]).astype(VAR4)
        v = np.concatenate([s.v for s in systems]).astype(VAR4)
        p = np.concatenate([s.p for s in systems]).astype(PARAM)
        md = np.concatenate([s.md for s in systems]).astype(BMD)
        assert md.itemsize == 24
        ns = len(systems)
        dts = np.broadcast_to(np.asarray(dt if dt is not None else 0.0, dtype=np.float64), (ns,)).copy()
        t0s = np.broadcast_to(np.asarray(t0 if t0 is not None else 0.0, dtype=np.float64), (ns,)).copy()
        h = C.c_void_p()
        _check(L.red_create(C.byref(cfg), ns, playing.ctypes.data_as(C.POINTER(C.c_uint32)), _p(r), _p(v),
                            _p(p), _p(md), _p(t0s), _p(dts), C.byref(h)))
        self.h = h
        self.n_systems = ns
        self.names = [s.names for s in systems]

    def close(self):
        if getattr(self, "h", None):
            load().red_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- integrator::step and the device-side loop --------------------------
    def step(self):
        d = C.c_double()
        _check(load().red_step(self.h, C.byref(d)))
        return d.value

    def launch_tries(self, n):
        _check(load().red_launch_tries(self.h, n))

    def synchronize(self):
        a, h = C.c_uint32(), C.c_uint32()
        _check(load().red_synchronize(self.h, C.byref(a), C.byref(h)))
        return a.value, h.value

    def handle_events(self, cap=4096):
        out = np.zeros(cap, EVENT)
        n = C.c_uint32()
        _check(load().red_handle_events(self.h, _p(out), cap, C.byref(n)))
        return out[:min(n.value, cap)].copy()

    def check_for_collision(self, cap=4096):
        out = np.zeros(cap, EVENT)
        n = C.c_uint32()
        _check(load().red_check_for_collision(self.h, _p(out), cap, C.byref(n)))
        return out[:min(n.value, cap)].copy()

    def check_for_ejection_hit_centrum(self, cap=4096):
        out = np.zeros(cap, EVENT)
        n = C.c_uint32()
        _check(load().red_check_for_ejection_hit_centrum(self.h, _p(out), cap, C.byref(n)))
        return out[:min(n.value, cap)].copy()

    # -- pp_disk seam ---------------------------------------------------------
    def info(self, sys=0):
        i = SystemInfo()
        _check(load().red_get_system_info(self.h, sys, C.byref(i)))
        return i

    def calc_dydx(self, sys, i, t):
        n = self.info(sys).n_total
        dy = np.zeros(n, VAR4)
        _check(load().red_calc_dydx(self.h, sys, i, t, _p(dy)))
        return dy

    def calc_integral(self, sys=0):
        I = Integral()
        _check(load().red_calc_integral(self.h, sys, C.byref(I)))
        return np.array(list(I.R)[:3] + list(I.V)[:3] + list(I.C)[:3] + [I.E])

    def energy_interacting(self, sys=0):
        out = np.zeros(4)
        _check(load().red_calc_energy_interacting(self.h, sys, _p(out)))
        return out

    def get_state(self, sys=0, out=None, parts="rvpm"):
        """System `sys` as a System; with `out`, the arrays named in `parts`
        (r, v, p, m = metadata) are written into out's arrays in place (which
        must be contiguous and hold n_total records) and out is returned."""
        if out is None:
            info = self.info(sys)
            n = info.n_total
            r, v, p, md = np.zeros(n, VAR4), np.zeros(n, VAR4), np.zeros(n, PARAM), np.zeros(n, BMD)
        else:
            n = load().red_n_bodies(self.h, sys)
            r, v, p, md = out.r, out.v, out.p, out.md
            for a, t in ((r, VAR4), (v, VAR4), (p, PARAM), (md, BMD)):
                _check_out(a, t, n)
        ptr = [_p(a) if k in parts else None for a, k in ((r, "r"), (v, "v"), (p, "p"), (md, "m"))]
        _check(load().red_get_state(self.h, sys, *ptr))
        if out is not None:
            return out
        s = System(r, v, p, md, np.array(info.playing, np.uint32))
        s.inactive = np.array(info.inactive, np.uint32)
        s.removed = np.array(info.removed, np.uint32)
        return s

    def set_state(self, sys, s, parts="rvpm"):
        """Writes the arrays of System s named in `parts` (r, v, p, m = metadata)."""
        arrs = [(s.r, VAR4, "r"), (s.v, VAR4, "v"), (s.p, PARAM, "p"), (s.md, BMD, "m")]
        keep = [np.ascontiguousarray(a, t) if k in parts else None for a, t, k in arrs]
        _check(load().red_set_state(self.h, sys, *[_p(a) if a is not None else None for a in keep]))

    def bodies(self, sys0=0, count=None):
        """Bodies of the systems [sys0, sys0 + count) (all from sys0 by default)."""
        count = self.n_systems - sys0 if count is None else count
        L = load()
        if count == 1:
            return int(L.red_n_bodies(self.h, sys0))
        return sum(int(L.red_n_bodies(self.h, k)) for k in range(sys0, sys0 + count))

    def get_states(self, out, sys0=0, count=None, parts="rvpm"):
        """The records of systems [sys0, sys0 + count), one system after the other,
        into out's arrays (a System or any object with contiguous r, v, p, md of
        bodies(sys0, count) records) in one call; returns out."""
        count = self.n_systems - sys0 if count is None else count
        n = self.bodies(sys0, count)
        ptrs = [None, None, None, None]
        for i, (a, t, k) in enumerate(((out.r, VAR4, "r"), (out.v, VAR4, "v"), (out.p, PARAM, "p"),
                                       (out.md, BMD, "m"))):
            if k in parts:
                _check_out(a, t, n)
                ptrs[i] = _addr(a)
        _check(load().red_get_states(self.h, sys0, count, *ptrs))
        return out

    def set_states(self, s, sys0=0, count=None, parts="rvpm"):
        """Writes the arrays of s named in `parts` (the records of systems
        [sys0, sys0 + count), one system after the other) in one call."""
        count = self.n_systems - sys0 if count is None else count
        n = self.bodies(sys0, count)
        keep = [None, None, None, None]   # the (contiguous) arrays stay referenced during the call
        ptrs = [None, None, None, None]
        for i, (a, t, k) in enumerate(((s.r, VAR4, "r"), (s.v, VAR4, "v"), (s.p, PARAM, "p"), (s.md, BMD, "m"))):
            if k in parts:
                a = np.ascontiguousarray(a, t)
                if len(a) != n:
                    raise ValueError("arrays must hold %d records" % n)
                keep[i] = a
                ptrs[i] = _addr(a)
        _check(load().red_set_states(self.h, sys0, count, *ptrs))

    def set_dt_next(self, sys, dt):
        _check(load().red_set_dt_next(self.h, sys, dt))

    def rebuild_vectors(self):
        _check(load().red_rebuild_vectors(self.h))

    def autotune(self):
        """red_autotune: picks the fastest launch plan on the live state (which
        it leaves unchanged); returns the plan and the measured try times."""
        _check(load().red_autotune(self.h))
        return self.plan_info()

    def plan_info(self):
        i = PlanInfo()
        _check(load().red_get_plan_info(self.h, C.byref(i)))
        return {"chunk": i.chunk, "lanes_cap": i.lanes_cap, "cluster": bool(i.cluster), "packed": bool(i.packed),
                "n_items": i.n_items,
                "candidates": i.candidates, "ms_per_try": i.ms_per_try,
                "ms_per_try_default": i.ms_per_try_default}

    def set_step_proposer(self, w_bf16, norm, safety=1.0, ratio_lo=0.5, ratio_hi=2.0):
        """Enables the learned proposals: w_bf16 (np.uint16, mlp_param_count()), norm (MlpNorm)."""
        w = np.ascontiguousarray(w_bf16, np.uint16)
        if w.size != mlp_param_count():
            raise ValueError("expected %d BF16 parameters" % mlp_param_count())
        _check(load().red_set_step_proposer(self.h, _p(w), C.byref(norm), safety, ratio_lo, ratio_hi))

    def clear_step_proposer(self):
        _check(load().red_clear_step_proposer(self.h))

    def log_features(self, capacity):
        _check(load().red_log_features(self.h, capacity))

    def feature_log(self, cap=1 << 20, reset=False):
        """Logged records as an (n, 14) float32 array: 12 features, log|dt| of the
        next accepted step, log(err / tol) of that step."""
        out = np.zeros((cap, MLP_NFEAT + 2), np.float32)
        n = C.c_uint32()
        _check(load().red_get_feature_log(self.h, _p(out), cap, C.byref(n), 1 if reset else 0))
        return out[:min(n.value, cap)].copy()

    def profile_try(self, cap=64):
        """Durations (ms) and kinds of the launches of one try, run kernel by kernel."""
        ms = np.zeros(cap, np.float32)
        kind = np.zeros(cap, np.int32)
        n = C.c_uint32()
        _check(load().red_profile_try(self.h, _p(ms), _p(kind), cap, C.byref(n)))
        return ms[:n.value].copy(), kind[:n.value].copy()

    @property
    def interactions_per_eval(self):
        return int(load().red_interactions_per_eval(self.h))

    @property
    def kernel_launches(self):
        return int(load().red_kernel_launches(self.h))
