"""CPU oracle for the red.cuda hot path -- TEST INFRASTRUCTURE, not the product.

Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` may
import this package.  It loads ``liboracle.so`` (built from ``red_oracle.c``
with ``-O2 -ffp-contract=off``) and exposes numpy-friendly wrappers.  Every
routine restates a function of suliaron/red.cuda; the citations live in
``red_oracle.c``.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

# numpy mirrors of red.type/red_type.h records (field order and size preserved)
VAR4 = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("w", "<f8")])
PARAM = np.dtype([("mass", "<f8"), ("radius", "<f8"), ("density", "<f8"), ("cd", "<f8")])
BMD = np.dtype({"names": ["id", "body_type", "mig_type", "mig_stop_at"],
                "formats": ["<i4", "<i4", "<i4", "<f8"],
                "offsets": [0, 4, 8, 16], "itemsize": 24})
GAS = np.dtype({"names": ["rho", "sch", "eta", "tau", "mfp", "temp", "c_vth", "gas_decrease",
                          "t0", "t1", "e_folding_time", "alpha", "mean_molecular_weight",
                          "particle_diameter"],
                "formats": [("<f8", 2)] * 6 + ["<f8", "<i4"] + ["<f8"] * 6,
                "offsets": [0, 16, 32, 48, 64, 80, 96, 104, 112, 120, 128, 136, 144, 152],
                "itemsize": 160})
EVENT = np.dtype({"names": ["event_name", "t", "d",
                            "id0", "idx0", "p0", "r0", "v0",
                            "id1", "idx1", "p1", "r1", "v1",
                            "id2", "idx2", "p2", "r2", "v2",
                            "ps", "rs", "vs"],
                  "formats": ["<i4", "<f8", "<f8",
                              "<i4", "<u4", PARAM, VAR4, VAR4,
                              "<i4", "<u4", PARAM, VAR4, VAR4,
                              "<i4", "<u4", PARAM, VAR4, VAR4,
                              PARAM, VAR4, VAR4],
                  "offsets": [0, 8, 16,
                              24, 28, 32, 64, 96,
                              128, 132, 136, 168, 200,
                              232, 236, 240, 272, 304,
                              336, 368, 400],
                  "itemsize": 432})

STAR, GIANT, ROCKY, PROTO, SUPERPL, PL, TP = range(7)
EULER, RK2, RK4, RKF78 = 0, 1, 2, 4
SEM_GPU, SEM_CPU = 0, 1
EV_NONE, EV_HIT_CENTRUM, EV_EJECTION, EV_COLLISION = range(4)
ERR_NOT_IMPLEMENTED = 1


class Integrator(C.Structure):
    _fields_ = [("type", C.c_int32), ("adaptive", C.c_int32), ("error_check_for_tp", C.c_int32),
                ("sem", C.c_int32), ("tolerance", C.c_double), ("dt_try", C.c_double),
                ("dt_did", C.c_double), ("dt_next", C.c_double), ("n_tried", C.c_uint64),
                ("n_passed", C.c_uint64), ("n_failed", C.c_uint64), ("nthreads", C.c_int32)]


def build(force=False):
    """Compile red_oracle.c into _build/liboracle.so (gcc, OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "red_oracle.c")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src),
                                             os.path.getmtime(os.path.join(HERE, "red_oracle.h")))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-std=c11", "-Wall", "-o", tmp, src, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        u32p = C.POINTER(C.c_uint32)
        L.orc_grav_accel.argtypes = [C.c_int, u32p, P, P, P, P, C.c_int]
        L.orc_drag_accel.argtypes = [C.c_double, P, u32p, P, P, P, P]
        L.orc_drag_accel.restype = None
        L.orc_calc_dydx.argtypes = [C.c_int, C.c_int, C.c_double, u32p, P, P, P, P, P, P, C.c_int]
        L.orc_step.argtypes = [C.POINTER(Integrator), C.POINTER(C.c_double), u32p, P, P, P, P, P]
        L.orc_check_collision.argtypes = [C.c_int, C.c_double, C.c_double, C.c_uint32, P, P, P, P,
                                          P, C.c_uint32, u32p]
        L.orc_check_collision_mt.argtypes = [C.c_int, C.c_double, C.c_double, C.c_uint32, P, P, P, P,
                                             P, C.c_uint32, u32p, C.c_int]
        L.orc_check_ejection_hit_centrum.argtypes = [C.c_double, C.c_double, C.c_double, C.c_uint32,
                                                     P, P, P, P, P, C.c_uint32, u32p]
        L.orc_populate_sp_events.argtypes = [P, C.c_uint32]
        L.orc_populate_sp_events.restype = C.c_uint32
        L.orc_handle_collision.argtypes = [P, u32p, P, P, P, P, u32p]
        L.orc_handle_ejection_hit_centrum.argtypes = [P, C.c_uint32, P, P, P, P, u32p]
        L.orc_rebuild_vectors.argtypes = [C.c_uint32, P, P, P, P, u32p, u32p, u32p, P]
        L.orc_rebuild_vectors.restype = C.c_uint32
        L.orc_calc_radius.argtypes = [C.c_double, C.c_double]
        L.orc_calc_radius.restype = C.c_double
        L.orc_calc_density.argtypes = [C.c_double, C.c_double]
        L.orc_calc_density.restype = C.c_double
        L.orc_calc_position_after_collision.argtypes = [C.c_double, C.c_double, P, P, P]
        L.orc_calc_position_after_collision.restype = None
        L.orc_calc_velocity_after_collision.argtypes = [C.c_double, C.c_double, P, P, P]
        L.orc_calc_velocity_after_collision.restype = None
        L.orc_calc_physical_properties.argtypes = [P, P, P]
        L.orc_calc_physical_properties.restype = None
        L.orc_calc_integral.argtypes = [C.c_uint32, P, P, P, P, P]
        L.orc_calc_integral.restype = None
        L.orc_calc_energy_interacting.argtypes = [u32p, P, P, P, P, P, C.c_int]
        L.orc_calc_energy_interacting.restype = None
        L.orc_interactions_per_eval.argtypes = [u32p]
        L.orc_interactions_per_eval.restype = C.c_uint64
        L.orc_bound.argtypes = [u32p, C.c_int, u32p]
        L.orc_bound.restype = None
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(C.POINTER(C.c_uint32))


class Body:
    """Host copy of one red system: r, v (var4), p (param), md (metadata), playing[7]."""

    def __init__(self, r, v, p, md, playing, names=None):
        # private copies: the oracle integrates in place
        self.r = np.array(r, dtype=VAR4, copy=True, order="C")
        self.v = np.array(v, dtype=VAR4, copy=True, order="C")
        self.p = np.array(p, dtype=PARAM, copy=True, order="C")
        self.md = np.array(md, dtype=BMD, copy=True, order="C")
        self.playing = np.array(playing, dtype=np.uint32, copy=True)
        self.inactive = np.zeros(7, np.uint32)
        self.removed = np.zeros(7, np.uint32)
        self.names = names

    def copy(self):
        b = Body(self.r.copy(), self.v.copy(), self.p.copy(), self.md.copy(), self.playing.copy(),
                 None if self.names is None else list(self.names))
        b.inactive = self.inactive.copy()
        b.removed = self.removed.copy()
        return b

    @property
    def n(self):
        return int(self.playing.sum())


def grav_accel(b, sem=SEM_GPU, nthreads=1):
    a = np.zeros(b.n, VAR4)
    pl, plp = _u32(b.playing)
    rc = lib().orc_grav_accel(sem, plp, _p(b.md), _p(b.p), _p(b.r), _p(a), nthreads)
    return rc, a


def calc_dydx(b, i, t, r=None, v=None, gas=None, sem=SEM_GPU, nthreads=1):
    r = b.r if r is None else r
    v = b.v if v is None else v
    dy = np.zeros(b.n, VAR4)
    pl, plp = _u32(b.playing)
    rc = lib().orc_calc_dydx(sem, i, t, plp, _p(b.md), _p(b.p), _p(gas), _p(r), _p(v), _p(dy), nthreads)
    return rc, dy


def make_integrator(kind, dt, adaptive=False, tol=0.0, error_check_for_tp=False, sem=SEM_GPU,
                    nthreads=1):
    ig = Integrator()
    ig.type = kind
    ig.adaptive = int(adaptive)
    ig.error_check_for_tp = int(error_check_for_tp)
    ig.sem = sem
    ig.tolerance = tol
    ig.dt_try = dt
    ig.dt_next = dt
    ig.nthreads = nthreads
    return ig


def step(ig, b, t, gas=None):
    """One red integrator step in place on b.r, b.v.  Returns (rc, t_new)."""
    tt = C.c_double(t)
    pl, plp = _u32(b.playing)
    rc = lib().orc_step(C.byref(ig), C.byref(tt), plp, _p(b.md), _p(b.p), _p(gas), _p(b.r), _p(b.v))
    return rc, tt.value


def check_collision(b, t, factor, sem=SEM_GPU, cap=None, nthreads=1):
    cap = max(16, b.n) if cap is None else cap
    ev = np.zeros(cap, EVENT)
    n = C.c_uint32(0)
    rc = lib().orc_check_collision_mt(sem, t, factor, b.n, _p(b.md), _p(b.p), _p(b.r), _p(b.v), _p(ev),
                                      cap, C.byref(n), nthreads)
    return rc, ev[:min(n.value, cap)].copy(), n.value


def check_ejection_hit_centrum(b, t, ejection, hit_centrum, cap=None):
    cap = max(16, b.n) if cap is None else cap
    ev = np.zeros(cap, EVENT)
    n = C.c_uint32(0)
    rc = lib().orc_check_ejection_hit_centrum(t, ejection, hit_centrum, b.n, _p(b.md), _p(b.p),
                                              _p(b.r), _p(b.v), _p(ev), cap, C.byref(n))
    return rc, ev[:min(n.value, cap)].copy(), n.value


def handle_collision(b, ev):
    ev = np.ascontiguousarray(ev, dtype=EVENT).copy()
    n = C.c_uint32(len(ev))
    ina, inap = _u32(b.inactive)
    rc = lib().orc_handle_collision(_p(ev), C.byref(n), _p(b.r), _p(b.v), _p(b.p), _p(b.md), inap)
    b.inactive[:] = ina
    return rc, ev[:n.value].copy()


def handle_ejection_hit_centrum(b, ev):
    ev = np.ascontiguousarray(ev, dtype=EVENT).copy()
    ina, inap = _u32(b.inactive)
    rc = lib().orc_handle_ejection_hit_centrum(_p(ev), len(ev), _p(b.r), _p(b.v), _p(b.p), _p(b.md), inap)
    b.inactive[:] = ina
    return rc, ev


def rebuild_vectors(b):
    pl, plp = _u32(b.playing)
    ina, inap = _u32(b.inactive)
    rem, remp = _u32(b.removed)
    perm = np.zeros(max(1, b.n), np.int32)
    k = lib().orc_rebuild_vectors(b.n, _p(b.r), _p(b.v), _p(b.p), _p(b.md), plp, inap, remp, _p(perm))
    b.r, b.v, b.p, b.md = b.r[:k].copy(), b.v[:k].copy(), b.p[:k].copy(), b.md[:k].copy()
    b.playing[:], b.inactive[:], b.removed[:] = pl, ina, rem
    if b.names is not None:
        b.names = [b.names[i] for i in perm[:k]]
    return perm[:k].copy()


def calc_integral(b):
    out = np.zeros(10)
    lib().orc_calc_integral(b.n, _p(b.md), _p(b.p), _p(b.r), _p(b.v), _p(out))
    return out


def energy_interacting(b, nthreads=1):
    out = np.zeros(4)
    pl, plp = _u32(b.playing)
    lib().orc_calc_energy_interacting(plp, _p(b.md), _p(b.p), _p(b.r), _p(b.v), _p(out), nthreads)
    return out


def interactions_per_eval(playing):
    pl, plp = _u32(playing)
    return int(lib().orc_interactions_per_eval(plp))


def bound(playing, which):
    pl, plp = _u32(playing)
    out = np.zeros(4, np.uint32)
    lib().orc_bound(plp, which, out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return tuple(int(x) for x in out)
