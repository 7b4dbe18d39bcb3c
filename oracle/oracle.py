"""ctypes wrapper of the CPU oracle (test infrastructure, not the product).

Only tests/, the smoke check and the benchmark's CPU-baseline leg import this
module.  It restates AstroNbodySim.jl's CPU Float64 direct sum
(src/directsum/gravity.jl, src/directsum/potential.jl) and integrator
(src/base/Timestep.jl, src/run.jl); see nbody_oracle.c for the line-by-line map.
"""
import ctypes
import os

import numpy as np

from .build import build_oracle

LAW_SPLINE_G2 = 0
LAW_PLUMMER = 1
CRIT_REF = 0
CRIT_ETA_SQRT_EPS = 1

_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_u8p = ctypes.POINTER(ctypes.c_uint8)


class _State(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("x", _dp), ("y", _dp), ("z", _dp),
        ("vx", _dp), ("vy", _dp), ("vz", _dp),
        ("ax", _dp), ("ay", _dp), ("az", _dp),
        ("pot", _dp), ("m", _dp),
        ("type", _i32p),
        ("ti_beg", _i64p), ("ti_end", _i64p),
        ("soft", ctypes.c_double * 6),
        ("G", ctypes.c_double),
        ("law", ctypes.c_int32),
        ("adaptive", ctypes.c_int32),
        ("criterion", ctypes.c_int32),
        ("nthreads", ctypes.c_int32),
        ("dt", ctypes.c_double),
        ("eta", ctypes.c_double),
        ("min_step", ctypes.c_double),
        ("max_step", ctypes.c_double),
        ("time_base", ctypes.c_int64),
        ("time_interval", ctypes.c_double),
        ("t_int", ctypes.c_int64),
        ("last_t_int", ctypes.c_int64),
        ("t_float", ctypes.c_double),
        ("last_t_float", ctypes.c_double),
        ("mode", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("bg_kind", ctypes.c_int32),
        ("mond", ctypes.c_int32),
        ("bg_gm", ctypes.c_double),
        ("bg_cx", ctypes.c_double),
        ("bg_cy", ctypes.c_double),
        ("bg_cz", ctypes.c_double),
        ("bg_rg", ctypes.c_double),
        ("mond_acc0", ctypes.c_double),
        ("mond_nu_index", ctypes.c_double),
        ("time_begin", ctypes.c_double),
        ("outputs_on", ctypes.c_int32),
        ("pad2", ctypes.c_int32),
        ("between_float", ctypes.c_double),
        ("between_int", ctypes.c_int64),
        ("next_out_float", ctypes.c_double),
        ("next_out_int", ctypes.c_int64),
        ("snap", _dp),
        ("snap_cap", ctypes.c_int64),
        ("snap_count", ctypes.c_int64),
    ]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        L = ctypes.CDLL(path)
        L.or_force.restype = ctypes.c_int
        L.or_force.argtypes = [
            ctypes.c_int64, _dp, _dp, _dp, _dp,
            ctypes.c_int64, _dp, _dp, _dp, _dp, _u8p,
            ctypes.c_double, ctypes.c_int, ctypes.c_int,
            _dp, _dp, _dp, _dp, ctypes.c_int,
        ]
        for name in ("or_compute_force",):
            getattr(L, name).argtypes = [ctypes.POINTER(_State), ctypes.c_int]
            getattr(L, name).restype = ctypes.c_int
        for name in ("or_compute_potential", "or_init_timesteps", "or_kick", "or_step",
                     "or_run_begin", "or_run_end", "or_sync_and_drift"):
            getattr(L, name).argtypes = [ctypes.POINTER(_State)]
            getattr(L, name).restype = ctypes.c_int
        L.or_half_kick.argtypes = [ctypes.POINTER(_State), ctypes.c_int]
        L.or_half_kick.restype = ctypes.c_int
        L.or_find_min_endstep.argtypes = [ctypes.POINTER(_State)]
        L.or_find_min_endstep.restype = ctypes.c_int64
        L.or_drift_to_int.argtypes = [ctypes.POINTER(_State), ctypes.c_int64]
        L.or_drift_to_int.restype = ctypes.c_int
        L.or_drift_to_float.argtypes = [ctypes.POINTER(_State), ctypes.c_double]
        L.or_drift_to_float.restype = ctypes.c_int
        L.or_diagnostics.argtypes = [ctypes.POINTER(_State), _dp]
        L.or_diagnostics.restype = ctypes.c_int
        L.or_jl_sum.argtypes = [_dp, ctypes.c_int64]
        L.or_jl_sum.restype = ctypes.c_double
        L.or_compensated_sum.argtypes = [_dp, ctypes.c_int64]
        L.or_compensated_sum.restype = ctypes.c_double
        L.or_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a, ct=_dp):
    if a is None:
        return ct()
    return a.ctypes.data_as(ct)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def jl_sum(a):
    a = _f64(a)
    return lib().or_jl_sum(_ptr(a), a.size)


def compensated_sum(a):
    a = _f64(a)
    return lib().or_compensated_sum(_ptr(a), a.size)


def max_threads():
    return lib().or_max_threads()


def force(src_pos, src_mass, tgt_pos, tgt_h, G=1.0, law=LAW_SPLINE_G2, mode=0,
          want_acc=True, want_pot=True, active=None, nthreads=0):
    """Acceleration and potential per unit mass at each target (FP64).

    src_pos (n,3), src_mass (n,), tgt_pos (t,3), tgt_h scalar or (t,).
    Restates src/directsum/gravity.jl:37-46 and src/directsum/potential.jl:33-41.
    """
    sp = _f64(src_pos).reshape(-1, 3)
    sx, sy, sz = (np.ascontiguousarray(sp[:, k]) for k in range(3))
    sm = _f64(src_mass)
    tp = _f64(tgt_pos).reshape(-1, 3)
    tx, ty, tz = (np.ascontiguousarray(tp[:, k]) for k in range(3))
    nt = tp.shape[0]
    th = np.broadcast_to(_f64(tgt_h), (nt,)).copy()
    acc = np.zeros((3, nt)) if want_acc else None
    pot = np.zeros(nt) if want_pot else None
    act = None
    if active is not None:
        act = np.ascontiguousarray(active, dtype=np.uint8)
    rc = lib().or_force(
        sm.size, _ptr(sx), _ptr(sy), _ptr(sz), _ptr(sm),
        nt, _ptr(tx), _ptr(ty), _ptr(tz), _ptr(th), _ptr(act, _u8p),
        G, law, mode,
        _ptr(acc[0]) if want_acc else _dp(), _ptr(acc[1]) if want_acc else _dp(),
        _ptr(acc[2]) if want_acc else _dp(), _ptr(pot), nthreads)
    if rc != 0:
        raise RuntimeError("oracle force failed: %d" % rc)
    return (acc.T.copy() if want_acc else None), pot


class OracleSim:
    """Integrator state mirroring AstroNbodySim's Simulation for DirectSum on CPU.

    Arrays are owned here (numpy) and passed to the C restatement by pointer.
    """

    def __init__(self, pos, vel, mass, ptype=None, soft=(1e-4,) * 6, G=1.0, law=LAW_SPLINE_G2,
                 dt=None, eta=0.025, min_step=1e-8, max_step=float("inf"), time_base=1 << 30,
                 time_begin=0.0, time_end=0.1, criterion=CRIT_REF, mode=0, nthreads=0,
                 bg_kind=0, bg_gm=0.0, bg_center=(0.0, 0.0, 0.0), bg_rg=0.0, mond=0,
                 mond_acc0=0.0, mond_nu_index=2.0, between_snapshots=0.0, max_snapshots=0):
        pos = _f64(pos).reshape(-1, 3)
        vel = _f64(vel).reshape(-1, 3)
        n = pos.shape[0]
        self.n = n
        self.x, self.y, self.z = (np.ascontiguousarray(pos[:, k]) for k in range(3))
        self.vx, self.vy, self.vz = (np.ascontiguousarray(vel[:, k]) for k in range(3))
        self.ax, self.ay, self.az = np.zeros(n), np.zeros(n), np.zeros(n)
        self.pot = np.zeros(n)
        self.m = _f64(np.broadcast_to(mass, (n,))).copy()
        self.type = np.ones(n, dtype=np.int32) if ptype is None else np.ascontiguousarray(ptype, dtype=np.int32)
        self.ti_beg = np.zeros(n, dtype=np.int64)
        self.ti_end = np.zeros(n, dtype=np.int64)
        s = _State()
        s.n = n
        for name in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "pot", "m"):
            setattr(s, name, _ptr(getattr(self, name)))
        s.type = _ptr(self.type, _i32p)
        s.ti_beg = _ptr(self.ti_beg, _i64p)
        s.ti_end = _ptr(self.ti_end, _i64p)
        for k in range(6):
            s.soft[k] = float(soft[k])
        s.G = G
        s.law = law
        s.adaptive = 0 if dt else 1
        s.criterion = criterion
        s.nthreads = nthreads
        s.dt = dt or 0.0
        s.eta = eta
        s.min_step = min_step
        s.max_step = max_step
        s.time_base = time_base
        s.time_interval = (time_end - time_begin) / time_base
        s.t_int = 0
        s.last_t_int = 0
        s.t_float = time_begin
        s.last_t_float = time_begin
        s.mode = mode
        s.bg_kind = bg_kind
        s.bg_gm = bg_gm
        s.bg_cx, s.bg_cy, s.bg_cz = (float(c) for c in bg_center)
        s.bg_rg = bg_rg
        s.mond = mond
        s.mond_acc0 = mond_acc0
        s.mond_nu_index = mond_nu_index
        # snapshot schedule (src/base/Config.jl:436-439, 749-750)
        s.time_begin = time_begin
        s.outputs_on = 1 if between_snapshots > 0 else 0
        s.between_float = between_snapshots
        s.between_int = int(np.floor(between_snapshots / s.time_interval)) if s.adaptive else 0
        s.next_out_float = time_begin + between_snapshots
        s.next_out_int = s.between_int
        self._snap = np.zeros((max(max_snapshots, 1), 2 + 6 * n))
        s.snap = _ptr(self._snap)
        s.snap_cap = max_snapshots
        s.snap_count = 0
        self._s = s

    def _call(self, name, *args):
        rc = getattr(lib(), name)(ctypes.byref(self._s), *args)
        if rc != 0:
            raise RuntimeError("oracle %s failed: %d" % (name, rc))

    @property
    def pos(self):
        return np.stack([self.x, self.y, self.z], axis=1)

    @property
    def vel(self):
        return np.stack([self.vx, self.vy, self.vz], axis=1)

    @property
    def acc(self):
        return np.stack([self.ax, self.ay, self.az], axis=1)

    @property
    def t_int(self):
        return self._s.t_int

    @property
    def t_float(self):
        return self._s.t_float

    def compute_force(self, want_pot=False):
        self._call("or_compute_force", 1 if want_pot else 0)

    def compute_potential(self):
        self._call("or_compute_potential")

    def init_timesteps(self):
        self._call("or_init_timesteps")

    def half_kick(self, forward):
        self._call("or_half_kick", forward)

    def kick(self):
        self._call("or_kick")

    def find_min_endstep(self):
        return lib().or_find_min_endstep(ctypes.byref(self._s))

    def drift_to_int(self, t):
        self._call("or_drift_to_int", t)

    def drift_to_float(self, t):
        self._call("or_drift_to_float", t)

    def sync_and_drift(self):
        """find_next_sync_point_and_drift (src/base/Timestep.jl:197-245)."""
        self._call("or_sync_and_drift")

    @property
    def snapshots(self):
        """Recorded snapshots: list of dicts with t_float, t_int, pos (n,3), vel (n,3)."""
        out = []
        n = self.n
        for k in range(min(self._s.snap_count, self._s.snap_cap)):
            r = self._snap[k]
            out.append({"t_float": float(r[0]), "t_int": int(r[1]),
                        "pos": np.stack([r[2:2 + n], r[2 + n:2 + 2 * n], r[2 + 2 * n:2 + 3 * n]], 1),
                        "vel": np.stack([r[2 + 3 * n:2 + 4 * n], r[2 + 4 * n:2 + 5 * n],
                                         r[2 + 5 * n:2 + 6 * n]], 1)})
        return out

    @property
    def next_output(self):
        return self._s.next_out_int, self._s.next_out_float

    def step(self, nsteps=1):
        for _ in range(nsteps):
            self._call("or_step")

    def run_begin(self):
        self._call("or_run_begin")

    def run_end(self):
        self._call("or_run_end")

    def diagnostics(self):
        out = np.zeros(8)
        rc = lib().or_diagnostics(ctypes.byref(self._s), _ptr(out))
        if rc != 0:
            raise RuntimeError("oracle diagnostics failed")
        return {"K": out[0], "W": out[1], "P": out[2:5].copy(), "L": out[5:8].copy()}
