"""Host-side mirror of AstroNbodySim.jl's Simulation / run API for the DirectSum
solver on the GPU device, driving libnbody_gb300.so through its C ABI.

Names, argument meaning and error behaviour follow the reference:
  Simulation(data; ForceSofteningTable, TimeStep, TimeBegin, TimeEnd, ...)
                                                 src/base/Config.jl:515-628, 968-1172
  compute_force(sim) / compute_force(sim, pos, h)  src/directsumgpu/gravity.jl:81-85,
                                                 src/directsum/gravity.jl:180-193
  compute_potential(sim)                          src/base/Potential.jl:21-24
  init_timesteps, leapfrog_half_kick, advance_and_find_timestep, find_min_endstep,
  step, run                                       src/directsumgpu/timestep.jl, src/run.jl
  TimeBetweenSnapshots + OutputFunc: snapshots at output times inside steps
  (find_next_sync_point_and_drift)               src/base/Timestep.jl:197-245
  total_kinetic / total_potential / total_energy / total_momentum /
  total_angular_momentum                          src/base/Energy.jl
Errors raised by the reference's CPU path (error("Timestep < MinStep ...")) come
back as NbodyError(NB_ERR_NUMERIC).  Units are stripped by the caller: every
value is a plain float in the caller's unit system with the matching G.
"""
import ctypes

import numpy as np

from . import _lib as L

LAWS = {"spline": L.NB_LAW_SPLINE_G2, "spline_g2": L.NB_LAW_SPLINE_G2, "plummer": L.NB_LAW_PLUMMER}
PRECISIONS = {"fp64": L.NB_PREC_FP64, "mixed": L.NB_PREC_MIXED}
CRITERIA = {"ref": L.NB_CRIT_REF, "eta_sqrt_eps": L.NB_CRIT_ETA_SQRT_EPS}


class GPU:
    """Device trait (src/base/Traits.jl); `id` is the CUDA ordinal."""

    def __init__(self, id=0):
        self.id = id


class DirectSum:
    """Gravity solver trait (src/base/Traits.jl)."""


class Newton:
    """Gravity model trait (src/base/Traits.jl): plain Newtonian forces."""


class Leapfrog:
    """Time integration trait: KDK leapfrog, i.e. the step loop between a
    forward and a backward half kick (src/run.jl:85-87, 171-173)."""


class Euler:
    """Time integration trait: the same step loop without the half kicks
    (src/run.jl:85-87 and 171-173 apply them only for Leapfrog)."""


class MOND1983Milgrom:
    """Gravity model trait: Newtonian forces scaled by the Milgrom (1983)
    interpolation nu(|a| / ACC0, MOND_nuIndex) (src/mond/milgrom1983.jl)."""


class PointMassField:
    """Background force of a point mass: a += -GM / |r|^2 * r / |r|, r = x -
    center (the attractor closure of test/Local-Timestep.jl:746)."""

    kind = L.NB_BG_POINT_MASS

    def __init__(self, GM, center=(0.0, 0.0, 0.0)):
        self.GM, self.center, self.rg = float(GM), tuple(float(c) for c in center), 0.0


class PseudoNewtonianField:
    """Background force of a compact object in the pseudo-Newtonian potential:
    a += -GM / (|r| - r_g)^2 * r / |r| (src/tools/BlackHole.jl:41-60)."""

    kind = L.NB_BG_PSEUDO_NEWTONIAN

    def __init__(self, GM, rg, center=(0.0, 0.0, 0.0)):
        self.GM, self.center, self.rg = float(GM), tuple(float(c) for c in center), float(rg)


# Checkpoint image header: magic[8], version, n, bytes, params_size, clock_size
# (int64 each), then nb_params.
_CKPT_PARAMS_OFFSET = 48


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Simulation:
    """DirectSum simulation resident on one GB300.

    data: mapping with "pos" (N,3), "vel" (N,3), "mass" (N,) and optional
    "collection" (N,) particle types 1..6 (default 1).
    TimeStep > 0 selects ConstantTimestep, TimeStep == 0 AdaptiveTimestep with
    TimeInterval = (TimeEnd - TimeBegin) / TimeBase (src/base/Config.jl:408-449).
    """

    def __init__(self, data, *, G=1.0, ForceSofteningTable=None, TimeStep=0.0, TimeBegin=0.0,
                 TimeEnd=0.1, TimeBase=1 << 30, ErrTolTimestep=0.025, MinStep=1.0e-8,
                 MaxStep=float("inf"), law="spline", precision="mixed", criterion="ref",
                 device=None, block=0, i_per_thread=0, j_split=0, tile_j=0, stages=0, tuning=None,
                 resort_every=0, bgforce=None,
                 GravityModel=None, ACC0=0.0, MOND_nuIndex=2.0, TimeIntegrationAlgorithm=None,
                 TimeBetweenSnapshots=None, OutputFunc=None):
        self._lib = L.load()
        p = L.nb_params()
        self._lib.nb_default_params(ctypes.byref(p))
        p.G = float(G)
        soft = ForceSofteningTable if ForceSofteningTable is not None else [1.0e-4] * 6
        soft = list(soft)
        if len(soft) != 6:
            raise ValueError("ForceSofteningTable needs 6 entries")
        for k in range(6):
            p.softening[k] = float(soft[k])
        p.law = LAWS[law]
        p.precision = PRECISIONS[precision]
        p.adaptive = 0 if TimeStep and TimeStep > 0 else 1
        p.criterion = CRITERIA[criterion]
        p.dt = float(TimeStep or 0.0)
        p.eta = float(ErrTolTimestep)
        p.min_step = float(MinStep)
        p.max_step = float(MaxStep)
        p.time_base = int(TimeBase)
        p.time_begin = float(TimeBegin)
        p.time_end = float(TimeEnd)
        p.device = (device.id if isinstance(device, GPU) else int(device or 0))
        # force post-processing (postprocessing_force, src/directsumgpu/gravity.jl:64-79)
        fields = list(bgforce) if isinstance(bgforce, (list, tuple)) else ([bgforce] if bgforce else [])
        if len(fields) > 1:
            raise ValueError("one analytic background field per simulation")
        if fields:
            f = fields[0]
            p.bg_kind, p.bg_gm, p.bg_rg = f.kind, f.GM, f.rg
            for k in range(3):
                p.bg_center[k] = f.center[k]
        if GravityModel is not None and (GravityModel is MOND1983Milgrom or
                                          isinstance(GravityModel, MOND1983Milgrom)):
            p.mond = L.NB_MOND_MILGROM1983
            p.mond_acc0 = float(ACC0)
            p.mond_nu_index = float(MOND_nuIndex)
        if tuning and not block and not i_per_thread and data is not None:
            # launch shape from the autotuner's table (nearest particle count)
            from . import autotune

            path = autotune.DEFAULT_TABLE if tuning == "auto" else tuning
            n0 = np.asarray(data["pos"]).reshape(-1, 3).shape[0]
            shape = autotune.lookup(n0, law=law, path=path)
            if shape:
                block, i_per_thread, j_split, tile_j, stages = shape
        p.block = int(block)
        p.i_per_thread = int(i_per_thread)
        p.j_split = int(j_split)
        p.tile_j = int(tile_j)
        p.stages = int(stages)
        p.resort_every = int(resort_every)
        self.tuned_shape = (int(block), int(i_per_thread), int(j_split), int(tile_j), int(stages))
        self.params = p
        alg = TimeIntegrationAlgorithm
        self.euler = alg is Euler or isinstance(alg, Euler) or alg == "Euler"
        if alg is not None and not self.euler and not (alg is Leapfrog or isinstance(alg, Leapfrog)
                                                       or alg == "Leapfrog"):
            raise ValueError("TimeIntegrationAlgorithm must be Leapfrog or Euler")
        # the library applies (or skips) the run's half kicks and keeps the
        # choice in checkpoint images
        p.algorithm = L.NB_ALG_EULER if self.euler else L.NB_ALG_LEAPFROG
        self.G = float(G)
        self.softening = [float(s) for s in soft]
        self.TimeBegin = float(TimeBegin)
        self.TimeEnd = float(TimeEnd)
        self.TimeStep = float(TimeStep or 0.0)
        self.TimeBase = int(TimeBase)
        self.adaptive = bool(p.adaptive)
        self.TimeInterval = (self.TimeEnd - self.TimeBegin) / self.TimeBase
        h = ctypes.c_void_p()
        rc = self._lib.nb_create(ctypes.byref(p), ctypes.byref(h))
        if rc != L.NB_OK:
            why = self._lib.nb_last_error(None)
            raise L.NbodyError(rc, "nb_create failed: %s" % (why.decode() if why else "?"))
        self.handle = h
        self.n = 0
        # sim.config.output.func: called with the simulation at every output
        # time (the initial conditions and each time the time line reaches
        # TimeBegin + k * TimeBetweenSnapshots)
        self.output_func = OutputFunc
        self.TimeBetweenSnapshots = 0.0
        if TimeBetweenSnapshots:
            self.set_snapshot_interval(TimeBetweenSnapshots)
        if data is not None:
            self.upload(data)

    # -- life cycle -------------------------------------------------------
    def close(self):
        if getattr(self, "handle", None):
            self._lib.nb_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        L.check(self.handle, rc)

    # -- data placement ----------------------------------------------------
    def upload(self, data):
        pos = _f64(data["pos"]).reshape(-1, 3)
        vel = _f64(data["vel"]).reshape(-1, 3)
        n = pos.shape[0]
        mass = _f64(np.broadcast_to(data["mass"], (n,)))
        coll = data.get("collection") if hasattr(data, "get") else None
        ctype = None if coll is None else np.ascontiguousarray(coll, dtype=np.int32)
        cols = [np.ascontiguousarray(pos[:, k]) for k in range(3)] + \
               [np.ascontiguousarray(vel[:, k]) for k in range(3)]
        self._ck(self._lib.nb_upload(self.handle, n, *[L.dptr(c) for c in cols], L.dptr(mass),
                                     L.i32ptr(ctype)))
        self.n = n
        self.mass = mass
        self.collection = (np.ones(n, dtype=np.int32) if ctype is None else ctype.copy())

    # -- checkpoint / restart ----------------------------------------------
    def checkpoint(self):
        """Image (bytes) of the device state: parameters, particles (x, v, a,
        pot, m, type, Ti_begstep, Ti_endstep) and the device time line
        (nb_checkpoint_save)."""
        nbytes = ctypes.c_int64()
        self._ck(self._lib.nb_checkpoint_size(self.handle, ctypes.byref(nbytes)))
        buf = np.empty(nbytes.value, dtype=np.uint8)
        self._ck(self._lib.nb_checkpoint_save(self.handle, buf.ctypes.data_as(ctypes.c_void_p),
                                              nbytes.value))
        return buf.tobytes()

    def restore(self, image):
        """Loads a checkpoint image into this handle (nb_checkpoint_load); the
        run continues bit-identically to the one that was saved."""
        buf = np.frombuffer(image, dtype=np.uint8)
        self._ck(self._lib.nb_checkpoint_load(self.handle, buf.ctypes.data_as(ctypes.c_void_p),
                                              buf.size))
        p = L.nb_params.from_buffer_copy(image, _CKPT_PARAMS_OFFSET)
        n = int(np.frombuffer(image, dtype=np.int64, count=1, offset=16)[0])
        # 11 FP64 arrays, types, two int64 bin arrays, the source permutation
        arrays = 11 * 8 * n + 2 * ((4 * n + 7) // 8 * 8) + 16 * n
        hdr = len(image) - arrays
        self.params = p
        self.euler = p.algorithm == L.NB_ALG_EULER
        self.G = p.G
        self.softening = list(p.softening)
        self.TimeBegin, self.TimeEnd = p.time_begin, p.time_end
        self.TimeStep = p.dt if not p.adaptive else 0.0
        self.TimeBase = int(p.time_base)
        self.adaptive = bool(p.adaptive)
        self.TimeInterval = (self.TimeEnd - self.TimeBegin) / self.TimeBase
        self.n = n
        self.mass = np.frombuffer(image, dtype=np.float64, count=n, offset=hdr + 10 * 8 * n).copy()
        self.collection = np.frombuffer(image, dtype=np.int32, count=n,
                                        offset=hdr + 11 * 8 * n).copy()

    def set_snapshot_interval(self, between):
        """TimeBetweenSnapshots (src/base/Config.jl:392-394, 436-439): output
        times TimeBegin + k * between; 0 turns output stops off."""
        self._ck(self._lib.nb_set_snapshot_interval(self.handle, float(between)))
        self.TimeBetweenSnapshots = float(between)

    def output_state(self):
        """(next output time on the integer line, next output time, stopped
        at an output, output stops so far)."""
        ni, nf = ctypes.c_int64(), ctypes.c_double()
        at, k = ctypes.c_int32(), ctypes.c_int64()
        self._ck(self._lib.nb_get_output_time(self.handle, ctypes.byref(ni), ctypes.byref(nf),
                                              ctypes.byref(at), ctypes.byref(k)))
        return ni.value, nf.value, bool(at.value), k.value

    def set_stream(self, stream_ptr):
        self._ck(self._lib.nb_set_stream(self.handle, ctypes.c_void_p(stream_ptr)))

    def stream(self):
        s = ctypes.c_void_p()
        self._ck(self._lib.nb_get_stream(self.handle, ctypes.byref(s)))
        return s.value or 0

    def download(self):
        n = self.n
        a = {k: np.empty(n) for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "pot")}
        tb = np.empty(n, dtype=np.int64)
        te = np.empty(n, dtype=np.int64)
        self._ck(self._lib.nb_download(self.handle, *[L.dptr(a[k]) for k in
                                                      ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "pot")],
                                       L.i64ptr(tb), L.i64ptr(te)))
        return {
            "pos": np.stack([a["x"], a["y"], a["z"]], 1),
            "vel": np.stack([a["vx"], a["vy"], a["vz"]], 1),
            "acc": np.stack([a["ax"], a["ay"], a["az"]], 1),
            "pot": a["pot"],
            "mass": self.mass.copy(),
            "ti_begstep": tb,
            "ti_endstep": te,
        }

    def upload_acc(self, acc):
        acc = _f64(acc).reshape(-1, 3)
        cols = [np.ascontiguousarray(acc[:, k]) for k in range(3)]
        self._ck(self._lib.nb_upload_acc(self.handle, *[L.dptr(c) for c in cols]))

    def upload_bins(self, ti_beg, ti_end):
        tb = np.ascontiguousarray(ti_beg, dtype=np.int64)
        te = np.ascontiguousarray(ti_end, dtype=np.int64)
        self._ck(self._lib.nb_upload_bins(self.handle, L.i64ptr(tb), L.i64ptr(te)))

    def time(self):
        ti = ctypes.c_int64()
        tf = ctypes.c_double()
        self._ck(self._lib.nb_get_time(self.handle, ctypes.byref(ti), ctypes.byref(tf)))
        return ti.value, tf.value


# ---------------------------------------------------------------------------
# Reference-named operations
# ---------------------------------------------------------------------------

def saverestart(sim, filename):
    """saverestart for (DirectSum, GPU) (src/restart.jl:14-19): the device state
    written to one file."""
    with open(filename, "wb") as f:
        f.write(sim.checkpoint())


def loadrestart(filename, device=None, OutputFunc=None):
    """loadrestart (src/restart.jl:129-139): a new Simulation on `device`
    (default: the saved one) holding the saved state, with the saved
    time-integration algorithm (Leapfrog or Euler) and snapshot schedule, as
    the reference's restart file keeps the whole SimConfig."""
    with open(filename, "rb") as f:
        image = f.read()
    p = L.nb_params.from_buffer_copy(image, _CKPT_PARAMS_OFFSET)
    between = float(np.frombuffer(image, dtype=np.float64, count=1,
                                  offset=_CKPT_PARAMS_OFFSET + ctypes.sizeof(L.nb_params))[0])
    inv = lambda d, v: next(k for k, x in d.items() if x == v)  # noqa: E731
    sim = Simulation(None, G=p.G, ForceSofteningTable=list(p.softening),
                     TimeStep=p.dt if not p.adaptive else 0.0, TimeBegin=p.time_begin,
                     TimeEnd=p.time_end, TimeBase=p.time_base, ErrTolTimestep=p.eta,
                     MinStep=p.min_step, MaxStep=p.max_step, law=inv(LAWS, p.law),
                     precision=inv(PRECISIONS, p.precision), criterion=inv(CRITERIA, p.criterion),
                     device=p.device if device is None else device, block=p.block,
                     i_per_thread=p.i_per_thread, j_split=p.j_split, tile_j=p.tile_j,
                     stages=p.stages, resort_every=p.resort_every,
                     TimeIntegrationAlgorithm=Euler if p.algorithm == L.NB_ALG_EULER else Leapfrog,
                     OutputFunc=OutputFunc)
    sim.restore(image)
    sim.TimeBetweenSnapshots = between
    return sim


def check_sync_point(sim):
    """check_sync_point (src/directsumgpu/timestep.jl:116-118): True when every
    particle's Ti_endstep is past the last min_endstep (a full sync point)."""
    v = ctypes.c_int32()
    sim._ck(sim._lib.nb_check_sync_point(sim.handle, ctypes.byref(v)))
    return bool(v.value)


def get_all_data(sim):
    """src/base/Config.jl:1228-1230 (download to host)."""
    return sim.download()


def set_softlen(sim, table):
    """set_softlen! (src/tools/SofteningLength.jl:87-89)."""
    arr = (ctypes.c_double * 6)(*[float(t) for t in table])
    sim._ck(sim._lib.nb_set_softening(sim.handle, arr))
    sim.softening = [float(t) for t in table]


def compute_force(sim, pos=None, SoftLength=None, want_potential=False):
    """compute_force(sim) on active particles, or the acceleration at probe
    points `pos` (M,3) with softening SoftLength (returns (M,3))."""
    if pos is None:
        sim._ck(sim._lib.nb_compute_force(sim.handle, L.NB_FORCE_POT if want_potential else 0))
        return None
    acc, _ = force_and_potential_at_points(sim, pos, SoftLength)
    return acc


def force_and_potential_at_points(sim, pos, SoftLength):
    pos = _f64(pos).reshape(-1, 3)
    m = pos.shape[0]
    cols = [np.ascontiguousarray(pos[:, k]) for k in range(3)]
    out = [np.empty(m) for _ in range(4)]
    sim._ck(sim._lib.nb_force_at_points(sim.handle, m, *[L.dptr(c) for c in cols], float(SoftLength),
                                        *[L.dptr(o) for o in out]))
    return np.stack(out[:3], 1), out[3]


def compute_potential(sim, pos=None, SoftLength=None, remove_self=True):
    """compute_potential(sim): potential of every particle, then the self-potential
    term of src/base/Potential.jl:5-24 (+G m / (h / 2.8)) as the reference's
    compute_potential(sim) does.  With `pos`, the potential at probe points."""
    if pos is not None:
        return force_and_potential_at_points(sim, pos, SoftLength)[1]
    sim._ck(sim._lib.nb_compute_potential(sim.handle))
    if remove_self:
        sim._ck(sim._lib.nb_remove_self_potential(sim.handle))
    return None


def init_timesteps(sim):
    sim._ck(sim._lib.nb_init_timesteps(sim.handle))


def leapfrog_half_kick(sim, forward):
    sim._ck(sim._lib.nb_half_kick(sim.handle, int(forward)))


def advance_and_find_timestep(sim):
    sim._ck(sim._lib.nb_kick(sim.handle))


def find_min_endstep(sim):
    v = ctypes.c_int64()
    sim._ck(sim._lib.nb_find_min_endstep(sim.handle, ctypes.byref(v)))
    return v.value


def drift_particles_adaptive_timestep(sim, next_int):
    sim._ck(sim._lib.nb_drift_to_int(sim.handle, int(next_int)))


def drift_particles_const_timestep(sim, next_float):
    sim._ck(sim._lib.nb_drift_to_float(sim.handle, float(next_float)))


def step(sim, nsteps=1):
    """step(sim, DirectSum, GPU) repeated nsteps times (CUDA-graph replay).
    With TimeBetweenSnapshots set, each step splits its drift at the output
    times inside it and calls sim.output_func there, as
    find_next_sync_point_and_drift does (src/base/Timestep.jl:197-245)."""
    nsteps = int(nsteps)
    if not sim.TimeBetweenSnapshots or sim.output_func is None:
        sim._ck(sim._lib.nb_step(sim.handle, nsteps))
        return
    done = 0
    k, at = ctypes.c_int64(), ctypes.c_int32()
    while done < nsteps:
        sim._ck(sim._lib.nb_step_until_output(sim.handle, nsteps - done, ctypes.byref(k),
                                              ctypes.byref(at)))
        done += k.value
        if at.value:
            sim.output_func(sim)


def step_until_output(sim, max_steps):
    """At most max_steps steps, stopping at the first output time reached:
    returns (steps completed, True if stopped at an output time).  The next
    call finishes the interrupted step."""
    k, at = ctypes.c_int64(), ctypes.c_int32()
    sim._ck(sim._lib.nb_step_until_output(sim.handle, int(max_steps), ctypes.byref(k),
                                          ctypes.byref(at)))
    return k.value, bool(at.value)


def counters(sim):
    """(steps taken by step(), pair evaluations they made)."""
    k = ctypes.c_int64()
    v = ctypes.c_double()
    sim._ck(sim._lib.nb_get_counters(sim.handle, ctypes.byref(k), ctypes.byref(v)))
    return k.value, v.value


def active_count(sim):
    v = ctypes.c_int64()
    sim._ck(sim._lib.nb_active_count(sim.handle, ctypes.byref(v)))
    return v.value


def const_step_count(begin, end, dt):
    """Number of loop iterations src/run.jl:101-168 performs in constant-step mode:
    the float time line t += dt until t >= End (same IEEE additions as the device)."""
    t = float(begin)
    k = 0
    while True:
        t = t + dt
        k += 1
        if t >= end:
            return k


def run(sim, nsteps=None):
    """src/run.jl:46-184 without logging: warm-up force, init timesteps,
    forward half kick, the initial snapshot (sim.output_func, if any), the step
    loop until TimeEnd (or exactly `nsteps` steps) with snapshots at the output
    times, backward half kick.  With TimeIntegrationAlgorithm Euler the half
    kicks are left out, as the reference does (the library applies the choice
    in nb_run_begin / nb_run_end)."""
    sim._ck(sim._lib.nb_run_begin(sim.handle))
    if sim.output_func is not None:
        sim.output_func(sim)  # src/run.jl:90
    if nsteps is not None:
        step(sim, nsteps)
    elif not sim.adaptive:
        step(sim, const_step_count(sim.TimeBegin, sim.TimeEnd, sim.TimeStep))
    else:
        while True:
            step(sim, 1)
            _, tf = sim.time()
            if tf >= sim.TimeEnd:
                break
    sim._ck(sim._lib.nb_run_end(sim.handle))


def diagnostics(sim, with_potential=True):
    d = L.nb_diag()
    sim._ck(sim._lib.nb_diagnostics(sim.handle, 1 if with_potential else 0, ctypes.byref(d)))
    return {
        "K": d.kinetic,
        "W": d.potential,
        "P": np.array(d.momentum[:]),
        "L": np.array(d.angular_momentum[:]),
    }


def total_kinetic(sim):
    return diagnostics(sim, with_potential=False)["K"]


def total_potential(sim):
    """total_potential(sim, DirectSum, ·) = 0.5 sum(pot .* mass) after a fresh
    potential pass (src/directsum/potential.jl:150-153)."""
    return diagnostics(sim, with_potential=True)["W"]


def total_energy(sim):
    d = diagnostics(sim, with_potential=True)
    return d["K"] + d["W"]


def total_momentum(sim):
    return diagnostics(sim, with_potential=False)["P"]


def total_angular_momentum(sim):
    return diagnostics(sim, with_potential=False)["L"]
