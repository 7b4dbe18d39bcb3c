"""Many-system engine: batching and continuous-batching serving on one GB300.

Thin host wrapper of the nb_engine_* / nb_batch_* C entry points.  The engine
keeps every admitted system resident in one device arena and advances all of
them together (constant-step leapfrog, mixed precision, one CUDA graph per
step); queued systems are admitted as arena space and slots free up.
"""
import ctypes

import numpy as np

from . import _lib as L
from .sim import LAWS


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Engine:
    def __init__(self, max_particles=1 << 24, max_systems=8192, G=1.0, law="spline", device=0,
                 max_steps_per_call=64, block=0, i_per_thread=0, tuning=None):
        self._lib = L.load()
        p = L.nb_engine_params()
        p.G = float(G)
        p.law = LAWS[law]
        p.device = int(device)
        p.max_particles = int(max_particles)
        p.max_systems = int(max_systems)
        p.max_steps_per_call = int(max_steps_per_call)
        if tuning and not block and not i_per_thread:
            # batch-force shape from the autotuner's table
            from . import autotune

            shape = autotune.lookup_batch(law=law, path=autotune.DEFAULT_TABLE if tuning == "auto"
                                          else tuning)
            if shape:
                block, i_per_thread = shape
        p.block = int(block)
        p.i_per_thread = int(i_per_thread)
        self.shape = (int(block) or 128, int(i_per_thread) or 2)
        h = ctypes.c_void_p()
        rc = self._lib.nb_engine_create(ctypes.byref(p), ctypes.byref(h))
        if rc != L.NB_OK:
            raise L.NbodyError(rc, "nb_engine_create failed")
        self.handle = h
        self.params = p

    def _ck(self, rc):
        if rc != L.NB_OK:
            msg = self._lib.nb_engine_last_error(self.handle)
            raise L.NbodyError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "handle", None):
            self._lib.nb_engine_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, data, softening, dt, nsteps):
        """Queue one system {"pos", "vel", "mass"}; returns its request id."""
        pos = _f64(data["pos"]).reshape(-1, 3)
        vel = _f64(data["vel"]).reshape(-1, 3)
        n = pos.shape[0]
        mass = _f64(np.broadcast_to(data["mass"], (n,)))
        cols = [np.ascontiguousarray(pos[:, k]) for k in range(3)] + \
               [np.ascontiguousarray(vel[:, k]) for k in range(3)] + [mass]
        rid = ctypes.c_int64()
        self._ck(self._lib.nb_batch_submit(self.handle, n, *[L.dptr(c) for c in cols], float(softening),
                                           float(dt), int(nsteps), ctypes.byref(rid)))
        return rid.value

    def run(self, max_steps=1 << 62):
        """Admit, advance all resident systems, retire finished ones; returns steps run."""
        k = ctypes.c_int64()
        self._ck(self._lib.nb_engine_run(self.handle, int(max_steps), ctypes.byref(k)))
        return k.value

    def run_async(self, max_steps=1 << 62):
        """nb_engine_run_async: completes the chunk in flight (if any), admits,
        launches the next chunk and returns while the GPU runs it; returns its
        step count (0: nothing resident)."""
        k = ctypes.c_int64()
        self._ck(self._lib.nb_engine_run_async(self.handle, int(max_steps), ctypes.byref(k)))
        return k.value

    def sync(self):
        """Waits for the chunk left by run_async."""
        self._ck(self._lib.nb_engine_sync(self.handle))

    def run_until_idle(self):
        while True:
            st = self.stats()
            if st["queued"] == 0 and st["running"] == 0:
                return
            self.run()

    def poll(self, rid):
        s = ctypes.c_int32()
        k = ctypes.c_int64()
        self._ck(self._lib.nb_batch_poll(self.handle, int(rid), ctypes.byref(s), ctypes.byref(k)))
        return s.value, k.value

    def fetch(self, rid, n):
        out = [np.empty(n) for _ in range(6)]
        self._ck(self._lib.nb_batch_fetch(self.handle, int(rid), *[L.dptr(o) for o in out]))
        return {"pos": np.stack(out[:3], 1), "vel": np.stack(out[3:], 1)}

    def cancel(self, rid):
        self._ck(self._lib.nb_batch_cancel(self.handle, int(rid)))

    def suspend(self, rid):
        """Evict a running system to host memory (nb_batch_suspend)."""
        self._ck(self._lib.nb_batch_suspend(self.handle, int(rid)))

    def resume(self, rid):
        """Queue a suspended system again (nb_batch_resume)."""
        self._ck(self._lib.nb_batch_resume(self.handle, int(rid)))

    def drain_done(self, cap=4096):
        """Ids of systems finished since the previous call."""
        out = []
        buf = (ctypes.c_int64 * cap)()
        while True:
            k = ctypes.c_int64()
            self._ck(self._lib.nb_engine_drain_done(self.handle, buf, cap, ctypes.byref(k)))
            out.extend(buf[i] for i in range(k.value))
            if k.value < cap:
                return out

    def stats(self):
        s = L.nb_engine_stats()
        self._ck(self._lib.nb_engine_get_stats(self.handle, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in L.nb_engine_stats._fields_}
