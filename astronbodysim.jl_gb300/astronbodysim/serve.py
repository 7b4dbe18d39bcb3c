"""Continuous-batching request loop over the many-system engine.

Integrate-this-system requests arrive as a Poisson stream.  Every request is a
Plummer or Hernquist sphere (50/50) with N log-uniform in [n_min, n_max], a
step count uniform in [steps_min, steps_max], a softening uniform in
[eps_min, eps_max] and a fixed dt.  Arrived requests are handed to the engine
while its own queue is short (the engine admits them FIFO as arena space and
system slots free up); every engine.run() advances all resident systems
together.  Latency = completion time - arrival time.

Initial conditions come from a seeded pool of large spheres: a request of N
particles takes N consecutive particles of a pool sphere (the particles of a
sphere are independent draws), recentred, with masses 1/N.
"""
import math
import time

import numpy as np

from .ics import hernquist, plummer


class RequestStream:
    def __init__(self, rate=200.0, seed=0, n_min=256, n_max=65536, steps_min=100,
                 steps_max=5000, eps_min=1e-3, eps_max=1e-2, dt=1e-3, pool_size=4):
        self.rate = rate
        self.rng = np.random.default_rng(seed)
        self.n_min, self.n_max = n_min, n_max
        self.steps_min, self.steps_max = steps_min, steps_max
        self.eps_min, self.eps_max = eps_min, eps_max
        self.dt = dt
        self.pool = {
            "plummer": [plummer(n_max, seed=1000 + k, com=False) for k in range(pool_size)],
            "hernquist": [hernquist(n_max, seed=2000 + k, com=False) for k in range(pool_size)],
        }
        self.t = 0.0

    def next(self):
        """Next request: (arrival time, n, nsteps, eps, kind, pool index, offset)."""
        self.t += self.rng.exponential(1.0 / self.rate)
        n = int(round(math.exp(self.rng.uniform(math.log(self.n_min), math.log(self.n_max)))))
        nsteps = int(self.rng.integers(self.steps_min, self.steps_max + 1))
        eps = float(self.rng.uniform(self.eps_min, self.eps_max))
        kind = "plummer" if self.rng.random() < 0.5 else "hernquist"
        k = int(self.rng.integers(0, len(self.pool[kind])))
        off = int(self.rng.integers(0, self.n_max - n + 1))
        return {"arrival": self.t, "n": n, "nsteps": nsteps, "eps": eps, "kind": kind, "k": k,
                "off": off}

    def system(self, req):
        src = self.pool[req["kind"]][req["k"]]
        sl = slice(req["off"], req["off"] + req["n"])
        pos = src["pos"][sl].copy()
        vel = src["vel"][sl].copy()
        pos -= pos.mean(0)
        vel -= vel.mean(0)
        return {"pos": pos, "vel": vel, "mass": np.full(req["n"], 1.0 / req["n"])}


def _percentiles(x):
    x = np.asarray(x, dtype=float)
    if not x.size:
        return {"n": 0, "p50_s": None, "p99_s": None}
    return {"n": int(x.size), "p50_s": float(np.percentile(x, 50)),
            "p99_s": float(np.percentile(x, 99))}


def serve(engine, stream, duration, chunk_steps=16, max_engine_queue=32, drain_after=False,
          log=None, policy="fifo", overlap=True):
    """Run the request loop for `duration` seconds of wall time.  Arrivals stop
    at `duration`; with drain_after the loop then continues until every arrived
    request has finished.  policy "fifo" hands requests to the engine in
    arrival order; "sjf" hands the waiting request with the least work
    (N^2 x steps) first.

    With overlap (and an engine that has run_async) each chunk of engine steps
    is only launched; while the GPU runs it the loop takes new arrivals,
    builds their initial conditions, submits them and collects finished
    results, and the engine admits the submitted systems at the next chunk
    boundary.  Without it every chunk is run to completion first.

    Latency = completion time - arrival time.  Two sets of percentiles are
    reported: over the completed requests only, and over every offered
    request, where a request still waiting or running at the end counts with
    its age at the end -- a lower bound of its latency (right-censored), so
    under overload these figures are lower bounds, not estimates."""
    if policy not in ("fifo", "sjf"):
        raise ValueError("policy must be 'fifo' or 'sjf'")
    overlap = overlap and hasattr(engine, "run_async")
    t0 = time.perf_counter()
    pending = []          # arrived, not yet handed to the engine
    inflight = {}         # engine id -> request
    lat = []
    nxt = stream.next()
    offered = 0
    offered_pairs = 0.0
    done_pairs = 0.0
    st0 = engine.stats()
    running_chunk = False

    def collect(tdone):
        nonlocal done_pairs
        for rid in engine.drain_done():
            req = inflight.pop(rid)
            lat.append(tdone - req["arrival"])
            done_pairs += float(req["n"]) ** 2 * req["nsteps"]
            engine.fetch(rid, req["n"])

    while True:
        now = time.perf_counter() - t0
        while nxt["arrival"] <= min(now, duration):
            pending.append(nxt)
            offered += 1
            offered_pairs += float(nxt["n"]) ** 2 * nxt["nsteps"]
            nxt = stream.next()
        queued = engine.stats()["queued"]
        if policy == "sjf" and len(pending) > 1:
            pending.sort(key=lambda r: float(r["n"]) ** 2 * r["nsteps"])
        while pending and queued < max_engine_queue:
            req = pending.pop(0)
            rid = engine.submit(stream.system(req), req["eps"], stream.dt, req["nsteps"])
            inflight[rid] = req
            queued += 1
        if inflight:
            if overlap:
                k = engine.run_async(chunk_steps)  # waits for the previous chunk, launches the next
                running_chunk = k > 0
            else:
                engine.run(chunk_steps)
            tdone = time.perf_counter() - t0
            collect(tdone)
            if log:
                log(len(lat), tdone)
        elif now < duration:
            time.sleep(max(0.0, min(nxt["arrival"], duration) - now))
        if now >= duration and (not drain_after or (not pending and not inflight)):
            break
    if running_chunk:
        engine.sync()
        collect(time.perf_counter() - t0)
    wall = time.perf_counter() - t0
    st1 = engine.stats()
    lat = np.array(lat)
    censored = [wall - r["arrival"] for r in pending] + [wall - r["arrival"] for r in inflight.values()]
    served = st1["interactions"] - st0["interactions"]
    gpu_s = (st1["gpu_ms"] - st0["gpu_ms"]) / 1e3
    return {
        "duration_s": duration,
        "wall_s": wall,
        "offered_requests": offered,
        "offered_rate_per_s": offered / duration,
        "offered_interactions_per_s": offered_pairs / duration,
        "completed": int(lat.size),
        "latency_completed": _percentiles(lat),
        "latency_all_requests_lower_bound": dict(_percentiles(np.concatenate([lat, censored])),
                                                 censored=len(censored)),
        "served_interactions": served,
        "served_interactions_per_s_wall": served / wall,
        "served_interactions_per_s_gpu": served / gpu_s if gpu_s > 0 else None,
        "completed_interactions": done_pairs,
        "backlog_requests": len(pending) + len(inflight),
        "resident_at_end": st1["running"],
        "policy": policy,
        "overlap": overlap,
    }


def ensemble_systems(nsys=4096, seed=0, n_min=64, n_max=8192, eps_min=1e-3, eps_max=1e-2):
    """Batched-ensemble workload: nsys independent systems, N log-uniform in
    [n_min, n_max], even index Plummer (a = 1), odd Hernquist (a = 1, truncated
    at 100 a), masses 1/N, softening uniform in [eps_min, eps_max]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nsys):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        eps = float(rng.uniform(eps_min, eps_max))
        d = plummer(n, seed=seed * 100003 + k) if k % 2 == 0 else hernquist(n, seed=seed * 100003 + k)
        out.append((d, eps))
    return out
