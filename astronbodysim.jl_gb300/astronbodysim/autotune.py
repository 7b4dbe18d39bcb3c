"""Autotuner for the force kernel's launch shape.

For each particle count it times nb_compute_force (mixed precision) with
every candidate shape -- the direct grid with (threads per CTA, targets per
thread, CTAs sharing an i-block's sources) from {128, 256} x {1, 2, 4} x
{1, .., 8}, and the persistent work-list kernel -- using CUDA events on the
handle's stream; then, at the fastest of those, the j-tile size (128, 256,
512 sources) and the depth of the shared-memory ring (3, 4, 6 stages).  The
fastest shape goes into a JSON table (tuning_gb300.json next to this file, or
a path given by the caller) as "block x targets x j-split x tile x stages".
Simulation(tuning=...) looks the table up by the nearest particle count of the
same law; without a table the library's built-in rule applies.
"""
import json
import math
import os

import numpy as np

from .ics import plummer

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_TABLE = os.path.join(HERE, "tuning_gb300.json")

CANDIDATES = [
    {"block": 128, "i_per_thread": 1, "j_split": 1},
    {"block": 128, "i_per_thread": 2, "j_split": 1},
    {"block": 128, "i_per_thread": 4, "j_split": 1},
    {"block": 256, "i_per_thread": 1, "j_split": 1},
    {"block": 256, "i_per_thread": 2, "j_split": 1},
    {"block": 128, "i_per_thread": 1, "j_split": 2},
    {"block": 128, "i_per_thread": 1, "j_split": 4},
    {"block": 128, "i_per_thread": 2, "j_split": 2},
    {"block": 128, "i_per_thread": 2, "j_split": 4},
    {"block": 128, "i_per_thread": 2, "j_split": 8},
    {"block": 128, "i_per_thread": 1, "j_split": 8},
    {"block": 256, "i_per_thread": 1, "j_split": 2},
    {"block": 128, "i_per_thread": 2, "j_split": 4},
    {"block": 256, "i_per_thread": 1, "j_split": 2},
    {"block": -1, "i_per_thread": 0, "j_split": 1},  # persistent work list
]


def _time_force(sim, reps):
    import torch

    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    from .sim import compute_force

    compute_force(sim)  # warm-up (also captures nothing; plain launches)
    times = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        compute_force(sim)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return float(np.median(times))


TILES = [(128, 3), (128, 4), (128, 6), (256, 3), (256, 6), (512, 3), (512, 4)]


def shape_key(block, ipt, js, tile=256, stages=4):
    return "%dx%dx%dx%dx%d" % (block, ipt, js, tile, stages)


def tune(sizes, law="spline", reps=3, eps=1e-3, seed=0, log=print):
    """Returns {"law": law, "entries": [{"n", "best", "ms": {shape: ms}}]}."""
    from .sim import Simulation

    entries = []
    for n in sizes:
        data = plummer(int(n), seed=seed)
        res = {}

        def run(block, ipt, js, tile=0, stages=0):
            sim = Simulation(data, ForceSofteningTable=[eps] * 6, TimeStep=1e-4, precision="mixed",
                             law=law, block=block, i_per_thread=ipt, j_split=js, tile_j=tile,
                             stages=stages)
            ms = _time_force(sim, reps)
            sim.close()
            return ms

        for c in CANDIDATES:
            if c["block"] == -1:
                res["worklist"] = run(-1, 0, 1)
            else:
                res[shape_key(c["block"], c["i_per_thread"], c["j_split"])] = run(
                    c["block"], c["i_per_thread"], c["j_split"])
        grid = min((k for k in res if k != "worklist"), key=res.get)
        b, i, j = (int(v) for v in grid.split("x")[:3])
        if b == 128 and i in (1, 2):
            for t, s in TILES:
                res[shape_key(b, i, j, t, s)] = run(b, i, j, t, s)
        best = min(res, key=res.get)
        entries.append({"n": int(n), "best": best, "ms": res,
                        "g_interactions_per_s": float(n) * n / (res[best] / 1e3) / 1e9})
        if log:
            log("n=%d best=%s %.3f ms (%s)" % (n, best, res[best],
                                               ", ".join("%s %.3f" % kv for kv in res.items())))
    return {"law": law, "entries": entries}


BATCH_CANDIDATES = [(128, 1), (128, 2), (256, 1), (256, 2)]


def tune_batch(nsys=1024, steps=40, law="spline", seed=5, log=print):
    """Batch-force shape for the many-system engine: runs an ensemble of nsys
    systems (N log-uniform in [64, 8192], half Plummer, half Hernquist) for
    `steps` steps with every shape and keeps the one with the highest
    interactions per GPU second."""
    from .engine import Engine
    from .serve import ensemble_systems

    ens = ensemble_systems(nsys, seed=seed)
    tot = sum(d["pos"].shape[0] for d, _ in ens)
    res = {}
    for b, i in BATCH_CANDIDATES:
        eng = Engine(max_particles=tot + 4096, max_systems=nsys, max_steps_per_call=steps, law=law,
                     block=b, i_per_thread=i)
        for d, eps in ens:
            eng.submit(d, eps, 1e-3, steps)
        eng.run_until_idle()
        st = eng.stats()
        eng.close()
        res["%dx%d" % (b, i)] = st["interactions"] / (st["gpu_ms"] / 1e3) / 1e9
    best = max(res, key=res.get)
    if log:
        log("batch best=%s (%s G interactions/s)" % (best, ", ".join("%s %.0f" % kv for kv in res.items())))
    return {"law": law, "best": best, "g_interactions_per_s": res, "systems": nsys, "steps": steps}


def save_batch(entry, path=DEFAULT_TABLE):
    old = load(path) or {}
    old.setdefault("batch", {})[entry["law"]] = entry
    with open(path, "w") as f:
        json.dump(old, f, indent=1, sort_keys=True)


def lookup_batch(law="spline", path=DEFAULT_TABLE):
    """(block, i_per_thread) of the engine's batch force, or None."""
    t = load(path)
    if not t or "batch" not in t or law not in t["batch"]:
        return None
    b, i = t["batch"][law]["best"].split("x")
    return int(b), int(i)


def save(table, path=DEFAULT_TABLE):
    old = load(path) or {}
    old[table["law"]] = table["entries"]
    with open(path, "w") as f:
        json.dump(old, f, indent=1, sort_keys=True)


def load(path=DEFAULT_TABLE):
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def lookup(n, law="spline", path=DEFAULT_TABLE):
    """(block, i_per_thread, j_split, tile_j, stages) of the tuned shape
    nearest to n in log space, or None."""
    t = load(path)
    if not t or law not in t or not t[law] or not isinstance(t[law], list):
        return None
    e = min(t[law], key=lambda e: abs(math.log(e["n"]) - math.log(max(1, n))))
    best = e["best"]
    if best == "worklist":
        return -1, 0, 0, 0, 0
    v = [int(x) for x in best.split("x")]
    if len(v) == 3:
        v += [256, 4]
    return tuple(v)
