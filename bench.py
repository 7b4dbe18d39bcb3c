"""Benchmark of the direct-sum hot path on one GB300 (replicas per GPU for N > 1).

Workload: Plummer sphere N = 2^20 (G = M = a = 1), equal masses, softening
eps = 1e-3 (Gadget-2 spline law, the reference's pair law), mixed precision
(FP32 pairs relative to FP64 tile origins, compensated sums, FP64 state),
constant-step leapfrog at dt = 1e-4.  One step = one KDK step of
step(sim, DirectSum, GPU): drift, FP32 pack, force on all N targets from all N
sources (N^2 interactions), kick -- one CUDA-graph replay.

Prints one JSON line (rank 0).  `value` = interactions/s of the timed steps with
state resident in HBM; `e2e` = the same metric through the public API with the
state copied from pinned host memory before and back after every step.
`--impl reference` times the CPU Float64 restatement of the reference's direct
sum (the oracle) on all host cores instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.join(REPO, "astronbodysim.jl_gb300")
for _p in (REPO, PKG_ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "G interactions/s at N=2^20, mixed vs FP64 at stated error; batch p50/p99 latency"
UNIT = "G interactions/s"
N_DEFAULT = 1 << 20
EPS = 1.0e-3
DT = 1.0e-4
FLOP_PER_INTERACTION = 20
L2_FLUSH_BYTES = 256 << 20
# kernels in one step graph at N = 2^20: clock advance, drift, 2 bounding-box,
# Morton keys, 8 radix passes x (histogram, 3-kernel scan, scatter), pack,
# force, kick, clock end; plus the join of a j-split force (or the fix-up of
# the work-list force)
STEP_KERNELS = 49


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_oracle_rate(data, n_targets, seed=7, nthreads=0, law="spline"):
    """Oracle (CPU Float64 restatement of src/directsum/gravity.jl:37-46, 80-101)
    on a bounded sample: n_targets seeded targets x all sources."""
    from oracle import oracle

    rng = np.random.default_rng(seed)
    idx = rng.choice(data["pos"].shape[0], size=n_targets, replace=False)
    t0 = time.perf_counter()
    oracle.force(data["pos"], data["mass"], data["pos"][idx], EPS, want_pot=False,
                 nthreads=nthreads,
                 law=oracle.LAW_SPLINE_G2 if law == "spline" else oracle.LAW_PLUMMER)
    dt = time.perf_counter() - t0
    return n_targets * data["pos"].shape[0] / dt, dt, oracle.max_threads() if nthreads == 0 else nthreads


def measured_fp32_peak(device):
    """FP32 FMA throughput measured on this GPU (nb_selftest_fp32_peak:
    independent fma.rn.f32x2 chains, CUDA events), TFLOP/s at 2 flop per lane."""
    import ctypes

    from astronbodysim import _lib as L

    tf, ms = ctypes.c_double(), ctypes.c_double()
    rc = L.load().nb_selftest_fp32_peak(int(device), 1, ctypes.byref(tf), ctypes.byref(ms))
    if rc != 0:
        return None
    return tf.value


def timed_forces(nb, sim, stream, flush, reps):
    """CUDA-event times (ms) of `reps` nb_compute_force calls on the handle's
    stream, each after an L2 flush outside the events."""
    import torch

    ev = []
    for _ in range(reps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        nb.compute_force(sim)
        with torch.cuda.stream(stream):
            e1.record(stream)
        ev.append((e0, e1))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def general_mass_leg(nb, data, args, local, stream, flush, oracle_targets=1024):
    """The same Plummer positions with masses m (1 + d_i), d_i ~ U[-1e-3, 1e-3]
    (seeded), so that no tile has one common mass: force throughput (CUDA
    events) and relative force errors against the oracle."""
    from oracle import oracle

    n = data["pos"].shape[0]
    rng = np.random.default_rng(77)
    d = {"pos": data["pos"], "vel": data["vel"],
         "mass": data["mass"] * (1.0 + rng.uniform(-1e-3, 1e-3, size=n))}
    sim = nb.Simulation(d, ForceSofteningTable=[EPS] * 6, TimeStep=DT, TimeEnd=1.0,
                        precision="mixed", law=args.law, device=local, tuning="auto")
    sim.set_stream(stream.cuda_stream)
    nb.compute_force(sim)
    ms = statistics.median(timed_forces(nb, sim, stream, flush, 3))
    sub = np.sort(rng.choice(n, size=oracle_targets, replace=False))
    g = nb.get_all_data(sim)
    a_ref, _ = oracle.force(d["pos"], d["mass"], d["pos"][sub], EPS, want_pot=False,
                            law=oracle.LAW_SPLINE_G2 if args.law == "spline" else oracle.LAW_PLUMMER)
    e = np.linalg.norm(g["acc"][sub] - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
    sim.close()
    return {"value": float(n) * n / (ms / 1e3) / 1e9, "unit": UNIT, "force_ms": ms,
            "masses": "m_i = (1/N)(1 + d_i), d_i ~ U[-1e-3, 1e-3]",
            "force_rel_median": float(np.median(e)), "force_rel_p99": float(np.quantile(e, 0.99)),
            "force_rel_max": float(e.max()), "error_targets": oracle_targets}


def fp64_leg(nb, data, args, local, stream, n_targets):
    """Plain FP64 form at full occupancy: acceleration only at n_targets
    seeded particles (probe points) from all N sources, one launch of
    k_force_fp64 timed with CUDA events around the call on the handle's
    stream (the call also copies the n_targets positions in and the
    accelerations out, 48 B per target)."""
    import ctypes

    import torch

    from astronbodysim import _lib as L
    from oracle import oracle

    n = data["pos"].shape[0]
    rng = np.random.default_rng(78)
    sub = np.sort(rng.choice(n, size=n_targets, replace=False))
    sim = nb.Simulation(data, ForceSofteningTable=[EPS] * 6, TimeStep=DT, TimeEnd=1.0,
                        precision="fp64", law=args.law, device=local)
    sim.set_stream(stream.cuda_stream)
    p = data["pos"][sub]
    cols = [np.ascontiguousarray(p[:, k]) for k in range(3)]
    out = [np.empty(n_targets) for _ in range(3)]
    lib = sim._lib
    nullp = ctypes.POINTER(ctypes.c_double)()

    def call(m):
        sim._ck(lib.nb_force_at_points(sim.handle, m, *[L.dptr(c) for c in cols], EPS,
                                       *[L.dptr(o) for o in out], nullp))

    call(1024)  # warm-up
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    call(n_targets)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    k = 256
    a_ref, _ = oracle.force(data["pos"], data["mass"], p[:k], EPS, want_pot=False,
                            law=oracle.LAW_SPLINE_G2 if args.law == "spline" else oracle.LAW_PLUMMER)
    a = np.stack([o[:k] for o in out], 1)
    e = np.linalg.norm(a - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
    sim.close()
    return {"value": float(n_targets) * n / (ms / 1e3) / 1e9, "unit": UNIT, "ms": ms,
            "sample": "%d targets x %d sources, acceleration only, one launch (%d CTAs of 128)"
                      % (n_targets, n, (n_targets + 127) // 128),
            "force_rel_max_256": float(e.max())}


def relaunch_replicas(gpus):
    """`bench.py --gpus N` started as one process: run it again as N replica
    processes (one per GPU) under torch.distributed.run on this node, and
    return their exit status.  Rank 0 prints the job's JSON line."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", str(gpus), "--master-addr", "127.0.0.1", "--master-port", str(port),
           os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def run_dry(args):
    """Launcher and aggregation check without a GPU: every rank (gloo) times
    a fixed host workload that takes rank + 1 units of 50 ms as its "steps",
    then the job time is the MAX over ranks and rank 0 prints the JSON line
    with n_gpus = world size, as the GPU bench does."""
    import torch.distributed as dist

    ws, rank, _ = dist_env()
    if ws > 1:
        dist.init_process_group("gloo")
        dist.barrier()
    t0 = time.perf_counter()
    time.sleep(0.05 * (rank + 1))
    total_s = time.perf_counter() - t0
    n = 1024
    value, e2e, total_s, _ = replica_rates(ws, args.steps, args.steps, n, total_s, total_s, None)
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                          "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * total_s / args.steps, "dry_run": True,
                          "scaling": "weak"}), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


def replica_rates(ws, steps, e2e_steps, n, total_s, t_e2e, device):
    """Whole-job rates of ws independent replicas (one system of n particles
    per rank, no data-path collective): the job time is the slowest rank's
    (MAX over ranks), and the job did ws x steps x n^2 interactions."""
    if ws > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([total_s, t_e2e], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s, t_e2e = float(t[0]), float(t[1])
    pairs = float(n) * float(n)
    return (ws * steps * pairs / total_s / 1e9, ws * e2e_steps * pairs / t_e2e / 1e9, total_s, t_e2e)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import astronbodysim as nb

    n = args.n
    data = nb.plummer(n, seed=2)
    targets = args.ref_targets
    for _ in range(args.warmup):
        cpu_oracle_rate(data, targets, law=args.law)
    total_pairs, total_t, cores = 0.0, 0.0, 1
    for k in range(args.steps):
        rate, dt, cores = cpu_oracle_rate(data, targets, seed=100 + k, law=args.law)
        total_pairs += rate * dt
        total_t += dt
    v = total_pairs / total_t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Plummer sphere)",
        # the native arm's workload, each step a bounded sample of it: the
        # reference's CPU direct sum (FP64) of seeded targets against all N
        # sources, i.e. the N^2 force that dominates a KDK step
        "config": {"workload": "plummer_n%d_eps1e-3_%s_mixed_kdk_dt1e-4" % (n, args.law), "n": n,
                   "law": args.law,
                   "sample": "%d seeded targets x %d sources per step, FP64 force only (the O(N) "
                             "kick and drift of a step are not timed)" % (targets, n)},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d targets x %d sources per step, OpenMP static blocks" % (targets, n)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import torch

    import astronbodysim as nb

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n = args.n
    data = nb.plummer(n, seed=2 + rank)
    sim = nb.Simulation(data, ForceSofteningTable=[EPS] * 6, TimeStep=DT, TimeEnd=1.0,
                        precision="mixed", law=args.law, device=local, block=args.block,
                        i_per_thread=args.ipt, j_split=args.jsplit, tile_j=args.tile, stages=args.stages,
                        tuning=None if (args.block or args.ipt or args.jsplit) else "auto",
                        resort_every=1)
    tuned = sim.tuned_shape
    stream = torch.cuda.Stream(device=dev)
    sim.set_stream(stream.cuda_stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    # ---- force accuracy vs the oracle on a seeded subsample (rank 0) -------
    acc_stats = {}
    if rank == 0 and not args.skip_accuracy:
        from oracle import oracle

        rng = np.random.default_rng(1234)
        sub = np.sort(rng.choice(n, size=args.acc_targets, replace=False))
        nb.compute_force(sim, want_potential=True)
        g = nb.get_all_data(sim)
        a_ref, p_ref = oracle.force(data["pos"], data["mass"], data["pos"][sub], EPS,
                                    law=oracle.LAW_SPLINE_G2 if args.law == "spline" else oracle.LAW_PLUMMER)
        e = np.linalg.norm(g["acc"][sub] - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
        ep = np.abs(g["pot"][sub] - p_ref) / np.abs(p_ref)
        acc_stats["mixed"] = {"force_rel_median": float(np.median(e)),
                              "force_rel_p99": float(np.quantile(e, 0.99)),
                              "force_rel_max": float(e.max()),
                              "pot_rel_median": float(np.median(ep)),
                              "pot_rel_p99": float(np.quantile(ep, 0.99))}
        # plain FP64 form on the same targets (probe points at the particles)
        sim64 = nb.Simulation(data, ForceSofteningTable=[EPS] * 6, TimeStep=DT, TimeEnd=1.0,
                              precision="fp64", law=args.law, device=local)
        a64, p64 = nb.force_and_potential_at_points(sim64, data["pos"][sub], EPS)
        e64 = np.linalg.norm(a64 - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
        ep64 = np.abs(p64 - p_ref) / np.abs(p_ref)
        acc_stats["fp64"] = {"force_rel_max": float(e64.max()), "pot_rel_max": float(ep64.max())}
        sim64.close()
        acc_stats["targets"] = int(len(sub))

    # ---- resident run: warm-up, then K timed steps ------------------------
    nb.run  # noqa: B018  (API reference for readers)
    d0 = nb.diagnostics(sim) if rank == 0 and not args.skip_accuracy else None
    sim._ck(sim._lib.nb_run_begin(sim.handle))
    for _ in range(args.warmup):
        nb.step(sim, 1)
    torch.cuda.synchronize(dev)
    if ws > 1:
        torch.distributed.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    ev = []
    torch.cuda.synchronize(dev)
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)  # L2 flush (256 MiB write), outside the events
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        nb.step(sim, 1)
        with torch.cuda.stream(stream):
            e1.record(stream)
        ev.append((e0, e1))
    torch.cuda.synchronize(dev)
    if ws > 1:
        torch.distributed.barrier()
    t_wall = time.perf_counter() - t_wall0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)

    # ---- force kernel alone (roofline), same stream ------------------------
    fev = []
    for _ in range(args.force_reps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        nb.compute_force(sim)
        with torch.cuda.stream(stream):
            e1.record(stream)
        fev.append((e0, e1))
    torch.cuda.synchronize(dev)
    clocks = sampler.stop()
    force_ms = statistics.mean(a.elapsed_time(b) for a, b in fev)

    # ---- energy drift of the run: synchronised state (virtual back half kick)
    if d0 is not None:
        nb.leapfrog_half_kick(sim, -1)
        d1 = nb.diagnostics(sim)
        e0, e1 = d0["K"] + d0["W"], d1["K"] + d1["W"]
        acc_stats["energy_drift_mixed_n%d" % n] = {
            "steps": args.warmup + args.steps, "dt": DT, "energy_rel_drift": (e1 - e0) / abs(e0),
            "momentum_abs_drift": float(np.linalg.norm(d1["P"] - d0["P"]))}
        acc_stats["energy_drift_mixed_vs_fp64_n32768"] = energy_drift_pair(nb, args.law, local)

    # ---- general masses and the plain FP64 form (throughput legs) ----------
    extra = {}
    if rank == 0 and not args.skip_accuracy:
        extra["general_mass"] = general_mass_leg(nb, data, args, local, stream, flush)
        extra["fp64_plain"] = fp64_leg(nb, data, args, local, stream, args.fp64_targets)
        extra["fp64_plain"]["mixed_over_fp64"] = (n * n / (force_ms / 1e3) / 1e9) / extra["fp64_plain"]["value"]

    # ---- end to end through the public API with host buffers ---------------
    pin = {k: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
           for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "m")}
    ptype = torch.ones(n, dtype=torch.int32, pin_memory=True).numpy()
    st = nb.get_all_data(sim)
    for k, col in (("x", st["pos"][:, 0]), ("y", st["pos"][:, 1]), ("z", st["pos"][:, 2]),
                   ("vx", st["vel"][:, 0]), ("vy", st["vel"][:, 1]), ("vz", st["vel"][:, 2]),
                   ("ax", st["acc"][:, 0]), ("ay", st["acc"][:, 1]), ("az", st["acc"][:, 2])):
        pin[k][:] = col
    pin["m"][:] = data["mass"]
    from astronbodysim import _lib as L

    lib = sim._lib
    h2d = 7 * 8 * n + 4 * n + 3 * 8 * n
    d2h = 9 * 8 * n
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        sim._ck(lib.nb_upload(sim.handle, n, *[L.dptr(pin[k]) for k in ("x", "y", "z", "vx", "vy", "vz", "m")],
                              L.i32ptr(ptype)))
        sim._ck(lib.nb_upload_acc(sim.handle, L.dptr(pin["ax"]), L.dptr(pin["ay"]), L.dptr(pin["az"])))
        nb.step(sim, 1)
        sim._ck(lib.nb_download(sim.handle, *[L.dptr(pin[k]) for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")],
                                None, None, None))
    t_e2e = time.perf_counter() - t0

    sim.close()

    # ---- batched ensemble (many independent systems, one engine) -----------
    batch = None if args.skip_batch else run_ensemble(nb, args, rank, local)

    # ---- serving sample (Poisson arrivals, continuous batching) ------------
    serve_stats = None
    if args.serve_seconds > 0:
        serve_stats = {}
        # the stated stream (overloaded on one GPU) and a sustainable load
        # (offered ~0.65 of what one GB300 serves), drained to the last request
        for name, rate, seconds, drain in (
                ("lambda_%g" % args.serve_rate, args.serve_rate, args.serve_seconds, False),
                ("lambda_%g_drained" % args.serve_sustainable_rate, args.serve_sustainable_rate,
                 args.serve_sustainable_seconds, True)):
            if seconds <= 0:
                continue
            stream = nb.RequestStream(rate=rate, seed=7 + rank)
            eng = nb.Engine(max_particles=args.serve_particles, max_systems=512,
                            max_steps_per_call=args.serve_chunk, device=local, law=args.law)
            st = nb.serve(eng, stream, seconds, chunk_steps=args.serve_chunk, drain_after=drain)
            eng.close()
            st.update(rate=rate, arena_particles=args.serve_particles, chunk_steps=args.serve_chunk)
            serve_stats[name] = st

    # ---- aggregate over ranks (replicas) -----------------------------------
    value, e2e_value, total_s, t_e2e = replica_rates(ws, args.steps, args.e2e_steps, n,
                                                     total_ms / 1e3, t_e2e, dev)
    pairs = float(n) * float(n)
    if batch is not None:
        batch["vs_single_system"] = batch["value"] / (value / ws)

    if rank == 0:
        peaks = measured_peaks()
        props = torch.cuda.get_device_properties(dev)
        sm_max = peaks.get("sm_max_mhz") or clocks.get("sm_max_mhz") or 2070.0
        nominal_tflops = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12
        fp32_measured = measured_fp32_peak(local)
        fp32_peak_tflops = fp32_measured or nominal_tflops
        achieved = FLOP_PER_INTERACTION * pairs / (force_ms / 1e3) / 1e12
        # the launch shape the handle used (built-in rule when no table entry)
        tuned_eff = tuned if tuned[:2] != (0, 0) else (128, 2 if n >= (1 << 16) else 1, 4, 0, 0)
        tuned_eff = tuple(tuned_eff[:3]) + (tuned_eff[3] or 256, tuned_eff[4] or 4)
        traffic = None
        tpath = os.path.join(REPO, "profiles", "force_mixed_traffic.json")
        if os.path.exists(tpath):
            try:
                with open(tpath) as f:
                    tj = json.load(f)
                if tj.get("shape") == "%dx%dx%dx%dx%d" % tuned_eff:
                    traffic = tj.get("bytes_per_launch_scaled_to_n%d" % n)
            except Exception:
                traffic = None
        cpu = None
        if not args.skip_cpu_baseline:
            rate, dt, cores = cpu_oracle_rate(data, args.cpu_targets, law=args.law)
            cpu = {"value": rate / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": "%d seeded targets x %d sources (%.1f s), OpenMP static blocks, FP64"
                             % (args.cpu_targets, n, dt)}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Plummer sphere, G=M=a=1)",
            "config": {"workload": "plummer_n%d_eps1e-3_%s_mixed_kdk_dt1e-4" % (n, args.law),
                       "n": n, "law": args.law, "precision": "mixed (fp32 pairs, fp64 origins/state)",
                       "step": "drift+Morton sort+pack+force(N^2)+kick, one CUDA graph replay "
                               "(sort every step: resort_every=1)",
                       "l2": "256 MiB write between timed steps, outside the events",
                       "parallelism": "replicas" if ws > 1 else "single GPU",
                       "force_kernel": ("block=%d i_per_thread=%d j_split=%d tile=%d stages=%d (%s)" % (
                           tuned_eff + ("explicit" if (args.block or args.ipt or args.jsplit) else
                                        ("autotuner table" if tuned[:2] != (0, 0) else
                                         "built-in rule of the library"),)))},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak_tflops,
                         "unit": "TFLOP/s", "frac": achieved / fp32_peak_tflops, "traffic": traffic,
                         "kernel": "k_force_mixed (+k_pack, k_force_join)", "force_ms": force_ms,
                         "peak_note": ("of measured: fma.rn.f32x2 throughput of this GPU (nb_selftest_fp32_peak); "
                                       "nominal SMs x 128 lanes x 2 x %.0f MHz = %.1f TFLOP/s; 20 flop/interaction"
                                       % (sm_max, nominal_tflops)) if fp32_measured else
                                      "of nominal: SMs x 128 lanes x 2 x sm_max_mhz; 20 flop/interaction",
                         "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of "
                                         "this launch shape at N = 2^18, scaled by N (profiles/force_mixed_traffic.json); "
                                         "null when the file names another shape"},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": args.e2e_steps},
            "gpu_launches": (STEP_KERNELS + (1 if tuned_eff[2] > 1 or tuned_eff[0] == -1 else 0)) * args.steps,
            "clocks": clocks,
            "accuracy": acc_stats,
            "general_mass": extra.get("general_mass"),
            "fp64_plain": extra.get("fp64_plain"),
            "batch": batch,
            "serve": serve_stats,
            "wall_s_timed": t_wall,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_ensemble(nb, args, rank=0, local=0):
    """Batched ensemble: args.batch_systems systems through one engine for
    args.batch_steps KDK steps; aggregate interactions/s over the engine's
    CUDA-event time."""
    ens = nb.ensemble_systems(args.batch_systems, seed=11 + rank)
    # optional large systems among the small ones (the tail of whole-i-block
    # work items: a large system's i-block sweeps all of its j-tiles)
    for k in range(args.batch_big):
        ens.append((nb.plummer(args.batch_big_n, seed=500 + k), 1e-3))
    tot = sum(d["pos"].shape[0] for d, _ in ens)
    nsys = len(ens)
    eng = nb.Engine(max_particles=tot + 4096, max_systems=nsys,
                    max_steps_per_call=args.batch_steps, device=local, law=args.law, tuning="auto")
    for d, eps in ens:
        eng.submit(d, eps, 1e-3, args.batch_steps)
    del ens
    t0 = time.perf_counter()
    eng.run_until_idle()
    t_batch_wall = time.perf_counter() - t0
    st = eng.stats()
    eng.close()
    return {"value": st["interactions"] / (st["gpu_ms"] / 1e3) / 1e9, "unit": UNIT,
            "systems": nsys, "large_systems": [args.batch_big, args.batch_big_n],
            "particles": tot, "steps": args.batch_steps,
            "interactions": st["interactions"], "gpu_s": st["gpu_ms"] / 1e3,
            "wall_s_incl_admission_and_retirement": t_batch_wall,
            "force_shape": "%dx%d (block x targets/thread)" % eng.shape,
            "workload": "N log-uniform [64, 8192], half Plummer / half Hernquist (a=1, r<100a), "
                        "m=1/N, eps U[1e-3, 1e-2], mixed, %d KDK steps dt=1e-3, one CUDA graph "
                        "per step" % args.batch_steps}


def energy_drift_pair(nb, law, device, n=32768, steps=10):
    """Energy / momentum drift of `steps` KDK steps at dt 1e-4 of a Plummer
    sphere (eps 1e-3), mixed and plain FP64 on the GPU from the same state."""
    data = nb.plummer(n, seed=99)
    out = {"n": n, "steps": steps, "dt": DT}
    for prec in ("mixed", "fp64"):
        sim = nb.Simulation(data, ForceSofteningTable=[EPS] * 6, TimeStep=DT, TimeEnd=1.0,
                            precision=prec, law=law, device=device)
        d0 = nb.diagnostics(sim)
        nb.run(sim, nsteps=steps)
        d1 = nb.diagnostics(sim)
        e0, e1 = d0["K"] + d0["W"], d1["K"] + d1["W"]
        out[prec] = {"energy_rel_drift": (e1 - e0) / abs(e0),
                     "momentum_abs_drift": float(np.linalg.norm(d1["P"] - d0["P"]))}
        if prec == "mixed":
            pos_m = nb.get_all_data(sim)["pos"]
        else:
            out["final_pos_max_abs_diff"] = float(np.abs(nb.get_all_data(sim)["pos"] - pos_m).max())
        sim.close()
    return out


def run_plummer4096(args):
    """The oracle-sized case: Plummer N = 4096 (G = M = a = 1), eps = 0.01, both
    laws; force + potential against the oracle, then 100 KDK steps at dt = 1e-3
    (energy drift), on the GPU (mixed and plain FP64) and in the oracle."""
    import torch

    import astronbodysim as nb
    from oracle import oracle

    n, h, dt, nsteps = 4096, 0.01, 1e-3, 100
    d = nb.plummer(n, seed=1)
    out = {"mode": "plummer4096", "n": n, "eps": h, "dt": dt, "steps": nsteps, "unit": UNIT}
    for law in ("spline", "plummer"):
        olaw = oracle.LAW_SPLINE_G2 if law == "spline" else oracle.LAW_PLUMMER
        a_ref, p_ref = oracle.force(d["pos"], d["mass"], d["pos"], h, law=olaw)
        o = oracle.OracleSim(d["pos"], d["vel"], d["mass"], soft=[h] * 6, dt=dt, time_end=1.0, law=olaw)
        o.compute_potential()
        od0 = o.diagnostics()
        t0 = time.perf_counter()
        o.run_begin()
        o.step(nsteps)
        o.run_end()
        t_or = time.perf_counter() - t0
        o.compute_potential()
        od1 = o.diagnostics()
        e0, e1 = od0["K"] + od0["W"], od1["K"] + od1["W"]
        res = {"oracle": {"energy_rel_drift": (e1 - e0) / abs(e0), "wall_s_100_steps": t_or,
                          "g_interactions_per_s": (nsteps + 1) * n * n / t_or / 1e9,
                          "cores": oracle.max_threads()}}
        for prec in ("mixed", "fp64"):
            sim = nb.Simulation(d, ForceSofteningTable=[h] * 6, TimeStep=dt, TimeEnd=1.0,
                                precision=prec, law=law)
            nb.compute_force(sim, want_potential=True)
            g = nb.get_all_data(sim)
            ea = np.linalg.norm(g["acc"] - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
            ep = np.abs(g["pot"] - p_ref) / np.abs(p_ref)
            dg0 = nb.diagnostics(sim)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            nb.run(sim, nsteps=nsteps)
            torch.cuda.synchronize()
            t_gpu = time.perf_counter() - t0
            dg1 = nb.diagnostics(sim)
            eg0, eg1 = dg0["K"] + dg0["W"], dg1["K"] + dg1["W"]
            res[prec] = {"force_rel_median": float(np.median(ea)), "force_rel_p99": float(np.quantile(ea, 0.99)),
                         "force_rel_max": float(ea.max()), "pot_rel_median": float(np.median(ep)),
                         "energy_rel_drift": (eg1 - eg0) / abs(eg0), "wall_s_100_steps": t_gpu,
                         "pos_max_abs_diff_vs_oracle": float(np.abs(nb.get_all_data(sim)["pos"] - o.pos).max())}
            sim.close()
        out[law] = res
    print(json.dumps(out), flush=True)
    return 0


def run_collision(args):
    """Two Hernquist spheres on a parabolic approach, adaptive power-of-two bins
    with dt_i = eta sqrt(eps / |a_i|) (eta 0.025, dt_max 1e-2), eps 5e-3.
    Throughput of the mixed adaptive run over `--base-steps` base steps of
    dt_max; with --fp64-compare also an FP64 GPU run of the same initial
    conditions (energy / momentum drift of both)."""
    import torch

    import astronbodysim as nb

    n_each = args.n_each
    data = nb.collision(n_each, seed=5, separation=20.0)
    T = args.base_steps * 1e-2
    out = {"mode": "collision", "n": 2 * n_each, "base_steps": args.base_steps, "eps": 5e-3,
           "criterion": "eta_sqrt_eps", "eta": 0.025, "dt_max": 1e-2, "unit": UNIT}
    for prec in (["mixed", "fp64"] if args.fp64_compare else ["mixed"]):
        sim = nb.Simulation(data, ForceSofteningTable=[5e-3] * 6, TimeEnd=T, MaxStep=1e-2,
                            ErrTolTimestep=0.025, criterion="eta_sqrt_eps", precision=prec,
                            tuning="auto" if prec == "mixed" else None)
        d0 = nb.diagnostics(sim)
        nb.compute_force(sim)
        nb.init_timesteps(sim)
        nb.leapfrog_half_kick(sim, +1)
        torch.cuda.synchronize()
        sampler = ClockSampler(0)
        sampler.start()
        t0 = time.perf_counter()
        while True:
            nb.step(sim, 1)
            _, tf = sim.time()
            if tf >= T:
                break
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clocks = sampler.stop()
        substeps, pairs = nb.counters(sim)
        nb.leapfrog_half_kick(sim, -1)
        d1 = nb.diagnostics(sim)
        e0, e1 = d0["K"] + d0["W"], d1["K"] + d1["W"]
        out[prec] = {"substeps": substeps, "wall_s": wall, "interactions": pairs,
                     "g_interactions_per_s": pairs / wall / 1e9,
                     "energy_rel_drift": (e1 - e0) / abs(e0),
                     "momentum_abs_drift": float(np.linalg.norm(d1["P"] - d0["P"])),
                     "angular_momentum_abs_drift": float(np.linalg.norm(d1["L"] - d0["L"])),
                     "clocks": clocks}
        sim.close()
    print(json.dumps(out), flush=True)
    return 0


def run_fp64(args):
    """The plain FP64 form alone: acceleration at --fp64-targets seeded
    particles of the Plummer sphere of --n from all its particles (one
    k_force_fp64 launch, CUDA events) -- one JSON line."""
    import torch

    import astronbodysim as nb

    data = nb.plummer(args.n, seed=2)
    stream = torch.cuda.Stream()
    out = fp64_leg(nb, data, args, 0, stream, args.fp64_targets)
    out.update(mode="fp64", n=args.n, law=args.law)
    print(json.dumps(out), flush=True)
    return 0


def run_serve(args):
    """Serving run alone (Poisson stream, continuous batching) -- one JSON line."""
    import astronbodysim as nb

    out = {"mode": "serve", "rate": args.serve_rate, "arena_particles": args.serve_particles,
           "chunk_steps": args.serve_chunk, "unit": UNIT, "seconds": args.serve_seconds,
           "drain_after": args.serve_drain}
    policies = ["fifo", "sjf"] if args.serve_policy == "both" else [args.serve_policy]
    for pol in policies:
        sampler = ClockSampler(0)
        sampler.start()
        stream = nb.RequestStream(rate=args.serve_rate, seed=7)  # the same arrivals for each policy
        eng = nb.Engine(max_particles=args.serve_particles, max_systems=512,
                        max_steps_per_call=args.serve_chunk, law=args.law)
        st = nb.serve(eng, stream, args.serve_seconds, chunk_steps=args.serve_chunk,
                      policy=pol, max_engine_queue=args.serve_queue, drain_after=args.serve_drain,
                      log=lambda k, t: print("completed %d at %.1f s" % (k, t), file=sys.stderr)
                      if k and k % 100 == 0 else None)
        eng.close()
        st["clocks"] = sampler.stop()
        out[pol] = st
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--law", default="spline", choices=["spline", "plummer"])
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--ipt", type=int, default=0)
    ap.add_argument("--jsplit", type=int, default=0)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--stages", type=int, default=0)
    ap.add_argument("--force-reps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--fp64-targets", type=int, default=152 * 128 * 4)
    ap.add_argument("--acc-targets", type=int, default=4096)
    ap.add_argument("--cpu-targets", type=int, default=2048)
    ap.add_argument("--ref-targets", type=int, default=1024)
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--skip-cpu-baseline", action="store_true")
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--batch-systems", type=int, default=4096)
    ap.add_argument("--batch-big", type=int, default=0, help="extra Plummer systems of --batch-big-n particles")
    ap.add_argument("--batch-big-n", type=int, default=65536)
    ap.add_argument("--batch-steps", type=int, default=1000)
    ap.add_argument("--serve-seconds", type=float, default=20.0)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-chunk", type=int, default=16)
    ap.add_argument("--serve-particles", type=int, default=1 << 22)
    ap.add_argument("--serve-policy", default="fifo", choices=["fifo", "sjf", "both"])
    ap.add_argument("--serve-drain", action="store_true")
    ap.add_argument("--serve-sustainable-rate", type=float, default=2.0)
    ap.add_argument("--serve-sustainable-seconds", type=float, default=30.0)
    ap.add_argument("--serve-queue", type=int, default=32)
    ap.add_argument("--mode", default="bench", choices=["bench", "serve", "collision", "tune", "ensemble", "fp64",
                                                         "plummer4096"])
    ap.add_argument("--n-each", type=int, default=1 << 20)
    ap.add_argument("--base-steps", type=int, default=2)
    ap.add_argument("--fp64-compare", action="store_true")
    ap.add_argument("--dry-run", action="store_true",
                    help="check the replica launcher and max-over-ranks aggregation on the host (no GPU)")
    args = ap.parse_args()
    world = os.environ.get("WORLD_SIZE")
    if args.gpus > 1 and world is None:
        return relaunch_replicas(args.gpus)
    if world is not None and int(world) != args.gpus:
        print("bench.py: --gpus %d but WORLD_SIZE=%s" % (args.gpus, world), file=sys.stderr)
        return 2
    if args.dry_run:
        return run_dry(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "serve":
        return run_serve(args)
    if args.mode == "fp64":
        return run_fp64(args)
    if args.mode == "collision":
        return run_collision(args)
    if args.mode == "plummer4096":
        return run_plummer4096(args)
    if args.mode == "ensemble":
        import astronbodysim as nb

        out = run_ensemble(nb, args)
        out["mode"] = "ensemble"
        print(json.dumps(out), flush=True)
        return 0
    if args.mode == "tune":
        from astronbodysim import autotune

        for law in ("spline", "plummer"):
            autotune.save(autotune.tune([1 << k for k in range(12, 21)], law=law, reps=3))
        autotune.save_batch(autotune.tune_batch(law="spline"))
        print(json.dumps(autotune.load()), flush=True)
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
