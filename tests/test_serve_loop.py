"""Host logic of the serving loop against a fake engine (no GPU): arrivals are
handed over in FIFO or shortest-job-first order, latencies and load are
accounted."""
import pytest

from astronbodysim.serve import RequestStream, serve


class FakeEngine:
    """Runs one request at a time; a request of work W finishes after
    ceil(W / 2e6) run() calls."""

    def __init__(self):
        self.queue, self.running, self.done, self.order = [], None, [], []
        self.interactions = 0.0
        self.next_id = 1

    def submit(self, data, eps, dt, nsteps):
        rid = self.next_id
        self.next_id += 1
        n = data["pos"].shape[0]
        self.queue.append([rid, float(n) ** 2 * nsteps])
        return rid

    def run(self, max_steps=16):
        if self.running is None and self.queue:
            self.running = self.queue.pop(0)
            self.order.append(self.running[0])
        if self.running is not None:
            step = min(self.running[1], 2e6)
            self.running[1] -= step
            self.interactions += step
            if self.running[1] <= 0:
                self.done.append(self.running[0])
                self.running = None
        return max_steps

    def drain_done(self):
        d, self.done = self.done, []
        return d

    def fetch(self, rid, n):
        return None

    def stats(self):
        return {"queued": len(self.queue), "running": int(self.running is not None),
                "interactions": self.interactions, "gpu_ms": self.interactions / 1e9}


@pytest.mark.parametrize("policy", ["fifo", "sjf"])
def test_serve_accounts_every_request(policy):
    stream = RequestStream(rate=400.0, seed=3, n_min=64, n_max=256, steps_min=10, steps_max=50,
                           pool_size=1)
    eng = FakeEngine()
    st = serve(eng, stream, 0.05, drain_after=True, policy=policy, max_engine_queue=1)
    assert st["completed"] == st["offered_requests"] > 0
    assert st["backlog_requests"] == 0
    lc, la = st["latency_completed"], st["latency_all_requests_lower_bound"]
    assert lc["p50_s"] <= lc["p99_s"]
    # drained: every offered request completed, nothing censored
    assert la["n"] == lc["n"] == st["offered_requests"] and la["censored"] == 0
    assert la["p99_s"] == lc["p99_s"]
    assert st["policy"] == policy and not st["overlap"]
    assert st["served_interactions"] == pytest.approx(st["completed_interactions"])


def test_overload_counts_unfinished_requests_as_censored():
    """Under overload the completed-only percentiles see only the lucky
    requests; the all-requests figures count every unfinished request with
    its age at the end (a lower bound of its latency)."""
    stream = RequestStream(rate=3000.0, seed=5, n_min=128, n_max=256, steps_min=40000, steps_max=50000,
                           pool_size=1)
    eng = FakeEngine()
    st = serve(eng, stream, 0.05, policy="fifo", max_engine_queue=4)
    la = st["latency_all_requests_lower_bound"]
    assert st["backlog_requests"] > 0 and la["censored"] == st["backlog_requests"]
    assert la["n"] == st["offered_requests"] == st["completed"] + la["censored"]
    if st["completed"]:
        assert la["p50_s"] >= 0.0


class FakeAsyncEngine(FakeEngine):
    """run_async launches a chunk that completes at the next run_async or
    sync call, as nb_engine_run_async does; records whether submits happened
    while a chunk was in flight."""

    def __init__(self):
        super().__init__()
        self.pending_chunk = False
        self.submits_in_flight = 0

    def submit(self, data, eps, dt, nsteps):
        if self.pending_chunk:
            self.submits_in_flight += 1
        return super().submit(data, eps, dt, nsteps)

    def run_async(self, max_steps=16):
        self.sync()
        if self.running is None and not self.queue:
            return 0
        self.pending_chunk = True
        return max_steps

    def sync(self):
        if self.pending_chunk:
            self.pending_chunk = False
            FakeEngine.run(self)


def test_overlapped_loop_submits_while_a_chunk_runs():
    stream = RequestStream(rate=2000.0, seed=6, n_min=64, n_max=128, steps_min=10, steps_max=20,
                           pool_size=1)
    eng = FakeAsyncEngine()
    st = serve(eng, stream, 0.05, drain_after=True, max_engine_queue=64)
    assert st["overlap"]
    assert st["completed"] == st["offered_requests"] > 0 and st["backlog_requests"] == 0
    assert eng.submits_in_flight > 0
    assert not eng.pending_chunk


def test_sjf_hands_over_the_smallest_waiting_request_first():
    stream = RequestStream(rate=1e6, seed=4, n_min=64, n_max=256, steps_min=10, steps_max=50,
                           pool_size=1)
    eng = FakeEngine()
    reqs = {}
    real_submit = eng.submit

    def submit(data, eps, dt, nsteps):
        rid = real_submit(data, eps, dt, nsteps)
        reqs[rid] = float(data["pos"].shape[0]) ** 2 * nsteps
        return rid

    eng.submit = submit
    # at 1e6 arrivals/s every request of the window arrives before the first hand-over
    serve(eng, stream, 1e-4, drain_after=True, policy="sjf", max_engine_queue=1)
    work = [reqs[r] for r in eng.order]
    assert len(work) > 3
    assert work[1:] == sorted(work[1:])


def test_unknown_policy():
    with pytest.raises(ValueError):
        serve(FakeEngine(), None, 1.0, policy="lifo")
