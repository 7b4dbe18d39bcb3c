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
    assert st["latency_p50_s"] <= st["latency_p99_s"]
    assert st["policy"] == policy
    assert st["served_interactions"] == pytest.approx(st["completed_interactions"])


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
