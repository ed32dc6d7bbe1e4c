"""The served loop's host logic without a GPU (serve.run_served with a fake
batch): every arrival is admitted once memory allows, given its requested
step count as a stop step, stepped in whole chunks, retired when its status
reads done, and counted once in the work and latency figures."""
import numpy as np

from platelet_fiber_gpu_gb300 import serve

DONE = 6


class FakeScene:
    def __init__(self, n):
        self.n_nodes = n


class FakeBatch:
    """Slots with a step counter and a stop step; admission against a budget
    in nodes; step(n) advances every live job and stops it at its stop."""
    log = []

    def __init__(self, budget):
        self.budget = budget
        self.jobs = {}
        self.next = 0
        FakeBatch.log.append(self)
        self.admitted = []
        self.retired = []
        self.steps_called = []

    def admit(self, sc, precision):
        if sum(j["n"] for j in self.jobs.values()) + sc.n_nodes > self.budget:
            return None
        s = self.next
        self.next += 1
        self.jobs[s] = dict(n=sc.n_nodes, step=0, stop=0)
        self.admitted.append(s)
        return s

    def set_stop(self, s, stop):
        self.jobs[s]["stop"] = stop

    def step(self, n):
        self.steps_called.append(n)
        for j in self.jobs.values():
            j["step"] = min(j["step"] + n, j["stop"]) if j["stop"] else j["step"] + n

    def status(self, s):
        j = self.jobs[s]
        return DONE if j["stop"] and j["step"] >= j["stop"] else 0

    def job(self, s):
        return self.jobs[s]

    def retire(self, s):
        j = self.jobs.pop(s)
        assert j["step"] == j["stop"]
        self.retired.append(s)

    def close(self):
        assert not self.jobs


def test_served_loop_accounts_every_job():
    scenes = [FakeScene(1000 * (i + 1)) for i in range(4)]
    r = serve.run_served(1, rate=400.0, duration=0.05, seed=9, budget=6000, chunk=25, steps_range=(30, 120),
                         batch_factory=FakeBatch, scenes=scenes)
    b = FakeBatch.log[-1]
    assert r["jobs"] >= 5
    assert len(b.admitted) == len(b.retired) == r["jobs"]
    assert set(b.steps_called) == {25}                      # whole chunks only
    assert 0 <= r["latency_p50_s"] <= r["latency_p99_s"]
    assert r["mlups"] > 0 and r["step_calls"] == len(b.steps_called)
    # the budget was respected and some arrivals waited for memory
    assert r["mean_live_jobs"] >= 1


def test_requested_steps_set_the_work():
    """Work counted = sum over jobs of nodes x requested steps (rng replayed)."""
    scenes = [FakeScene(500)]
    r = serve.run_served(1, rate=200.0, duration=0.03, seed=3, budget=10 ** 9, chunk=10, steps_range=(5, 40),
                         batch_factory=FakeBatch, scenes=scenes)
    rng = np.random.default_rng(3)
    t, req = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / 200.0))
        if t > 0.03:
            break
        rng.integers(1)
        req.append(int(rng.integers(5, 41)))
    assert r["jobs"] == len(req)
    assert r["node_steps"] == 500 * sum(req)


def test_on_finish_sees_each_job_once_at_its_requested_step():
    """The served loop hands every finished job to on_finish, with its scene
    index and requested step count, before retiring it."""
    scenes = [FakeScene(300), FakeScene(700)]
    seen = []
    r = serve.run_served(1, rate=300.0, duration=0.05, seed=5, budget=10 ** 9, chunk=10, steps_range=(5, 40),
                         batch_factory=FakeBatch, scenes=scenes,
                         on_finish=lambda idx, req, job: seen.append((idx, req, job["step"], job["n"])))
    assert len(seen) == r["jobs"] >= 3
    for idx, req, step, n in seen:
        assert step == req and n == scenes[idx].n_nodes
