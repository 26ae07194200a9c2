"""The serving scheduler's host logic, on the CPU with a stand-in batch: every request completes
with exactly its step count, admissions respect the memory budget, membership changes while
systems are in flight, and the loop ends (bounded by a timeout)."""
import numpy as np
import pytest

from openmm_rigidbody_plugin_gb300 import serving


class FakeSystem:
    def __init__(self, n):
        self.num_atoms = n
        self.num_bodies = n // 3


class FakeBatch:
    """Each system's state is a step counter; checkpoint/restore carry it over."""

    def __init__(self, systems, **kw):
        self.systems = systems
        self.offsets = np.concatenate([[0], np.cumsum([s.num_atoms for s in systems])])
        self.bodies_per_system = np.array([s.num_bodies for s in systems])
        self.counter = np.zeros(len(systems), dtype=np.int64)
        self.last_launch_count = 0
        self.log = []

    def set_graph_steps(self, k):
        pass

    def checkpoint(self):
        return [(c,) for c in self.counter]

    def restore(self, states):
        self.counter = np.array([s[0] for s in states], dtype=np.int64)

    def step(self, k, dt):
        self.counter += k
        self.last_launch_count = 2 * k

    def get_system_state(self, s):
        n = self.offsets[s + 1] - self.offsets[s]
        x = np.full((n, 3), float(self.counter[s]))
        return x, x

    def energies(self):
        return np.stack([self.counter] * 3, axis=1).astype(float)


def _requests(rng, n):
    return [serving.Request(i, FakeSystem(int(rng.integers(30, 600))), int(rng.integers(5, 300)), arrival=0.0)
            for i in range(n)]


@pytest.mark.timeout(60)
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_every_request_completes_with_its_steps(seed):
    rng = np.random.default_rng(seed)
    reqs = _requests(rng, 25)
    budget = serving.BYTES_PER_ATOM * 1500
    server = serving.Server(budget_bytes=budget, chunk_steps=40, batch_factory=FakeBatch, sync=lambda: None)
    done = server.run(reqs, realtime=False)
    assert sorted(r.rid for r in done) == list(range(25))
    for r in done:
        assert r.done_steps == r.steps == sum(r.chunks)
        assert r.result["energies"][0] == r.steps  # the state followed the request across rebuilds
    assert server.rebuilds > 3


@pytest.mark.timeout(60)
def test_budget_too_small_for_a_request_is_an_error():
    server = serving.Server(budget_bytes=serving.BYTES_PER_ATOM * 100, batch_factory=FakeBatch, sync=lambda: None)
    with pytest.raises(ValueError):
        server.run([serving.Request(0, FakeSystem(300), 10, 0.0)], realtime=False)


@pytest.mark.timeout(60)
def test_realtime_arrivals_are_admitted_as_they_come():
    reqs = [serving.Request(i, FakeSystem(60), 50, arrival=0.02 * i) for i in range(6)]
    server = serving.Server(chunk_steps=10, batch_factory=FakeBatch, sync=lambda: None, min_interval=0.0)
    done = server.run(reqs, realtime=True)
    assert len(done) == 6
    for r in done:
        assert r.admitted >= r.arrival and r.completed >= r.admitted
