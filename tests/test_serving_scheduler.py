"""The serving scheduler's host logic, on the CPU with a stand-in batch: every request completes
with exactly its step count, admissions respect the memory budget the batches report, groups are
created while others are in flight and compacted when mostly finished, failed systems are stopped
without touching the others, and the loop ends (bounded by a timeout)."""
import numpy as np
import pytest

from openmm_rigidbody_plugin_gb300 import serving


class FakeSystem:
    def __init__(self, n):
        self.num_atoms = n
        self.num_bodies = n // 3


BYTES_PER_ATOM = 1000  # what a stand-in batch reports holding


class FakeBatch:
    """Each system's state is a step counter; checkpoint/restore carry it over. A system whose
    atom count is 13 fails at its 7th step."""

    live_bytes = 0  # bytes held by all stand-in batches alive

    def __init__(self, systems, **kw):
        self.systems = systems
        self.memory_bytes = BYTES_PER_ATOM * sum(s.num_atoms for s in systems)
        FakeBatch.live_bytes += self.memory_bytes
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

    def __del__(self):
        FakeBatch.live_bytes -= self.memory_bytes

    def step(self, k, dt, stream=None):
        self.counter += k
        self.last_launch_count = 2 * k

    def status(self):
        return np.array([5 if s.num_atoms == 13 and c >= 7 else 0 for s, c in zip(self.systems, self.counter)],
                        dtype=np.int32)

    def get_system_state(self, s):
        n = self.offsets[s + 1] - self.offsets[s]
        x = np.full((n, 3), float(self.counter[s]))
        return x, x

    def energies(self):
        return np.stack([self.counter] * 3, axis=1).astype(float)


class FakeEvent:
    """A stand-in stream event: the stand-in batches finish their chunks at once."""

    def record(self, stream):
        pass

    def synchronize(self):
        pass

    def query(self):
        return True


def _server(**kw):
    kw.setdefault("batch_factory", FakeBatch)
    return serving.Server(sync=lambda: None, free_memory=lambda: 1e15, stream_factory=lambda: None, reserve_bytes=0,
                          event_factory=FakeEvent, **kw)


def _requests(rng, n):
    return [serving.Request(i, FakeSystem(int(rng.integers(30, 600))), int(rng.integers(5, 300)), arrival=0.0)
            for i in range(n)]


@pytest.mark.timeout(60)
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_every_request_completes_with_its_steps(seed):
    rng = np.random.default_rng(seed)
    reqs = _requests(rng, 25)
    budget = BYTES_PER_ATOM * 1500
    peak = []

    class Tracked(FakeBatch):
        def step(self, k, dt, stream=None):
            peak.append(FakeBatch.live_bytes)
            super().step(k, dt, stream)

    server = _server(budget_bytes=budget, chunk_steps=40, batch_factory=Tracked)
    done = server.run(reqs, realtime=False)
    assert sorted(r.rid for r in done) == list(range(25))
    for r in done:
        assert r.done_steps == r.steps == sum(r.chunks)
        assert r.result["energies"][0] == r.steps  # the state followed the request across compactions
    assert server.groups_created > 3
    assert max(peak) <= budget and server.peak_bytes <= budget


@pytest.mark.timeout(60)
def test_budget_too_small_for_a_request_is_an_error():
    server = _server(budget_bytes=BYTES_PER_ATOM * 100)
    with pytest.raises(ValueError):
        server.run([serving.Request(0, FakeSystem(300), 10, 0.0)], realtime=False)


@pytest.mark.timeout(60)
def test_realtime_arrivals_are_admitted_as_they_come():
    reqs = [serving.Request(i, FakeSystem(60), 50, arrival=0.02 * i) for i in range(6)]
    server = _server(chunk_steps=10, min_interval=0.0)
    done = server.run(reqs, realtime=True)
    assert len(done) == 6
    for r in done:
        assert r.admitted >= r.arrival and r.completed >= r.admitted


@pytest.mark.timeout(60)
def test_failed_request_is_stopped_and_the_others_complete():
    reqs = [serving.Request(i, FakeSystem(n), 30, arrival=0.0) for i, n in enumerate([60, 13, 90, 45])]
    done = _server(chunk_steps=5).run(reqs, realtime=False)
    by = {r.rid: r for r in done}
    assert by[1].failed and by[1].result is None and by[1].done_steps == 10  # stopped at the chunk's end
    for i in (0, 2, 3):
        assert by[i].failed is None and by[i].result["energies"][0] == 30


@pytest.mark.timeout(60)
def test_mostly_finished_group_is_compacted_exactly():
    reqs = [serving.Request(0, FakeSystem(900), 10, 0.0), serving.Request(1, FakeSystem(100), 200, 0.0)]
    server = _server(chunk_steps=10)
    done = server.run(reqs, realtime=False)
    assert server.compactions >= 1
    assert {r.rid: r.result["energies"][0] for r in done} == {0: 10, 1: 200}


@pytest.mark.timeout(60)
@pytest.mark.parametrize("seed", [3, 4])
def test_groups_advance_independently(seed):
    """Chunks finish in any order (a stand-in event completes at random unless waited on): each
    group launches its next chunk as soon as its own finishes, every request still completes with
    exactly its steps, and groups run several chunks while another's is in flight."""
    rng = np.random.default_rng(seed)
    launched = []

    class RandomEvent(FakeEvent):
        def __init__(self):
            self.done = False

        def synchronize(self):
            self.done = True

        def query(self):
            self.done = self.done or bool(rng.random() < 0.3)
            return self.done

    class Logged(FakeBatch):
        def step(self, k, dt, stream=None):
            launched.append(id(self))
            super().step(k, dt, stream)

    reqs = _requests(rng, 20)
    server = serving.Server(sync=lambda: None, free_memory=lambda: 1e15, stream_factory=lambda: None, reserve_bytes=0,
                            event_factory=RandomEvent, batch_factory=Logged, budget_bytes=BYTES_PER_ATOM * 2000,
                            chunk_steps=20)
    done = server.run(reqs, realtime=False)
    assert sorted(r.rid for r in done) == list(range(20))
    for r in done:
        assert r.done_steps == r.steps == sum(r.chunks)
        assert r.result["energies"][0] == r.steps
    # some group launched two chunks in a row while others were in flight
    assert any(a == b for a, b in zip(launched, launched[1:]))
