"""Serving: simulation requests of different sizes admitted into one running batch.

Requests arrive over time (a seeded Poisson stream in the benchmark). The server admits them in
arrival order while the device-memory budget allows, keeps every admitted system's state resident
in one ``BatchedSystems`` and advances all of them together, chunk by chunk: a request that arrives
while others are on the GPU joins the batch at the next chunk boundary, and a finished request
leaves it. When the membership changes the batch is rebuilt and every continuing system's state is
carried over exactly (``checkpoint``/``restore``), so a request's trajectory does not depend on
its company: run alone with the same chunk boundaries it is bit for bit the same.

Each completed request records its arrival, admission and completion times (seconds from the
start), its final positions, velocities and [U, KE_t, KE_r], and the chunk lengths it was stepped
with.
"""
import time
from dataclasses import dataclass, field

import numpy as np

from . import batch as _batch

BYTES_PER_ATOM = 256  # planning estimate of device memory per atom (buffers, cells, body state)


@dataclass
class Request:
    rid: int
    system: object      # workloads.System (positions, velocities, masses, body indices, species, box)
    steps: int
    arrival: float      # seconds from the start of the stream
    admitted: float = None
    completed: float = None
    done_steps: int = 0
    chunks: list = field(default_factory=list)
    result: dict = None

    @property
    def num_atoms(self):
        return self.system.num_atoms

    @property
    def latency(self):
        return None if self.completed is None else self.completed - self.arrival


class Server:
    """Continuous batching of simulation requests on one device.

    Requests are admitted in arrival order while the memory budget allows. The running batch is
    rebuilt (continuing systems carried over exactly) when admitted requests are waiting and at
    least `min_interval` seconds have passed since the last rebuild, when finished systems hold
    more than `dead_fraction` of the batch's atoms, or when nothing in it is still running. A
    finished request's result is taken at its own last step; until the next rebuild its system
    stays in the batch and is stepped along with the others.
    """

    def __init__(self, budget_bytes=150e9, chunk_steps=100, dt=0.002, precision="mixed", rotation_mode=0,
                 graph_steps=25, device=0, min_interval=0.5, dead_fraction=0.5, batch_factory=None, sync=None):
        self.budget = float(budget_bytes)
        self.chunk = int(chunk_steps)
        self.dt = float(dt)
        self.precision = precision
        self.mode = rotation_mode
        self.graph_steps = graph_steps
        self.device = device
        self.min_interval = float(min_interval)
        self.dead_fraction = float(dead_fraction)
        self.rebuilds = 0
        self.launches = 0
        self.body_steps = 0
        self.seconds = {"rebuild": 0.0, "step": 0.0, "results": 0.0}
        # the batch type and the device synchronisation (replaceable to test the scheduling on CPU)
        self._factory = batch_factory or _batch.BatchedSystems.from_systems
        self._sync = sync

    def _memory(self, reqs):
        return sum(r.num_atoms for r in reqs) * BYTES_PER_ATOM

    def _rebuild(self, members, saved):
        b = self._factory([r.system for r in members], rotation_mode=self.mode, precision=self.precision,
                          device=self.device)
        if any(r.rid in saved for r in members):
            fresh = b.checkpoint()
            b.restore([saved.get(r.rid, fresh[k]) for k, r in enumerate(members)])
        if self.graph_steps:
            b.set_graph_steps(self.graph_steps)
        self.rebuilds += 1
        return b

    def run(self, requests, realtime=True):
        """Serve `requests` (arrival times in seconds from now); returns them, completed. With
        realtime=False every request counts as arrived at the start and rebuilds are not spaced."""
        if self._sync is None:
            import torch
            self._sync = torch.cuda.synchronize
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        members, waiting, done = [], [], []
        b = None
        last_rebuild = -1e30
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0 if realtime else 0.0
        while pending or waiting or any(r.completed is None for r in members):
            t = now()
            if members and all(r.completed is not None for r in members):
                members, b = [], None  # everything in the batch has finished: release it
            while pending and (pending[0].arrival <= t or not realtime):
                nxt = pending[0]
                if self._memory(members) + self._memory(waiting) + self._memory([nxt]) > self.budget:
                    if not members and not waiting:
                        raise ValueError(f"request {nxt.rid} ({nxt.num_atoms} atoms) exceeds the memory budget")
                    break
                pending.pop(0)
                nxt.admitted = t
                waiting.append(nxt)
            live = [r for r in members if r.completed is None]
            dead_atoms = sum(r.num_atoms for r in members if r.completed is not None)
            all_atoms = max(1, sum(r.num_atoms for r in members))
            if not live and not waiting:  # idle until the next arrival
                time.sleep(max(0.0, min(pending[0].arrival - t, 0.01)))
                continue
            if (not live or dead_atoms > self.dead_fraction * all_atoms or
                    (waiting and (not realtime or t - last_rebuild >= self.min_interval))):
                tr = time.perf_counter()
                saved = {}
                if b is not None and live:
                    states = b.checkpoint()
                    saved = {r.rid: states[k] for k, r in enumerate(members) if r.completed is None}
                members = live + waiting
                waiting = []
                b = self._rebuild(members, saved)
                last_rebuild = now()
                self.seconds["rebuild"] += time.perf_counter() - tr
                live = [r for r in members if r.completed is None]
            k = min(self.chunk, min(r.steps - r.done_steps for r in live))
            ts = time.perf_counter()
            b.step(k, self.dt)
            self._sync()
            self.seconds["step"] += time.perf_counter() - ts
            self.launches += b.last_launch_count
            self.body_steps += k * int(b.bodies_per_system.sum())
            for r in live:
                r.done_steps += k
                r.chunks.append(k)
            finished = [i for i, r in enumerate(members) if r.completed is None and r.done_steps == r.steps]
            if finished:
                tf = time.perf_counter()
                e = b.energies()
                t = now()
                for i in finished:
                    r = members[i]
                    x, v = b.get_system_state(i)
                    r.result = {"positions": x, "velocities": v, "energies": e[i].copy()}
                    r.completed = t
                    done.append(r)
                self.seconds["results"] += time.perf_counter() - tf
        return done


def serve_alone(request, precision="mixed", rotation_mode=0, dt=0.002):
    """The request run by itself with the chunk boundaries it had in the mix."""
    b = _batch.BatchedSystems.from_systems([request.system], rotation_mode=rotation_mode, precision=precision)
    for k in request.chunks:
        b.step(k, dt)
    x, v = b.get_state()
    return {"positions": x, "velocities": v, "energies": b.energies()[0]}


def poisson_stream(rate, duration, atoms_range, steps_range, seed=8):
    """Seeded Poisson arrivals of water-box requests with log-uniform sizes (atoms) and step counts."""
    from . import workloads as W
    rng = np.random.default_rng(seed)
    t, out, rid = 0.0, [], 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        atoms = float(np.exp(rng.uniform(np.log(atoms_range[0]), np.log(atoms_range[1]))))
        steps = int(np.exp(rng.uniform(np.log(steps_range[0]), np.log(steps_range[1]))))
        nw = max(8, int(round(atoms / 3)))
        out.append(Request(rid, W.water_box(nw, seed=seed * 1000003 + rid), steps, t))
        rid += 1
    return out
