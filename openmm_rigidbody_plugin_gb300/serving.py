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
    """Continuous batching of simulation requests on one device."""

    def __init__(self, budget_bytes=150e9, chunk_steps=100, dt=0.002, precision="mixed", rotation_mode=0,
                 graph_steps=25, device=0):
        self.budget = float(budget_bytes)
        self.chunk = int(chunk_steps)
        self.dt = float(dt)
        self.precision = precision
        self.mode = rotation_mode
        self.graph_steps = graph_steps
        self.device = device
        self.rebuilds = 0

    def _memory(self, reqs):
        return sum(r.num_atoms for r in reqs) * BYTES_PER_ATOM

    def _rebuild(self, active, saved):
        b = _batch.BatchedSystems.from_systems([r.system for r in active], rotation_mode=self.mode,
                                               precision=self.precision, device=self.device)
        if any(r.rid in saved for r in active):
            fresh = b.checkpoint()
            b.restore([saved.get(r.rid, fresh[k]) for k, r in enumerate(active)])
        if self.graph_steps:
            b.set_graph_steps(self.graph_steps)
        self.rebuilds += 1
        return b

    def run(self, requests, realtime=True):
        """Serve `requests` (arrival times in seconds from now); returns them, completed."""
        import torch
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        active, done = [], []
        b = None
        changed = False
        t0 = time.perf_counter()
        clock = (lambda: time.perf_counter() - t0) if realtime else None
        vt = 0.0  # virtual clock when not in real time: every request has arrived already
        while pending or active:
            now = clock() if realtime else vt
            while pending and (pending[0].arrival <= now or not realtime):
                nxt = pending[0]
                if self._memory(active) + self._memory([nxt]) > self.budget:
                    if not active:
                        raise ValueError(f"request {nxt.rid} ({nxt.num_atoms} atoms) exceeds the memory budget")
                    break
                pending.pop(0)
                nxt.admitted = now
                active.append(nxt)
                changed = True
            if not active:
                time.sleep(max(0.0, min(pending[0].arrival - now, 0.01)))
                continue
            if changed:
                saved = {}
                if b is not None:
                    states = b.checkpoint()
                    saved = {r.rid: states[k] for k, r in enumerate(members)}
                members = list(active)
                b = self._rebuild(members, saved)
                changed = False
            k = min(self.chunk, min(r.steps - r.done_steps for r in members))
            b.step(k, self.dt)
            torch.cuda.synchronize()
            for r in members:
                r.done_steps += k
                r.chunks.append(k)
            finished = [i for i, r in enumerate(members) if r.done_steps == r.steps]
            if finished:
                x, v = b.get_state()
                e = b.energies()
                now = clock() if realtime else vt
                for i in finished:
                    r = members[i]
                    a0, a1 = b.offsets[i], b.offsets[i + 1]
                    r.result = {"positions": x[a0:a1].copy(), "velocities": v[a0:a1].copy(), "energies": e[i].copy()}
                    r.completed = now
                    done.append(r)
                active = [r for r in active if r.done_steps < r.steps]
                changed = True
            elif any(r not in members for r in active):
                changed = True
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
