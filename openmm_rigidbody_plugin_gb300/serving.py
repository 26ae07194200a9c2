"""Serving: simulation requests of different sizes admitted into running batches on one device.

Requests arrive over time (a seeded Poisson stream in the benchmark). The server admits them in
arrival order while the device-memory budget allows, and keeps every admitted system's state
resident. Requests admitted together form a group: one ``BatchedSystems`` created from their
systems alone, so an arrival never rebuilds the systems already running. Every group advances
chunk by chunk on its own CUDA stream, so the groups' kernels overlap on the device; a finished
request leaves its result at its own last step. A group is freed when all its requests are done,
and compacted (its running systems carried over exactly into a new group, ``checkpoint`` /
``restore``) when finished or failed systems hold most of its atoms.

Admission counts device memory the library actually holds: every group's ``memory_bytes``
(rbx_batch_memory) is added to the memory in use once the group exists, and a waiting request is
charged at the largest bytes per atom measured so far (from a probe batch at start-up, then from
every group created). The budget is the smaller of the given one and the device's free memory at
start-up less a reserve.

A request's trajectory does not depend on its company: the forces a step call starts from are
formed from neighbour lists built at its starting positions (by the previous call, or after a move
between groups by the call itself), and every system is integrated independently, so run alone
with the same chunk lengths it is bit for bit the same (``serve_alone``).

A request whose system fails (a non-finite state after a step, or forces beyond the fixed-point
range) is stopped at the end of that chunk and completed with ``failed`` set and no result; the
others are unaffected.
"""
import time
from dataclasses import dataclass, field

import numpy as np

from . import batch as _batch



@dataclass
class Request:
    rid: int
    system: object      # workloads.System (positions, velocities, masses, body indices, species, box)
    steps: int
    arrival: float      # seconds from the start of the stream
    admitted: float = None
    started: float = None
    completed: float = None
    done_steps: int = 0
    chunks: list = field(default_factory=list)
    result: dict = None
    failed: str = None
    atoms: int = None   # atom count when `system` is made on demand by `make_system`
    make_system: object = None
    bodies: int = None  # rigid bodies (set when the request joins a group)

    def get_system(self):
        """The request's system, made on first use when the stream carries only its recipe."""
        if self.system is None:
            self.system = self.make_system()
        return self.system

    @property
    def num_atoms(self):
        return self.atoms if self.system is None else self.system.num_atoms

    @property
    def latency(self):
        return None if self.completed is None else self.completed - self.arrival


class _Group:
    """One batch of requests admitted together, stepped on its own stream."""

    def __init__(self, gid, batch, members, nbytes, stream):
        self.gid = gid
        self.batch = batch
        self.members = members
        self.bytes = nbytes
        self.stream = stream
        self.k = 0
        self.event = None       # recorded after the chunk in flight
        self.in_flight = False
        self.t_launch = 0.0

    def live(self):
        return [r for r in self.members if r.completed is None]

    def dead_atoms(self):
        return sum(r.num_atoms for r in self.members if r.completed is not None)

    def atoms(self):
        return sum(r.num_atoms for r in self.members)


class Server:
    """Continuous batching of simulation requests on one device.

    budget_bytes   device memory the server may hold (also capped by the free memory at start-up
                   less `reserve_bytes`)
    chunk_steps    steps per call; a group's chunk is shortened to end exactly at the earliest
                   completion among its requests
    keep_states    results carry the final positions and velocities (else the energies only)
    min_interval   seconds between group creations while earlier requests are running (arrivals
                   in between are admitted together)
    dead_fraction  a group whose finished or failed systems hold more than this fraction of its
                   atoms is compacted

    Groups advance independently: each has at most one chunk in flight on its stream, marked by an
    event; the loop waits for the oldest chunk, takes every chunk that has finished, and launches the
    next chunk of each of those groups at once, so a small group never waits for a large one and
    the host's admissions, group creations and result reads overlap the device's work.
    """

    def __init__(self, budget_bytes=150e9, chunk_steps=100, dt=0.002, precision="mixed", rotation_mode=0,
                 graph_steps=25, device=0, min_interval=0.05, dead_fraction=0.5, reserve_bytes=2e9,
                 batch_factory=None, sync=None, free_memory=None, stream_factory=None, keep_states=True,
                 event_factory=None):
        self.budget = float(budget_bytes)
        self.chunk = int(chunk_steps)
        self.dt = float(dt)
        self.precision = precision
        self.mode = rotation_mode
        self.graph_steps = graph_steps
        self.device = device
        self.min_interval = float(min_interval)
        self.dead_fraction = float(dead_fraction)
        self.reserve = float(reserve_bytes)
        self.keep_states = bool(keep_states)  # False: results hold the energies only
        self.groups_created = 0
        self.compactions = 0
        self.readmissions = 0  # groups released at creation because they held more than estimated
        self.launches = 0
        self.body_steps = 0
        self.peak_bytes = 0
        self.bytes_per_atom = None
        self.seconds = {"create": 0.0, "step": 0.0, "results": 0.0}
        # the batch type, device synchronisation, free-memory query and streams (replaceable to test
        # the scheduling on the CPU)
        self._factory = batch_factory or _batch.BatchedSystems.from_systems
        self._sync = sync
        self._free_memory = free_memory
        self._stream_factory = stream_factory
        self._event_factory = event_factory

    # ---------------------------------------------------------------------------------------
    def _torch_defaults(self):
        import torch
        if self._sync is None:
            self._sync = torch.cuda.synchronize
        if self._free_memory is None:
            self._free_memory = lambda: torch.cuda.mem_get_info(self.device)[0]
        if self._stream_factory is None:
            self._stream_factory = lambda: torch.cuda.Stream(self.device)
        if self._event_factory is None:
            self._event_factory = torch.cuda.Event

    def _make(self, systems):
        return self._factory(systems, rotation_mode=self.mode, precision=self.precision, device=self.device)

    def _measure(self, b, atoms):
        nbytes = int(b.memory_bytes)
        bpa = nbytes / max(atoms, 1)
        self.bytes_per_atom = bpa if self.bytes_per_atom is None else max(self.bytes_per_atom, bpa)
        return nbytes

    def _estimate(self, reqs):
        return sum(r.num_atoms for r in reqs) * self.bytes_per_atom

    def _probe(self, first):
        """Bytes per atom of a small batch of the first request's kind (created and released)."""
        sysm = first.get_system()
        b = self._make([sysm])
        self._measure(b, sysm.num_atoms)
        del b

    def _create(self, gid, members, saved=None):
        b = self._make([r.get_system() for r in members])
        for r in members:
            if r.bodies is None:
                r.bodies = int(r.get_system().num_bodies)
        if saved:
            fresh = b.checkpoint()
            b.restore([saved.get(r.rid, fresh[k]) for k, r in enumerate(members)])
        if self.graph_steps:
            b.set_graph_steps(self.graph_steps)
        nbytes = self._measure(b, sum(r.num_atoms for r in members))
        self.groups_created += 1
        return _Group(gid, b, members, nbytes, self._stream_factory())

    # ---------------------------------------------------------------------------------------
    def run(self, requests, realtime=True):
        """Serve `requests` (arrival times in seconds from now); returns them, completed (in the
        order they completed). With realtime=False every request counts as arrived at the start."""
        self._torch_defaults()
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        if not pending:
            return []
        budget = min(self.budget, float(self._free_memory()) - self.reserve)
        self.budget_used = budget
        self._probe(pending[0])
        groups, waiting, done = [], [], []
        in_use = 0
        last_create = -1e30
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0 if realtime else 0.0
        while pending or waiting or any(g.live() for g in groups):
            t = now()
            # admission, in arrival order, against the memory held plus the waiting requests
            while pending and (pending[0].arrival <= t or not realtime):
                nxt = pending[0]
                if in_use + self._estimate(waiting + [nxt]) > budget:
                    if not groups and not waiting:
                        raise ValueError(f"request {nxt.rid} ({nxt.num_atoms} atoms) exceeds the memory budget "
                                         f"({budget:.3g} bytes at {self.bytes_per_atom:.0f} bytes per atom)")
                    break
                pending.pop(0)
                nxt.admitted = t
                waiting.append(nxt)
            running = [g for g in groups if g.live()]
            if waiting and (not running or not realtime or t - last_create >= self.min_interval):
                tc = time.perf_counter()
                g = self._create(self.groups_created, waiting)
                if in_use + g.bytes > budget:
                    # the group holds more than its estimate: release it and admit its requests again
                    # later, at the bytes per atom it measured (`_measure` keeps the largest)
                    g.batch = None
                    self.readmissions += 1
                    if not groups:
                        raise ValueError(f"requests {[r.rid for r in waiting]} need {g.bytes} bytes, more than "
                                         f"the memory budget ({budget:.3g} bytes)")
                    for r in reversed(waiting):
                        r.admitted = None
                        pending.insert(0, r)
                    waiting = []
                else:
                    for r in waiting:
                        r.started = now()
                    groups.append(g)
                    in_use += g.bytes
                    self.peak_bytes = max(self.peak_bytes, in_use)
                    waiting = []
                last_create = now()
                self.seconds["create"] += time.perf_counter() - tc
                running = [g for g in groups if g.live()]
            if not running:  # idle until the next arrival
                if pending:
                    time.sleep(max(0.0, min(pending[0].arrival - now(), 0.01)))
                continue
            # the next chunk of every running group without one in flight, each on its own stream
            ts = time.perf_counter()
            for g in running:
                if g.in_flight:
                    continue
                g.k = min(self.chunk, min(r.steps - r.done_steps for r in g.live()))
                g.batch.step(g.k, self.dt, stream=g.stream)
                self.launches += g.batch.last_launch_count
                g.event = self._event_factory()
                g.event.record(g.stream)
                g.in_flight = True
                g.t_launch = time.perf_counter()
            # wait for the oldest chunk in flight; take every chunk that has finished
            min(running, key=lambda g: g.t_launch).event.synchronize()
            finished_chunks = [g for g in running if g.event.query()]
            self.seconds["step"] += time.perf_counter() - ts
            tf = time.perf_counter()
            for g in finished_chunks:
                g.in_flight = False
                live = g.live()
                self.body_steps += g.k * sum(r.bodies for r in live)
                for r in live:
                    r.done_steps += g.k
                    r.chunks.append(g.k)
                status = g.batch.status()
                finished = [i for i, r in enumerate(g.members) if r.completed is None and
                            (r.done_steps == r.steps or status[i] != 0)]
                if finished:
                    e = g.batch.energies()
                    tnow = now()
                    for i in finished:
                        r = g.members[i]
                        if status[i] != 0:
                            r.failed = "numeric failure: a non-finite state or forces beyond the fixed-point range"
                        elif self.keep_states:
                            x, v = g.batch.get_system_state(i)
                            r.result = {"positions": x, "velocities": v, "energies": e[i].copy()}
                        else:
                            r.result = {"energies": e[i].copy()}
                        r.completed = tnow
                        if r.make_system is not None:
                            r.system = None  # made again on demand (seeded)
                        done.append(r)
            self.seconds["results"] += time.perf_counter() - tf
            # release finished groups; compact mostly-finished ones (not while a chunk is in flight)
            kept = []
            for g in groups:
                if g.in_flight:
                    kept.append(g)
                    continue
                live = g.live()
                if not live:
                    in_use -= g.bytes
                    g.batch = None
                    continue
                if g.dead_atoms() > self.dead_fraction * g.atoms():
                    tc = time.perf_counter()
                    states = g.batch.checkpoint()
                    saved = {r.rid: states[k] for k, r in enumerate(g.members) if r.completed is None}
                    in_use -= g.bytes
                    g.batch = None
                    ng = self._create(g.gid, live, saved)
                    in_use += ng.bytes
                    self.compactions += 1
                    self.seconds["create"] += time.perf_counter() - tc
                    g = ng
                kept.append(g)
            groups = kept
        return done


def serve_alone(request, precision="mixed", rotation_mode=0, dt=0.002):
    """The request run by itself with the chunk lengths it had in the mix."""
    b = _batch.BatchedSystems.from_systems([request.get_system()], rotation_mode=rotation_mode, precision=precision)
    for k in request.chunks:
        b.step(k, dt)
    x, v = b.get_state()
    return {"positions": x, "velocities": v, "energies": b.energies()[0]}


def poisson_stream(rate, duration, atoms_range, steps_range, seed=8, lazy=False):
    """Seeded Poisson arrivals of rigid-water requests with log-uniform sizes (atoms) and step
    counts. With lazy=True each request carries its recipe and makes its system when first used."""
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
        sd = seed * 1000003 + rid
        make = (lambda nw=nw, sd=sd: W.mixed_system(n_bodies=nw, n_free=0, fractions=(1.0, 0.0, 0.0), seed=sd))
        if lazy:
            out.append(Request(rid, None, steps, t, atoms=3 * nw, make_system=make))
        else:
            out.append(Request(rid, make(), steps, t))
        rid += 1
    return out
