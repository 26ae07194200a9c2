"""Benchmark of the rigid-body integration step (one JSON line on rank 0).

Default workload (the batched-replicas configuration): 4096 independent systems per GPU, body
counts log-uniform in [64, 4096] (70 % 3-site waters, 20 % 5-atom tetrahedra, 10 % 12-atom planar
rings), each in its own periodic box at 1 g/cm^3, cutoff LJ + reaction-field forces from the
library's neighbour-list kernel, 300 K, dt 2 fs, rotation mode 0, mixed precision. One step is one full
velocity-Verlet step of every system (forces, then the integrator), all systems in one launch per
kernel, runs of steps replayed from captured CUDA graphs. The working set (2.2 GB of integrator
traffic per step, the neighbour lists besides) exceeds the 129 MB L2, so no flush is needed between
steps. Consecutive step calls take one force evaluation per step (a call starts from the forces the
previous one ended with).

  value   body-steps/s = bodies x steps / device time of exactly --steps steps (CUDA events on the
          launching stream, max over ranks), inputs resident in HBM
  plain / speedup_vs_plain  the same systems stepped one system per launch (one handle each, the
          plain drop-in way), from the same exact state, and the ratio; both energy drifts, and
          whether the final states and energies of the two arms are bit-equal
  e2e     the same metric through the public API with host buffers: positions and velocities in
          (set_state), the steps in chunks of 10 with the energies read back after each, positions
          and velocities out (wall clock; `seconds` splits it into the three parts)
  roofline  the integrator launches of the batched step (algorithmic bytes / event-timed launch
          time) against the measured HBM peak; the force kernels' share of the step beside it
  single_system  the single-large-system integrator step (1,000,000 bodies + 100,000 free atoms,
          fixed seeded forces sd 500 kJ/mol/nm, the fused step kernel), with its own roofline, e2e
          through the host-buffer C ABI and CPU baseline
  cpu_baseline  the CPU port of the reference integrator (oracle) with FP64 all-pairs forces on the
          box's host cores, on the four smallest systems
  clocks  nvidia-smi samples over the timed steps and repeats of them (a window of at least 1.5 s)

--workload single|served|water|precision selects the other workloads (their own lines).
--impl reference times the CPU implementation of the same workload on the host cores.
Multi-GPU (torchrun): world x --systems systems are generated once and assigned to ranks by body
count (partition.assign_systems); every rank steps its own share (weak scaling, no collective on
the data path); timings are max-reduced over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "body-steps/s batched/served vs plain at equal energy drift; p50/p99 latency"
UNIT = "body-steps/s"
def workload_name(bodies, free):
    """The single-system workload as benched (1,000,000 bodies and 100,000 free atoms by default)."""
    return (f"single large system: {bodies:,} rigid bodies (70% 3-site water, 20% 5-atom tetrahedra, "
            f"10% 12-atom rings) + {free:,} free LJ atoms; integrator-only, fixed seeded Gaussian forces "
            "sd 500 kJ/mol/nm; dt 2 fs")
# Algorithmic bytes of one fused step (drop-in OpenMM layout, atom velocities not materialised):
#   per body   273 B (single/mixed): r, v, q, pi float-float read + write (224) + 1/m and 1/I as
#                     float-float, three moment gaps (44) + first atom (4) + rotation class (1)
#              261 B (double): FP64 state (224) + 1/m, 1/I (32) + first atom (4) + class (1)
#   per atom    64 B: body-frame d FP32 (12) + slot (4) + fixed-point force (24) + posq.xyz and
#                     posqCorrection.xyz written (24); double: d FP64 (24) + slot + force + posq.xyz
#                     FP64 written (24) = 76 B
#   per free   128 B: force (24) + velocity read/write (48) + position and correction read/write
#                     (48) + 1/m (8)
BYTES_PER_BODY = {"single": 273, "mixed": 273, "double": 261}
BYTES_PER_BODY_ATOM = {"single": 64, "mixed": 64, "double": 76}
BYTES_PER_FREE = 128


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="rbx", choices=["rbx", "reference"])
    p.add_argument("--mode", type=int, default=0, help="rotation mode: 0 exact, n NO-SQUISH substeps")
    p.add_argument("--precision", default="mixed", choices=["single", "mixed", "double"])
    p.add_argument("--bodies", type=int, default=1_000_000)
    p.add_argument("--free", type=int, default=100_000)
    p.add_argument("--e2e-steps", type=int, default=30)
    p.add_argument("--replan", action="store_true",
                   help="single: also time rbx_set_atom_locations after OpenMM-style reorderings (key 'replan')")
    p.add_argument("--refined", action="store_true",
                   help="single: refined (shadow) energies on; each fused step also writes the stencil sums")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--reference-seconds", type=float, default=90.0,
                   help="bound on the timed CPU work of --impl reference")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--workload", default="batched", choices=["single", "batched", "water", "served", "precision"],
                   help="batched (default): many independent systems, full steps with the library's force field, "
                        "against one system per launch, with the single-system figures as an extra key; single: "
                        "the 1e6-body integrator step; water: 512 rigid waters, full steps")
    p.add_argument("--systems", type=int, default=4096, help="batched: number of systems per GPU")
    p.add_argument("--min-bodies", type=int, default=64, help="batched: smallest system (bodies)")
    p.add_argument("--max-bodies", type=int, default=4096, help="batched: largest system (bodies)")
    p.add_argument("--no-single", action="store_true", help="batched: skip the single-system figures")
    p.add_argument("--single-steps", type=int, default=500, help="batched: timed steps of the single-system figures")
    p.add_argument("--relax-steps", type=int, default=400, help="batched/water: relaxation before dynamics")
    p.add_argument("--graph-steps", type=int, default=50, help="batched/water: steps per captured CUDA graph")
    p.add_argument("--no-autotune", action="store_true",
                   help="batched/water: keep --graph-steps and the default cell-kernel block size")
    p.add_argument("--plain-systems", type=int, default=32, help="batched: systems run one per launch")
    p.add_argument("--tile-threads", default="auto", choices=["auto", "256", "128"],
                   help="single: step-kernel tile shape (auto: the faster of both, timed before the warm-up)")
    p.add_argument("--pbodies", type=int, default=8192, help="precision: near-degenerate bodies")
    p.add_argument("--pwaters", type=int, default=20000, help="precision: waters")
    p.add_argument("--psteps", type=int, default=1000, help="precision: steps per run")
    p.add_argument("--rate", type=float, default=200.0, help="served: request arrivals per second")
    p.add_argument("--duration", type=float, default=60.0, help="served: seconds of arrivals")
    p.add_argument("--max-atoms", type=int, default=200000, help="served: largest request (atoms)")
    p.add_argument("--min-steps", type=int, default=100, help="served: shortest request (steps)")
    p.add_argument("--max-steps", type=int, default=2000, help="served: longest request (steps)")
    p.add_argument("--plain-requests", type=int, default=24, help="served: requests also run one at a time")
    p.add_argument("--admit-interval", type=float, default=0.25,
                   help="served: seconds between group creations while others run")
    p.add_argument("--plain-steps", type=int, default=0,
                   help="batched: steps of the one-per-launch arm (0: the same as --steps)")
    return p.parse_args()


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend)
    return world, rank, local


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def build_workload(args, seed_offset=0):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = W.mixed_system(n_bodies=args.bodies, n_free=args.free, seed=3 + seed_offset)
    F = W.gaussian_forces(s.num_atoms, seed=5 + seed_offset)
    return s, F


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def host_link(h2d, d2h, device, reps=10):
    """The host-link bound of an e2e step: the same bytes moved by plain pinned-memory copies
    (cudaMemcpyAsync through torch), host->device and device->host each alone and both at once on
    two streams, timed with CUDA events. The e2e step cannot beat `copies_both_ms`."""
    import torch
    dev_in = torch.empty(h2d, dtype=torch.uint8, device=device)
    dev_out = torch.zeros(d2h, dtype=torch.uint8, device=device)
    h_in = torch.zeros(h2d, dtype=torch.uint8).pin_memory()
    h_out = torch.empty(d2h, dtype=torch.uint8).pin_memory()
    s_in, s_out = torch.cuda.Stream(device), torch.cuda.Stream(device)

    def run(which):
        cur = torch.cuda.current_stream(device)
        s_in.wait_stream(cur)
        s_out.wait_stream(cur)
        if which != "out":
            with torch.cuda.stream(s_in):
                dev_in.copy_(h_in, non_blocking=True)
        if which != "in":
            with torch.cuda.stream(s_out):
                h_out.copy_(dev_out, non_blocking=True)
        cur.wait_stream(s_in)
        cur.wait_stream(s_out)

    ms = {}
    for which in ("in", "out", "both"):
        for _ in range(3):
            run(which)
        torch.cuda.synchronize(device)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            run(which)
        b.record()
        b.synchronize()
        ms[which] = a.elapsed_time(b) / reps
    return {"h2d_gbs": h2d / ms["in"] / 1e6, "d2h_gbs": d2h / ms["out"] / 1e6, "copies_both_ms": ms["both"]}


def ncu_traffic_batched(bodies):
    """DRAM bytes of one fused step launch of the batched workload (mode 0, mixed) from the
    committed ncu summary, captured on 1024 systems and scaled to `bodies`; None without it."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    if "fused_batched_mode0_mixed_bytes_per_launch" not in d:
        return None
    return d["fused_batched_mode0_mixed_bytes_per_launch"] * bodies / d["batched_bodies"]


def ncu_traffic(mode, precision, bodies):
    """DRAM bytes of one fused step launch from the committed ncu summary (profiles/traffic.json),
    captured on a smaller case of the same mix and scaled to `bodies` (traffic is proportional to
    the number of bodies, atoms and free atoms, which scale together). None when no capture of this
    mode/precision is committed."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    key = f"fused_mode{mode}_{precision}_400k_bytes_per_launch"
    if key not in d:
        return None
    return d[key] * bodies / d["bodies"]


class ClockSampler:
    """nvidia-smi clock / throttle sampling; only samples that arrive between mark_start() and
    mark_end() (the timed region) are summarised."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, period_ms=50):
        self.gpu = gpu_index
        self.period_ms = period_ms
        self.proc = None
        self.thread = None
        self.lines = []  # (host time, csv line)
        self.t0 = self.t1 = None

    def _reader(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line))

    def __enter__(self):
        import threading
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._reader, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_end(self):
        self.t1 = time.perf_counter()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=5)

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0 = self.t0 if self.t0 is not None else -np.inf
        t1 = self.t1 if self.t1 is not None else np.inf
        for t, line in self.lines:
            if not t0 <= t <= t1:
                continue
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "period_ms": self.period_ms}


def cpu_baseline(s, F, args, seconds):
    """The oracle port of the reference CPU integrator on a bounded sample of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    from openmm_rigidbody_plugin_gb300 import workloads as W
    threads = os.cpu_count() or 1
    frac = 0.2  # a sample of 200,000 bodies at the default size: larger than the host caches
    sub = W.mixed_system(n_bodies=max(1000, int(args.bodies * frac)), n_free=int(args.free * frac), seed=3)
    Fs = W.gaussian_forces(sub.num_atoms, seed=5)
    o = oracle.Oracle(sub.masses, sub.body_indices, mode=args.mode, robust=True)
    o.setup(sub.positions, sub.velocities, Fs)
    o.run_fixed_force(0.002, Fs, 1, threads)
    t = o.run_fixed_force(0.002, Fs, 1, threads)
    steps = max(1, min(20000, int(seconds / max(t, 1e-6))))
    t = o.run_fixed_force(0.002, Fs, steps, threads)
    nb = o.num_bodies
    # one thread, as the Reference platform runs (a smaller sample, about 5 s)
    sub1 = W.mixed_system(n_bodies=max(1000, int(args.bodies * 0.02)), n_free=int(args.free * 0.02), seed=3)
    F1 = W.gaussian_forces(sub1.num_atoms, seed=5)
    o1 = oracle.Oracle(sub1.masses, sub1.body_indices, mode=args.mode, robust=True)
    o1.setup(sub1.positions, sub1.velocities, F1)
    t1 = o1.run_fixed_force(0.002, F1, 1, 1)
    steps1 = max(1, min(20000, int(5.0 / max(t1, 1e-6))))
    t1 = o1.run_fixed_force(0.002, F1, steps1, 1)
    return {"value": nb * steps / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{nb} bodies + {o.num_free} free atoms of the same mix, {steps} steps "
                      f"(part1+part2, fixed forces), {t:.1f} s, {threads} threads",
            "one_thread": {"value": o1.num_bodies * steps1 / t1, "unit": UNIT,
                           "sample": f"{o1.num_bodies} bodies + {o1.num_free} free atoms, {steps1} steps, {t1:.1f} s"}}


def run_reference(args, world, rank):
    """CPU implementation of the step on the host cores (rank 0 only). Each step integrates the
    full workload unless --steps of them would take longer than --reference-seconds; then each
    step integrates a seeded sample of the same mix, sized to fit that time."""
    if rank != 0:
        return
    if args.workload in ("batched", "water"):
        return run_reference_full_steps(args, world)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    from openmm_rigidbody_plugin_gb300 import workloads as W
    threads = os.cpu_count() or 1
    s, F = build_workload(args)
    o = oracle.Oracle(s.masses, s.body_indices, mode=args.mode, robust=True)
    o.setup(s.positions, s.velocities, F)
    t1 = o.run_fixed_force(0.002, F, 1, threads)
    sample = "full workload"
    if args.steps * t1 > args.reference_seconds:
        frac = args.reference_seconds / (args.steps * t1)
        nb_s = max(1000, int(args.bodies * frac))
        s = W.mixed_system(n_bodies=nb_s, n_free=int(args.free * nb_s / max(args.bodies, 1)), seed=3)
        F = W.gaussian_forces(s.num_atoms, seed=5)
        o = oracle.Oracle(s.masses, s.body_indices, mode=args.mode, robust=True)
        o.setup(s.positions, s.velocities, F)
        sample = f"a {nb_s}-body sample of the same mix per step (full workload x {args.steps} steps exceeds " \
                 f"{args.reference_seconds:.0f} s)"
    for _ in range(args.warmup):
        o.run_fixed_force(0.002, F, 1, threads)
    t = o.run_fixed_force(0.002, F, args.steps, threads)
    nb = o.num_bodies
    value = nb * args.steps / t
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": workload_name(args.bodies, args.free) + f"; rotation mode {args.mode}", "bodies": nb,
                      "atoms": int(s.num_atoms), "implementation": "CPU port of RigidBodySystem::integratePart1/2 "
                      "(robust variant: the reference's own eigen-solver and exact rotation produce NaN for the "
                      "tetrahedra and rings of this mix)"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"{sample}, {args.steps} steps, {threads} threads, {t:.1f} s"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def time_replan(k, buf, s, repeats=3):
    """Wall time of rbx_set_atom_locations after OpenMM-style reorderings (whole molecules moved to
    new slots, the buffers moved first as OpenMM moves them), best of `repeats`; the first call,
    which allocates the re-plan scratch, is not counted."""
    import torch
    rng = np.random.default_rng(11)
    bidx = np.asarray(s.body_indices)
    times, moves = [], []
    for r in range(repeats + 1):
        key = rng.random(int(bidx.max()) + 1)[np.maximum(bidx, 0)]
        free = bidx <= 0
        key[free] = rng.random(int(free.sum()))
        slot_to_atom = np.argsort(key, kind="stable")
        loc = np.empty(len(slot_to_atom), dtype=np.int64)
        loc[slot_to_atom] = np.arange(len(slot_to_atom))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        buf.relocate(loc)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        k.set_atom_locations(loc)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if r:
            moves.append(t1 - t0)
            times.append(t2 - t1)
    return {"set_atom_locations_ms": 1e3 * min(times), "buffer_moves_ms": 1e3 * min(moves),
            "what": "molecules shuffled to new slots; buffer moves = the posq/correction/velm/force gathers "
                    "OpenMM itself does (torch indexing here)"}


def choose_tile(k, buf, dt, stream, args, launches=40):
    """The step kernel's tile shape for the timed steps: as asked, or (auto, single/mixed) the faster
    of 256 and 128 threads over `launches` event-timed fused steps each, after 5 untimed ones. Both
    shapes give bit-identical results, so the trial only advances the warm-up. Returns (threads,
    {threads: ms per step} or None)."""
    import torch
    from openmm_rigidbody_plugin_gb300 import _lib
    if args.tile_threads != "auto":
        k.tile_threads = int(args.tile_threads)
        return k.tile_threads, None
    if args.precision == "double":
        return k.tile_threads, None
    trial = {}
    for nt in (256, 128):
        try:
            k.tile_threads = nt
        except _lib.RbxError:  # a body of more than 512 atoms
            continue
        for _ in range(5):
            k.fused(buf, dt, stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(launches):
            k.fused(buf, dt, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        trial[nt] = e0.elapsed_time(e1) / launches
    best = min(trial, key=trial.get)
    k.tile_threads = best
    return best, trial


def measure_single(args, world, rank, local, with_cpu=True, steps=None):
    """The single-large-system integrator step (the drop-in path): the fused step kernel timed over
    `steps` launches, its roofline, e2e through the host-buffer C ABI, and the CPU port beside it.
    Returns the JSON object (rank 0) or None."""
    import torch
    from openmm_rigidbody_plugin_gb300 import build, kernel
    torch.cuda.set_device(local)
    build.build_library()
    steps = steps or args.steps
    s, F = build_workload(args, seed_offset=0)
    dt = 0.002
    k = kernel.IntegratorKernel(s.masses, s.body_indices, rotation_mode=args.mode, precision=args.precision,
                                device=local)
    buf = kernel.DeviceBuffers(s.num_atoms, precision=args.precision, device=local)
    buf.set_positions(s.positions)
    buf.set_velocities(s.velocities, s.masses)
    buf.set_forces(F)
    k.upload_state(s.positions, s.velocities)
    if args.refined:
        k.set_compute_refined_energies(True)
    nb, nf = k.num_bodies, k.num_free
    nba = int(s.num_atoms) - nf
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()

    k.part1(buf, dt, stream)
    tile_threads, tile_trial = choose_tile(k, buf, dt, stream, args)
    for _ in range(args.warmup):
        k.fused(buf, dt, stream)
    torch.cuda.synchronize()
    barrier(world)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        time.sleep(0.3)  # nvidia-smi start-up
        torch.cuda.synchronize()
        clocks.mark_start()
        start.record(stream)
        for _ in range(steps):
            k.fused(buf, dt, stream)
        end.record(stream)
        torch.cuda.synchronize()
        repeats = 0
        while time.perf_counter() - clocks.t0 < 1.0:  # clock window of at least 1 s
            for _ in range(steps):
                k.fused(buf, dt, stream)
            torch.cuda.synchronize()
            repeats += 1
        clocks.mark_end()
    launches = steps
    t_dev = start.elapsed_time(end) / 1e3
    t_dev = max_over_ranks(t_dev, world)
    k.part2(buf, dt, stream)
    ke = k.kinetic_energies(buf, stream)
    if not np.all(np.isfinite(ke)):
        raise RuntimeError(f"non-finite kinetic energy after the timed steps: {ke}")
    refined = None
    if args.refined:
        refined = {"kinetic": [float(e) for e in k.refined_kinetic_energies(buf, stream)],
                   "potential_refinement": k.potential_energy_refinement(buf, stream)}
    replan = time_replan(k, buf, s) if args.replan else None
    value = world * nb * steps / t_dev
    bytes_step = BYTES_PER_BODY[args.precision] * nb + BYTES_PER_BODY_ATOM[args.precision] * nba + BYTES_PER_FREE * nf
    if args.refined:  # stencil sums written by every fused step: 7 values per body, 3 per free atom
        es = 8 if args.precision == "double" else 4
        bytes_step += 7 * es * nb + 3 * es * nf
    per_launch = t_dev / steps
    peak, peak_kind = peaks()
    achieved = bytes_step / per_launch / 1e9
    traffic = None if args.refined else ncu_traffic(args.mode, args.precision, nb)  # captured for the plain kernel

    # e2e through the host-buffer C ABI (pinned host arrays, copies inside the timed region):
    # every step uploads its forces and downloads its positions and velocities; consecutive
    # steps are pipelined (rbx_step_host_async), so one step's copies overlap another's kernels
    x_h = [torch.empty((s.num_atoms, 3), dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    v_h = [torch.empty((s.num_atoms, 3), dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    f_h = torch.from_numpy(np.ascontiguousarray(F)).pin_memory().numpy()
    ke2 = kernel.IntegratorKernel(s.masses, s.body_indices, rotation_mode=args.mode, precision=args.precision,
                                  device=local)
    ke2.tile_threads = tile_threads
    ke2.context_set_state(s.positions, s.velocities, stream)
    for i in range(2):
        ke2.step_host_async(1, dt, f_h, x_h[i % 2], v_h[i % 2], stream)
    ke2.step_host_wait()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.e2e_steps):
        ke2.step_host_async(1, dt, f_h, x_h[i % 2], v_h[i % 2], stream)
    ke2.step_host_wait()
    t_e2e = max_over_ranks((time.perf_counter() - t0) / args.e2e_steps, world)
    e2e = {"value": world * nb / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(F.size * 8),
           "d2h_bytes_per_step": int(2 * s.num_atoms * 3 * 8),
           "call": "rbx_step_host_async per step (forces in, one step = part1 + part2, positions and velocities "
                   "out, pinned host arrays), steps pipelined, rbx_step_host_wait at the end"}
    link = host_link(e2e["h2d_bytes_per_step"], e2e["d2h_bytes_per_step"], local)
    link["e2e_ms_per_step"] = 1e3 * t_e2e
    link["frac"] = link["copies_both_ms"] / link["e2e_ms_per_step"]
    link["what"] = "the same bytes by plain pinned copies, both directions at once: the bound of the e2e step"
    e2e["host_link"] = link

    if rank != 0:
        return None
    cpu = None
    if with_cpu:
        cpu = cpu_baseline(s, F, args, args.cpu_seconds)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": {"mixed": "f32 atoms + f64 body state", "double": "f64", "single": "f32"}[args.precision],
           "data": "synthetic",
           "config": {"workload": workload_name(args.bodies, args.free) + f"; rotation mode {args.mode}; {args.precision} precision"
                                  + ("; refined energies on" if args.refined else ""),
                      "bodies_per_gpu": nb, "body_atoms_per_gpu": nba, "free_atoms_per_gpu": nf,
                      "tile_threads": tile_threads, "tile_trial_ms_per_step": tile_trial,
                      "l2": "working set > 129 MB L2 (no flush needed)", "parallelism": f"{world} independent replicas"},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "peak_source": peak_kind, "traffic": traffic, "algorithmic_bytes_per_launch": bytes_step,
                        "kernel": "rbx::step_kernel (fused)"},
           "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
           "clocks": dict(clocks.summary(), window=f"the timed {steps} steps plus {repeats} repeats of them (at least 1 s)"),
           "kinetic_energy_after": [float(ke[0]), float(ke[1])]}
    if refined is not None:
        out["refined_after"] = refined
    if replan is not None:
        out["replan"] = replan
    return out


def run_gpu(args, world, rank, local):
    out = measure_single(args, world, rank, local, with_cpu=not args.no_cpu)
    if out is not None:
        print(json.dumps(out), flush=True)


def _drift(e_pre, e_post, steps, dt, dof):
    """Energy drift per system: kJ/mol/ns/DOF and |dE|/|E0| of the total energy U + KE_t + KE_r."""
    tot0, tot1 = e_pre.sum(axis=1), e_post.sum(axis=1)
    per_ns = (tot1 - tot0) / (steps * dt * 1e-3) / np.asarray(dof, dtype=np.float64)
    rel = np.abs(tot1 - tot0) / np.abs(tot0)
    return {"kj_mol_ns_dof_median_abs": float(np.median(np.abs(per_ns))),
            "kj_mol_ns_dof_max_abs": float(np.max(np.abs(per_ns))),
            "rel_dE_median": float(np.median(rel)), "rel_dE_max": float(np.max(rel))}


def cpu_full_steps(systems, x, v, offsets, seconds):
    """The oracle's full step (CPU port of the reference integrator + FP64 O(N^2) LJ + reaction-field
    forces on all host threads) over the given systems, for about `seconds`."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    from openmm_rigidbody_plugin_gb300 import workloads as W
    threads = os.cpu_count() or 1
    runs = []
    for k, s in enumerate(systems):
        q, sg, ep = W.nonbonded(s)
        rc = W.cutoff_for(s.box)
        o = oracle.Oracle(s.masses, s.body_indices, mode=0, robust=True)
        force = (lambda R, s=s, q=q, sg=sg, ep=ep, rc=rc:
                 oracle.lj_rf([0, s.num_atoms], [s.box], [rc], R, q, sg, ep, s.body_indices, nthreads=threads)[0])
        o.setup(x[offsets[k]:offsets[k + 1]], v[offsets[k]:offsets[k + 1]], force(x[offsets[k]:offsets[k + 1]]))
        runs.append((o, force, s.num_bodies))
    steps, body_steps, t0 = 0, 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for o, force, nb in runs:
            o.part1(0.002, force(o.R))
            o.part2(0.002, force(o.R))
            body_steps += nb
        steps += 1
    t = time.perf_counter() - t0
    return {"value": body_steps / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(runs)} systems ({sum(r[2] for r in runs)} bodies), {steps} full steps each "
                      f"(integrator + FP64 all-pairs LJ/RF forces on {threads} threads), {t:.1f} s"}


def run_reference_full_steps(args, world):
    """CPU full steps (oracle integrator + FP64 LJ/RF forces, all host threads) on the batched or
    water workload: the four smallest systems of the batch (a bounded sample; the starting
    structures are the generated ones, not relaxed, since the relaxation runs on the GPU)."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    if args.workload == "water":
        systems = [W.water_box(512, seed=1)]
        config = {"workload": "512 rigid 3-site waters, cubic box at 1 g/cm3, cutoff 0.9 nm LJ + reaction field, "
                              "dt 2 fs, rotation mode 0, mixed precision, full steps",
                  "parallelism": f"{world} independent replicas"}
    else:
        counts = W.batch_body_counts(args.systems * world, lo=args.min_bodies, hi=args.max_bodies, seed=6)
        pick = np.argsort(counts, kind="stable")[:4]
        systems = W.batch_systems(args.systems * world, lo=args.min_bodies, hi=args.max_bodies, seed=6, only=pick)
        config = batched_config(args, world)
    x = np.concatenate([s.positions for s in systems])
    v = np.concatenate([s.velocities for s in systems])
    offs = np.concatenate([[0], np.cumsum([s.num_atoms for s in systems])])
    r = cpu_full_steps(systems, x, v, offs, args.reference_seconds / 3)
    out = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
           "implementation": "CPU port of RigidBodySystem::integratePart1/2 (robust variant) + FP64 all-pairs "
                             "cutoff LJ/RF forces",
           "cpu_baseline": r, "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                                      "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def batched_systems_for_rank(args, world, rank):
    """The rank's share of the batched-replicas workload: world x --systems systems (seeded once),
    assigned to ranks by their body counts (partition.assign_systems, longest first), so every rank
    holds about --systems systems' worth of bodies (weak scaling) and no system is on two ranks."""
    from openmm_rigidbody_plugin_gb300 import partition
    from openmm_rigidbody_plugin_gb300 import workloads as W
    counts = W.batch_body_counts(args.systems * world, lo=args.min_bodies, hi=args.max_bodies, seed=6)
    owner, _ = partition.assign_systems(counts, world)
    mine = np.flatnonzero(owner == rank)
    return mine, W.batch_systems(args.systems * world, lo=args.min_bodies, hi=args.max_bodies, seed=6, only=mine)


def batched_config(args, world):
    """The `config` of the batched workload, identical in both arms."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    counts = W.batch_body_counts(args.systems * world, lo=args.min_bodies, hi=args.max_bodies, seed=6)
    return {"workload": (f"batched replicas: {args.systems} independent systems per GPU, body counts "
                         f"log-uniform in [{args.min_bodies}, {args.max_bodies}] (70% 3-site water, 20% 5-atom "
                         "tetrahedra, 10% 12-atom rings), each in its own cubic box at 1 g/cm3, cutoff 0.9 nm "
                         "(0.49 box below 1.84 nm) LJ + reaction field, 300 K, dt 2 fs, rotation mode 0, mixed "
                         "precision, full steps (forces + integrator)"),
            "systems_per_gpu": args.systems, "bodies_total": int(counts.sum()), "steps": args.steps,
            "parallelism": f"{world} rank(s); systems assigned to ranks by body count, no collective on the data path",
            "l2": "working set (about 1 GB per GPU) > 129 MB L2, no flush needed"}


def run_batched(args, world, rank, local):
    """Many independent systems stepped together (full steps: neighbour-list forces + integrator, one
    launch per kernel per step, runs of steps replayed from captured CUDA graphs), against the same
    systems stepped one system per launch (the plain drop-in way), at equal energy drift."""
    import torch
    from openmm_rigidbody_plugin_gb300 import batch, build
    from openmm_rigidbody_plugin_gb300 import workloads as W
    torch.cuda.set_device(local)
    build.build_library()
    dt = 0.002
    if args.workload == "water":
        systems = [W.water_box(512, seed=1 + 1000 * rank)]
        config = {"workload": "512 rigid 3-site waters, cubic box at 1 g/cm3, cutoff 0.9 nm LJ + reaction field, "
                              "dt 2 fs, rotation mode 0, mixed precision, full steps",
                  "parallelism": f"{world} independent replicas"}
    else:
        _, systems = batched_systems_for_rank(args, world, rank)
        config = batched_config(args, world)
    nb = sum(s.num_bodies for s in systems)
    na = sum(s.num_atoms for s in systems)
    t0 = time.perf_counter()
    b = batch.BatchedSystems.from_systems(systems, relax_steps=args.relax_steps, device=local)
    b.set_graph_steps(args.graph_steps)
    setup_s = time.perf_counter() - t0
    dof = b.num_dof
    b.step(max(args.warmup, 3), dt)
    # the autotuner picks the schedule on this batch (and restores its state exactly)
    tuning = b.autotune(dt, trial_steps=3) if not args.no_autotune else None
    x0, v0 = b.get_state()
    b.set_state(x0, v0)
    # warm-up: at least W steps, and enough for the first CUDA-graph capture to happen here; both
    # arms then start from the exact state after it (checkpoint / restore)
    graph_k = tuning["graph_steps"] if tuning else args.graph_steps
    b.step(max(args.warmup, graph_k + 1), dt)
    ckpt = b.checkpoint()
    e_pre = b.energies()
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    barrier(world)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    builds0 = b.list_builds()
    with ClockSampler(local) as clocks:
        time.sleep(0.3)
        torch.cuda.synchronize()
        clocks.mark_start()
        start.record(stream)
        b.step(args.steps, dt)
        end.record(stream)
        torch.cuda.synchronize()
        launches = b.last_launch_count
        builds = (b.list_builds() - builds0).astype(np.int64)
        e_post = b.energies()
        plain_idx = np.unique(np.linspace(0, len(systems) - 1, min(args.plain_systems, len(systems))).astype(int))
        final_b = [b.get_system_state(int(k)) for k in plain_idx] if args.plain_systems > 0 else []
        # the clocks are sampled over the timed steps and over repeats of them until the window
        # lasts at least 1.5 s, so that a short timed region still has its own clock record
        repeats = 0
        while time.perf_counter() - clocks.t0 < 1.5:
            b.step(args.steps, dt)
            torch.cuda.synchronize()
            repeats += 1
        clocks.mark_end()
    t_dev = max_over_ranks(start.elapsed_time(end) / 1e3, world)
    value = world * nb * args.steps / t_dev
    drift = _drift(e_pre, e_post, args.steps, dt, dof)

    # kernel split (event-timed direct launches; same work): a call of k steps that follows another
    # takes k force evaluations and k + 1 integrator launches (part1, k - 1 fused, part2)
    k_split = 20
    b.set_timing(True)
    b.step(k_split, dt)
    ms_f, ms_i, _ = b.kernel_times()
    b.set_timing(False)
    bytes_step = BYTES_PER_BODY["mixed"] * nb + BYTES_PER_BODY_ATOM["mixed"] * na
    t_int = ms_i / (k_split + 1) / 1e3  # per integrator launch
    peak, peak_kind = peaks()
    achieved = bytes_step / t_int / 1e9

    # e2e through the public API with host buffers: the systems' positions and velocities go in
    # from pinned host memory (set_state, which also builds every body on the device), the steps
    # run in chunks of 10 with the energies read back after each chunk, and the final positions
    # and velocities come back to pinned host memory
    xh = torch.from_numpy(np.ascontiguousarray(x0)).pin_memory().numpy()
    vh = torch.from_numpy(np.ascontiguousarray(v0)).pin_memory().numpy()
    chunk = 10
    nchunks = max(1, args.steps // chunk)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    b.set_state(xh, vh)
    t1 = time.perf_counter()
    for _ in range(nchunks):
        b.step(chunk, dt)
        b.energies()
    t2 = time.perf_counter()
    xo, vo = b.get_state()
    t3 = time.perf_counter()
    t_e2e = max_over_ranks(t3 - t0, world)
    e2e_steps = nchunks * chunk
    e2e = {"value": world * nb * e2e_steps / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": int(2 * 24 * na / e2e_steps),
           "d2h_bytes_per_step": int((2 * 24 * na + 24 * len(systems) * nchunks) / e2e_steps),
           "call": f"BatchedSystems.set_state (positions and velocities in), {nchunks} x (step({chunk}) + "
                   "energies()), get_state (positions and velocities out): rbx_batch_set_state, rbx_batch_step, "
                   "rbx_batch_energies, rbx_batch_get_state; wall clock",
           "seconds": {"set_state": t1 - t0, "steps_and_energies": t2 - t1, "get_state": t3 - t2}}

    # the same systems, one system per launch (the plain drop-in way: one context per system)
    plain = None
    if args.workload == "batched" and args.plain_systems > 0:
        idx = plain_idx
        off = b.offsets
        handles = []
        plain_steps = args.plain_steps or args.steps
        for k in idx:
            h = batch.BatchedSystems.from_systems([systems[k]], device=local)
            h.set_graph_steps(graph_k)
            h.set_state(x0[off[k]:off[k + 1]], v0[off[k]:off[k + 1]])
            h.step(max(args.warmup, graph_k + 1), dt)  # warm-up and the graph capture, untimed
            h.restore([ckpt[k]])                      # the batched arm's starting state, exactly
            handles.append(h)
        e_pre_p = np.array([h.energies()[0] for h in handles])
        torch.cuda.synchronize()
        pa, pb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pa.record(stream)
        for h in handles:
            h.step(plain_steps, dt)
        pb.record(stream)
        torch.cuda.synchronize()
        t_plain = pa.elapsed_time(pb) / 1e3
        e_post_p = np.array([h.energies()[0] for h in handles])
        nb_p = sum(systems[k].num_bodies for k in idx)
        plain = {"value": nb_p * plain_steps / t_plain, "unit": UNIT, "systems": int(len(idx)),
                 "bodies": int(nb_p), "steps": plain_steps,
                 "energy_drift": _drift(e_pre_p, e_post_p, plain_steps, dt, dof[idx]),
                 "how": "each system its own handle (rbx_batch of one system), steps launched system after system"}
        if plain_steps == args.steps:  # the same systems inside the batch, over the same steps
            plain["batched_energy_drift_same_systems"] = _drift(e_pre[idx], e_post[idx], args.steps, dt, dof[idx])
            plain["same_final_energies_as_batched"] = bool(np.array_equal(e_post_p, e_post[idx]))
            plain["final_energies_max_abs_diff"] = [float(v) for v in np.abs(e_post_p - e_post[idx]).max(axis=0)]
            same_state = [bool(np.array_equal(h.get_state()[0], xb) and np.array_equal(h.get_state()[1], vb))
                          for h, (xb, vb) in zip(handles, final_b)]
            plain["same_final_state_as_batched"] = f"{sum(same_state)} of {len(same_state)} systems"
            plain["status_nonzero"] = {"batched": int(np.count_nonzero(b.status())),
                                       "plain": int(sum(int(np.count_nonzero(h.status())) for h in handles))}
        del handles
    single = None
    if args.workload == "batched" and not args.no_single:
        del b
        single = measure_single(args, world, rank, local, with_cpu=not args.no_cpu, steps=args.single_steps)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        pick = [0] if args.workload == "water" else list(np.argsort([s.num_bodies for s in systems])[:4])
        off = np.concatenate([[0], np.cumsum([s.num_atoms for s in systems])])
        sub = [systems[k] for k in pick]
        xs = np.concatenate([x0[off[k]:off[k + 1]] for k in pick])
        vs = np.concatenate([v0[off[k]:off[k + 1]] for k in pick])
        offs = np.concatenate([[0], np.cumsum([s.num_atoms for s in sub])])
        cpu = cpu_full_steps(sub, xs, vs, offs, args.cpu_seconds)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 atoms + f64 body state", "data": "synthetic",
           "config": config,
           "setup": {"systems_on_rank0": len(systems), "bodies_on_rank0": nb, "atoms_on_rank0": na,
                     "relax_steps": args.relax_steps, "seconds": setup_s, "autotune": tuning},
           "energy_drift": drift, "plain": plain,
           "neighbour_lists": {"builds_per_system_in_timed_steps_mean": float(builds.mean()),
                               "force_evaluations": args.steps,
                               "atoms_rebuilt_per_evaluation": float(np.sum(builds * np.array(
                                   [s.num_atoms for s in systems])) / args.steps / na)},
           "speedup_vs_plain": (value / world / plain["value"]) if plain else None,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "peak_source": peak_kind, "traffic": ncu_traffic_batched(nb) if args.workload == "batched" else None,
                        "algorithmic_bytes_per_launch": bytes_step,
                        "kernel": "rbx::step_kernel_f (the integrator launches of the batched step: part1, fused, "
                                  "part2; bytes per fused launch)",
                        "integrator_ms_per_step": ms_i / k_split, "integrator_ms_per_launch": ms_i / (k_split + 1),
                        "force_ms_per_step": ms_f / k_split,
                        "force_share": ms_f / (ms_f + ms_i)},
           "cpu_baseline": cpu, "e2e": e2e, "clocks": dict(clocks.summary(), window=(
               f"the timed {args.steps} steps plus {repeats} repeats of them (at least 1.5 s)")),
           "gpu_launches": launches}
    if single is not None:
        out["single_system"] = single
    print(json.dumps(out), flush=True)


def run_served(args, world, rank, local):
    """Continuous batching of a seeded Poisson stream of simulation requests (serving.Server), with
    p50/p99 completion latency and aggregate body-steps/s, against a one-request-at-a-time server on
    the first requests of the same stream (their latency served and alone, and whether each result
    is the same bit for bit)."""
    import torch
    from openmm_rigidbody_plugin_gb300 import batch, build, serving
    torch.cuda.set_device(local)
    build.build_library()
    stream = serving.poisson_stream(args.rate, args.duration, (100, args.max_atoms), (args.min_steps, args.max_steps),
                                    seed=8 + 1000 * rank, lazy=True)
    nreq = len(stream)
    # warm the library (module load, kernel attributes) outside the served clock
    warm = batch.BatchedSystems.from_systems([stream[0].get_system()])
    warm.set_graph_steps(25)
    warm.step(60, 0.002)
    del warm
    torch.cuda.synchronize()
    server = serving.Server(budget_bytes=150e9, chunk_steps=100, graph_steps=25, device=local, keep_states=False,
                            min_interval=args.admit_interval)
    barrier(world)
    with ClockSampler(local) as clocks:
        clocks.mark_start()
        t0 = time.perf_counter()
        done = server.run(stream, realtime=True)
        wall = time.perf_counter() - t0
        clocks.mark_end()
    wall = max_over_ranks(wall, world)
    ok = [r for r in done if r.failed is None]
    lat = np.array([r.latency for r in ok])
    body_steps = sum(r.bodies * r.steps for r in ok)
    value = world * body_steps / wall
    # one request at a time (the plain way), on the first requests of the stream: each request's
    # service time alone, then the FIFO queue replayed on the same arrival times
    sub = sorted(ok, key=lambda r: r.rid)[:min(args.plain_requests, len(ok))]
    service, same = [], 0
    for r in sub:
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        alone = serving.serve_alone(r)
        torch.cuda.synchronize()
        service.append(time.perf_counter() - t1)
        same += int(np.array_equal(alone["energies"], r.result["energies"]))
        r.system = None
    fin, lat_plain = 0.0, []
    for r, t_s in zip(sub, service):
        fin = max(fin, r.arrival) + t_s
        lat_plain.append(fin - r.arrival)
    lat_plain = np.array(lat_plain)
    plain_value = sum(r.bodies * r.steps for r in sub) / sum(service)
    lat_sub = np.array([r.latency for r in sub])
    # the whole stream served one request at a time: service times from a least-squares fit of the
    # measured ones (seconds = a + b x body-steps), queued first come first served
    work = np.array([r.bodies * r.steps for r in sub], dtype=np.float64)
    coef = np.linalg.lstsq(np.stack([np.ones_like(work), work], axis=1), np.array(service), rcond=None)[0]
    fin, lat_fifo = 0.0, []
    for r in sorted(ok, key=lambda r: (r.arrival, r.rid)):
        fin = max(fin, r.arrival) + max(coef[0] + coef[1] * r.bodies * r.steps, 0.0)
        lat_fifo.append(fin - r.arrival)
    lat_fifo = np.array(lat_fifo)
    if rank != 0:
        return
    bytes_in = sum(r.num_atoms * 48 for r in done)    # positions + velocities in
    bytes_out = sum(24 for r in done)                 # energies out
    total_steps = sum(r.steps for r in done)
    pct = lambda a, q: float(np.percentile(a, q)) if len(a) else None
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": total_steps,
           "warmup": 60, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 atoms + f64 body state", "data": "synthetic",
           "config": {"workload": f"served: Poisson arrivals at {args.rate:g} req/s for {args.duration:g} s "
                                  f"({nreq} requests), rigid-water systems of 100 to {args.max_atoms} atoms "
                                  f"(log-uniform), {args.min_steps} to {args.max_steps} steps (log-uniform), dt 2 fs, "
                                  "cutoff LJ + reaction field, mixed precision; 150 GB budget (capped by the free "
                                  "device memory); chunks of 100 steps, 25-step CUDA graphs, one group (batch) per "
                                  "admission, groups on their own streams",
                      "requests": nreq, "parallelism": f"{world} independent replicas"},
           "serving": {"wall_seconds": wall, "completed": len(ok), "failed": len(done) - len(ok),
                       "groups_created": server.groups_created, "compactions": server.compactions,
                       "budget_bytes": server.budget_used, "peak_bytes": server.peak_bytes,
                       "bytes_per_atom_measured": server.bytes_per_atom, "server_seconds": server.seconds},
           "latency_s": {"p50": pct(lat, 50), "p99": pct(lat, 99), "max": float(lat.max()) if len(lat) else None},
           "plain": {"value": plain_value, "unit": UNIT, "requests": len(sub),
                     "latency_s": {"p50": pct(lat_plain, 50), "p99": pct(lat_plain, 99)},
                     "served_latency_same_requests_s": {"p50": pct(lat_sub, 50), "p99": pct(lat_sub, 99)},
                     "same_energies_alone_and_served": f"{same} of {len(sub)}",
                     "whole_stream_one_at_a_time_latency_s": {"p50": pct(lat_fifo, 50), "p99": pct(lat_fifo, 99),
                                                              "model_seconds": [float(coef[0]), float(coef[1])],
                                                              "how": "service time a + b x body-steps fitted to the "
                                                                     "measured requests, first come first served"},
                     "how": "each request alone (its own handle, same chunk lengths), queued first come first "
                            "served on the same arrival times"},
           "speedup_vs_plain": value / world / plain_value,
           "roofline": None, "cpu_baseline": None,
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": int(bytes_in / max(total_steps, 1)),
                   "d2h_bytes_per_step": int(bytes_out / max(total_steps, 1)),
                   "call": "serving.Server.run (host structures in, energies out; wall clock)"},
           "clocks": clocks.summary(), "gpu_launches": server.launches}
    print(json.dumps(out), flush=True)


def run_precision(args, world, rank, local):
    """Precision study: near-degenerate bodies (two principal moments 1+eps apart, eps log-uniform in
    [1e-8, 1e-2]) among waters, full steps with the library's force field; every precision and
    rotation mode from the same relaxed state; energy drift and trajectory error after --psteps
    steps against the double-precision run of the same mode and step size."""
    import torch
    from openmm_rigidbody_plugin_gb300 import batch, build
    from openmm_rigidbody_plugin_gb300 import workloads as W
    torch.cuda.set_device(local)
    build.build_library()
    s = W.near_degenerate_system(args.pbodies, args.pwaters, seed=7 + 1000 * rank)
    b0 = batch.BatchedSystems.from_systems([s], relax_steps=args.relax_steps, device=local)
    x0, v0 = b0.get_state()
    dof = int(b0.num_dof[0])
    del b0
    rows, stream = [], torch.cuda.current_stream()
    mixed_rate = None
    with ClockSampler(local) as clocks:
        clocks.mark_start()
        for dt in (0.001, 0.004):
            for mode in (0, 1, 4, 16):
                runs = {}
                for prec in ("double", "mixed", "single"):
                    b = batch.BatchedSystems.from_systems([s], rotation_mode=mode, precision=prec, device=local)
                    b.set_graph_steps(50)
                    b.set_state(x0, v0)
                    e0 = b.energies()[0]
                    early = []
                    t, done = 0.0, 0
                    for n in (10, 100, args.psteps):  # trajectory samples after 10, 100 and all steps
                        a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                        torch.cuda.synchronize()
                        a.record(stream)
                        b.step(n - done, dt)
                        c.record(stream)
                        torch.cuda.synchronize()
                        t += a.elapsed_time(c) / 1e3
                        done = n
                        early.append(b.get_state())
                    e1 = b.energies()[0]
                    x, v = early[-1]
                    runs[prec] = (x, v, e0, e1, t, early)
                    if prec == "mixed" and mode == 0 and dt == 0.001:
                        mixed_rate = s.num_bodies * args.psteps / t
                xd, vd = runs["double"][0], runs["double"][1]
                rel = lambda a, r: float(np.max(np.abs(a - r)) / np.max(np.abs(r)))
                for prec, (x, v, e0, e1, t, early) in runs.items():
                    de = float(e1.sum() - e0.sum())
                    ed = runs["double"][5]
                    rows.append({"dt_ps": dt, "mode": mode, "precision": prec, "ms_per_step": 1e3 * t / args.psteps,
                                 "drift_kj_mol_ns_dof": de / (args.psteps * dt * 1e-3) / dof,
                                 "rel_dE": abs(de) / abs(float(e0.sum())),
                                 "traj_err_x_vs_double": rel(x, xd), "traj_err_v_vs_double": rel(v, vd),
                                 "traj_err_x_10_100_steps": [rel(early[0][0], ed[0][0]), rel(early[1][0], ed[1][0])],
                                 "traj_err_v_10_100_steps": [rel(early[0][1], ed[0][1]), rel(early[1][1], ed[1][1])]})
        clocks.mark_end()
    if rank != 0:
        return
    out = {"metric": METRIC, "value": mixed_rate, "unit": UNIT, "n_gpus": world, "steps": args.psteps, "warmup": 0,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 atoms + f64 body state",
           "data": "synthetic",
           "config": {"workload": f"precision study: {args.pbodies} near-degenerate rigid bodies (planar 4-atom "
                                  "crosses, two principal moments 1+eps apart, eps log-uniform in [1e-8, 1e-2]) + "
                                  f"{args.pwaters} waters at 1 g/cm3, cutoff LJ + reaction field; {args.psteps} "
                                  "steps at dt 1 and 4 fs in single, mixed and double, rotation modes 0, 1, 4, 16; "
                                  "value = mixed, mode 0, 1 fs (the stated 100,000-step runs shortened to "
                                  f"{args.psteps})",
                      "bodies": int(s.num_bodies), "atoms": int(s.num_atoms), "dof": dof,
                      "forces": "FP32 neighbour-list force pass in every precision (the study varies the integrator)"},
           "precision_study": rows, "roofline": None, "cpu_baseline": None,
           "e2e": None, "clocks": clocks.summary(), "gpu_launches": None}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    world, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload in ("batched", "water"):
        run_batched(args, world, rank, local)
    elif args.workload == "served":
        run_served(args, world, rank, local)
    elif args.workload == "precision":
        run_precision(args, world, rank, local)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
