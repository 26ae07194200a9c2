"""Host-side partitioning for several GPUs: replicas only.

Systems are independent in the integrator and in the force field, so a multi-GPU run gives each
rank its own systems and needs no collective on the data path; results and energies are gathered
only for reporting. ``assign_systems`` balances the work (bodies x steps) over the ranks by
longest-processing-time-first; ``gather_by_system`` puts per-system results back in system order
on every rank (torch.distributed, any backend).
"""
import numpy as np


def assign_systems(work, world_size):
    """Rank of each system: systems in decreasing work, each to the least-loaded rank (ties to the
    lower rank). Returns (rank per system, load per rank)."""
    work = np.asarray(work, dtype=np.float64)
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    rank = np.empty(len(work), dtype=np.int64)
    load = np.zeros(world_size)
    for s in np.argsort(-work, kind="stable"):
        r = int(np.argmin(load))
        rank[s] = r
        load[r] += work[s]
    return rank, load


def local_systems(work, world_size, rank):
    """Indices of the systems a rank owns, in increasing order."""
    owner, _ = assign_systems(work, world_size)
    return np.nonzero(owner == rank)[0]


def gather_by_system(local_values, local_index, num_systems, group=None):
    """Every rank's per-system rows (local_values[k] for system local_index[k]) -> one array in
    system order, on every rank."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (list(map(int, local_index)), np.asarray(local_values).tolist()), group=group)
    rows = [None] * num_systems
    for idx, vals in parts:
        for s, v in zip(idx, vals):
            if rows[s] is not None:
                raise ValueError(f"system {s} reported by two ranks")
            rows[s] = v
    if any(r is None for r in rows):
        raise ValueError("a system was reported by no rank")
    return np.array(rows)
