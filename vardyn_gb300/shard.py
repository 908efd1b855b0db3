"""Independent assimilation windows over GPUs: replicas only.

The reference runs one process per window and hands GPUs out round-robin
(run_assimilation.py:27-349); windows never exchange data. Here one process
per GPU takes a share of the windows:

- :func:`assign` splits windows over ranks by greedy bin-packing of their
  cost ny * nx * nstep (longest first, each to the least-loaded rank, ties to
  the lower rank): deterministic, every rank computes the same split, and the
  largest load is at most 4/3 of the best split's;
- :func:`max_over_ranks` is the one collective of a timed run: the slowest
  rank's time;
- :func:`gather_to_root` collects per-window results on rank 0 through the
  host (pickled objects over a CPU process group), after the timed region.
"""
import torch
import torch.distributed as dist


def window_cost(ny, nx, nstep):
    """Work of one window: grid points times model steps."""
    return int(ny) * int(nx) * int(nstep)


def assign(costs, world):
    """owner[i] in [0, world) for every window i, and the load of each rank."""
    world = int(world)
    if world < 1:
        raise ValueError("world must be >= 1")
    costs = [int(c) for c in costs]
    if any(c < 0 for c in costs):
        raise ValueError("window costs must be >= 0")
    owner = [0] * len(costs)
    loads = [0] * world
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (loads[q], q))
        owner[i] = r
        loads[r] += costs[i]
    return owner, loads


def windows_of(owner, rank):
    """Indices of the windows rank ``rank`` runs, in window order."""
    return [i for i, r in enumerate(owner) if r == rank]


def max_over_ranks(x, device=None):
    """The largest ``x`` over all ranks (``x`` itself without a process
    group). ``device``: where the reduction tensor lives (the rank's GPU
    under NCCL, the CPU under gloo)."""
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_to_root(local, group=None):
    """Merge per-rank dicts {window index: result} on rank 0 (None on the
    other ranks). ``group`` should be a gloo group: results travel through
    host memory, never through a data-path collective."""
    if not (dist.is_available() and dist.is_initialized()):
        return dict(local)
    rank = dist.get_rank()
    world = dist.get_world_size(group)
    parts = [None] * world if rank == 0 else None
    dist.gather_object(dict(local), parts, dst=0, group=group)
    if rank != 0:
        return None
    merged = {}
    for p in parts:
        dup = merged.keys() & p.keys()
        if dup:
            raise RuntimeError(f"windows {sorted(dup)} were run by two ranks")
        merged.update(p)
    return merged
