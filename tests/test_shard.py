"""Windows over ranks (vardyn_gb300/shard.py): the greedy split, and two
gloo ranks on the CPU running their share of the windows with the oracle's
model, timed by the slowest rank and gathered on rank 0 through the host."""
import itertools
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from vardyn_gb300.shard import assign, gather_to_root, max_over_ranks, window_cost, windows_of

SIZES = [(16, 20, 6), (24, 24, 3), (16, 16, 9), (20, 28, 4), (18, 18, 2), (24, 20, 5), (16, 24, 7)]


def test_assign_covers_every_window_once_and_is_deterministic():
    costs = [window_cost(*s) for s in SIZES]
    owner, loads = assign(costs, 3)
    assert sorted(itertools.chain.from_iterable(windows_of(owner, r) for r in range(3))) == list(range(len(SIZES)))
    assert loads == [sum(c for c, o in zip(costs, owner) if o == r) for r in range(3)]
    assert assign(costs, 3) == (owner, loads)


def test_assign_is_within_the_greedy_bound_of_the_best_split():
    rng = np.random.default_rng(0)
    for _ in range(30):
        costs = [int(c) for c in rng.integers(1, 50, size=7)]
        for world in (2, 3):
            _, loads = assign(costs, world)
            best = min(max(sum(c for c, o in zip(costs, split) if o == r) for r in range(world))
                       for split in itertools.product(range(world), repeat=len(costs)))
            assert max(loads) <= (4 / 3 - 1 / (3 * world)) * best + 1e-9


def test_assign_edge_cases():
    assert assign([], 2) == ([], [0, 0])
    assert assign([5, 5], 4) == ([0, 1], [5, 5, 0, 0])        # ties go to the lower rank
    assert assign([3, 3, 3], 1) == ([0, 0, 0], [9])
    with pytest.raises(ValueError):
        assign([1], 0)
    with pytest.raises(ValueError):
        assign([-1], 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_window(k):
    from oracle.qg1l import QgmOracle
    ny, nx, nstep = SIZES[k]
    rng = np.random.default_rng(100 + k)
    h0 = 0.05 * rng.standard_normal((ny, nx))
    m = QgmOracle(dx=np.full((ny, nx), 1e4), dy=np.full((ny, nx), 1e4), dt=600.0, SSH=h0, c=2.7,
                  time_scheme="rk2")
    return m.step(h0, np.zeros((ny, nx)), nstep)


def _worker(rank, world, port, out, mode):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        owner, _ = assign([window_cost(*s) for s in SIZES], world)
        mine = windows_of(owner, rank)
        if mode == "duplicate":
            mine = sorted(set(mine) | {0})
        local = {k: _run_window(k) for k in mine}
        slowest = max_over_ranks(float(len(mine) + rank))   # stands in for a timed region
        merged = gather_to_root(local)
        if rank == 0:
            np.savez(out, slowest=slowest, n=len(merged), **{f"w{k}": v for k, v in merged.items()})
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_process(tmp_path):
    out = str(tmp_path / "merged.npz")
    mp.spawn(_worker, args=(2, _free_port(), out, "normal"), nprocs=2, join=True)
    got = np.load(out)
    owner, _ = assign([window_cost(*s) for s in SIZES], 2)
    assert int(got["n"]) == len(SIZES)
    assert float(got["slowest"]) == max(len(windows_of(owner, r)) + r for r in range(2))
    for k in range(len(SIZES)):
        assert np.array_equal(got[f"w{k}"], _run_window(k), equal_nan=True)


def test_a_window_run_by_two_ranks_is_reported(tmp_path):
    out = str(tmp_path / "merged.npz")
    with pytest.raises(Exception, match="run by two ranks"):
        mp.spawn(_worker, args=(2, _free_port(), out, "duplicate"), nprocs=2, join=True)
    assert not os.path.exists(out)


def test_helpers_without_a_process_group():
    assert max_over_ranks(2.5) == 2.5
    assert gather_to_root({3: "x"}) == {3: "x"}


def test_mixed_workload_split_keeps_the_window_set():
    """bench.py's 64-window mixed workload: one rank holds every window with
    ordinals 0..count-1 per side; over 2 or 4 ranks the shares are disjoint,
    cover the same set, and the busiest rank holds at most 4/3 of the best
    split's work (the greedy bound)."""
    import bench
    nstep = 960
    one = bench.mixed_windows(nstep)
    assert sum(len(k) for k in one.values()) == bench.M4_WINDOWS
    assert all(k == list(range(len(k))) for k in one.values())
    total = sum(n * n * nstep * len(k) for n, k in one.items())
    for world in (2, 4):
        parts = [bench.mixed_windows(nstep, r, world) for r in range(world)]
        merged = {}
        for p in parts:
            for n, k in p.items():
                assert not set(merged.get(n, [])) & set(k)
                merged.setdefault(n, []).extend(k)
        assert {n: sorted(k) for n, k in merged.items()} == one
        loads = [sum(n * n * nstep * len(k) for n, k in p.items()) for p in parts]
        assert max(loads) <= (4 / 3) * max(total / world, max(n * n * nstep for n in one))
