"""CPU tests of bench.py's multi-rank host logic (no GPU): two gloo ranks combine the timed
region (max) and the processed units (sum) like the NCCL ranks of a multi-GPU run; every rank
solves its own slice of the volume sequence; the reference arm runs on rank 0 only; a run
with --gpus N > 1 and no torchrun launches its own ranks, and a WORLD_SIZE that disagrees
with --gpus is refused."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, units = bench.combine_ranks(10.0 + 5.0 * rank, 1000.0 * (rank + 1), world)
        out[rank] = (ms, units)
    finally:
        dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    world = 2
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    # both ranks see the slowest rank's time and the units of all ranks
    assert res[0] == res[1] == (15.0, 3000.0)


def test_combine_ranks_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.combine_ranks(12.5, 77.0, 1) == (12.5, 77.0)


def test_rank_slices_are_disjoint_and_rank0_is_unchanged():
    from taufactor_gb300.synthetic import batch_256

    whole = batch_256(4, 12, 2.0, first=0)
    r0 = batch_256(2, 12, 2.0, first=0)
    r1 = batch_256(2, 12, 2.0, first=2)
    assert np.array_equal(np.concatenate([r0, r1]), whole)
    assert not np.array_equal(r0, r1)


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")

    class Args:
        gpus, steps, warmup = 2, 1, 0

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(Args())
    assert buf.getvalue() == ""


def _partition_target(out):
    """A rank of a self-launched run: the slice bench.run_ours solves, gathered over gloo."""
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo")
    try:
        rank, world = dist.get_rank(), dist.get_world_size()
        assert int(os.environ["LOCAL_RANK"]) == rank and os.environ["MASTER_ADDR"] == "127.0.0.1"
        mine = torch.tensor(list(bench.rank_volumes(rank, 3)), dtype=torch.int64)
        got = [torch.empty_like(mine) for _ in range(world)]
        dist.all_gather(got, mine)
        out[rank] = [g.tolist() for g in got]
    finally:
        dist.destroy_process_group()


def test_self_launched_ranks_partition_the_volumes():
    sys.path.insert(0, ROOT)
    import bench

    with mp.Manager() as mgr:
        out = mgr.dict()
        bench.spawn_ranks(3, _partition_target, out)
        res = dict(out)
    assert sorted(res) == [0, 1, 2]
    sets = res[0]
    assert res[1] == res[2] == sets  # every rank sees the same partition
    flat = [i for part in sets for i in part]
    assert sorted(flat) == list(range(9)) and len(set(flat)) == 9  # disjoint, nothing left out
    assert sets[0] == [0, 1, 2]  # rank 0 solves the single-GPU workload


def test_world_size_must_match_gpus():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.check_world(1, {}) is False
    assert bench.check_world(4, {}) is True  # no torchrun: bench launches its 4 ranks itself
    assert bench.check_world(4, {"WORLD_SIZE": "4"}) is False  # torchrun did
    import pytest

    with pytest.raises(SystemExit):
        bench.check_world(8, {"WORLD_SIZE": "2"})


def test_volume_split_across_devices_is_balanced_and_complete():
    from taufactor_gb300.batch import split_volumes
    from taufactor_gb300.synthetic import _uneven_draws

    shapes, _ = _uneven_draws(64, (64, 96, 128, 192, 256))
    sizes = [int(np.prod(s)) for s in shapes]
    for n in (1, 2, 3, 8):
        parts = split_volumes(sizes, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        loads = [sum(sizes[i] for i in p) for p in parts]
        # greedy largest-first: no part exceeds the mean by more than the largest volume
        assert max(loads) - sum(sizes) / n <= max(sizes)
