"""CPU tests of bench.py's multi-rank host logic (no GPU): two gloo ranks combine the timed
region (max) and the processed units (sum) like the NCCL ranks of a multi-GPU run; every rank
solves its own slice of the volume sequence; the reference arm runs on rank 0 only."""
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
