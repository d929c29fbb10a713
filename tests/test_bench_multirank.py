"""The benchmark's multi-rank logic on CPU with gloo, world size 2: the barrier, the
max-over-ranks timing reduction, and the per-rank batches (independent instances, no
exchange between ranks)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    import __graft_entry__ as ge
    P = ge.load_package().problems
    bench._barrier(ws)
    got = bench._max_over_ranks(1.5 + rank, ws)
    params, nint, tsp, y0 = bench.rank_batch(P, 64, rank)
    out[rank] = (got, float(params[:, 0].sum()), int(nint.sum()), bench._dist())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ws = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        os.environ["WORLD_SIZE"] = str(ws)
        try:
            mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        finally:
            os.environ.pop("WORLD_SIZE", None)
            os.environ.pop("RANK", None)
        res = dict(out)
    assert sorted(res) == [0, 1]
    assert res[0][0] == res[1][0] == 2.5            # max over ranks, seen by both
    assert res[0][1] != res[1][1]                   # different instances per rank
    assert res[0][3] == (2, 0) and res[1][3] == (2, 1)
