"""Multi-GPU bookkeeping of bench.py on CPU: two gloo ranks stand in for two
GPUs.  The bench runs one independent replica per rank (its own seeded pair
list, no collective on the data path); the only cross-rank steps are a barrier
around the timed region and the max over ranks of the elapsed time, from which
rank 0 reports the whole job's rate (all ranks' pairs over the slowest rank's
time).  The reference arm runs on rank 0 alone.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "codim-ipc_gb300")]
    import bench
    import workloads
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        # each replica's workload is seeded by its rank
        w = workloads.contact_pairs(1000, seed=rank)
        local_s = 0.5 + rank  # rank 1 is the slower replica
        dist.barrier()
        slowest = bench.max_over_ranks(local_s, "cpu")
        rate = bench.whole_job_mpairs(slowest, w["type"].shape[0], 4, ws)
        out[rank] = (slowest, rate, float(w["x"][:10].sum()))
        # the reference arm: ranks other than 0 return at once, printing nothing
        if rank != 0:
            bench.run_reference(None)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_max_over_ranks():
    ws = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    assert set(res) == {0, 1}
    for r in range(ws):
        slowest, rate, _ = res[r]
        assert slowest == 1.5
        assert np.isclose(rate, 1000 * ws * 4 / 1.5 / 1e6)
    assert res[0][2] != res[1][2]  # different seeded workloads per replica
