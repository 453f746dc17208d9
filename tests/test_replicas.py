"""Multi-GPU is replicas only (one condensate per rank, no data-path
collective); the whole-job rate is the units of all ranks over the slowest
rank's time.  Checked with world_size 2 on the gloo backend, on CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(ws),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    import bench
    w, r, _ = bench.dist_setup()
    assert (w, r) == (ws, rank)
    bench.barrier(w)
    # rank 1 is the slow one: 2 s for 100 units; rank 0 1 s for 100 units
    rate = bench.whole_job_rate(w, 100, 1.0 + rank)
    slowest = bench.max_over_ranks(w, 1.0 + rank)
    out[rank] = (rate, slowest)
    dist.destroy_process_group()


def test_replica_rate_is_sum_over_slowest_rank():
    ws = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()  # no fork of this multi-threaded process
    out = mgr.dict()
    mp.spawn(_worker, args=(ws, port, out), nprocs=ws, join=True)
    for rank in range(ws):
        rate, slowest = out[rank]
        assert slowest == pytest.approx(2.0)
        assert rate == pytest.approx(100.0)  # 2 ranks x 100 units / 2 s
