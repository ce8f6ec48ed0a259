"""The multi-GPU form of bench.py is replicas: each rank stitches its own
frames, the job time is the slowest rank's, and no collective touches the
data path.  Checked here with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    d = bench.dist_init(world, use_cuda=False)
    local_ms = 100.0 + 50.0 * rank          # rank 1 is the slower replica
    ms_max = bench.reduce_max(local_ms, d)
    bench.barrier(d)
    q.put((rank, ms_max, bench.aggregate_mpix(world, 10, 4096 * 2048, ms_max)))
    d.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [150.0, 150.0]
    # 2 ranks x 10 canvases of 8.39 Mpx in 150 ms
    assert res[0][2] == pytest.approx(2 * 10 * 4096 * 2048 / 0.150 / 1e6)


def test_single_process_needs_no_group():
    assert bench.dist_init(1, use_cuda=False) is None
    assert bench.reduce_max(3.5, None) == 3.5
