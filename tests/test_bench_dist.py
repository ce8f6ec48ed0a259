"""The multi-GPU form of bench.py is replicas: each rank stitches its own
frames on the GPU of its local rank, the job time is the slowest rank's, and
no collective touches the data path.  Checked here with two gloo ranks on
CPU, running bench.measure_replica (the headline measurement) with the
render replaced by a host stub."""
import os
import socket
import sys
import time

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


class StubReplica:
    """A replica whose steps take a fixed host time per frame (rank 1 is the slower one)."""

    frames_per_step = 8
    canvas_px = 4096 * 2048

    def __init__(self, local):
        self.device = bench.rank_device(local, use_cuda=False)
        self.local = local
        self.steps_run = []

    def run(self, steps):
        self.steps_run.append(steps)
        per_frame_ms = 1.0 + 0.5 * self.local
        time.sleep(steps * self.frames_per_step * per_frame_ms / 1e3)
        return steps * self.frames_per_step * per_frame_ms


class Args:
    steps, warmup = 10, 3


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    w, r, local = bench.dist_env()
    d = bench.dist_init(w, use_cuda=False)
    rep = StubReplica(local)
    m = bench.measure_replica(rep, Args, w, d)
    q.put((r, local, rep.device, rep.steps_run, m["ms"], m["ms_max"], m["value"]))
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
    # each rank ran its warm-up then its timed steps, on its own device
    assert [r[3] for r in res] == [[3, 10], [3, 10]]
    assert [r[1] for r in res] == [0, 1]
    assert [r[4] for r in res] == [80.0, 120.0]
    # both ranks report the slowest rank's time
    assert [r[5] for r in res] == [120.0, 120.0]
    # 2 ranks x 10 steps x 8 canvases of 8.39 Mpx in 120 ms
    assert res[0][6] == pytest.approx(2 * 10 * 8 * 4096 * 2048 / 0.120 / 1e6)


def test_rank_to_device():
    assert bench.rank_device(3, use_cuda=True) == "cuda:3"
    assert bench.rank_device(3, use_cuda=False) == "cpu"


def test_single_process_needs_no_group():
    assert bench.dist_init(1, use_cuda=False) is None
    assert bench.reduce_max(3.5, None) == 3.5


def test_gpus_relaunches_under_torchrun():
    cmd = bench.relaunch_cmd(["--gpus", "4", "--steps", "5"], 4, 29555)
    assert cmd[:3] == [sys.executable, "-m", "torch.distributed.run"]
    assert "--nproc-per-node=4" in cmd and "127.0.0.1" in cmd and "29555" in cmd
    assert cmd[-4:] == ["--gpus", "4", "--steps", "5"]
    assert cmd[-5].endswith("bench.py")


def test_gpus_must_match_world_size(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("LOCAL_RANK", "0")
    assert bench.main(["--gpus", "4"]) == 2
    assert "WORLD_SIZE 2" in capsys.readouterr().out
