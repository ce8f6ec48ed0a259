#!/usr/bin/env python
"""Benchmark of the panorama stitch path on GB300.

Headline: stitched output Mpix/s of the plain per-frame path on the
6-camera rig (6 x 1920x1080 rectilinear, 100 deg -> 4096x2048 equirect,
8-level multiband blend, per-camera LUT gains), frames resident in HBM,
issued in turn on eight streams so eight frames are in flight (the
single-stream figure is reported beside it).  A step is one frame on each
of the eight streams: eight stitched frames.
The same line carries:
  e2e         the same metric through the C ABI with pinned host frames in
              and the host canvas out (H2D + D2H inside the timed region),
              beside its host-link bound (a copy-only loop of the same bytes);
  e2e_nv12 / e2e_planar  the same with NV12 host planes out, and with NV12
              decoder frames in as well (1.5 bytes per source pixel);
  roofline    the dominant kernel's algorithmic GB/s against the measured
              HBM copy bandwidth (CUDA events around every launch of a
              profiled pass over the same workload), and its DRAM bytes per
              launch from the committed ncu summary of the workload;
  launch_shape  the launch shape the autotuner chose after prepare (untimed)
              and its ms per frame against the default shape's;
  linear_blend  the linear-blend render mode (highQualityBlend 0) on the same rig;
  batched     four rigs of uneven size per launch sequence (CUDA graph);
  serve       16 live streams over those rigs, Poisson 30 fps arrivals,
              continuous batching: p50 / p99 frame latency and Mpix/s;
  cpu_baseline  the CPU restatement of the reference path on the host cores.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                  [--workload c2|c5] [--scale K (profiler captures)]

Under torchrun each rank stitches its own replica on its own GPU (weak
scaling, no collective on the data path); rank 0 prints one JSON line.
`--gpus N` without torchrun relaunches the script under torchrun with N
ranks; under torchrun, N must equal WORLD_SIZE.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "stitched output Mpix/s at 4096x2048 (6 cams); p50/p99 frame latency in serve loop"
METRICS = {"c2": METRIC, "c5": "stitched output Mpix/s at 7680x3840 (8 cams)"}
WORKLOADS = {
    "c2": "6x rectilinear 1920x1080 (100 deg hfov; yaw 0/90/180/270, pitch +-90) -> 4096x2048 equirect, "
          "8-level integer multiband blend, per-camera per-channel LUT gains U[0.8,1.2]",
    "c5": "8x rectilinear 3840x2160 (120 deg hfov; yaw every 45 deg) -> 7680x3840 equirect, 10-level integer "
          "multiband blend, per-camera per-channel LUT gains U[0.7,1.3], noise +-20",
}
WORKLOAD = WORKLOADS["c2"]


# ----------------------------------------------------------------------------- distributed
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world, use_cuda):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("nccl" if use_cuda else "gloo")
    return dist


def rank_device(local: int, use_cuda: bool) -> str:
    """The device a replica runs on: the GPU of its local rank."""
    return f"cuda:{local}" if use_cuda else "cpu"


def relaunch_cmd(argv, gpus: int, port: int):
    """torchrun command that runs this script with `gpus` ranks (one per GPU) and the same arguments."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
            "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + list(argv)


def measure_replica(replica, args, world: int, dist=None, device=None) -> dict:
    """The headline measurement of one rank: W untimed warm-up steps, a barrier, K timed steps, then the
    slowest rank's time and the whole job's Mpix/s (every rank stitched K steps of its own frames)."""
    replica.run(args.warmup)
    barrier(dist)
    ms = replica.run(args.steps)
    ms_max = reduce_max(ms, dist, device)
    barrier(dist)
    return {"ms": ms, "ms_max": ms_max,
            "value": aggregate_mpix(world, args.steps * replica.frames_per_step, replica.canvas_px, ms_max)}


def reduce_max(value: float, dist=None, device=None) -> float:
    """Max of a float over all ranks (identity without a process group)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_mpix(world: int, steps: int, canvas_px: int, ms_max: float) -> float:
    """Whole-job Mpix/s: every rank stitched `steps` canvases; the slowest rank's time counts."""
    return world * steps * canvas_px / (ms_max / 1e3) / 1e6


def barrier(dist=None):
    if dist is not None:
        dist.barrier()


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        loaded = [r[0] for r in rows if r[2] > 200.0] or [r[0] for r in rows]
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "power_w_max": max(r[2] for r in rows)}


# ----------------------------------------------------------------------------- helpers
def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


NCU_TRAFFIC = {"c2": "ncu_traffic.txt", "c5": "ncu_traffic_c5.txt"}


def ncu_traffic(kernel: str, workload: str, alg_bytes_per_launch: float):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary of the workload, if any.  A line
    `kernel bytes` was captured on the workload itself; a line `kernel bytes alg_bytes` on a scaled-down
    copy of it (the full one holds too much device memory for a capture), and is scaled to a full launch by
    the algorithmic bytes, which the kernel's traffic follows."""
    name = NCU_TRAFFIC.get(workload)
    path = os.path.join(ROOT, "profiles", name) if name else None
    if not path or not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel and not line.startswith("#"):
            try:
                nbytes = float(parts[1])
                return nbytes if len(parts) < 3 else round(nbytes * alg_bytes_per_launch / float(parts[2]))
            except (ValueError, ZeroDivisionError):
                return None
    return None


def workload_rig(args):
    """The workload's rig, divided by --scale for profiler captures."""
    from panostitcher_gb300 import synth as S
    cfg = S.rig(args.workload)
    return S.scaled_rig(cfg, args.scale) if args.scale > 1 else cfg


def pinned_copy(a: np.ndarray):
    import torch
    t = torch.empty(a.shape, dtype=torch.uint8, pin_memory=True)
    arr = t.numpy()
    arr[...] = a
    return arr, t


def link_bound(h2d_srcs, d2h_dsts, steps, dev):
    """Seconds for `steps` copy-only steps over the host link: per step the
    bytes an e2e render moves (every camera frame up, the outputs down), the
    uploads and the downloads on two streams."""
    import torch
    up = [torch.empty(t.shape, dtype=t.dtype, device=dev) for t in h2d_srcs[0]]
    down = [torch.empty(t.shape, dtype=t.dtype, device=dev) for t in d2h_dsts]
    s_up, s_down = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)

    def go(n):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for k in range(n):
            with torch.cuda.stream(s_up):
                for d, h in zip(up, h2d_srcs[k % len(h2d_srcs)]):
                    d.copy_(h, non_blocking=True)
            with torch.cuda.stream(s_down):
                for h, d in zip(d2h_dsts, down):
                    h.copy_(d, non_blocking=True)
        torch.cuda.synchronize()
        return time.perf_counter() - t

    go(3)
    return go(steps)


def link_fields(e2e, secs, frames, npx, frames_per_step):
    """The e2e line's host-link bound: the copy-only rate of the same bytes (`frames` frames' worth)."""
    bound = frames * npx / secs / 1e6
    steps = frames / frames_per_step
    return {"value": round(bound, 3), "unit": "Mpix/s",
            "h2d_gbs": round(steps * e2e["h2d_bytes_per_step"] / secs / 1e9, 1),
            "d2h_gbs": round(steps * e2e["d2h_bytes_per_step"] / secs / 1e9, 1),
            "frac": round(e2e["value"] / bound, 4),
            "how": "copy-only loop of the same pinned buffers: frames up and outputs down on two streams"}


# ----------------------------------------------------------------------------- our arm
def workload_config(args, cfg, levels, frames_per_step, l2, parallelism):
    """The `config` of both arms' lines: the same keys, the workload named by what it is."""
    W, H = cfg.dst_size
    c = {"workload": WORKLOADS[args.workload], "canvas": [W, H], "cams": cfg.num_cams, "src": list(cfg.src_size),
         "levels": levels, "frames_per_step": frames_per_step, "l2": l2, "parallelism": parallelism}
    if args.scale > 1:
        c["workload"] += f"; every size divided by {args.scale}"
    return c


def l2_note(pool, frame_mb):
    return f"inputs larger than L2: {pool} distinct {frame_mb:.1f} MB frames cycled"


class CudaReplica:
    """One rank's render on its own GPU: the rig prepared, a pool of frames in HBM, and a timed loop that
    issues each step's frames in turn on `inflight` streams (one frame per stream per step), so up to
    that many frames are in flight (the render keeps eight state slots)."""

    def __init__(self, args, local):
        import torch
        import panostitcher_gb300 as P
        from panostitcher_gb300 import synth as S
        torch.cuda.set_device(local)
        self.torch = torch
        self.dev = torch.device(rank_device(local, True))
        self.cfg = cfg = workload_rig(args)
        W, H = cfg.dst_size
        self.canvas_px = W * H
        self.args = args
        self.r = r = P.CudaPanoramaRender2()
        t = time.perf_counter()
        r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
        self.prepare_s = time.perf_counter() - t
        # launch-shape autotuning (untimed, like prepare): frames issued the way
        # the timed loop issues them
        self.tune = None
        if not args.no_tune:
            t = time.perf_counter()
            self.tune = r.autotune(frames_per_trial=20, in_flight=min(args.inflight, 8))
            self.tune["seconds"] = round(time.perf_counter() - t, 2)
        fs = S.FrameSource(cfg)
        self.pool_host = [fs.frame(k) for k in range(args.pool)]
        self.pool_dev = [[torch.from_numpy(f).to(self.dev) for f in fr] for fr in self.pool_host]
        self.luts = S.luts(cfg)
        self.streams = [torch.cuda.Stream(device=self.dev) for _ in range(args.inflight)]
        self.dsts = [torch.empty((H, W, 4), dtype=torch.uint8, device=self.dev) for _ in range(args.inflight)]
        self.frames_per_step = args.inflight

    def frames(self, nframes, nstreams):
        """ms of device time for `nframes` frames issued round-robin on `nstreams` streams."""
        torch = self.torch
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ends = [torch.cuda.Event() for _ in range(nstreams)]
        torch.cuda.synchronize()
        e0.record()
        for st in self.streams[:nstreams]:
            st.wait_event(e0)
        for k in range(nframes):
            q = k % nstreams
            self.r.render(self.pool_dev[k % self.args.pool], self.dsts[q], self.luts, stream=self.streams[q],
                          check=True)
        cur = torch.cuda.current_stream()
        for q in range(nstreams):
            ends[q].record(self.streams[q])
            cur.wait_event(ends[q])
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def run(self, steps):
        return self.frames(steps * self.frames_per_step, self.frames_per_step)


def run_ours(args, world, rank, local, dist):
    import torch
    import panostitcher_gb300 as P
    from panostitcher_gb300 import build as B

    B.build()
    rep = CudaReplica(args, local)
    r, cfg, dev = rep.r, rep.cfg, rep.dev
    W, H = cfg.dst_size
    npx = W * H
    fps = rep.frames_per_step
    pool_host, pool_dev, luts, dst = rep.pool_host, rep.pool_dev, rep.luts, rep.dsts[0]
    tune = rep.tune
    sampler = ClockSampler(local)
    sampler.start()
    m = measure_replica(rep, args, world, dist, dev)
    clocks = sampler.stop()
    ms_max = m["ms_max"]
    # one frame at a time, with the launch shape tuned for that (cached after
    # the first call), then the in-flight shape again for the legs below
    single_frames = max(10, args.steps)
    single_shape = r.launch_shape()
    if not args.no_tune:
        single_shape = r.autotune(frames_per_trial=20, in_flight=1)["shape"]
    rep.frames(args.warmup, 1)
    single_ms = rep.frames(single_frames, 1) / single_frames
    if not args.no_tune:
        r.autotune(frames_per_trial=20, in_flight=min(args.inflight, 8))
    value = m["value"]
    out = {"metric": METRICS[args.workload], "value": round(value, 3), "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 5), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u8/i32",
           "data": f"synthetic: seeded smooth field + per-frame noise, pool of {args.pool} frames in HBM",
           "gpu_launches": args.steps * fps * r.launches_per_frame,
           "frames_per_step": fps, "ms_per_frame": round(ms_max / (args.steps * fps), 5),
           "single_stream": {"value": round(npx / single_ms / 1e3, 3), "ms_per_frame": round(single_ms, 5),
                             "frames": single_frames, "launch_shape": single_shape},
           "clocks": clocks}
    resident = r.resident_bytes
    frame_mb = sum(f.nbytes for f in pool_host[0]) / 1e6
    out["config"] = workload_config(args, cfg, r.num_levels, fps, l2_note(args.pool, frame_mb), f"replicas x{world}")
    out["setup"] = {"prepare_s": round(rep.prepare_s, 3), "full_mask": r.full_mask,
                    "resident_mb": round(resident / 1e6)}
    out["launch_shape"] = tune if tune is not None else {"shape": r.launch_shape(), "tuned": False}

    # ---- e2e: pinned host frames in, host canvas out, through the C ABI
    pinned, pinned_t = [], []
    for fr in pool_host:
        cams, cams_t = [], []
        for f in fr:
            a, tt = pinned_copy(f)
            cams.append(a)
            cams_t.append(tt)
        pinned.append(cams)
        pinned_t.append(cams_t)
    hdst, hdst_t = pinned_copy(np.zeros((H, W, 4), np.uint8))
    e2e_steps = args.e2e_steps or args.steps
    e2e_frames = e2e_steps * fps  # a step is fps frames, as in the device-resident loop
    for k in range(max(2, args.warmup)):
        r.render(pinned[k % args.pool], hdst, luts, check=True)
    torch.cuda.synchronize()
    barrier(dist)
    t = time.perf_counter()
    for k in range(e2e_frames):
        r.render(pinned[k % args.pool], hdst, luts, check=True)
    torch.cuda.synchronize()
    e2e_s = reduce_max(time.perf_counter() - t, dist, dev)
    out["e2e"] = {"value": round(world * e2e_frames * npx / e2e_s / 1e6, 3), "unit": "Mpix/s",
                  "h2d_bytes_per_step": int(fps * sum(f.nbytes for f in pinned[0])),
                  "d2h_bytes_per_step": int(fps * hdst.nbytes), "steps": e2e_steps, "frames_per_step": fps,
                  "path": "ps_render_render, pinned BGR32 host frames -> pinned BGR32 host canvas"}
    out["e2e"]["link_bound"] = link_fields(out["e2e"], link_bound(pinned_t, [hdst_t], e2e_frames, dev), e2e_frames,
                                           npx, fps)

    # ---- e2e with the encoder handoff: NV12 planes downloaded (the Task layer's render + cvt + download)
    hy, hy_t = pinned_copy(np.zeros((H, W), np.uint8))
    huv, huv_t = pinned_copy(np.zeros((H // 2, W), np.uint8))
    for k in range(2):
        r.render_yuv(pinned[k % args.pool], [hy, huv], luts, P.PS_FMT_NV12, check=True)
    torch.cuda.synchronize()
    barrier(dist)
    t = time.perf_counter()
    for k in range(e2e_frames):
        r.render_yuv(pinned[k % args.pool], [hy, huv], luts, P.PS_FMT_NV12, check=True)
    torch.cuda.synchronize()
    nv12_s = reduce_max(time.perf_counter() - t, dist, dev)
    out["e2e_nv12"] = {"value": round(world * e2e_frames * npx / nv12_s / 1e6, 3), "unit": "Mpix/s",
                       "h2d_bytes_per_step": int(fps * sum(f.nbytes for f in pinned[0])),
                       "d2h_bytes_per_step": int(fps * (hy.nbytes + huv.nbytes)), "steps": e2e_steps,
                       "frames_per_step": fps,
                       "path": "ps_render_render_yuv, pinned BGR32 host frames -> pinned NV12 host planes "
                               "(conversion fused into the level-0 blend)"}
    out["e2e_nv12"]["link_bound"] = link_fields(out["e2e_nv12"], link_bound(pinned_t, [hy_t, huv_t], e2e_frames, dev),
                                                e2e_frames, npx, fps)

    # ---- e2e of the whole handoff: NV12 decoder frames in, NV12 encoder planes
    # out.  The input planes are made from the BGR pool by the library's own
    # device conversion, then staged in pinned host memory.
    Ws, Hs = cfg.src_size
    nv12_t, nv12_h, nv12_dev = [], [], []
    for fr in pool_dev:
        cams_t, cams_h, cams_d = [], [], []
        for f in fr:
            y = torch.empty((Hs, Ws), dtype=torch.uint8, device=dev)
            uv = torch.empty((Hs // 2, Ws), dtype=torch.uint8, device=dev)
            P.cvt_bgr32_to_yuv(f, [y, uv], P.PS_FMT_NV12)
            ha, ht = pinned_copy(y.cpu().numpy())
            ua, ut = pinned_copy(uv.cpu().numpy())
            cams_t += [ht, ut]
            cams_h.append([ha, ua])
            cams_d.append([y, uv])
        nv12_t.append(cams_t)
        nv12_h.append(cams_h)
        nv12_dev.append(cams_d)
    for k in range(2):
        r.render_planar(nv12_h[k % args.pool], luts=luts, ydst=[hy, huv], check=True)
    torch.cuda.synchronize()
    barrier(dist)
    t = time.perf_counter()
    for k in range(e2e_frames):
        r.render_planar(nv12_h[k % args.pool], luts=luts, ydst=[hy, huv], check=True)
    torch.cuda.synchronize()
    pl_s = reduce_max(time.perf_counter() - t, dist, dev)
    out["e2e_planar"] = {"value": round(world * e2e_frames * npx / pl_s / 1e6, 3), "unit": "Mpix/s",
                         "h2d_bytes_per_step": int(fps * sum(x.nbytes for x in nv12_t[0])),
                         "d2h_bytes_per_step": int(fps * (hy.nbytes + huv.nbytes)), "steps": e2e_steps,
                         "frames_per_step": fps,
                         "path": "ps_render_render_planar, pinned NV12 host frames -> pinned NV12 host planes "
                                 "(decoder frames converted on the device, encoder conversion fused into the "
                                 "level-0 blend)"}
    out["e2e_planar"]["link_bound"] = link_fields(out["e2e_planar"],
                                                  link_bound([nv12_t[k] for k in range(args.pool)], [hy_t, huv_t],
                                                             e2e_frames, dev), e2e_frames, npx, fps)
    # the conversion kernel alone (device planes, profiled pass)
    r.profile(True)
    for k in range(10):
        r.render_planar(nv12_dev[k % args.pool], dst, luts, check=True)
    torch.cuda.synchronize()
    n5, ms5, b5 = r.profile_read(5)
    r.profile(False)
    out["e2e_planar"]["k_yuv_to_bgr32"] = {"us_per_frame": round(ms5 / max(n5, 1) * 1e3, 2),
                                           "alg_GBps": round(b5 / max(ms5, 1e-9) / 1e6, 1)}

    # ---- roofline: profiled pass (a CUDA event pair around every launch).
    # Launches are timed one at a time with the default launch shape (full
    # one-wave grids, the tail kernel for the top levels), as the committed
    # ncu summaries capture them.
    r.set_launch_shape(**P.CudaPanoramaRender2.SHAPE_DEFAULT)
    r.profile(True)
    prof_steps = min(args.steps, 30)
    for k in range(prof_steps):
        r.render(pool_dev[k % args.pool], dst, luts, check=True)
    torch.cuda.synchronize()
    kernels = {}
    total_ms = 0.0
    for kind, name in r.KERNELS.items():
        n, kms, kb = r.profile_read(kind)
        if n == 0:
            continue
        kernels[name] = {"launches_per_frame": n // prof_steps, "ms_per_frame": kms / prof_steps,
                         "alg_bytes_per_launch": kb / max(n, 1), "gbs": kb / max(kms, 1e-9) / 1e6}
        total_ms += kms
    by_level = {}
    for kind, name in r.KERNELS.items():
        if name not in kernels:
            continue
        lv = []
        for level in range(r.num_levels + 1):
            n, kms, kb = r.profile_read(kind, level)
            if n:
                lv.append([level, round(kms / prof_steps * 1e3, 2), round(kb / max(kms, 1e-9) / 1e6, 1)])
        by_level[name] = lv
    r.profile(False)
    for k in kernels.values():
        k["share"] = round(k["ms_per_frame"] * prof_steps / max(total_ms, 1e-9), 4)
    dom = max(kernels, key=lambda k: kernels[k]["ms_per_frame"])
    peak, peak_src = measured_peak()
    achieved = kernels[dom]["gbs"]
    # the committed ncu summaries cover the full-size workloads
    traffic = ncu_traffic(dom, args.workload, kernels[dom]["alg_bytes_per_launch"]) if args.scale == 1 else None
    out["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                       "peak_source": peak_src, "unit": "GB/s", "frac": round(achieved / peak, 4),
                       "traffic": traffic,
                       "alg_bytes_per_launch": round(kernels[dom]["alg_bytes_per_launch"]),
                       "frame_alg_bytes": round(r.algorithmic_bytes(4, 4)),
                       "frame_alg_gbs": round(r.algorithmic_bytes(4, 4) / (ms_max / (args.steps * fps)) / 1e6, 1)}
    out["kernels"] = {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                      for k, v in kernels.items()}
    out["kernels_by_level"] = {"columns": ["level", "us_per_frame", "alg_GBps"], **by_level}

    def guarded(fn, *a):
        try:
            return fn(*a)
        except Exception as e:  # an extra leg failing must not lose the headline line
            return {"error": f"{type(e).__name__}: {e}"}

    if world == 1 and not args.no_linear:
        out["linear_blend"] = guarded(run_linear, args, dev)
    if world == 1 and not args.no_batched and args.workload == "c2":
        out["batched"] = guarded(run_batched, args, dev)
    if world == 1 and not args.no_serve and args.workload == "c2":
        out["serve"] = guarded(run_serve, args, dev)
    if world == 1 and rank == 0 and not args.no_cpu:
        res = guarded(cpu_baseline, args, r, cfg, pool_host, luts)
        out["parity"] = res.pop("parity", None) if isinstance(res, dict) else None
        out["cpu_baseline"] = res
    return out


def run_linear(args, dev):
    """The linear-blend render mode on the same rig: weights feathered with a radius of 5% of the
    canvas width (as CudaPanoramaRender prepares them), fp32 weighted accumulation."""
    import torch
    import panostitcher_gb300 as P
    from panostitcher_gb300 import synth as S
    cfg = workload_rig(args)
    W, H = cfg.dst_size
    radius = int(W * 0.05)
    r = P.CudaPanoramaRender2()
    t = time.perf_counter()
    r.prepare(cfg.cams, 0, radius, cfg.src_size, cfg.dst_size, check=True)
    prep = time.perf_counter() - t
    fs = S.FrameSource(cfg)
    pool = [[torch.from_numpy(f).to(dev) for f in fs.frame(k)] for k in range(2)]
    luts = S.luts(cfg)
    dst = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
    for k in range(5):
        r.render(pool[k % 2], dst, luts, check=True)
    torch.cuda.synchronize()
    steps = max(10, args.steps // 2)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(steps):
        r.render(pool[k % 2], dst, luts, check=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"mpix_s": round(W * H / ms / 1e3, 1), "ms_per_frame": round(ms, 4), "radius": radius,
            "launches_per_frame": r.launches_per_frame, "prepare_s": round(prep, 3), "steps": steps,
            "frame_alg_gbs": round(r.algorithmic_bytes(4, 4) / ms / 1e6, 1)}


def run_batched(args, dev):
    """Four rigs of uneven size (c3a..c3d) in one launch sequence per tick, against the plain per-frame path
    on the same rigs.  Both forms run their CUDA graphs with the same number of ticks in flight: tick k goes
    out on stream k % inflight, with its own outputs; a plain tick is one render per rig on that stream."""
    import torch
    import panostitcher_gb300 as P
    from panostitcher_gb300 import synth as S
    names = ["c3a", "c3b", "c3c", "c3d"]
    cfgs = [S.rig(n) for n in names]
    nq = args.inflight
    renders, pools, luts = [], [], []
    for c in cfgs:
        r = P.CudaPanoramaRender2()
        r.prepare(c.cams, 1, c.levels, c.src_size, c.dst_size, check=True)
        renders.append(r)
        fs = S.FrameSource(c)
        pools.append([[torch.from_numpy(f).to(dev) for f in fs.frame(k)] for k in range(2)])
        luts.append(S.luts(c))
    dsts = [[torch.empty((c.dst_size[1], c.dst_size[0], 4), dtype=torch.uint8, device=dev) for c in cfgs]
            for _ in range(nq)]
    streams = [torch.cuda.Stream(device=dev) for _ in range(nq)]
    px = sum(c.canvas_pixels for c in cfgs)
    steps = max(20, args.steps)
    res = {"rigs": {n: f"{c.num_cams}x{c.src_size[0]}x{c.src_size[1]} -> {c.dst_size[0]}x{c.dst_size[1]}, "
                       f"{r.num_levels} levels" for n, c, r in zip(names, cfgs, renders)},
           "ticks": steps, "ticks_in_flight": nq}

    # each rig's launch shape tuned for this many ticks in flight (untimed), used by both forms
    res["launch_shapes"] = {}
    for n, r in zip(names, renders):
        if not args.no_tune:
            r.autotune(in_flight=nq)
        res["launch_shapes"][n] = r.launch_shape()

    def timed(tick, nticks):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for st in streams:
            st.wait_event(e0)
        for k in range(nticks):
            tick(k, streams[k % nq], dsts[k % nq])
        cur = torch.cuda.current_stream()
        for st in streams:
            cur.wait_stream(st)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def batched(k, st, ds):
        P.render_batch(renders, [p[k % 2] for p in pools], ds, luts, stream=st)

    def plain(k, st, ds):
        for r, p, lt, d in zip(renders, pools, luts, ds):
            r.render(p[k % 2], d, lt, stream=st, check=True)

    timed(batched, max(nq, args.warmup))
    bms = timed(batched, steps)
    timed(plain, max(nq, args.warmup))
    pms = timed(plain, steps)
    # the plain path one tick at a time (one stream), as a per-frame caller issues it, with the rigs'
    # shapes tuned for one frame at a time
    for r in renders:
        r.set_graph(True)
        if not args.no_tune:
            r.autotune(in_flight=1)
    timed(lambda k, st, ds: plain(k, streams[0], dsts[0]), 3)
    sms = timed(lambda k, st, ds: plain(k, streams[0], dsts[0]), steps)
    res.update({"mpix_s": round(steps * px / (bms / 1e3) / 1e6, 1),
                "plain_mpix_s": round(steps * px / (pms / 1e3) / 1e6, 1),
                "plain_one_stream_mpix_s": round(steps * px / (sms / 1e3) / 1e6, 1),
                "ms_per_tick": round(bms / steps, 4), "plain_ms_per_tick": round(pms / steps, 4),
                "speedup_vs_plain": round(pms / bms, 3),
                "speedup_vs_plain_one_stream": round(sms / bms, 3),
                "plain": "graph-captured renders, one per rig, same ticks in flight and launch shapes"})
    return res


def run_serve(args, dev, seconds=None):
    """16 live streams over the four batched rigs; Poisson 30 fps arrivals."""
    from panostitcher_gb300 import synth as S
    from panostitcher_gb300.serve import StitchServer
    seconds = seconds or args.serve_seconds
    names = ["c3a", "c3b", "c3c", "c3d"]
    cfgs = {n: S.rig(n) for n in names}
    rng = np.random.default_rng(2024)
    assign = [names[i] for i in rng.integers(0, 4, 16)]
    srv = StitchServer(int(120e9), max_batch=16)
    try:
        t = time.perf_counter()
        ids = [srv.admit(cfgs[n].cams, cfgs[n].levels, cfgs[n].src_size, cfgs[n].dst_size) for n in assign]
        admit_s = time.perf_counter() - t
        # one pool of two pinned frames per rig type, shared by its streams
        keep, frames = [], {}
        for n in names:
            fs = S.FrameSource(cfgs[n])
            frames[n] = []
            for k in range(2):
                cams = []
                for f in fs.frame(k):
                    a, tt = pinned_copy(f)
                    keep.append(tt)
                    cams.append(a)
                frames[n].append(cams)
        luts = {n: np.ascontiguousarray(S.luts(cfgs[n])) for n in names}
        events = []
        for n, sid in zip(assign, ids):
            if sid is None:
                continue
            t = rng.uniform(0, 1 / 30)
            k = 0
            while t < seconds:
                events.append((t, sid, n, k))
                t += rng.exponential(1 / 30)
                k += 1
        events.sort()
        lat, wall = srv.run_trace([e[1] for e in events], [e[0] for e in events],
                                  [frames[e[2]][e[3] % 2] for e in events], [luts[e[2]] for e in events], None)
        lat_ms = lat * 1e3
        px = sum(cfgs[e[2]].canvas_pixels for e in events)
        return {"streams": len(assign), "admitted": sum(i is not None for i in ids),
                "rigs": {n: assign.count(n) for n in names}, "frames": len(events), "seconds": seconds,
                "p50_ms": round(float(np.percentile(lat_ms, 50)), 3),
                "p99_ms": round(float(np.percentile(lat_ms, 99)), 3), "max_ms": round(float(lat_ms.max()), 3),
                "mpix_s": round(px / wall / 1e6, 1), "resident_gb": round(srv.resident_bytes / 1e9, 2),
                "budget_gb": 120, "admit_s": round(admit_s, 2),
                "arrivals": "Poisson 30 fps per stream, seeded offsets",
                "io": "pinned host frames uploaded per frame; outputs kept on the device"}
    finally:
        srv.close()


def cpu_baseline(args, r, cfg, pool_host, luts):
    """The oracle (CPU restatement of the reference path, pinned to the reference's own code) on the host
    cores, and the parity of the product against it on the same frames.

    The oracle does what the reference's CPU render does: it derives its maps, coverage and seams from
    the camera parameters (getReprojectMapsAndMasks at prepare, untimed), then per frame applies the
    LUTs, remaps and blends (timed).  Parity, from the same run:
      - geometry: map values whose float bits differ, coverage and seam pixels that differ, between the
        product's FP64 device geometry and the oracle's;
      - remap: the product's remap (ps_reproject_to_16s, the arithmetic of the render's k_remap) against
        the oracle's double-precision bilinear through the same maps, every camera of one frame: the
        histogram of per-channel differences;
      - output: the product's render against the oracle's render of the same frame, each from its own
        geometry: the histogram of per-channel differences;
      - secondary: the product's render against the reference's CPU render semantics
        (TilingMultibandBlendFast: x255 masked pyrDown, R >> 8 normalisation), which the reference's
        CPU and CUDA blends do not share: the histogram of per-channel differences.
    The timed value is the reference's CPU render (CPUPanoramaRender: LUT, bilinear remap, the CPU
    multiband blend) restated in the oracle and pinned bit for bit to the reference's own
    TilingMultibandBlendFast; the CudaAccel-semantics oracle is timed beside it.  Also times the CPU
    render on the 2-camera fisheye rig (2048x1024, 100 frames) and on the 8-camera 7680x3840 rig (a few
    frames)."""
    import torch
    import oracle as O
    import panostitcher_gb300 as P
    from panostitcher_gb300 import synth as S
    threads = os.cpu_count() or 1
    n = cfg.num_cams
    W, H = cfg.dst_size
    t = time.perf_counter()
    maps = [O.reproject_map(p, cfg.src_size, cfg.dst_size, threads=threads) for p in cfg.cams]
    cov = np.stack([m[2] for m in maps])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov, threads=threads)
    ob = O.Blender(cov, seams, cfg.levels)
    cb = O.CpuBlender(cov, seams, cfg.levels)
    geometry_s = time.perf_counter() - t
    xm, ym = [m[0] for m in maps], [m[1] for m in maps]

    def hist(a, b):
        d = a.astype(np.int32) - b.astype(np.int32)
        v, c = np.unique(d, return_counts=True)
        return {str(int(x)): int(y) for x, y in zip(v, c)}

    # ---- parity
    pmaps = [r.maps(i, cfg.dst_size) for i in range(n)]
    pcov = np.stack([r.coverage(i, cfg.dst_size) for i in range(n)])
    pseams = np.stack([r.seam(i, cfg.dst_size) for i in range(n)])
    map_diff = 0
    for i in range(n):
        both = (cov[i] > 0) & (pcov[i] > 0)
        map_diff += int((both & ((pmaps[i][0].view(np.uint32) != xm[i].view(np.uint32)) |
                                 (pmaps[i][1].view(np.uint32) != ym[i].view(np.uint32)))).sum())
    frame = pool_host[0]
    remap_hist = {}
    for i in range(n):
        dev_out = torch.empty((H, W, 4), dtype=torch.int16, device="cuda")
        P.reproject_to_16s(torch.from_numpy(frame[i]).cuda(), torch.from_numpy(pmaps[i][0]).cuda(),
                           torch.from_numpy(pmaps[i][1]).cuda(), dev_out,
                           torch.from_numpy(np.ascontiguousarray(luts[i].reshape(-1))).cuda())
        ref = O.reproject_16s(frame[i], pmaps[i][0], pmaps[i][1], luts[i])
        got = dev_out.cpu().numpy()
        for k, v in hist(got[..., :3][pcov[i] > 0], ref[..., :3][pcov[i] > 0]).items():
            remap_hist[k] = remap_hist.get(k, 0) + v
    got = np.zeros((H, W, 4), np.uint8)
    r.render(frame, got, luts, check=True)
    torch.cuda.synchronize()
    ref = ob.render(frame, luts, xm, ym, threads)
    cref = cb.render(frame, luts, xm, ym, threads)
    parity = {"rig": WORKLOADS[args.workload],
              "geometry": {"map_values_differing": map_diff,
                           "coverage_px_differing": int(((cov > 0) != (pcov > 0)).sum()),
                           "seam_px_differing": int(((seams > 0) != (pseams > 0)).sum()),
                           "covered_px": int((cov > 0).sum())},
              "remap_delta_histogram": remap_hist,
              "output_delta_histogram": hist(got[..., :3], ref[..., :3]),
              "cpu_semantics_delta_histogram": hist(got[..., :3], cref[..., :3]),
              "bar": "remap within +-1 LSB of the double-precision bilinear; output bit-exact given the same "
                     "geometry (tests/test_gpu_e2e_parity.py bounds the rest)",
              "oracle": "C restatement pinned bit for bit to the reference's Remap.cpp, ZReproject.cpp, "
                        "CudaPyramid2.cu, MultiBandBlend.cpp and Pyramid.cpp (built here from the reference "
                        "tree; tests/test_ref_pin.py)"}

    # ---- timing
    def timed(render):
        frames = 0
        t = time.perf_counter()
        while True:
            render(pool_host[frames % len(pool_host)], luts, xm, ym, threads)
            frames += 1
            el = time.perf_counter() - t
            if el >= args.cpu_seconds:
                return frames, el

    frames, el = timed(cb.render)
    cframes, cel = timed(ob.render)
    res = {"value": round(frames * W * H / el / 1e6, 4), "unit": "Mpix/s", "cores": threads, "kind": "port",
           "sample": f"{frames} full frames of the {cfg.num_cams}-camera {W}x{H} rig through the reference's "
                     f"CPU render (LUT + bilinear remap + TilingMultibandBlendFast) in {el:.1f} s; geometry "
                     f"from the camera parameters {geometry_s:.1f} s before, untimed",
           "cudaaccel_semantics": {"value": round(cframes * W * H / cel / 1e6, 4), "unit": "Mpix/s",
                                   "sample": f"{cframes} frames of the oracle of the product's own semantics "
                                             f"(CudaTilingMultibandBlendFast) in {cel:.1f} s"},
           "parity": parity}
    if args.scale == 1 and not args.no_cpu_rigs:
        res["other_rigs"] = {"c1": cpu_rig_timing("c1", 100, threads), "c5": cpu_rig_timing("c5", 8, threads)}
    return res


def cpu_rig_timing(name, nframes, threads):
    """The reference's CPU render (LUT + remap + TilingMultibandBlendFast, restated in the oracle) on
    another benchmark rig: nframes frames on the host cores."""
    import oracle as O
    from panostitcher_gb300 import synth as S
    cfg = S.rig(name)
    W, H = cfg.dst_size
    maps = [O.reproject_map(p, cfg.src_size, cfg.dst_size, threads=threads) for p in cfg.cams]
    cov = np.stack([m[2] for m in maps])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov, threads=threads)
    ob = O.CpuBlender(cov, seams, cfg.levels)
    fs = S.FrameSource(cfg)
    pool = [fs.frame(k) for k in range(2)]
    luts = S.luts(cfg)
    ob.render(pool[0], luts, [m[0] for m in maps], [m[1] for m in maps], threads)
    t = time.perf_counter()
    for k in range(nframes):
        ob.render(pool[k % 2], luts, [m[0] for m in maps], [m[1] for m in maps], threads)
    el = time.perf_counter() - t
    return {"value": round(nframes * W * H / el / 1e6, 4), "unit": "Mpix/s", "frames": nframes,
            "ms_per_frame": round(el / nframes * 1e3, 2), "cores": threads,
            "rig": f"{cfg.num_cams}x{cfg.src_size[0]}x{cfg.src_size[1]} -> {W}x{H}, {ob.levels} levels"}


# ----------------------------------------------------------------------------- reference arm
def run_reference(args, world, rank):
    """The reference's own CPU implementation of the path, CPUPanoramaRender::render (LUT, bilinear remap,
    TilingMultibandBlendFast), as the oracle restates it and pins bit for bit to the reference's own code,
    on all host cores: per step, the same frames_per_step frames of the same workload as our arm; the
    number of timed steps is bounded by --ref-seconds."""
    import oracle as O
    from panostitcher_gb300 import synth as S
    O.build()
    cfg = workload_rig(args)
    W, H = cfg.dst_size
    threads = os.cpu_count() or 1
    fps = args.inflight
    maps = [O.reproject_map(p, cfg.src_size, cfg.dst_size, threads=threads) for p in cfg.cams]
    cov = np.stack([m[2] for m in maps])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov, threads=threads)
    ob = O.CpuBlender(cov, seams, cfg.levels)
    fs = S.FrameSource(cfg)
    pool = [fs.frame(k) for k in range(args.pool)]
    luts = S.luts(cfg)
    xm, ym = [m[0] for m in maps], [m[1] for m in maps]

    def step(k):
        for f in range(fps):
            ob.render(pool[(k * fps + f) % args.pool], luts, xm, ym, threads)

    t = time.perf_counter()
    step(0)
    one = time.perf_counter() - t
    warm = min(args.warmup, 1)
    for k in range(warm - 1):
        step(k)
    steps = max(1, min(args.steps, int(args.ref_seconds / max(one, 1e-3))))
    t = time.perf_counter()
    for k in range(steps):
        step(k)
    el = time.perf_counter() - t
    value = steps * fps * W * H / el / 1e6
    frame_mb = sum(f.nbytes for f in pool[0]) / 1e6
    sample = f"{steps} of {args.steps} steps ({fps} full {cfg.num_cams}-camera {W}x{H} frames each through " \
             f"the reference's CPU render: LUT + bilinear remap + TilingMultibandBlendFast, {threads} threads), " \
             f"{warm} warm-up"
    return {"impl": "reference", "metric": METRICS[args.workload], "value": round(value, 4), "unit": "Mpix/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el / steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/i32",
            "data": "synthetic: seeded smooth field + per-frame noise",
            "config": workload_config(args, cfg, ob.levels, fps, l2_note(args.pool, frame_mb), f"replicas x{world}"),
            "cpu_baseline": {"value": round(value, 4), "unit": "Mpix/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "Mpix/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--pool", type=int, default=4)
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c2")
    ap.add_argument("--scale", type=int, default=1,
                    help="divide the workload's source and canvas sizes by this (small profiler captures)")
    ap.add_argument("--inflight", type=int, default=8, help="caller streams of the device-resident loop")
    ap.add_argument("--e2e-steps", type=int, default=0)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-seconds", type=float, default=90.0)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-linear", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-cpu-rigs", action="store_true", help="skip the CPU timings of the c1 and c5 rigs")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_env()
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        # one rank per GPU: run this script under torchrun with the same arguments
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        return subprocess.call(relaunch_cmd(sys.argv[1:] if argv is None else argv, args.gpus, port))
    if world != args.gpus:
        print(json.dumps({"error": f"--gpus {args.gpus} but WORLD_SIZE {world}: launch one rank per GPU"}),
              flush=True)
        return 2
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, world, rank)), flush=True)
        return 0
    import torch
    dist = dist_init(world, torch.cuda.is_available())
    out = run_ours(args, world, rank, local, dist)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
