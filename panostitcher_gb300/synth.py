"""Seeded synthetic rigs and frame content for the stitch benchmarks.

No public dataset is involved: the benchmark rigs are described by camera
parameters and sizes only, and frame content is a seeded smooth field plus
per-frame integer noise.  Everything is derived from SplitMix64 counters, so
the same (seed, camera, channel, frame) always gives the same pixels.

Content per camera and channel (B, G, R):
    field(x, y) = 128 + 80 * (1/8) * sum_{m=1..8} sin(2*pi*(u_m*x/W + v_m*y/H) + phi_m)
    u_m, v_m ~ U[0.5, 8] cycles per image, phi_m ~ U[0, 2*pi)
    pixel = clamp(rint(field) + noise, 0, 255),  noise ~ U{-A..A} per frame
Gains: per camera per channel k ~ U[lo, hi]; LUT lut[v] = sat(rint(k * v))
(getLUT, source/Blend/ExposureColorOptimize.cpp:1217-1223).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser over a uint64 array (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = (x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def key(*parts: int) -> int:
    """Hash a tuple of non-negative ints into one 64-bit counter base."""
    h = np.uint64(0x243F6A8885A308D3)
    for p in parts:
        h = splitmix64(np.array([h ^ np.uint64(p & 0xFFFFFFFFFFFFFFFF)], np.uint64))[0]
    return int(h)


def uniform(k: int, count: int, lo: float, hi: float) -> np.ndarray:
    """count values uniform in [lo, hi) from counter base k."""
    z = splitmix64(np.uint64(k) + np.arange(count, dtype=np.uint64))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


def photo_param(image_type=0, hfov=90.0, yaw=0.0, pitch=0.0, roll=0.0, **extra) -> dict:
    """PhotoParam as a dict (source/Warp/ZReproject.h:17-50); unset fields 0."""
    p = dict(image_type=image_type, crop_mode=0, crop_x=0, crop_y=0, crop_width=0, crop_height=0,
             circle_x=0, circle_y=0, circle_r=0, hfov=float(hfov), vfov=0.0, alpha=0.0, beta=0.0,
             gamma=0.0, shift_x=0.0, shift_y=0.0, shear_x=0.0, shear_y=0.0, yaw=float(yaw),
             pitch=float(pitch), roll=float(roll))
    p.update(extra)
    return p


@dataclass
class RigConfig:
    name: str
    cams: list
    src_size: tuple          # (W, H) of every camera frame
    dst_size: tuple          # (W, H) of the equirectangular canvas
    levels: int              # requested multiband levels
    gain_range: tuple = (1.0, 1.0)
    noise: int = 10
    seed: int = 1234
    frames: int = 1
    extra: dict = field(default_factory=dict)

    @property
    def num_cams(self) -> int:
        return len(self.cams)

    @property
    def canvas_pixels(self) -> int:
        return self.dst_size[0] * self.dst_size[1]


def _levels_rule(w, h):
    """floor(log2(min side)) - 3, the batched-rig level rule."""
    return int(math.floor(math.log2(min(w, h)))) - 3


def rig(name: str, seed: int = 1234) -> RigConfig:
    """The benchmark rigs.

    c1:  2 full-frame fisheye 1280x960, 200 deg, yaw 0/180 -> 2048x1024, 5 levels, gains 1.0
    c2:  6 rectilinear 1920x1080, 100 deg, yaw 0/90/180/270 + pitch +-90 -> 4096x2048, 8 levels
    c3a: 2 fisheye 2048x2048, 200 deg, yaw 0/180 -> 3840x1920
    c3b: = c2
    c3c: 4 rectilinear 1280x960, 110 deg, yaw 0/90/180/270 -> 2560x1280
    c3d: 8 rectilinear 2704x2028, 120 deg, yaw every 45 deg -> 7680x3840
    c5:  8 rectilinear 3840x2160, 120 deg, yaw every 45 deg -> 7680x3840, 10 levels,
         gains U[0.7,1.3], noise +-20
    ricoh: one 1920x960 dual-fisheye frame, two circular 200 deg fisheyes back to back,
         each camera's crop one 960x960 half -> 2048x1024, 5 levels (the rig
         CudaRicohPanoramaRender stitches from one frame)
    """
    if name == "c1":
        cams = [photo_param(1, 200.0, 0.0), photo_param(1, 200.0, 180.0)]
        return RigConfig(name, cams, (1280, 960), (2048, 1024), 5, (1.0, 1.0), 10, seed, 100)
    if name in ("c2", "c3b"):
        cams = [photo_param(0, 100.0, y) for y in (0.0, 90.0, 180.0, 270.0)]
        cams += [photo_param(0, 100.0, 0.0, 90.0), photo_param(0, 100.0, 0.0, -90.0)]
        return RigConfig(name, cams, (1920, 1080), (4096, 2048), 8 if name == "c2" else _levels_rule(4096, 2048),
                         (0.8, 1.2), 10, seed, 300)
    if name == "c3a":
        cams = [photo_param(1, 200.0, 0.0), photo_param(1, 200.0, 180.0)]
        return RigConfig(name, cams, (2048, 2048), (3840, 1920), _levels_rule(3840, 1920), (0.8, 1.2), 10, seed)
    if name == "c3c":
        cams = [photo_param(0, 110.0, y) for y in (0.0, 90.0, 180.0, 270.0)]
        return RigConfig(name, cams, (1280, 960), (2560, 1280), _levels_rule(2560, 1280), (0.8, 1.2), 10, seed)
    if name == "c3d":
        cams = [photo_param(0, 120.0, 45.0 * k) for k in range(8)]
        return RigConfig(name, cams, (2704, 2028), (7680, 3840), _levels_rule(7680, 3840), (0.8, 1.2), 10, seed)
    if name == "c5":
        cams = [photo_param(0, 120.0, 45.0 * k) for k in range(8)]
        return RigConfig(name, cams, (3840, 2160), (7680, 3840), 10, (0.7, 1.3), 20, seed, 120)
    if name == "ricoh":
        cams = [photo_param(3, 200.0, 0.0, crop_x=0, crop_y=0, crop_width=960, crop_height=960),
                photo_param(3, 200.0, 180.0, crop_x=960, crop_y=0, crop_width=960, crop_height=960)]
        return RigConfig(name, cams, (1920, 960), (2048, 1024), 5, (0.9, 1.1), 10, seed)
    raise KeyError(name)


def scaled_rig(base: RigConfig, factor: int, name: str | None = None) -> RigConfig:
    """Same cameras, source and canvas sizes divided by factor (for tests);
    crop rectangles and circles, in source pixels, are divided too."""
    sw, sh = base.src_size
    dw, dh = base.dst_size
    dw2 = max(4, (dw // factor) // 4 * 4)
    cams = []
    for c in base.cams:
        c = dict(c)
        for k in ("crop_x", "crop_y", "crop_width", "crop_height", "circle_x", "circle_y", "circle_r"):
            c[k] = int(c[k]) // factor
        cams.append(c)
    return RigConfig(name or f"{base.name}/{factor}", cams,
                     (max(2, sw // factor), max(2, sh // factor)), (dw2, dw2 // 2), base.levels,
                     base.gain_range, base.noise, base.seed, base.frames)


def gains(cfg: RigConfig) -> np.ndarray:
    """Per camera, per channel (B, G, R) gains, shape (n, 3)."""
    lo, hi = cfg.gain_range
    if lo == hi:
        return np.full((cfg.num_cams, 3), lo, np.float64)
    return uniform(key(cfg.seed, 0x6A1), cfg.num_cams * 3, lo, hi).reshape(cfg.num_cams, 3)


def lut_from_gain(k: float) -> np.ndarray:
    """lut[v] = saturate_cast<uchar>(k*v): round half to even, clamp."""
    return np.clip(np.rint(k * np.arange(256, dtype=np.float64)), 0, 255).astype(np.uint8)


def luts(cfg: RigConfig) -> np.ndarray:
    """(n, 3, 256) uint8 LUTs, channel order B, G, R."""
    g = gains(cfg)
    return np.stack([np.stack([lut_from_gain(g[i, c]) for c in range(3)]) for i in range(cfg.num_cams)])


def smooth_field(cfg: RigConfig, cam: int) -> np.ndarray:
    """(H, W, 3) float64 smooth field of one camera (no noise)."""
    W, H = cfg.src_size
    x = np.arange(W, dtype=np.float64) / W
    y = np.arange(H, dtype=np.float64) / H
    out = np.empty((H, W, 3), np.float64)
    for c in range(3):
        prm = uniform(key(cfg.seed, 0xF1E1D, cam, c), 24, 0.0, 1.0).reshape(8, 3)
        acc = np.zeros((H, W), np.float64)
        for m in range(8):
            u = 0.5 + 7.5 * prm[m, 0]
            v = 0.5 + 7.5 * prm[m, 1]
            phi = 2.0 * math.pi * prm[m, 2]
            ax = 2.0 * math.pi * u * x
            by = 2.0 * math.pi * v * y + phi
            # sin(a + b) = sin a cos b + cos a sin b, as outer products
            acc += np.outer(np.cos(by), np.sin(ax)) + np.outer(np.sin(by), np.cos(ax))
        out[:, :, c] = 128.0 + 80.0 * acc / 8.0
    return out


def noise(cfg: RigConfig, cam: int, frame: int, shape) -> np.ndarray:
    """Integer noise U{-A..A} for one camera frame, shape (H, W, 3)."""
    a = cfg.noise
    count = int(np.prod(shape))
    z = splitmix64(np.uint64(key(cfg.seed, 0x4015E, cam, frame)) + np.arange(count, dtype=np.uint64))
    return ((z >> np.uint64(32)) % np.uint64(2 * a + 1)).astype(np.int32).reshape(shape) - a


class FrameSource:
    """Generates camera frames of a rig; caches the smooth fields."""

    def __init__(self, cfg: RigConfig, channels: int = 4):
        assert channels in (3, 4)
        self.cfg = cfg
        self.channels = channels
        self._base = [np.rint(smooth_field(cfg, i)).astype(np.int32) for i in range(cfg.num_cams)]

    def frame(self, frame: int) -> list:
        """List of n (H, W, channels) uint8 frames; channel 3 (if any) is 0."""
        out = []
        for i, base in enumerate(self._base):
            v = np.clip(base + noise(self.cfg, i, frame, base.shape), 0, 255).astype(np.uint8)
            if self.channels == 4:
                v = np.concatenate([v, np.zeros(v.shape[:2] + (1,), np.uint8)], axis=2)
            out.append(np.ascontiguousarray(v))
        return out
