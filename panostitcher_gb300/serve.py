"""Live-stream serving over the C ABI (ps_server_*).

``StitchServer`` keeps every admitted stream's rig resident, admits streams
against a device-memory budget, and replays arrival traces in real time with
continuous batching (see csrc/ps_server.cpp).
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib as L
from ._lib import Image, PhotoParam, PsError, check, lib
from .render import as_image


class StitchServer:
    def __init__(self, budget_bytes: int, max_batch: int = 16):
        h = C.c_void_p()
        check(lib().ps_server_create(int(budget_bytes), int(max_batch), C.byref(h)))
        self._h = h

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().ps_server_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def admit(self, cams: Sequence[dict], blend_param: int, src_size, dst_size) -> int | None:
        """Stream id, or None when the stream does not fit the budget."""
        arr = (PhotoParam * len(cams))(*[PhotoParam.from_dict(p) for p in cams])
        sid = C.c_int()
        st = lib().ps_server_admit(self._h, arr, len(cams), blend_param, src_size[0], src_size[1], dst_size[0],
                                   dst_size[1], C.byref(sid))
        if st == L.PS_ENOMEM:
            return None
        check(st)
        return sid.value

    def remove(self, stream_id: int) -> None:
        check(lib().ps_server_remove(self._h, stream_id))

    @property
    def resident_bytes(self) -> int:
        return lib().ps_server_resident_bytes(self._h)

    def run_trace(self, stream_ids: Sequence[int], arrival_s: Sequence[float], frames: Sequence[Sequence],
                  luts: Sequence | None = None, dsts: Sequence | None = None):
        """Replay arrivals in real time.  frames[k]: camera images of frame k
        (host numpy; pinned memory keeps uploads asynchronous); dsts[k]: host
        or device canvas per frame, or None to keep outputs on the device.
        Returns (latency seconds per frame, wall seconds)."""
        m = len(stream_ids)
        keep = []
        srcs = []
        for fr in frames:
            arr = (Image * len(fr))(*[as_image(f) for f in fr])
            keep.append(arr)
            srcs.append(C.cast(arr, C.POINTER(Image)))
        sp = (C.POINTER(Image) * m)(*srcs)
        lp = None
        if luts is not None:
            la = [None if lt is None else np.ascontiguousarray(lt, np.uint8) for lt in luts]
            keep.append(la)
            lp = (C.c_void_p * m)(*[None if a is None else a.ctypes.data for a in la])
        dp = None
        if dsts is not None:
            dp = (Image * m)(*[as_image(d) for d in dsts])
        ids = (C.c_int * m)(*stream_ids)
        arr_ns = (C.c_longlong * m)(*[int(round(t * 1e9)) for t in arrival_s])
        lat = (C.c_longlong * m)()
        wall = C.c_longlong()
        check(lib().ps_server_run_trace(self._h, m, ids, arr_ns, sp, lp, dp, lat, C.byref(wall)))
        return np.array(lat[:], dtype=np.float64) / 1e9, wall.value / 1e9
