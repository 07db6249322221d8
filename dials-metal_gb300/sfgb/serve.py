"""ctypes binding of the served form (include/sf_api.h, sf_server_*): a
request loop for frames arriving from several detector streams at once, each
sweep's frame ring and 3-D labeller resident on the device, sweeps admitted
by device memory, continuous batching across sweeps of one frame shape.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import api, labeller

SF_EBUSY = -5


class ServerOptions(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_size_t), ("max_batch", ctypes.c_size_t),
                ("ring", ctypes.c_size_t), ("capacity_divisor", ctypes.c_size_t),
                ("coalesce_us", ctypes.c_size_t), ("label_capacity", ctypes.c_size_t)]


class FrameDone(ctypes.Structure):
    _fields_ = [("sweep", ctypes.c_int64), ("frame", ctypes.c_int64),
                ("n_signal", ctypes.c_uint32), ("status", ctypes.c_int),
                ("latency_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("batches", ctypes.c_uint64), ("batch_frames", ctypes.c_uint64),
                ("label_calls", ctypes.c_uint64), ("label_frames", ctypes.c_uint64),
                ("launch_seconds", ctypes.c_double), ("label_seconds", ctypes.c_double),
                ("launch_max_seconds", ctypes.c_double), ("label_max_seconds", ctypes.c_double)]


class Busy(RuntimeError):
    """The device-memory budget is taken; retry once a sweep closes."""


_bound = False


def _lib():
    global _bound
    L = labeller._lib()
    if not _bound:
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.sf_default_server_options.argtypes = [ctypes.POINTER(ServerOptions)]
        L.sf_server_open.argtypes = [ctypes.POINTER(ServerOptions)]
        L.sf_server_open.restype = vp
        L.sf_server_close.argtypes = [vp]
        L.sf_server_sweep_bytes.argtypes = [vp, sz, sz, ctypes.POINTER(labeller.LabelOptions)]
        L.sf_server_sweep_bytes.restype = sz
        L.sf_server_used_bytes.argtypes = [vp]
        L.sf_server_used_bytes.restype = sz
        L.sf_server_open_sweep.argtypes = [vp, sz, sz, ctypes.POINTER(api.ThresholdParams),
                                           ctypes.POINTER(labeller.LabelOptions),
                                           ctypes.POINTER(ctypes.c_int64)]
        L.sf_server_open_sweep.restype = ctypes.c_int
        L.sf_server_submit.argtypes = [vp, ctypes.c_int64, ctypes.c_int64, vp]
        L.sf_server_submit.restype = ctypes.c_int
        L.sf_server_submit_chunk.argtypes = [vp, ctypes.c_int64, ctypes.c_int64, vp, sz,
                                             ctypes.c_char_p]
        L.sf_server_submit_chunk.restype = ctypes.c_int
        L.sf_server_poll.argtypes = [vp, ctypes.POINTER(FrameDone), sz, ctypes.c_int]
        L.sf_server_poll.restype = sz
        for name in ("sf_server_finish_sweep", "sf_server_close_sweep"):
            getattr(L, name).argtypes = [vp, ctypes.c_int64]
            getattr(L, name).restype = ctypes.c_int
        L.sf_server_labeller.argtypes = [vp, ctypes.c_int64]
        L.sf_server_labeller.restype = vp
        L.sf_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
        L.sf_server_sweep_error.argtypes = [vp, ctypes.c_int64]
        L.sf_server_sweep_error.restype = ctypes.c_char_p
        _bound = True
    return L


class Server:
    def __init__(self, hbm_budget: int = 0, max_batch: int = 16, ring: int = 32,
                 capacity_divisor: int = 16, coalesce_us: int = 1000, label_capacity: int = 0):
        L = _lib()
        o = ServerOptions(hbm_budget, max_batch, ring, capacity_divisor, coalesce_us,
                          label_capacity)
        self._s = L.sf_server_open(ctypes.byref(o))
        if not self._s:
            raise api.SpotFinderError("server refused its options: " + api.last_error())
        self._keep = {}  # (sweep, frame) -> host array kept alive until done
        self._lock = threading.Lock()

    def sweep_bytes(self, height: int, width: int) -> int:
        return _lib().sf_server_sweep_bytes(self._s, height, width, None)

    @property
    def used_bytes(self) -> int:
        return _lib().sf_server_used_bytes(self._s)

    def open_sweep(self, height: int, width: int, params: api.Params | None = None,
                   min_spot_size: int = 3, max_spot_size: int = 1000,
                   max_separation: float = 2.0, two_d: bool = False) -> int:
        sid = ctypes.c_int64(0)
        p = (params or api.Params()).c()
        lo = labeller.LabelOptions(min_spot_size, max_spot_size, max_separation, int(two_d))
        rc = _lib().sf_server_open_sweep(self._s, height, width, ctypes.byref(p),
                                         ctypes.byref(lo), ctypes.byref(sid))
        if rc == SF_EBUSY:
            raise Busy("the device-memory budget is taken")
        api._check(rc, "open sweep")
        return sid.value

    def submit(self, sweep: int, frame: int, image) -> None:
        """image: a (h, w) uint32 array (kept alive here until the frame is
        done) or an integer host address."""
        if isinstance(image, np.ndarray):
            if image.dtype != np.uint32 or not image.flags.c_contiguous:
                raise ValueError("a contiguous uint32 frame")
            ptr = image.ctypes.data
            with self._lock:
                self._keep[(sweep, frame)] = image
        else:
            ptr = int(image)
        rc = _lib().sf_server_submit(self._s, sweep, frame, ptr)
        if rc == api.SF_EBADARG:
            raise ValueError("submit: frames go in ascending order to an open sweep")
        if rc != 0:
            raise api.SpotFinderError(f"submit ({rc}): {self.sweep_error(sweep)}")

    def submit_chunk(self, sweep: int, frame: int, chunk, algorithm: str = "bslz4",
                     nbytes: int | None = None) -> None:
        """A 32-bit frame as a compressed chunk (filter header and all):
        a uint8 array (kept alive here until the frame is done) or an integer
        host address with nbytes. Raises api.DataError, the frame not taken,
        when the chunk's header or framing is wrong."""
        if isinstance(chunk, np.ndarray):
            chunk = np.ascontiguousarray(chunk).view(np.uint8).ravel()
            ptr, n = chunk.ctypes.data, chunk.size
            with self._lock:
                self._keep[(sweep, frame)] = chunk
        else:
            ptr, n = int(chunk), int(nbytes)
        rc = _lib().sf_server_submit_chunk(self._s, sweep, frame, ptr, n, algorithm.encode())
        if rc == api.SF_EDATA:
            with self._lock:
                self._keep.pop((sweep, frame), None)
            raise api.DataError(api.last_error())
        if rc == api.SF_EBADARG:
            raise ValueError("submit: frames go in ascending order to an open sweep")
        if rc != 0:
            raise api.SpotFinderError(f"submit ({rc}): {self.sweep_error(sweep)}")

    def poll(self, max_n: int = 4096, wait_ms: int = 0) -> list:
        buf = (FrameDone * max_n)()
        n = _lib().sf_server_poll(self._s, buf, max_n, wait_ms)
        out = []
        with self._lock:
            for i in range(n):
                d = buf[i]
                self._keep.pop((d.sweep, d.frame), None)
                out.append({"sweep": d.sweep, "frame": d.frame, "n_signal": d.n_signal,
                            "status": d.status, "latency_ms": d.latency_ms})
        return out

    def stats(self) -> dict:
        st = ServerStats()
        _lib().sf_server_get_stats(self._s, ctypes.byref(st))
        return {n: getattr(st, n) for n, _ in ServerStats._fields_}

    def sweep_error(self, sweep: int) -> str:
        return (_lib().sf_server_sweep_error(self._s, sweep) or b"").decode()

    def finish_sweep(self, sweep: int, read: bool = True):
        """Wait for the sweep's frames, close its open spots and (read=True)
        return its spots, kept pixels and counts."""
        L = _lib()
        rc = L.sf_server_finish_sweep(self._s, sweep)
        if rc != 0:
            raise api.SpotFinderError(f"finish sweep ({rc}): {self.sweep_error(sweep)}")
        return labeller.result_of(L.sf_server_labeller(self._s, sweep)) if read else None

    def n_spots(self, sweep: int) -> int:
        """Spots the sweep has produced so far (nothing is copied)."""
        L = _lib()
        return int(L.sf_label_n_spots(L.sf_server_labeller(self._s, sweep)))

    def close_sweep(self, sweep: int) -> None:
        api._check(_lib().sf_server_close_sweep(self._s, sweep), "close sweep")

    def close(self) -> None:
        if getattr(self, "_s", None):
            _lib().sf_server_close(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
