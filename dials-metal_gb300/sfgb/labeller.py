"""ctypes binding of the device labeller (include/sf_api.h, sf_label_*): the
counterpart of dials_spots::Labeller (src/spots/dials_spots.hh:108-158).

`add()` takes one frame's host signal list (Labeller::add); `add_device()`
takes a batch of frames whose lists are already on the device, e.g. straight
from api.DeviceThreshold. Errors the reference throws for raise here.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import api

# src/spots/dials_spots.hh:50-54 and :57-79
PIXEL_DTYPE = np.dtype([("frame", "<i4"), ("index", "<u4"), ("value", "<u4")])
SPOT_DTYPE = np.dtype([("bbox", "<i4", (6,)), ("position", "<f8", (3,)),
                       ("variance", "<f8", (3,)), ("intensity", "<f8"),
                       ("intensity_variance", "<f8"), ("n_signal", "<u4"),
                       ("first", "<u8")], align=True)
COUNT_NAMES = ("signal_pixels", "groups", "too_small", "too_large", "separated",
               "accepted")


class LabelOptions(ctypes.Structure):
    _fields_ = [("min_spot_size", ctypes.c_size_t), ("max_spot_size", ctypes.c_size_t),
                ("max_separation", ctypes.c_double), ("two_d", ctypes.c_int)]


class ReflOptions(ctypes.Structure):
    """refl::Options (src/spots/refl.hh:53-64)."""
    _fields_ = [("panel", ctypes.c_size_t), ("id", ctypes.c_int),
                ("identifier", ctypes.c_char_p), ("shoeboxes", ctypes.c_int)]


def _refl_options(shoeboxes: bool, identifier: str, id: int, panel: int) -> ReflOptions:
    return ReflOptions(panel, id, identifier.encode() if identifier else None, int(shoeboxes))


_bound = False


def _lib():
    global _bound
    L = api.lib()
    if not _bound:
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.sf_default_label_options.argtypes = [ctypes.POINTER(LabelOptions)]
        L.sf_label_open.argtypes = [sz, sz, ctypes.POINTER(LabelOptions), sz]
        L.sf_label_open.restype = vp
        L.sf_label_close.argtypes = [vp]
        L.sf_label_add.argtypes = [vp, ctypes.c_int64, vp, sz]
        L.sf_label_add.restype = ctypes.c_int
        L.sf_label_add_device.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), sz, vp, sz, vp, vp]
        L.sf_label_add_device.restype = ctypes.c_int
        L.sf_label_finish.argtypes = [vp]
        L.sf_label_finish.restype = ctypes.c_int
        for name in ("sf_label_n_spots", "sf_label_n_pixels", "sf_label_live"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = sz
        L.sf_label_spots.argtypes = [vp, vp, sz]
        L.sf_label_spots.restype = ctypes.c_int
        L.sf_label_pixels.argtypes = [vp, vp, sz]
        L.sf_label_pixels.restype = ctypes.c_int
        L.sf_label_counts.argtypes = [vp, vp]
        L.sf_refl_write.argtypes = [ctypes.c_char_p, vp, sz, vp, sz, sz,
                                    ctypes.POINTER(ReflOptions)]
        L.sf_refl_write.restype = ctypes.c_int
        L.sf_label_write_refl.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ReflOptions)]
        L.sf_label_write_refl.restype = ctypes.c_int
        _bound = True
    return L


@dataclass
class LabelResult:
    spots: np.ndarray
    pixels: np.ndarray
    counts: dict = field(default_factory=dict)


class DeviceLabeller:
    def __init__(self, height: int, width: int, min_spot_size: int = 3,
                 max_spot_size: int = 1000, max_separation: float = 2.0,
                 two_d: bool = False, live_capacity: int = 0):
        L = _lib()
        o = LabelOptions(min_spot_size, max_spot_size, max_separation, int(two_d))
        self._h = L.sf_label_open(height, width, ctypes.byref(o), live_capacity)
        if not self._h:
            raise ValueError("labeller rejected: " + api.last_error())

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: {api.last_error()} ({rc})")

    def add(self, frame: int, signal: np.ndarray) -> None:
        signal = np.ascontiguousarray(signal, api.SIGNAL_DTYPE)
        self._check(_lib().sf_label_add(self._h, frame, signal.ctypes.data, len(signal)),
                    f"frame {frame}")

    def add_device(self, frames, lists_ptr: int, stride: int, counts_ptr: int,
                   stream_ptr: int | None = None) -> None:
        arr = (ctypes.c_int64 * len(frames))(*frames)
        self._check(_lib().sf_label_add_device(self._h, arr, len(frames), lists_ptr, stride,
                                               counts_ptr, stream_ptr), f"frames {frames}")

    def finish(self) -> LabelResult:
        L = _lib()
        self._check(L.sf_label_finish(self._h), "finish")
        return self.result()

    def result(self) -> LabelResult:
        return result_of(self._h)

    @property
    def live(self) -> int:
        return _lib().sf_label_live(self._h)

    def write_refl(self, path: str, shoeboxes: bool = True, identifier: str = "",
                   id: int = 0, panel: int = 0) -> None:
        """refl::write of the spots so far (src/spots/refl.hh:72-74), the
        shoebox column built on the device."""
        o = _refl_options(shoeboxes, identifier, id, panel)
        self._check(_lib().sf_label_write_refl(self._h, path.encode(), ctypes.byref(o)),
                    f"writing {path}")

    def close(self):
        if getattr(self, "_h", None):
            _lib().sf_label_close(self._h)
            self._h = None

    def __del__(self):
        self.close()


def result_of(handle) -> LabelResult:
    """The spots, kept pixels and counts a labeller handle holds so far."""
    L = _lib()
    ns, npx = L.sf_label_n_spots(handle), L.sf_label_n_pixels(handle)
    spots = np.zeros(ns, SPOT_DTYPE)
    pixels = np.zeros(npx, PIXEL_DTYPE)
    for rc, what in ((L.sf_label_spots(handle, spots.ctypes.data, ns), "spots"),
                     (L.sf_label_pixels(handle, pixels.ctypes.data, npx), "pixels")):
        if rc != 0:
            raise RuntimeError(f"{what}: {api.last_error()} ({rc})")
    c = np.zeros(6, np.uint64)
    L.sf_label_counts(handle, c.ctypes.data)
    return LabelResult(spots, pixels, dict(zip(COUNT_NAMES, map(int, c))))


def write_refl(path: str, spots: np.ndarray, pixels: np.ndarray, width: int,
               shoeboxes: bool = True, identifier: str = "", id: int = 0,
               panel: int = 0) -> None:
    """refl::write (src/spots/refl.hh:72-74) of host spot and pixel arrays;
    needs no GPU."""
    spots = np.ascontiguousarray(spots, SPOT_DTYPE)
    pixels = np.ascontiguousarray(pixels, PIXEL_DTYPE)
    o = _refl_options(shoeboxes, identifier, id, panel)
    rc = _lib().sf_refl_write(path.encode(), spots.ctypes.data, len(spots), pixels.ctypes.data,
                              len(pixels), width, ctypes.byref(o))
    if rc != 0:
        raise RuntimeError(f"writing {path}: {api.last_error()} ({rc})")
