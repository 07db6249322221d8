"""Seeded synthetic sweeps (csrc/synth.c) for tests and benchmarks.

Named presets follow the benchmark workloads: each is a raw uint32 sweep with
the masks stamped in as the sentinel 0xFFFFFFFF.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import _paths


class SynthParams(ctypes.Structure):
    _fields_ = [("height", ctypes.c_uint32), ("width", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("n_frames", ctypes.c_int),
                ("bg_edge", ctypes.c_double), ("bg_centre", ctypes.c_double),
                ("n_rings", ctypes.c_int), ("ring_amplitude", ctypes.c_double),
                ("spots_per_frame", ctypes.c_double),
                ("sigma_xy_min", ctypes.c_double), ("sigma_xy_max", ctypes.c_double),
                ("sigma_z_min", ctypes.c_double), ("sigma_z_max", ctypes.c_double),
                ("peak_min", ctypes.c_double), ("peak_max", ctypes.c_double),
                ("eiger_gaps", ctypes.c_int),
                ("row_band_start", ctypes.c_uint32), ("row_band_len", ctypes.c_uint32),
                ("col_band_start", ctypes.c_uint32), ("col_band_len", ctypes.c_uint32),
                ("n_hot", ctypes.c_uint32), ("saturated_fraction", ctypes.c_double),
                ("saturated_value", ctypes.c_uint32)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = _paths.synth_lib()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is not built; run __graft_entry__.build()")
        L = ctypes.CDLL(path)
        L.sf_synth_default_params.argtypes = [ctypes.POINTER(SynthParams)]
        L.sf_synth_open.argtypes = [ctypes.POINTER(SynthParams)]
        L.sf_synth_open.restype = ctypes.c_void_p
        L.sf_synth_close.argtypes = [ctypes.c_void_p]
        L.sf_synth_n_spots.argtypes = [ctypes.c_void_p]
        L.sf_synth_n_spots.restype = ctypes.c_size_t
        L.sf_synth_frame.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.sf_synth_frame.restype = ctypes.c_int
        sz, vp = ctypes.c_size_t, ctypes.c_void_p
        L.sf_chunk_bound.argtypes = [sz, sz]
        L.sf_chunk_bound.restype = sz
        L.sf_chunk_bslz4.argtypes = [vp, sz, ctypes.c_uint, sz, vp, sz]
        L.sf_chunk_bslz4.restype = ctypes.c_int64
        L.sf_chunk_lz4.argtypes = [vp, sz, sz, vp, sz]
        L.sf_chunk_lz4.restype = ctypes.c_int64
        L.sf_lz4_bound.argtypes = [sz]
        L.sf_lz4_bound.restype = sz
        L.sf_lz4_block.argtypes = [vp, sz, vp]
        L.sf_lz4_block.restype = sz
        L.sf_bitshuffle.argtypes = [vp, vp, sz, sz]
        _lib = L
    return _lib


def default_params() -> SynthParams:
    p = SynthParams()
    lib().sf_synth_default_params(ctypes.byref(p))
    return p


def preset(name: str, **overrides) -> SynthParams:
    """Workload presets.

    plain_1m   100 x 1024x1024, Poisson 0.5, 200 spots/frame (sigma_xy 1.2,
               sigma_z 0.8, peak 50-2000 log-uniform), an 8-row and an
               8-column masked band, 20 hot pixels.
    eiger_16m  4362x4148 (EIGER2 16M tiling, module gaps masked), Poisson 0.3
               at the edge rising to 1.5 at the centre, 3000 spots/frame
               spanning 2-5 frames.
    batch_4m / batch_9m  2162x2068 / 3262x3108, Poisson 1.0, 1500 spots,
               sigma_xy 1-2.
    dense_16m  4362x4148, Poisson 20 plus three diffuse rings, 20000 spots,
               2% of pixels at a saturated-overload count, 500 hot pixels.
    """
    p = default_params()
    if name == "plain_1m":
        p.height, p.width, p.n_frames = 1024, 1024, 100
        p.bg_edge = p.bg_centre = 0.5
        p.spots_per_frame = 200.0
        p.row_band_start, p.row_band_len = 500, 8
        p.col_band_start, p.col_band_len = 300, 8
        p.n_hot = 20
        p.seed = 1000
    elif name == "eiger_16m":
        p.height, p.width, p.n_frames = 4362, 4148, 900
        p.bg_edge, p.bg_centre = 0.3, 1.5
        p.spots_per_frame = 3000.0
        p.sigma_xy_min, p.sigma_xy_max = 1.0, 1.5
        p.sigma_z_min, p.sigma_z_max = 0.5, 1.0
        p.eiger_gaps = 1
        p.seed = 2000
    elif name in ("batch_4m", "batch_9m"):
        p.height, p.width = (2162, 2068) if name == "batch_4m" else (3262, 3108)
        p.n_frames = 64
        p.bg_edge = p.bg_centre = 1.0
        p.spots_per_frame = 1500.0
        p.sigma_xy_min, p.sigma_xy_max = 1.0, 2.0
        p.seed = 3000 if name == "batch_4m" else 3001
    elif name == "dense_16m":
        p.height, p.width, p.n_frames = 4362, 4148, 1200
        p.bg_edge = p.bg_centre = 20.0
        p.n_rings, p.ring_amplitude = 3, 15.0
        p.spots_per_frame = 20000.0
        p.sigma_xy_min, p.sigma_xy_max = 1.0, 1.5
        p.saturated_fraction, p.saturated_value = 0.02, 1_000_000
        p.n_hot = 500
        p.eiger_gaps = 1
        p.seed = 5000
    elif name != "default":
        raise ValueError(f"unknown preset {name}")
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


class Sweep:
    """Frames of one seeded sweep, generated on demand."""

    def __init__(self, params: SynthParams):
        self.params = params
        self._h = lib().sf_synth_open(ctypes.byref(params))
        if not self._h:
            raise ValueError("synthetic sweep parameters rejected")

    @property
    def shape(self):
        return (self.params.height, self.params.width)

    @property
    def n_frames(self) -> int:
        return self.params.n_frames

    def frame(self, index: int, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.shape, np.uint32)
        assert out.dtype == np.uint32 and out.flags.c_contiguous and out.size == self.shape[0] * self.shape[1]
        if lib().sf_synth_frame(self._h, index, out.ctypes.data) != 0:
            raise ValueError(f"frame {index} out of range")
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().sf_synth_close(self._h)
            self._h = None


def chunk(frame: np.ndarray, algorithm: str = "bslz4", block_bytes: int = 0,
          out: np.ndarray | None = None) -> np.ndarray:
    """The frame as an HDF5 writer stores a compressed chunk ("bslz4" or
    "lz4", with the 12-byte filter header), as uint8. block_bytes 0 takes
    bitshuffle's default block (bslz4) or one block for the frame (lz4). With
    `out` the chunk is written there (a view of its first bytes returned)."""
    frame = np.ascontiguousarray(frame)
    nbytes = frame.nbytes
    cap = lib().sf_chunk_bound(nbytes, block_bytes if algorithm == "bslz4" or block_bytes
                               else max(nbytes, 1))
    if out is None:
        out = np.empty(cap, np.uint8)
    elif out.nbytes < cap:
        raise ValueError(f"chunk buffer of {out.nbytes} bytes, need {cap}")
    ptr = frame.ctypes.data if frame.size else None
    if algorithm == "bslz4":
        n = lib().sf_chunk_bslz4(ptr or out.ctypes.data, frame.size, frame.itemsize,
                                 block_bytes, out.ctypes.data, out.nbytes)
    elif algorithm == "lz4":
        n = lib().sf_chunk_lz4(ptr or out.ctypes.data, nbytes, block_bytes, out.ctypes.data,
                               out.nbytes)
    else:
        raise ValueError(f"unknown compression algorithm {algorithm}")
    if n < 0:
        raise ValueError("chunk writer refused the frame")
    return out[:n]


def lz4_block(data: bytes) -> bytes:
    """One LZ4 block of `data` (this module's matcher)."""
    src = np.frombuffer(bytes(data), np.uint8)
    dst = np.empty(lib().sf_lz4_bound(src.size), np.uint8)
    n = lib().sf_lz4_block(src.ctypes.data if src.size else dst.ctypes.data, src.size,
                           dst.ctypes.data)
    return dst[:n].tobytes()


def bitshuffle(elements: np.ndarray) -> np.ndarray:
    """The bit planes of a block of elements (a multiple of 8 of them)."""
    e = np.ascontiguousarray(elements)
    out = np.empty(e.nbytes, np.uint8)
    lib().sf_bitshuffle(e.ctypes.data, out.ctypes.data, e.size, e.itemsize)
    return out
