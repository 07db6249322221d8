"""ctypes bindings for the CPU oracle (oracle/liboracle.so) and, where it was
built, the reference's own CPU code (oracle/_ref/libref.so).

TEST INFRASTRUCTURE ONLY. Imported by tests/, by __graft_entry__.smoke() and
by the CPU-baseline leg of bench.py, as the checker; the product never imports
it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")

# src/spots/signal_pixel.hh:20-28
SIGNAL_DTYPE = np.dtype([("index", "<u4"), ("value", "<u4"), ("background", "<f4"),
                         ("population", "<u2"), ("reserved", "<u2")])
# src/spots/dials_spots.hh:50-54
PIXEL_DTYPE = np.dtype([("frame", "<i4"), ("index", "<u4"), ("value", "<u4")])
# src/spots/dials_spots.hh:57-79, flattened
SPOT_DTYPE = np.dtype([("bbox", "<i4", (6,)), ("position", "<f8", (3,)),
                       ("variance", "<f8", (3,)), ("intensity", "<f8"),
                       ("intensity_variance", "<f8"), ("n_signal", "<u4"),
                       ("first", "<u8")], align=True)

DISPERSION_EXTENDED = 0
DISPERSION = 1


class OracleParams(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int), ("kernel_x", ctypes.c_int),
                ("kernel_y", ctypes.c_int), ("gain", ctypes.c_double),
                ("sigma_b", ctypes.c_double), ("sigma_s", ctypes.c_double),
                ("min_local", ctypes.c_int), ("global_threshold", ctypes.c_double)]


@dataclass
class Params:
    """Threshold parameters; the defaults are the reference's hard-wired ones
    (src/spots/dext.cc:37-40, :99, :203)."""
    algorithm: int = DISPERSION_EXTENDED
    kernel_x: int = 3
    kernel_y: int = 3
    gain: float = 1.0
    sigma_b: float = 6.0
    sigma_s: float = 3.0
    min_local: int = 2
    global_threshold: float = 0.0

    def c(self) -> OracleParams:
        return OracleParams(self.algorithm, self.kernel_x, self.kernel_y, self.gain,
                            self.sigma_b, self.sigma_s, self.min_local,
                            self.global_threshold)


def build(quiet: bool = True) -> None:
    """Compile the oracle restatement (always) and the reference library (only
    where the reference tree exists)."""
    srcs = [os.path.join(HERE, f) for f in ("sf_oracle.c", "sf_oracle_decompress.c",
                                            "sf_oracle_frames.c")]
    tmp = LIB_PATH + ".tmp"
    subprocess.run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                    *srcs, "-o", tmp, "-lm", "-lpthread"], check=True)
    os.replace(tmp, LIB_PATH)
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True,
                   stdout=subprocess.DEVNULL if quiet else None,
                   stderr=subprocess.DEVNULL if quiet else None)


_lib = None
_ref = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        for name in ("or_dext_u32", "or_dext_u16"):
            f = getattr(L, name)
            f.argtypes = [vp, sz, sz, ctypes.POINTER(OracleParams), vp, sz,
                          ctypes.POINTER(sz), vp]
            f.restype = ctypes.c_int
        L.or_label_open.argtypes = [sz, sz, sz, sz, ctypes.c_double, ctypes.c_int]
        L.or_label_open.restype = vp
        L.or_label_add.argtypes = [vp, ctypes.c_int64, vp, sz]
        L.or_label_add.restype = ctypes.c_int
        L.or_label_finish.argtypes = [vp]
        for name in ("or_label_n_spots", "or_label_n_pixels"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = sz
        for name in ("or_label_spots", "or_label_pixels"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = vp
        L.or_label_counts.argtypes = [vp, vp]
        L.or_label_close.argtypes = [vp]
        L.or_lz4_decode.argtypes = [vp, sz, vp, sz]
        L.or_lz4_decode.restype = ctypes.c_long
        L.or_bitunshuffle.argtypes = [vp, vp, sz, sz]
        L.or_bshuf_default_block.argtypes = [sz]
        L.or_bshuf_default_block.restype = sz
        L.or_decompress_image.argtypes = [vp, sz, ctypes.c_char_p, ctypes.c_uint, sz, sz, vp,
                                          sz, ctypes.c_char_p, sz]
        L.or_decompress_image.restype = ctypes.c_int
        for name in ("or_scan_u16", "or_scan_u32"):
            getattr(L, name).argtypes = [vp, sz, vp]
        L.or_narrow_to_16.argtypes = [vp, sz, vp, vp]
        L.or_narrow_to_16.restype = ctypes.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_PATH)
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        for name in ("ref_dext_u32", "ref_dext_u16"):
            f = getattr(R, name)
            f.argtypes = [vp, sz, sz, vp, sz, ctypes.POINTER(sz)]
            f.restype = ctypes.c_int
        R.ref_make_frame.argtypes = [sz, sz, ctypes.c_uint64, ctypes.c_double,
                                     ctypes.c_int, vp]
        R.ref_fused_make_u16.argtypes = [sz, sz, ctypes.c_uint, ctypes.c_double, vp]
        R.ref_fused_make_u32.argtypes = [sz, sz, ctypes.c_uint, ctypes.c_double, vp]
        R.ref_label_open.argtypes = [sz, sz, sz, sz, ctypes.c_double, ctypes.c_int]
        R.ref_label_open.restype = vp
        R.ref_label_add.argtypes = [vp, ctypes.c_int64, vp, sz]
        R.ref_label_add.restype = ctypes.c_int
        R.ref_label_finish.argtypes = [vp]
        for name in ("ref_label_n_spots", "ref_label_n_pixels"):
            getattr(R, name).argtypes = [vp]
            getattr(R, name).restype = sz
        R.ref_label_spots.argtypes = [vp, vp]
        R.ref_label_pixels.argtypes = [vp, vp]
        R.ref_label_counts.argtypes = [vp, vp]
        R.ref_label_write_refl.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
        R.ref_label_write_refl.restype = ctypes.c_int
        R.ref_label_write_refl_opts.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_char_p, ctypes.c_size_t]
        R.ref_label_write_refl_opts.restype = ctypes.c_int
        R.ref_label_close.argtypes = [vp]
        _ref = R
    return _ref


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def dext(frame: np.ndarray, params: Params | None = None,
         with_mask: bool = False):
    """Threshold one frame (uint16 or uint32, shape (h, w)). Returns the
    signal pixels ascending by index (and the byte mask if asked)."""
    frame = np.ascontiguousarray(frame)
    if frame.dtype == np.uint32:
        fn = lib().or_dext_u32
    elif frame.dtype == np.uint16:
        fn = lib().or_dext_u16
    else:
        raise TypeError("frames are uint16 or uint32")
    h, w = frame.shape
    p = (params or Params()).c()
    cap = max(1024, h * w // 4)
    out = np.zeros(cap, SIGNAL_DTYPE)
    found = ctypes.c_size_t(0)
    mask = np.zeros((h, w), np.uint8) if with_mask else None
    rc = fn(_ptr(frame), h, w, ctypes.byref(p), _ptr(out), cap, ctypes.byref(found),
            _ptr(mask) if with_mask else None)
    if rc == -2:
        out = np.zeros(found.value, SIGNAL_DTYPE)
        rc = fn(_ptr(frame), h, w, ctypes.byref(p), _ptr(out), found.value,
                ctypes.byref(found), _ptr(mask) if with_mask else None)
    if rc != 0:
        raise ValueError(f"oracle threshold rejected the frame ({rc})")
    out = out[:found.value].copy()
    return (out, mask) if with_mask else out


def decompress_image(data, algorithm: str, bit_depth: int, height: int,
                     width: int) -> np.ndarray:
    """decompress::image (src/spots/decompress.cc:77-134): the chunk as HDF5
    stored it ("bslz4", "lz4" or "" for none) to a (height, width) frame of
    bit_depth bits. Raises RuntimeError with the reference's text."""
    buf = np.frombuffer(bytes(data), np.uint8) if not isinstance(data, np.ndarray) else \
        np.ascontiguousarray(data).view(np.uint8).ravel()
    dtype = {8: np.uint8, 16: np.uint16, 32: np.uint32}.get(bit_depth, np.uint8)
    nbytes = height * width * bit_depth // 8
    out = np.zeros(max(nbytes, 1), np.uint8)
    err = ctypes.create_string_buffer(256)
    rc = lib().or_decompress_image(_ptr(buf) if buf.size else None, buf.size,
                                   algorithm.encode(), bit_depth, height, width, _ptr(out),
                                   nbytes, err, 256)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    if bit_depth not in (8, 16, 32):
        return out[:nbytes]
    return out[:nbytes].view(dtype).reshape(height, width)


def lz4_decode(block: bytes, capacity: int) -> bytes:
    """One LZ4 block, as LZ4_decompress_safe reads it; raises ValueError with
    the negative code on a bad stream."""
    src = np.frombuffer(bytes(block), np.uint8)
    out = np.zeros(max(capacity, 1), np.uint8)
    r = lib().or_lz4_decode(_ptr(src) if src.size else None, src.size, _ptr(out), capacity)
    if r < 0:
        raise ValueError(r)
    return out[:r].tobytes()


def bitunshuffle(planes: np.ndarray, n: int, esize: int) -> np.ndarray:
    """The elements of one bitshuffle block from its bit planes (n a
    multiple of 8), as bytes."""
    planes = np.ascontiguousarray(planes, np.uint8)
    out = np.zeros(n * esize, np.uint8)
    lib().or_bitunshuffle(_ptr(planes), _ptr(out), n, esize)
    return out


def scan_frame(frame: np.ndarray) -> tuple:
    """mxi_max's scan<T> (apps/mxi_max.cc:47-67) of a uint16 or uint32
    frame: (largest non-marker value, bad pixels, tile joins, valid pixels
    at 0xFFFD or above)."""
    frame = np.ascontiguousarray(frame)
    out = np.zeros(4, np.uint64)
    fn = lib().or_scan_u32 if frame.dtype == np.uint32 else lib().or_scan_u16
    if frame.dtype not in (np.uint16, np.uint32):
        raise TypeError("frames are uint16 or uint32")
    fn(_ptr(frame), frame.size, _ptr(out))
    return tuple(int(x) for x in out)


def narrow_to_16(frame: np.ndarray):
    """find_spots.cc:169-182: (the frame truncated to 16 bits, the largest
    non-marker value, whether it is below 0xFFFD)."""
    frame = np.ascontiguousarray(frame, np.uint32)
    out = np.empty(frame.shape, np.uint16)
    worst = ctypes.c_uint32(0)
    ok = lib().or_narrow_to_16(_ptr(frame), frame.size, _ptr(out), ctypes.byref(worst))
    return out, worst.value, bool(ok)


def ref_dext(frame: np.ndarray) -> np.ndarray:
    """The reference's own dext<T>() on one frame."""
    frame = np.ascontiguousarray(frame)
    fn = ref().ref_dext_u32 if frame.dtype == np.uint32 else ref().ref_dext_u16
    h, w = frame.shape
    cap = max(1024, h * w)
    out = np.zeros(cap, SIGNAL_DTYPE)
    found = ctypes.c_size_t(0)
    rc = fn(_ptr(frame), h, w, _ptr(out), cap, ctypes.byref(found))
    if rc != 0:
        raise ValueError(f"reference dext returned {rc}")
    return out[:found.value].copy()


def ref_make_frame(h: int, w: int, seed: int, background: float,
                   with_mask: bool) -> np.ndarray:
    out = np.zeros((h, w), np.uint16)
    ref().ref_make_frame(h, w, seed, background, int(with_mask), _ptr(out))
    return out


def ref_fused_make(h: int, w: int, seed: int, mean: float, dtype) -> np.ndarray:
    out = np.zeros((h, w), dtype)
    fn = ref().ref_fused_make_u16 if dtype == np.uint16 else ref().ref_fused_make_u32
    fn(h, w, seed, mean, _ptr(out))
    return out


@dataclass
class LabelResult:
    spots: np.ndarray
    pixels: np.ndarray
    counts: dict = field(default_factory=dict)


def spot_fields_equal(a: np.ndarray, b: np.ndarray) -> bool:
    """Field-by-field bit equality of two spot tables (struct padding is
    not part of the data)."""
    if len(a) != len(b):
        return False
    return all(np.ascontiguousarray(a[name]).tobytes() ==
               np.ascontiguousarray(b[name]).tobytes() for name in SPOT_DTYPE.names)


COUNT_NAMES = ("signal_pixels", "groups", "too_small", "too_large", "separated",
               "accepted")


class Labeller:
    """The oracle restatement of dials_spots::Labeller."""

    def __init__(self, height, width, min_spot_size=3, max_spot_size=1000,
                 max_separation=2.0, two_d=False):
        self._h = lib().or_label_open(height, width, min_spot_size, max_spot_size,
                                      max_separation, int(two_d))
        if not self._h:
            raise ValueError("labeller options rejected")

    def add(self, frame: int, signal: np.ndarray) -> None:
        signal = np.ascontiguousarray(signal, SIGNAL_DTYPE)
        rc = lib().or_label_add(self._h, frame, _ptr(signal), len(signal))
        if rc != 0:
            raise RuntimeError(f"labeller refused frame {frame} ({rc})")

    def finish(self) -> LabelResult:
        L = lib()
        L.or_label_finish(self._h)
        ns, npx = L.or_label_n_spots(self._h), L.or_label_n_pixels(self._h)
        spots = np.zeros(ns, SPOT_DTYPE)
        pixels = np.zeros(npx, PIXEL_DTYPE)
        if ns:
            ctypes.memmove(_ptr(spots), L.or_label_spots(self._h), ns * SPOT_DTYPE.itemsize)
        if npx:
            ctypes.memmove(_ptr(pixels), L.or_label_pixels(self._h), npx * PIXEL_DTYPE.itemsize)
        c = np.zeros(6, np.uint64)
        L.or_label_counts(self._h, _ptr(c))
        return LabelResult(spots, pixels, dict(zip(COUNT_NAMES, map(int, c))))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().or_label_close(self._h)
            self._h = None


class RefLabeller:
    """The reference's own dials_spots::Labeller."""

    def __init__(self, height, width, min_spot_size=3, max_spot_size=1000,
                 max_separation=2.0, two_d=False):
        self._h = ref().ref_label_open(height, width, min_spot_size, max_spot_size,
                                       max_separation, int(two_d))
        if not self._h:
            raise ValueError("labeller options rejected")

    def add(self, frame: int, signal: np.ndarray) -> None:
        signal = np.ascontiguousarray(signal, SIGNAL_DTYPE)
        if ref().ref_label_add(self._h, frame, _ptr(signal), len(signal)) != 0:
            raise RuntimeError(f"reference labeller refused frame {frame}")

    def finish(self) -> LabelResult:
        R = ref()
        R.ref_label_finish(self._h)
        ns, npx = R.ref_label_n_spots(self._h), R.ref_label_n_pixels(self._h)
        spots = np.zeros(ns, SPOT_DTYPE)
        pixels = np.zeros(npx, PIXEL_DTYPE)
        if ns:
            R.ref_label_spots(self._h, _ptr(spots))
        if npx:
            R.ref_label_pixels(self._h, _ptr(pixels))
        c = np.zeros(6, np.uint64)
        R.ref_label_counts(self._h, _ptr(c))
        return LabelResult(spots, pixels, dict(zip(COUNT_NAMES, map(int, c))))

    def write_refl(self, path: str, shoeboxes: bool = True, identifier: str = "",
                   id: int = 0, panel: int = 0) -> None:
        """The reference's refl::write (src/spots/refl.cc:223-351) of the
        spots so far."""
        if ref().ref_label_write_refl_opts(self._h, path.encode(), int(shoeboxes), id,
                                           identifier.encode(), panel) != 0:
            raise RuntimeError("reference refl::write failed")

    def __del__(self):
        if getattr(self, "_h", None):
            ref().ref_label_close(self._h)
            self._h = None
