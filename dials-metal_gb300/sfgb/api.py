"""ctypes bindings of the C ABI (include/sf_api.h, libsfgb.so).

The host-frame calls mirror the reference's threshold backend
(src/spots/dext_gpu.hh): `find()` is gpu::find<T>, returning the signal
pixels ascending by index, with the same 0 / -1 / -2 status meanings turned
into Python exceptions the way mxi_find turns them into runtime errors
(src/spots/find_spots.cc:410-416). The device calls take torch CUDA tensors
and enqueue on the current torch stream.

There is no CPU fallback: if the library is missing or no sm_103a device is
present these raise.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import _paths

SF_OK, SF_EBADARG, SF_EOVERFLOW, SF_ECUDA, SF_EUNSUPPORTED = 0, -1, -2, -3, -4
SF_EDATA = -6
DISPERSION_EXTENDED, DISPERSION = 0, 1

# src/spots/signal_pixel.hh:20-28
SIGNAL_DTYPE = np.dtype([("index", "<u4"), ("value", "<u4"), ("background", "<f4"),
                         ("population", "<u2"), ("reserved", "<u2")])


class ThresholdParams(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int), ("kernel_x", ctypes.c_int),
                ("kernel_y", ctypes.c_int), ("gain", ctypes.c_double),
                ("sigma_b", ctypes.c_double), ("sigma_s", ctypes.c_double),
                ("min_local", ctypes.c_int), ("global_threshold", ctypes.c_double)]


class FrameScan(ctypes.Structure):
    _fields_ = [("largest", ctypes.c_uint64), ("bad", ctypes.c_uint64),
                ("joins", ctypes.c_uint64), ("over", ctypes.c_uint64)]


class StageTimes(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("upload", "stage0", "stage1", "stage2", "fused", "copy", "sort")]


@dataclass
class Params:
    """Threshold parameters. Defaults are the reference's fixed ones."""
    algorithm: int = DISPERSION_EXTENDED
    kernel_x: int = 3
    kernel_y: int = 3
    gain: float = 1.0
    sigma_b: float = 6.0
    sigma_s: float = 3.0
    min_local: int = 2
    global_threshold: float = 0.0

    def c(self) -> ThresholdParams:
        return ThresholdParams(self.algorithm, self.kernel_x, self.kernel_y, self.gain,
                               self.sigma_b, self.sigma_s, self.min_local,
                               self.global_threshold)


class SpotFinderError(RuntimeError):
    pass


class OverflowError_(SpotFinderError):
    """More signal pixels than the output holds (status -2)."""


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = _paths.core_lib()
        if not os.path.exists(path):
            raise SpotFinderError(f"{path} is not built; run __graft_entry__.build()")
        L = ctypes.CDLL(path)
        vp, sz, u32p = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p
        L.sf_default_params.argtypes = [ctypes.POINTER(ThresholdParams)]
        L.sf_backend.restype = ctypes.c_char_p
        L.sf_available.restype = ctypes.c_int
        L.sf_unavailable_reason.restype = ctypes.c_char_p
        L.sf_memory_free.restype = sz
        L.sf_host_alloc.argtypes = [sz]
        L.sf_host_alloc.restype = vp
        L.sf_host_free.argtypes = [vp]
        L.sf_last_error.restype = ctypes.c_char_p
        for name in ("sf_find_u32", "sf_find_u16"):
            getattr(L, name).argtypes = [vp, sz, sz, vp, sz, ctypes.POINTER(sz)]
            getattr(L, name).restype = ctypes.c_int
        for name in ("sf_find_u32_params", "sf_find_u16_params"):
            getattr(L, name).argtypes = [vp, sz, sz, ctypes.POINTER(ThresholdParams), vp,
                                         sz, ctypes.POINTER(sz)]
            getattr(L, name).restype = ctypes.c_int
        L.sf_profile_stages.argtypes = [ctypes.c_int]
        L.sf_profiling.restype = ctypes.c_int
        L.sf_last_stage_times.argtypes = [ctypes.POINTER(StageTimes)]
        L.sf_workspace_bytes.argtypes = [sz, sz, sz]
        L.sf_workspace_bytes.restype = sz
        for name in ("sf_threshold_u32_device", "sf_threshold_u16_device"):
            getattr(L, name).argtypes = [vp, sz, sz, ctypes.POINTER(ThresholdParams), vp,
                                         sz, u32p, u32p, u32p, vp, sz, vp]
            getattr(L, name).restype = ctypes.c_int
        L.sf_batch_workspace_bytes.argtypes = [sz, sz, sz, sz]
        L.sf_batch_workspace_bytes.restype = sz
        for name in ("sf_threshold_u32_batch_device", "sf_threshold_u16_batch_device"):
            getattr(L, name).argtypes = [vp, sz, sz, sz, ctypes.POINTER(ThresholdParams), vp,
                                         sz, u32p, u32p, u32p, vp, sz, vp]
            getattr(L, name).restype = ctypes.c_int
        szp = ctypes.POINTER(sz)
        L.sf_mixed_batch_workspace_bytes.argtypes = [sz, szp, szp, sz]
        L.sf_mixed_batch_workspace_bytes.restype = sz
        L.sf_mixed_batch_mask_words.argtypes = [sz, szp, szp]
        L.sf_mixed_batch_mask_words.restype = sz
        L.sf_threshold_u32_mixed_batch_device.argtypes = [vp, szp, szp, sz,
                                                          ctypes.POINTER(ThresholdParams), vp,
                                                          sz, u32p, u32p, u32p, vp, sz, vp]
        L.sf_threshold_u32_mixed_batch_device.restype = ctypes.c_int
        L.sf_plan_create.argtypes = [sz, sz, sz, sz, ctypes.POINTER(ThresholdParams)]
        L.sf_plan_create.restype = vp
        L.sf_plan_destroy.argtypes = [vp]
        for name in ("sf_plan_run", "sf_plan_tune"):
            getattr(L, name).argtypes = [vp, vp, sz, vp]
            getattr(L, name).restype = ctypes.c_int
        L.sf_plan_configure.argtypes = [vp, ctypes.c_int, sz]
        L.sf_plan_configure.restype = ctypes.c_int
        L.sf_plan_frames_per_launch.argtypes = [vp]
        L.sf_plan_frames_per_launch.restype = sz
        L.sf_plan_run_rows.argtypes = [vp]
        L.sf_plan_run_rows.restype = ctypes.c_int
        L.sf_plan_graphs.argtypes = [vp]
        L.sf_plan_graphs.restype = sz
        for name in ("sf_plan_lists", "sf_plan_counts", "sf_plan_masks"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = vp
        L.sf_plan_result.argtypes = [vp, sz, vp, sz, ctypes.POINTER(sz)]
        L.sf_plan_result.restype = ctypes.c_int
        L.sf_frame_bytes.argtypes = [sz, sz, ctypes.c_uint]
        L.sf_frame_bytes.restype = sz
        for name in ("sf_decompress_image", "sf_decompress_device"):
            getattr(L, name).argtypes = [vp, sz, ctypes.c_char_p, ctypes.c_uint, sz, sz, vp, sz]
            getattr(L, name).restype = ctypes.c_int
        L.sf_find_compressed.argtypes = [vp, sz, ctypes.c_char_p, ctypes.c_uint, sz, sz,
                                         ctypes.POINTER(ThresholdParams), vp, sz,
                                         ctypes.POINTER(sz)]
        L.sf_find_compressed.restype = ctypes.c_int
        L.sf_find_narrowed.argtypes = [vp, sz, ctypes.c_char_p, sz, sz,
                                       ctypes.POINTER(ThresholdParams), vp, sz,
                                       ctypes.POINTER(sz), ctypes.POINTER(ctypes.c_uint32)]
        L.sf_find_narrowed.restype = ctypes.c_int
        L.sf_scan_device.argtypes = [vp, sz, ctypes.c_uint, ctypes.POINTER(FrameScan)]
        L.sf_scan_device.restype = ctypes.c_int
        L.sf_scan_compressed.argtypes = [vp, sz, ctypes.c_char_p, ctypes.c_uint, sz, sz,
                                         ctypes.POINTER(FrameScan)]
        L.sf_scan_compressed.restype = ctypes.c_int
        _lib = L
    return _lib


def backend() -> str:
    return lib().sf_backend().decode()


def available() -> bool:
    return bool(lib().sf_available())


def unavailable_reason() -> str:
    return lib().sf_unavailable_reason().decode()


def last_error() -> str:
    return lib().sf_last_error().decode()


def _check(rc: int, what: str) -> None:
    if rc == SF_OK:
        return
    if rc == SF_EOVERFLOW:
        raise OverflowError_(f"{what}: more signal pixels than the output holds")
    if rc == SF_EBADARG:
        raise ValueError(f"{what}: bad argument")
    if rc == SF_EUNSUPPORTED:
        raise SpotFinderError(f"{what}: unsupported by this backend")
    raise SpotFinderError(f"{what}: {last_error()}")


def find(frame: np.ndarray, params: Params | None = None,
         capacity: int | None = None) -> np.ndarray:
    """Threshold one host frame (uint16/uint32, (h, w)); the signal pixels
    ascending by index. capacity defaults to the reference's device bound,
    one record per 16 bytes of frame (src/spots/dext_cuda.cu:741)."""
    frame = np.ascontiguousarray(frame)
    if frame.ndim != 2:
        raise ValueError("a frame is two-dimensional")
    h, w = frame.shape
    if capacity is None:
        capacity = max(1, frame.nbytes // 16)
    out = np.empty(capacity, SIGNAL_DTYPE)
    found = ctypes.c_size_t(0)
    L = lib()
    if frame.dtype == np.uint32:
        fn, fnp = L.sf_find_u32, L.sf_find_u32_params
    elif frame.dtype == np.uint16:
        fn, fnp = L.sf_find_u16, L.sf_find_u16_params
    else:
        raise TypeError("frames are uint16 or uint32")
    if params is None:
        rc = fn(frame.ctypes.data, h, w, out.ctypes.data, capacity, ctypes.byref(found))
    else:
        p = params.c()
        rc = fnp(frame.ctypes.data, h, w, ctypes.byref(p), out.ctypes.data, capacity,
                 ctypes.byref(found))
    _check(rc, "threshold")
    return out[:found.value].copy()


class DataError(SpotFinderError):
    """A compressed chunk that does not describe its frame: where the
    reference's decompress::image throws std::runtime_error."""


def _chunk_bytes(data) -> np.ndarray:
    if isinstance(data, np.ndarray):
        return np.ascontiguousarray(data).view(np.uint8).ravel()
    return np.frombuffer(bytes(data), np.uint8)


def _check_chunk(rc: int, what: str) -> None:
    if rc == SF_EDATA:
        raise DataError(last_error())
    if rc == SF_EUNSUPPORTED:
        raise SpotFinderError(f"{what}: {last_error()}")
    _check(rc, what)


def frame_bytes(height: int, width: int, bit_depth: int) -> int:
    """decompress::frame_bytes (src/spots/decompress.hh:18-19)."""
    return lib().sf_frame_bytes(height, width, bit_depth)


def decompress_image(data, algorithm: str, bit_depth: int, height: int,
                     width: int) -> np.ndarray:
    """decompress::image (src/spots/decompress.hh:28-30), decoded on the
    device: a chunk as HDF5 stored it ("bslz4", "lz4", or "" for none) to a
    (height, width) host frame. Raises DataError where the reference throws,
    with its text."""
    buf = _chunk_bytes(data)
    n = frame_bytes(height, width, bit_depth)
    dtype = {16: np.uint16, 32: np.uint32}.get(bit_depth, np.uint8)
    out = np.empty(max(n, 1), np.uint8)
    rc = lib().sf_decompress_image(buf.ctypes.data if buf.size else None, buf.size,
                                   algorithm.encode(), bit_depth, height, width,
                                   out.ctypes.data, n)
    _check_chunk(rc, "decompress")
    out = out[:n]
    return out.view(dtype).reshape(height, width) if dtype is not np.uint8 else out


def decompress_device(data, algorithm: str, bit_depth: int, height: int, width: int,
                      out=None):
    """As decompress_image, into a device tensor (torch, cuda; allocated
    when `out` is None); returns it once the frame is there."""
    import torch
    buf = _chunk_bytes(data)
    n = frame_bytes(height, width, bit_depth)
    if out is None:
        dt = {16: torch.int16, 32: torch.int32}.get(bit_depth, torch.uint8)
        out = torch.empty((height, width) if dt is not torch.uint8 else (max(n, 1),), dtype=dt,
                          device="cuda")
    rc = lib().sf_decompress_device(buf.ctypes.data if buf.size else None, buf.size,
                                    algorithm.encode(), bit_depth, height, width,
                                    out.data_ptr(), out.numel() * out.element_size())
    _check_chunk(rc, "decompress")
    return out


def find_compressed(data, algorithm: str, bit_depth: int, height: int, width: int,
                    params: Params | None = None, capacity: int | None = None) -> np.ndarray:
    """The chunk decoded on the device and thresholded there
    (sf_find_compressed): the signal pixels ascending by index."""
    buf = _chunk_bytes(data)
    if capacity is None:
        capacity = max(1, frame_bytes(height, width, bit_depth) // 16)
    out = np.empty(capacity, SIGNAL_DTYPE)
    found = ctypes.c_size_t(0)
    p = params.c() if params is not None else None
    rc = lib().sf_find_compressed(buf.ctypes.data if buf.size else None, buf.size,
                                  algorithm.encode(), bit_depth, height, width,
                                  ctypes.byref(p) if p is not None else None, out.ctypes.data,
                                  capacity, ctypes.byref(found))
    _check_chunk(rc, "threshold")
    return out[:found.value].copy()


class NarrowError(DataError):
    """A 32-bit frame with a valid count too large for 16 bits (the
    reference's --gpu-force refusal, src/spots/find_spots.cc:786-792)."""

    def __init__(self, message: str, offending: int):
        super().__init__(message)
        self.offending = offending


def find_narrowed(data, algorithm: str, height: int, width: int,
                  params: Params | None = None, capacity: int | None = None) -> np.ndarray:
    """--gpu-force on the device (sf_find_narrowed): a 32-bit frame or chunk
    narrowed to 16 bits (narrow_to_16) and thresholded as a 16-bit frame.
    Raises NarrowError (with .offending) for counts of 0xFFFD or more."""
    buf = _chunk_bytes(data)
    if capacity is None:
        capacity = max(1, height * width * 4 // 16)
    out = np.empty(capacity, SIGNAL_DTYPE)
    found = ctypes.c_size_t(0)
    worst = ctypes.c_uint32(0)
    p = params.c() if params is not None else None
    rc = lib().sf_find_narrowed(buf.ctypes.data if buf.size else None, buf.size,
                                algorithm.encode(), height, width,
                                ctypes.byref(p) if p is not None else None, out.ctypes.data,
                                capacity, ctypes.byref(found), ctypes.byref(worst))
    if rc == SF_EDATA and worst.value >= 0xFFFD:
        raise NarrowError(last_error(), worst.value)
    _check_chunk(rc, "threshold")
    return out[:found.value].copy()


def _scan_tuple(s: "FrameScan") -> tuple:
    return (int(s.largest), int(s.bad), int(s.joins), int(s.over))


def scan_device(frame) -> tuple:
    """mxi_max's scan<T> (apps/mxi_max.cc:47-67) of a device frame (a torch
    int16/int32 tensor holding 16- or 32-bit pixels): (largest non-marker
    count, bad pixels, tile joins, valid pixels at 0xFFFD or above)."""
    depth = frame.element_size() * 8
    s = FrameScan()
    _check(lib().sf_scan_device(frame.data_ptr(), frame.numel(), depth, ctypes.byref(s)),
           "scan")
    return _scan_tuple(s)


def scan_compressed(data, algorithm: str, bit_depth: int, height: int, width: int) -> tuple:
    """mxi_max's worker step (decompress::image, then scan<T>) with the chunk
    decoded and scanned on the device."""
    buf = _chunk_bytes(data)
    s = FrameScan()
    rc = lib().sf_scan_compressed(buf.ctypes.data if buf.size else None, buf.size,
                                  algorithm.encode(), bit_depth, height, width, ctypes.byref(s))
    _check_chunk(rc, "scan")
    return _scan_tuple(s)


def profile_stages(on: bool) -> None:
    lib().sf_profile_stages(int(on))


def last_stage_times() -> dict:
    t = StageTimes()
    lib().sf_last_stage_times(ctypes.byref(t))
    return {n: getattr(t, n) for n, _ in StageTimes._fields_}


class DeviceThreshold:
    """Device-resident threshold of frames already in HBM (torch tensors).

    Holds the output list, bitmask, count and workspace for frames of one
    shape, and enqueues on the given (default: current) torch stream.
    """

    def __init__(self, height: int, width: int, capacity: int | None = None,
                 params: Params | None = None, dtype=None, word_prefix: bool = False):
        import torch
        self.h, self.w = height, width
        self.capacity = capacity if capacity is not None else max(1, height * width // 4)
        self.params = (params or Params()).c()
        dev = torch.device("cuda")
        self.out = torch.empty(self.capacity * 16, dtype=torch.uint8, device=dev)
        self.words_per_row = (width + 31) // 32
        self.bits = torch.empty(self.words_per_row * height, dtype=torch.int32, device=dev)
        self.count = torch.zeros(1, dtype=torch.int32, device=dev)
        self.word_prefix = (torch.empty(self.words_per_row * height, dtype=torch.int32,
                                        device=dev) if word_prefix else None)
        nbytes = lib().sf_workspace_bytes(height, width, self.capacity)
        if nbytes == 0:
            raise ValueError("frame shape rejected")
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=dev)

    def __call__(self, image, stream=None) -> None:
        import torch
        if image.device.type != "cuda" or not image.is_contiguous():
            raise ValueError("a contiguous CUDA tensor")
        if tuple(image.shape[-2:]) != (self.h, self.w):
            raise ValueError("frame shape differs from this threshold's")
        s = stream if stream is not None else torch.cuda.current_stream()
        L = lib()
        if image.dtype in (torch.int32, torch.uint32):
            fn = L.sf_threshold_u32_device
        elif image.dtype in (torch.int16, torch.uint16):
            fn = L.sf_threshold_u16_device
        else:
            raise TypeError("frames are 16- or 32-bit")
        rc = fn(image.data_ptr(), self.h, self.w, ctypes.byref(self.params),
                self.out.data_ptr(), self.capacity, self.bits.data_ptr(),
                self.count.data_ptr(),
                self.word_prefix.data_ptr() if self.word_prefix is not None else None,
                self.workspace.data_ptr(), self.workspace.numel(), s.cuda_stream)
        _check(rc, "device threshold")

    def result(self) -> np.ndarray:
        """Synchronise and return the signal list (host copy)."""
        import torch
        torch.cuda.current_stream().synchronize()
        n = int(self.count.item()) & 0xffffffff
        if n > self.capacity:
            raise OverflowError_(f"{n} signal pixels, capacity {self.capacity}")
        raw = self.out[: n * 16].cpu().numpy()
        return raw.view(SIGNAL_DTYPE).copy()

    def mask(self) -> np.ndarray:
        """The strong-pixel mask as booleans (h, w) (host copy)."""
        words = self.bits.cpu().numpy().view(np.uint32).reshape(self.h, self.words_per_row)
        bits = np.unpackbits(words.view(np.uint8).reshape(self.h, -1), axis=1,
                             bitorder="little")
        return bits[:, : self.w].astype(bool)


MAX_BATCH = 64


class MixedBatch:
    """Batched device threshold of frames of different shapes
    (sf_threshold_u32_mixed_batch_device): up to MAX_BATCH 32-bit frames in
    HBM per call, each with its own shape, one launch sequence on the
    reference's window; each frame's list, mask and count as a single-frame
    call gives. Outputs are laid out for the batch's envelope."""

    def __init__(self, shapes, capacity: int | None = None, params: Params | None = None,
                 word_prefix: bool = False):
        import torch
        n = len(shapes)
        if not 1 <= n <= MAX_BATCH:
            raise ValueError(f"1 to {MAX_BATCH} frames per batch")
        self.shapes = [(int(h), int(w)) for h, w in shapes]
        self.n = n
        self._hs = (ctypes.c_size_t * n)(*[h for h, _ in self.shapes])
        self._ws = (ctypes.c_size_t * n)(*[w for _, w in self.shapes])
        H = max(h for h, _ in self.shapes)
        W = max(w for _, w in self.shapes)
        self.capacity = capacity if capacity is not None else max(1, H * W // 4)
        self.params = (params or Params()).c()
        L = lib()
        self.slot = L.sf_mixed_batch_mask_words(n, self._hs, self._ws)
        nbytes = L.sf_mixed_batch_workspace_bytes(n, self._hs, self._ws, self.capacity)
        if nbytes == 0 or self.slot == 0:
            raise ValueError("frame shapes or batch size rejected")
        dev = torch.device("cuda")
        self.out = torch.empty((n, self.capacity * 16), dtype=torch.uint8, device=dev)
        self.bits = torch.empty((n, self.slot), dtype=torch.int32, device=dev)
        self.counts = torch.zeros(n, dtype=torch.int32, device=dev)
        self.word_prefix = (torch.empty((n, self.slot), dtype=torch.int32, device=dev)
                            if word_prefix else None)
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        self._ptrs = (ctypes.c_void_p * MAX_BATCH)()

    def __call__(self, frames, stream=None) -> None:
        """frames: contiguous 32-bit CUDA tensors, frame j of shapes[j]."""
        import torch
        frames = list(frames)
        if len(frames) != self.n:
            raise ValueError(f"{self.n} frames")
        for j, f in enumerate(frames):
            if f.device.type != "cuda" or not f.is_contiguous() or \
                    f.dtype not in (torch.int32, torch.uint32):
                raise ValueError("contiguous 32-bit CUDA tensors")
            if tuple(f.shape) != self.shapes[j]:
                raise ValueError(f"frame {j} is not {self.shapes[j]}")
            self._ptrs[j] = f.data_ptr()
        s = stream if stream is not None else torch.cuda.current_stream()
        rc = lib().sf_threshold_u32_mixed_batch_device(
            ctypes.cast(self._ptrs, ctypes.c_void_p), self._hs, self._ws, self.n,
            ctypes.byref(self.params), self.out.data_ptr(), self.capacity,
            self.bits.data_ptr(), self.counts.data_ptr(),
            self.word_prefix.data_ptr() if self.word_prefix is not None else None,
            self.workspace.data_ptr(), self.workspace.numel(), s.cuda_stream)
        _check(rc, "mixed-shape batched device threshold")

    def count(self, j: int) -> int:
        import torch
        torch.cuda.current_stream().synchronize()
        return int(self.counts[j].item()) & 0xffffffff

    def result(self, j: int) -> np.ndarray:
        n = self.count(j)
        if n > self.capacity:
            raise OverflowError_(f"{n} signal pixels, capacity {self.capacity}")
        return self.out[j, : n * 16].cpu().numpy().view(SIGNAL_DTYPE).copy()

    def words(self, j: int, which=None) -> np.ndarray:
        """Frame j's mask words (or word positions), its own rows."""
        h, w = self.shapes[j]
        src = self.bits if which is None else which
        return src[j, : (w + 31) // 32 * h].cpu().numpy().view(np.uint32)

    def mask(self, j: int) -> np.ndarray:
        h, w = self.shapes[j]
        words = self.words(j).reshape(h, (w + 31) // 32)
        bits = np.unpackbits(words.view(np.uint8).reshape(h, -1), axis=1, bitorder="little")
        return bits[:, :w].astype(bool)


class DeviceBatch:
    """Batched device threshold (sf_threshold_*_batch_device): up to
    MAX_BATCH same-shaped frames already in HBM per call, one launch
    sequence, each frame's list, mask and count as a single-frame call gives.
    """

    def __init__(self, height: int, width: int, max_frames: int,
                 capacity: int | None = None, params: Params | None = None,
                 word_prefix: bool = False):
        import torch
        if not 1 <= max_frames <= MAX_BATCH:
            raise ValueError(f"1 to {MAX_BATCH} frames per batch")
        self.h, self.w, self.n = height, width, max_frames
        self.capacity = capacity if capacity is not None else max(1, height * width // 4)
        self.params = (params or Params()).c()
        dev = torch.device("cuda")
        self.words_per_row = (width + 31) // 32
        self.words = self.words_per_row * height
        self.out = torch.empty((max_frames, self.capacity * 16), dtype=torch.uint8, device=dev)
        self.bits = torch.empty((max_frames, self.words), dtype=torch.int32, device=dev)
        self.counts = torch.zeros(max_frames, dtype=torch.int32, device=dev)
        self.word_prefix = (torch.empty((max_frames, self.words), dtype=torch.int32,
                                        device=dev) if word_prefix else None)
        nbytes = lib().sf_batch_workspace_bytes(max_frames, height, width, self.capacity)
        if nbytes == 0:
            raise ValueError("frame shape or batch size rejected")
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        self._ptrs = (ctypes.c_void_p * MAX_BATCH)()
        self.last = 0

    def __call__(self, frames, stream=None) -> None:
        """frames: a sequence of contiguous (h, w) CUDA tensors, or one
        (n, h, w) tensor; all 32-bit or all 16-bit."""
        import torch
        frames = list(frames)
        if not 1 <= len(frames) <= self.n:
            raise ValueError(f"1 to {self.n} frames")
        dt = frames[0].dtype
        for f in frames:
            if f.device.type != "cuda" or not f.is_contiguous() or f.dtype != dt:
                raise ValueError("contiguous CUDA tensors of one dtype")
            if tuple(f.shape) != (self.h, self.w):
                raise ValueError("frame shape differs from this batch's")
        for j, f in enumerate(frames):
            self._ptrs[j] = f.data_ptr()
        s = stream if stream is not None else torch.cuda.current_stream()
        L = lib()
        if dt in (torch.int32, torch.uint32):
            fn = L.sf_threshold_u32_batch_device
        elif dt in (torch.int16, torch.uint16):
            fn = L.sf_threshold_u16_batch_device
        else:
            raise TypeError("frames are 16- or 32-bit")
        rc = fn(ctypes.cast(self._ptrs, ctypes.c_void_p), len(frames), self.h, self.w,
                ctypes.byref(self.params), self.out.data_ptr(), self.capacity,
                self.bits.data_ptr(), self.counts.data_ptr(),
                self.word_prefix.data_ptr() if self.word_prefix is not None else None,
                self.workspace.data_ptr(), self.workspace.numel(), s.cuda_stream)
        _check(rc, "batched device threshold")
        self.last = len(frames)

    def result(self, j: int) -> np.ndarray:
        """Synchronise and return frame j's signal list (host copy)."""
        import torch
        torch.cuda.current_stream().synchronize()
        n = int(self.counts[j].item()) & 0xffffffff
        if n > self.capacity:
            raise OverflowError_(f"{n} signal pixels, capacity {self.capacity}")
        return self.out[j, : n * 16].cpu().numpy().view(SIGNAL_DTYPE).copy()

    def mask(self, j: int) -> np.ndarray:
        words = self.bits[j].cpu().numpy().view(np.uint32).reshape(self.h, self.words_per_row)
        bits = np.unpackbits(words.view(np.uint8).reshape(self.h, -1), axis=1,
                             bitorder="little")
        return bits[:, : self.w].astype(bool)


class Plan:
    """A batch plan (sf_plan_*): tuned run length and CUDA-graph replay of
    the batched threshold for one frame shape; outputs stay on the device."""

    def __init__(self, height: int, width: int, max_frames: int,
                 capacity: int | None = None, params: Params | None = None):
        self.h, self.w, self.n = height, width, max_frames
        self.capacity = capacity if capacity is not None else max(1, height * width // 4)
        self.words = (width + 31) // 32 * height
        p = (params or Params()).c()
        self._p = lib().sf_plan_create(height, width, max_frames, self.capacity,
                                       ctypes.byref(p))
        if not self._p:
            raise SpotFinderError("plan: " + last_error())
        self._ptrs = (ctypes.c_void_p * MAX_BATCH)()

    def close(self):
        if self._p:
            lib().sf_plan_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _set(self, frames):
        frames = list(frames)
        if not 1 <= len(frames) <= self.n:
            raise ValueError(f"1 to {self.n} frames")
        for j, f in enumerate(frames):
            if tuple(f.shape) != (self.h, self.w) or not f.is_contiguous():
                raise ValueError("contiguous frames of the plan's shape")
            self._ptrs[j] = f.data_ptr()
        return len(frames)

    def __call__(self, frames, stream=None) -> None:
        import torch
        n = self._set(frames)
        s = stream if stream is not None else torch.cuda.current_stream()
        _check(lib().sf_plan_run(self._p, ctypes.cast(self._ptrs, ctypes.c_void_p), n,
                                 s.cuda_stream), "plan run")

    def tune(self, frames, stream=None) -> int:
        import torch
        n = self._set(frames)
        s = stream if stream is not None else torch.cuda.current_stream()
        _check(lib().sf_plan_tune(self._p, ctypes.cast(self._ptrs, ctypes.c_void_p), n,
                                  s.cuda_stream), "plan tune")
        return lib().sf_plan_run_rows(self._p)

    def configure(self, run_rows: int = 0, frames_per_launch: int = 0) -> None:
        _check(lib().sf_plan_configure(self._p, run_rows, frames_per_launch), "plan configure")

    @property
    def frames_per_launch(self) -> int:
        """The tuned frames per launch sequence (0: all of a call's)."""
        return int(lib().sf_plan_frames_per_launch(self._p))

    @property
    def graphs(self) -> int:
        return int(lib().sf_plan_graphs(self._p))

    def result(self, j: int) -> np.ndarray:
        """Wait for the plan's work and return frame j's list (host copy)."""
        out = np.empty(self.capacity, SIGNAL_DTYPE)
        found = ctypes.c_size_t(0)
        rc = lib().sf_plan_result(self._p, j, out.ctypes.data, self.capacity,
                                  ctypes.byref(found))
        _check(rc, "plan result")
        return out[: found.value].copy()

    @property
    def lists_ptr(self) -> int:
        """Device address of frame 0's list (frame j's at + j * capacity records)."""
        return lib().sf_plan_lists(self._p)

    @property
    def counts_ptr(self) -> int:
        """Device address of the per-frame counts (uint32)."""
        return lib().sf_plan_counts(self._p)

    def mask(self, j: int) -> np.ndarray:
        """Frame j's strong-pixel mask as booleans (h, w), after the plan's
        work (host copy)."""
        words_per_row = (self.w + 31) // 32
        words = np.empty(self.words, np.uint32)
        cudart = _cudart()
        if cudart.cudaDeviceSynchronize() != 0:
            raise SpotFinderError("cudaDeviceSynchronize failed")
        src = lib().sf_plan_masks(self._p) + j * self.words * 4
        if cudart.cudaMemcpy(ctypes.c_void_p(words.ctypes.data), ctypes.c_void_p(src),
                             ctypes.c_size_t(words.nbytes), 2) != 0:
            raise SpotFinderError("reading a plan's mask failed")
        bits = np.unpackbits(words.view(np.uint8).reshape(self.h, words_per_row * 4), axis=1,
                             bitorder="little")
        return bits[:, : self.w].astype(bool)


_cudart_lib = None


def _cudart() -> ctypes.CDLL:
    """The CUDA runtime libsfgb.so was linked against (already loaded)."""
    global _cudart_lib
    if _cudart_lib is None:
        lib()
        _cudart_lib = ctypes.CDLL("libcudart.so.13")
        _cudart_lib.cudaMemcpy.restype = ctypes.c_int
        _cudart_lib.cudaDeviceSynchronize.restype = ctypes.c_int
    return _cudart_lib
