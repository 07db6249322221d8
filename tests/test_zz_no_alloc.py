"""The threshold entry point that allocates nothing
(sf_threshold_u32_device_noalloc), for callers that may not allocate device
memory themselves: a plugin living inside a host application whose own
allocator owns all device memory, or a detector-stream loop that must not
stall on an allocation. Its scratch is a fixed array inside the library.

Two calls in a row, on different frames, must each give exactly what the
ordinary device entry point (with a caller-supplied workspace) gives: the
same signal count, the same signal list byte for byte, the same bitmask and
the same word prefixes. The second call also shows that what the first call
left in the shared array does not leak into the next result.

This file is collected last so that a run stopping at its first failure has
already run every other test; it passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(L):
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    from sfgb import api
    f = L.sf_threshold_u32_device_noalloc
    f.argtypes = [vp, sz, sz, ctypes.POINTER(api.ThresholdParams), vp, sz, vp, vp, vp, vp]
    f.restype = ctypes.c_int
    return f


def _outputs(torch, h, w, capacity):
    dev = torch.device("cuda")
    wpr = (w + 31) // 32
    return dict(out=torch.zeros(capacity * 16, dtype=torch.uint8, device=dev),
                bits=torch.zeros(wpr * h, dtype=torch.int32, device=dev),
                count=torch.zeros(1, dtype=torch.int32, device=dev),
                prefix=torch.zeros(wpr * h, dtype=torch.int32, device=dev))


def _host(o, capacity):
    n = int(o["count"].item()) & 0xffffffff
    assert n <= capacity
    return (n, o["out"][: n * 16].cpu().numpy().tobytes(),
            o["bits"].cpu().numpy().tobytes(), o["prefix"].cpu().numpy().tobytes())


# The default parameters take the streamed lattice path; a non-integral
# sigma_b takes the tile path, which uses the array's staging list, tile bases
# and row totals as well.
@pytest.mark.parametrize("param_set", [{}, {"sigma_b": 6.5}], ids=["lattice", "tile"])
def test_noalloc_matches_workspace_entry_point_twice(param_set):
    torch = pytest.importorskip("torch")
    from sfgb import api, synth
    if not api.available():
        pytest.fail("no usable GB300: " + api.unavailable_reason())
    L = api.lib()
    noalloc = _bind(L)
    h, w, capacity = 1536, 1300, 200_000
    sweep = synth.Sweep(synth.preset("eiger_16m", height=h, width=w, n_frames=2,
                                     spots_per_frame=500.0, seed=4242))
    params = api.Params(**param_set).c()
    stream = torch.cuda.current_stream()
    ws = torch.empty(L.sf_workspace_bytes(h, w, capacity), dtype=torch.uint8,
                     device="cuda")
    for frame_no in (0, 1):
        frame = torch.from_numpy(sweep.frame(frame_no).view(np.int32)).cuda()
        ref = _outputs(torch, h, w, capacity)
        rc = L.sf_threshold_u32_device(
            frame.data_ptr(), h, w, ctypes.byref(params), ref["out"].data_ptr(),
            capacity, ref["bits"].data_ptr(), ref["count"].data_ptr(),
            ref["prefix"].data_ptr(), ws.data_ptr(), ws.numel(), stream.cuda_stream)
        assert rc == 0, api.last_error()
        got = _outputs(torch, h, w, capacity)
        rc = noalloc(frame.data_ptr(), h, w, ctypes.byref(params), got["out"].data_ptr(),
                     capacity, got["bits"].data_ptr(), got["count"].data_ptr(),
                     got["prefix"].data_ptr(), stream.cuda_stream)
        assert rc == 0, api.last_error()
        torch.cuda.synchronize()
        want_t, got_t = _host(ref, capacity), _host(got, capacity)
        assert want_t[0] > 0
        assert got_t == want_t, f"frame {frame_no}: no-alloc result differs"


def test_noalloc_refuses_capacity_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from sfgb import api
    if not api.available():
        pytest.fail("no usable GB300: " + api.unavailable_reason())
    noalloc = _bind(api.lib())
    params = api.Params().c()
    frame = torch.zeros(64 * 64, dtype=torch.int32, device="cuda")
    o = _outputs(torch, 64, 64, 16)
    # Refused on the host, before any device work is enqueued.
    rc = noalloc(frame.data_ptr(), 64, 64, ctypes.byref(params), o["out"].data_ptr(),
                 524_289, o["bits"].data_ptr(), o["count"].data_ptr(), None,
                 torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    assert "capacity" in api.last_error()
