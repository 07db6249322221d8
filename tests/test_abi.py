"""The C ABI without a GPU: the library loads, exports every entry point
include/sf_api.h declares, and refuses bad arguments before touching a
device."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO


def _declared(header):
    text = open(os.path.join(REPO, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sf_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    from sfgb import api
    L = api.lib()
    names = _declared("sf_api.h")
    assert "sf_find_u32" in names and "sf_threshold_u32_device" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_unavailable_without_a_device_says_why():
    from sfgb import api
    if api.available():
        pytest.skip("a device is present")
    assert api.unavailable_reason()


def test_defaults_are_the_references():
    from sfgb import api
    p = api.ThresholdParams()
    api.lib().sf_default_params(ctypes.byref(p))
    assert (p.algorithm, p.kernel_x, p.kernel_y, p.gain, p.sigma_b, p.sigma_s,
            p.min_local, p.global_threshold) == (0, 3, 3, 1.0, 6.0, 3.0, 2, 0.0)


def test_bad_arguments_are_refused_before_the_device():
    from sfgb import api
    L = api.lib()
    found = ctypes.c_size_t(7)
    out = np.zeros(4, api.SIGNAL_DTYPE)
    frame = np.zeros((4, 4), np.uint32)
    # null image, zero extents, index overflow: -1 (dext.cc:14-23)
    assert L.sf_find_u32(None, 4, 4, out.ctypes.data, 4, ctypes.byref(found)) == -1
    assert found.value == 0
    assert L.sf_find_u32(frame.ctypes.data, 0, 4, out.ctypes.data, 4,
                         ctypes.byref(found)) == -1
    assert L.sf_find_u32(frame.ctypes.data, 1 << 16, 1 << 16, out.ctypes.data, 4,
                         ctypes.byref(found)) == -1
    # kernel sizes other than 2..4, or non-square: unsupported (-4)
    p = api.Params(kernel_x=5, kernel_y=5).c()
    assert L.sf_find_u32_params(frame.ctypes.data, 4, 4, ctypes.byref(p),
                                out.ctypes.data, 4, ctypes.byref(found)) == -4
    p = api.Params(kernel_x=3, kernel_y=2).c()
    assert L.sf_find_u32_params(frame.ctypes.data, 4, 4, ctypes.byref(p),
                                out.ctypes.data, 4, ctypes.byref(found)) == -4
    p = api.Params(min_local=-1).c()
    assert L.sf_find_u32_params(frame.ctypes.data, 4, 4, ctypes.byref(p),
                                out.ctypes.data, 4, ctypes.byref(found)) == -1


def test_workspace_size_rejects_bad_shapes():
    from sfgb import api
    assert api.lib().sf_workspace_bytes(0, 5, 10) == 0
    assert api.lib().sf_workspace_bytes(4362, 4148, 1000) > 1000 * 16


def test_noalloc_limits_are_the_documented_ones():
    """The entry point that allocates nothing accepts a call when the
    workspace layout fits its fixed 32 MiB and capacity is at most 524,288
    records: an EIGER2 16M frame at the full capacity fits, one record more
    is refused, and so is a frame whose layout is too large. Refusals happen
    on the host, before any device is touched."""
    from sfgb import api
    L = api.lib()
    f = L.sf_threshold_u32_device_noalloc
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    f.argtypes = [vp, sz, sz, ctypes.POINTER(api.ThresholdParams), vp, sz, vp, vp, vp, vp]
    f.restype = ctypes.c_int
    limit = 32 << 20
    assert L.sf_workspace_bytes(4362, 4148, 524_288) <= limit
    params = api.Params().c()
    # Host-side refusals only: the pointers are never dereferenced.
    fake = 1 << 20
    assert f(fake, 4362, 4148, ctypes.byref(params), fake, 524_289, fake, fake, None,
             None) == -1
    assert "capacity" in api.last_error()
    # A 2^25-pixel frame 16 pixels wide has too many tiles for the array.
    h, w = (1 << 25) // 16, 16
    assert L.sf_workspace_bytes(h, w, 524_288) > limit
    assert f(fake, h, w, ctypes.byref(params), fake, 524_288, fake, fake, None, None) == -1
    assert "32 MiB" in api.last_error()
    # Every frame of up to 2^25 pixels with both sides at least 256 fits.
    for h in (256, 1024, 4096, 5793, 32768, 131072):
        w = (1 << 25) // h
        if w >= 256:
            assert L.sf_workspace_bytes(h, w, 524_288) <= limit, (h, w)
