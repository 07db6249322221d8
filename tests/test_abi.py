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
