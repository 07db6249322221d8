"""The CUDA threshold against the oracle and the reference's golden
fixtures, through the C ABI. Integer fields and the float background must
agree bit for bit: the masks and the signal lists are exact."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from sfgb import api as a
    if not a.available():
        pytest.fail("no usable GB300: " + a.unavailable_reason())
    return a


def _same(got, want, what=""):
    if got.tobytes() == want.tobytes():
        return
    gi, wi = set(got["index"].tolist()), set(want["index"].tolist())
    raise AssertionError(f"{what}: {len(got)} vs {len(want)} signal pixels; only GPU "
                         f"{sorted(gi - wi)[:5]}, only CPU {sorted(wi - gi)[:5]}")


def test_fused_cases_golden(api):
    # tests/spots/test_dext_fused.cc's 48 frames, u16 and u32.
    g = np.load(os.path.join(GOLDEN, "dext_fused_cases.npz"))
    for i in range(len(g["meta"])):
        _same(api.find(g[f"frame_{i}"]), g[f"signal_{i}"], f"case {i} {g['meta'][i]}")


def test_device_frames_golden(api):
    # tests/spots/test_dext_gpu.cc's 7 frames, as 16-bit and widened to 32.
    g = np.load(os.path.join(GOLDEN, "dext_device_frames.npz"))
    for i, name in enumerate(g["names"]):
        f = g[f"frame_{i}"]
        _same(api.find(f), g[f"signal16_{i}"], f"{name} u16")
        f32 = f.astype(np.uint32)
        if name == "entirely masked":
            f32[:] = 0xFFFFFFFF
        _same(api.find(f32), g[f"signal32_{i}"], f"{name} u32")


def test_sweep_frames_golden(api):
    g = np.load(os.path.join(GOLDEN, "sweep_small.npz"))
    for i, f in enumerate(g["frames"]):
        _same(api.find(f), g[f"signal_{i}"], f"sweep frame {i}")


@pytest.mark.parametrize("h,w", [(1, 1), (1, 40), (40, 1), (2, 3), (31, 33), (33, 31),
                                 (64, 64), (65, 97), (100, 1000)])
def test_ragged_shapes(api, h, w):
    from sfgb import synth
    p = synth.preset("plain_1m", height=max(h, 8), width=max(w, 8), n_frames=1,
                     spots_per_frame=max(1.0, h * w / 2000.0), n_hot=3, seed=h * 1000 + w)
    f = synth.Sweep(p).frame(0)[:h, :w].copy()
    for frame in (f, np.minimum(f, 0xFFFD).astype(np.uint16)):
        _same(api.find(frame, capacity=h * w), O.dext(frame), f"{h}x{w} {frame.dtype}")


@pytest.mark.parametrize("params", [
    dict(kernel_x=2, kernel_y=2), dict(kernel_x=4, kernel_y=4),
    dict(algorithm=1), dict(algorithm=1, kernel_x=2, kernel_y=2),
    dict(gain=1.5), dict(gain=0.8, sigma_b=4.5, sigma_s=2.5),
    dict(min_local=5), dict(min_local=0), dict(global_threshold=3.0),
    dict(global_threshold=2.5), dict(global_threshold=50.0), dict(min_local=30),
    dict(sigma_b=3.0, sigma_s=2.0)])
def test_parameters_against_oracle(api, params):
    # No reference test pins these settings; the oracle restatement is the
    # specification (it equals the reference at the defaults).
    from sfgb import synth
    sw = synth.Sweep(synth.preset("batch_4m", height=300, width=420, n_frames=2, seed=5,
                                  spots_per_frame=40.0, n_hot=15, row_band_start=77,
                                  row_band_len=3))
    f = sw.frame(1)
    P = api.Params(**params)
    po = O.Params(**params)
    _same(api.find(f, P, capacity=f.size), O.dext(f, po), f"{params} u32")
    f16 = np.minimum(f, 0xFFFD).astype(np.uint16)
    f16[f == 0xFFFFFFFF] = 0xFFFF
    _same(api.find(f16, P, capacity=f.size), O.dext(f16, po), f"{params} u16")


def test_sums_of_squares_wrap(api):
    # Values near 2^32 - 3: sum(I^2) over a window wraps modulo 2^64, and the
    # reference's uint64 arithmetic is reproduced exactly (dext.hh:23-25).
    rng = np.random.default_rng(7)
    f = rng.integers(0xFFFF0000, 0xFFFFFFFD, size=(96, 130), dtype=np.uint64).astype(np.uint32)
    low = rng.integers(0, 50, size=f.shape).astype(np.uint32)
    mix = rng.random(f.shape) < 0.3
    f[mix] = low[mix]
    f[::7, ::5] = 3
    f[10:20, 10:20] = 0xFFFFFFFE
    _same(api.find(f, capacity=f.size), O.dext(f), "wrapping sums")


def test_bright_dense_frame(api):
    # Poisson 20 with rings, saturated-overload pixels at 10^6 and hot pixels:
    # windows leave the integer route and take the double sequence.
    from sfgb import synth
    p = synth.preset("dense_16m", height=520, width=700, n_frames=2, spots_per_frame=400.0)
    f = synth.Sweep(p).frame(0)
    _same(api.find(f, capacity=f.size), O.dext(f), "dense")


def test_all_masked_and_all_zero(api):
    for v in (0xFFFFFFFE, 0xFFFFFFFF, 0):
        assert len(api.find(np.full((70, 90), v, np.uint32))) == 0


def test_capacity_overflow_is_refused(api):
    g = np.load(os.path.join(GOLDEN, "dext_device_frames.npz"))
    f = g["frame_5"].astype(np.uint32)
    n = len(g["signal32_5"])
    with pytest.raises(api.OverflowError_):
        api.find(f, capacity=n - 1)
    _same(api.find(f, capacity=n), g["signal32_5"], "exact capacity")


def test_device_resident_matches_host_path_and_mask(api):
    import torch
    from sfgb import synth
    sw = synth.Sweep(synth.preset("eiger_16m", height=1100, width=1050, n_frames=3,
                                  spots_per_frame=300.0, seed=9))
    f = sw.frame(2)
    dt = api.DeviceThreshold(f.shape[0], f.shape[1], word_prefix=True)
    dt(torch.from_numpy(f.view(np.int32)).cuda())
    got = dt.result()
    want, mask = O.dext(f, with_mask=True)
    _same(got, want, "device-resident")
    assert np.array_equal(dt.mask(), mask.astype(bool))
    # word_prefix: list position of each word's first strong pixel
    wp = dt.word_prefix.cpu().numpy().view(np.uint32).reshape(f.shape[0], -1)
    words = dt.bits.cpu().numpy().view(np.uint32).reshape(f.shape[0], -1)
    counts = np.array([bin(int(x)).count("1") for x in words.ravel()]).reshape(words.shape)
    assert np.array_equal(wp.ravel(), np.concatenate([[0], np.cumsum(counts.ravel())[:-1]]))


def test_full_size_eiger_frame(api):
    # One 4362 x 4148 frame with the EIGER2 module gaps, as the benchmark.
    from sfgb import synth
    sw = synth.Sweep(synth.preset("eiger_16m", n_frames=2))
    f = sw.frame(1)
    _same(api.find(f), O.dext(f), "16M frame")
