"""The oracle restatement against fixtures produced by the reference's own
CPU code (tests/golden/make_golden.py): bit-exact signal lists from
dext<T>() (src/spots/dext.cc) and byte-exact spot tables from
dials_spots::Labeller (src/spots/dials_spots.cc)."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_fused_cases_bit_exact():
    # tests/spots/test_dext_fused.cc:109-119: 8 sizes x 3 means x 2 types.
    g = _load("dext_fused_cases.npz")
    n = len(g["meta"])
    assert n == 48
    for i in range(n):
        got = O.dext(g[f"frame_{i}"])
        want = g[f"signal_{i}"]
        assert got.tobytes() == want.tobytes(), f"case {i} {g['meta'][i]}"


def test_device_frames_bit_exact():
    # tests/spots/test_dext_gpu.cc:147-171, in 16 bits and widened to 32.
    g = _load("dext_device_frames.npz")
    for i, name in enumerate(g["names"]):
        f = g[f"frame_{i}"]
        assert O.dext(f).tobytes() == g[f"signal16_{i}"].tobytes(), name
        f32 = f.astype(np.uint32)
        if name == "entirely masked":
            f32 = np.full(f.shape, 0xFFFFFFFF, np.uint32)
        assert O.dext(f32).tobytes() == g[f"signal32_{i}"].tobytes(), name


def test_entirely_masked_is_empty():
    # tests/spots/test_dext_squares.cc: an all-sentinel frame finds nothing.
    for dt, v in ((np.uint16, 0xFFFE), (np.uint32, 0xFFFFFFFE)):
        assert len(O.dext(np.full((40, 50), v, dt))) == 0


def test_bad_arguments():
    # dext.cc:14-23: zero extents are refused.
    with pytest.raises(ValueError):
        O.dext(np.zeros((0, 5), np.uint32))


@pytest.mark.parametrize("tag,two_d,skip", [("3d", False, None), ("2d", True, None),
                                             ("gap", False, 7)])
def test_sweep_labelling_matches_reference(tag, two_d, skip):
    g = _load("sweep_small.npz")
    frames = g["frames"]
    lab = O.Labeller(frames.shape[1], frames.shape[2], two_d=two_d)
    for i, f in enumerate(frames):
        s = O.dext(f)
        assert s.tobytes() == g[f"signal_{i}"].tobytes(), f"frame {i}"
        if i != skip:
            lab.add(i, s)
    r = lab.finish()
    assert O.spot_fields_equal(r.spots, g[f"spots_{tag}"])
    assert r.pixels.tobytes() == g[f"pixels_{tag}"].tobytes()
    assert [r.counts[k] for k in O.COUNT_NAMES] == list(map(int, g[f"counts_{tag}"]))


def test_defaults_reduce_to_reference_with_explicit_params():
    g = _load("dext_device_frames.npz")
    f = g["frame_5"].astype(np.uint32)
    p = O.Params(gain=1.0, sigma_b=6.0, sigma_s=3.0, min_local=2, kernel_x=3,
                 kernel_y=3, global_threshold=0.0)
    assert O.dext(f, p).tobytes() == g["signal32_5"].tobytes()


@pytest.mark.skipif(not O.ref_available(), reason="reference tree not built here")
def test_oracle_against_live_reference_other_seeds():
    # Wider than the fixtures: the reference's generator at more seeds.
    for seed in range(100, 106):
        for dt in (np.uint16, np.uint32):
            f = O.ref_fused_make(97, 131, seed, 3.0, dt)
            assert O.dext(f).tobytes() == O.ref_dext(f).tobytes()
