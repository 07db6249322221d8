"""The reflection-table writer (sf_refl_write, sf_label_write_refl) against
files the reference's own refl::write (src/spots/refl.cc:223-351) wrote for
the golden sweep's spot tables (tests/golden/make_golden.py): byte for byte,
with and without shoeboxes, with an identifier, id and panel, in 3-D and 2-D.
The host writer needs no GPU; the device writer builds the shoebox column in
device memory from a device labeller's pixels."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN

IDENT = "5b0f3c2e-9d41-4a7b-8e16-2c7d9a01f4b3"  # make_golden.REFL_IDENTIFIER
CASES = [  # fixture, spot table, writer options
    ("refl_small.refl", "3d", dict()),
    ("refl_small_opts.refl", "3d", dict(shoeboxes=False, identifier=IDENT, id=3, panel=1)),
    ("refl_small_2d.refl", "2d", dict(identifier=IDENT)),
]


def _golden(name):
    with open(os.path.join(GOLDEN, name), "rb") as f:
        return f.read()


def _first_difference(a, b):
    n = min(len(a), len(b))
    return next((i for i in range(n) if a[i] != b[i]), n)


@pytest.mark.parametrize("fixture,tag,opts", CASES)
def test_host_writer_matches_reference(tmp_path, fixture, tag, opts):
    from sfgb import labeller
    g = np.load(os.path.join(GOLDEN, "sweep_small.npz"))
    path = str(tmp_path / "t.refl")
    labeller.write_refl(path, g[f"spots_{tag}"], g[f"pixels_{tag}"], g["frames"].shape[2],
                        **opts)
    got, want = open(path, "rb").read(), _golden(fixture)
    assert got == want, (f"{fixture}: {len(got)} vs {len(want)} bytes, first difference at "
                         f"{_first_difference(got, want)}")


def test_host_writer_empty_table(tmp_path):
    from sfgb import labeller
    p = str(tmp_path / "empty.refl")
    labeller.write_refl(p, np.zeros(0, labeller.SPOT_DTYPE), np.zeros(0, labeller.PIXEL_DTYPE),
                        100)
    data = open(p, "rb").read()
    # [ "dials::af::reflection_table", 2, { ... "nrows": 0 ... } ]
    assert data[:2] == bytes([0x93, 0xBB]) and b"nrows\x00" in data


def test_host_writer_decodes_as_msgpack(tmp_path):
    msgpack = pytest.importorskip("msgpack")
    from sfgb import labeller
    g = np.load(os.path.join(GOLDEN, "sweep_small.npz"))
    spots = g["spots_3d"]
    p = str(tmp_path / "t.refl")
    labeller.write_refl(p, spots, g["pixels_3d"], g["frames"].shape[2], identifier=IDENT, id=3)
    kind, version, table = msgpack.unpackb(open(p, "rb").read(), strict_map_key=False)
    assert (kind, version) == ("dials::af::reflection_table", 2)
    assert table["identifiers"] == {3: IDENT} and table["nrows"] == len(spots)
    assert list(table["data"]) == sorted(table["data"])  # columns in name order
    typ, (rows, blob) = table["data"]["xyzobs.px.value"]
    assert typ == "vec3<double>" and rows == len(spots)
    assert np.array_equal(np.frombuffer(blob, "<f8").reshape(-1, 3), spots["position"])
    typ, (rows, blob) = table["data"]["n_signal"]
    assert np.array_equal(np.frombuffer(blob, "<i4"), spots["n_signal"].astype(np.int32))


def test_host_writer_refusals(tmp_path):
    from sfgb import labeller
    g = np.load(os.path.join(GOLDEN, "sweep_small.npz"))
    spots, pixels = g["spots_3d"].copy(), g["pixels_3d"]
    with pytest.raises(RuntimeError):  # refl.cc:227: a frame width of zero
        labeller.write_refl(str(tmp_path / "a.refl"), spots, pixels, 0)
    bad = spots.copy()
    bad["first"][-1] = len(pixels)  # its pixels are not in the array
    with pytest.raises(RuntimeError):
        labeller.write_refl(str(tmp_path / "b.refl"), bad, pixels, 320)
    with pytest.raises(RuntimeError):  # refl.cc:40: cannot write the file
        labeller.write_refl(str(tmp_path / "no" / "such" / "dir.refl"), spots, pixels, 320)


@pytest.mark.gpu
@pytest.mark.parametrize("fixture,tag,opts", CASES)
def test_device_writer_matches_reference(tmp_path, fixture, tag, opts):
    # The device labeller's spots of the golden sweep, written with the
    # shoebox column built on the device.
    from sfgb import labeller
    g = np.load(os.path.join(GOLDEN, "sweep_small.npz"))
    frames = g["frames"]
    d = labeller.DeviceLabeller(frames.shape[1], frames.shape[2], two_d=(tag == "2d"))
    for i in range(len(frames)):
        d.add(i, g[f"signal_{i}"])
    r = d.finish()
    assert O.spot_fields_equal(r.spots, g[f"spots_{tag}"])
    path = str(tmp_path / "d.refl")
    d.write_refl(path, **opts)
    got, want = open(path, "rb").read(), _golden(fixture)
    assert got == want, (f"{fixture}: {len(got)} vs {len(want)} bytes, first difference at "
                         f"{_first_difference(got, want)}")


@pytest.mark.gpu
def test_device_writer_on_a_threshold_sweep(tmp_path):
    # A sweep thresholded and labelled on the device: the device writer and
    # the host writer on the labeller's spots and pixels give one file.
    import torch
    from sfgb import api, labeller, synth
    p = synth.preset("eiger_16m", height=600, width=700, n_frames=6, spots_per_frame=60.0,
                     seed=31)
    sw = synth.Sweep(p)
    dt = api.DeviceThreshold(p.height, p.width)
    lab = labeller.DeviceLabeller(p.height, p.width)
    for i in range(p.n_frames):
        dt(torch.from_numpy(sw.frame(i).view(np.int32)).cuda())
        lab.add(i, dt.result())
    r = lab.finish()
    assert len(r.spots) > 0
    a, b = str(tmp_path / "dev.refl"), str(tmp_path / "host.refl")
    lab.write_refl(a, identifier=IDENT)
    labeller.write_refl(b, r.spots, r.pixels, p.width, identifier=IDENT)
    assert open(a, "rb").read() == open(b, "rb").read()
