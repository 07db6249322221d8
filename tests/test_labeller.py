"""3-D spot labelling: the device labeller (sf_label_*) against the oracle
restatement of dials_spots::Labeller, which is itself pinned to the
reference's own output (tests/golden/sweep_small.npz).

The known-answer cases restate tests/spots/test_dials_spots.cc:76-417 (a
1-2-1 row, a streak over three frames in 3-D and 2-D, a missing frame, row
wrap and diagonals are not edges, no early emission, the size filters and the
peak-centroid filter). Spot tables must agree field for field, bit for bit;
the kept pixels and counts exactly.
"""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN

H, W = 8, 10


def flat(indices, value=1):
    s = np.zeros(len(indices), O.SIGNAL_DTYPE)
    s["index"] = indices
    s["value"] = value
    return s


def pix(pairs):
    s = np.zeros(len(pairs), O.SIGNAL_DTYPE)
    s["index"] = [p[0] for p in pairs]
    s["value"] = [p[1] for p in pairs]
    return s


PLAIN = dict(max_separation=0.0)
CASES = {
    "one_two_one": (PLAIN, [(0, pix([(0, 1), (1, 2), (2, 1)]))]),
    "streak_3d": (PLAIN, [(f, flat([0, 1, 2])) for f in range(3)]),
    "streak_2d": (dict(PLAIN, two_d=True), [(f, flat([0, 1, 2])) for f in range(3)]),
    "missing_frame": (PLAIN, [(f, flat([0, 1, 2])) for f in (0, 1, 3, 4)]),
    "row_wrap": (dict(PLAIN, min_spot_size=1), [(0, flat([9, 10]))]),
    "above": (dict(PLAIN, min_spot_size=1), [(0, flat([0, 10]))]),
    "diagonal": (dict(PLAIN, min_spot_size=1), [(0, flat([0, 11]))]),
    "diagonal_z": (dict(PLAIN, min_spot_size=1), [(0, flat([0])), (1, flat([10]))]),
    "no_early_emit": (PLAIN, [(0, flat([0, 1, 2])), (1, flat([40, 41, 42]))]),
    "too_small": (PLAIN, [(0, flat([0, 1])), (1, flat([40, 41, 42]))]),
    "too_large": (dict(PLAIN, max_spot_size=5), [(0, flat([0, 1, 2, 3, 4, 5]))]),
    "head_and_tail": (dict(max_separation=2.0),
                      [(0, pix([(0, 100), (1, 5), (2, 4), (3, 3)]))]),
    "far_peak": (dict(max_separation=2.0),
                 [(0, pix([(0, 10), (1, 10), (2, 10), (3, 10), (4, 10), (5, 10), (6, 10),
                           (7, 11)]))]),
    "single_pixel": (dict(PLAIN, min_spot_size=1), [(0, pix([(33, 7)]))]),
    "long_streak": (PLAIN, [(f, flat([5, 6, 7])) for f in range(40)]),
    "merge_through_frame": (PLAIN, [(0, flat([0, 1, 3, 4])), (1, flat([1, 2, 3])),
                                    (2, flat([70, 71, 72]))]),
    "gap_and_two_d": (dict(PLAIN, two_d=True), [(0, flat([0, 1, 2])), (5, flat([0, 1, 2]))]),
}


def run_oracle(opts, frames):
    lab = O.Labeller(H, W, **opts)
    for f, s in frames:
        lab.add(f, s)
    return lab.finish()


def test_known_answers_oracle():
    # Hand-derived values from tests/spots/test_dials_spots.cc.
    r = run_oracle(*CASES["one_two_one"])
    (s,) = r.spots
    assert s["n_signal"] == 3 and s["intensity"] == 4.0
    assert tuple(s["position"]) == (1.5, 0.5, 0.5)
    assert abs(s["variance"][0] - (0.8 / 4.0 + 1.0 / 12.0)) < 1e-12
    assert tuple(s["bbox"]) == (0, 3, 0, 1, 0, 1)
    r = run_oracle(*CASES["streak_3d"])
    assert len(r.spots) == 1 and r.spots[0]["n_signal"] == 9
    assert abs(r.spots[0]["variance"][2] - (0.75 / 9.0 + 1.0 / 12.0)) < 1e-12
    assert len(run_oracle(*CASES["streak_2d"]).spots) == 3
    r = run_oracle(*CASES["missing_frame"])
    assert [s["n_signal"] for s in r.spots] == [6, 6]
    assert len(run_oracle(*CASES["row_wrap"]).spots) == 2
    assert len(run_oracle(*CASES["above"]).spots) == 1
    assert len(run_oracle(*CASES["diagonal"]).spots) == 2
    assert len(run_oracle(*CASES["diagonal_z"]).spots) == 2
    r = run_oracle(*CASES["too_small"])
    assert len(r.spots) == 1 and r.counts["too_small"] == 1 and r.counts["groups"] == 2
    assert r.counts["signal_pixels"] == 5
    assert run_oracle(*CASES["too_large"]).counts["too_large"] == 1
    assert run_oracle(*CASES["head_and_tail"]).counts["separated"] == 0
    assert run_oracle(*CASES["far_peak"]).counts["separated"] == 1


def test_label_options_refused_without_a_device():
    # dials_spots.cc:21-30: refused before any device memory is touched.
    from sfgb import api, labeller
    for kw in (dict(min_spot_size=0), dict(min_spot_size=5, max_spot_size=4)):
        with pytest.raises(ValueError):
            labeller.DeviceLabeller(H, W, **kw)
    with pytest.raises(ValueError):
        labeller.DeviceLabeller(0, W)
    assert api.last_error()


def _same(a, b, what):
    assert O.spot_fields_equal(a.spots, b.spots), f"{what}: spots differ ({len(a.spots)} vs {len(b.spots)})"
    assert a.pixels.tobytes() == b.pixels.tobytes(), f"{what}: kept pixels differ"
    assert a.counts == b.counts, f"{what}: {a.counts} vs {b.counts}"


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_known_answers_device(name):
    from sfgb import labeller
    opts, frames = CASES[name]
    d = labeller.DeviceLabeller(H, W, **opts)
    for f, s in frames:
        d.add(f, s)
    _same(d.finish(), run_oracle(opts, frames), name)


@pytest.mark.gpu
def test_no_early_emission_and_live_count():
    from sfgb import labeller
    d = labeller.DeviceLabeller(H, W, max_separation=0.0)
    d.add(0, flat([0, 1, 2]))
    assert len(d.result().spots) == 0 and d.live == 3
    d.add(1, flat([40, 41, 42]))
    assert len(d.result().spots) == 1 and d.live == 3
    assert len(d.finish().spots) == 2 and d.live == 0


@pytest.mark.gpu
def test_out_of_order_refused():
    from sfgb import labeller
    d = labeller.DeviceLabeller(H, W)
    d.add(3, flat([0, 1, 2]))
    with pytest.raises(RuntimeError):
        d.add(3, flat([0]))
    with pytest.raises(RuntimeError):
        d.add(2, flat([0]))
    with pytest.raises(RuntimeError):
        d.add(4, flat([5, 4]))  # not ascending
    with pytest.raises(RuntimeError):
        d.add(4, flat([H * W]))  # off the frame


@pytest.mark.gpu
@pytest.mark.parametrize("tag,two_d,skip", [("3d", False, None), ("2d", True, None),
                                             ("gap", False, 7)])
def test_golden_sweep_host_lists(tag, two_d, skip):
    from sfgb import labeller
    g = np.load(os.path.join(GOLDEN, "sweep_small.npz"))
    frames = g["frames"]
    d = labeller.DeviceLabeller(frames.shape[1], frames.shape[2], two_d=two_d)
    for i in range(len(frames)):
        if i != skip:
            d.add(i, g[f"signal_{i}"])
    r = d.finish()
    assert O.spot_fields_equal(r.spots, g[f"spots_{tag}"])
    assert r.pixels.tobytes() == g[f"pixels_{tag}"].tobytes()
    assert [r.counts[k] for k in O.COUNT_NAMES] == list(map(int, g[f"counts_{tag}"]))


def _device_sweep(frames, frame_numbers, batch, two_d=False, **opts):
    """Threshold every frame on the device and label the lists in batches,
    never copying a list to the host."""
    import torch
    from sfgb import api, labeller
    h, w = frames.shape[1:]
    cap = h * w // 4
    lists = torch.empty((batch, cap * 16), dtype=torch.uint8, device="cuda")
    counts = torch.zeros(batch, dtype=torch.int32, device="cuda")
    dt = api.DeviceThreshold(h, w, capacity=cap)
    lab = labeller.DeviceLabeller(h, w, two_d=two_d, **opts)
    stream = torch.cuda.current_stream()
    pending = []
    for f, num in zip(frames, frame_numbers):
        j = len(pending)
        dt(torch.from_numpy(f.view(np.int32)).cuda())
        lists[j].copy_(dt.out)
        counts[j : j + 1].copy_(dt.count)
        pending.append(num)
        if len(pending) == batch:
            lab.add_device(pending, lists.data_ptr(), cap, counts.data_ptr(), stream.cuda_stream)
            pending = []
    if pending:
        lab.add_device(pending, lists.data_ptr(), cap, counts.data_ptr(), stream.cuda_stream)
    return lab.finish()


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [1, 4, 5, 12])
def test_golden_sweep_device_lists(batch):
    g = np.load(os.path.join(GOLDEN, "sweep_small.npz"))
    r = _device_sweep(g["frames"], list(range(len(g["frames"]))), batch)
    assert O.spot_fields_equal(r.spots, g["spots_3d"])
    assert r.pixels.tobytes() == g["pixels_3d"].tobytes()
    assert [r.counts[k] for k in O.COUNT_NAMES] == list(map(int, g["counts_3d"]))


@pytest.mark.gpu
@pytest.mark.parametrize("two_d,batch,gaps", [(False, 8, False), (False, 3, True),
                                              (True, 8, False), (False, 16, True)])
def test_random_sweeps_against_oracle(two_d, batch, gaps):
    from sfgb import synth
    p = synth.preset("plain_1m", height=300, width=350, n_frames=24, spots_per_frame=60.0,
                     seed=900 + batch + 10 * gaps + 100 * two_d, row_band_start=120,
                     row_band_len=3, col_band_start=50, col_band_len=2, n_hot=9)
    sw = synth.Sweep(p)
    frames = np.stack([sw.frame(i) for i in range(p.n_frames)])
    numbers = [i + (5 if gaps and i >= 10 else 0) + (2 if gaps and i >= 17 else 0)
               for i in range(p.n_frames)]
    got = _device_sweep(frames, numbers, batch, two_d=two_d)
    lab = O.Labeller(p.height, p.width, two_d=two_d)
    for f, n in zip(frames, numbers):
        lab.add(n, O.dext(f))
    _same(got, lab.finish(), f"two_d={two_d} batch={batch} gaps={gaps}")


@pytest.mark.gpu
def test_plain_1m_sweep_against_oracle():
    # The plain CPU reference workload's shape: 1024 x 1024, 200 spots/frame,
    # masked bands and hot pixels; 20 frames in batches of 16.
    from sfgb import synth
    p = synth.preset("plain_1m", n_frames=20)
    sw = synth.Sweep(p)
    frames = np.stack([sw.frame(i) for i in range(p.n_frames)])
    got = _device_sweep(frames, list(range(p.n_frames)), 16)
    lab = O.Labeller(p.height, p.width)
    for i, f in enumerate(frames):
        lab.add(i, O.dext(f))
    want = lab.finish()
    assert len(want.spots) > 100
    _same(got, want, "plain_1m")


@pytest.mark.gpu
def test_live_capacity_overflow_is_reported():
    from sfgb import labeller
    d = labeller.DeviceLabeller(100, 100, live_capacity=16)
    with pytest.raises(RuntimeError):
        d.add(0, flat(list(range(0, 40, 2))))


def _disc_sweep(h, w, seed):
    """Four frames of host lists: a disc of radius 45 on frames 0-2 (a 3-D
    spot of about 19,000 pixels, beyond a block's shared-memory sort), a disc
    of radius 22 on every frame (about 6,000, sorted by one block), and
    scattered pixels (small spots and singles)."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    lists = []
    for f in range(4):
        m = (yy - 100) ** 2 + (xx - 560) ** 2 < 22 ** 2
        if f < 3:
            m |= (yy - 300) ** 2 + (xx - 200) ** 2 < 45 ** 2
        m |= rng.random((h, w)) < 0.04
        # Peaked at each disc's centre (so the peak-separation filter keeps
        # the discs), with noise.
        prof = (4000 * np.exp(-((yy - 300) ** 2 + (xx - 200) ** 2) / 800.0) +
                2000 * np.exp(-((yy - 100) ** 2 + (xx - 560) ** 2) / 200.0))
        idx = np.flatnonzero(m)
        s = np.zeros(len(idx), O.SIGNAL_DTYPE)
        s["index"] = idx
        s["value"] = prof.ravel()[idx].astype(np.uint32) + rng.integers(1, 20, len(idx))
        lists.append(s)
    return lists


@pytest.mark.gpu
@pytest.mark.parametrize("max_spot_size", [20000, 1000])
def test_spots_beyond_shared_memory_sorts_against_oracle(max_spot_size):
    import torch
    from sfgb import labeller
    h, w = 600, 700
    lists = _disc_sweep(h, w, 77)
    opts = dict(max_spot_size=max_spot_size, max_separation=2.0)
    lab = O.Labeller(h, w, **opts)
    for f, s in enumerate(lists):
        lab.add(f, s)
    want = lab.finish()
    if max_spot_size == 20000:
        assert want.spots["n_signal"].max() > 16000  # the big disc is accepted
    else:
        assert want.counts["too_large"] >= 2
    # One frame a call from host lists.
    d = labeller.DeviceLabeller(h, w, **opts)
    for f, s in enumerate(lists):
        d.add(f, s)
    _same(d.finish(), want, f"host lists, max_spot_size {max_spot_size}")
    # All four frames in one call from device lists.
    cap = max(len(s) for s in lists)
    dev = torch.zeros((4, cap * 16), dtype=torch.uint8, device="cuda")
    for j, s in enumerate(lists):
        dev[j, : len(s) * 16] = torch.from_numpy(s.view(np.uint8).copy()).cuda()
    counts = torch.tensor([len(s) for s in lists], dtype=torch.int32, device="cuda")
    d = labeller.DeviceLabeller(h, w, **opts)
    d.add_device([0, 1, 2, 3], dev.data_ptr(), cap, counts.data_ptr(),
                 torch.cuda.current_stream().cuda_stream)
    _same(d.finish(), want, f"one call, max_spot_size {max_spot_size}")


@pytest.mark.gpu
@pytest.mark.parametrize("bad", [0, 33, 63])
def test_device_list_beyond_its_stride_is_refused(bad):
    """A count above the lists' stride (a threshold that overflowed) fails the
    whole call, wherever the frame sits in a 64-frame batch; the same batch
    with every count in range labels as the oracle does."""
    import torch
    from sfgb import labeller
    h, w, nb, cap = 20, 30, 64, 40
    rng = np.random.default_rng(5 + bad)
    lists = []
    for f in range(nb):
        idx = np.sort(rng.choice(h * w, size=int(rng.integers(0, cap + 1)), replace=False))
        s = np.zeros(len(idx), O.SIGNAL_DTYPE)
        s["index"] = idx
        s["value"] = rng.integers(1, 100, len(idx))
        lists.append(s)
    dev = torch.zeros((nb, cap * 16), dtype=torch.uint8, device="cuda")
    for j, s in enumerate(lists):
        dev[j, : len(s) * 16] = torch.from_numpy(s.view(np.uint8).copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    counts = [len(s) for s in lists]
    lab = O.Labeller(h, w)
    for f, s in enumerate(lists):
        lab.add(f, s)
    want = lab.finish()
    d = labeller.DeviceLabeller(h, w)
    ok = torch.tensor(counts, dtype=torch.int32, device="cuda")
    d.add_device(list(range(nb)), dev.data_ptr(), cap, ok.data_ptr(), stream)
    _same(d.finish(), want, "64 frames in one call")
    counts[bad] = cap + 1
    over = torch.tensor(counts, dtype=torch.int32, device="cuda")
    d = labeller.DeviceLabeller(h, w)
    with pytest.raises(RuntimeError, match="exceeds its capacity"):
        d.add_device(list(range(nb)), dev.data_ptr(), cap, over.data_ptr(), stream)
