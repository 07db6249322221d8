"""Bit-exact parity at the benchmark workloads' full sizes.

Each test generates a workload's seeded frames at the size the benchmarks
time, thresholds them on the device through the batched form (a plan: one
launch sequence for the batch, replayed as a CUDA graph) and compares with
the oracle: each frame's signal list byte for byte and its strong-pixel mask
bit for bit. Where the workload labels, the device labeller's spot table is
compared field by field and bit for bit, and the kept pixels and the counts
exactly, with the oracle's restatement of dials_spots::Labeller fed the
oracle's lists in frame order -- the acceptance test of the reference
(tests/spots/regression.sh:240-255: the GPU table equals the CPU table byte
for byte) at these sizes.

  eiger_16m   64 consecutive 4362 x 4148 frames (EIGER2 16M gaps, Poisson
              0.3 -> 1.5, 3000 spots a frame spanning 2-5 frames) through
              one 64-frame plan launch, labelled in one call of 64 frames
              and in calls of 7; the .refl with shoeboxes built on the device
              against the same file written from the oracle's table.
  dense_16m   4 consecutive 16M frames of Poisson 20 plus three rings, 20000
              spots, 2% overloads at 10^6 counts, 500 hot pixels, labelled
              (many merges across frames); and the sub-case with the
              overloads at 2^32 - 3, where window sums of squares wrap modulo
              2^64.
  batch_4m / batch_9m  full 2162 x 2068 and 3262 x 3108 batches of 16 frames
              at kernel sizes 2, 3 and 4 and with the plain dispersion
              algorithm (settings the reference hard-wires away: there the
              oracle's generalisation is the specification).
  plain_1m    100 frames of 1024 x 1024 through the plain dispersion
              algorithm and through dispersion_extended, labelled.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _oracle_lists(frames, params=None):
    """The oracle's threshold of every frame, one frame a host thread."""
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        return list(ex.map(lambda f: O.dext(f, params), frames))


def _mask_of(signal, shape):
    m = np.zeros(shape[0] * shape[1], bool)
    m[signal["index"]] = True
    return m.reshape(shape)


def _oracle_label(lists, numbers, shape, **opts):
    lab = O.Labeller(shape[0], shape[1], **opts)
    for n, s in zip(numbers, lists):
        lab.add(n, s)
    return lab.finish()


def _same_table(got, want, what):
    assert O.spot_fields_equal(got.spots, want.spots), \
        f"{what}: spot tables differ ({len(got.spots)} vs {len(want.spots)} spots)"
    assert got.pixels.tobytes() == want.pixels.tobytes(), f"{what}: kept pixels differ"
    assert got.counts == want.counts, f"{what}: {got.counts} vs {want.counts}"


def _plan_threshold(frames, params=None, max_frames=64):
    """The frames through one plan launch (a second, replayed from its CUDA
    graph, must give the same); returns the plan and the device frames."""
    import torch
    from sfgb import api
    h, w = frames[0].shape
    dev = [torch.from_numpy(f.view(np.int32)).cuda() for f in frames]
    plan = api.Plan(h, w, max_frames, params=params)
    stream = torch.cuda.current_stream()
    plan(dev, stream=stream)
    first = [plan.result(j).tobytes() for j in range(len(frames))]
    plan(dev, stream=stream)  # the captured graph's replay
    plan(dev, stream=stream)
    for j in range(len(frames)):
        assert plan.result(j).tobytes() == first[j], f"frame {j}: graph replay differs"
    return plan, dev


def _check_threshold(plan, frames, want, what):
    for j, f in enumerate(frames):
        got = plan.result(j)
        assert got.tobytes() == want[j].tobytes(), \
            f"{what} frame {j}: signal list differs ({len(got)} vs {len(want[j])})"
        assert np.array_equal(plan.mask(j), _mask_of(want[j], f.shape)), \
            f"{what} frame {j}: mask differs"


def _label_from_plan(plan, numbers, batch, shape, live_capacity=0, **opts):
    """The plan's device lists labelled batch frames a call, never copied to
    the host."""
    import torch
    from sfgb import labeller
    lab = labeller.DeviceLabeller(shape[0], shape[1], live_capacity=live_capacity, **opts)
    stream = torch.cuda.current_stream()
    for s in range(0, len(numbers), batch):
        part = numbers[s: s + batch]
        lab.add_device(part, plan.lists_ptr + s * plan.capacity * 16, plan.capacity,
                       plan.counts_ptr + 4 * s, stream.cuda_stream)
    return lab


def test_eiger16m_sweep_thresholded_and_labelled(tmp_path):
    from sfgb import labeller, synth
    n = 64
    sw = synth.Sweep(synth.preset("eiger_16m", n_frames=n))
    frames = [sw.frame(i) for i in range(n)]
    want = _oracle_lists(frames)
    assert min(len(s) for s in want) > 50_000
    plan, _ = _plan_threshold(frames)
    _check_threshold(plan, frames, want, "eiger_16m")
    shape = frames[0].shape
    numbers = list(range(100, 100 + n))
    ref = _oracle_label(want, numbers, shape)
    assert len(ref.spots) > 10_000 and ref.counts["accepted"] == len(ref.spots)
    # Spots spanning 2-5 frames: merges across frames within a call and
    # across calls.
    assert (ref.spots["bbox"][:, 5] - ref.spots["bbox"][:, 4]).max() >= 3
    for batch in (64, 7):
        lab = _label_from_plan(plan, numbers, batch, shape, live_capacity=16 << 20)
        got = lab.finish()
        _same_table(got, ref, f"eiger_16m labelled {batch} frames a call")
        if batch == 7:
            # Shoeboxes built on the device, against the same file written
            # from the oracle's table (sf_refl_write is pinned byte for byte
            # to the reference's refl::write).
            dev_path, host_path = tmp_path / "device.refl", tmp_path / "oracle.refl"
            lab.write_refl(str(dev_path))
            labeller.write_refl(str(host_path), ref.spots, ref.pixels, shape[1])
            assert dev_path.read_bytes() == host_path.read_bytes()


@pytest.mark.parametrize("overload", [1_000_000, 0xFFFFFFFD], ids=["1e6", "2^32-3"])
def test_dense16m_frames_thresholded_and_labelled(overload):
    from sfgb import synth
    n = 4
    sw = synth.Sweep(synth.preset("dense_16m", n_frames=n, saturated_value=overload))
    frames = [sw.frame(i) for i in range(n)]
    want = _oracle_lists(frames)
    assert min(len(s) for s in want) > 300_000
    if overload > 0xFFFF0000:
        # Windows holding several of these pixels wrap their sum of squares.
        assert any((s["value"] == overload).sum() > 1000 for s in want)
    plan, _ = _plan_threshold(frames, max_frames=n)
    _check_threshold(plan, frames, want, f"dense_16m overload {overload}")
    shape = frames[0].shape
    numbers = list(range(n))
    ref = _oracle_label(want, numbers, shape)
    assert len(ref.spots) > 1000
    for batch in (4, 3):
        got = _label_from_plan(plan, numbers, batch, shape, live_capacity=16 << 20).finish()
        _same_table(got, ref, f"dense_16m overload {overload}, {batch} frames a call")


BATCH_PARAMS = {
    "k2": dict(kernel_x=2, kernel_y=2),
    "k3": dict(),
    "k4": dict(kernel_x=4, kernel_y=4),
    "dispersion": dict(algorithm=1),
}


@pytest.mark.parametrize("preset", ["batch_4m", "batch_9m"])
@pytest.mark.parametrize("setting", sorted(BATCH_PARAMS))
def test_batch_4m_9m_full_batches(preset, setting):
    from sfgb import api, synth
    n = 16
    sw = synth.Sweep(synth.preset(preset, n_frames=n))
    frames = [sw.frame(i) for i in range(n)]
    kw = BATCH_PARAMS[setting]
    want = _oracle_lists(frames, O.Params(**kw))
    assert min(len(s) for s in want) > 1000
    plan, dev = _plan_threshold(frames, params=api.Params(**kw), max_frames=n)
    _check_threshold(plan, frames, want, f"{preset} {setting}")
    # The plain per-frame device path gives the batch's results.
    single = api.DeviceThreshold(*frames[0].shape, params=api.Params(**kw))
    for j in (0, n - 1):
        single(dev[j])
        assert single.result().tobytes() == want[j].tobytes()


@pytest.mark.parametrize("algorithm", [1, 0], ids=["dispersion", "dispersion_extended"])
def test_plain_1m_sweep_labelled(algorithm):
    from sfgb import api, synth
    n = 100
    sw = synth.Sweep(synth.preset("plain_1m", n_frames=n))
    frames = [sw.frame(i) for i in range(n)]
    want = _oracle_lists(frames, O.Params(algorithm=algorithm))
    shape = frames[0].shape
    ref = _oracle_label(want, list(range(n)), shape, min_spot_size=3)
    assert len(ref.spots) > 1000
    # Thresholded 64 frames a plan launch and labelled 64 frames a call (the
    # plan's batch), then the remaining 36.
    import torch
    from sfgb import labeller
    lab = labeller.DeviceLabeller(*shape, min_spot_size=3)
    stream = torch.cuda.current_stream()
    for start in (0, 64):
        part = frames[start: start + 64]
        plan, _ = _plan_threshold(part, params=api.Params(algorithm=algorithm))
        _check_threshold(plan, part, want[start: start + 64], f"plain_1m {algorithm}")
        lab.add_device(list(range(start, start + len(part))), plan.lists_ptr, plan.capacity,
                       plan.counts_ptr, stream.cuda_stream)
        del plan
    _same_table(lab.finish(), ref, f"plain_1m algorithm {algorithm}")
