"""Batch plans (sf_plan_*): the tuned run length and CUDA-graph replays give
the same lists as the oracle, frame for frame, for every pointer set."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    from sfgb import api as a
    if not a.available():
        pytest.fail("no usable GB300: " + a.unavailable_reason())
    return a


def _frames(h, w, n, seed):
    from sfgb import synth
    sw = synth.Sweep(synth.preset("eiger_16m", height=h, width=w, n_frames=n,
                                  spots_per_frame=h * w / 3000.0, seed=seed))
    return [sw.frame(i) for i in range(n)]


def test_plan_graph_replays_and_tuning(api):
    import torch
    h, w = 520, 700
    frames = _frames(h, w, 8, seed=77)
    want = [O.dext(f) for f in frames]
    dev = [torch.from_numpy(f.view(np.int32)).cuda() for f in frames]
    plan = api.Plan(h, w, 4, capacity=h * w)
    sets = [dev[0:4], dev[4:8], dev[2:6]]
    for rep in range(3):
        for k, group in enumerate(sets):
            plan(group)
            base = (0, 4, 2)[k]
            for j in range(4):
                got = plan.result(j)
                assert got.tobytes() == want[base + j].tobytes(), (rep, k, j)
    assert plan.graphs == len(sets)
    rr = plan.tune(dev[0:4])
    assert rr >= 16
    assert plan.graphs == 0
    plan(dev[4:8])
    plan(dev[4:8])
    for j in range(4):
        assert plan.result(j).tobytes() == want[4 + j].tobytes()
    plan(dev[5:7])  # a shorter batch through the same plan
    for j in range(2):
        assert plan.result(j).tobytes() == want[5 + j].tobytes()
    plan.close()


def test_plan_refuses_bad_shapes(api):
    with pytest.raises(api.SpotFinderError):
        api.Plan(0, 10, 4)
    with pytest.raises(api.SpotFinderError):
        api.Plan(10, 10, 65)


@pytest.mark.parametrize("per_launch,run_rows", [(16, 0), (32, 48), (0, 96)])
def test_plan_frames_per_launch(api, per_launch, run_rows):
    # A 48-frame call split into launch sequences of per_launch frames (the
    # tuner's other knob) gives every frame the oracle's list.
    import torch
    h, w = 160, 384
    frames = _frames(h, w, 48, seed=5 + per_launch)
    want = [O.dext(f) for f in frames]
    dev = [torch.from_numpy(f.view(np.int32)).cuda() for f in frames]
    plan = api.Plan(h, w, 48, capacity=h * w // 4)
    plan.configure(run_rows, per_launch)
    for rep in range(2):  # direct, then a captured graph
        plan(dev)
        for j in range(48):
            assert plan.result(j).tobytes() == want[j].tobytes(), (rep, j)
    assert plan.frames_per_launch == per_launch
    plan.tune(dev)
    assert plan.frames_per_launch in (0, 16, 32)
    plan(dev)
    for j in range(0, 48, 7):
        assert plan.result(j).tobytes() == want[j].tobytes()
    plan.close()
