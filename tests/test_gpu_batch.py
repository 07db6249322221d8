"""The batched device threshold (sf_threshold_*_batch_device): every frame of
a batch must give the list, mask and count the oracle gives for it alone,
bit for bit, whatever else shares the launch (frames handed to the 64-bit
path, dense frames, frames that overflow their capacity)."""
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


def _same(got, want, what=""):
    if got.tobytes() == want.tobytes():
        return
    gi, wi = set(got["index"].tolist()), set(want["index"].tolist())
    raise AssertionError(f"{what}: {len(got)} vs {len(want)} signal pixels; only GPU "
                         f"{sorted(gi - wi)[:5]}, only CPU {sorted(wi - gi)[:5]}")


def _mixed_frames(h, w, n, seed):
    """Spot frames with EIGER-style gaps, plus one with values near 2^32
    (the 64-bit path) and one dense Poisson-20 frame when n allows."""
    from sfgb import synth
    sw = synth.Sweep(synth.preset("eiger_16m", height=h, width=w, n_frames=n,
                                  spots_per_frame=h * w / 3000.0, seed=seed))
    frames = [sw.frame(i) for i in range(n)]
    rng = np.random.default_rng(seed)
    if n >= 3:
        f = frames[1].copy()
        big = rng.random(f.shape) < 0.002
        f[big] = rng.integers(0xFFFF0000, 0xFFFFFFFD, size=int(big.sum()), dtype=np.uint64)
        frames[1] = f
    if n >= 4:
        d = synth.preset("dense_16m", height=h, width=w, n_frames=1,
                         spots_per_frame=h * w / 1000.0, seed=seed + 1)
        frames[2] = synth.Sweep(d).frame(0)
    return frames


def _run(api, frames, params=None, capacity=None, offset=0):
    import torch
    h, w = frames[0].shape
    cap = capacity if capacity is not None else h * w
    b = api.DeviceBatch(h, w, len(frames), capacity=cap, params=params, word_prefix=True)
    if offset:
        # Frames 4 bytes off the 16-byte grid: the kernels take scalar loads.
        store = torch.empty((len(frames), h * w + 4), dtype=torch.int32, device="cuda")
        views = []
        for j, f in enumerate(frames):
            v = store[j, 1:1 + h * w].view(h, w)
            v.copy_(torch.from_numpy(f.view(np.int32)))
            views.append(v)
    else:
        views = [torch.from_numpy(f.view(np.int32)).cuda() for f in frames]
    b(views)
    torch.cuda.synchronize()
    return b


@pytest.mark.parametrize("h,w,n", [(300, 480, 1), (257, 700, 5), (300, 701, 4), (40, 300, 64)])
def test_batch_against_oracle(api, h, w, n):
    frames = _mixed_frames(h, w, n, seed=h + w + n)
    b = _run(api, frames)
    for j, f in enumerate(frames):
        want, mask = O.dext(f, with_mask=True)
        _same(b.result(j), want, f"{h}x{w} frame {j} of {n}")
        assert np.array_equal(b.mask(j), mask.astype(bool)), f"mask of frame {j}"
        wp = b.word_prefix[j].cpu().numpy().view(np.uint32)
        words = b.bits[j].cpu().numpy().view(np.uint32)
        counts = np.array([bin(int(x)).count("1") for x in words])
        assert np.array_equal(wp, np.concatenate([[0], np.cumsum(counts)[:-1]]))


@pytest.mark.parametrize("params", [dict(kernel_x=2, kernel_y=2), dict(kernel_x=4, kernel_y=4),
                                    dict(min_local=30), dict(global_threshold=50.0),
                                    dict(sigma_b=3.0, sigma_s=2.0), dict(algorithm=1),
                                    dict(gain=1.5)])
def test_batch_parameters(api, params):
    frames = _mixed_frames(200, 333, 4, seed=11)
    b = _run(api, frames, params=api.Params(**params))
    for j, f in enumerate(frames):
        _same(b.result(j), O.dext(f, O.Params(**params)), f"{params} frame {j}")


@pytest.mark.parametrize("h,w,n", [(300, 480, 3), (257, 700, 5), (120, 722, 4), (40, 364, 64)])
def test_batch_16bit_against_oracle(api, h, w, n):
    # 16-bit frames in one launch (sf_threshold_u16_batch_device): the
    # lattice path where 4 | width, the tile path otherwise; each frame's
    # list and mask as the oracle gives them for it alone.
    import torch
    frames = []
    for f in _mixed_frames(h, w, n, seed=h * 7 + w + n):
        g = np.minimum(f, 0xFFFD).astype(np.uint16)  # valid counts below the markers
        g[f >= 0xFFFFFFFE] = 0xFFFF
        frames.append(g)
    b = api.DeviceBatch(h, w, n, capacity=h * w)
    b([torch.from_numpy(g.view(np.int16)).cuda() for g in frames])
    torch.cuda.synchronize()
    for j, g in enumerate(frames):
        want, mask = O.dext(g, with_mask=True)
        _same(b.result(j), want, f"{h}x{w} u16 frame {j} of {n}")
        assert np.array_equal(b.mask(j), mask.astype(bool)), f"mask of u16 frame {j}"


def test_batch_unaligned_frames(api):
    frames = _mixed_frames(180, 400, 4, seed=3)
    b = _run(api, frames, offset=1)
    for j, f in enumerate(frames):
        _same(b.result(j), O.dext(f), f"unaligned frame {j}")


def test_batch_overflow_is_per_frame(api):
    frames = _mixed_frames(220, 360, 3, seed=21)
    want = [O.dext(f) for f in frames]
    cap = len(want[0]) - 1
    b = _run(api, frames, capacity=cap)
    with pytest.raises(api.OverflowError_):
        b.result(0)
    for j in range(1, len(frames)):
        if len(want[j]) <= cap:
            _same(b.result(j), want[j], f"frame {j} beside an overflow")


def test_batch_16m_frames(api):
    # Four 4362 x 4148 frames with the EIGER2 gaps, as the benchmark batches.
    from sfgb import synth
    sw = synth.Sweep(synth.preset("eiger_16m", n_frames=4))
    frames = [sw.frame(i) for i in range(4)]
    b = _run(api, frames, capacity=frames[0].size // 4)
    for j, f in enumerate(frames):
        _same(b.result(j), O.dext(f), f"16M frame {j}")


@pytest.mark.parametrize("kernel", [2, 3, 4])
def test_batch_near_threshold_windows(api, kernel):
    # Negative-binomial backgrounds whose dispersion index sits at the
    # stage-0 threshold (about 1 + sigma_b sqrt(2 / (n - 1))): many windows
    # fall between the two integer bounds and are decided by the exact pass,
    # which then clears the neighbourhoods of those that are not signal.
    rng = np.random.default_rng(40 + kernel)
    n = (2 * kernel + 1) ** 2
    index = 1.0 + 6.0 * np.sqrt(2.0 / (n - 1))
    frames = []
    for j in range(4):
        mean = 2.0 + j
        p = 1.0 / index
        r = mean * p / (1.0 - p)
        f = rng.negative_binomial(r, p, size=(190, 260)).astype(np.uint32)
        f[rng.random(f.shape) < 0.002] = 0xFFFFFFFF
        frames.append(f)
    params = dict(kernel_x=kernel, kernel_y=kernel)
    b = _run(api, frames, params=api.Params(**params))
    for j, f in enumerate(frames):
        want, mask = O.dext(f, O.Params(**params), with_mask=True)
        _same(b.result(j), want, f"kernel {kernel} frame {j}")
        assert np.array_equal(b.mask(j), mask.astype(bool))


def _run_mixed(api, frames, params=None, capacity=None):
    import torch
    b = api.MixedBatch([f.shape for f in frames], capacity=capacity, params=params,
                       word_prefix=True)
    b([torch.from_numpy(f.view(np.int32)).cuda() for f in frames])
    torch.cuda.synchronize()
    return b


def _check_mixed(b, frames, params=None, what=""):
    for j, f in enumerate(frames):
        want, mask = O.dext(f, O.Params(**params) if params else None, with_mask=True)
        _same(b.result(j), want, f"{what} frame {j} ({f.shape[0]}x{f.shape[1]})")
        assert np.array_equal(b.mask(j), mask.astype(bool)), f"{what} mask of frame {j}"
        wp = b.words(j, b.word_prefix)
        counts = np.array([bin(int(x)).count("1") for x in b.words(j)])
        assert np.array_equal(wp, np.concatenate([[0], np.cumsum(counts)[:-1]])), what


# Frames of several detector shapes in one launch sequence (the lattice path
# for the reference's window), each compared with the oracle alone: the
# largest first, last and in the middle, frames narrower and shorter than the
# envelope, a frame handed to the 64-bit path and a dense one among them.
MIXED_SHAPES_ALIGNED = [(520, 712), (300, 480), (1030, 1064), (64, 96), (257, 700),
                        (40, 300), (300, 1064)]
MIXED_SHAPES_ODD = [(257, 701), (300, 480), (1030, 1065), (31, 33), (520, 700)]


@pytest.mark.parametrize("shapes", [MIXED_SHAPES_ALIGNED, MIXED_SHAPES_ODD],
                         ids=["aligned", "odd_widths"])
def test_mixed_shapes_against_oracle(api, shapes):
    frames = []
    for k, (h, w) in enumerate(shapes):
        frames += _mixed_frames(h, w, 4, seed=7 * k + h)[k % 4:k % 4 + 1]
    b = _run_mixed(api, frames)
    _check_mixed(b, frames, what="mixed")


@pytest.mark.parametrize("params", [dict(kernel_x=2, kernel_y=2), dict(kernel_x=4, kernel_y=4),
                                    dict(algorithm=1), dict(gain=1.5)])
def test_mixed_shapes_other_settings(api, params):
    # Settings off the lattice path: frames of another shape run one launch
    # sequence each, into the same envelope layout.
    frames = [_mixed_frames(h, w, 4, seed=h + w)[0]
              for h, w in [(200, 333), (120, 512), (257, 96)]]
    b = _run_mixed(api, frames, params=api.Params(**params))
    _check_mixed(b, frames, params, what=str(params))


def test_mixed_detector_sizes_full(api):
    # The served workload's detectors in one launch: a 16M frame (EIGER2
    # gaps), a 9M, a 4M and a 1M one, as their sweeps would batch.
    from sfgb import synth
    frames = []
    for name, h, w in [("eiger_16m", 4362, 4148), ("eiger_16m", 3262, 3108),
                       ("eiger_16m", 2162, 2068), ("plain_1m", 1030, 1064)]:
        p = synth.preset(name, height=h, width=w, n_frames=2)
        frames.append(synth.Sweep(p).frame(1))
    b = _run_mixed(api, frames, capacity=frames[0].size // 4)
    _check_mixed(b, frames, what="detectors")
