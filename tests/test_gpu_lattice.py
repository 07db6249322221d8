"""Edge cases of the kernel-3,3 threshold path: stage 0 decided on a lattice
of every third row and column, the erosion bound that follows, the exact check
on listed 8 x 28 tiles and stage 2 on the same tiles. Each frame is built to
stress one part (masked pixels on lattice points, bands at every phase, strip
and tile boundaries, spots in a tile's last columns, saturated and 64-bit
pixels) and must give the oracle's list and mask bit for bit. Frames whose
width is a multiple of 8 also run as 16-bit frames, whose tests are the
reference's float ones (src/spots/dext.hh:31-33)."""
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


def _spots(h, w, n, seed, peak=(50.0, 2000.0)):
    from sfgb import synth
    p = synth.preset("eiger_16m", height=h, width=w, n_frames=1, spots_per_frame=float(n),
                     seed=seed)
    p.eiger_gaps = 0
    return synth.Sweep(p).frame(0)


def _blob(f, y, x, peak, sigma=1.2):
    h, w = f.shape
    ys, xs = np.mgrid[max(0, y - 6):min(h, y + 7), max(0, x - 6):min(w, x + 7)]
    g = peak * np.exp(-((ys - y) ** 2 + (xs - x) ** 2) / (2 * sigma * sigma))
    sub = f[ys, xs].astype(np.float64) + np.floor(g)
    f[ys, xs] = np.minimum(sub, 0xFFFFFFFD).astype(np.uint32)


def _as_u16(f):
    """The frame as 16-bit pixels: valid values clamped below the masked
    sentinels, the sentinels kept."""
    g = np.minimum(f, 0xFFFD).astype(np.uint16)
    g[f == 0xFFFFFFFE] = 0xFFFE
    g[f == 0xFFFFFFFF] = 0xFFFF
    return g


def _check_batch(api, frames, what, params=None, also16=True):
    import torch
    h, w = frames[0].shape
    sets = [("u32", frames)]
    if also16 and w % 8 == 0:
        sets.append(("u16", [_as_u16(f) for f in frames]))
    for kind, fs in sets:
        b = api.DeviceBatch(h, w, len(fs), capacity=h * w, word_prefix=True,
                            params=api.Params(**params) if params else None)
        view = np.int32 if fs[0].dtype == np.uint32 else np.int16
        b([torch.from_numpy(f.view(view)).cuda() for f in fs])
        torch.cuda.synchronize()
        for j, f in enumerate(fs):
            want, mask = O.dext(f, O.Params(**params) if params else None, with_mask=True)
            _same(b.result(j), want, f"{what} {kind} frame {j}")
            assert np.array_equal(b.mask(j), mask.astype(bool)), f"{what} {kind} frame {j} mask"


@pytest.mark.parametrize("phase", [(0, 0), (2, 2), (1, 2), (2, 0)])
def test_masked_pixels_on_lattice_points(api, phase):
    # Masked and hot pixels on every lattice point of one phase over half the
    # frame: the bound must treat a masked centre as set, and the pixels whose
    # only lattice neighbours are masked must still be checked exactly.
    py, px = phase
    f = _spots(260, 400, 120, seed=11 + 3 * py + px)
    g = f.copy()
    g[py::3, px:200:3] = 0xFFFFFFFE
    g[py + 60::6, 200 + px::6] = 0xFFFFFFFF
    _check_batch(api, [f, g], f"lattice phase {phase}")


def test_masked_bands_at_every_phase(api):
    # Row and column bands of widths 1-4 starting at every residue mod 3,
    # across spots: valid pixels beside a band see few lattice pixels.
    frames = []
    for k, width in enumerate((1, 2, 3, 4)):
        f = _spots(240, 424, 150, seed=30 + k)
        for r in range(3):
            y0, x0 = 20 + 70 * r + k, 30 + 130 * r + k
            f[y0:y0 + width, :] = 0xFFFFFFFE
            f[:, x0:x0 + width] = 0xFFFFFFFF
        frames.append(f)
    _check_batch(api, frames, "bands")


@pytest.mark.parametrize("h,w", [(1, 3), (2, 29), (7, 28), (8, 31), (9, 33), (17, 356),
                                 (31, 359), (33, 360), (40, 361), (23, 364), (12, 719),
                                 (25, 720), (19, 721), (16, 724)])
def test_strip_and_tile_boundaries(api, h, w):
    # Widths around the lattice pass's 360-column strips and the exact check's
    # 28-column tiles, heights around its 8-row tiles and 3-row triples;
    # widths not a multiple of 4 take the direct-load variant.
    rng = np.random.default_rng(h * 1000 + w)
    f = rng.poisson(1.0, size=(h, w)).astype(np.uint32)
    for _ in range(max(1, h * w // 300)):
        _blob(f, int(rng.integers(0, h)), int(rng.integers(0, w)), float(rng.uniform(40, 900)))
    f[rng.random(f.shape) < 0.01] = 0xFFFFFFFF
    _same(api.find(f, capacity=h * w), O.dext(f), f"{h}x{w}")


def test_spots_on_tile_corners_and_last_columns(api):
    # Bright spots centred on and beside the corners of the 8 x 28 tiles and in
    # a tile's last six columns (whose windows need the second column pass).
    f = np.random.default_rng(5).poisson(0.8, size=(200, 616)).astype(np.uint32)
    for j, y in enumerate(range(8, 192, 24)):
        for k, x in enumerate(range(28, 600, 56)):
            dy, dx = (j + k) % 3 - 1, (0, 1, -1, 22, 25, 27)[(j * 7 + k) % 6]
            _blob(f, y + dy, x + dx if dx in (0, 1, -1) else x - 28 + dx,
                  300.0 + 40.0 * ((j + k) % 7))
    _check_batch(api, [f], "tile corners")


def test_saturated_and_wide_pixels_near_spots(api):
    # Values around the lattice pass's saturation (2^15 - 1), the 32-bit
    # sums' bound (narrow_max, 9363), the 32-bit stage-2 sums' bound (2^24)
    # and far above, next to spots; the other frames of the batch stay narrow,
    # so the 64-bit stage 2 is taken per frame.
    base = _spots(220, 330, 100, seed=77)
    frames = [base.copy()]
    for k, vals in enumerate(((32766, 32767, 32768, 40000),
                              (9362, 9363, 9364, 20000),
                              ((1 << 24) - 1, 1 << 24, (1 << 24) + 1, 1_000_000),
                              (0xFFFFFFFD, 0xFFFFFFFC, 3_000_000_000, 70_000))):
        f = base.copy()
        rng = np.random.default_rng(100 + k)
        for i, v in enumerate(vals):
            for _ in range(6):
                y, x = int(rng.integers(5, 215)), int(rng.integers(5, 325))
                _blob(f, y, x, 500.0)
                f[y + (i % 3) - 1, x + (i // 3)] = v
        frames.append(f)
    frames.append(base.copy())
    _check_batch(api, frames, "saturated")


def test_frame_of_signal_everywhere(api):
    # High-variance texture: nearly every window is stage-0 signal, so the
    # bound passes most of the frame and nearly every tile is listed.
    rng = np.random.default_rng(9)
    f = (rng.integers(0, 2, size=(150, 296)) * rng.integers(50, 400, size=(150, 296)))
    f = f.astype(np.uint32)
    f[::37, :] = 0xFFFFFFFE
    _check_batch(api, [f, np.ascontiguousarray(f[:, ::-1])], "signal everywhere")


@pytest.mark.parametrize("h,w", [(1, 8), (7, 16), (9, 24), (17, 360), (31, 368), (33, 720),
                                 (40, 728), (12, 1000), (25, 1024)])
def test_strip_and_tile_boundaries_16bit(api, h, w):
    # 16-bit frames with widths that are multiples of 8 take the lattice path.
    rng = np.random.default_rng(h * 977 + w)
    f = rng.poisson(1.0, size=(h, w)).astype(np.uint32)
    for _ in range(max(1, h * w // 300)):
        _blob(f, int(rng.integers(0, h)), int(rng.integers(0, w)), float(rng.uniform(40, 900)))
    f[rng.random(f.shape) < 0.01] = 0xFFFFFFFF
    g = _as_u16(f)
    _same(api.find(g, capacity=h * w), O.dext(g), f"{h}x{w} u16")


@pytest.mark.parametrize("params", [
    dict(), dict(gain=1.5), dict(gain=0.8, sigma_b=4.5, sigma_s=2.5), dict(min_local=5),
    dict(min_local=0), dict(global_threshold=3.0), dict(global_threshold=40.5),
    dict(sigma_b=3.0, sigma_s=2.0)])
def test_16bit_parameters(api, params):
    # The 16-bit lattice path takes any gain and sigmas (its tests are float).
    frames = [_spots(230, 400, 120, seed=60 + k) for k in range(2)]
    frames[1][::41, :] = 0xFFFFFFFE
    g = [_as_u16(f) for f in frames]
    _check_batch(api, g, f"u16 {params}", params=params, also16=False)


def test_16bit_bright_values(api):
    # Values up to the largest valid 16-bit pixel: sums of squares wrap
    # modulo 2^32 in the reference's 32-bit accumulators, as here.
    rng = np.random.default_rng(12)
    f = rng.integers(0, 50, size=(200, 320)).astype(np.uint32)
    big = rng.random(f.shape) < 0.05
    f[big] = rng.integers(30000, 0xFFFD, size=int(big.sum()))
    for y, x in ((40, 40), (100, 200), (150, 300)):
        _blob(f, y, x, 60000.0)
    _check_batch(api, [_as_u16(f)], "u16 bright", also16=False)
