"""The served form (sf_server_*): sweeps submitted frame by frame from several
streams at once give, sweep for sweep, the spots the reference's labeller
gives for that sweep alone (golden fixture and oracle), whatever they are
mixed with; admission is by the device-memory budget."""
import os
import threading

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve():
    from sfgb import api, serve as s
    if not api.available():
        pytest.fail("no usable GB300: " + api.unavailable_reason())
    return s


def _oracle_sweep(frames, numbers):
    lab = O.Labeller(frames[0].shape[0], frames[0].shape[1])
    for f, n in zip(frames, numbers):
        lab.add(n, O.dext(f))
    return lab.finish()


def _synth(h, w, n, seed):
    from sfgb import synth
    sw = synth.Sweep(synth.preset("plain_1m", height=h, width=w, n_frames=n,
                                  spots_per_frame=h * w / 1500.0, seed=seed,
                                  row_band_start=h // 3, row_band_len=3,
                                  col_band_start=w // 4, col_band_len=2, n_hot=5))
    return [sw.frame(i) for i in range(n)]


def test_one_sweep_matches_golden(serve):
    g = np.load(os.path.join(GOLDEN, "sweep_small.npz"))
    frames = [np.ascontiguousarray(f) for f in g["frames"]]
    srv = serve.Server(max_batch=4, ring=8)
    sid = srv.open_sweep(*frames[0].shape)
    for i, f in enumerate(frames):
        srv.submit(sid, i, f)
    res = srv.finish_sweep(sid)
    done = []
    while len(done) < len(frames):
        done += srv.poll(wait_ms=100)
    assert O.spot_fields_equal(res.spots, g["spots_3d"])
    assert res.pixels.tobytes() == g["pixels_3d"].tobytes()
    by_frame = {d["frame"]: d for d in done}
    for i in range(len(frames)):
        assert by_frame[i]["status"] == 0
        assert by_frame[i]["n_signal"] == len(g[f"signal_{i}"])
        assert by_frame[i]["latency_ms"] > 0
    srv.close_sweep(sid)
    srv.close()


def test_same_alone_and_in_the_mix(serve):
    sweeps = {
        "a": (_synth(300, 350, 14, 1), list(range(14))),
        "b": (_synth(300, 350, 11, 2), [3 + i + (4 if i > 5 else 0) for i in range(11)]),
        "c": (_synth(200, 260, 17, 3), list(range(17))),
    }
    want = {k: _oracle_sweep(*v) for k, v in sweeps.items()}
    srv = serve.Server(max_batch=5, ring=6)
    ids = {k: srv.open_sweep(*v[0][0].shape) for k, v in sweeps.items()}

    def feed(k):
        frames, numbers = sweeps[k]
        for f, n in zip(frames, numbers):
            srv.submit(ids[k], n, f)

    threads = [threading.Thread(target=feed, args=(k,)) for k in sweeps]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    got = {k: srv.finish_sweep(ids[k]) for k in sweeps}
    for k in sweeps:
        assert O.spot_fields_equal(got[k].spots, want[k].spots), k
        assert got[k].pixels.tobytes() == want[k].pixels.tobytes(), k
        assert got[k].counts == want[k].counts, k
        srv.close_sweep(ids[k])
    srv.close()


def test_admission_by_budget(serve):
    probe = serve.Server(hbm_budget=1 << 40, max_batch=4, ring=8)
    probe.close_sweep(probe.open_sweep(256, 320))
    probe_sweep = probe.open_sweep(256, 320)
    one = probe.used_bytes  # a sweep and its shape group
    probe.close_sweep(probe_sweep)
    probe.close()
    srv = serve.Server(hbm_budget=int(one * 1.3), max_batch=4, ring=8)
    a = srv.open_sweep(256, 320)
    with pytest.raises(serve.Busy):
        srv.open_sweep(256, 320)
    srv.close_sweep(a)
    b = srv.open_sweep(256, 320)
    assert srv.used_bytes > 0
    srv.close_sweep(b)
    srv.close()


def test_results_count_against_the_budget(serve):
    """A sweep's spots and pixels held on the device count against the
    budget: with room for one sweep and about 3 MiB of results, a long dense
    sweep fails with SF_EBUSY once its stores would grow past the budget,
    instead of growing; the server never holds more than its budget."""
    from sfgb import api
    h, w, n = 512, 640, 80
    frames = _synth(h, w, n, seed=91)
    probe = serve.Server(hbm_budget=1 << 40, max_batch=4, ring=8)
    sid = probe.open_sweep(h, w)
    one = probe.used_bytes  # the sweep and its shape group, no results yet
    for i in range(n):
        probe.submit(sid, i, frames[i])
    probe.finish_sweep(sid, read=False)
    # The results are counted, and they outgrow the budget below.
    assert probe.used_bytes - one > (3 << 20)
    probe.close_sweep(sid)
    assert probe.used_bytes == 0
    probe.close()

    budget = one + (3 << 20)
    srv = serve.Server(hbm_budget=budget, max_batch=4, ring=8)
    sid = srv.open_sweep(h, w)
    done = []
    for i in range(n):
        try:
            srv.submit(sid, i, frames[i])
        except api.SpotFinderError:
            break  # the sweep has already failed
        assert srv.used_bytes <= budget
    with pytest.raises(api.SpotFinderError):
        srv.finish_sweep(sid)
    assert "budget" in srv.sweep_error(sid)
    done += srv.poll(4096, 100)
    assert any(d["status"] == serve.SF_EBUSY for d in done)
    assert srv.used_bytes <= budget
    srv.close_sweep(sid)
    assert srv.used_bytes == 0
    srv.close()


def test_out_of_order_refused(serve):
    srv = serve.Server(max_batch=2, ring=2)
    sid = srv.open_sweep(64, 64)
    f = np.zeros((64, 64), np.uint32)
    srv.submit(sid, 5, f)
    with pytest.raises(ValueError):
        srv.submit(sid, 5, f)
    with pytest.raises(ValueError):
        srv.submit(sid, 4, f)
    srv.finish_sweep(sid)
    srv.close()


def test_compressed_chunks_served(serve):
    # The same sweeps submitted as bitshuffle+LZ4 and LZ4 chunks (mixed with a
    # sweep of raw frames) give the spots of the raw frames; a chunk with a
    # bad header is refused at submit and the frame is not taken.
    from sfgb import api, synth
    a = (_synth(300, 350, 9, 7), list(range(9)))
    b = (_synth(200, 260, 8, 8), list(range(8)))
    want_a, want_b = _oracle_sweep(*a), _oracle_sweep(*b)
    chunks_a = [synth.chunk(f, "bslz4") for f in a[0]]
    chunks_b = [synth.chunk(f, "lz4", 4096) for f in b[0]]
    srv = serve.Server(max_batch=4, ring=6)
    ia, ib, ic = srv.open_sweep(300, 350), srv.open_sweep(200, 260), srv.open_sweep(300, 350)
    bad = chunks_a[0].copy()
    bad[7] ^= 1  # the header's frame size
    with pytest.raises(api.DataError):
        srv.submit_chunk(ia, 0, bad)
    for i in range(9):
        srv.submit_chunk(ia, a[1][i], chunks_a[i])
        srv.submit(ic, a[1][i], a[0][i])
        if i < 8:
            srv.submit_chunk(ib, b[1][i], chunks_b[i], "lz4")
    got_a, got_b, got_c = srv.finish_sweep(ia), srv.finish_sweep(ib), srv.finish_sweep(ic)
    for got, want in ((got_a, want_a), (got_b, want_b), (got_c, want_a)):
        assert O.spot_fields_equal(got.spots, want.spots)
        assert got.pixels.tobytes() == want.pixels.tobytes()
    for sid in (ia, ib, ic):
        srv.close_sweep(sid)
    srv.close()


def test_undecodable_chunk_fails_its_sweep(serve):
    # A chunk whose framing is sound but whose first block is not LZ4: the
    # frame and its sweep fail with the decoder's text; other sweeps go on.
    from sfgb import api, synth
    frames = _synth(120, 160, 3, 9)
    good = [synth.chunk(f) for f in frames]
    broken = good[1].copy()
    broken[16:20] = [0xF0, 0xFF, 0xFF, 0xFF]
    srv = serve.Server(max_batch=4, ring=6)
    s1, s2 = srv.open_sweep(120, 160), srv.open_sweep(120, 160)
    srv.submit_chunk(s1, 0, good[0])
    srv.submit_chunk(s1, 1, broken)
    for i in range(3):
        srv.submit_chunk(s2, i, good[i])
    done = []
    while len(done) < 5:
        done += srv.poll(wait_ms=100)
    status = {(d["sweep"], d["frame"]): d["status"] for d in done}
    assert status[(s1, 1)] == api.SF_EDATA
    assert "bitshuffle decompression failed" in srv.sweep_error(s1)
    assert all(status[(s2, i)] == 0 for i in range(3))
    want = _oracle_sweep(frames, [0, 1, 2])
    got = srv.finish_sweep(s2)
    assert O.spot_fields_equal(got.spots, want.spots)
    srv.close_sweep(s1)
    srv.close_sweep(s2)
    srv.close()
