"""Frame decompression: decompress::image (src/spots/decompress.cc:77-134)
for chunks stored bitshuffle+LZ4 ("bslz4"), LZ4 ("lz4") or uncompressed.

The oracle (oracle/sf_oracle_decompress.c) is pinned to the LZ4 library
itself through tests/golden/lz4_blocks.npz (blocks the library wrote, and
damaged blocks with whether the library accepts them); bitshuffle's bit
planes are checked against their definition. The device decoder
(sf_decompress_image, sf_decompress_device, sf_find_compressed) must give
the oracle's frame byte for byte, and refuse what the reference refuses with
the reference's text. Chunks of synthetic frames come from the package's
chunk writer (synth.chunk), whose blocks the LZ4 library must read."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN


def _golden():
    return np.load(os.path.join(GOLDEN, "lz4_blocks.npz"))


def _frame(h, w, dtype, seed, mean=1.0):
    rng = np.random.default_rng(seed)
    f = rng.poisson(mean, (h, w)).astype(dtype)
    top = np.iinfo(dtype).max
    f[rng.random((h, w)) < 0.01] = top
    f[rng.random((h, w)) < 0.002] = rng.integers(1000, top - 2, dtype=dtype)
    return f


CHUNKS = [  # shape, dtype, algorithm, block bytes
    ((1, 1), np.uint32, "bslz4", 0), ((3, 5), np.uint16, "bslz4", 0),
    ((37, 101), np.uint32, "bslz4", 0), ((64, 64), np.uint16, "bslz4", 0),
    ((300, 517), np.uint32, "bslz4", 0), ((300, 517), np.uint16, "bslz4", 0),
    ((257, 300), np.uint32, "bslz4", 4096), ((200, 333), np.uint16, "bslz4", 48),
    ((211, 190), np.uint32, "bslz4", 32768), ((150, 160), np.uint16, "bslz4", 20000),
    ((37, 101), np.uint32, "lz4", 0), ((300, 517), np.uint32, "lz4", 8192),
    ((120, 77), np.uint16, "lz4", 1000), ((5, 5), np.uint32, "", 0),
]


# Sequences of every shape the device's windowed parse treats differently:
# literal runs of 0-14 bytes (taken a 32-byte window at a time) and of 15 or
# more (the byte-by-byte parse), match lengths with no extra byte, one extra
# byte up to 254 and a 255 (a second extra byte), offsets 1 (a run), 2-31
# (patterns copied in doubling passes), and longer (whole copies, words for
# long ones, every source alignment), and sequences that start anywhere in a
# window, so that some straddle its end.
_LITS = [0, 0, 0, 0, 1, 1, 2, 3, 4, 5, 7, 11, 13, 14, 15, 16, 17, 33, 270, 300]
_MLS = [4, 4, 5, 6, 7, 9, 12, 16, 18, 19, 20, 31, 32, 33, 47, 63, 64, 65, 100, 128, 129,
        200, 272, 273, 274, 300, 512, 513, 600, 1000]
_OFFS = [1, 2, 3, 4, 5, 6, 7, 8, 9, 13, 16, 17, 31, 32, 33, 63, 100, 126, 127, 128, 129,
         130, 255, 256, 257, 300, 1000, 4095]


def _lz4_length(blk, v):
    while v >= 255:
        blk.append(255)
        v -= 255
    blk.append(v)


def _lz4_random_block(rng, total):
    """One LZ4 block of random sequences that decodes to `total` bytes (at
    least 13), keeping LZ4's end-of-block rules (a final literal run of 12
    bytes or more); returns (block, decoded bytes)."""
    out, blk = bytearray(), bytearray()
    while True:
        left = total - len(out)
        nl = int(rng.choice(_LITS))
        ml = int(rng.choice(_MLS))
        if len(out) + nl == 0:
            nl = 1
        if nl + ml + 12 > left:
            break
        lits = rng.integers(0, 3 if rng.random() < 0.7 else 256, nl, dtype=np.uint8)
        off = min(int(rng.choice(_OFFS)), len(out) + nl)
        blk.append(min(nl, 15) << 4 | min(ml - 4, 15))
        if nl >= 15:
            _lz4_length(blk, nl - 15)
        blk += lits.tobytes()
        blk += off.to_bytes(2, "little")
        if ml - 4 >= 15:
            _lz4_length(blk, ml - 19)
        out += lits.tobytes()
        for _ in range(ml):
            out.append(out[-off])
    nl = total - len(out)
    blk.append(min(nl, 15) << 4)
    if nl >= 15:
        _lz4_length(blk, nl - 15)
    blk += rng.integers(0, 256, nl, dtype=np.uint8).tobytes()
    out += blk[len(blk) - nl:]
    return bytes(blk), bytes(out)


def _lz4_chunk(block, n):
    """A one-block "lz4" chunk of n decoded bytes."""
    return n.to_bytes(8, "big") + bytes(4) + len(block).to_bytes(4, "big") + block


def _bslz4_chunk(rng, elem, nblocks):
    """A "bslz4" chunk of nblocks 8192-byte blocks of random sequences (the
    bit planes of 8192 // elem elements each); returns (chunk, frame bytes),
    the frame from the planes by bitshuffle's definition."""
    blocks, frame = [], bytearray()
    n = 8192 // elem
    for _ in range(nblocks):
        blk, planes = _lz4_random_block(rng, 8192)
        blocks.append(blk)
        bits = np.unpackbits(np.frombuffer(planes, np.uint8).reshape(8 * elem, n // 8),
                             axis=1, bitorder="little")  # [plane 8j + k][element]
        vals = np.zeros(n, np.uint64)
        for r in range(8 * elem):
            vals |= bits[r].astype(np.uint64) << np.uint64(r)
        frame += vals.astype({2: np.uint16, 4: np.uint32}[elem]).tobytes()
    hdr = len(frame).to_bytes(8, "big") + (8192).to_bytes(4, "big")
    body = b"".join(len(b).to_bytes(4, "big") + b for b in blocks)
    return hdr + body, bytes(frame)


def test_random_sequences_are_lz4_blocks():
    # The crafted blocks decode, by the oracle, to what their sequences say;
    # where the LZ4 library is at hand it reads them too.
    rng = np.random.default_rng(11)
    pa = None
    try:
        import pyarrow as pa
    except ImportError:
        pass
    for total in [13, 40, 100, 1000, 8192, 20000]:
        for _ in range(4):
            blk, out = _lz4_random_block(rng, total)
            assert O.lz4_decode(blk, total) == out
            if pa is not None:
                assert pa.decompress(blk, decompressed_size=total, codec="lz4_raw",
                                     asbytes=True) == out


# ---------------------------------------------------------------------------
# The oracle and the chunk writer, on the CPU.
# ---------------------------------------------------------------------------

def test_oracle_reads_the_lz4_librarys_blocks():
    g = _golden()
    k = 0
    while f"raw_{k}" in g.files:
        raw = g[f"raw_{k}"].tobytes()
        assert O.lz4_decode(g[f"blk_{k}"].tobytes(), len(raw)) == raw, k
        k += 1
    assert k == 10


def test_oracle_accepts_what_the_lz4_library_accepts():
    g = _golden()
    k = 0
    while f"bad_{k}" in g.files:
        n = int(g[f"bad_n_{k}"])
        try:
            ok = len(O.lz4_decode(g[f"bad_{k}"].tobytes(), n)) == n
        except ValueError:
            ok = False
        assert ok == bool(g[f"bad_ok_{k}"]), k
        k += 1
    assert k == 7


def test_oracle_reads_chunks_of_the_librarys_blocks():
    g = _golden()
    assert np.array_equal(O.decompress_image(g["chunk_lz4"], "lz4", 32, 96, 130),
                          g["frame_lz4"])
    assert np.array_equal(O.decompress_image(g["chunk_bslz4"], "bslz4", 16, 101, 84),
                          g["frame_bslz4"])


def test_chunk_writer_blocks_are_read_by_the_lz4_library():
    pa = pytest.importorskip("pyarrow")
    from sfgb import synth
    rng = np.random.default_rng(3)
    for n in (1, 12, 13, 100, 4096, 8192, 30000):
        for data in (rng.integers(0, 256, n, dtype=np.uint8).tobytes(), bytes(n),
                     rng.poisson(0.4, n).astype(np.uint8).tobytes()):
            blk = synth.lz4_block(data)
            back = pa.decompress(blk, decompressed_size=n, codec="lz4_raw", asbytes=True)
            assert back == data
            assert O.lz4_decode(blk, n) == data


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32, np.uint64])
def test_bit_planes_are_bitshuffles(dtype):
    # Plane 8j + k holds bit k of byte j of every element, element i at bit
    # i % 8 of the plane's byte i / 8.
    from sfgb import synth
    rng = np.random.default_rng(4)
    n = 2056
    e = rng.integers(0, np.iinfo(dtype).max, n, dtype=dtype, endpoint=True)
    planes = synth.bitshuffle(e)
    size = e.itemsize
    b = e.view(np.uint8).reshape(n, size)
    for j in range(size):
        for k in range(8):
            row = planes[(8 * j + k) * (n // 8):(8 * j + k + 1) * (n // 8)]
            assert np.array_equal(np.unpackbits(row, bitorder="little"), (b[:, j] >> k) & 1)
    assert np.array_equal(O.bitunshuffle(planes, n, size).view(dtype), e)


def test_bitshuffle_default_block():
    # 8192 bytes' worth, a multiple of 8, at least 128 elements.
    assert [O.lib().or_bshuf_default_block(e) for e in (1, 2, 4, 8, 100)] == \
        [8192, 4096, 2048, 1024, 128]


@pytest.mark.parametrize("shape,dtype,alg,block", CHUNKS)
def test_oracle_round_trip(shape, dtype, alg, block):
    from sfgb import synth
    f = _frame(*shape, dtype, seed=shape[0] * 7 + shape[1])
    data = synth.chunk(f, alg, block) if alg else f.view(np.uint8).ravel()
    assert np.array_equal(O.decompress_image(data, alg, f.itemsize * 8, *shape), f)


def _corrupt_cases():
    """Chunks the host refuses before any device work, with the reference's
    text (decompress.cc:80-134)."""
    from sfgb import synth
    f = _frame(40, 60, np.uint32, 9)
    c = synth.chunk(f, "bslz4").tobytes()
    l4 = synth.chunk(f, "lz4", 1024).tobytes()
    size = f.nbytes
    hdr = size.to_bytes(8, "big")
    return [
        ("too short", c[:11], "bslz4", 32, "too short for a filter header"),
        ("header size", (size + 4).to_bytes(8, "big") + c[8:], "bslz4", 32,
         f"filter header says {size + 4} bytes uncompressed, expected {size}"),
        ("bit depth", c, "bslz4", 16,
         f"filter header says {size} bytes uncompressed, expected {size // 2}"),
        ("unknown", c, "zstd", 32, "unknown compression algorithm zstd"),
        ("raw size", f.tobytes()[:-4], "", 32,
         f"uncompressed frame is {size - 4} bytes, expected {size}"),
        ("lz4 truncated", l4[:12 + 2], "lz4", 32, "lz4 data truncated"),
        ("lz4 zero block", hdr + (1024).to_bytes(4, "big") + bytes(4), "lz4", 32,
         "lz4 block size out of range"),
        ("lz4 block past end", l4[:-1], "lz4", 32, "lz4 block size out of range"),
        ("bslz4 block size", hdr + (12).to_bytes(4, "big") + c[12:], "bslz4", 32,
         "bitshuffle decompression failed with code -81"),
    ]


def test_oracle_refusals_are_the_references():
    for what, data, alg, depth, text in _corrupt_cases():
        with pytest.raises(RuntimeError) as e:
            O.decompress_image(np.frombuffer(data, np.uint8), alg, depth, 40, 60)
        assert str(e.value) == text, what


def test_host_refusals_need_no_device():
    # The chunk's header and framing are checked on the host before any
    # device work: the C ABI refuses these without a GPU, with the same text.
    from sfgb import api
    for what, data, alg, depth, text in _corrupt_cases():
        with pytest.raises(api.DataError) as e:
            api.decompress_image(data, alg, depth, 40, 60)
        assert str(e.value) == text, what
    assert api.frame_bytes(4362, 4148, 32) == 4362 * 4148 * 4
    # Bitshuffle chunks of 8-bit pixels are decoded by the reference, not here.
    from sfgb import synth
    f8 = np.zeros((8, 8), np.uint8)
    with pytest.raises(api.SpotFinderError):
        api.decompress_image(synth.chunk(f8, "bslz4"), "bslz4", 8, 8, 8)


def test_more_host_refusals_need_no_device():
    # Framing errors of bitshuffle chunks past their end (code -1, where
    # bitshuffle itself would read past the chunk), pixel sizes the device
    # path does not take, and the find / scan entry points refusing the same
    # chunks before any device work.
    from sfgb import api, synth
    f = _frame(20, 24, np.uint32, 3)  # 480 elements: one partial block
    c = synth.chunk(f, "bslz4").tobytes()
    for cut in (14, 17, len(c) - 1):
        with pytest.raises(api.DataError) as e:
            api.decompress_image(c[:cut], "bslz4", 32, 20, 24)
        assert str(e.value) == "bitshuffle decompression failed with code -1"
        with pytest.raises(RuntimeError) as e:
            O.decompress_image(np.frombuffer(c[:cut], np.uint8), "bslz4", 32, 20, 24)
        assert str(e.value) == "bitshuffle decompression failed with code -1"
    g = _frame(7, 9, np.uint32, 4)  # 63 elements: a block of 56 and 7 raw
    cg = synth.chunk(g, "bslz4").tobytes()
    with pytest.raises(api.DataError):
        api.decompress_image(cg[:-2], "bslz4", 32, 7, 9)  # the raw tail cut short
    with pytest.raises(api.DataError) as e:
        api.find_compressed(c[:11], "bslz4", 32, 20, 24)
    assert str(e.value) == "too short for a filter header"
    with pytest.raises(api.SpotFinderError):
        api.find_compressed(c, "bslz4", 8, 20, 24)  # thresholds take 16 or 32 bits
    with pytest.raises(api.SpotFinderError) as e:
        api.scan_compressed(c, "bslz4", 8, 20, 24)
    assert "8-bit pixels" in str(e.value)
    with pytest.raises(api.DataError) as e:
        api.scan_compressed(c, "zstd", 32, 20, 24)
    assert str(e.value) == "unknown compression algorithm zstd"
    with pytest.raises(api.DataError) as e:
        api.find_narrowed(c[:12 + 3], "bslz4", 20, 24)
    assert str(e.value) == "bitshuffle decompression failed with code -1"


def test_uncompressed_host_copy_needs_no_device():
    from sfgb import api
    f = _frame(30, 40, np.uint16, 2)
    assert np.array_equal(api.decompress_image(f.tobytes(), "", 16, 30, 40), f)


# ---------------------------------------------------------------------------
# The device decoder.
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def api():
    from sfgb import api as a
    if not a.available():
        pytest.fail("no usable GB300: " + a.unavailable_reason())
    return a


@pytest.mark.gpu
@pytest.mark.parametrize("shape,dtype,alg,block", CHUNKS)
def test_device_decode_matches_the_oracle(api, shape, dtype, alg, block):
    import torch
    from sfgb import synth
    f = _frame(*shape, dtype, seed=shape[0] * 13 + shape[1])
    data = synth.chunk(f, alg, block) if alg else f.view(np.uint8).ravel()
    want = O.decompress_image(data, alg, f.itemsize * 8, *shape)
    assert np.array_equal(want, f)
    assert np.array_equal(api.decompress_image(data, alg, f.itemsize * 8, *shape), want)
    d = api.decompress_device(data, alg, f.itemsize * 8, *shape)
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy().view(dtype), want)


@pytest.mark.gpu
def test_device_decodes_the_librarys_chunks(api):
    g = _golden()
    assert np.array_equal(api.decompress_image(g["chunk_lz4"], "lz4", 32, 96, 130),
                          g["frame_lz4"])
    assert np.array_equal(api.decompress_image(g["chunk_bslz4"], "bslz4", 16, 101, 84),
                          g["frame_bslz4"])
    # Each of the library's blocks as a one-block "lz4" chunk of its bytes.
    k = 0
    while f"raw_{k}" in g.files:
        raw = g[f"raw_{k}"]
        blk = g[f"blk_{k}"].tobytes()
        if raw.size:
            chunk = raw.size.to_bytes(8, "big") + bytes(4) + len(blk).to_bytes(4, "big") + blk
            got = api.decompress_image(chunk, "lz4", 8, 1, raw.size)
            assert np.array_equal(got, raw), k
        k += 1


@pytest.mark.gpu
def test_device_accepts_what_the_lz4_library_accepts(api):
    # The damaged blocks as one-block "lz4" chunks: refused (with the
    # reference's text) exactly where the library refuses them, and the
    # context still usable after each refusal.
    g = _golden()
    k = 0
    while f"bad_{k}" in g.files:
        n = int(g[f"bad_n_{k}"])
        blk = g[f"bad_{k}"].tobytes()
        chunk = n.to_bytes(8, "big") + bytes(4) + len(blk).to_bytes(4, "big") + blk
        if bool(g[f"bad_ok_{k}"]):
            assert api.decompress_image(chunk, "lz4", 8, 1, n).size == n
        else:
            with pytest.raises(api.DataError) as e:
                api.decompress_image(chunk, "lz4", 8, 1, n)
            assert str(e.value).startswith("lz4 "), k
        k += 1
    f = _frame(20, 30, np.uint32, 5)
    from sfgb import synth
    assert np.array_equal(api.decompress_image(synth.chunk(f), "bslz4", 32, 20, 30), f)


@pytest.mark.gpu
def test_device_decodes_random_sequences(api):
    # Every sequence shape of the windowed parse, in plain LZ4 blocks
    # (decoded straight into the frame) and in bitshuffle blocks of 16- and
    # 32-bit pixels (decoded in shared memory: byte copies and word copies).
    rng = np.random.default_rng(12)
    for total in [13, 31, 32, 33, 64, 100, 1000, 8192, 20000, 65536]:
        for _ in range(3):
            blk, out = _lz4_random_block(rng, total)
            got = api.decompress_image(_lz4_chunk(blk, total), "lz4", 8, 1, total)
            assert got.tobytes() == out, total
    for elem in (2, 4):
        for nblocks in (1, 3, 16):
            chunk, frame = _bslz4_chunk(rng, elem, nblocks)
            w = len(frame) // elem
            want = O.decompress_image(chunk, "bslz4", 8 * elem, 1, w)
            assert want.tobytes() == frame
            got = api.decompress_image(chunk, "bslz4", 8 * elem, 1, w)
            assert got.tobytes() == frame, (elem, nblocks)


@pytest.mark.gpu
def test_device_refuses_what_the_oracle_refuses(api):
    # Random sequences with bytes changed at random: the device accepts the
    # block with the oracle's bytes, or refuses it, as the oracle does.
    rng = np.random.default_rng(13)
    refused = 0
    for case in range(200):
        total = int(rng.choice([40, 300, 2000, 8192]))
        blk, _ = _lz4_random_block(rng, total)
        bad = bytearray(blk)
        for _ in range(int(rng.integers(1, 4))):
            bad[int(rng.integers(0, len(bad)))] = int(rng.integers(0, 256))
        chunk = _lz4_chunk(bytes(bad), total)
        try:
            want = O.decompress_image(chunk, "lz4", 8, 1, total)
        except RuntimeError as e:
            with pytest.raises(api.DataError) as d:
                api.decompress_image(chunk, "lz4", 8, 1, total)
            assert str(d.value).startswith("lz4 "), case
            refused += 1
            continue
        got = api.decompress_image(chunk, "lz4", 8, 1, total)
        assert got.tobytes() == want.tobytes(), case
    assert 20 < refused < 200


@pytest.mark.gpu
def test_device_refuses_a_damaged_bitshuffle_block(api):
    from sfgb import synth
    f = _frame(100, 120, np.uint32, 6)
    c = bytearray(synth.chunk(f).tobytes())
    c[16:20] = bytes([0xF0, 0xFF, 0xFF, 0xFF])  # the first block: a literal run past its end
    with pytest.raises(api.DataError) as e:
        api.decompress_image(bytes(c), "bslz4", 32, 100, 120)
    assert str(e.value) == "bitshuffle decompression failed with code -91"
    with pytest.raises(api.DataError):
        api.find_compressed(bytes(c), "bslz4", 32, 100, 120)
    assert np.array_equal(api.decompress_image(synth.chunk(f), "bslz4", 32, 100, 120), f)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,alg,block", [(np.uint32, "bslz4", 0), (np.uint16, "bslz4", 0),
                                             (np.uint32, "lz4", 65536), (np.uint16, "", 0)])
def test_find_compressed_matches_the_oracle(api, dtype, alg, block):
    from sfgb import synth
    p = synth.preset("eiger_16m", height=700, width=900, n_frames=2, spots_per_frame=150.0,
                     seed=41)
    sw = synth.Sweep(p)
    for i in range(2):
        f = sw.frame(i)
        if dtype == np.uint16:
            g = np.minimum(f, 0xFFFD).astype(np.uint16)
            g[f == 0xFFFFFFFF] = 0xFFFF
            f = g
        data = synth.chunk(f, alg, block) if alg else f.view(np.uint8).ravel()
        got = api.find_compressed(data, alg, f.itemsize * 8, *f.shape)
        want = O.dext(f)
        assert got.tobytes() == want.tobytes(), (alg, i)


@pytest.mark.gpu
def test_find_compressed_with_parameters(api):
    from sfgb import synth
    f = _frame(333, 444, np.uint32, 8, mean=3.0)
    for params in (api.Params(gain=1.5), api.Params(kernel_x=2, kernel_y=2),
                   api.Params(algorithm=api.DISPERSION)):
        got = api.find_compressed(synth.chunk(f), "bslz4", 32, 333, 444, params=params)
        want = O.dext(f, O.Params(algorithm=params.algorithm, kernel_x=params.kernel_x,
                                  kernel_y=params.kernel_y, gain=params.gain))
        assert got.tobytes() == want.tobytes()


@pytest.mark.gpu
def test_full_frame_round_trip(api):
    # A 4362 x 4148 frame: the decoded frame is the frame, and the signal
    # list from its chunk is the list from the frame itself.
    from sfgb import synth
    f = synth.Sweep(synth.preset("eiger_16m", n_frames=1)).frame(0)
    c = synth.chunk(f)
    assert c.size * 8 < f.nbytes
    assert np.array_equal(api.decompress_image(c, "bslz4", 32, *f.shape), f)
    got = api.find_compressed(c, "bslz4", 32, *f.shape)
    assert got.tobytes() == api.find(f).tobytes()
    assert got.tobytes() == O.dext(f).tobytes()
    # mxi_max's scan of the chunk, and --gpu-force on it (its counts fit).
    assert api.scan_compressed(c, "bslz4", 32, *f.shape) == O.scan_frame(f)
    narrowed, worst, ok = O.narrow_to_16(f)
    assert ok
    got = api.find_narrowed(c, "bslz4", *f.shape)
    assert got.tobytes() == O.dext(narrowed).tobytes()


# ---------------------------------------------------------------------------
# mxi_max's scan and the --gpu-force narrowing, on the device.
# ---------------------------------------------------------------------------

def test_scan_oracle_known_answers():
    # Markers are max() - 1 (bad) and max() (tile join); 0xFFFD and above
    # valid counts are "over" (apps/mxi_max.cc:47-67).
    f = np.array([[1, 2, 0xFFFFFFFE, 0xFFFFFFFF], [70000, 0xFFFD, 5, 0]], np.uint32)
    assert O.scan_frame(f) == (70000, 1, 1, 2)
    g = np.array([[1, 0xFFFE, 0xFFFF, 0xFFFF], [0xFFFD, 7, 0, 0xFFFC]], np.uint16)
    assert O.scan_frame(g) == (0xFFFD, 1, 2, 1)
    n, worst, ok = O.narrow_to_16(f)
    assert (worst, ok) == (70000, False)
    assert n.ravel().tolist() == [1, 2, 0xFFFE, 0xFFFF, 70000 & 0xFFFF, 0xFFFD, 5, 0]
    assert O.narrow_to_16(np.array([0xFFFC, 0xFFFFFFFF], np.uint32))[1:] == (0xFFFC, True)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.uint16, np.uint32])
def test_scan_matches_the_oracle(api, dtype):
    import torch
    from sfgb import synth
    for h, w, seed in ((1, 1, 1), (3, 7, 2), (257, 301, 3), (1000, 1030, 4)):
        f = _frame(h, w, dtype, seed, mean=4.0)
        if f.size > 10:
            f.ravel()[5] = np.iinfo(dtype).max - 1
            f.ravel()[-3] = 0xFFFD if dtype == np.uint16 else 123456
        want = O.scan_frame(f)
        view = np.int16 if dtype == np.uint16 else np.int32
        d = torch.from_numpy(f.view(view)).cuda()
        assert api.scan_device(d) == want
        assert api.scan_device(d.view(-1)[1:]) == O.scan_frame(f.ravel()[1:])  # unaligned
        c = synth.chunk(f) if f.size >= 8 else f.view(np.uint8).ravel()
        alg = "bslz4" if f.size >= 8 else ""
        assert api.scan_compressed(c, alg, f.itemsize * 8, h, w) == want


@pytest.mark.gpu
def test_narrowed_threshold_matches_the_oracle(api):
    # --gpu-force: the 32-bit frame narrowed as narrow_to_16 narrows it, then
    # the 16-bit threshold (the reference's float tests).
    from sfgb import synth
    p = synth.preset("eiger_16m", height=600, width=800, n_frames=1, spots_per_frame=80.0,
                     seed=77)
    f = synth.Sweep(p).frame(0)
    f = np.where(f >= 0xFFFFFFFE, f, np.minimum(f, 0xFFFC)).astype(np.uint32)
    narrowed, worst, ok = O.narrow_to_16(f)
    assert ok
    want = O.dext(narrowed)
    for alg in ("", "bslz4", "lz4"):
        data = synth.chunk(f, alg, 65536) if alg else f.view(np.uint8).ravel()
        got = api.find_narrowed(data, alg, *f.shape)
        assert got.tobytes() == want.tobytes(), alg


@pytest.mark.gpu
def test_narrowed_threshold_refuses_large_counts(api):
    from sfgb import synth
    f = np.minimum(_frame(100, 128, np.uint32, 12), 0xFFFC)
    f[50, 60] = 0xFFFD
    with pytest.raises(api.NarrowError) as e:
        api.find_narrowed(synth.chunk(f), "bslz4", 100, 128)
    assert e.value.offending == 0xFFFD
    f[50, 60] = 0xFFFC
    got = api.find_narrowed(synth.chunk(f), "bslz4", 100, 128)
    assert got.tobytes() == O.dext(O.narrow_to_16(f)[0]).tobytes()
