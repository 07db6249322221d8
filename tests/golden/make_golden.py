"""Regenerate the golden fixtures in this directory from the reference's own
CPU code (oracle/_ref/libref.so, built in place from the reference tree by
oracle/build_ref.sh). Run from the repository root where the reference tree
exists:

    python tests/golden/make_golden.py

Fixtures:
  dext_fused_cases.npz    the 48 frames of tests/spots/test_dext_fused.cc
                          (8 sizes x 3 means x {u16, u32}, seeds 1..24, the
                          reference's own generator) with dext<T>()'s output
  dext_device_frames.npz  the 7 frames of tests/spots/test_dext_gpu.cc
                          (synthetic_frame.hh make_frame) with dext<u16>()'s
                          output and dext<u32>()'s output on the frame widened
                          to 32 bits
  sweep_small.npz         a 12-frame 256 x 320 uint32 sweep from this
                          package's generator, with dext<u32>() per frame and
                          dials_spots::Labeller's spots, kept pixels and
                          counts in 3-D and 2-D, and with frame 7 missing (a gap)
  refl_small.refl         refl::write of the 3-D spot table of sweep_small,
                          shoeboxes on (byte-exact writer fixture)
  refl_small_opts.refl    the same table without shoeboxes, with id 3, panel 1
                          and an experiment identifier
  refl_small_2d.refl      refl::write of the 2-D spot table, shoeboxes on, with
                          an identifier
  lz4_blocks.npz          LZ4 blocks written by the LZ4 library (pyarrow's
                          "lz4_raw" codec) over assorted inputs, corrupted
                          variants with whether the library accepts them, and
                          two chunks framed as HDF5 stores them whose blocks
                          the library wrote: "lz4" (a uint32 frame, 4096-byte
                          blocks) and "bslz4" (a uint16 frame's bit planes,
                          bitshuffle's default blocks, a partial last block
                          and 4 raw tail elements)

Only the reflection-table fixtures: python tests/golden/make_golden.py refl
Only the LZ4 fixtures (needs pyarrow, not the reference):
    python tests/golden/make_golden.py lz4
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "dials-metal_gb300"))

import oracle as O  # noqa: E402

REFL_IDENTIFIER = "5b0f3c2e-9d41-4a7b-8e16-2c7d9a01f4b3"

FUSED_SIZES = [(1, 1), (5, 7), (32, 32), (33, 65), (100, 37), (67, 300), (257, 511), (64, 96)]
DEVICE_FRAMES = [("exact tile", 32, 32, 1, 12.0, False),
                 ("under one tile", 19, 27, 2, 8.0, False),
                 ("ragged", 200, 301, 3, 15.0, False),
                 ("ragged, masked", 200, 301, 4, 15.0, True),
                 ("dark", 128, 128, 5, 1.0, False),
                 ("module", 512, 1030, 6, 20.0, True)]


def fused_cases():
    out = {}
    meta = []
    seed = 1
    i = 0
    for (h, w) in FUSED_SIZES:
        for mean in (0.3, 2.0, 12.0):
            for dt in (np.uint16, np.uint32):
                f = O.ref_fused_make(h, w, seed, mean, dt)
                out[f"frame_{i}"] = f
                out[f"signal_{i}"] = O.ref_dext(f)
                meta.append((h, w, seed, mean, 16 if dt == np.uint16 else 32))
                i += 1
            seed += 1
    out["meta"] = np.array(meta, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "dext_fused_cases.npz"), **out)
    return i


def device_frames():
    out = {}
    names = []
    for i, (name, h, w, seed, bg, masked) in enumerate(DEVICE_FRAMES):
        f = O.ref_make_frame(h, w, seed, bg, masked)
        out[f"frame_{i}"] = f
        out[f"signal16_{i}"] = O.ref_dext(f)
        out[f"signal32_{i}"] = O.ref_dext(f.astype(np.uint32))
        names.append(name)
    # The all-masked frame the device test builds by hand.
    i = len(DEVICE_FRAMES)
    f = np.full((64, 64), 0xFFFF, np.uint16)
    out[f"frame_{i}"] = f
    out[f"signal16_{i}"] = O.ref_dext(f)
    out[f"signal32_{i}"] = O.ref_dext(np.full((64, 64), 0xFFFFFFFF, np.uint32))
    names.append("entirely masked")
    out["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "dext_device_frames.npz"), **out)
    return len(names)


def sweep_small():
    from sfgb import synth
    p = synth.preset("plain_1m", height=256, width=320, n_frames=12,
                     spots_per_frame=25.0, row_band_start=100, row_band_len=3,
                     col_band_start=200, col_band_len=2, n_hot=10, seed=77)
    sw = synth.Sweep(p)
    frames = np.stack([sw.frame(i) for i in range(p.n_frames)])
    out = {"frames": frames}
    signals = [O.ref_dext(f) for f in frames]
    for i, s in enumerate(signals):
        out[f"signal_{i}"] = s
    for tag, two_d, skip in (("3d", False, None), ("2d", True, None), ("gap", False, 7)):
        lab = O.RefLabeller(p.height, p.width, two_d=two_d)
        for i, s in enumerate(signals):
            if i == skip:
                continue
            lab.add(i, s)
        r = lab.finish()
        out[f"spots_{tag}"] = r.spots
        out[f"pixels_{tag}"] = r.pixels
        out[f"counts_{tag}"] = np.array([r.counts[k] for k in O.COUNT_NAMES], np.uint64)
        if tag == "3d":
            lab.write_refl(os.path.join(HERE, "refl_small.refl"), shoeboxes=True)
            lab.write_refl(os.path.join(HERE, "refl_small_opts.refl"), shoeboxes=False,
                           identifier=REFL_IDENTIFIER, id=3, panel=1)
        if tag == "2d":
            lab.write_refl(os.path.join(HERE, "refl_small_2d.refl"), shoeboxes=True,
                           identifier=REFL_IDENTIFIER)
    np.savez_compressed(os.path.join(HERE, "sweep_small.npz"), **out)
    return len(out["spots_3d"])


def lz4_blocks():
    """LZ4 blocks from the LZ4 library itself (pyarrow's lz4_raw codec)."""
    import pyarrow as pa
    from sfgb import synth

    def lz4(data: bytes) -> bytes:
        return pa.compress(data, codec="lz4_raw", asbytes=True)

    def accepted(block: bytes, n: int) -> bool:
        try:
            return len(pa.decompress(block, decompressed_size=n, codec="lz4_raw",
                                     asbytes=True)) == n
        except OSError:
            return False

    rng = np.random.default_rng(2024)
    raws = [b"", b"a", bytes(12), bytes(13), bytes(range(256)) * 3,
            rng.integers(0, 256, 5000, dtype=np.uint8).tobytes(),
            rng.poisson(0.7, 8192).astype(np.uint8).tobytes(),
            (b"spotfinder" * 1000)[:9999], bytes(70000),
            rng.integers(0, 4, 100000, dtype=np.uint8).tobytes()]
    out = {}
    for k, raw in enumerate(raws):
        out[f"raw_{k}"] = np.frombuffer(raw, np.uint8)
        out[f"blk_{k}"] = np.frombuffer(lz4(raw), np.uint8)
    # Damaged blocks, each with the size it should decode to and whether the
    # library accepts it: case 7 truncated, with a literal run past the end,
    # with a byte added; a match reaching before the output's start; a match
    # into the last 5 bytes; a match whose literals reach the last 12 bytes
    # of output; a well-formed block of 36 bytes.
    good = lz4(raws[7])
    n7 = len(raws[7])
    bad = [(good[:-1], n7), (b"\xf0\xff\xff" + good[3:], n7), (good + b"\x00", n7),
           (b"\x40abcd\x09\x00\x50hello", 13), (b"\x40abcd\x04\x00\x00", 8),
           (b"\x40abcd\x04\x00\x50hello", 13),
           (b"\xf4\x01" + b"0123456789abcdef" + b"\x04\x00\xc0" + b"tail of bloc", 36)]
    for k, (blk, n) in enumerate(bad):
        out[f"bad_{k}"] = np.frombuffer(blk, np.uint8)
        out[f"bad_n_{k}"] = np.array(n)
        out[f"bad_ok_{k}"] = np.array(accepted(blk, n))
    # An "lz4" chunk: 12-byte header, blocks of 4096 bytes.
    f32 = rng.poisson(1.2, (96, 130)).astype(np.uint32)
    f32[::17, :] = 0xFFFFFFFF
    raw = f32.tobytes()
    parts = [len(raw).to_bytes(8, "big"), (4096).to_bytes(4, "big")]
    for at in range(0, len(raw), 4096):
        blk = lz4(raw[at:at + 4096])
        parts += [len(blk).to_bytes(4, "big"), blk]
    out["frame_lz4"] = f32
    out["chunk_lz4"] = np.frombuffer(b"".join(parts), np.uint8)
    # A "bslz4" chunk: bitshuffle's default 4096-element blocks of a uint16
    # frame, the last partial block, then 4 elements raw.
    f16 = rng.poisson(2.0, (101, 84)).astype(np.uint16)
    f16[:, 40:44] = 0xFFFF
    e = f16.ravel()
    bs = 4096
    nfull, last = e.size // bs, e.size % bs - e.size % bs % 8
    parts = [(e.size * 2).to_bytes(8, "big"), (bs * 2).to_bytes(4, "big")]
    for b in range(nfull + (1 if last else 0)):
        n = bs if b < nfull else last
        blk = lz4(synth.bitshuffle(e[b * bs:b * bs + n]).tobytes())
        parts += [len(blk).to_bytes(4, "big"), blk]
    parts.append(e[nfull * bs + last:].tobytes())
    out["frame_bslz4"] = f16
    out["chunk_bslz4"] = np.frombuffer(b"".join(parts), np.uint8)
    np.savez_compressed(os.path.join(HERE, "lz4_blocks.npz"), **out)
    return len(raws)


if __name__ == "__main__":
    if sys.argv[1:] == ["lz4"]:
        print("lz4 cases:", lz4_blocks())
        sys.exit(0)
    if not O.ref_available():
        O.build(quiet=False)
    if not O.ref_available():
        sys.exit("the reference library could not be built (no reference tree?)")
    if sys.argv[1:] == ["refl"]:
        # The reflection-table fixtures alone (sweep_small.npz rewritten with
        # the same content).
        print("sweep spots (3-D):", sweep_small())
        sys.exit(0)
    print("fused cases:", fused_cases())
    print("device frames:", device_frames())
    print("sweep spots (3-D):", sweep_small())
