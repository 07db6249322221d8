"""Benchmark of the spot-finder hot path on EIGER2 16M-shaped frames.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (`eiger_16m`): 4362 x 4148 uint32 frames with the EIGER2 module gaps
masked, Poisson background 0.3 at the edge rising to 1.5 at the centre, 3000
spots per frame spanning 2-5 frames, dispersion_extended at the reference's
defaults. Seeded synthetic frames stand in for detector data.

A step is one batch of 64 frames through the whole hot path: the threshold
(a tuned plan's launch sequence replayed as a CUDA graph) and the 3-D
labelling of the batch's signal lists into spots (sf_label_add_device), both
on the device. `value` is frames/s with the frames already in HBM (a pool of
distinct frames larger than L2, cycled); the roofline is the threshold's
launch sequence, timed inside each step. `e2e` is the same path through the
served API (sf_server_*): pinned host frames submitted at full rate, each
copied in, thresholded and labelled in order, and every sweep's spot table
read back, inside the timed region. Its `threshold_only` entry is the
threshold alone through the C ABI's host-frame call (sf_find_u32, the
gpu::find drop-in) from one host thread a core, with `u16` / `bslz4_u*`
variants (16-bit frames; bitshuffle+LZ4 chunks decoded on the device).

--impl reference times the reference's CPU path on this host's cores: the
CPU restatement of dext() plus the streaming labeller (the reference's own
code is not present on the GPU host), one frame per worker thread.

Under torchrun each rank processes its own sweep (independent sweeps: no
exchange), the timing is the max over ranks, and rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "dials-metal_gb300"))

METRIC = "16M-frame frames/s (device & end-to-end) as % HBM roofline; served p50/p99 latency"
WORKLOAD = ("eiger_16m: 4362x4148 uint32 (EIGER2 16M tiling, module gaps masked), "
            "Poisson 0.3 edge -> 1.5 centre, 3000 spots/frame spanning 2-5 frames, "
            "dispersion_extended defaults (kernel 3,3, gain 1, sigma_b 6, sigma_s 3, "
            "min_local 2)")
H, W = 4362, 4148


# DRAM bytes (read + write) that one 16M frame of the eiger_16m workload costs
# across the threshold's kernels in a timed 64-frame launch, from an ncu
# capture of this bench without cache flushes between kernels (11,235 MB for
# the launch: lat_stage01 5,266 MB, lat_verify 2,098 MB, lat_stage2 2,621 MB,
# the scans and the list 1,250 MB); the algorithmic bytes are 76.5 MB a frame.
DRAM_BYTES_PER_FRAME = 162.0e6


# Kernels a timed step launches: the threshold plan's graph (lat_stage01,
# lat_tiles, lat_verify, mask_sums, mask_prefix, lat_stage2, pass_sums,
# pass_scatter) and the labeller's (27 kernels and six three-kernel
# exclusive scans; sf_label.cu, Labeller::enqueue).
THRESHOLD_KERNELS = 8
LABEL_KERNELS = 45


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float, world: int, device=None) -> float:
    """Max of a per-rank float across ranks (identity when world == 1)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, world: int, device=None) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0, path: str | None = None):
        self.index = index
        self.path = path
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self._t.join(timeout=2)
        if self.path:
            with open(self.path, "w") as f:
                f.write(self.QUERY + "\n" + "\n".join(self.lines) + "\n")
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_gbs() -> tuple[float, str]:
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def make_pool(n_frames: int, seed_offset: int):
    from sfgb import synth
    p = synth.preset("eiger_16m", n_frames=max(n_frames, 2))
    p.seed = p.seed + seed_offset
    sw = synth.Sweep(p)
    return [sw.frame(i) for i in range(n_frames)]


def cpu_baseline(frames, seconds_budget: float = 20.0, threads: int | None = None) -> dict:
    """The CPU path (dext restatement + labeller) on this host: one frame per
    worker thread, labelling in frame order, as mxi_find -j N does
    (src/spots/find_spots.cc:732-891), over a bounded sample."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.dext(frames[0])  # warm (and measure one frame single-threaded)
    one = time.perf_counter() - t0
    # About seconds_budget of wall time on all threads.
    n = int(seconds_budget * threads / max(one, 1e-3))
    n = max(threads, min(n, 16 * threads))
    lab = oracle.Labeller(H, W)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        results = ex.map(lambda i: oracle.dext(frames[i % len(frames)]), range(n))
        for i, sig in enumerate(results):
            lab.add(i, sig)
    lab.finish()
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{n} frames of the eiger_16m workload (threshold + 3-D labelling), "
                      f"{threads} threads, {dt:.1f} s; 1 frame on 1 thread {one * 1e3:.0f} ms"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    frames = make_pool(4, 0)
    best = None
    for _ in range(args.warmup):
        cpu_baseline(frames, seconds_budget=2.0)
    vals = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(frames, seconds_budget=6.0))
    elapsed = time.perf_counter() - t_all
    v = statistics.median([x["value"] for x in vals])
    best = vals[0]
    line = {"metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": elapsed / max(args.steps, 1) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": run_config(args.frames_per_step, args.pool), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "frames/s", "cores": best["cores"],
                             "kind": "port", "sample": best["sample"] +
                             " (the reference's CPU dext/Labeller restated in C and pinned "
                             "to the reference's own output; the reference's own build "
                             "does not travel to the GPU host)"},
            "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


SERVED_DETECTORS = {
    "1M": ("plain_1m", 1065, 1030),
    "4M": ("batch_4m", 2162, 2068),
    "9M": ("batch_9m", 3262, 3108),
    "16M": ("eiger_16m", H, W),
    "16M-dense": ("dense_16m", H, W),
}


def served(seconds: float = 4.0, seed: int = 4000, rates=None, chunks: bool = False,
           kinds=None, label_capacity: int = 0, capacity_divisor: int = 16) -> dict:
    """The served form on the mixed-detector workload: six sweeps (16M, 16M,
    9M, 4M, 4M, 1M) arriving at once, each with Poisson frame arrivals at a
    rate drawn from 100-750 Hz, submitted as they arrive from pinned host
    frames (with `chunks`, as bitshuffle+LZ4 chunks decoded on the device);
    every frame thresholded and labelled. p50/p99 are submit-to-labelled
    latencies over all frames."""
    import ctypes
    from sfgb import api, serve, synth
    L = api.lib()
    rng = np.random.default_rng(seed)
    kinds = kinds or ["16M", "16M", "9M", "4M", "4M", "1M"]
    pools, ptrs = {}, []
    for k in set(kinds):
        name, h, w = SERVED_DETECTORS[k]
        p = synth.preset(name, height=h, width=w, n_frames=4)
        sw = synth.Sweep(p)
        pool = []
        for i in range(4):
            f = sw.frame(i)
            data = synth.chunk(f) if chunks else f.view(np.uint8).ravel()
            ptr = L.sf_host_alloc(data.size)
            np.ctypeslib.as_array((ctypes.c_uint8 * data.size).from_address(ptr))[:] = data
            pool.append((ptr, data.size))
            ptrs.append(ptr)
        pools[k] = pool
    srv = serve.Server(max_batch=16, ring=32, label_capacity=label_capacity,
                       capacity_divisor=capacity_divisor)
    drawn = rng.uniform(100.0, 750.0, size=len(kinds))
    rates = drawn if rates is None else np.asarray(rates, dtype=float)
    ids = [srv.open_sweep(SERVED_DETECTORS[k][1], SERVED_DETECTORS[k][2]) for k in kinds]
    arrivals = [np.cumsum(rng.exponential(1.0 / r, size=int(r * seconds * 1.5) + 8))
                for r in rates]
    arrivals = [a[a < seconds] for a in arrivals]
    done = []
    stop = threading.Event()

    def feed(i):
        t0 = start_t[0]
        for n, t in enumerate(arrivals[i]):
            dt = t0 + t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            # The pool repeats every 4 frames: a gap in the frame numbers at
            # each repeat closes every spot there (dials_spots.cc:65-69), as
            # spots end in a real sweep, instead of stitching the repeats.
            ptr, nbytes = pools[kinds[i]][n % 4]
            if chunks:
                srv.submit_chunk(ids[i], n + n // 4, ptr, "bslz4", nbytes)
            else:
                srv.submit(ids[i], n + n // 4, ptr)

    last = [0.0]

    def collect():
        deadline = time.perf_counter() + seconds + 120.0
        while (not stop.is_set() or len(done) < total) and time.perf_counter() < deadline:
            got = srv.poll(4096, 50)
            if got:
                last[0] = time.perf_counter()
                done.extend(got)

    total = int(sum(len(a) for a in arrivals))
    start_t = [time.perf_counter() + 0.2]
    feeders = [threading.Thread(target=feed, args=(i,)) for i in range(len(kinds))]
    col = threading.Thread(target=collect)
    col.start()
    for t in feeders:
        t.start()
    for t in feeders:
        t.join()
    spots = 0
    failed = []
    for sid in ids:
        try:
            srv.finish_sweep(sid, read=False)
        except api.SpotFinderError as e:  # reported in the line, not fatal to the run
            failed.append(str(e))
        spots += srv.n_spots(sid)
    stop.set()
    col.join()
    # Served throughput: frames over the time from the first arrival to the
    # last frame labelled (reading the results back afterwards is not serving).
    wall = last[0] - start_t[0]
    stats = srv.stats()
    srv.close()
    for ptr in ptrs:
        L.sf_host_free(ptr)
    lat = np.array([d["latency_ms"] for d in done])
    bad = sum(1 for d in done if d["status"] != 0)
    by = {}
    for k in sorted(set(kinds)):
        sel = np.array([d["latency_ms"] for d in done
                        if kinds[ids.index(d["sweep"])] == k])
        by[k] = {"frames": int(len(sel)), "p50_ms": float(np.percentile(sel, 50)),
                 "p99_ms": float(np.percentile(sel, 99))}
    offered = float(sum(rates))
    link = sum(len(arrivals[i]) * (pools[kinds[i]][0][1] if chunks else
                                   SERVED_DETECTORS[kinds[i]][1] * SERVED_DETECTORS[kinds[i]][2] * 4)
               for i in range(len(kinds))) / seconds / 1e9
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "frames": int(len(lat)), "frames_per_s": len(lat) / wall,
            "offered_frames_per_s": offered, "errors": bad, "spots": spots,
            "host_link_gbs_offered": link,
            "failed_sweeps": failed,
            "server": stats,
            "by_detector": by,
            "workload": f"{len(kinds)} concurrent sweeps ({', '.join(kinds)}), Poisson arrivals at "
                        + ", ".join(f"{r:.0f}" for r in rates) + f" Hz for {seconds:.0f} s, "
                        + ("as bitshuffle+LZ4 chunks (sf_server_submit_chunk), " if chunks else "")
                        + "threshold and 3-D labelling of every frame (sf_server_*)"}


def served_e2e(n_frames: int, frames_per_step: int, h2d_gbs=None, n_sweeps: int = 4,
               pool: int = 8, chunks: bool = False) -> dict:
    """The whole path end to end through the served API (sf_server_*): four
    16M sweeps of pinned host frames (or, with `chunks`, their bitshuffle+LZ4
    chunks) submitted as fast as the calls return, each frame copied in,
    thresholded and labelled in order on the device; then every sweep
    finished and its spot table read back to the host. Timed from the first
    submit to the last spot table on the host."""
    import ctypes
    from sfgb import labeller, serve, synth
    L = lab = serve._lib()
    p = synth.preset("eiger_16m", n_frames=pool)
    p.seed = p.seed + 77
    sw = synth.Sweep(p)
    host = []
    for i in range(pool):
        f = sw.frame(i)
        data = synth.chunk(f) if chunks else f.view(np.uint8).ravel()
        ptr = L.sf_host_alloc(data.size)
        if not ptr:
            raise SystemExit("sf_host_alloc failed")
        np.ctypeslib.as_array((ctypes.c_uint8 * data.size).from_address(ptr))[:] = data
        host.append((ptr, data.size))
    srv = serve.Server(max_batch=16, ring=32)

    def run(n_per_sweep):
        ids = [srv.open_sweep(H, W) for _ in range(n_sweeps)]
        for k in range(n_per_sweep):
            # Consecutive frame numbers, a gap where the pool repeats.
            for i, sid in enumerate(ids):
                ptr, nbytes = host[(k + i) % pool]
                if chunks:
                    srv.submit_chunk(sid, k + k // pool, ptr, "bslz4", nbytes)
                else:
                    srv.submit(sid, k + k // pool, ptr)
        want, got = n_per_sweep * n_sweeps, 0
        deadline = time.perf_counter() + 120.0
        while got < want and time.perf_counter() < deadline:
            got += len(srv.poll(4096, 20))
        if got < want:
            raise SystemExit(f"served e2e: {got} of {want} frames done")
        d2h = 0
        for sid in ids:
            srv.finish_sweep(sid, read=False)
            h = L.sf_server_labeller(srv._s, sid)
            ns = lab.sf_label_n_spots(h)
            spots = np.empty(ns, labeller.SPOT_DTYPE)
            if lab.sf_label_spots(h, spots.ctypes.data, ns) != 0:
                raise SystemExit("served e2e: reading spots failed")
            d2h += spots.nbytes
            srv.close_sweep(sid)
        return d2h

    run(2 * pool)  # warm-up: every launch shape captured once
    per = max(1, n_frames // n_sweeps)
    t0 = time.perf_counter()
    d2h = run(per)
    dt = time.perf_counter() - t0
    srv.close()
    frames = per * n_sweeps
    steps = frames / frames_per_step
    h2d = sum(n for _, n in host) / pool * frames
    for ptr, _ in host:
        L.sf_host_free(ptr)
    out = {"value": frames / dt, "unit": "frames/s",
           "h2d_bytes_per_step": int(h2d / steps), "d2h_bytes_per_step": int(d2h / steps),
           "frames": frames, "seconds": dt, "achieved_h2d_gbs": h2d / dt / 1e9,
           "path": f"sf_server_* (the served API): {n_sweeps} 16M sweeps of "
                   + ("bitshuffle+LZ4 chunks decoded on the device" if chunks else
                      "raw uint32 frames") + " in pinned host memory, submitted at full rate, "
                   "copied in, thresholded and labelled in frame order on the device; every "
                   "sweep finished and its spot table read back to the host inside the timed "
                   "region"}
    if h2d_gbs and not chunks:
        out["h2d_peak_gbs"] = h2d_gbs
        out["frac_of_h2d_peak"] = out["achieved_h2d_gbs"] / h2d_gbs
    return out


def batched_legs(dev, steps: int = 5, warmup: int = 3) -> dict:
    """The batched form's own workload: 4M (2162x2068) and 9M (3262x3108)
    frames, Poisson 1.0, 1500 spots a frame, 64 distinct frames in HBM a
    shape (larger than L2). Per kernel size 2,2 / 3,3 / 4,4
    (dispersion_extended) and for the dispersion algorithm (kernel 3,3), a
    plan tuned on the frames (frames a launch sequence, 64/32/16, and the
    strip run length) replayed as a CUDA graph, beside the plain per-frame
    device path on the same frames; and a mixed batch of the served
    detectors (4 frames each of 16M, 9M, 4M and 1M) in one launch sequence
    beside the same frames thresholded shape by shape."""
    import torch
    from sfgb import api, synth
    stream = torch.cuda.Stream(device=dev)
    peak = measured_peak_gbs()[0]

    def timed(fn, reps):
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                fn()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b) / reps

    out = {}
    settings = {"dispersion_extended_k2": dict(kernel_x=2, kernel_y=2),
                "dispersion_extended_k3": dict(),
                "dispersion_extended_k4": dict(kernel_x=4, kernel_y=4),
                "dispersion_k3": dict(algorithm=1)}
    for name, (h, w) in {"batch_4m": (2162, 2068), "batch_9m": (3262, 3108)}.items():
        n = 64
        sw = synth.Sweep(synth.preset(name, n_frames=n))
        pool = torch.stack([torch.from_numpy(sw.frame(i).view(np.int32))
                            for i in range(n)]).to(dev)
        views = [pool[j] for j in range(n)]
        per = {}
        for key, kw in settings.items():
            params = api.Params(**kw)
            plan = api.Plan(h, w, n, capacity=h * w // 16, params=params)
            with torch.cuda.stream(stream):
                rr = plan.tune(views, stream=stream)
            ms = timed(lambda: plan(views, stream=stream), steps)
            sig = int(np.mean([len(plan.result(j)) for j in range(0, n, 8)]))
            single = api.DeviceThreshold(h, w, params=params, capacity=h * w // 16)

            def plain():
                for v in views:
                    single(v, stream=stream)
            ms1 = timed(plain, 2)
            algo = n * (h * w * 4 + (h * w + 7) // 8 + 16 * sig)
            per[key] = {"frames_per_s": n / (ms / 1e3), "us_per_frame": ms * 1e3 / n,
                        "achieved_gbs": algo / (ms / 1e3) / 1e9,
                        "frac_of_hbm": algo / (ms / 1e3) / 1e9 / peak,
                        "tuned_run_rows": rr,
                        "tuned_frames_per_launch": plan.frames_per_launch or n,
                        "plain_per_frame_frames_per_s": n / (ms1 / 1e3),
                        "batched_over_plain": ms1 / ms, "signal_pixels_per_frame": sig}
            plan.close()
            del single
        out[name] = per
        del pool, views

    # The dense-background stress frames (Poisson 20 plus rings, 20000 spots,
    # 2% overloads at 10^6 counts, 500 hot pixels): 16 frames in HBM through
    # a tuned plan, and their labelling on the device, 16 frames a call.
    from sfgb import labeller
    n = 16
    sw = synth.Sweep(synth.preset("dense_16m", n_frames=n))
    pool = torch.stack([torch.from_numpy(sw.frame(i).view(np.int32)) for i in range(n)]).to(dev)
    views = [pool[j] for j in range(n)]
    plan = api.Plan(H, W, n, capacity=H * W // 4)
    with torch.cuda.stream(stream):
        plan.tune(views, stream=stream)
    ms = timed(lambda: plan(views, stream=stream), steps)
    sig = int(np.mean([len(plan.result(j)) for j in range(0, n, 4)]))
    lab = labeller.DeviceLabeller(H, W, live_capacity=32 << 20)
    nb = [0]

    def label():
        nb[0] += 1
        lab.add_device(list(range(nb[0], nb[0] + n)), plan.lists_ptr, plan.capacity,
                       plan.counts_ptr, stream.cuda_stream)
        nb[0] += n
    ms_l = timed(label, steps)
    algo = n * (H * W * 4 + (H * W + 7) // 8 + 16 * sig)
    out["dense_16m"] = {"threshold_us_per_frame": ms * 1e3 / n,
                        "threshold_frac_of_hbm": algo / (ms / 1e3) / 1e9 / peak,
                        "labelling_us_per_frame": ms_l * 1e3 / n,
                        "frames_per_s": n / ((ms + ms_l) / 1e3),
                        "signal_pixels_per_frame": sig,
                        "spots": int(lab.finish().spots.size)}
    del lab, plan, pool, views

    # Mixed detector sizes in one launch sequence.
    shapes = [("eiger_16m", H, W), ("batch_9m", 3262, 3108), ("batch_4m", 2162, 2068),
              ("plain_1m", 1065, 1030)]
    frames = []
    for name, h, w in shapes:
        sw = synth.Sweep(synth.preset(name, height=h, width=w, n_frames=4))
        frames += [torch.from_numpy(sw.frame(i).view(np.int32)).to(dev) for i in range(4)]
    mixed = api.MixedBatch([tuple(f.shape) for f in frames], capacity=H * W // 16)
    ms_mixed = timed(lambda: mixed(frames, stream=stream), steps)
    groups = [api.DeviceBatch(h, w, 4, capacity=H * W // 16) for _, h, w in shapes]

    def by_shape():
        for k, g in enumerate(groups):
            g(frames[4 * k:4 * k + 4], stream=stream)
    ms_shapes = timed(by_shape, steps)
    px = sum(int(f.numel()) for f in frames)
    out["mixed_detectors"] = {
        "frames": len(frames), "one_launch_us": ms_mixed * 1e3,
        "frames_per_s": len(frames) / (ms_mixed / 1e3),
        "megapixels_per_s": px / (ms_mixed / 1e3) / 1e6,
        "per_shape_launches_us": ms_shapes * 1e3,
        "one_launch_over_per_shape": ms_shapes / ms_mixed,
        "path": "sf_threshold_u32_mixed_batch_device: 4 frames each of 4362x4148, 3262x3108, "
                "2162x2068 and 1065x1030 in one launch sequence, against "
                "sf_threshold_u32_batch_device once per shape"}
    return out


def run_config(frames_per_step: int, pool: int) -> dict:
    """The workload both arms report (the reference arm names the same)."""
    return {"workload": WORKLOAD, "frames_per_step": frames_per_step,
            "frame_pool": f"{pool} distinct frames resident in HBM "
                          f"({pool * H * W * 4 / 1e9:.2f} GB), cycled",
            "l2": "inputs larger than L2: each frame is 72.4 MB and consecutive frames differ",
            "stage": "threshold (all three dext stages + ordered emit) and 3-D labelling "
                     f"(grouping, filters, spot table), {frames_per_step} frames a step"}


def plan_run_rows(plan) -> int:
    from sfgb import api
    return int(api.lib().sf_plan_run_rows(plan._p))


def run_ours(args):
    import torch
    from sfgb import api
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    if not api.available():
        raise SystemExit("no usable GB300: " + api.unavailable_reason())

    B = args.frames_per_step
    pool_n = args.pool
    frames = make_pool(pool_n, seed_offset=rank)
    pool = torch.stack([torch.from_numpy(f.view(np.int32)) for f in frames]).to(dev)
    stream = torch.cuda.Stream(device=dev)
    views = [pool[j % pool_n] for j in range(B)]

    # The batched form: a plan tuned on these frames, its launch sequence
    # replayed as a CUDA graph (the same frame buffers every step).
    plan = api.Plan(H, W, B)
    with torch.cuda.stream(stream):
        # --no-tune keeps the default geometry (a short, fixed launch count
        # before the timed steps, for profiler captures).
        run_rows = 0 if args.no_tune else plan.tune(views, stream=stream)
        for w in range(args.warmup):
            plan(views, stream=stream)
    stream.synchronize()
    counts = np.array([len(plan.result(j)) for j in range(B)])
    n_signal = int(counts.mean())

    # The timed step: the batch's threshold (the plan's graph) and the 3-D
    # labelling of its lists on the device (sf_label_add_device: its launch
    # sequence replayed as a graph, the call's status read back), so a step
    # covers the path the reference's CPU arm times. Frame numbers are
    # consecutive within a step, with a gap between steps (the same frames
    # come round again) that closes the spots there.
    from sfgb import labeller
    lab = labeller.DeviceLabeller(H, W, live_capacity=(B + 16) * 200_000)
    nb = [0]

    def step():
        plan(views, stream=stream)
        ev_mid = torch.cuda.Event(enable_timing=True)
        ev_mid.record(stream)
        nb[0] += 1
        lab.add_device(list(range(nb[0], nb[0] + B)), plan.lists_ptr, plan.capacity,
                       plan.counts_ptr, stream.cuda_stream)
        nb[0] += B
        return ev_mid

    with torch.cuda.stream(stream):
        for w in range(args.warmup):
            step()
    stream.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    mids = []
    clocks = ClockSampler(local, args.clocks_csv)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        start.record(stream)
        for s in range(args.steps):
            ev[s][0].record(stream)
            mids.append(step())
            ev[s][1].record(stream)
        end.record(stream)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    clock = clocks.stop()
    elapsed_ms = start.elapsed_time(end)
    elapsed_ms = max_over_ranks(elapsed_ms, world, dev)
    frames_done = sum_over_ranks(args.steps * B, world, dev)
    value = frames_done / (elapsed_ms / 1e3)
    # The threshold's share of each step (the plan's graph, CUDA events on
    # its stream) sets the roofline; the labelling's the rest.
    launch_ms = statistics.mean(a.elapsed_time(m) for (a, _), m in zip(ev, mids))
    label_ms = statistics.mean(m.elapsed_time(b) for (_, b), m in zip(ev, mids))

    # The same batches pipelined as a detector stream would run them: batch
    # s + 1's threshold is queued before batch s is labelled on a second,
    # higher-priority stream, so the two overlap on the device (two plans of
    # the same tuning hold alternate batches' lists). Reported beside the
    # step: the overlap slows each threshold launch, so the roofline stays
    # with the timed step above.
    plans = [plan, api.Plan(H, W, B)]
    plans[1].configure(plan_run_rows(plan), plan.frames_per_launch)
    lstream = torch.cuda.Stream(device=dev, priority=-1)

    def pipelined(n):
        def threshold(k):
            plans[k % 2](views, stream=stream)
            t = torch.cuda.Event()
            t.record(stream)
            return t

        pending = threshold(0)
        for k in range(n):
            done = pending
            if k + 1 < n:
                pending = threshold(k + 1)
            lstream.wait_event(done)
            nb[0] += 1
            pk = plans[k % 2]
            lab.add_device(list(range(nb[0], nb[0] + B)), pk.lists_ptr, pk.capacity,
                           pk.counts_ptr, lstream.cuda_stream)
            nb[0] += B

    with torch.cuda.stream(stream):
        pipelined(args.warmup)
        torch.cuda.synchronize(dev)
        pa, pb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pa.record(stream)
        pipelined(args.steps)
        lstream.wait_stream(stream)
        pb.record(lstream)
    torch.cuda.synchronize(dev)
    pipelined_fps = args.steps * B / (pa.elapsed_time(pb) / 1e3)
    plans[1].close()
    label_res = lab.finish()
    del lab
    graphs = plan.graphs

    # Roofline of the threshold launch sequence: algorithmic bytes per frame
    # (the frame read once, the bitmask written, the signal list written).
    algo_bytes = B * (H * W * 4 + (H * W + 7) // 8 + 16 * n_signal)
    peak, peak_kind = measured_peak_gbs()
    achieved = algo_bytes / (launch_ms / 1e3) / 1e9

    # The threshold alone, the same plan and frames (the figure before the
    # labelling joined the step).
    with torch.cuda.stream(stream):
        ta, tb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ta.record(stream)
        for _ in range(args.steps):
            plan(views, stream=stream)
        tb.record(stream)
    torch.cuda.synchronize(dev)
    threshold_only = args.steps * B / (ta.elapsed_time(tb) / 1e3)

    # The plain per-frame device path (one launch sequence per frame).
    single = api.DeviceThreshold(H, W)
    with torch.cuda.stream(stream):
        for j in range(4):
            single(pool[j % pool_n], stream=stream)
        stream.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n_single = max(B, 16)
        a.record(stream)
        for j in range(n_single):
            single(pool[j % pool_n], stream=stream)
        b.record(stream)
    torch.cuda.synchronize(dev)
    per_frame = n_single / (a.elapsed_time(b) / 1e3)
    del single

    # The same frames as 16-bit pixels (the reference's published GPU numbers
    # are all for 16-bit frames): device-resident batches of B through the
    # batched threshold, CUDA events around each batch.
    u16_line = None
    if not args.no_u16:
        def as_u16(f):
            g = np.minimum(f, 0xFFFD).astype(np.uint16)
            g[f == 0xFFFFFFFE] = 0xFFFE
            g[f == 0xFFFFFFFF] = 0xFFFF
            return g
        pool16 = torch.stack([torch.from_numpy(as_u16(f).view(np.int16)) for f in frames]).to(dev)
        views16 = [pool16[j % pool_n] for j in range(B)]
        batch16 = api.DeviceBatch(H, W, B)
        with torch.cuda.stream(stream):
            for _ in range(max(args.warmup, 3)):
                batch16(views16, stream=stream)
            e16 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(args.steps)]
            for a16, b16 in e16:
                a16.record(stream)
                batch16(views16, stream=stream)
                b16.record(stream)
        torch.cuda.synchronize(dev)
        ms16 = statistics.mean(a.elapsed_time(b) for a, b in e16)
        n16 = int(batch16.counts[0].item())
        bytes16 = B * (H * W * 2 + (H * W + 7) // 8 + 16 * n16)
        u16_line = {
            "frames_per_s": B / (ms16 / 1e3), "us_per_frame": ms16 * 1e3 / B,
            "achieved_gbs": bytes16 / (ms16 / 1e3) / 1e9,
            "frac_of_hbm": bytes16 / (ms16 / 1e3) / 1e9 / measured_peak_gbs()[0],
            "signal_pixels_frame0": n16,
            "path": f"sf_threshold_u16_batch_device, {B} frames a launch, the same frames as "
                    "16-bit pixels (valid values clamped below the masked sentinels)",
            "reference_published": "16M u16 frame kernel time 8.9 ms (CUDA, RTX 4060) and "
                                   "3.9 ms (Metal, M4 Max; unavailable on this box), "
                                   "docs/outstanding.md:130-131",
        }
        del batch16, pool16, views16

    label = {"ms_per_frame": label_ms / B, "frames_per_s": B / (label_ms / 1e3),
             "spots": int(len(label_res.spots)),
             "path": f"sf_label_add_device on the plan's lists, {B} frames per call (its "
                     "launch sequence replayed as a CUDA graph, the call's status read "
                     "back), inside each timed step after the threshold; CUDA events"}

    # The host link's own speed: pinned frames copied to the device.
    h2d_gbs = None
    if not args.no_e2e:
        hbuf = torch.empty((4, H * W), dtype=torch.int32).pin_memory()
        dbuf = torch.empty((4, H * W), dtype=torch.int32, device=dev)
        streams = [torch.cuda.Stream(device=dev) for _ in range(2)]
        for _ in range(2):
            for k in range(4):
                with torch.cuda.stream(streams[k % 2]):
                    dbuf[k].copy_(hbuf[k], non_blocking=True)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        reps = 8
        for _ in range(reps):
            for k in range(4):
                with torch.cuda.stream(streams[k % 2]):
                    dbuf[k].copy_(hbuf[k], non_blocking=True)
        torch.cuda.synchronize(dev)
        h2d_gbs = reps * 4 * H * W * 4 / (time.perf_counter() - t0) / 1e9
        del hbuf, dbuf

    # End to end through the C ABI host-frame call (gpu::find drop-in), from
    # several host threads as mxi_find's -j workers call it.
    e2e_thr = None
    if not args.no_e2e:
        import ctypes
        from concurrent.futures import ThreadPoolExecutor
        L = api.lib()
        host = []
        for f in frames[: min(pool_n, 8)]:
            ptr = L.sf_host_alloc(f.nbytes)
            if not ptr:
                raise SystemExit("sf_host_alloc failed")
            arr = np.ctypeslib.as_array((ctypes.c_uint32 * f.size).from_address(ptr))
            arr[:] = f.ravel()
            host.append(ptr)
        T = args.e2e_threads or os.cpu_count() or 8
        outs = []
        for _ in range(T):
            ptr = L.sf_host_alloc(H * W // 4 * 16)
            if not ptr:
                raise SystemExit("sf_host_alloc failed")
            outs.append(ptr)
        tls = threading.local()
        slot_lock = threading.Lock()
        slots = list(range(T))

        def e2e_frame(k):
            if not hasattr(tls, "slot"):
                with slot_lock:
                    tls.slot = slots.pop()
            found = ctypes.c_size_t(0)
            rc = L.sf_find_u32(host[k % len(host)], H, W, outs[tls.slot], H * W // 4,
                               ctypes.byref(found))
            if rc != 0:
                raise SystemExit(f"sf_find_u32 failed: {rc} {api.last_error()}")
            # The drop-in's last step (shim/dext_sfgb.cc): the records found
            # copied out of the thread's pinned staging into the caller's
            # own vector, sized to the count.
            n = found.value
            signal = np.empty(n * 16, np.uint8)
            if n:
                ctypes.memmove(signal.ctypes.data, outs[tls.slot], n * 16)
            return n

        with ThreadPoolExecutor(max_workers=T) as ex:
            list(ex.map(e2e_frame, range(max(args.warmup, 1) * max(B, T))))
            if world > 1:
                torch.distributed.barrier()
            t0 = time.perf_counter()
            n_e2e = args.steps * B
            d2h = sum(4 + 16 * n for n in ex.map(e2e_frame, range(n_e2e)))
            t1 = time.perf_counter()
        e_ms = max_over_ranks((t1 - t0) * 1e3, world, dev)
        e2e_thr = {"value": sum_over_ranks(n_e2e, world, dev) / (e_ms / 1e3),
               "unit": "frames/s", "h2d_bytes_per_step": B * H * W * 4,
               "d2h_bytes_per_step": int(d2h / args.steps),
               "path": f"sf_find_u32 (C ABI) from {T} host threads in the call sequence of "
                       "the gpu::find<uint32_t> drop-in (shim/dext_sfgb.cc): pinned host "
                       "frames; per frame the copy in, the threshold, the list's read-back "
                       "into the thread's pinned staging and its copy into a list sized to "
                       "the count",
               "h2d_peak_gbs": h2d_gbs,
               "achieved_h2d_gbs": None,
               "frac_of_h2d_peak": None}
        e2e_thr["achieved_h2d_gbs"] = e2e_thr["value"] * H * W * 4 / 1e9
        if h2d_gbs:
            e2e_thr["frac_of_h2d_peak"] = e2e_thr["achieved_h2d_gbs"] / h2d_gbs
        if not args.no_u16:
            # The same frames as 16-bit pixels through sf_find_u16 (the
            # gpu::find<uint16_t> drop-in): half the bytes over the host link.
            host16 = []
            for f in frames[: min(pool_n, 8)]:
                g = np.minimum(f, 0xFFFD).astype(np.uint16)
                g[f == 0xFFFFFFFE] = 0xFFFE
                g[f == 0xFFFFFFFF] = 0xFFFF
                ptr = L.sf_host_alloc(g.nbytes)
                if not ptr:
                    raise SystemExit("sf_host_alloc failed")
                np.ctypeslib.as_array((ctypes.c_uint16 * g.size).from_address(ptr))[:] = g.ravel()
                host16.append(ptr)
            slots.extend(range(T))
            tls16 = threading.local()

            def e2e_frame16(k):
                if not hasattr(tls16, "slot"):
                    with slot_lock:
                        tls16.slot = slots.pop()
                found = ctypes.c_size_t(0)
                rc = L.sf_find_u16(host16[k % len(host16)], H, W, outs[tls16.slot],
                                   H * W // 4, ctypes.byref(found))
                if rc != 0:
                    raise SystemExit(f"sf_find_u16 failed: {rc} {api.last_error()}")
                return found.value

            with ThreadPoolExecutor(max_workers=T) as ex:
                list(ex.map(e2e_frame16, range(max(args.warmup, 1) * max(B, T))))
                t0 = time.perf_counter()
                list(ex.map(e2e_frame16, range(args.steps * B)))
                t1 = time.perf_counter()
            v16 = args.steps * B / (t1 - t0)
            e2e_thr["u16"] = {"value": v16, "unit": "frames/s",
                          "h2d_bytes_per_step": B * H * W * 2,
                          "achieved_h2d_gbs": v16 * H * W * 2 / 1e9,
                          "path": f"sf_find_u16 from {T} host threads, the same frames as "
                                  "16-bit pixels in pinned host memory"}
            for ptr in host16:
                L.sf_host_free(ptr)
        if not args.no_bslz4:
            # The same frames as bitshuffle+LZ4 chunks (how an EIGER's HDF5
            # stores them) through sf_find_compressed: only the chunk crosses
            # the host link, decoded and thresholded on the device
            # (find_spots.cc:772-800 with decompress::image on the device).
            from sfgb import synth
            for depth in (32, 16):
                chunks = []
                for f in frames[: min(pool_n, 8)]:
                    if depth == 16:
                        g = np.minimum(f, 0xFFFD).astype(np.uint16)
                        g[f == 0xFFFFFFFE] = 0xFFFE
                        g[f == 0xFFFFFFFF] = 0xFFFF
                        f = g
                    c = synth.chunk(f, "bslz4")
                    ptr = L.sf_host_alloc(c.size)
                    if not ptr:
                        raise SystemExit("sf_host_alloc failed")
                    np.ctypeslib.as_array((ctypes.c_uint8 * c.size).from_address(ptr))[:] = c
                    chunks.append((ptr, c.size))
                slots.extend(range(T))
                tlsc = threading.local()

                def e2e_chunk(k, depth=depth, chunks=chunks, tlsc=tlsc):
                    if not hasattr(tlsc, "slot"):
                        with slot_lock:
                            tlsc.slot = slots.pop()
                    found = ctypes.c_size_t(0)
                    ptr, n = chunks[k % len(chunks)]
                    rc = L.sf_find_compressed(ptr, n, b"bslz4", depth, H, W, None,
                                              outs[tlsc.slot], H * W // 4, ctypes.byref(found))
                    if rc != 0:
                        raise SystemExit(f"sf_find_compressed failed: {rc} {api.last_error()}")
                    return n

                with ThreadPoolExecutor(max_workers=T) as ex:
                    list(ex.map(e2e_chunk, range(max(args.warmup, 1) * max(B, T))))
                    t0 = time.perf_counter()
                    nbytes = sum(ex.map(e2e_chunk, range(args.steps * B)))
                    t1 = time.perf_counter()
                vc = args.steps * B / (t1 - t0)
                e2e_thr[f"bslz4_u{depth}"] = {
                    "value": vc, "unit": "frames/s",
                    "h2d_bytes_per_step": int(nbytes / args.steps),
                    "compression": args.steps * B * H * W * depth / 8 / nbytes,
                    "achieved_h2d_gbs": nbytes / (t1 - t0) / 1e9,
                    "path": f"sf_find_compressed from {T} host threads: the same frames as "
                            f"{depth}-bit bitshuffle+LZ4 chunks (8192-byte blocks) in pinned "
                            "host memory, decoded and thresholded on the device"}
                for ptr, _ in chunks:
                    L.sf_host_free(ptr)
        for ptr in host + outs:
            L.sf_host_free(ptr)

    # End to end through the served API (the whole path: host frames in,
    # threshold, 3-D labelling, the spot tables read back), fed at full rate.
    e2e = None
    if not args.no_e2e:
        e2e = served_e2e(args.steps * B, B, h2d_gbs)
        e2e["threshold_only"] = e2e_thr
        if not args.no_bslz4:
            e2e["bslz4_u32"] = served_e2e(args.steps * B, B, h2d_gbs, chunks=True)

    batched = None
    if rank == 0 and not args.no_batched:
        batched = batched_legs(dev)

    served_line = None
    if rank == 0 and not args.no_served:
        del plan
        torch.cuda.empty_cache()
        served_line = served(args.served_seconds)
        # The same six sweeps all at the top of the 100-750 Hz range.
        keep = ("p50_ms", "p99_ms", "frames", "frames_per_s", "offered_frames_per_s", "errors",
                "host_link_gbs_offered", "failed_sweeps")
        served_line["at_max_rate"] = {
            k: v for k, v in served(args.served_seconds, rates=[750.0] * 6).items() if k in keep}
        if not args.no_bslz4:
            # The same, and at 1.5 times the rate (beyond what raw frames can
            # cross the host link at), with the frames as chunks.
            for tag, hz in (("bslz4_at_max_rate", 750.0), ("bslz4_at_1.5x_max_rate", 1125.0)):
                served_line[tag] = {
                    k: v for k, v in served(args.served_seconds, rates=[hz] * 6,
                                            chunks=True).items() if k in keep}
        # The dense-background stress: eight 16M sweeps of Poisson 20 plus
        # rings, 20000 spots and 2% overloads a frame, at 50 Hz each. A dense
        # frame has about 800,000 signal pixels and several million candidates
        # of the erosion bound: lists of one record per 4 pixels, and
        # labellers that hold a whole call of such frames.
        dense = served(args.served_seconds, rates=[50.0] * 8, kinds=["16M-dense"] * 8,
                       label_capacity=32 << 20, capacity_divisor=4)
        served_line["dense_16m"] = {k: v for k, v in dense.items()
                                    if k in keep + ("spots", "workload")}

    base = None
    if rank == 0 and not args.no_cpu_baseline:
        base = cpu_baseline(frames[:4], seconds_budget=args.cpu_seconds)

    if world > 1:
        torch.distributed.barrier()
    if rank == 0:
        if args.traffic is not None:
            traffic, traffic_source = args.traffic, "given on the command line"
        else:
            traffic = DRAM_BYTES_PER_FRAME * B
            traffic_source = (
                "ncu dram__bytes_read.sum + dram__bytes_write.sum of one timed 32-frame launch "
                "of this workload (32 frames in HBM), one capture a kernel for its 8 kernels, no "
                "cache flush between kernels "
                f"({DRAM_BYTES_PER_FRAME / 1e6:.1f} MB a frame), times the {B} frames of a launch; "
                "a frame's traffic grows a little with the batch")
        line = {
            "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": run_config(B, pool_n),
            "details": {"signal_pixels_per_frame": n_signal,
                       "threshold_only_frames_per_s": threshold_only,
                       "pipelined_frames_per_s": pipelined_fps,
                       "plain_per_frame_frames_per_s": per_frame,
                       "batched_over_plain": threshold_only / per_frame,
                       "threshold_ms_per_step": launch_ms,
                       "labelling_ms_per_step": label_ms,
                       "tuned_run_rows": run_rows, "cuda_graphs": graphs},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_kind,
                         "kernel": "threshold launch sequence of a batch (lat_stage01, "
                                   "lat_tiles, lat_verify, mask_sums, mask_prefix, lat_stage2, "
                                   "pass_sums, pass_scatter) replayed as one CUDA graph, "
                                   "CUDA events around each batch",
                         "algorithmic_bytes_per_launch": algo_bytes,
                         "launch_ms": launch_ms, "traffic": traffic,
                         "traffic_source": traffic_source},
            "cpu_baseline": base, "e2e": e2e, "labelling": label, "u16": u16_line,
            "served": served_line,
            "batched": batched,
            "clocks": clock,
            "gpu_launches": (THRESHOLD_KERNELS + LABEL_KERNELS) * args.steps,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--frames-per-step", type=int, default=64)
    ap.add_argument("--pool", type=int, default=64)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-threads", type=int, default=0,
                    help="host threads of the end-to-end legs (0: one a core, as mxi_find -j)")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the plan's default geometry (no tuning launches)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 4M/9M tuned-plan and mixed-detector legs")
    ap.add_argument("--no-u16", action="store_true")
    ap.add_argument("--no-bslz4", action="store_true")
    ap.add_argument("--clocks-csv", default=None,
                    help="also write the nvidia-smi samples of the timed region here")
    ap.add_argument("--served-seconds", type=float, default=4.0)
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per threshold launch from an ncu capture")
    args = ap.parse_args(argv)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
