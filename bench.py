#!/usr/bin/env python3
"""Benchmark of the GB300 S2TC encoder (one JSON line on rank 0).

Default workload: one 4096x4096 RGBA8 image -> DXT5 with SRGB_MIXED distance,
the all-16 endpoint search (RANDOM_COLORS=0) and LOOP refinement, SIMPLE
dither.  A step is one compression of one image.

* ``value``: texels/s with the inputs resident in HBM (s2tc_gpu_compress on
  device buffers), timed with CUDA events on the launching stream over K
  back-to-back steps.  The inputs rotate over four distinct 64 MB images
  (256 MB > the 129 MB L2), so every step reads its input cold.
* ``e2e``: the same metric through the reference-compatible C entry point
  tx_compress_dxtn with pinned host buffers (upload, kernels, download, sync).
* ``roofline``: the dominant kernel's algorithmic bytes per launch over its
  average launch time (library-recorded CUDA events on the launching stream)
  against the measured HBM copy bandwidth.
* ``cpu_baseline``: the CPU port of the reference encoder (oracle/) on one
  core, on the first workload image; its bytes are also compared with the GPU
  output (``bit_exact``).

``--impl reference`` times the reference's CPU implementation instead (the
reference library compiled from its sources when present, else the CPU port),
one worker process per host core, each compressing a band of the workload.

Multi-GPU (torchrun): every rank compresses its own images (replicas, no
collective on the data path); value = all ranks' texels / the slowest rank's
time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "texels/s"
NIMG = 4

WORKLOADS = {
    "value_noise_4096_dxt5_srgb_mixed_all16_loop": dict(
        w=4096, h=4096, sc=4, fmt=0x83F3, dither=1, metric=3, nrandom=0, refine=2, gen="value_noise", seed=2),
    # the same texture with Floyd-Steinberg dither: a two-dimensional
    # wavefront, latency-bound rather than bandwidth-bound
    "value_noise_4096_dxt5_srgb_mixed_all16_loop_fs": dict(
        w=4096, h=4096, sc=4, fmt=0x83F3, dither=2, metric=3, nrandom=0, refine=2, gen="value_noise", seed=2),
    "plain_1024_dxt1_wavg_quick_always": dict(
        w=1024, h=1024, sc=4, fmt=0x83F1, dither=1, metric=5, nrandom=-1, refine=1, gen="plain", seed=1),
    "plain_4096_dxt1_wavg_quick_always": dict(
        w=4096, h=4096, sc=4, fmt=0x83F1, dither=1, metric=5, nrandom=-1, refine=1, gen="plain", seed=1),
    "plain_8192_dxt1_wavg_quick_always": dict(
        w=8192, h=8192, sc=4, fmt=0x83F1, dither=1, metric=5, nrandom=-1, refine=1, gen="plain", seed=1),
    "normal_map_2048_dxt1_normalmap_rand64_loop": dict(
        w=2048, h=2048, sc=3, fmt=0x83F1, dither=1, metric=7, nrandom=64, refine=2, gen="normal", seed=4),
    # 256 textures (log-uniform 4..2048, aspect <= 4:1) with full mip chains,
    # mixed DXT1/DXT3/DXT5, RGB8/RGBA8: one batched graph launch per step
    "mip_chains_256_wavg_rand64_always": dict(
        w=0, h=0, sc=0, fmt=0, dither=1, metric=5, nrandom=64, refine=1, gen="mips", seed=3, count=256),
    # the first 64 of those textures (a size that ncu captures whole)
    "mip_chains_64_wavg_rand64_always": dict(
        w=0, h=0, sc=0, fmt=0, dither=1, metric=5, nrandom=64, refine=1, gen="mips", seed=3, count=64),
    # 64 RGB8 normal maps of 2048x2048 (16 distinct maps, each used four
    # times) in one batched graph launch
    "normal_maps_64x2048_dxt1_normalmap_rand64_loop": dict(
        w=2048, h=2048, sc=3, fmt=0x83F1, dither=1, metric=7, nrandom=64, refine=2, gen="normal_batch", seed=4,
        count=64, distinct=16),
    # the reference's tools on the GPU: whole-image decode (s2tc_decompress),
    # S3TC -> S2TC block rewrite (s2tc_from_s3tc), mip chain + DDS
    # (s2tc_compress); HBM-bound except the DDS pipeline's encoder
    "decode_8192_dxt5": dict(w=8192, h=8192, sc=4, fmt=0x83F3, gen="tool", tool="decode", seed=6),
    "from_s3tc_8192_dxt5": dict(w=8192, h=8192, sc=4, fmt=0x83F3, gen="tool", tool="from_s3tc", seed=7),
    "dds_4096_dxt1_wavg_quick_always": dict(w=4096, h=4096, sc=4, fmt=0x83F1, dither=1, metric=5, nrandom=-1, refine=1,
                                            gen="tool", tool="dds", seed=1),
    # latency of one synchronous tx_compress_dxtn call on small images with the
    # default knobs (pageable buffers, as a GL driver passes them)
    "small_calls_dxt1_wavg_quick_always": dict(
        w=0, h=0, sc=4, fmt=0x83F1, dither=1, metric=5, nrandom=-1, refine=1, gen="small", seed=3,
        sizes=[64, 128, 256, 512, 1024]),
    # requests of log-uniform size 64..4096, DXT1/DXT5, WAVG/SRGB_MIXED/NORMALMAP,
    # through the continuous-batching request loop under a 32 GB budget; a
    # step is 1000 requests
    "serving_requests_64_4096_budget32g": dict(
        w=0, h=0, sc=4, fmt=0, dither=1, metric=-1, nrandom=-1, refine=1, gen="serving", seed=5,
        budget=32 << 30, per_step=1000),
}
DEFAULT_WORKLOAD = "value_noise_4096_dxt5_srgb_mixed_all16_loop"
FMT_NAMES = {0x83F0: "DXT1(RGB)", 0x83F1: "DXT1", 0x83F2: "DXT3", 0x83F3: "DXT5"}


def make_image(wl: dict, seed: int, rows: int | None = None) -> np.ndarray:
    """Workload image (flattened); with `rows`, an image of the same recipe
    and width but only that many rows."""
    from s2tc_gb300 import workloads
    w, h = wl["w"], wl["h"] if rows is None else rows
    if wl["gen"] == "value_noise":
        img = workloads.value_noise_rgba(seed, w, h)
    elif wl["gen"] == "plain":
        img = workloads.plain_rgba(seed, w, h)
    else:
        img = workloads.normal_map(seed, w, h)
    return np.ascontiguousarray(img.reshape(-1))


def algorithmic_bytes_per_texel(wl: dict) -> float:
    """Input read once + output written once (the 5:6:5 intermediate is not
    counted: a fused encoder would not materialise it)."""
    return wl["sc"] + (8 if wl["fmt"] in (0x83F0, 0x83F1) else 16) / 16.0


def roofline_note(dominant: str, wl: dict) -> str:
    """What bounds the dominant kernel of an image workload (from its ncu
    captures), beside the HBM fraction that the line reports."""
    tail = ""
    if dominant == "dither":
        if wl["dither"] == 2:
            return ("the Floyd-Steinberg wavefront is latency-bound (a chain of width + 2 * height "
                    "dependent steps)" + tail)
        return ("the exact SIMPLE dither is integer-ALU bound (its per-segment state tables and "
                "replay cost about 100 integer operations per texel)" + tail)
    if wl["nrandom"] < 0:
        return "the quick-mode encoder's per-block arithmetic is integer-ALU bound" + tail
    if wl["nrandom"] > 0:
        return "the random-candidate pair search is integer-ALU bound" + tail
    return "the all-pairs search is integer-ALU bound" + tail


def issue_roofline(wl_name: str, stage: str, stage_ms: float, texels: int, sm_mhz: float, sms: int) -> dict | None:
    """The integer-issue roofline of one stage of a workload: warp
    instructions that the stage's kernels issue per texel (from one ncu
    capture of the same workload, profiles/inst_counts.json) times the texels
    of a launch, over the stage's live CUDA-event time, against one warp
    instruction per scheduler per cycle (4 per SM) at the sampled SM clock;
    and the integer-ALU pipe's share against its own peak rate."""
    # batches of the same recipe use the per-texel counts of the captured one
    alias = {"mip_chains_256_wavg_rand64_always": "mip_chains_64_wavg_rand64_always",
             "normal_maps_64x2048_dxt1_normalmap_rand64_loop": "normal_map_2048_dxt1_normalmap_rand64_loop"}
    src = alias.get(wl_name, wl_name)
    try:
        counts = json.loads((ROOT / "profiles" / "inst_counts.json").read_text())[src]
        if stage == "batch" and "batch" not in counts:
            # a batch of whole images: the per-texel sum of the dither and encoder stages
            d = {k: counts["dither"][k] + counts["encode"][k]
                 for k in ("warp_inst_per_texel", "alu_inst_per_texel")}
            d["alu_peak_per_sm_cycle"] = counts["encode"]["alu_peak_per_sm_cycle"]
        else:
            d = counts[stage]
    except Exception:
        return None
    t = stage_ms / 1000.0
    hz = sm_mhz * 1e6
    inst = d["warp_inst_per_texel"] * texels
    alu = d["alu_inst_per_texel"] * texels
    issue_peak = sms * 4 * hz
    alu_peak = sms * d["alu_peak_per_sm_cycle"] * hz
    return {"bound": "alu", "kernel": stage, "achieved": inst / t / 1e9, "peak": issue_peak / 1e9,
            "unit": "G warp-instructions/s", "frac": inst / t / issue_peak,
            "alu_pipe_frac": alu / t / alu_peak, "warp_inst_per_launch": inst,
            "peak_source": f"{sms} SMs x 4 schedulers x 1 instruction/cycle at the sampled {sm_mhz:.0f} MHz",
            "counts_source": f"profiles/inst_counts.json, {src} (ncu smsp__inst_executed.sum, "
                             "sm__inst_executed_pipe_alu.sum per texel)"}


def config_dict(wl_name: str, wl: dict) -> dict:
    import s2tc_gb300 as s2
    if wl["gen"] == "tool":
        d = {"workload": wl_name, "width": wl["w"], "height": wl["h"], "format": FMT_NAMES[wl["fmt"]],
             "tool": {"decode": "s2tc_decompress (s2tc_gpu_decode)", "from_s3tc": "s2tc_from_s3tc (s2tc_gpu_from_s3tc)",
                      "dds": "s2tc_compress (s2tc_compress_dds, every mip level)"}[wl["tool"]],
             "l2": "inputs and outputs larger than the 129 MB L2"}
        if wl["tool"] == "dds":
            d.update(dither=s2.DITHER_NAMES[wl["dither"]], colordist=s2.COLORDIST_NAMES[wl["metric"]],
                     random_colors=wl["nrandom"], refine=s2.REFINE_NAMES[wl["refine"]],
                     l2="one 64 MB image and its levels; timed end to end per call")
        return d
    if wl["gen"] == "normal_batch":
        return {"workload": wl_name, "maps": wl["count"], "distinct_maps": wl["distinct"], "width": wl["w"],
                "height": wl["h"], "srccomps": 3, "format": "DXT1", "dither": s2.DITHER_NAMES[wl["dither"]],
                "colordist": "NORMALMAP", "random_colors": wl["nrandom"], "refine": s2.REFINE_NAMES[wl["refine"]],
                "l2": "the batch's inputs (805 MB) and rand words (13 GB) exceed the 129 MB L2"}
    if wl["gen"] == "small":
        return {"workload": wl_name, "sizes": [f"{n}x{n}" for n in wl["sizes"]], "srccomps": 4, "format": "DXT1",
                "dither": "SIMPLE", "colordist": "WAVG", "random_colors": -1, "refine": "ALWAYS",
                "entry": "tx_compress_dxtn, pageable host buffers", "l2": "small images: L2-resident by design"}
    if wl["gen"] == "serving":
        return {"workload": wl_name, "requests_per_step": wl["per_step"], "sizes": "log-uniform 64..4096 per side",
                "formats": "DXT1/DXT5 uniform", "colordist": "WAVG/SRGB_MIXED/NORMALMAP uniform",
                "dither": "SIMPLE", "random_colors": -1, "refine": "ALWAYS", "budget_bytes": wl["budget"],
                "pixels": "per-request windows of one pre-generated 4096x8192 plain (noise + gradient) image at "
                          "seeded offsets",
                "l2": "the requests' inputs (GBs per step) exceed the 129 MB L2"}
    if wl["gen"] == "mips":
        return {"workload": wl_name, "textures": wl["count"], "base_sizes": "log-uniform 4..2048, aspect <= 4:1",
                "levels": "full mip chains to 1x1", "formats": "DXT1/DXT3/DXT5 by thirds",
                "srccomps": "3 and 4 alternating", "dither": s2.DITHER_NAMES[wl["dither"]],
                "colordist": s2.COLORDIST_NAMES[wl["metric"]], "random_colors": wl["nrandom"],
                "refine": s2.REFINE_NAMES[wl["refine"]],
                "l2": "the batch's inputs (over 100 MB) and rand words (GBs) exceed the 129 MB L2"}
    return {"workload": wl_name, "width": wl["w"], "height": wl["h"], "srccomps": wl["sc"],
            "format": FMT_NAMES[wl["fmt"]], "dither": s2.DITHER_NAMES[wl["dither"]],
            "colordist": s2.COLORDIST_NAMES[wl["metric"]], "random_colors": wl["nrandom"],
            "refine": s2.REFINE_NAMES[wl["refine"]],
            "l2": f"inputs rotate over {NIMG} resident images larger in total than the 129 MB L2"}


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """Samples SM clock and clock-event reasons through NVML (read only)
    while running."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, cuda_index: int = 0):
        self.samples: list[int] = []
        self.reasons = 0
        self.max_mhz = None
        self._stop = threading.Event()
        self._nvml = None
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                return
            handle = ctypes.c_void_p()
            ok = False
            try:
                import torch
                p = torch.cuda.get_device_properties(cuda_index)
                bus = f"{p.pci_domain_id:08X}:{p.pci_bus_id:02X}:{p.pci_device_id:02X}.0".encode()
                ok = nv.nvmlDeviceGetHandleByPciBusId_v2(ctypes.c_char_p(bus), ctypes.byref(handle)) == 0
            except Exception:
                ok = False
            if not ok and nv.nvmlDeviceGetHandleByIndex_v2(cuda_index, ctypes.byref(handle)) != 0:
                return
            mx = ctypes.c_uint()
            if nv.nvmlDeviceGetMaxClockInfo(handle, 1, ctypes.byref(mx)) == 0:
                self.max_mhz = mx.value
            try:
                self._reasons_fn = nv.nvmlDeviceGetCurrentClocksEventReasons
            except AttributeError:
                self._reasons_fn = nv.nvmlDeviceGetCurrentClocksThrottleReasons
            self._nvml, self._h = nv, handle
        except OSError:
            self._nvml = None

    def _run(self):
        nv, h = self._nvml, self._h
        mhz, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self._stop.is_set():
            if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(mhz)) == 0:
                self.samples.append(mhz.value)
            if self._reasons_fn(h, ctypes.byref(rs)) == 0:
                self.reasons |= rs.value
            time.sleep(0.002)

    def __enter__(self):
        if self._nvml is not None:
            self._t = threading.Thread(target=self._run, daemon=True)
            self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._nvml is not None:
            self._t.join()

    def summary(self) -> dict:
        if self._nvml is None or not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": [], "samples": 0,
                    "note": "NVML unavailable" if self._nvml is None else "no samples"}
        return {"sm_mhz": statistics.median(self.samples), "sm_max_mhz": self.max_mhz,
                "reasons": [n for b, n in self.REASONS.items() if self.reasons & b],
                "samples": len(self.samples)}


# --------------------------------------------------------------- CPU legs

_WORKER_IMAGES: dict = {}


def _cpu_worker(args):
    """One CPU compression of a workload band (runs in a spawned process);
    returns (seconds, output).  The image is made once per process."""
    wl_name, rows, use_ref, seed = args
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    wl = WORKLOADS[wl_name]
    key = (wl_name, rows)
    if key not in _WORKER_IMAGES:
        _WORKER_IMAGES[key] = make_image(wl, wl["seed"], None if rows == wl["h"] else rows)
    img = _WORKER_IMAGES[key]
    enc = pyoracle.Reference() if use_ref else pyoracle.Oracle()
    t0 = time.perf_counter()
    out = enc.compress(wl["sc"], wl["w"], rows, img, wl["fmt"], wl["dither"], wl["metric"], wl["nrandom"],
                       wl["refine"], seed=seed)
    return time.perf_counter() - t0, out, os.getpid()


def _oracle_worker(job):
    """The oracle's bytes for one image (runs in a spawned process); returns
    their CRC-32.  `words`: the random candidates' words, or None."""
    import zlib
    sc, w, h, px, fmt, dither, metric, nrandom, refine, words = job
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    out = pyoracle.Oracle().compress(sc, w, h, px, fmt, dither, metric, nrandom, refine, rand_words=words)
    return zlib.crc32(out.tobytes())


def oracle_crcs(jobs: list) -> list:
    """CRC-32 of the oracle's output for each job, one spawned process per
    job (up to the host's cores)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(max(1, min(len(jobs), os.cpu_count() or 1))) as pool:
        return pool.map(_oracle_worker, jobs, chunksize=1)


def sample_levels(shapes: list, budget: int = 6_000_000, want: int = 8) -> list:
    """Indices of a sample of images for the oracle check: the largest one,
    a 1x1, a 2x2 and a 3xN level where present, a level whose sides are not
    multiples of 4, then evenly spaced others, the rest of the sample within
    `budget` texels."""
    n = len(shapes)
    picks = [max(range(n), key=lambda i: shapes[i][0] * shapes[i][1])]
    for pred in (lambda w, h: w == 1 and h == 1, lambda w, h: w == 2 and h == 2,
                 lambda w, h: w == 3 or h == 3, lambda w, h: (w % 4 or h % 4) and w * h > 64):
        i = next((i for i in range(n) if pred(*shapes[i]) and i not in picks), None)
        if i is not None:
            picks.append(i)
    tex = sum(shapes[i][0] * shapes[i][1] for i in picks[1:])
    for i in range(0, n, max(1, n // (2 * want))):
        if len(picks) >= want:
            break
        t = shapes[i][0] * shapes[i][1]
        if i not in picks and tex + t <= budget:
            picks.append(i)
            tex += t
    return sorted(picks)


def reference_kind() -> tuple[bool, str]:
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    if pyoracle.Reference.available():
        return True, "reference"
    pyoracle.ensure_built()
    return False, "port"


def run_reference_arm(args, wl_name: str, wl: dict) -> None:
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    use_ref, kind = reference_kind()
    cores = os.cpu_count() or 1
    # a band of rows sized to about a second of single-core work per step
    rows = min(wl["h"], 1024 if wl["metric"] in (3, 7) or wl["nrandom"] >= 0 else 4096)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        times = []
        for step in range(args.warmup + args.steps):
            # all workers compress concurrently; the step lasts as long as the
            # slowest, or the whole map when a worker ran two tasks in a row
            t0 = time.perf_counter()
            res = pool.map(_cpu_worker, [(wl_name, rows, use_ref, 1 + step)] * cores, chunksize=1)
            wall = time.perf_counter() - t0
            if step >= args.warmup:
                concurrent = len({r[2] for r in res}) == cores
                times.append(max(r[0] for r in res) if concurrent else wall)
    texels = cores * wl["w"] * rows
    total = sum(times)
    value = texels * len(times) / total
    sample = f"{cores} processes, each the first {rows} rows ({wl['w']}x{rows}) of the workload image per step"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "texels/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "config": config_dict(wl_name, wl),
            "cpu_baseline": {"value": value, "unit": "texels/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "texels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


_BATCH_IMAGES: dict = {}


def _batch_images(wl_name: str, wl: dict, worker: int, nworkers: int, budget: int):
    """The images one reference-arm worker compresses: every nworkers-th
    level of the batched workload until `budget` texels (a band of rows when
    one image is larger)."""
    key = (wl_name, worker, nworkers)
    if key in _BATCH_IMAGES:
        return _BATCH_IMAGES[key]
    from s2tc_gb300 import workloads
    picked, tex = [], 0
    if wl["gen"] == "mips":
        textures = workloads.mip_textures(wl["seed"], count=wl["count"], lo=4, hi=2048)
        levels = [(t["srccomps"], t["fmt"], lvl) for t in textures for lvl in t["levels"]]
        for k in range(worker, len(levels), nworkers):
            sc, fmt, lvl = levels[k]
            picked.append((sc, fmt, np.ascontiguousarray(lvl)))
            tex += lvl.shape[0] * lvl.shape[1]
            if tex >= budget:
                break
    else:
        img = workloads.normal_map(wl["seed"] + worker % wl["distinct"], wl["w"], wl["h"])
        rows = max(4, (budget // wl["w"]) & ~3)
        picked.append((3, wl["fmt"], np.ascontiguousarray(img[:rows])))
    _BATCH_IMAGES[key] = picked
    return picked


def _batch_worker(args):
    """One reference-arm step of a worker: its images through the CPU
    encoder (knobs and rand() seeded per worker); returns (seconds, texels)."""
    wl_name, worker, nworkers, use_ref, seed, budget = args
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    wl = WORKLOADS[wl_name]
    imgs = _batch_images(wl_name, wl, worker, nworkers, budget)
    enc = pyoracle.Reference() if use_ref else pyoracle.Oracle()
    pyoracle.srand(seed * 1009 + worker)
    t0 = time.perf_counter()
    tex = 0
    for sc, fmt, img in imgs:
        h, w = img.shape[:2]
        enc.compress(sc, w, h, img.reshape(-1), fmt, wl["dither"], wl["metric"], wl["nrandom"], wl["refine"])
        tex += w * h
    return time.perf_counter() - t0, tex, os.getpid()


def run_reference_arm_batch(args, wl_name: str, wl: dict) -> None:
    """The reference's CPU encoder on a batched workload: one process per host
    core, each compressing its own share of the images (a bounded sample)."""
    import multiprocessing as mp
    if int(os.environ.get("RANK", "0")) != 0:
        return
    use_ref, kind = reference_kind()
    cores = os.cpu_count() or 1
    budget = 400_000
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        times, texels = [], 0
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_batch_worker, [(wl_name, k, cores, use_ref, step, budget) for k in range(cores)],
                           chunksize=1)
            wall = time.perf_counter() - t0
            if step >= args.warmup:
                concurrent = len({r[2] for r in res}) == cores
                times.append(max(r[0] for r in res) if concurrent else wall)
                texels = sum(r[1] for r in res)
    total = sum(times)
    value = texels * len(times) / total
    sample = (f"{cores} processes, each its share of the workload's images up to {budget} texels "
              f"({texels} texels per step)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "texels/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "config": config_dict(wl_name, wl),
            "cpu_baseline": {"value": value, "unit": "texels/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "texels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_port(wl_name: str, wl: dict, gpu_out0: np.ndarray | None) -> dict:
    """The CPU port on one core, on the full first workload image."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        dt, out, _ = pool.map(_cpu_worker, [(wl_name, wl["h"], False, 1)])[0]
    res = {"value": wl["w"] * wl["h"] / dt, "unit": "texels/s", "cores": 1, "kind": "port",
           "sample": f"one full {wl['w']}x{wl['h']} image, single thread ({dt:.2f} s)"}
    if gpu_out0 is not None:
        res["bit_exact"] = bool(np.array_equal(out, gpu_out0))
    return res


# ------------------------------------------------------------ batch workload

def run_batch_workload(args, wl_name: str, wl: dict) -> None:
    """Batched workloads (uneven mip chains, or many normal maps): one batched
    graph launch vs one s2tc_gpu_compress per image, both with the same
    resident rand words."""
    import torch
    import s2tc_gb300 as s2
    from s2tc_gb300 import workloads
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    opt = s2.options(wl["dither"], wl["metric"], wl["nrandom"], wl["refine"])
    layouts = {}
    if not args.no_autotune:
        for f in ((0x83F1, 0x83F2, 0x83F3) if wl["gen"] == "mips" else (wl["fmt"],)):
            s2.autotune(opt, f, 1024, 1024)
            layouts[FMT_NAMES[f]] = s2.get_layout(opt, f)
    if wl["gen"] == "mips":
        tex = workloads.mip_textures(wl["seed"], count=wl["count"], lo=4, hi=2048)
        levels = [(t, lvl) for t in tex for lvl in t["levels"]]
    else:
        maps = [workloads.normal_map(wl["seed"] + i, wl["w"], wl["h"]) for i in range(wl["distinct"])]
        levels = [({"fmt": wl["fmt"], "srccomps": 3}, maps[i % wl["distinct"]]) for i in range(wl["count"])]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(11)
    images, host_src = [], []
    texels = 0
    in_bytes = out_bytes = rand_bytes = 0
    for t, lvl in levels:
        h, w = lvl.shape[:2]
        flat = np.ascontiguousarray(lvl.reshape(-1))
        words = s2.rand_words(w, h, t["fmt"], opt)
        rw = torch.randint(0, 2**31 - 1, (max(1, words),), dtype=torch.int32, device="cuda", generator=gen)
        n = s2.compressed_size(w, h, t["fmt"])
        images.append({"src": torch.from_numpy(flat).cuda(), "width": w, "height": h, "srccomps": t["srccomps"],
                       "format": t["fmt"], "dst": torch.empty(n, dtype=torch.uint8, device="cuda"), "rand": rw})
        host_src.append(torch.from_numpy(flat).pin_memory())
        texels += w * h
        in_bytes += flat.nbytes
        out_bytes += n
        rand_bytes += 4 * words
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    batch = s2.Batch(images, opt)
    ref_out = [torch.empty_like(im["dst"]) for im in images]
    each_arr = s2.image_array([dict(im, dst=d) for im, d in zip(images, ref_out)])

    def per_image(dsts):
        # the per-image path, driven from C: one s2tc_gpu_compress per level
        s2.gpu_compress_each(images, opt, sp, arr=each_arr)

    for _ in range(args.warmup):
        batch.run(sp)
        per_image(ref_out)
    s2.gpu_synchronize(sp)
    bit_exact = all(torch.equal(im["dst"], r) for im, r in zip(images, ref_out))
    # the batch's bytes against the oracle, given the same words, on a sample
    # (the largest level, edge levels; for the normal maps eight whole maps)
    import zlib
    shapes = [(im["width"], im["height"]) for im in images]
    sample = sample_levels(shapes) if wl["gen"] == "mips" else list(range(min(8, len(images))))
    jobs = []
    for i in sample:
        im = images[i]
        words = s2.rand_words(im["width"], im["height"], im["format"], opt)
        jobs.append((im["srccomps"], im["width"], im["height"], levels[i][1].reshape(-1), im["format"],
                     wl["dither"], wl["metric"], wl["nrandom"], wl["refine"],
                     im["rand"][:words].cpu().numpy().view(np.uint32) if words else None))
    want_crc = oracle_crcs(jobs)
    got_crc = [zlib.crc32(images[i]["dst"].cpu().numpy().tobytes()) for i in sample]
    oracle_check = {"bit_exact_vs_oracle": want_crc == got_crc, "images_checked": len(sample),
                    "sizes_checked": [list(shapes[i]) for i in sample],
                    "texels_checked": sum(shapes[i][0] * shapes[i][1] for i in sample)}
    del jobs

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0

    l0 = s2.kernel_launches()
    with ClockSampler(0) as clk:
        t_batch = timed(lambda: batch.run(sp))
    launches = s2.kernel_launches() - l0
    t_single = timed(lambda: per_image(ref_out))
    s2.gpu_synchronize(sp)
    value = args.steps * texels / t_batch
    single = args.steps * texels / t_single

    # where the time goes, by level size: each class of images as a batch of
    # its own and through the per-image path (same rand words)
    breakdown = {}
    for cls, lo, hi in (("le_64x64", 0, 64 * 64), ("le_256x256", 64 * 64, 256 * 256), ("gt_256x256", 256 * 256, 1 << 62)):
        sub = [im for im in images if lo < im["width"] * im["height"] <= hi]
        if not sub:
            continue
        tex = sum(im["width"] * im["height"] for im in sub)
        sub_out = [torch.empty_like(im["dst"]) for im in sub]
        sub_arr = s2.image_array([dict(im, dst=d) for im, d in zip(sub, sub_out)])
        sb = s2.Batch(sub, opt)
        sb.run(sp)
        s2.gpu_compress_each(sub, opt, sp, arr=sub_arr)
        s2.gpu_synchronize(sp)
        tb = timed(lambda: sb.run(sp))
        te = timed(lambda: s2.gpu_compress_each(sub, opt, sp, arr=sub_arr))
        s2.gpu_synchronize(sp)
        sb.close()
        breakdown[cls] = {"images": len(sub), "texels": tex, "batched_ms": 1000 * tb / args.steps,
                          "per_image_ms": 1000 * te / args.steps, "per_image_over_batched": te / tb,
                          "share_of_per_image_time": None}
    tot_e = sum(b["per_image_ms"] for b in breakdown.values())
    for b in breakdown.values():
        b["share_of_per_image_time"] = b["per_image_ms"] / tot_e if tot_e else None

    # end to end through the batch API as a reference user calls it: pinned
    # host pixels in, blocks out, and the random candidates drawn from the
    # process's libc rand() stream (in image order, as one tx_compress_dxtn
    # call per image would draw them; the library generates those words on the
    # GPU and advances libc's state)
    host_out = [torch.empty(im["dst"].numel(), dtype=torch.uint8).pin_memory() for im in images]
    libc_images = [{k: v for k, v in im.items() if k != "rand"} for im in images]
    libc_batch = s2.Batch(libc_images, opt)

    def e2e_step():
        for im, hs in zip(images, host_src):
            im["src"].copy_(hs, non_blocking=True)
        libc_batch.run(sp)
        for im, ho in zip(images, host_out):
            ho.copy_(im["dst"], non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    libc_batch.close()

    # the same images through the reference-compatible entry point, one
    # synchronous tx_compress_dxtn call per image (host buffers)
    s2.set_env(wl["dither"], wl["metric"], wl["nrandom"], wl["refine"])
    lib = s2.load()
    host_dst = [torch.empty(im["dst"].numel(), dtype=torch.uint8).pin_memory() for im in images]

    def per_image_host():
        for im, hs, hd in zip(images, host_src, host_dst):
            lib.tx_compress_dxtn(im["srccomps"], im["width"], im["height"], hs.data_ptr(), im["format"],
                                 hd.data_ptr(), 0)

    per_image_host()
    t0 = time.perf_counter()
    host_passes = max(1, args.steps // 5)
    for _ in range(host_passes):
        per_image_host()
    t_host = (time.perf_counter() - t0) / host_passes

    cpu = None
    if not args.no_cpu_baseline:
        # the CPU port on a bounded sample: the first levels until ~1.5 M
        # texels (a band of rows of the first image when that alone is larger)
        sys.path.insert(0, str(ROOT / "oracle"))
        import pyoracle
        oracle = pyoracle.Oracle()
        sample, sample_tex = [], 0
        for t, lvl in levels:
            if not sample and lvl.shape[0] * lvl.shape[1] > 1_500_000:
                rows = max(4, (1_000_000 // lvl.shape[1]) & ~3)
                sample.append((t, np.ascontiguousarray(lvl[:rows])))
                sample_tex = rows * lvl.shape[1]
                break
            sample.append((t, lvl))
            sample_tex += lvl.shape[0] * lvl.shape[1]
            if sample_tex >= 1_000_000:
                break
        pyoracle.srand(1)
        c0 = time.perf_counter()
        for t, lvl in sample:
            h, w = lvl.shape[:2]
            oracle.compress(t["srccomps"], w, h, lvl.reshape(-1), t["fmt"], wl["dither"], wl["metric"],
                            wl["nrandom"], wl["refine"])
        dt = time.perf_counter() - c0
        cpu = {"value": sample_tex / dt, "unit": "texels/s", "cores": 1, "kind": "port",
               "sample": f"the first {len(sample)} images (a band of rows when the first is large; {sample_tex} texels), "
                          f"single thread ({dt:.2f} s)"}
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs") or 6800.0
    alg = in_bytes + out_bytes
    achieved = alg / (t_batch / args.steps) / 1e9
    clocks = clk.summary()
    hbm_line = {"bound": "hbm", "kernel": "batch step", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": None}
    alu = issue_roofline(wl_name, "batch", 1000 * t_batch / args.steps, texels, clocks.get("sm_mhz") or 2070.0,
                         torch.cuda.get_device_properties(0).multi_processor_count)
    roofline = dict(alu, hbm=hbm_line) if alu else hbm_line
    roofline["note"] = "the random-candidate pair search (one warp per block) is integer-ALU bound"
    line = {"metric": METRIC, "value": value, "unit": "texels/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * t_batch / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": dict(config_dict(wl_name, wl), images=len(images), texels=texels,
                           launch_layout=layouts or "default"),
            "per_image": {"value": single, "unit": "texels/s", "ms_per_step": 1000 * t_single / args.steps,
                          "launches_per_step": None},
            "batched_over_per_image": value / single, "by_level_size": breakdown,
            "bit_exact_batched_vs_per_image": bit_exact,
            **oracle_check,
            "per_image_tx_compress_dxtn": {"value": texels / t_host, "unit": "texels/s", "ms_per_step": 1000 * t_host,
                                           "note": "one synchronous call per image, pinned host buffers"},
            "e2e_over_per_image_tx_compress_dxtn": (args.steps * texels / t_e2e) / (texels / t_host),
            "e2e": {"value": args.steps * texels / t_e2e, "unit": "texels/s",
                    "h2d_bytes_per_step": in_bytes, "d2h_bytes_per_step": out_bytes,
                    "rand": "libc rand() stream, generated on the device",
                    "ms_per_step": 1000 * t_e2e / args.steps},
            "gpu_launches": launches,
            "roofline": roofline,
            "cpu_baseline": cpu, "clocks": clocks}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- tool workloads

def run_tool_workload(args, wl_name: str, wl: dict) -> None:
    """The reference's tools on the GPU.  decode / from_s3tc: device-resident
    blocks (two rotating inputs larger than L2), CUDA events around K launches;
    e2e through the in-memory file entry points.  dds: s2tc_compress_dds with
    host buffers (it is end to end by construction)."""
    import torch
    import s2tc_gb300 as s2
    from s2tc_gb300 import workloads
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    w, h, fmt = wl["w"], wl["h"], wl["fmt"]
    npx = w * h
    bs = 8 if fmt in (0x83F0, 0x83F1) else 16
    nblocks = ((w + 3) // 4) * ((h + 3) // 4)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs") or 6800.0
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    oracle = pyoracle.Oracle()
    rng = np.random.default_rng(wl["seed"])
    cpu = None
    if wl["tool"] in ("decode", "from_s3tc"):
        blocks = [rng.integers(0, 256, nblocks * bs, dtype=np.uint8) for _ in range(2)]
        d_in = [torch.from_numpy(b).cuda() for b in blocks]
        if wl["tool"] == "decode":
            d_out = [torch.empty(npx * 4, dtype=torch.uint8, device="cuda") for _ in range(2)]
            launch = lambda i: s2.gpu_decode(d_in[i % 2], fmt, w, h, d_out[i % 2], 0, False, sp)
            alg = nblocks * bs + npx * 4
        else:
            d_out = [torch.empty_like(x) for x in d_in]
            launch = lambda i: s2.gpu_from_s3tc(d_in[i % 2], d_out[i % 2], nblocks, fmt, sp)
            alg = 2 * nblocks * bs
        for i in range(args.warmup):
            launch(i)
        torch.cuda.synchronize()
        l0 = s2.kernel_launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(0) as clk:
            e0.record(stream)
            for i in range(args.steps):
                launch(i)
            e1.record(stream)
            torch.cuda.synchronize()
        launches = s2.kernel_launches() - l0
        t = e0.elapsed_time(e1) / 1000.0
        value = args.steps * npx / t
        achieved = alg / (t / args.steps) / 1e9
        # parity of the timed kernel on a sample of its output
        if wl["tool"] == "decode":
            got = d_out[0].cpu().numpy().reshape(h, w, 4)
            for (i, j) in ((0, 0), (w - 1, h - 1), (1234, 567), (w // 2, h // 3)):
                assert np.array_equal(got[j, i], oracle.fetch(2 if fmt == 0x83F3 else 0, 1, w, blocks[0], i, j))
        else:
            got = d_out[0][: 1000 * bs].cpu().numpy()
            assert np.array_equal(got, oracle.from_s3tc_blocks(blocks[0][: 1000 * bs], 2 if fmt == 0x83F3 else 0))
        # end to end through the in-memory file entry point
        hdr = bytearray(128)
        hdr[0:4] = b"DDS "
        hdr[12:16] = h.to_bytes(4, "little")
        hdr[16:20] = w.to_bytes(4, "little")
        hdr[84:88] = (b"DXT5" if fmt == 0x83F3 else b"DXT1")
        dds = bytes(hdr) + blocks[0].tobytes()
        fn = s2.decompress_dds if wl["tool"] == "decode" else s2.from_s3tc_dds
        fn(dds)
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps // 4)):
            fn(dds)
        t_e2e = (time.perf_counter() - t0) / max(1, args.steps // 4)
        e2e = {"value": npx / t_e2e, "unit": "texels/s", "h2d_bytes_per_step": len(dds),
               "d2h_bytes_per_step": (18 + npx * 4) if wl["tool"] == "decode" else len(dds),
               "ms_per_step": 1000 * t_e2e, "note": "host file in, host file out, pageable buffers"}
        if not args.no_cpu_baseline:
            rows = 512
            if wl["tool"] == "decode":
                sub = bytes(hdr[:12]) + rows.to_bytes(4, "little") + bytes(hdr[16:]) + \
                    blocks[0][: (rows // 4) * (w // 4) * bs].tobytes()
                c0 = time.perf_counter()
                oracle.decompress(sub)
            else:
                sub = bytes(hdr) + blocks[0][: (rows // 4) * (w // 4) * bs].tobytes()
                c0 = time.perf_counter()
                oracle.from_s3tc(sub)
            dt = time.perf_counter() - c0
            cpu = {"value": rows * w / dt, "unit": "texels/s", "cores": 1, "kind": "port",
                   "sample": f"the first {rows} rows ({rows * w} texels), single thread ({dt:.2f} s)"}
        kernel = "k_decode" if wl["tool"] == "decode" else "k_from_s3tc"
        traffic = None
        try:
            traffic = json.loads((ROOT / "profiles" / "traffic.json").read_text()).get(wl_name, {}).get(kernel)
        except Exception:
            pass
        roofline = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                    "frac": achieved / hbm, "traffic": traffic, "algorithmic_bytes_per_launch": alg}
        ms = 1000 * t / args.steps
    else:
        img = workloads.plain_rgba(wl["seed"], w, h)
        opt = s2.options(wl["dither"], wl["metric"], wl["nrandom"], wl["refine"])
        out0 = s2.compress_dds(img, w, h, fmt, opt)
        for _ in range(args.warmup - 1):
            s2.compress_dds(img, w, h, fmt, opt)
        l0 = s2.kernel_launches()
        with ClockSampler(0) as clk:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                s2.compress_dds(img, w, h, fmt, opt)
            t = time.perf_counter() - t0
        launches = s2.kernel_launches() - l0
        levels_tex = 0
        lw, lh = w, h
        while True:
            levels_tex += lw * lh
            if lw == 1 and lh == 1:
                break
            lw, lh = max(1, lw // 2), max(1, lh // 2)
        value = args.steps * levels_tex / t
        ms = 1000 * t / args.steps
        e2e = {"value": value, "unit": "texels/s", "h2d_bytes_per_step": npx * 4, "d2h_bytes_per_step": len(out0),
               "ms_per_step": ms, "note": "host RGBA in, host DDS file out; the call is the step"}
        alg = levels_tex * 4 + len(out0)
        achieved = alg / (t / args.steps) / 1e9
        roofline = {"bound": "hbm", "kernel": "pipeline", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                    "frac": achieved / hbm, "traffic": None,
                    "note": "whole call including host copies; the encoder is integer-bound"}
        if not args.no_cpu_baseline:
            small = np.ascontiguousarray(img[:512, :512])
            c0 = time.perf_counter()
            want = oracle.dds(small, 512, 512, fmt, wl["dither"], wl["metric"], wl["nrandom"], wl["refine"])
            dt = time.perf_counter() - c0
            got = s2.compress_dds(small, 512, 512, fmt, opt)
            cpu = {"value": (512 * 512 * 4 // 3) / dt, "unit": "texels/s", "cores": 1, "kind": "port",
                   "sample": f"a 512x512 crop with its mip chain, single thread ({dt:.2f} s)",
                   "bit_exact": got == want}
    line = {"metric": METRIC, "value": value, "unit": "texels/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": config_dict(wl_name, wl),
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------- serving workload

def _lindley(arrivals, service):
    """Latencies of a single FIFO server that takes the requests one at a
    time (the per-request path) under the given arrival times."""
    lat, free = [], 0.0
    for a, s in zip(arrivals, service):
        start = max(a, free)
        free = start + s
        lat.append(free - a)
    return lat


def run_serving_workload(args, wl_name: str, wl: dict) -> None:
    """The continuous-batching request loop (s2tc_server_*) against the plain
    per-request path (one tx_compress_dxtn per request): saturated
    throughput, then Poisson arrivals at fractions of that rate with the
    server's own p50/p99 latencies (submit to blocks in host memory)."""
    import threading
    import zlib
    import torch
    import s2tc_gb300 as s2
    from s2tc_gb300 import workloads
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    nreq = args.steps * wl["per_step"]
    reqs = workloads.serving_requests(wl["seed"], count=nreq, lo=64, hi=4096)
    # one pinned pool of pixels; request i reads a window at a seeded offset
    pool_img = np.concatenate([workloads.plain_rgba(wl["seed"], 4096, 4096),
                               workloads.plain_rgba(wl["seed"] + 1, 4096, 4096)]).reshape(-1)
    pool = torch.from_numpy(pool_img).pin_memory()
    half = pool_img.nbytes // 2
    rng = np.random.default_rng(wl["seed"])
    offs = (rng.integers(0, half // 256, nreq) * 256).tolist()
    sizes = [(r["width"], r["height"], r["fmt"]) for r in reqs]
    opts = {m: s2.options(wl["dither"], m, wl["nrandom"], wl["refine"]) for m in (3, 5, 7)}
    out_sizes = [s2.compressed_size(w, h, f) for w, h, f in sizes]
    texels = [w * h for w, h, _ in sizes]
    base = pool.data_ptr()
    ring_bytes = 2 << 30
    ring = torch.empty(ring_bytes, dtype=torch.uint8).pin_memory()
    rbase = ring.data_ptr()
    lib = s2.load()

    def serve(arrivals, check=None):
        """Submit every request at its arrival time (None: all at once);
        outputs go to a ring of pinned memory that the waiter frees in order."""
        srv = s2.Server(wl["budget"])
        ids = [0] * nreq
        lat = [0.0] * nreq
        cond = threading.Condition()
        state = {"consumed": 0, "submitted": 0}
        dst_off = [0] * nreq
        crcs = {}

        def waiter():
            for i in range(nreq):
                with cond:
                    cond.wait_for(lambda: state["submitted"] > i)
                lat[i] = srv.wait(ids[i])
                if check is not None and i in check:
                    crcs[i] = zlib.crc32(ctypes.string_at(rbase + dst_off[i], out_sizes[i]))
                with cond:
                    state["consumed"] = i + 1
                    cond.notify_all()

        th = threading.Thread(target=waiter)
        th.start()
        head = 0

        def fits(i, n):
            # unconsumed outputs occupy the arc from the oldest one's offset
            # (tail) up to head
            c = state["consumed"]
            if c >= i:
                return True
            tail = dst_off[c]
            if tail < head:
                return head + n <= ring_bytes
            return tail > head and head + n <= tail

        t0 = time.perf_counter()
        for i in range(nreq):
            n = out_sizes[i]
            if head + n > ring_bytes:
                head = 0
            if not fits(i, n):
                with cond:
                    cond.wait_for(lambda: fits(i, n))
            if arrivals is not None:
                due = t0 + arrivals[i]
                while True:
                    dt = due - time.perf_counter()
                    if dt <= 0:
                        break
                    time.sleep(dt if dt > 2e-4 else 0)
            w, h, f = sizes[i]
            dst_off[i] = head
            ids[i] = srv.submit(base + offs[i], 4, w, h, f, opts[reqs[i]["metric"]], rbase + head)
            head += (n + 255) // 256 * 256
            with cond:
                state["submitted"] = i + 1
                cond.notify_all()
        th.join()
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        return wall, lat, st, crcs

    # the per-request path: one synchronous tx_compress_dxtn per request
    check = set(range(0, nreq, 10))
    want = {}
    service = [0.0] * nreq
    out1 = torch.empty(max(out_sizes), dtype=torch.uint8).pin_memory()
    cur = [None]

    def per_request(i):
        w, h, f = sizes[i]
        m = reqs[i]["metric"]
        if cur[0] != m:
            s2.set_env(wl["dither"], m, wl["nrandom"], wl["refine"])
            cur[0] = m
        lib.tx_compress_dxtn(4, w, h, base + offs[i], f, out1.data_ptr(), 0)

    for i in range(min(nreq, 50)):
        per_request(i)
    for i in range(nreq):
        t0 = time.perf_counter()
        per_request(i)
        service[i] = time.perf_counter() - t0
        if i in check:
            want[i] = zlib.crc32(ctypes.string_at(out1.data_ptr(), out_sizes[i]))
    t_single = sum(service)
    total_tex = sum(texels)

    serve(None)  # warm-up: streams, pinned tables, first-use of the kernels
    l0 = s2.kernel_launches()
    with ClockSampler(0) as clk:
        wall, lat, st, crcs = serve(None, check)
    launches = s2.kernel_launches() - l0
    bit_exact = all(crcs.get(i) == want[i] for i in check)
    # the server's bytes against the oracle on a sample of the checked
    # requests: the largest, the smallest, one per distance metric, others
    # spread over the sizes
    chk = sorted(check)
    picked = [chk[j] for j in sample_levels([(sizes[i][0], sizes[i][1]) for i in chk], budget=20_000_000)]
    for m in (3, 5, 7):
        if not any(reqs[i]["metric"] == m for i in picked):
            i = next((i for i in chk if reqs[i]["metric"] == m and texels[i] <= 1 << 20), None)
            if i is not None:
                picked.append(i)
    smallest = min(chk, key=lambda i: texels[i])
    if smallest not in picked:
        picked.append(smallest)
    jobs = [(4, sizes[i][0], sizes[i][1], pool_img[offs[i]:offs[i] + texels[i] * 4], sizes[i][2], wl["dither"],
             reqs[i]["metric"], wl["nrandom"], wl["refine"], None) for i in picked]
    oracle_ok = oracle_crcs(jobs) == [crcs.get(i) for i in picked]
    value = total_tex / wall
    rate_max = nreq / wall
    poisson = []
    for frac in (0.5, 0.8):
        rate = frac * rate_max
        arr = np.cumsum(np.random.default_rng(17).exponential(1.0 / rate, nreq)).tolist()
        pw, plat, pst, _ = serve(arr)
        single_lat = _lindley(arr, service)
        poisson.append({"rate_rps": rate, "offered_frac_of_saturation": frac,
                        "texels_per_s": total_tex / pw,
                        "p50_ms": float(np.percentile(plat, 50)), "p99_ms": float(np.percentile(plat, 99)),
                        "rounds": pst["rounds"], "max_inflight_rounds": pst["max_inflight_rounds"],
                        "per_request_path_p50_ms": 1000 * float(np.percentile(single_lat, 50)),
                        "per_request_path_p99_ms": 1000 * float(np.percentile(single_lat, 99))})
    in_b = sum(t * 4 for t in texels)
    out_b = sum(out_sizes)
    line = {"metric": METRIC, "value": value, "unit": "texels/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * wall / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": dict(config_dict(wl_name, wl), requests=nreq, texels=total_tex),
            "e2e": {"value": value, "unit": "texels/s", "h2d_bytes_per_step": in_b // args.steps,
                    "d2h_bytes_per_step": out_b // args.steps,
                    "note": "host buffers in and out; the loop is end to end by construction"},
            "saturated": {"rounds": st["rounds"], "max_round_requests": st["max_round_requests"],
                          "max_inflight_rounds": st["max_inflight_rounds"],
                          "pool_high_water": st["pool_high_water"],
                          "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))},
            "per_request": {"value": total_tex / t_single, "unit": "texels/s",
                            "ms_per_request_mean": 1000 * t_single / nreq},
            "server_over_per_request": value / (total_tex / t_single),
            "poisson": poisson, "bit_exact_sampled": bit_exact, "bit_exact_requests_checked": len(check),
            "bit_exact_vs_oracle": oracle_ok, "oracle_requests_checked": len(picked),
            "oracle_sizes_checked": [[sizes[i][0], sizes[i][1]] for i in sorted(picked)],
            "gpu_launches": launches, "cpu_baseline": None, "clocks": clk.summary(),
            "roofline": None}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ small calls

def run_small_calls(args, wl_name: str, wl: dict) -> None:
    """Per-call latency of tx_compress_dxtn on small square images (the cost a
    GL driver sees per texture upload): pageable numpy buffers, one call after
    another, host wall clock per call; each size checked against the oracle
    once.  `value` is the texels/s of the largest size's calls."""
    import torch
    import s2tc_gb300 as s2
    from s2tc_gb300 import workloads
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    oracle = pyoracle.Oracle()
    lib = s2.load()
    s2.set_env(wl["dither"], wl["metric"], wl["nrandom"], wl["refine"])
    l0 = s2.kernel_launches()
    sizes, exact, launches = {}, True, {}
    with ClockSampler(0) as clk:
        for n in wl["sizes"]:
            img = np.ascontiguousarray(workloads.plain_rgba(wl["seed"], n, n).reshape(-1))
            out = np.zeros(s2.compressed_size(n, n, wl["fmt"]), np.uint8)
            for _ in range(max(args.warmup, 3) * 10):
                lib.tx_compress_dxtn(4, n, n, img.ctypes.data, wl["fmt"], out.ctypes.data, 0)
            want = oracle.compress(4, n, n, img, wl["fmt"], wl["dither"], wl["metric"], wl["nrandom"], wl["refine"])
            exact &= bool(np.array_equal(out, want))
            calls = max(20, args.steps * 10)
            k0 = s2.kernel_launches()
            ts = []
            for _ in range(calls):
                t0 = time.perf_counter()
                lib.tx_compress_dxtn(4, n, n, img.ctypes.data, wl["fmt"], out.ctypes.data, 0)
                ts.append(time.perf_counter() - t0)
            launches[f"{n}x{n}"] = (s2.kernel_launches() - k0) / calls
            ts = np.array(ts) * 1e6
            # the kernels' own device time per call (library CUDA events)
            s2.set_timing(True)
            for _ in range(20):
                lib.tx_compress_dxtn(4, n, n, img.ctypes.data, wl["fmt"], out.ctypes.data, 0)
            dms, ems, ncalls = s2.stage_ms()
            s2.set_timing(False)
            sizes[f"{n}x{n}"] = {"median_us": float(np.median(ts)), "p10_us": float(np.percentile(ts, 10)),
                                 "p90_us": float(np.percentile(ts, 90)), "calls": calls,
                                 "kernel_us": 1000 * (dms + ems) / max(1, ncalls)}
    big = f"{wl['sizes'][-1]}x{wl['sizes'][-1]}"
    value = wl["sizes"][-1] ** 2 / (sizes[big]["median_us"] * 1e-6)
    line = {"metric": METRIC, "value": value, "unit": "texels/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sizes[big]["median_us"] / 1000, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": dict(config_dict(wl_name, wl), sizes=wl["sizes"]),
            "latency_per_call": sizes, "kernel_launches_per_call": launches, "bit_exact_vs_oracle": exact,
            "e2e": {"value": value, "unit": "texels/s", "h2d_bytes_per_step": wl["sizes"][-1] ** 2 * 4,
                    "d2h_bytes_per_step": s2.compressed_size(wl["sizes"][-1], wl["sizes"][-1], wl["fmt"]),
                    "note": "pageable host buffers; one synchronous call per step"},
            "gpu_launches": int(round(launches[big] * (max(20, args.steps * 10)))),
            "roofline": None, "cpu_baseline": None, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- multi-rank

def aggregate_ranks(seconds: float, units: int, dist=None, device: str = "cpu"):
    """Replicas: every rank processed `units` in `seconds`; the job took the
    slowest rank's time and processed all ranks' units.  Returns
    (max seconds over ranks, units of all ranks / that time)."""
    world = 1
    if dist is not None and dist.is_initialized():
        import torch
        world = dist.get_world_size()
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        seconds = float(t.item())
    return seconds, world * units / seconds


# ------------------------------------------------------------------- GPU arm

def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU port leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch layouts")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.warmup < 3 and args.impl == "gb300":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        if wl["gen"] in ("mips", "normal_batch"):
            run_reference_arm_batch(args, args.workload, wl)
            return
        if wl["gen"] in ("serving", "tool", "small"):
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the encoder workloads"}))
            return
        run_reference_arm(args, args.workload, wl)
        return
    if wl["gen"] in ("mips", "normal_batch"):
        run_batch_workload(args, args.workload, wl)
        return
    if wl["gen"] == "serving":
        run_serving_workload(args, args.workload, wl)
        return
    if wl["gen"] == "tool":
        run_tool_workload(args, args.workload, wl)
        return
    if wl["gen"] == "small":
        run_small_calls(args, args.workload, wl)
        return

    import torch
    import s2tc_gb300 as s2
    from s2tc_gb300 import build as s2build
    if not s2.LIB_PATH.exists():
        s2build.build_library()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    w, h, sc, fmt = wl["w"], wl["h"], wl["sc"], wl["fmt"]
    npx = w * h
    out_bytes = s2.compressed_size(w, h, fmt)
    opt = s2.options(wl["dither"], wl["metric"], wl["nrandom"], wl["refine"])
    layout = None
    if not args.no_autotune:
        s2.autotune(opt, fmt, min(w, 2048), min(h, 2048))
        layout = s2.get_layout(opt, fmt)
    images = [make_image(wl, wl["seed"] + 100 * rank + i) for i in range(NIMG)]
    d_src = [torch.from_numpy(im).cuda() for im in images]
    d_dst = [torch.empty(out_bytes, dtype=torch.uint8, device="cuda") for _ in range(NIMG)]
    d_rand = None
    nwords = s2.rand_words(w, h, fmt, opt)
    if nwords:
        # replayed rand() words for one image, reused by every step
        sys.path.insert(0, str(ROOT / "oracle"))
        rng = np.random.default_rng(9)
        d_rand = torch.from_numpy(rng.integers(0, 2**31, nwords, dtype=np.int64).astype(np.uint32)).cuda()
    # a dedicated stream: the library treats a null stream as "use my own"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    assert sp != 0

    def step(i, rand=d_rand):
        s2.gpu_compress(sc, w, h, d_src[i % NIMG], fmt, d_dst[i % NIMG], opt=opt, d_rand=rand, stream=sp)

    # first warm-up step: image 0 with libc rand() replayed from srand(1), the
    # output the CPU leg checks; the timed steps reuse one stored rand stream
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    pyoracle.srand(1)
    step(0, None)
    s2.gpu_synchronize(sp)
    out0 = d_dst[0].cpu().numpy()
    for i in range(1, args.warmup):
        step(i)
    s2.gpu_synchronize(sp)

    # --- device-resident timed region
    s2.set_timing(True)
    l0 = s2.kernel_launches()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for i in range(args.steps):
            step(i)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    launches = s2.kernel_launches() - l0
    dither_ms, encode_ms, calls = s2.stage_ms()
    s2.set_timing(False)
    s2.gpu_synchronize(sp)
    elapsed = ev0.elapsed_time(ev1) / 1000.0
    elapsed, value = aggregate_ranks(elapsed, args.steps * npx, dist, "cuda")

    # --- end to end through tx_compress_dxtn with pinned host buffers
    e2e = None
    if not args.no_e2e:
        s2.set_env(wl["dither"], wl["metric"], wl["nrandom"], wl["refine"])
        h_src = [torch.from_numpy(im).pin_memory() for im in images]
        h_dst = torch.empty(out_bytes, dtype=torch.uint8).pin_memory()
        lib = s2.load()
        for i in range(min(args.warmup, 3)):
            lib.tx_compress_dxtn(sc, w, h, h_src[i % NIMG].data_ptr(), fmt, h_dst.data_ptr(), 0)
        barrier()
        call_s = []
        t0 = time.perf_counter()
        for i in range(args.steps):
            c0 = time.perf_counter()
            lib.tx_compress_dxtn(sc, w, h, h_src[i % NIMG].data_ptr(), fmt, h_dst.data_ptr(), 0)
            call_s.append(time.perf_counter() - c0)
        t_e2e = time.perf_counter() - t0
        barrier()
        t_e2e, e2e_value = aggregate_ranks(t_e2e, args.steps * npx, dist, "cuda")
        e2e = {"value": e2e_value, "unit": "texels/s",
               "h2d_bytes_per_step": npx * sc, "d2h_bytes_per_step": out_bytes,
               "ms_per_step": 1000 * t_e2e / args.steps,
               # the spread of the synchronous calls (this rank): the value above
               # is the mean; a slow call on a busy host shows up here
               "ms_per_call_median": 1000 * float(np.median(call_s)),
               "ms_per_call_max": 1000 * float(np.max(call_s))}

    # --- roofline of the dominant kernel
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs")
    peak_note = "measured" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or 6800.0
    enc_launch_ms = encode_ms / max(1, calls)
    dit_launch_ms = dither_ms / max(1, calls)
    alg_bytes = algorithmic_bytes_per_texel(wl) * npx
    dominant = "encode" if enc_launch_ms >= dit_launch_ms else "dither"
    dom_ms = max(enc_launch_ms, dit_launch_ms)
    achieved = alg_bytes / (dom_ms / 1000.0) / 1e9
    hbm = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
           "frac": achieved / hbm_peak, "peak_source": peak_note, "traffic": None}
    prof = ROOT / "profiles" / "traffic.json"
    if prof.exists():
        try:
            hbm["traffic"] = json.loads(prof.read_text()).get(args.workload, {}).get(dominant)
        except Exception:
            pass
    clocks = clk.summary()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    alu = issue_roofline(args.workload, dominant, dom_ms, npx, clocks.get("sm_mhz") or 2070.0, sms)
    search = wl["nrandom"] >= 0 or wl["metric"] == 7
    if alu is not None and (search or dominant == "dither"):
        # integer-bound kernels: the issue roofline first, HBM beside it
        roofline = dict(alu, hbm=hbm)
    else:
        roofline = dict(hbm, alu=alu)
    roofline["stage_ms_per_launch"] = {"dither": dit_launch_ms, "encode": enc_launch_ms}
    roofline["note"] = roofline_note(dominant, wl)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_port(args.workload, wl, out0)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "texels/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * elapsed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
                "config": dict(config_dict(args.workload, wl), launch_layout=layout or "default"),
                "e2e": e2e, "gpu_launches": launches,
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
                "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
