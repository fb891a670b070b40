#!/usr/bin/env python3
"""Benchmark of the lossy VarDCT pixel path + SSIMULACRA2 on GB300.

Workload (one "step"): the quality controller's probe — encode transform,
reconstruct (dequantize, IDCT, Gaborish, 3-step EPF, colour, 16-bit depth
round trip) and SSIMULACRA2 against the precomputed source — over a batch of
8 distinct 2048x2048 RGB16 synthetic images (seeded; mixed DCT8/16/32 cover
from select_blocks; CfL; Gaborish; uniform sharpness 7; global_scale 40000).
Source moments for the metric are precomputed once per image, outside the
timed region, as the reference's evaluator does (evaluator.rs:88 ->
reference.rs:90).

The DCTs run in the precision named by --precision (the headline): "fp32"
(the reference's butterflies, bit-exact), "bf16x3" or "bf16x6"
(split-precision contractions on the tcgen05 tensor cores).  Every mode is
timed on the same inputs and reported under `precision_modes`.

Prints one JSON line.  `value` is source MPix/s with inputs resident in HBM;
`e2e` is the same metric through the C ABI with pinned host buffers (the H2D
copy of each image and the D2H read of each score inside the timed region).
`parity` states each mode's errors on image 0 of the step (full size)
against the CPU restatement of the reference and against the FP64 truth;
`scoring` times SSIMULACRA2 on 32 pairs of 4096x3072 RGB8 (source against
reconstruction); `search` times the batched quality search (64 uneven RGB8
frames x 8 candidate quantizers = 512 probes in one CUDA graph launch) and,
under `navigate`, the quality controller's own search over the same frames;
`decode` times 256 cjxl streams decoded to 8-bit sRGB by one graph launch
and counts the samples 1 DN off djxl's decodes.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

W, H, BITS = 2048, 2048, 16
IMAGES_PER_STEP = 8
GLOBAL_SCALE = 40000
WORKLOAD = ("2048x2048 RGB16 quality probe: encode transform (XYB, inverse Gaborish, DCT8/16/32, "
            "CfL, quantize) + reconstruct (Gaborish, 3-step EPF, 16-bit depth) + SSIMULACRA2 "
            "(6 scales)")

PRECISIONS = ("fp32", "bf16x3", "bf16x6")

# Algorithmic HBM bytes per source pixel of the path's three parts (the
# minimum each must move: RGB16 in + int32 coefficients out for the encode
# transform; coefficients in + f32 planes out for the reconstruction;
# candidate planes + the reference's nine moment planes over the pyramid for
# SSIMULACRA2).
GROUP_BYTES_PER_PX = {"encode": 18.2, "reconstruct": 24.2, "ssim": 60.0}
STAGE_GROUP = {"xyb": "encode", "precondition": "encode", "fdct_luma": "encode", "cfl": "encode",
               "quant_chroma": "encode", "render_varblocks": "reconstruct",
               "gaborish": "reconstruct", "epf": "reconstruct", "colour": "reconstruct",
               "ssim": "ssim", "ssim_rows": "ssim", "ssim_col_ripple": "ssim",
               "ssim_col_out": "ssim"}
# The metric's blur kernels, each timed under its own stage: algorithmic bytes
# per pixel of every pyramid scale (f32 planes read and written once):
# k_blur_rows<3> reads the candidate's and the reference's positive XYB and
# writes the nine row-pass planes (15 planes); k_blur_col_out<3> (the column
# pass with the ripple's segment scan inside) reads the nine and the
# reference's mu, sigma11 and XYB and the candidate's XYB (21).  The column
# ripple's stage now holds only the reset of the scan's flags.
KERNEL_STAGES = {"ssim_rows": ("k_blur_rows<3>", 60.0),
                 "ssim_col_out": ("k_blur_col_out<3>", 84.0)}


def pyramid_pixels(w: int, h: int) -> int:
    """Pixels over SSIMULACRA2's scales (halving, rounded up, while 8x8 fits;
    at most six)."""
    total, s = 0, 0
    while s < 6 and w >= 8 and h >= 8:
        total += w * h
        w, h, s = (w + 1) // 2, (h + 1) // 2, s + 1
    return total


def shard_units(units: list, rank: int, world: int) -> list:
    """Replicas: each rank takes a disjoint slice of the images."""
    return units[rank::world]


def max_over_ranks(t: float) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return t
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    x = torch.tensor([t], dtype=torch.float64, device=dev)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []
        self.first = threading.Event()
        self.skip = 0

    def start(self):
        """Starts sampling every 100 ms and returns once the first sample is
        in (nvidia-smi takes a moment to start), so that the timed region
        that follows is covered from its beginning."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            self.first.wait(timeout=5.0)
            self.skip = len(self.lines)  # samples before the timed region
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self.first.set()

    def stop(self) -> dict:
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        mhz, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[self.skip:] or self.lines
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                maxes.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(mhz) if mhz else None,
                "sm_max_mhz": max(maxes) if maxes else None,
                "reasons": sorted(reasons), "samples": len(mhz)}


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def step_seeds(rank: int, world: int) -> list:
    return shard_units(list(range(IMAGES_PER_STEP * world)), rank, world)


def make_workload(rank: int, world: int):
    """This rank's share of the step's images (RGB only; covers are chosen
    by select_blocks at the probe's quantizer)."""
    from jpxl_gb300 import synth

    return [synth.synthetic_rgb(W, H, seed=1000 + s, bits=BITS) for s in step_seeds(rank, world)]


def oracle_cover(rgb, gs):
    """The restatement's select_blocks (the reference arm's cover)."""
    from oracle import loader

    rc, cover, _ = loader.select_blocks(rgb, global_scale=gs, gaborish=True)
    assert rc == 0
    return cover


def cpu_probe(rgb, cover, np, full=False):
    """The CPU restatement's probe on one image (encode, render at depth, score);
    with `full`, also its plan and rendered planes."""
    import jpxl_gb300 as jg
    from oracle import loader

    h, w = rgb.shape[:2]
    hf = np.ones(cover.shape, np.uint32)
    sh = np.full(cover.shape, 7, np.uint8)
    rc, plan = loader.encode(rgb, cover, hf, global_scale=GLOBAL_SCALE, gaborish=True)
    assert rc == 0
    rc, lin = loader.reconstruct(w, h, cover, hf, sh, plan, global_scale=GLOBAL_SCALE,
                                 gaborish=True, epf_iters=3, out_kind=3, bits=BITS)
    assert rc == 0
    src = jg.srgb_to_linear_planes(rgb, BITS)
    score = loader.ssim2(src, lin)[0]
    return (plan, lin, score) if full else score


def at_depth_f64(lin, np, bits=BITS):
    """The f64 truth of the output depth round trip: round(linear_to_srgb(x)
    * max) clamped, back through srgb_to_linear, all in f64."""
    mx = float((1 << bits) - 1)
    a = np.abs(lin)
    e = np.where(a <= 0.0031308, 12.92 * a, 1.055 * np.power(a, 1 / 2.4) - 0.055)
    e = np.where(lin < 0, -e, e)
    lvl = np.clip(np.round(e * mx), 0, mx) / mx
    return np.where(lvl <= 0.04045, lvl / 12.92, np.power((lvl + 0.055) / 1.055, 2.4))


def _mismatches(a, b, np):
    d = a.astype(np.int64) - b.astype(np.int64)
    return {"adjacent": int(np.count_nonzero(np.abs(d) == 1)),
            "other": int(np.count_nonzero(np.abs(d) > 1))}


def gpu_parity(ctx, rgb, cover, np):
    """Every mode's errors on one full-size image: against the CPU restatement
    of the reference (plan, pixels at depth, score) and against the FP64
    truth (linear pixels, score).  Also times the restatement's probe on that
    image as the single-thread CPU baseline."""
    import jpxl_gb300 as jg
    from oracle import loader

    h, w = rgb.shape[:2]
    hf = np.ones(cover.shape, np.uint32)
    sh = np.full(cover.shape, 7, np.uint8)
    t0 = time.perf_counter()
    plan_c, lin_c, score_c = cpu_probe(rgb, cover, np, full=True)
    cpu_s = time.perf_counter() - t0
    kw = dict(global_scale=GLOBAL_SCALE, gaborish=True, epf_iters=3)
    rc, truth_lin = loader.fp64_reconstruct(w, h, cover, hf, sh, plan_c, out_kind=1, **kw)
    assert rc == 0
    src = jg.srgb_to_linear_planes(rgb, BITS)
    truth_score = loader.fp64_ssim2(src, at_depth_f64(truth_lin, np))[0]
    layout = jg.Layout(ctx, w, h, cover, 1, 7)
    ref = jg.PrecomputedReference(ctx, src)
    out = {"sample": (f"image 0 of the step ({w}x{h}); 'oracle' = the CPU restatement of the "
                      "reference's arithmetic, 'fp64' = the same algorithm in f64 throughout "
                      "(render of the reference's plan; its score at 16-bit depth)"),
           "fp64_truth_score": truth_score,
           "oracle_score": score_c,
           "oracle_score_vs_fp64": abs(score_c - truth_score)}
    ref_plan = layout.empty_plan()
    ref_plan.qcoeff[...] = plan_c["qcoeff"]
    ref_plan.lf[...] = plan_c["lf"]
    ref_plan.cfl_x[...] = plan_c["cfl_x"]
    ref_plan.cfl_b[...] = plan_c["cfl_b"]
    ref_plan.lf_factors = plan_c["lf_factors"]
    plan32 = None
    for prec in PRECISIONS:
        req = jg.EncodeRequest.with_global_scale(GLOBAL_SCALE, gaborish=True, epf_iters=3,
                                                 precision=prec)
        plan = ctx.encode_transform(layout, rgb, req)
        if prec == "fp32":
            plan32 = plan
        # pixels: this mode's render of the reference's plan
        renderer = jg.PlanRenderer(ctx)
        lin = renderer.render(layout, ref_plan, req, out="linear_at_depth", bits=BITS)
        linear = renderer.render(layout, ref_plan, req, out="linear").astype(np.float64)
        score = ctx.probe(layout, ref, rgb, req)
        err = np.abs(linear - truth_lin)
        o = {
            "qcoeff_mismatches": _mismatches(plan.qcoeff, plan_c["qcoeff"], np),
            "lf_mismatches": _mismatches(plan.lf, plan_c["lf"], np),
            "cfl_mismatches": int(np.count_nonzero(plan.cfl_x != plan_c["cfl_x"]) +
                                  np.count_nonzero(plan.cfl_b != plan_c["cfl_b"])),
            "pixel_max_abs": float(np.max(np.abs(lin.astype(np.float64) - lin_c))),
            # linear-at-depth values are one per 16-bit level
            "dn_mismatches": int(np.count_nonzero(lin != lin_c)),
            "score": score,
            "score_abs_diff": float(abs(score - score_c)),
            "vs_fp64": {"pixel_max_abs": float(err.max()),
                        "pixel_rmse": float(np.sqrt(np.mean(err ** 2))),
                        "score_abs_diff": float(abs(score - truth_score))},
        }
        if prec != "fp32":
            o["qcoeff_mismatches_vs_fp32"] = _mismatches(plan.qcoeff, plan32.qcoeff, np)
        out[prec] = o
    ref.close()
    layout.close()
    return out, w * h / cpu_s / 1e6


def run_reference(args):
    """The CPU arm: the restatement of the reference on all host threads, one
    full-size image of the workload per thread per step."""
    import concurrent.futures

    import numpy as np

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import loader

    from jpxl_gb300 import synth

    loader.build()
    threads = os.cpu_count() or 1
    pool = concurrent.futures.ThreadPoolExecutor(max_workers=threads)
    # The step's images (the GPU arm's seeds, cycled), with the restatement's
    # own covers chosen before the timed region.
    seeds = [1000 + (i % IMAGES_PER_STEP) for i in range(threads)]
    uniq = sorted(set(seeds))
    base = dict(zip(uniq, pool.map(lambda s: synth.synthetic_rgb(W, H, seed=s, bits=BITS), uniq)))
    covers = dict(zip(uniq, pool.map(lambda s: oracle_cover(base[s], GLOBAL_SCALE), uniq)))
    images = [(base[s], covers[s]) for s in seeds]

    def step():
        list(pool.map(lambda t: cpu_probe(t[0], t[1], np), images))

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    mpix = W * H * threads * args.steps / 1e6
    value = mpix / dt
    sample = (f"{threads} concurrent {W}x{H} RGB16 probes per step (the GPU arm's images, "
              f"cycled), one per host thread; the C++ restatement of the reference, -O3")
    print(json.dumps({
        "impl": "reference", "metric": "probe MPix/s (encode+reconstruct+SSIMULACRA2)",
        "value": round(value, 4), "unit": "MPix/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "images_per_step": threads,
                                         "width": W, "height": H, "bits": BITS,
                                         "global_scale": GLOBAL_SCALE},
        "cpu_baseline": {"value": round(value, 4), "unit": "MPix/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "MPix/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


SEARCH_IMAGES = 64
SEARCH_CANDIDATES = (16000, 22000, 30000, 40000, 52000, 68000, 90000, 120000)
SEARCH_THRESHOLD = 85.0


def search_workload(np):
    """64 RGB8 frames of uneven sizes, w ~ U[256, 3840], h ~ U[256, 2160], cut
    at seeded offsets from four seeded 3840x2160 generator images."""
    from jpxl_gb300 import synth

    masters = [synth.synthetic_rgb(3840, 2160, seed=9000 + m, bits=8) for m in range(4)]
    rng = np.random.default_rng(2024)
    frames = []
    for i in range(SEARCH_IMAGES):
        w, h = int(rng.integers(256, 3841)), int(rng.integers(256, 2161))
        x0, y0 = int(rng.integers(0, 3840 - w + 1)), int(rng.integers(0, 2160 - h + 1))
        rgb = np.ascontiguousarray(masters[i % 4][y0:y0 + h, x0:x0 + w])
        frames.append(rgb)
    return frames


def run_search(ctx, torch, np, steps, precisions):
    """The batched quality search: every frame x every candidate quantizer as
    one graph launch of 512 probes; the chosen quantizer per frame is the
    coarsest whose score reaches the threshold.  The launch shape comes from
    the autotuner (jpxl_gb300.tune, on the headline precision's batch);
    timed per precision."""
    import jpxl_gb300 as jg

    frames = search_workload(np)
    keep, slots = [], []
    for rgb in frames:
        h, w = rgb.shape[:2]
        ref = jg.PrecomputedReference(ctx, jg.srgb_to_linear_planes(rgb, 8))
        dev = torch.from_numpy(rgb).cuda()
        keep.append((None, ref, dev))
        for gs in SEARCH_CANDIDATES:
            # Each candidate quantizer gets its own cover, as the reference's
            # plan build selects one per probe (lib.rs:555 -> :804).
            req = jg.EncodeRequest.with_global_scale(gs, gaborish=True, epf_iters=3)
            layout = jg.Layout(ctx, w, h, jg.select_blocks(ctx, rgb, req), 1, 7)
            keep.append((layout, None, None))
            slots.append((layout, ref, dev, gs))
    torch.cuda.synchronize()
    px = sum(rgb.shape[0] * rgb.shape[1] for rgb in frames) * len(SEARCH_CANDIDATES)
    result = {
        "workload": (f"{len(frames)} RGB8 frames of uneven sizes (w 256-3840, h 256-2160) x "
                     f"{len(SEARCH_CANDIDATES)} candidate global scales = {len(slots)} probes "
                     "(encode, render at depth, SSIMULACRA2) as one CUDA graph launch; each "
                     "probe's cover from select_blocks at its quantizer"),
        "unit": "MPix/s (rendered+scored)", "steps": steps,
        "threshold": SEARCH_THRESHOLD}
    stream = torch.cuda.current_stream()

    def items_for(prec):
        return [jg.BatchItem(layout, ref, dev.data_ptr(), 8,
                             jg.EncodeRequest.with_global_scale(gs, gaborish=True, epf_iters=3,
                                                                precision=prec))
                for layout, ref, dev, gs in slots]

    # The batch's launch shape (lanes, and the tensor-core kernels' CTAs per
    # SM) from the autotuner, tuned on the headline precision's batch; the
    # cache goes to a scratch file, each run tunes afresh.
    from jpxl_gb300 import tune
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        tuned = tune.tune_batch(ctx, items_for(precisions[0]), precision=precisions[0],
                                device=torch.cuda.get_device_name(), lanes=(2, 4, 8),
                                tc_ctas=None if precisions[0] == "fp32" else (2, 4),
                                reps=2, warmup=1, path=Path(td) / "tune.json")
    result["tuned"] = tuned
    result["lanes"] = tuned["lanes"]
    previous_ctas = tune.set_tc_ctas_per_sm(ctx.lib, tuned["tc_ctas_per_sm"])
    for prec in precisions:
        items = items_for(prec)
        batch = jg.BatchProbe(ctx, items, lanes=tuned["lanes"])
        scores = torch.zeros(len(items), dtype=torch.float64, device="cuda")
        for _ in range(2):
            batch.run_device(scores.data_ptr())
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            batch.run_device(scores.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        sc = scores.cpu().numpy().reshape(len(frames), len(SEARCH_CANDIDATES))
        chosen = []
        for row in sc:
            ok = [gs for gs, v in zip(SEARCH_CANDIDATES, row) if v >= SEARCH_THRESHOLD]
            chosen.append(min(ok) if ok else None)
        batch.close()
        result[prec] = {
            "value": round(px / (ms / 1e3) / 1e6, 2), "ms_per_batch": round(ms, 2),
            "frames_meeting_threshold": sum(c is not None for c in chosen),
            "chosen_global_scale": {str(gs): chosen.count(gs) for gs in SEARCH_CANDIDATES}}
    tune.set_tc_ctas_per_sm(ctx.lib, previous_ctas)
    result["value"] = result[precisions[0]]["value"]
    result["navigate"] = run_navigate(ctx, frames, [(ref, dev) for _, ref, dev in keep
                                                    if ref is not None], np)
    for layout, ref, _ in keep:
        if ref is not None:
            ref.close()
        if layout is not None:
            layout.close()
    return result


def run_navigate(ctx, frames, refs_devs, np):
    """The quality controller's own search (jpxl_gb300.quality: the baseline
    solve of search_frame_perceptual, Balanced budget) over the same frames
    toward the same threshold, every frame starting at global scale 40000:
    the frames navigate in lockstep, one jpxlg batch per round.  Timed on
    the host clock (cover selection, batch creation and every round)."""
    from jpxl_gb300 import quality as q

    sframes = [q.SearchFrame(rgb, dev.data_ptr(), ref, 8)
               for rgb, (ref, dev) in zip(frames, refs_devs)]
    starts = [q.rung_for_global_scale(40000)] * len(frames)
    t0 = time.perf_counter()
    prober = q.BatchedProber(ctx, sframes)
    outs = q.search(prober, starts, SEARCH_THRESHOLD, "balanced",
                    quant_lf=prober.request.quant_lf)
    sec = time.perf_counter() - t0
    px = sum(rgb.shape[0] * rgb.shape[1] * len(o.probes) for rgb, o in zip(frames, outs))
    statuses = {}
    for o in outs:
        statuses[o.status] = statuses.get(o.status, 0) + 1
    gs = sorted(o.quantizer.global_scale for o in outs)
    return {"workload": f"{len(frames)} frames, target {SEARCH_THRESHOLD}, Balanced budget, "
                        "start at global scale 40000",
            "ms": round(sec * 1e3, 1), "rounds": prober.batches, "probes": prober.probes,
            "probes_per_frame": round(prober.probes / len(frames), 2),
            "frames_per_s": round(len(frames) / sec, 2),
            "probed_mpix_s": round(px / sec / 1e6, 2),
            "frames_meeting_target": sum(o.score >= SEARCH_THRESHOLD for o in outs),
            "statuses": statuses,
            "chosen_global_scale": {"min": gs[0], "median": gs[len(gs) // 2], "max": gs[-1]}}


SCORING_ORIGINALS = 2
SCORING_SCALES_PER_ORIGINAL = 16
SW, SH = 4096, 3072


def run_scoring(ctx, torch, np, steps):
    """SSIMULACRA2 on 32 pairs of 4096x3072 RGB8: an original from the
    generator against its VarDCT reconstruction (select_blocks cover, CfL,
    Gaborish, 3-step EPF, 8-bit sRGB) at a seeded global scale in
    [20000, 80000].  Two figures: candidate side against precomputed
    references (the evaluator's pattern; device-resident, CUDA events), and
    score_pair end to end (both sides, host-resident linear planes in, score
    out, wall clock)."""
    import ctypes as C

    import jpxl_gb300 as jg
    from jpxl_gb300 import synth

    rng = np.random.default_rng(3100)
    pairs, refs, host = [], [], []
    for o in range(SCORING_ORIGINALS):
        rgb = synth.synthetic_rgb(SW, SH, seed=3100 + o, bits=8)
        src = jg.srgb_to_linear_planes(rgb, 8)
        ref = jg.PrecomputedReference(ctx, src)
        refs.append(ref)
        for _ in range(SCORING_SCALES_PER_ORIGINAL):
            gs = int(rng.integers(20000, 80001))
            req = jg.EncodeRequest.with_global_scale(gs, gaborish=True, epf_iters=3)
            layout = jg.Layout(ctx, SW, SH, jg.select_blocks(ctx, rgb, req), 1, 7)
            plan = ctx.encode_transform(layout, rgb, req)
            dec = jg.PlanRenderer(ctx).render(layout, plan, req, out="srgb8")
            layout.close()
            lin = jg.srgb_to_linear_planes(dec, 8)
            pairs.append((ref, torch.from_numpy(lin).cuda()))
            if len(host) < 4:
                host.append((src, lin))
    torch.cuda.synchronize()
    out = torch.zeros(len(pairs), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

    def device_round():
        for k, (ref, cand) in enumerate(pairs):
            ctx.check(ctx.lib.jpxlg_ssim2_score(ctx.handle, ref.handle,
                                                C.c_void_p(cand.data_ptr()), jg.MEM_DEVICE,
                                                C.c_void_p(out.data_ptr() + 8 * k), None, None))

    device_round()
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        device_round()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    scores = out.cpu().numpy()
    # score_pair end to end on a few host pairs (reference side included):
    # the median of three rounds.
    jg.score_pair(ctx, *host[0])
    rounds = []
    for _ in range(3):
        t0 = time.perf_counter()
        for src, lin in host:
            jg.score_pair(ctx, src, lin)
        rounds.append((time.perf_counter() - t0) / len(host))
    pair_s = statistics.median(rounds)
    for ref in refs:
        ref.close()
    px = SW * SH
    return {"workload": (f"{len(pairs)} pairs of {SW}x{SH} RGB8 ({SCORING_ORIGINALS} generator "
                         f"originals x {SCORING_SCALES_PER_ORIGINAL} seeded global scales in "
                         "[20000, 80000]); source against its reconstruction"),
            "unit": "MPix/s", "value": round(px * len(pairs) / (ms / 1e3) / 1e6, 2),
            "ms_per_pair": round(ms / len(pairs), 3),
            "score_pair_e2e_mpix_s": round(px / pair_s / 1e6, 2),
            "score_pair_e2e_ms": round(pair_s * 1e3, 2),
            "scores_range": [round(float(scores.min()), 4), round(float(scores.max()), 4)]}


def run_select(ctxs, streams, images, dev_rgb, covers, req, steps, px_total, torch, np):
    """Block selection over the step's device-resident images, one context
    per stream; checks that the device maps equal the set-up's host maps."""
    import jpxl_gb300 as jg

    maps = torch.empty((len(images), (H + 7) // 8, (W + 7) // 8), dtype=torch.uint8,
                       device="cuda")

    def select_step(contexts):
        for i in range(len(images)):
            jg.select_blocks_device(contexts[i % len(contexts)], W, H, dev_rgb[i].data_ptr(),
                                    BITS, req, maps[i].data_ptr())

    for _ in range(3):
        select_step(ctxs)
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(streams[0])
    for st in streams[1:]:
        st.wait_event(s0)
    for _ in range(steps):
        select_step(ctxs)
    for st in streams[1:]:
        done = torch.cuda.Event()
        done.record(st)
        streams[0].wait_event(done)
    s1.record(streams[0])
    torch.cuda.synchronize()
    ms = max_over_ranks(s0.elapsed_time(s1))
    if not np.array_equal(maps.cpu().numpy(), np.stack(covers)):
        raise RuntimeError("device and host block selection disagree")
    return {"value": round(px_total / (ms / 1e3) / 1e6, 2), "unit": "MPix/s",
            "ms_per_step": round(ms / steps, 3),
            "what": ("select_blocks (XYB, inverse Gaborish, DCT8/16/32 scoring, "
                     "quadtree decision) over the step's images, device-resident"),
            "sequential_fallbacks": sum(c.cover_fallbacks for c in ctxs)}


DECODE_WITH_DJXL = ("50_vardct_mixed_gray_128x128_nofilters_d1", "51_vardct_mixed_gray_128x128_nofilters_d4",
                    "52_vardct_mixed_gray_128x128_filters_d1", "53_vardct_mixed_gray_128x128_filters_d4",
                    "63_vardct_outofgamut_rgb_64x64_nofilters_d4",
                    "70_progressive_ac_gray_128x128_nofilters",
                    "71_qprogressive_ac_gray_128x128_nofilters", "72_lfframe_gray_128x128_nofilters",
                    "73_progressive_all_gray_128x128_nofilters",
                    "82_alpha_vardct_rgba_64x64_nofilters",
                    "109_orientation_transpose_vardct_rgba_64x64")
DECODE_OTHERS = ("06_gradient_300x200_lossy", "64_vardct_lfgroupseam_rgb_128x2176_nofilters_d6")
DECODE_N = 256


def _quantize_8(np, v):
    """jpxl-decode decode.rs:3498 quantize_sample at max 255."""
    s = v.astype(np.float32) * np.float32(255.0)
    r = np.where(s >= 0, np.floor(s + np.float32(0.5)), np.ceil(s - np.float32(0.5)))
    return np.where(np.isfinite(r), np.clip(r, 0, 255), 0).astype(np.int32)


def run_decode(ctx, reps, np):
    """Batched decode: the committed cjxl VarDCT streams repeated to 256,
    rendered to 8-bit sRGB by one graph launch (jpxlg_decode_batch_*), with
    the FP32 IDCTs and with the split-precision ones (square varblocks on the
    tensor cores).  The host parses every stream (headers, TOC,
    entropy-coded sections) at open; each graph launch copies the staged
    coefficients in, renders all 256 frames over the default lanes (up to
    32) and copies the 8-bit pixels back to pinned host memory.  `value` is end to end: parse
    of all streams plus one FP32 graph run, per second.  Against djxl's
    decodes (the .npy beside 11 of the 13 fixtures, quantized as
    quantize_sample does) the samples 1 DN off are counted per mode.  The
    streams are parsed on one host thread per core (open_codestreams)."""
    import jpxl_gb300 as jg

    names = DECODE_WITH_DJXL + DECODE_OTHERS
    order = [names[i % len(names)] for i in range(DECODE_N)]
    gdir = ROOT / "tests" / "golden" / "codestream"
    data = {n: (gdir / (n + ".jxl")).read_bytes() for n in names}
    workers = os.cpu_count() or 1
    t0 = time.perf_counter()
    streams = jg.open_codestreams([data[n] for n in order], workers=workers)
    parse = time.perf_counter() - t0
    px = sum(s.info["width"] * s.info["height"] for s in streams)
    refs = {n: _quantize_8(np, np.load(gdir / (n + ".npy"))[0][:, :, :3])
            for n in DECODE_WITH_DJXL}
    modes = {}
    try:
        for prec in ("fp32", "bf16x6", "bf16x3"):
            batch = jg.DecodeBatch(ctx, streams, "srgb8", precision=prec)
            try:
                for _ in range(3):
                    outs = batch.run()
                t0 = time.perf_counter()
                for _ in range(reps):
                    batch.run()
                graph = (time.perf_counter() - t0) / reps
                off = samples = worst = 0
                for n, s, out in zip(order, streams, outs):
                    if n not in refs:
                        continue
                    ref = refs[n]
                    got = out.transpose(1, 0, 2) if s.info["orientation"] == 5 else out
                    got = got[:, :, :ref.shape[2]]  # a grey image's value is plane 0
                    d = np.abs(got.astype(np.int32) - ref)
                    off += int((d > 0).sum())
                    worst = max(worst, int(d.max()))
                    samples += d.size
            finally:
                batch.close()
            modes[prec] = {"graph_ms": round(graph * 1e3, 3),
                           "graph_mpix_s": round(px / graph / 1e6, 2),
                           "vs_djxl_8bit": {"samples": samples, "samples_1dn_off": off,
                                            "max_dn": worst}}
    finally:
        for s in streams:
            s.close()
    fp = modes["fp32"]
    return {"workload": f"{DECODE_N} cjxl VarDCT streams ({len(names)} committed fixtures, "
                        "tests/golden/codestream, repeated), one graph launch to 8-bit sRGB",
            "unit": "MPix/s", "streams": DECODE_N, "pixels": px,
            "value": round(px / (parse + fp["graph_ms"] / 1e3) / 1e6, 2),
            "parse_ms": round(parse * 1e3, 3), "parse_mpix_s": round(px / parse / 1e6, 2),
            "parse_threads": workers,
            "graph_ms": fp["graph_ms"], "graph_mpix_s": fp["graph_mpix_s"],
            "vs_djxl_8bit": fp["vs_djxl_8bit"], "precision_modes": modes}


def roofline_of(stages: dict, n_img: int) -> dict:
    """The dominant kernel's achieved HBM bandwidth (its algorithmic bytes
    per launch over its CUDA-event time on one stream) as a fraction of the
    measured copy bandwidth, with its DRAM traffic per probe from the
    committed ncu capture; `parts` gives the same for the path's three parts
    (18.2, 24.2 and 60 algorithmic bytes per source pixel for the encode
    transform, the reconstruction and SSIMULACRA2)."""
    peak, peak_kind = measured_peaks()
    px = W * H * n_img
    groups = {}
    for stage, (ms, launches) in stages.items():
        g = STAGE_GROUP[stage]
        t = groups.setdefault(g, [0.0, 0])
        t[0] += ms
        t[1] += launches
    parts = {}
    for g, (ms, launches) in groups.items():
        achieved = GROUP_BYTES_PER_PX[g] * px / (ms / 1e3) / 1e9
        parts[g] = {"bytes_per_px": GROUP_BYTES_PER_PX[g], "ms_per_probe": round(ms / n_img, 4),
                    "achieved": round(achieved, 1), "frac": round(achieved / peak, 4),
                    "launches_per_probe": launches // max(n_img, 1)}
    tf = ROOT / "profiles" / "traffic_probe_2048x2048_rgb16.json"
    cap = json.loads(tf.read_text()) if tf.exists() and (W, H) == (2048, 2048) else None
    if cap:
        for g in parts:
            parts[g]["traffic_per_probe"] = cap["groups"].get(g)
    ppx = pyramid_pixels(W, H)
    kernels = {}
    for st, (name, bpp) in KERNEL_STAGES.items():
        ms, launches = stages.get(st, (0.0, 0))
        if ms <= 0 or launches <= 0:
            continue
        per_launch_bytes = bpp * ppx * n_img / launches
        achieved = bpp * ppx * n_img / (ms / 1e3) / 1e9
        kernels[st] = {"kernel": name, "bytes_per_px": bpp,
                       "launches_per_probe": launches // max(n_img, 1),
                       "us_per_launch": round(ms * 1e3 / launches, 2),
                       "algorithmic_bytes_per_launch": int(per_launch_bytes),
                       "achieved": round(achieved, 1), "frac": round(achieved / peak, 4),
                       "traffic_per_probe": (cap or {}).get("kernels", {}).get(st)}
    if not kernels:
        top = max(parts, key=lambda g: parts[g]["ms_per_probe"])
        return {"kernel": f"{top} stage", "bound": "hbm", "achieved": parts[top]["achieved"],
                "peak": peak, "unit": "GB/s", "frac": parts[top]["frac"],
                "peak_kind": peak_kind, "traffic": None, "parts": parts}
    top = max(kernels, key=lambda k: stages[k][0])
    kt = kernels[top]
    return {"kernel": f"{kt['kernel']} ({kt['launches_per_probe']} launches per probe, every "
                      "pyramid scale)",
            "bound": "hbm", "achieved": kt["achieved"], "peak": peak, "unit": "GB/s",
            "frac": kt["frac"], "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": kt["algorithmic_bytes_per_launch"],
            "traffic": (int(kt["traffic_per_probe"] / kt["launches_per_probe"])
                        if kt["traffic_per_probe"] and kt["launches_per_probe"] else None),
            "traffic_unit": "bytes per launch, the mean over one probe's launches (DRAM read + "
                            "write, ncu)",
            "traffic_basis": (cap or {}).get("source"),
            "limiter": "FP32 pipe (double-float FIR), see profiles/",
            "kernels": kernels, "parts": parts}


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    import jpxl_gb300 as jg
    from jpxl_gb300 import build

    build.build()
    images = make_workload(rank, world)
    # One context per stream: images alternate over the streams so that the
    # small launches of one probe overlap the work of another.  Dedicated
    # torch streams carry both the library's work and the timing events (the
    # default stream's handle is 0, which the library reads as "own stream").
    nstreams = max(1, args.streams)
    ctxs, streams = [], []
    for _ in range(nstreams):
        c = jg.Context(local)
        st = torch.cuda.Stream()
        c.set_stream(st.cuda_stream)
        if c.stream != st.cuda_stream:
            raise RuntimeError("the library did not adopt the timing stream")
        ctxs.append(c)
        streams.append(st)
    ctx = ctxs[0]
    torch.cuda.set_stream(streams[0])
    reqs = {p: jg.EncodeRequest.with_global_scale(GLOBAL_SCALE, gaborish=True, epf_iters=3,
                                                  precision=p) for p in PRECISIONS}
    req = reqs[args.precision]
    layouts, refs, dev_rgb, host_rgb, covers = [], [], [], [], []
    for rgb in images:
        # The probe's cover is the encoder's own choice at this quantizer.
        covers.append(jg.select_blocks(ctx, rgb, reqs["fp32"], BITS))
        layouts.append(jg.Layout(ctx, W, H, covers[-1], 1, 7))
        src = torch.from_numpy(jg.srgb_to_linear_planes(rgb, BITS)).cuda()
        refs.append(jg.PrecomputedReference(ctx, device_ptr=src.data_ptr(), width=W, height=H))
        torch.cuda.synchronize()
        del src
        t = torch.from_numpy(rgb.view(np.int16)).cuda()
        dev_rgb.append(t)
        pinned = torch.empty(rgb.shape, dtype=torch.int16, pin_memory=True)
        pinned.copy_(torch.from_numpy(rgb.view(np.int16)))
        host_rgb.append(pinned)
    scores = torch.zeros(len(images), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for c in ctxs:
        c.synchronize()

    def device_step(contexts, r):
        for i in range(len(images)):
            contexts[i % len(contexts)].probe_device(layouts[i], refs[i], dev_rgb[i].data_ptr(),
                                                     BITS, r, scores.data_ptr() + 8 * i)

    def timed(r, steps, sampler=None):
        for _ in range(max(args.warmup, 3)):
            device_step(ctxs, r)
        torch.cuda.synchronize()
        if sampler:
            sampler.start()
        launches0 = sum(c.launches for c in ctxs)
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(streams[0])
        for st in streams[1:]:
            st.wait_event(e0)
        for _ in range(steps):
            device_step(ctxs, r)
        for st in streams[1:]:
            done = torch.cuda.Event()
            done.record(st)
            streams[0].wait_event(done)
        e1.record(streams[0])
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1)
        launches = sum(c.launches for c in ctxs) - launches0
        return max_over_ranks(ms), launches

    def stage_breakdown(r, steps):
        ctx.stage_times()  # reset
        ctx.stage_timing(True)
        for _ in range(steps):
            device_step([ctx], r)
        ctx.synchronize()
        st = ctx.stage_times()
        ctx.stage_timing(False)
        return st

    px_per_step = W * H * len(images) * world
    # The headline mode, timed with the clock sampler running.
    sampler = ClockSampler(local)
    ms_max, launches = timed(req, args.steps, sampler)
    clocks = sampler.stop()
    px_total = px_per_step * args.steps
    value = px_total / (ms_max / 1e3) / 1e6
    head_scores = scores.cpu().numpy().copy()
    # Every precision mode on the same inputs, and each one's stage times.
    modes, stage_sets = {}, {}
    mode_list = [p for p in PRECISIONS if p in args.modes.split(",") or p == args.precision]
    for p in mode_list:
        if p == args.precision:
            ms_p, p_scores = ms_max, head_scores
        else:
            ms_p, _ = timed(reqs[p], args.steps)
            p_scores = scores.cpu().numpy().copy()
        stage_sets[p] = stage_breakdown(reqs[p], args.steps)
        dct_ms = (stage_sets[p]["fdct_luma"][0] + stage_sets[p]["render_varblocks"][0]) / \
            (args.steps * len(images))
        modes[p] = {"value": round(px_total / (ms_p / 1e3) / 1e6, 2),
                    "ms_per_step": round(ms_p / args.steps, 3),
                    "dct_stages_ms_per_image": round(dct_ms, 4),
                    "stages_ms": {k: round(v[0] / args.steps, 4)
                                  for k, v in stage_sets[p].items()},
                    "scores": [round(float(x), 6) for x in p_scores]}
    for p in mode_list:
        if "fp32" not in modes:
            break
        modes[p]["vs_fp32"] = round(modes[p]["value"] / modes["fp32"]["value"], 4)
        modes[p]["dct_stages_vs_fp32"] = round(
            modes["fp32"]["dct_stages_ms_per_image"] / modes[p]["dct_stages_ms_per_image"], 3)
    stages = stage_sets[args.precision]

    # Block selection (the plan build's first stage) over the same images,
    # device-resident, one context per stream as above.
    select = None if args.no_select else run_select(
        ctxs, streams, images, dev_rgb, covers, reqs["fp32"], args.steps, px_total, torch, np)

    # e2e through the C ABI with pinned host buffers: host threads, each with
    # its own context, probing their share of the images (host mode copies
    # the image in and the score out, and returns when the score is in
    # place).  By default the same contexts (and as many threads) as the
    # device-timed run.
    host_scores = [None] * len(images)
    n_e2e = max(1, min(args.e2e_threads, len(images)))
    e2e_ctxs = list(ctxs[:n_e2e])
    while len(e2e_ctxs) < n_e2e:
        e2e_ctxs.append(jg.Context(local))

    def host_worker(t, steps):
        c = e2e_ctxs[t]
        for _ in range(steps):
            for i in range(t, len(images), n_e2e):
                host_scores[i] = c.probe(layouts[i], refs[i], host_rgb[i].numpy().view(np.uint16),
                                         req, BITS)

    def host_step(steps):
        threads = [threading.Thread(target=host_worker, args=(t, steps)) for t in range(n_e2e)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()

    host_step(max(args.warmup, 3))
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    host_step(args.steps)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = px_total / e2e_s / 1e6
    if not np.allclose(head_scores, host_scores):
        raise RuntimeError(f"device and host probes disagree: {head_scores} {host_scores}")

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    roofline = roofline_of(stages, len(images) * args.steps)
    decode = None if args.no_decode else run_decode(ctx, 20, np)
    # Parity of every mode on image 0 at full size (the oracle's probe on it
    # is also the single-thread CPU baseline).
    cpu_value, parity = None, None
    if not args.no_cpu:
        parity, cpu_value = gpu_parity(ctx, images[0], covers[0], np)
    scoring = None if args.no_scoring else run_scoring(ctx, torch, np, 3)
    search = None if args.no_search else run_search(
        ctx, torch, np, 3, (args.precision,) + tuple(p for p in ("fp32",) if p != args.precision))

    line = {
        "metric": "probe MPix/s (encode+reconstruct+SSIMULACRA2)",
        "value": round(value, 2), "unit": "MPix/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(ms_max / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "fp32" else f"f32 ({args.precision} DCTs)",
        "precision": args.precision,
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "images_per_step": IMAGES_PER_STEP, "width": W,
                   "height": H, "bits": BITS, "global_scale": GLOBAL_SCALE,
                   "cover": ("select_blocks at global_scale 40000 (DCT8/16/32 quadtree "
                             "rate-distortion), chosen on the GPU before the timed region"),
                   "l2": (f"inputs larger than L2: {IMAGES_PER_STEP} distinct images, "
                          f"{W * H * 6 * IMAGES_PER_STEP / 1e6:.0f} MB of RGB16 per step"),
                   "parallelism": f"replicas x{world}", "streams": nstreams},
        "precision_modes": modes,
        "stages_ms": {k: round(v[0] / args.steps, 4) for k, v in stages.items()},
        "roofline": roofline,
        "cpu_baseline": {"value": None if cpu_value is None else round(cpu_value, 4),
                         "unit": "MPix/s", "cores": 1, "kind": "port",
                         "sample": (f"image 0 of the step ({W}x{H} RGB16), the full probe "
                                    "(encode, render at depth, score) on one thread; the C++ "
                                    "restatement of the reference, -O3")},
        "e2e": {"value": round(e2e, 2), "unit": "MPix/s",
                "h2d_bytes_per_step": int(sum(r.nbytes for r in images)),
                "d2h_bytes_per_step": 8 * len(images), "host_threads": n_e2e},
        "parity": parity,
        "scoring": scoring,
        "search": search,
        "select": select,
        "decode": decode,
        "gpu_launches": int(launches),
        "cfl_sequential_fallbacks": sum(c.cfl_fallbacks for c in ctxs),
        "clocks": clocks,
        "scores": [round(float(s), 6) for s in head_scores],
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16x6", choices=list(PRECISIONS),
                    help="DCT precision of the headline figure")
    ap.add_argument("--modes", default=",".join(PRECISIONS),
                    help="precision modes timed besides the headline (comma-separated)")
    # Smaller cases for profiler captures (the headline workload is the default).
    ap.add_argument("--size", type=int, default=None, help="square image side (profiling)")
    ap.add_argument("--images", type=int, default=None, help="images per step (profiling)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the parity / CPU baseline leg")
    ap.add_argument("--no-search", action="store_true",
                    help="skip the batched quality-search leg")
    ap.add_argument("--no-scoring", action="store_true",
                    help="skip the 4096x3072 scoring leg")
    ap.add_argument("--no-select", action="store_true",
                    help="skip the block-selection timing leg (covers are still selected)")
    ap.add_argument("--no-decode", action="store_true", help="skip the stream-decode leg")
    ap.add_argument("--streams", type=int, default=4,
                    help="contexts (each with its own stream) that images alternate over")
    ap.add_argument("--e2e-threads", type=int, default=4,
                    help="host threads (each with its own context) of the end-to-end leg; "
                         "4 and 8 measured alike")
    args = ap.parse_args()
    global W, H, IMAGES_PER_STEP
    if args.size:
        W = H = args.size
    if args.images:
        IMAGES_PER_STEP = args.images
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
