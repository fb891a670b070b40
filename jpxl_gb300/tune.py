"""Autotuner of the batched probe's launch shape.

A batch of probes (BatchProbe, one CUDA graph) has two run-time knobs that
change its speed but not its results: how many lanes (internal contexts,
each with its own stream and workspace) the probes are spread over, and how
many persistent CTAs per SM the split-precision tensor-core kernels take
(JPXLG_TUNE_TC_CTAS_PER_SM).  `tune_batch` times every combination on the
caller's own items (each a fresh graph, warmed up, then timed over several
launches with the device synchronised around them), keeps the fastest and
caches it in a JSON file under a key made of the device, the precision and
the workload's size, so that later processes start from the tuned shape
(`tuned_shape`).  The scores do not depend on the shape: every probe runs
the same arithmetic whatever lane or grid runs it.
"""
from __future__ import annotations

import json
import os
import time
from dataclasses import dataclass
from pathlib import Path

TUNE_TC_CTAS_PER_SM = 0  # include/jpxlg.h JPXLG_TUNE_TC_CTAS_PER_SM


def cache_path() -> Path:
    """The tuning cache: $JPXLG_TUNE_CACHE, else ~/.cache/jpxl_gb300/tune.json."""
    env = os.environ.get("JPXLG_TUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "jpxl_gb300" / "tune.json"


def workload_key(device: str, precision: str, n_items: int, pixels: int) -> str:
    """Batches of the same precision whose probe count and pixel total fall in
    the same power-of-two buckets share a tuned shape."""
    return f"{device}|{precision}|n{max(n_items, 1).bit_length()}|px{max(pixels, 1).bit_length()}"


def set_tc_ctas_per_sm(lib, value: int) -> int:
    old = lib.jpxlg_tune_set(TUNE_TC_CTAS_PER_SM, int(value))
    if old < 0:
        raise ValueError(f"tc_ctas_per_sm {value} refused ({old})")
    return old


@dataclass
class Trial:
    lanes: int
    tc_ctas_per_sm: int
    ms: float


def search(time_fn, lanes=(2, 4, 6, 8), tc_ctas=(4,)) -> tuple[Trial, list[Trial]]:
    """Times time_fn(lanes, tc_ctas_per_sm) -> milliseconds for every
    combination; returns the fastest trial (the first of equal times) and
    all of them in the order they ran."""
    trials = [Trial(l, c, float(time_fn(l, c))) for c in tc_ctas for l in lanes]
    best = min(trials, key=lambda t: t.ms)
    return best, trials


def load_cache(path: Path | None = None) -> dict:
    p = path or cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def save_cache(entries: dict, path: Path | None = None) -> None:
    p = path or cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    tmp = p.with_suffix(".tmp")
    tmp.write_text(json.dumps(entries, indent=1, sort_keys=True))
    tmp.replace(p)


def tuned_shape(key: str, path: Path | None = None) -> dict | None:
    """The cached {"lanes", "tc_ctas_per_sm", "ms"} of a workload key."""
    return load_cache(path).get(key)


def tune_batch(ctx, items: list, *, precision: str, device: str = "gpu0",
               lanes=(2, 4, 6, 8), tc_ctas=None, reps: int = 3, warmup: int = 2,
               path: Path | None = None, write: bool = True) -> dict:
    """Times the batch of `items` (BatchItem) for every lanes x CTAs-per-SM
    combination, caches and returns the fastest as {"key", "lanes",
    "tc_ctas_per_sm", "ms", "trials"}.  The CTAs-per-SM knob is swept only
    for the split precisions (the FP32 kernels do not read it); it is left at
    its previous value afterwards."""
    from . import BatchProbe

    if tc_ctas is None:
        tc_ctas = (2, 3, 4) if precision != "fp32" else (ctx.lib.jpxlg_tune_get(TUNE_TC_CTAS_PER_SM),)
    pixels = sum(it.layout.width * it.layout.height for it in items)
    key = workload_key(device, precision, len(items), pixels)
    previous = ctx.lib.jpxlg_tune_get(TUNE_TC_CTAS_PER_SM)

    def time_fn(nl: int, nc: int) -> float:
        set_tc_ctas_per_sm(ctx.lib, nc)
        batch = BatchProbe(ctx, items, lanes=nl)
        try:
            for _ in range(warmup):
                batch.run()
            ctx.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                batch.run()
            return (time.perf_counter() - t0) * 1e3 / reps
        finally:
            batch.close()

    try:
        best, trials = search(time_fn, lanes, tc_ctas)
    finally:
        set_tc_ctas_per_sm(ctx.lib, previous)
    entry = {"lanes": best.lanes, "tc_ctas_per_sm": best.tc_ctas_per_sm, "ms": round(best.ms, 3)}
    if write:
        cache = load_cache(path)
        cache[key] = entry
        save_cache(cache, path)
    return {"key": key, **entry,
            "trials": [{"lanes": t.lanes, "tc_ctas_per_sm": t.tc_ctas_per_sm,
                        "ms": round(t.ms, 3)} for t in trials]}
