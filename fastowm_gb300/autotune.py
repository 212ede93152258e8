"""Autotuner for batched tiles: picks the leaf size (the reference's -s
maxNumber knob, CPP-TBB-CPU/application/owm_optim3.cpp:27) per tile size
class by timing real batched runs on the device.

Size classes are point-count bands; for each band a sample of tiles from the
batched-tiles generator (config 4) is run with every candidate leaf size and
the fastest is kept.  Results are exact for every choice (the leaf size only
changes the hierarchy), so tuning is purely a speed decision.
"""
from __future__ import annotations

import json
import time
from pathlib import Path

import numpy as np

DEFAULT_BOUNDS = (150_000, 500_000, 1_000_000, 1 << 40)
DEFAULT_LEAVES = (16, 32, 64, 128, 256)


def _class_tiles(F, lo: int, hi: int, want: int, config: int = 4, start: int = 0, limit: int = 4096):
    tiles = []
    for t in range(start, start + limit):
        spec, W, Ov, B, mn, seed = F.synth_config(config, t)
        if lo < spec.n <= hi:
            xyz, bb = F.synth_cloud(spec, seed)
            tiles.append((xyz, bb, F.run_cfg(W, Ov, B, mn)))
            if len(tiles) >= want:
                break
    return tiles


def tune_leaf_classes(ctx, bounds=DEFAULT_BOUNDS, leaves=DEFAULT_LEAVES, tiles_per_class: int = 6, reps: int = 3,
                      cache: str | Path | None = None) -> dict:
    """Returns {"bounds": [...], "leaves": [...], "ms": {...}} and, if cache is
    given, stores it there (JSON)."""
    import fastowm_gb300 as F

    batch = F.Batch(ctx)
    chosen, timings = [], {}
    lo = 0
    for hi in bounds:
        tiles = _class_tiles(F, lo, min(hi, 5_000_000), tiles_per_class)
        best, best_ms = leaves[1], float("inf")
        for leaf in leaves:
            batch.set_leaf_classes([1 << 40], [leaf])
            batch.run(tiles)  # warm-up (allocations)
            ts = []
            for _ in range(reps):
                t0 = time.perf_counter()
                batch.run(tiles)
                ts.append(1e3 * (time.perf_counter() - t0))
            ms = float(np.median(ts))
            timings[f"{lo}-{hi}:{leaf}"] = round(ms, 3)
            if ms < best_ms:
                best, best_ms = leaf, ms
        chosen.append(best)
        lo = hi
    batch.close()
    out = {"bounds": list(bounds), "leaves": chosen, "ms": timings}
    if cache:
        Path(cache).write_text(json.dumps(out, indent=1))
    return out


def apply(batch, tuned: dict) -> None:
    batch.set_leaf_classes(tuned["bounds"], tuned["leaves"])


def tune_leaf_single(ctx, cloud, make_cfg, leaves=(32, 64, 128, 256), reps: int = 3) -> dict:
    """Leaf size for one cloud: times owm_run on the device-resident cloud
    with each candidate (make_cfg(leaf) -> RunCfg) and returns
    {"leaf": best, "ms": {leaf: median ms}}.  Every choice gives the same
    seeds; the tuner checks that too."""
    import torch

    import fastowm_gb300 as F

    stream = torch.cuda.ExternalStream(F.lib().owm_ctx_stream(ctx.handle))
    timings, ref = {}, None
    for leaf in leaves:
        cfg = make_cfg(leaf)
        seeds = ctx.run(cloud, cfg)  # warm-up (buffers)
        if ref is None:
            ref = seeds
        elif not np.array_equal(seeds, ref):
            raise RuntimeError(f"leaf {leaf}: seeds differ from leaf {leaves[0]}")
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.run(cloud, cfg)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        timings[leaf] = round(float(np.median(ts)), 3)
    best = min(timings, key=timings.get)
    return {"leaf": best, "ms": timings}
