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


# Launch-shape candidates (owm_ctx_set_tuning); results never depend on them.
GATHER_BLOCKS = (128, 256, 512)
CELL_WARPS = (2, 4, 8)
WALK_PATCHES = (2, 4, 8, 16)


def _timed_median(fn, stream, reps: int) -> float:
    import torch

    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def tune_shapes_single(ctx, cloud, cfg, walk: bool = False, reps: int = 3) -> dict:
    """Launch shapes for one cloud and run config: coordinate search over the
    gather's block size, the stage-3 cell walk's warps per block and (for the
    tree-walk stage 1) the walk's window patch, each timed by owm_run on the
    device-resident cloud, every candidate's seeds checked against the first.
    Leaves the best shapes set on ctx; returns {"tuning": {...}, "ms": {...}}."""
    import torch

    import fastowm_gb300 as F

    stream = torch.cuda.ExternalStream(F.lib().owm_ctx_stream(ctx.handle))
    ref = ctx.run(cloud, cfg)
    timings = {}
    knobs = [("gather_block", GATHER_BLOCKS), ("cell_warps", CELL_WARPS)]
    if walk:
        knobs.append(("walk_patch_x", WALK_PATCHES))
    for name, values in knobs:
        best, best_ms = None, float("inf")
        for v in values:
            ctx.set_tuning(**{name: v})
            seeds = ctx.run(cloud, cfg)  # warm-up, and the exactness check
            if not np.array_equal(seeds, ref):
                raise RuntimeError(f"{name}={v}: seeds differ")
            ms = _timed_median(lambda: ctx.run(cloud, cfg), stream, reps)
            timings[f"{name}={v}"] = round(ms, 4)
            if ms < best_ms:
                best, best_ms = v, ms
        ctx.set_tuning(**{name: best})
    return {"tuning": ctx.tuning(), "ms": timings}


def tune_shapes_classes(ctx, bounds=DEFAULT_BOUNDS, tiles_per_class: int = 8, reps: int = 3, walk: bool = True,
                        config: int = 4) -> dict:
    """Launch shapes per tile size class: for each point-count band a sample
    of tiles (config 4 generator) runs one tile per owm_run, and a coordinate
    search picks the gather block, the cell-walk warps and -- for the
    tree-walk stage 1 -- the walk's window patch that minimise the band's
    total device time; every candidate's seeds are checked against the
    first's.  Returns {"bounds": [...], "classes": [{"tuning", "ms"}, ...]};
    ctx is left with its shapes from before."""
    import torch

    import fastowm_gb300 as F

    stream = torch.cuda.ExternalStream(F.lib().owm_ctx_stream(ctx.handle))
    saved = ctx.tuning()
    out, lo = [], 0
    for hi in bounds:
        tiles = _class_tiles(F, lo, min(hi, 5_000_000), tiles_per_class, config=config)
        lo = hi
        if not tiles:
            out.append(None)
            continue
        clouds = [(ctx.cloud(xyz, bb), cfg) for xyz, bb, cfg in tiles]
        knobs = [("gather_block", GATHER_BLOCKS, False), ("cell_warps", CELL_WARPS, False)]
        if walk:
            knobs.append(("walk_patch_x", WALK_PATCHES, True))
        timings = {}
        for name, values, use_walk in knobs:
            runs = [(cl, F.run_cfg(cfg.wsize, cfg.overlap, cfg.bsize, cfg.tree.max_number, stage1_walk=use_walk))
                    for cl, cfg in clouds]
            refs = [ctx.run(cl, c2) for cl, c2 in runs]
            best, best_ms = None, float("inf")
            for v in values:
                ctx.set_tuning(**{name: v})
                for (cl, c2), ref in zip(runs, refs):
                    if not np.array_equal(ctx.run(cl, c2), ref):
                        raise RuntimeError(f"{name}={v}: seeds differ")

                def all_tiles():
                    for cl, c2 in runs:
                        ctx.run(cl, c2)

                ms = _timed_median(all_tiles, stream, reps)
                timings[f"{name}={v}"] = round(ms, 4)
                if ms < best_ms:
                    best, best_ms = v, ms
            ctx.set_tuning(**{name: best})
        out.append({"tuning": ctx.tuning(), "ms": timings})
        for cl, _ in clouds:
            cl.close()
        ctx.set_tuning(**saved)
    return {"bounds": list(bounds), "classes": out}
