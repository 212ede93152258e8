"""Launch shapes (owm_ctx_set_tuning) change only speed: the stage-1 walk's
window patch, the stage-3 cell walk's warps per block and the gather's block
size all give the same seeds, for one cloud and for a batch, and the
autotuner's picks are exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cloud(F, n=250_000, w=90.0, h=110.0, B=6):
    spec, W, Ov, _, mn, seed = F.synth_config(1)
    spec.n, spec.x1, spec.y1 = n, spec.x0 + w, spec.y0 + h
    xyz, bb = F.synth_cloud(spec, seed)
    return xyz, bb, W, Ov, B, mn


def test_shapes_give_identical_seeds(owm, oracle):
    ctx = owm.Context(0)
    assert ctx.tuning() == {"walk_patch_x": 4, "cell_warps": 4, "gather_block": 256}
    xyz, bb, W, Ov, B, mn = _cloud(owm)
    want, _ = oracle.run(xyz, bb, W, Ov, B)
    cloud = ctx.cloud(xyz, bb)
    for walk in (False, True):
        cfg = owm.run_cfg(W, Ov, B, mn, stage1_walk=walk)
        for patch in (1, 2, 8, 32):
            for warps in (2, 8):
                for gb in (128, 512):
                    ctx.set_tuning(walk_patch_x=patch, cell_warps=warps, gather_block=gb)
                    np.testing.assert_array_equal(ctx.run(cloud, cfg), want)
    # owm_stage1 (the walk) and owm_stage3 with the last shapes
    tree = ctx.tree(cloud, owm.OWM_TREE_MAX_NUMBER, mn)
    p = owm.params(bb, xyz.shape[0], W, Ov, B)
    op = oracle.params(bb, xyz.shape[0], W, Ov, B)
    np.testing.assert_array_equal(ctx.stage1(tree, p), oracle.stage1(xyz, op))
    llp = oracle.stage2(oracle.stage1(xyz, op), Ov)
    np.testing.assert_array_equal(ctx.stage3(tree, p, llp), oracle.stage3(xyz, op, llp))
    tree.close()
    cloud.close()
    ctx.close()


def test_shapes_rejected_and_kept(owm):
    ctx = owm.Context(0)
    for bad in ({"walk_patch_x": 3}, {"walk_patch_x": 64}, {"cell_warps": 3}, {"cell_warps": 16},
                {"gather_block": 64}, {"gather_block": 1024}):
        with pytest.raises(owm.OwmError):
            ctx.set_tuning(**bad)
    ctx.set_tuning(cell_warps=8)
    ctx.set_tuning(gather_block=128)  # 0 fields keep the others
    assert ctx.tuning() == {"walk_patch_x": 4, "cell_warps": 8, "gather_block": 128}
    ctx.close()


def test_batch_shapes_identical(owm):
    ctx = owm.Context(0)
    tiles = []
    for t in range(6):
        spec, W, Ov, B, mn, seed = owm.synth_config(4, t)
        spec.n = min(spec.n, 120_000)
        xyz, bb = owm.synth_cloud(spec, seed)
        tiles.append((xyz, bb, owm.run_cfg(W, Ov, B, mn, stage1_walk=(t % 2 == 1))))
    batch = owm.Batch(ctx)
    ref = batch.run(tiles)
    for patch, warps, gb in ((1, 2, 128), (32, 8, 512), (8, 4, 256)):
        ctx.set_tuning(walk_patch_x=patch, cell_warps=warps, gather_block=gb)
        got = batch.run(tiles)
        for a, b in zip(got, ref):
            np.testing.assert_array_equal(a, b)
    batch.close()
    ctx.close()


def test_autotuner_shapes_exact(owm):
    from fastowm_gb300 import autotune

    ctx = owm.Context(0)
    xyz, bb, W, Ov, B, mn = _cloud(owm, n=150_000, w=70.0, h=80.0)
    cloud = ctx.cloud(xyz, bb)
    cfg = owm.run_cfg(W, Ov, B, mn, stage1_walk=True)
    ref = ctx.run(cloud, cfg)
    r = autotune.tune_shapes_single(ctx, cloud, cfg, walk=True, reps=1)
    assert set(r["tuning"]) == {"walk_patch_x", "cell_warps", "gather_block"}
    assert len(r["ms"]) == len(autotune.GATHER_BLOCKS) + len(autotune.CELL_WARPS) + len(autotune.WALK_PATCHES)
    np.testing.assert_array_equal(ctx.run(cloud, cfg), ref)
    cloud.close()
    classes = autotune.tune_shapes_classes(ctx, bounds=(200_000, 1 << 40), tiles_per_class=2, reps=1)
    assert len(classes["classes"]) == 2 and all(c is None or "tuning" in c for c in classes["classes"])
    ctx.close()
