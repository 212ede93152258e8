"""Batched tiles and the serving loop on the GPU: every tile's seeds must be
exactly what owm_run gives for that tile alone (and what the oracle gives)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tiles(F, k, n_scale=0.05, start=0):
    """k config-4 tiles, shrunk to n_scale of their size (same densities)."""
    out = []
    for t in range(start, start + k):
        spec, W, Ov, B, mn, seed = F.synth_config(4, t)
        n0 = spec.n
        spec.n = max(2000, int(n0 * n_scale))
        side = (spec.x1 - spec.x0) * np.sqrt(spec.n / n0)
        spec.x1, spec.y1 = spec.x0 + side, spec.y0 + side
        xyz, bb = F.synth_cloud(spec, seed)
        out.append((xyz, bb, F.run_cfg(W, Ov, B, mn)))
    return out


def _alone(F, ctx, tiles):
    res = []
    for xyz, bb, cfg in tiles:
        c = ctx.cloud(xyz, bb)
        res.append(ctx.run(c, cfg))
        c.close()
    return res


def test_batch_equals_alone_and_oracle(owm, oracle, ctx):
    tiles = _tiles(owm, 24)
    # odd shapes in the same batch: tiny tile, no stage 3, overlap 0, odd W
    xyz, bb, cfg = tiles[3]
    tiles.append((xyz[:20].copy(), owm.bbox_of(xyz[:20]), owm.run_cfg(10, 0.8, 20, 32)))
    tiles.append((xyz, bb, owm.run_cfg(9, 0.8, 0, 16)))
    tiles.append((xyz, bb, owm.run_cfg(10, 0.0, 15, 64)))
    alone = _alone(owm, ctx, tiles)
    b = owm.Batch(ctx)
    got = b.run(tiles)
    for k, (g, a) in enumerate(zip(got, alone)):
        np.testing.assert_array_equal(g, a, err_msg=f"tile {k}")
    for k in (0, 5, len(tiles) - 1):
        xyz, bb, cfg = tiles[k]
        want, _ = oracle.run(xyz, bb, cfg.wsize, cfg.overlap, cfg.bsize)
        np.testing.assert_array_equal(got[k], want)
    b.close()


def test_batch_graph_replay_and_leaf_classes(owm, ctx):
    tiles = _tiles(owm, 16, start=30)
    alone = _alone(owm, ctx, tiles)
    b = owm.Batch(ctx)
    b.set_graphs(True)
    for _ in range(3):  # capture, then replay twice
        got = b.run(tiles)
        for g, a in zip(got, alone):
            np.testing.assert_array_equal(g, a)
    b.set_leaf_classes([20_000, 60_000, 1 << 40], [16, 64, 128])
    for _ in range(2):
        got = b.run(tiles)
        for g, a in zip(got, alone):
            np.testing.assert_array_equal(g, a)
    b.close()


def test_server_mix_equals_alone(owm, ctx):
    tiles = _tiles(owm, 40, start=60)
    alone = _alone(owm, ctx, tiles)
    # a budget that holds about two small batches: forces waiting and eviction
    est = 600 << 20
    srv = owm.Server(0, hbm_budget_bytes=est, max_tiles_per_batch=6, max_inflight_batches=3,
                     max_points_per_batch=1 << 22)
    tickets = [srv.submit(xyz, bb, cfg) for xyz, bb, cfg in tiles]
    lat = []
    for k, t in enumerate(tickets):
        p = owm.params(tiles[k][1], tiles[k][0].shape[0], tiles[k][2].wsize, tiles[k][2].overlap, tiles[k][2].bsize)
        seeds, ms = srv.wait(t, p.ncells + p.ngrid + 1)
        np.testing.assert_array_equal(seeds, alone[k], err_msg=f"tile {k}")
        lat.append(ms)
    st = srv.stats()
    assert st.completed == len(tiles) and st.submitted == len(tiles)
    assert st.batches >= 2 and st.peak_bytes <= est
    assert min(lat) > 0.0
    srv.close()


def test_server_rejects_tile_over_budget(owm):
    xyz, bb, cfg = _tiles(owm, 1, n_scale=1.0, start=5)[0]
    srv = owm.Server(0, hbm_budget_bytes=1 << 20)
    with pytest.raises(owm.OwmError) as e:
        srv.submit(xyz, bb, cfg)
    assert e.value.status == -2
    srv.close()


def test_batch_stage1_classes_equals_walk(owm, ctx):
    """Stage 1 of a batch by window classes (default) and by the persistent
    tree walk (any tile with stage1_walk set switches the batch) agree, tile
    by tile; ties included (config-3 style z quantisation)."""
    tiles = _tiles(owm, 20, start=90)
    walk = [(xyz, bb, owm.run_cfg(cfg.wsize, cfg.overlap, cfg.bsize, cfg.tree.max_number, stage1_walk=True))
            for xyz, bb, cfg in tiles]
    # ties: quantise z of two tiles to 1 cm
    for k in (2, 7):
        xyz, bb, cfg = tiles[k]
        q = xyz.copy()
        q[:, 2] = np.round(q[:, 2] * 100.0) / 100.0
        tiles[k] = (q, bb, cfg)
        walk[k] = (q, bb, walk[k][2])
    b = owm.Batch(ctx)
    got_cls = b.run(tiles)
    got_walk = b.run(walk)
    mixed = tiles[:-1] + walk[-1:]  # one tile asks for the walk
    got_mixed = b.run(mixed)
    for k in range(len(tiles)):
        np.testing.assert_array_equal(got_cls[k], got_walk[k], err_msg=f"tile {k}")
        np.testing.assert_array_equal(got_cls[k], got_mixed[k], err_msg=f"tile {k} (mixed)")
    b.close()
