"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

The bar is bit-exact integer equality of point ids: window minima per
window, LLP lists, stage-3 lists and the final seed list (same order: stage-3
ids in cell order, then LLPs ascending).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cloud(F, config, n=None, w=None, h=None, tile=0, **over):
    spec, W, Ov, B, mn, seed = F.synth_config(config, tile)
    if n is not None:
        spec.n = n
    if w is not None:
        spec.x1 = spec.x0 + w
    if h is not None:
        spec.y1 = spec.y0 + h
    for k, v in over.items():
        setattr(spec, k, v)
    xyz, bb = F.synth_cloud(spec, seed)
    return xyz, bb, W, Ov, B, mn


def _run_both(F, O, ctx, xyz, bb, W, Ov, B, mn=32, policy=None, min_radius=0.1):
    """GPU path with both stage-1 algorithms (window classes, tree walk) vs the oracle."""
    pol = F.OWM_TREE_MAX_NUMBER if policy is None else policy
    cloud = ctx.cloud(xyz, bb)
    got = ctx.run(cloud, F.run_cfg(W, Ov, B, mn, pol, min_radius))
    walk = ctx.run(cloud, F.run_cfg(W, Ov, B, mn, pol, min_radius, stage1_walk=True))
    want, nllp = O.run(xyz, bb, W, Ov, B)
    cloud.close()
    np.testing.assert_array_equal(walk, got)
    return got, want, nllp


def test_small_run_matches_oracle(owm, oracle, ctx):
    xyz, bb, W, Ov, B, mn = _cloud(owm, 1, n=200_000, w=80, h=100)
    got, want, _ = _run_both(owm, oracle, ctx, xyz, bb, W, Ov, B, mn)
    assert len(want) > 0
    np.testing.assert_array_equal(got, want)


def test_config1_full_stagewise(owm, oracle, ctx):
    """Config 1 at full size: every stage equal to the oracle."""
    xyz, bb, W, Ov, B, mn = _cloud(owm, 1)
    p = owm.params(bb, xyz.shape[0], W, Ov, B)
    op = oracle.params(bb, xyz.shape[0], W, Ov, B)
    assert (p.ncols, p.nrows, p.min_num_points, p.ncols_grid, p.nrows_grid) == (
        op.ncols, op.nrows, op.min_num_points, op.ncols_grid, op.nrows_grid)
    cloud = ctx.cloud(xyz, bb)
    tree = ctx.tree(cloud, owm.OWM_TREE_MAX_NUMBER, mn)
    assert tree.check()
    info = tree.info()
    assert info.root_count == xyz.shape[0]
    z = xyz[:, 2]
    assert info.root_min_id == int(np.lexsort((np.arange(1, len(z) + 1), z))[0]) + 1
    win = ctx.stage1(tree, p)
    win_o = oracle.stage1(xyz, op)
    np.testing.assert_array_equal(win, win_o)
    llp = ctx.stage2(win, Ov)
    llp_o = oracle.stage2(win_o, Ov)
    np.testing.assert_array_equal(llp, llp_o)
    s3 = ctx.stage3(tree, p, llp)
    s3_o = oracle.stage3(xyz, op, llp_o)
    np.testing.assert_array_equal(s3, s3_o)
    got = ctx.run(cloud, owm.run_cfg(W, Ov, B, mn))
    np.testing.assert_array_equal(got, np.concatenate([s3_o, llp_o]))
    tree.close()
    cloud.close()


@pytest.mark.parametrize("overlap", [0.5, 0.8])
def test_config3_ties_holes_strips(owm, oracle, ctx, overlap):
    """Strips, holes, 1 cm z ties, odd B = 15 (cells with 1 m gaps)."""
    xyz, bb, W, _, B, mn = _cloud(owm, 3, n=2_000_000, w=400, h=400)
    assert np.unique(xyz[:, 2]).size < xyz.shape[0]  # ties really occur
    got, want, _ = _run_both(owm, oracle, ctx, xyz, bb, W, overlap, B, mn)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("policy,mn,mr", [(1, 1, 0.1), (1, 4, 0.1), (1, 16, 0.1), (1, 64, 0.1), (1, 128, 0.1),
                                          (1, 256, 0.1), (1, 3, 0.1), (1, 100, 0.1), (1, 1000, 0.1),
                                          (0, 32, 0.1), (0, 32, 0.5), (0, 32, 3.0)])
def test_tree_policies_same_result(owm, oracle, ctx, policy, mn, mr):
    xyz, bb, W, Ov, B, _ = _cloud(owm, 1, n=150_000, w=70, h=90)
    got, want, _ = _run_both(owm, oracle, ctx, xyz, bb, W, Ov, B, mn, policy, mr)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("W,Ov,B", [(9, 0.8, 15), (10, 0.5, 20), (16, 0.8, 20), (8, 0.8, 0), (10, 0.0, 20),
                                    (7, 0.3, 11), (12, 0.8, 20)])
def test_window_geometry_variants(owm, oracle, ctx, W, Ov, B):
    """Odd W (a (W-1)-wide window), odd B, B = 0 (no stage 3), overlap 0."""
    xyz, bb, _, _, _, _ = _cloud(owm, 1, n=120_000, w=60, h=75)
    got, want, _ = _run_both(owm, oracle, ctx, xyz, bb, W, Ov, B)
    np.testing.assert_array_equal(got, want)


def test_large_stage3_grid(owm, oracle, ctx):
    """2 m cells over 1100 m x 1100 m (303,601 > 2^18 cells: the multi-launch
    ordered compaction of stage 3); sparse points, so most cells hold no LLP
    and stage 3 answers about 227,000 of them."""
    xyz, bb, _, _, _, _ = _cloud(owm, 1, n=600_000, w=1100, h=1100)
    got, want, nllp = _run_both(owm, oracle, ctx, xyz, bb, 6, 0.5, 2)
    assert len(want) - nllp > 200_000
    np.testing.assert_array_equal(got, want)


def test_tiny_and_degenerate_clouds(owm, oracle, ctx):
    rng = np.random.default_rng(5)
    cases = []
    # a handful of points, windows larger than the cloud
    for n in (1, 2, 3, 17, 100):
        xyz = np.column_stack([1000 + rng.random(n) * 7, 2000 + rng.random(n) * 5, 50 + rng.random(n)])
        cases.append(xyz)
    # sparse cloud: minNumPoints == 0 (windows with no point keep the sentinel id 0)
    xyz = np.column_stack([5000 + rng.random(50) * 400, 7000 + rng.random(50) * 400, rng.random(50)])
    cases.append(xyz)
    # duplicated (x, y) positions, z ties, negative and near-zero coordinates
    base = np.column_stack([-20 + rng.random(3000) * 40, -15 + rng.random(3000) * 30, np.round(rng.random(3000), 2)])
    cases.append(np.concatenate([base, base[:500]]))
    for xyz in cases:
        bb = owm.bbox_of(xyz)
        if bb.max_x - bb.min_x < 0.01 or bb.max_y - bb.min_y < 0.01:
            continue
        # overlap 0 on the sparse cloud: many empty windows report the
        # sentinel id 0, and every valid minimum is kept (0 repeats)
        for (W, Ov, B) in ((10, 0.8, 20), (4, 0.5, 3), (6, 0.0, 10)):
            got, want, _ = _run_both(owm, oracle, ctx, xyz, bb, W, Ov, B, 4)
            np.testing.assert_array_equal(got, want)


def test_deterministic_repeat(owm, ctx):
    xyz, bb, W, Ov, B, mn = _cloud(owm, 1, n=300_000, w=100, h=120)
    cloud = ctx.cloud(xyz, bb)
    a = ctx.run(cloud, owm.run_cfg(W, Ov, B, mn))
    b = ctx.run(cloud, owm.run_cfg(W, Ov, B, mn))
    c = ctx.run_host(xyz, bb, owm.run_cfg(W, Ov, B, mn))
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)
    cloud.close()


def test_nonfinite_input_rejected(owm, ctx):
    xyz, bb, W, Ov, B, mn = _cloud(owm, 1, n=10_000, w=30, h=30)
    xyz[77, 2] = np.nan
    with pytest.raises(owm.OwmError) as e:
        ctx.run_host(xyz, bb, owm.run_cfg(W, Ov, B, mn))
    assert e.value.status == -1
    xyz[77, 2] = 100.0
    ctx.run_host(xyz, bb, owm.run_cfg(W, Ov, B, mn))  # context still usable


def test_header_bbox_narrower_than_data(owm, oracle, ctx):
    """The reference takes the bbox from the file header; points may fall
    outside it (class tables then fall back to searching)."""
    xyz, bb, W, Ov, B, mn = _cloud(owm, 1, n=150_000, w=70, h=90)
    hb = owm.Bbox(bb.min_x + 3.3, bb.min_y + 1.7, bb.max_x - 2.1, bb.max_y - 4.4)
    got, want, _ = _run_both(owm, oracle, ctx, xyz, hb, W, Ov, B, mn)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("xr,yr,W,Ov,B", [
    ((1000.0, 1100.0), (3000.0, 3080.0), 10, 0.8, 20),   # x crosses 1024: no x table, y table
    ((3000.0, 3080.0), (1000.0, 1100.0), 10, 0.8, 20),   # the same with the axes swapped
    ((4100.0, 5600.0), (8200.0, 8260.0), 2, 0.9, 5),     # 0.2 m step: about 24,000 x-table cells
])
def test_class_table_axes(owm, oracle, ctx, xr, yr, W, Ov, B):
    """Stage 1 by window classes looks a point's sub-cell up in a per-axis
    table when the axis's keys are linear over the bbox (positive, one binary
    exponent), and searches the edge arrays otherwise: one axis of each kind,
    and a table of many cells, against the oracle."""
    rng = np.random.default_rng(11)
    n = 300_000
    xyz = np.column_stack([xr[0] + rng.random(n) * (xr[1] - xr[0]), yr[0] + rng.random(n) * (yr[1] - yr[0]),
                           np.round(100 + rng.random(n) * 3, 3)])
    bb = owm.bbox_of(xyz)
    got, want, _ = _run_both(owm, oracle, ctx, xyz, bb, W, Ov, B, 32)
    assert len(want) > 0
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("policy,mn,mr", [(1, 32, 0.1), (1, 16, 0.1), (1, 128, 0.1), (0, 32, 0.4)])
def test_large_cloud_policies(owm, oracle, ctx, policy, mn, mr):
    """1.5 M points (persistent pipelined sort), both leaf policies, both stage-1 algorithms."""
    xyz, bb, W, Ov, B, _ = _cloud(owm, 1, n=1_500_000, w=240, h=310)
    got, want, _ = _run_both(owm, oracle, ctx, xyz, bb, W, Ov, B, mn, policy, mr)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("n,mn,bits", [(200_000, 32, 16), (1_500_000, 32, 18), (1_500_000, 128, 16),
                                       (5_000_000, 256, 16), (5_000_000, 4, 22)])
def test_key_width_rule(owm, ctx, n, mn, bits):
    """Morton key width: the fewest bits per axis (8..12) with at most half a
    leaf of points per finest cell; the tree stays well-formed at every width."""
    xyz, bb, _, _, _, _ = _cloud(owm, 1, n=n, w=300, h=300)
    cloud = ctx.cloud(xyz, bb)
    tree = ctx.tree(cloud, max_number=mn)
    info = tree.info()
    assert info.key_bits == bits
    assert info.root_count == n and tree.check()
    cloud.close()
