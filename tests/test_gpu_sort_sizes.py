"""The build's radix sort at sizes that reach every path of its ranked pass.

Sorts of at least 64 tiles of 4096 keys run k_rs_downsweep_rank, which
stages tiles by TMA as rows of 32 keys: keys past the last full row, and
positions past n in the last tile, take its plain-load path.  These cases
use odd sizes above that threshold (n % 32 != 0), for key + value sorts (the
tree build) and keys-only sorts (stage 2 over windows), each checked against
the oracle or a host restatement.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [300_007, 262_145, 1_048_607])
def test_run_at_ragged_sizes(owm, oracle, n):
    spec, W, Ov, B, mn, seed = owm.synth_config(1)
    spec.n = n
    xyz, bb = owm.synth_cloud(spec, seed)
    ctx = owm.Context(0)
    cloud = ctx.cloud(xyz, bb)
    want, _ = oracle.run(xyz, bb, W, Ov, B)
    for leaf in (32, 256):
        np.testing.assert_array_equal(ctx.run(cloud, owm.run_cfg(W, Ov, B, leaf)), want)
    tree = ctx.tree(cloud, owm.OWM_TREE_MAX_NUMBER, 64)
    assert tree.check()
    assert tree.info().root_count == n
    tree.close()
    cloud.close()
    ctx.close()


def _llp(win, overlap):
    v = np.sort(np.asarray(win, dtype=np.int64))
    v = v[v >= 0]
    if overlap == 0.0:
        return v
    u, c = np.unique(v, return_counts=True)
    return u[c >= 2]


@pytest.mark.parametrize("ncells", [300_001, 1_048_575])
def test_stage2_keys_only_ragged(owm, ncells):
    """owm_stage2 sorts the window ids (keys only) at sizes past the ranked
    pass's threshold, n % 32 != 0 (its keys are 32-bit: four 8-bit digits;
    the allocation-free stage 2 sorts narrower keys through the ranked pass,
    tests/test_zz_no_alloc.py)."""
    rng = np.random.default_rng(ncells)
    win = rng.integers(0, 99_999_999, ncells)
    win[rng.random(ncells) < 0.05] = -1
    win[: ncells // 3] = rng.integers(0, 1000, ncells // 3)  # many repeats
    ctx = owm.Context(0)
    for ov in (0.8, 0.0):
        np.testing.assert_array_equal(ctx.stage2(win.copy(), ov), _llp(win, ov))
    ctx.close()


def test_overlap_zero_run_sorts_windows(owm, oracle):
    """owm_run with overlap 0 takes stage 2 by sorting the window results
    (keys only, key width from the point count): 300,007 points over 600 x
    600 m at W 1 give 361,201 windows, more than 262,144, so that sort runs
    the ranked pass."""
    spec, W, _, B, mn, seed = owm.synth_config(1)
    spec.n = 300_007
    spec.x1, spec.y1 = spec.x0 + 600.0, spec.y0 + 600.0
    xyz, bb = owm.synth_cloud(spec, seed)
    W, Ov = 1, 0.0
    p = owm.params(bb, spec.n, W, Ov, B)
    assert p.ncells > 262_144
    ctx = owm.Context(0)
    cloud = ctx.cloud(xyz, bb)
    want, _ = oracle.run(xyz, bb, W, Ov, B)
    np.testing.assert_array_equal(ctx.run(cloud, owm.run_cfg(W, Ov, B, mn)), want)
    cloud.close()
    ctx.close()
