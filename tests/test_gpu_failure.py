"""The bounded-walk failure path on the GPU, made without a fault.

Every data-dependent device loop of the path is bounded: the stage-1 tree
walk by a step count, the stage-3 cell walk by a round count and its node
stack by its size.  On a well-formed tree those bounds are never reached, so
these tests lower the limit through owm_ctx_set_walk_limit: a normal walk on
a small cloud then gives up, sets the walk-bound bit of the device status
word, and its call returns OWM_ETIMEOUT.  Every index stays in range (the
tree is untouched; only the loop stops early), and the same context then runs
a correct job once the limit is lifted.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OWM_ETIMEOUT = -4
WALK_BOUND_BIT = 2


def _small(F, n=150_000, w=70.0, h=80.0):
    spec, W, Ov, B, mn, seed = F.synth_config(1)
    spec.n, spec.x1, spec.y1 = n, spec.x0 + w, spec.y0 + h
    xyz, bb = F.synth_cloud(spec, seed)
    return xyz, bb, W, Ov, mn


def test_stage1_walk_limit_times_out_then_recovers(owm, oracle):
    ctx = owm.Context(0)
    xyz, bb, W, Ov, mn = _small(owm)
    cloud = ctx.cloud(xyz, bb)
    tree = ctx.tree(cloud, owm.OWM_TREE_MAX_NUMBER, mn)
    p = owm.params(bb, xyz.shape[0], W, Ov, 20)
    ctx.set_walk_limit(3)
    with pytest.raises(owm.OwmError) as e:
        ctx.stage1(tree, p)
    assert e.value.status == OWM_ETIMEOUT
    assert ctx.device_status() & WALK_BOUND_BIT
    # the whole path with the walk as stage 1 stops the same way
    with pytest.raises(owm.OwmError) as e:
        ctx.run(cloud, owm.run_cfg(W, Ov, 20, mn, stage1_walk=True))
    assert e.value.status == OWM_ETIMEOUT
    # lifted: the same context, tree and cloud give the exact answer again
    ctx.set_walk_limit(0)
    win = ctx.stage1(tree, p)
    assert ctx.device_status() & WALK_BOUND_BIT == 0
    want = oracle.stage1(xyz, oracle.params(bb, xyz.shape[0], W, Ov, 20))
    np.testing.assert_array_equal(win, want)
    got = ctx.run(cloud, owm.run_cfg(W, Ov, 20, mn, stage1_walk=True))
    np.testing.assert_array_equal(got, oracle.run(xyz, bb, W, Ov, 20)[0])
    tree.close()
    cloud.close()
    ctx.close()


def test_stage3_cell_walk_limit_times_out_then_recovers(owm, oracle):
    """Bsize 3 with Wsize 10 leaves most 3 m cells without an LLP, so stage 3
    walks the tree for them (window classes do stage 1 and need no walk)."""
    ctx = owm.Context(0)
    xyz, bb, W, Ov, mn = _small(owm)
    B = 3
    cloud = ctx.cloud(xyz, bb)
    cfg = owm.run_cfg(W, Ov, B, mn)
    want, _ = oracle.run(xyz, bb, W, Ov, B)
    np.testing.assert_array_equal(ctx.run(cloud, cfg), want)
    ctx.set_walk_limit(1)  # one round: the root alone, its children never popped
    with pytest.raises(owm.OwmError) as e:
        ctx.run(cloud, cfg)
    assert e.value.status == OWM_ETIMEOUT
    assert ctx.device_status() & WALK_BOUND_BIT
    tree = ctx.tree(cloud, owm.OWM_TREE_MAX_NUMBER, mn)
    p = owm.params(bb, xyz.shape[0], W, Ov, B)
    llp = oracle.stage2(oracle.stage1(xyz, oracle.params(bb, xyz.shape[0], W, Ov, B)), Ov)
    with pytest.raises(owm.OwmError) as e:
        ctx.stage3(tree, p, llp)
    assert e.value.status == OWM_ETIMEOUT
    ctx.set_walk_limit(0)
    np.testing.assert_array_equal(ctx.run(cloud, cfg), want)
    np.testing.assert_array_equal(ctx.stage3(tree, p, llp),
                                  oracle.stage3(xyz, oracle.params(bb, xyz.shape[0], W, Ov, B), llp))
    assert ctx.device_status() & WALK_BOUND_BIT == 0
    tree.close()
    cloud.close()
    ctx.close()


def test_walk_limit_rejects_negative(owm):
    ctx = owm.Context(0)
    with pytest.raises(owm.OwmError):
        ctx.set_walk_limit(-1)
    ctx.close()
