"""owm_run_host_submit / owm_run_host_wait: two runs in flight per context,
the copy of one overlapping the compute of the other; results must be exactly
those of the synchronous owm_run_host."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cloud(owm, n, seed):
    spec, W, Ov, B, mn, _ = owm.synth_config(1)
    side = (spec.x1 - spec.x0) * np.sqrt(n / spec.n)
    spec.n, spec.x1, spec.y1 = n, spec.x0 + side, spec.y0 + side
    xyz, bb = owm.synth_cloud(spec, seed)
    return xyz, bb, owm.run_cfg(W, Ov, B, mn)


def test_async_runs_equal_sync(owm, ctx):
    a = _cloud(owm, 600_000, 11)
    b = _cloud(owm, 250_000, 12)
    ra = ctx.run_host(*a)
    rb = ctx.run_host(*b)
    t1 = ctx.run_host_submit(*a)
    t2 = ctx.run_host_submit(*b)
    with pytest.raises(owm.OwmError) as e:  # both slots busy
        ctx.run_host_submit(*a)
    assert e.value.status == owm._lib.OWM_EAGAIN
    np.testing.assert_array_equal(ctx.run_host_wait(t1), ra)
    t3 = ctx.run_host_submit(*a)
    np.testing.assert_array_equal(ctx.run_host(*b), rb)  # a synchronous run in between
    np.testing.assert_array_equal(ctx.run_host_wait(t2), rb)
    np.testing.assert_array_equal(ctx.run_host_wait(t3), ra)
    with pytest.raises(owm.OwmError):  # already collected
        ctx.run_host_wait(t3)
    # a longer stream, always two in flight
    pending = []
    for k in range(6):
        src = a if k % 2 == 0 else b
        pending.append((ctx.run_host_submit(*src), ra if k % 2 == 0 else rb))
        if len(pending) == 2:
            t, want = pending.pop(0)
            np.testing.assert_array_equal(ctx.run_host_wait(t), want)
    for t, want in pending:
        np.testing.assert_array_equal(ctx.run_host_wait(t), want)


def test_async_failed_submit_leaves_context_usable(owm, ctx):
    a = _cloud(owm, 200_000, 13)
    xyz, bb, cfg = a
    bad = owm.run_cfg(cfg.wsize, cfg.overlap, cfg.bsize, 0)  # a leaf capacity below 1 is invalid
    with pytest.raises(owm.OwmError) as e:
        ctx.run_host_submit(xyz, bb, bad)
    assert e.value.status == -1  # OWM_EINVAL, after the copy was queued: submit waited for it
    want = ctx.run_host(*a)
    np.testing.assert_array_equal(ctx.run_host_wait(ctx.run_host_submit(*a)), want)
