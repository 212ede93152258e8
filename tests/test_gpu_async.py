"""owm_run_host_submit / owm_run_host_wait and owm_run_submit / owm_run_wait:
two runs in flight per context, the copy (or the host-side launch work) of one
overlapping the compute of the other; results must be exactly those of the
synchronous owm_run_host and owm_run."""
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


def test_device_submit_equals_run(owm, oracle, ctx):
    """owm_run_submit on device clouds shares the two slots with the host
    form; every ticket gives exactly owm_run's seeds."""
    a = _cloud(owm, 600_000, 21)
    b = _cloud(owm, 250_000, 22)
    ca, cb = ctx.cloud(a[0], a[1]), ctx.cloud(b[0], b[1])
    ra, rb = ctx.run(ca, a[2]), ctx.run(cb, b[2])
    W, Ov, B = b[2].wsize, b[2].overlap, b[2].bsize
    np.testing.assert_array_equal(rb, oracle.run(b[0], b[1], W, Ov, B)[0])
    t1 = ctx.run_submit(ca, a[2])
    t2 = ctx.run_host_submit(*b)  # the host form takes the other slot
    with pytest.raises(owm.OwmError) as e:
        ctx.run_submit(cb, b[2])
    assert e.value.status == owm._lib.OWM_EAGAIN
    info = owm.RunInfo()
    np.testing.assert_array_equal(ctx.run_wait(t1, info), ra)
    assert info.n_seeds == ra.size and info.params.ncells > 0
    np.testing.assert_array_equal(ctx.run_host_wait(t2), rb)
    pending = []
    for k in range(8):
        cl, cfg, want = (ca, a[2], ra) if k % 3 else (cb, b[2], rb)
        pending.append((ctx.run_submit(cl, cfg), want))
        if len(pending) == 2:
            t, w = pending.pop(0)
            np.testing.assert_array_equal(ctx.run_wait(t), w)
    np.testing.assert_array_equal(ctx.run(cb, b[2]), rb)  # a synchronous run with one in flight
    for t, w in pending:
        np.testing.assert_array_equal(ctx.run_wait(t), w)
    ca.close()
    cb.close()


def test_device_submit_reports_walk_bound_at_wait(owm):
    """A run whose stage-3 cell walk gives up (walk limit 1, Bsize 3) is
    submitted normally; its wait returns OWM_ETIMEOUT, and the context then
    runs the same cloud correctly.  Its own context: the limit is a context
    setting."""
    ctx = owm.Context(0)
    xyz, bb, cfg = _cloud(owm, 150_000, 23)
    cfg3 = owm.run_cfg(cfg.wsize, cfg.overlap, 3, cfg.tree.max_number)
    cl = ctx.cloud(xyz, bb)
    want = ctx.run(cl, cfg3)
    ctx.set_walk_limit(1)
    t = ctx.run_submit(cl, cfg3)
    with pytest.raises(owm.OwmError) as e:
        ctx.run_wait(t)
    assert e.value.status == -4  # OWM_ETIMEOUT
    ctx.set_walk_limit(0)
    np.testing.assert_array_equal(ctx.run_wait(ctx.run_submit(cl, cfg3)), want)
    cl.close()
    ctx.close()
