"""Points given as device memory: owm_cloud_create (read in place when 8-byte
aligned on the context's device, through a device copy otherwise) and
owm_run_host, with and without a bbox (device input: the bbox from the copy
on the context's device).  Every result equals the host-input one."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cloud(owm, n=300_000, seed=31):
    spec, W, Ov, B, mn, _ = owm.synth_config(1)
    side = (spec.x1 - spec.x0) * np.sqrt(n / spec.n)
    spec.n, spec.x1, spec.y1 = n, spec.x0 + side, spec.y0 + side
    xyz, bb = owm.synth_cloud(spec, seed)
    return xyz, bb, owm.run_cfg(W, Ov, B, mn)


def _dptr(t):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))


def _device_cloud(owm, ctx, ptr, n, bbox):
    h = C.c_void_p()
    rc = owm.lib().owm_cloud_create(ctx.handle, ptr, n, C.byref(bbox) if bbox is not None else None, C.byref(h))
    assert rc == 0, rc
    b = owm.Bbox()
    assert owm.lib().owm_cloud_bbox(h, C.byref(b)) == 0
    return owm.Cloud(ctx, h, n, b)


def test_cloud_from_device_memory(owm, ctx):
    torch = pytest.importorskip("torch")
    xyz, bb, cfg = _cloud(owm)
    want = ctx.run(ctx.cloud(xyz, bb), cfg)
    d = torch.from_numpy(xyz).to("cuda:0")
    # aligned, read in place; with and without a bbox (the data's = the generator's)
    for bbox in (bb, None):
        cl = _device_cloud(owm, ctx, _dptr(d), xyz.shape[0], bbox)
        assert cl.bbox.astuple() == bb.astuple()
        np.testing.assert_array_equal(cl.points(), xyz)
        np.testing.assert_array_equal(ctx.run(cl, cfg), want)
        cl.close()
    # not 8-byte aligned: the same bytes 4 bytes into a device buffer
    raw = torch.zeros(xyz.nbytes + 8, dtype=torch.uint8, device="cuda:0")
    raw[4:4 + xyz.nbytes] = torch.from_numpy(xyz.view(np.uint8).reshape(-1)).to("cuda:0")
    p4 = C.cast(C.c_void_p(raw.data_ptr() + 4), C.POINTER(C.c_double))
    cl = _device_cloud(owm, ctx, p4, xyz.shape[0], None)
    assert cl.bbox.astuple() == bb.astuple()
    np.testing.assert_array_equal(cl.points(), xyz)
    np.testing.assert_array_equal(ctx.run(cl, cfg), want)
    cl.close()


def test_run_host_with_device_input(owm, ctx):
    torch = pytest.importorskip("torch")
    xyz, bb, cfg = _cloud(owm, 250_000, 32)
    want = ctx.run_host(xyz, bb, cfg)
    d = torch.from_numpy(xyz).to("cuda:0")
    n = xyz.shape[0]
    p = owm.params(bb, n, cfg.wsize, cfg.overlap, cfg.bsize)
    out = np.empty(p.ncells + p.ngrid + 1, dtype=np.int64)
    for bbox in (bb, None):
        k = C.c_int64()
        rc = owm.lib().owm_run_host(ctx.handle, _dptr(d), n, C.byref(bbox) if bbox is not None else None,
                                    C.byref(cfg), out.ctypes.data_as(C.POINTER(C.c_int64)), out.size, C.byref(k), None)
        assert rc == 0, rc
        np.testing.assert_array_equal(out[:k.value], want)
        t = C.c_int64()
        rc = owm.lib().owm_run_host_submit(ctx.handle, _dptr(d), n, C.byref(bbox) if bbox is not None else None,
                                           C.byref(cfg), out.ctypes.data_as(C.POINTER(C.c_int64)), out.size,
                                           C.byref(t))
        assert rc == 0, rc
        rc = owm.lib().owm_run_host_wait(ctx.handle, t.value, C.byref(k), None)
        assert rc == 0, rc
        np.testing.assert_array_equal(out[:k.value], want)
