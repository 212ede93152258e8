"""owm_stage2_noalloc: the allocation-free stage 2 for callers that cannot
allocate device memory (their host owns every device byte through its own
pool, or forbids allocation on the streams it lends them).

Called through the C ABI with caller-owned device buffers, and compared with
the allocating owm_stage2 on two calls in a row (different inputs, so a
stale result left in the shared static working array would show).  The ids
are integers, so the comparison is exact.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _windows(F, ctx, config, n, w, h, overlap=None):
    spec, W, Ov, B, mn, seed = F.synth_config(config)
    spec.n, spec.x1, spec.y1 = n, spec.x0 + w, spec.y0 + h
    if overlap is not None:
        Ov = overlap
    xyz, bb = F.synth_cloud(spec, seed)
    cloud = ctx.cloud(xyz, bb)
    tree = ctx.tree(cloud, F.OWM_TREE_MAX_NUMBER, mn)
    p = F.params(bb, n, W, Ov, B)
    win = ctx.stage1(tree, p)
    tree.close()
    cloud.close()
    return win, Ov, n


def _noalloc(F, torch, win, overlap, npoints):
    d_win = torch.as_tensor(win, dtype=torch.int64).cuda()
    d_llp = torch.full((win.size,), -7, dtype=torch.int64, device="cuda")
    n = C.c_int64(-1)
    stream = torch.cuda.current_stream().cuda_stream
    rc = F.lib().owm_stage2_noalloc(C.c_void_p(stream), C.c_void_p(d_win.data_ptr()), win.size, overlap, npoints,
                                    C.c_void_p(d_llp.data_ptr()), C.byref(n))
    assert rc == 0, F.lib().owm_status_string(rc)
    return d_llp[: n.value].cpu().numpy()


def test_noalloc_stage2_matches_allocating_stage2(owm):
    torch = pytest.importorskip("torch")
    ctx = owm.Context(0)
    cases = [_windows(owm, ctx, 1, 400_000, 120, 150), _windows(owm, ctx, 3, 300_000, 150, 150, overlap=0.5)]
    for win, overlap, npts in cases:  # two calls in a row through the shared static array
        want = ctx.stage2(win.copy(), overlap)
        got = _noalloc(owm, torch, win, overlap, npts)
        assert want.size > 0
        np.testing.assert_array_equal(got, want)
    ctx.close()


def test_noalloc_rejects_oversize(owm):
    torch = pytest.importorskip("torch")
    d = torch.zeros(4, dtype=torch.int64, device="cuda")
    n = C.c_int64(-1)
    rc = owm.lib().owm_stage2_noalloc(None, C.c_void_p(d.data_ptr()), (1 << 20) + 1, 0.8, 1000,
                                      C.c_void_p(d.data_ptr()), C.byref(n))
    assert rc == -6  # OWM_ERANGE, before any work is issued
    assert n.value == -1
