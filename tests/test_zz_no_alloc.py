"""owm_stage2_noalloc: the allocation-free stage 2 for callers that cannot
allocate device memory (their host owns every device byte through its own
pool, or forbids allocation on the streams it lends them).

Called through the C ABI with caller-owned device buffers, and compared with
the allocating owm_stage2 on calls in a row (different inputs, so a stale
result left in the shared static working array would show).  The ids are
integers, so the comparison is exact.  Also: ids above npoints are refused
(OWM_EINVAL) instead of giving a wrong list, overlap 0 keeps every valid
minimum, npoints on either side of a power of two (the top key bit of the
sort), and a stream other than the default one.
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


def _noalloc_rc(F, torch, win, overlap, npoints, stream=None):
    d_win = torch.as_tensor(win, dtype=torch.int64).cuda()
    d_llp = torch.full((win.size,), -7, dtype=torch.int64, device="cuda")
    n = C.c_int64(-1)
    st = stream if stream is not None else torch.cuda.current_stream()
    with torch.cuda.stream(st):
        rc = F.lib().owm_stage2_noalloc(C.c_void_p(st.cuda_stream), C.c_void_p(d_win.data_ptr()), win.size, overlap,
                                        npoints, C.c_void_p(d_llp.data_ptr()), C.byref(n))
    torch.cuda.synchronize()
    return rc, n.value, d_llp


def _noalloc(F, torch, win, overlap, npoints, stream=None):
    rc, n, d_llp = _noalloc_rc(F, torch, win, overlap, npoints, stream)
    assert rc == 0, F.lib().owm_status_string(rc)
    return d_llp[:n].cpu().numpy()


def _llp_of(win, overlap):
    """Stage 2 restated on the host: ids that occur at least twice (overlap >
    0) or every valid id (overlap == 0), ascending."""
    v = np.sort(np.asarray(win, dtype=np.int64))
    v = v[v >= 0]
    if overlap == 0.0:
        return v
    u, c = np.unique(v, return_counts=True)
    return u[c >= 2]


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


def test_noalloc_overlap_zero_and_key_width_edges(owm):
    """overlap 0 through the entry point, and synthetic window lists whose
    largest id is npoints itself, for npoints just below, at and just above a
    power of two (the sort orders only the key bits that ids up to npoints
    need, with "none" above them)."""
    torch = pytest.importorskip("torch")
    ctx = owm.Context(0)
    win, _, npts = _windows(owm, ctx, 1, 200_000, 90, 100, overlap=0.0)
    want = ctx.stage2(win.copy(), 0.0)
    np.testing.assert_array_equal(_noalloc(owm, torch, win, 0.0, npts), want)
    np.testing.assert_array_equal(want, _llp_of(win, 0.0))
    rng = np.random.default_rng(11)
    side = torch.cuda.Stream()
    for npoints in ((1 << 20) - 2, (1 << 20) - 1, 1 << 20, (1 << 16) + 1):
        w = rng.integers(max(0, npoints - 3000), npoints + 1, 200_000)
        w[rng.random(w.size) < 0.1] = -1
        w[:3] = npoints  # the largest id, repeated
        for ov in (0.8, 0.0):
            got = _noalloc(owm, torch, w, ov, npoints, stream=side)
            np.testing.assert_array_equal(got, _llp_of(w, ov))
            np.testing.assert_array_equal(got, ctx.stage2(w.copy(), ov))
    ctx.close()


def test_noalloc_rejects_ids_above_npoints(owm):
    """An id above npoints names no point: OWM_EINVAL, not a wrong list; the
    next call with valid ids is exact again (the flag is cleared per call)."""
    torch = pytest.importorskip("torch")
    w = np.array([5, 5, 7, 7, 9, 1001, -1], dtype=np.int64)
    rc, _, _ = _noalloc_rc(owm, torch, w, 0.8, 1000)
    assert rc == -1  # OWM_EINVAL
    w[5] = 1000
    np.testing.assert_array_equal(_noalloc(owm, torch, w, 0.8, 1000), [5, 7])
    big = np.full(64, 1 << 40, dtype=np.int64)
    rc, _, _ = _noalloc_rc(owm, torch, big, 0.5, 1 << 20)
    assert rc == -1


def test_noalloc_at_its_limit(owm):
    """The allocation-free stage 2 at its largest size (1,048,576 windows) and
    just below it (n % 32 != 0), two calls in a row: ids up to 5,000,000 make
    23-bit sort keys (digits of 8, 8 and 7 bits), so the last pass is the
    ranked, TMA-staged keys-only pass at a size that takes its ragged path."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    ctx = owm.Context(0)
    for ncells in (1 << 20, (1 << 20) - 33):
        w = rng.integers(0, 5_000_000, ncells)
        w[rng.random(ncells) < 0.1] = -1
        got = _noalloc(owm, torch, w, 0.8, 5_000_000)
        np.testing.assert_array_equal(got, _llp_of(w, 0.8))
        np.testing.assert_array_equal(got, ctx.stage2(w.copy(), 0.8))
    ctx.close()
