"""fastowm_gb300 -- GB300-native OWM ground-seed path (Python host binding).

A thin layer over the C ABI (``include/owm_gb300.h``) of the in-tree native
library.  Names follow the reference's entry points
(CPP-TBB-CPU/include/optim3_func.hpp:73-93 and the reference application
CPP-TBB-CPU/application/owm_optim3.cpp):

    read_xyz        readXYZfile            (optim3_func.cpp:665-722)
    params          application parameter block (owm_optim3.cpp:92-132)
    Context.tree    parallel_qtree + storeMinAndNumPoints (optim3_func.cpp:220-307)
    Context.stage1  stage1                 (optim3_func.cpp:541-561)
    Context.stage2  std::sort + stage2     (owm_optim3.cpp:160-188, optim3_func.cpp:610-625)
    Context.stage3  LLP grid + stage3      (owm_optim3.cpp:192-205, optim3_func.cpp:627-662)
    Context.run     owm_optim3.cpp's loop body, result = stage-3 ids ++ LLPs

Point ids are 1-based positions in the input order (the reference's
cloud[] index); -1 means "no minimum".  Every compute call runs on the GPU;
there is no CPU fallback, and a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _lib
from ._lib import (OWM_EAGAIN, OWM_ECUDA, OWM_OK, OWM_TREE_MAX_NUMBER, OWM_TREE_MIN_RADIUS, Bbox, Params, RunCfg, RunInfo,  # noqa: F401
                   ServerCfg, ServerStats, SynthSpec, TileDesc, TreeCfg, TreeInfo, Tuning)

__all__ = ["OwmError", "round2d", "params", "bbox_of", "read_xyz", "write_xyz_ids", "check_results",
           "synth_config", "synth_cloud", "Context", "Batch", "Server", "TreeCfg", "RunCfg", "lib"]


class OwmError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = lib().owm_status_string(status).decode()
        if status == OWM_ECUDA:
            detail = lib().owm_last_error().decode()
            if detail:
                msg = f"{msg}: {detail}"
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


def lib():
    return _lib.load()


def _check(rc: int, what: str):
    if rc != OWM_OK:
        raise OwmError(rc, what)


def _f64p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i64p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def _as_xyz(xyz) -> np.ndarray:
    a = np.ascontiguousarray(xyz, dtype=np.float64)
    if a.ndim != 2 or a.shape[1] != 3:
        raise ValueError("xyz must have shape (n, 3)")
    return a


def _bbox(b) -> Bbox | None:
    if b is None:
        return None
    if isinstance(b, Bbox):
        return b
    return Bbox(*map(float, b))


def round2d(z: float) -> float:
    """optim3_func.cpp:1-3 (the C library's round(), half away from zero)."""
    import math
    v = z * 100.0
    r = math.floor(abs(v) + 0.5)
    return math.copysign(r, v) / 100.0


def params(bbox, npoints: int, wsize: int, overlap: float, bsize: int) -> Params:
    p = Params()
    _check(lib().owm_params_compute(C.byref(_bbox(bbox)), npoints, wsize, overlap, bsize, C.byref(p)), "params")
    return p


def bbox_of(xyz) -> Bbox:
    a = _as_xyz(xyz)
    b = Bbox()
    _check(lib().owm_bbox_of(_f64p(a), a.shape[0], C.byref(b)), "bbox_of")
    return b


def read_xyz(path: str):
    """readXYZfile: returns (xyz (n,3) float64, Bbox)."""
    ptr = C.POINTER(C.c_double)()
    n = C.c_int64()
    b = Bbox()
    _check(lib().owm_xyz_read(str(path).encode(), C.byref(ptr), C.byref(n), C.byref(b)), f"read {path}")
    try:
        arr = np.ctypeslib.as_array(ptr, shape=(n.value * 3,)).copy().reshape(-1, 3)
    finally:
        lib().owm_host_free(C.cast(ptr, C.c_void_p))
    return arr, b


def write_xyz_ids(path: str, xyz, ids) -> None:
    a = _as_xyz(xyz)
    i = np.ascontiguousarray(ids, dtype=np.int64)
    _check(lib().owm_xyz_write_ids(str(path).encode(), _f64p(a), a.shape[0], _i64p(i), i.size), f"write {path}")


def check_results(gold_xyz, xyz, ids, displace: float) -> float:
    g, a = _as_xyz(gold_xyz), _as_xyz(xyz)
    i = np.ascontiguousarray(ids, dtype=np.int64)
    return lib().owm_check_results(_f64p(g), g.shape[0], _f64p(a), a.shape[0], _i64p(i), i.size, displace)


def synth_config(config: int, tile: int = 0):
    """Returns (spec, wsize, overlap, bsize, max_number, seed) of a workload config."""
    s = SynthSpec()
    w, b, m = C.c_uint32(), C.c_uint32(), C.c_int32()
    o = C.c_double()
    seed = C.c_uint64()
    _check(lib().owm_synth_config(config, tile, C.byref(s), C.byref(w), C.byref(o), C.byref(b), C.byref(m),
                                  C.byref(seed)), "synth_config")
    return s, w.value, o.value, b.value, m.value, seed.value


def synth_cloud(spec: SynthSpec, seed: int, nthreads: int = 0, out: np.ndarray | None = None):
    """Generates the seeded cloud: returns (xyz (n,3), Bbox)."""
    xyz = out if out is not None else np.empty((spec.n, 3), dtype=np.float64)
    b = Bbox()
    _check(lib().owm_synth_cloud(C.byref(spec), seed, _f64p(xyz), C.byref(b), nthreads), "synth_cloud")
    return xyz, b


def tree_cfg(policy: int = OWM_TREE_MAX_NUMBER, max_number: int = 32, min_radius: float = 0.1,
             level: int = 5) -> TreeCfg:
    return TreeCfg(policy, max_number, min_radius, level)


def run_cfg(wsize: int, overlap: float, bsize: int, max_number: int = 32, policy: int = OWM_TREE_MAX_NUMBER,
            min_radius: float = 0.1, stage1_walk: bool = False) -> RunCfg:
    """stage1_walk: False = exact window classes (default), True = per-window tree walk."""
    return RunCfg(wsize, bsize, overlap, tree_cfg(policy, max_number, min_radius), 1 if stage1_walk else 0, 0)


class _Child:
    """A device object owned by a Context: closed before the context is, and
    never released through a context that is already gone."""

    def close(self):
        h, self.handle = getattr(self, "handle", None), None
        ctx = getattr(self, "ctx", None)
        if h and ctx is not None and getattr(ctx, "handle", None):
            self._destroy(h)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Cloud(_Child):
    def __init__(self, ctx: "Context", handle: C.c_void_p, n: int, bbox: Bbox):
        self.ctx, self.handle, self.n, self.bbox = ctx, handle, n, bbox
        ctx._children.add(self)

    def _destroy(self, h):
        lib().owm_cloud_destroy(h)

    def points(self) -> np.ndarray:
        """The cloud's points copied to the host, [n, 3] float64."""
        out = np.empty((self.n, 3), dtype=np.float64)
        _check(lib().owm_cloud_copy_out(self.handle, _f64p(out), self.n), "cloud_copy_out")
        return out


class Tree(_Child):
    def __init__(self, ctx: "Context", handle: C.c_void_p, cloud: Cloud):
        self.ctx, self.handle, self.cloud = ctx, handle, cloud  # keeps the cloud alive
        ctx._children.add(self)

    def _destroy(self, h):
        lib().owm_tree_destroy(h)

    def info(self) -> TreeInfo:
        i = TreeInfo()
        _check(lib().owm_tree_get_info(self.ctx.handle, self.handle, C.byref(i)), "tree info")
        return i

    def check(self) -> bool:
        return lib().owm_tree_check(self.ctx.handle, self.handle) == OWM_OK


class Context:
    """One GPU stream and its cached device buffers.  Clouds and trees made
    from it are released before it is."""

    def __init__(self, device: int = 0):
        self._children = weakref.WeakSet()
        h = C.c_void_p()
        _check(lib().owm_ctx_create(device, C.byref(h)), "ctx_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            for ch in sorted(list(self._children), key=lambda o: 0 if isinstance(o, (Tree, Batch)) else 1):
                ch.close()
            lib().owm_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        _check(lib().owm_ctx_sync(self.handle), "sync")

    @property
    def launches(self) -> int:
        return lib().owm_ctx_launches(self.handle)

    def device_status(self) -> int:
        """The device status word: bit 0 non-finite input, bit 1 a bounded
        tree walk stopped (the call returned OWM_ETIMEOUT)."""
        st = C.c_int32()
        _check(lib().owm_ctx_device_status(self.handle, C.byref(st)), "device_status")
        return st.value

    def set_tuning(self, walk_patch_x: int = 0, cell_warps: int = 0, gather_block: int = 0) -> None:
        """Launch shapes of this context's kernels (0 keeps a field); the
        results do not depend on them."""
        t = Tuning(walk_patch_x, cell_warps, gather_block, 0)
        _check(lib().owm_ctx_set_tuning(self.handle, C.byref(t)), "set_tuning")

    def tuning(self) -> dict:
        t = Tuning()
        _check(lib().owm_ctx_get_tuning(self.handle, C.byref(t)), "get_tuning")
        return t.asdict()

    def set_walk_limit(self, limit: int) -> None:
        """Step limit of the bounded tree walks (0 = their structural bounds)."""
        _check(lib().owm_ctx_set_walk_limit(self.handle, limit), "set_walk_limit")

    def cloud(self, xyz, bbox=None) -> Cloud:
        a = _as_xyz(xyz)
        h = C.c_void_p()
        b = _bbox(bbox) or bbox_of(a)
        _check(lib().owm_cloud_create(self.handle, _f64p(a), a.shape[0], C.byref(b), C.byref(h)), "cloud_create")
        return Cloud(self, h, a.shape[0], b)

    def _parsed_cloud(self, h: C.c_void_p) -> Cloud:
        b = Bbox()
        _check(lib().owm_cloud_bbox(h, C.byref(b)), "cloud_bbox")
        return Cloud(self, h, int(lib().owm_cloud_size(h)), b)

    def cloud_parse_xyz(self, text) -> Cloud:
        """Parses .xyz text (bytes, or a uint8 array such as a pinned host
        buffer) on the device into a cloud (owm_cloud_parse_xyz)."""
        h = C.c_void_p()
        if isinstance(text, (bytes, bytearray)):
            buf = bytes(text)
            _check(lib().owm_cloud_parse_xyz(self.handle, buf, len(buf), C.byref(h)), "cloud_parse_xyz")
        else:
            a = np.ascontiguousarray(text, dtype=np.uint8).reshape(-1)
            _check(lib().owm_cloud_parse_xyz(self.handle, C.cast(a.ctypes.data, C.c_char_p), a.size, C.byref(h)),
                   "cloud_parse_xyz")
        return self._parsed_cloud(h)

    def cloud_load_xyz(self, path: str) -> Cloud:
        """Reads and parses an .xyz file on the device (owm_cloud_load_xyz)."""
        h = C.c_void_p()
        _check(lib().owm_cloud_load_xyz(self.handle, str(path).encode(), C.byref(h)), "cloud_load_xyz")
        return self._parsed_cloud(h)

    def tree(self, cloud: Cloud, policy: int = OWM_TREE_MAX_NUMBER, max_number: int = 32, min_radius: float = 0.1,
             level: int = 5) -> Tree:
        h = C.c_void_p()
        cfg = tree_cfg(policy, max_number, min_radius, level)
        _check(lib().owm_tree_build(self.handle, cloud.handle, C.byref(cfg), C.byref(h)), "tree_build")
        return Tree(self, h, cloud)

    def stage1(self, tree: Tree, p: Params) -> np.ndarray:
        out = np.empty(p.ncells, dtype=np.int64)
        _check(lib().owm_stage1(self.handle, tree.handle, C.byref(p), _i64p(out)), "stage1")
        return out

    def stage2(self, win_min: np.ndarray, overlap: float) -> np.ndarray:
        """Returns the LLPs (ascending); win_min is left sorted/compacted like the reference's minIDs."""
        w = np.ascontiguousarray(win_min, dtype=np.int64)
        n = C.c_int64()
        _check(lib().owm_stage2(self.handle, _i64p(w), w.size, overlap, C.byref(n)), "stage2")
        return w[: n.value].copy()

    def stage3(self, tree: Tree, p: Params, llp) -> np.ndarray:
        l = np.ascontiguousarray(llp, dtype=np.int64)
        out = np.empty(max(p.ngrid, 1), dtype=np.int64)
        n = C.c_int64()
        _check(lib().owm_stage3(self.handle, tree.handle, C.byref(p), _i64p(l), l.size, _i64p(out), out.size,
                                C.byref(n)), "stage3")
        return out[: n.value].copy()

    def run(self, cloud: Cloud, cfg: RunCfg, info: RunInfo | None = None) -> np.ndarray:
        """Whole path; returns stage-3 ids followed by the LLPs."""
        p = Params()
        # capacity: ncells + ngrid is always enough
        _check(lib().owm_params_compute(C.byref(cloud.bbox), cloud.n, cfg.wsize, cfg.overlap, cfg.bsize,
                                        C.byref(p)), "params")
        out = np.empty(p.ncells + max(p.ngrid, 0) + 1, dtype=np.int64)
        n = C.c_int64()
        inf = info if info is not None else RunInfo()
        _check(lib().owm_run(self.handle, cloud.handle, C.byref(cfg), _i64p(out), out.size, C.byref(n),
                             C.byref(inf)), "run")
        return out[: n.value].copy()

    def run_host(self, xyz, bbox, cfg: RunCfg, info: RunInfo | None = None, out: np.ndarray | None = None):
        a = _as_xyz(xyz)
        b = _bbox(bbox) or bbox_of(a)
        p = params(b, a.shape[0], cfg.wsize, cfg.overlap, cfg.bsize)
        cap = p.ncells + max(p.ngrid, 0) + 1
        if out is None or out.size < cap:
            out = np.empty(cap, dtype=np.int64)
        n = C.c_int64()
        inf = info if info is not None else RunInfo()
        _check(lib().owm_run_host(self.handle, _f64p(a), a.shape[0], C.byref(b), C.byref(cfg), _i64p(out), out.size,
                                  C.byref(n), C.byref(inf)), "run_host")
        return out[: n.value].copy()

    def run_host_submit(self, xyz, bbox, cfg: RunCfg, out: np.ndarray | None = None) -> int:
        """Queues owm_run_host asynchronously; returns a ticket for run_host_wait.
        xyz and the output array are kept alive until the wait."""
        a = _as_xyz(xyz)
        b = _bbox(bbox) or bbox_of(a)
        p = params(b, a.shape[0], cfg.wsize, cfg.overlap, cfg.bsize)
        cap = p.ncells + max(p.ngrid, 0) + 1
        if out is None or out.size < cap:
            out = np.empty(cap, dtype=np.int64)
        t = C.c_int64()
        _check(lib().owm_run_host_submit(self.handle, _f64p(a), a.shape[0], C.byref(b), C.byref(cfg), _i64p(out),
                                         out.size, C.byref(t)), "run_host_submit")
        if not hasattr(self, "_pending"):
            self._pending = {}
        self._pending[t.value] = (a, out)
        return t.value

    def run_host_wait(self, ticket: int, info: RunInfo | None = None) -> np.ndarray:
        n = C.c_int64()
        inf = info if info is not None else RunInfo()
        rc = lib().owm_run_host_wait(self.handle, ticket, C.byref(n), C.byref(inf))
        _, out = self._pending.pop(ticket, (None, None)) if hasattr(self, "_pending") else (None, None)
        _check(rc, "run_host_wait")
        return out[: n.value].copy()

    def run_submit(self, cloud: Cloud, cfg: RunCfg, out: np.ndarray | None = None) -> int:
        """Queues owm_run on a device cloud asynchronously; returns a ticket for
        run_wait.  The cloud and the output array are kept alive until the wait."""
        p = params(cloud.bbox, cloud.n, cfg.wsize, cfg.overlap, cfg.bsize)
        cap = p.ncells + max(p.ngrid, 0) + 1
        if out is None or out.size < cap:
            out = np.empty(cap, dtype=np.int64)
        t = C.c_int64()
        _check(lib().owm_run_submit(self.handle, cloud.handle, C.byref(cfg), _i64p(out), out.size, C.byref(t)),
               "run_submit")
        if not hasattr(self, "_pending"):
            self._pending = {}
        self._pending[t.value] = (cloud, out)
        return t.value

    def run_wait(self, ticket: int, info: RunInfo | None = None) -> np.ndarray:
        n = C.c_int64()
        inf = info if info is not None else RunInfo()
        rc = lib().owm_run_wait(self.handle, ticket, C.byref(n), C.byref(inf))
        _, out = self._pending.pop(ticket, (None, None)) if hasattr(self, "_pending") else (None, None)
        _check(rc, "run_wait")
        return out[: n.value].copy()


class Batch(_Child):
    """Many tiles built and queried together (one launch per stage)."""

    def __init__(self, ctx: Context):
        h = C.c_void_p()
        _check(lib().owm_batch_create(ctx.handle, C.byref(h)), "batch_create")
        self.ctx, self.handle = ctx, h
        ctx._children.add(self)

    def _destroy(self, h):
        lib().owm_batch_destroy(h)

    def set_graphs(self, on: bool):
        _check(lib().owm_batch_set_graphs(self.handle, 1 if on else 0), "set_graphs")

    def set_leaf_classes(self, bounds, leaves):
        b = np.ascontiguousarray(bounds, dtype=np.int64)
        l = np.ascontiguousarray(leaves, dtype=np.int32)
        _check(lib().owm_batch_set_leaf_classes(self.handle, b.size, _i64p(b),
                                                l.ctypes.data_as(C.POINTER(C.c_int32))), "set_leaf_classes")

    def run(self, tiles, info: RunInfo | None = None):
        """tiles: list of (xyz, bbox, RunCfg).  Returns a list of seed arrays."""
        descs, keep, cap = tile_descs(tiles)
        out = np.empty(cap, dtype=np.int64)
        offs = np.empty(len(tiles) + 1, dtype=np.int64)
        inf = info if info is not None else RunInfo()
        _check(lib().owm_batch_run(self.handle, descs, len(tiles), _i64p(out), out.size, _i64p(offs), C.byref(inf)),
               "batch_run")
        return [out[offs[t]:offs[t + 1]].copy() for t in range(len(tiles))]


def tile_descs(tiles):
    descs = (TileDesc * len(tiles))()
    keep, cap = [], 0
    for t, (xyz, bbox, cfg) in enumerate(tiles):
        a = _as_xyz(xyz)
        keep.append(a)
        b = _bbox(bbox) or bbox_of(a)
        p = params(b, a.shape[0], cfg.wsize, cfg.overlap, cfg.bsize)
        cap += p.ncells + max(p.ngrid, 0) + 1
        descs[t] = TileDesc(_f64p(a), a.shape[0], b, cfg)
    return descs, keep, cap


class Server:
    """Continuous-batching request loop over device-resident tiles."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 120 << 30, max_tiles_per_batch: int = 64,
                 max_inflight_batches: int = 2, max_points_per_batch: int = 64 << 20, use_graphs: bool = False,
                 copy_on_submit: bool = True):
        cfg = ServerCfg(hbm_budget_bytes, max_tiles_per_batch, max_inflight_batches, max_points_per_batch,
                        1 if use_graphs else 0, 1 if copy_on_submit else 0)
        self._borrowed = {}  # ticket -> array kept alive while the server borrows it
        h = C.c_void_p()
        _check(lib().owm_server_create(device, C.byref(cfg), C.byref(h)), "server_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            lib().owm_server_destroy(self.handle)
            self.handle = None

    __del__ = close

    def submit(self, xyz, bbox, cfg: RunCfg) -> int:
        a = _as_xyz(xyz)
        b = _bbox(bbox) or bbox_of(a)
        d = TileDesc(_f64p(a), a.shape[0], b, cfg)
        t = C.c_int64()
        _check(lib().owm_server_submit(self.handle, C.byref(d), C.byref(t)), "submit")
        self._borrowed[t.value] = a
        return t.value

    def wait(self, ticket: int, cap: int, timeout_ms: float = 60000.0):
        out = np.empty(max(cap, 1), dtype=np.int64)
        n = C.c_int64()
        lat = C.c_double()
        _check(lib().owm_server_wait(self.handle, ticket, _i64p(out), out.size, C.byref(n), C.byref(lat),
                                     timeout_ms), "wait")
        self._borrowed.pop(ticket, None)
        return out[: n.value].copy(), lat.value

    def poll(self, ticket: int, cap: int):
        out = np.empty(max(cap, 1), dtype=np.int64)
        n = C.c_int64()
        lat = C.c_double()
        rc = lib().owm_server_poll(self.handle, ticket, _i64p(out), out.size, C.byref(n), C.byref(lat))
        if rc == OWM_EAGAIN:
            return None
        self._borrowed.pop(ticket, None)
        _check(rc, "poll")
        return out[: n.value].copy(), lat.value

    def stats(self) -> ServerStats:
        s = ServerStats()
        _check(lib().owm_server_get_stats(self.handle, C.byref(s)), "stats")
        return s
