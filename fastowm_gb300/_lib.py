"""ctypes declarations of the C ABI in ``include/owm_gb300.h``.

The library is the in-tree ``libowm_gb300.so`` built by
``fastowm_gb300.build``; there is no Python or CPU implementation of the
path behind these bindings.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libowm_gb300.so"

OWM_OK, OWM_EINVAL, OWM_ENOMEM, OWM_ECUDA, OWM_ETIMEOUT, OWM_EIO, OWM_ERANGE, OWM_EAGAIN = 0, -1, -2, -3, -4, -5, -6, -7
OWM_TREE_MIN_RADIUS, OWM_TREE_MAX_NUMBER = 0, 1

i64, i32, u32, f64, f32, u64 = C.c_int64, C.c_int32, C.c_uint32, C.c_double, C.c_float, C.c_uint64
P = C.POINTER


class Bbox(C.Structure):
    _fields_ = [("min_x", f64), ("min_y", f64), ("max_x", f64), ("max_y", f64)]

    def astuple(self):
        return (self.min_x, self.min_y, self.max_x, self.max_y)


class Params(C.Structure):
    _fields_ = [("npoints", i64), ("wsize", u32), ("bsize", u32), ("overlap", f64), ("bbox", Bbox),
                ("width", f64), ("height", f64), ("density", f64), ("displace", f64),
                ("min_num_points", u32), ("ncols", u32), ("nrows", u32), ("ncols_grid", u32),
                ("nrows_grid", u32), ("ncells", i64), ("ngrid", i64)]


class SynthSpec(C.Structure):
    _fields_ = [("n", i64), ("x0", f64), ("y0", f64), ("x1", f64), ("y1", f64), ("amplitude", f64),
                ("wavelength", f64), ("noise_sigma", f64), ("lifted_frac", f64), ("lift_lo", f64),
                ("lift_hi", f64), ("z_quantum", f64), ("tie_free", i32), ("strips", i32), ("holes", i32),
                ("_pad", i32)]


class TreeCfg(C.Structure):
    _fields_ = [("policy", i32), ("max_number", i32), ("min_radius", f32), ("level", i32)]


class Tuning(C.Structure):
    """owm_tuning: launch shapes of a context's kernels (0 = keep the default)."""
    _fields_ = [("walk_patch_x", i32), ("cell_warps", i32), ("gather_block", i32), ("_pad", i32)]

    def asdict(self):
        return {"walk_patch_x": self.walk_patch_x, "cell_warps": self.cell_warps, "gather_block": self.gather_block}


class TreeInfo(C.Structure):
    _fields_ = [("npoints", i64), ("nleaves", i64), ("nnodes", i64), ("root_count", i64),
                ("root_min_id", i64), ("max_leaf", i32), ("key_bits", i32)]


class RunCfg(C.Structure):
    _fields_ = [("wsize", u32), ("bsize", u32), ("overlap", f64), ("tree", TreeCfg), ("stage1_walk", i32),
                ("_pad", i32)]


class RunInfo(C.Structure):
    _fields_ = [("ms_tree", f64), ("ms_stage1", f64), ("ms_stage2", f64), ("ms_stage3", f64), ("ms_total", f64),
                ("n_llp", i64), ("n_stage3", i64), ("n_seeds", i64), ("params", Params)]


class TileDesc(C.Structure):
    _fields_ = [("xyz", P(f64)), ("n", i64), ("bbox", Bbox), ("cfg", RunCfg)]


class ServerCfg(C.Structure):
    _fields_ = [("hbm_budget_bytes", i64), ("max_tiles_per_batch", i32), ("max_inflight_batches", i32),
                ("max_points_per_batch", i64), ("use_graphs", i32), ("copy_on_submit", i32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", i64), ("completed", i64), ("batches", i64), ("points_done", i64),
                ("bytes_in_use", i64), ("peak_bytes", i64), ("busy_ms", f64)]


vp = C.c_void_p
# name -> (restype, argtypes); the same list is checked against the header by the tests
SIGNATURES = {
    "owm_params_compute": (C.c_int, [P(Bbox), i64, u32, f64, u32, P(Params)]),
    "owm_bbox_of": (C.c_int, [P(f64), i64, P(Bbox)]),
    "owm_xyz_read": (C.c_int, [C.c_char_p, P(P(f64)), P(i64), P(Bbox)]),
    "owm_xyz_write_ids": (C.c_int, [C.c_char_p, P(f64), i64, P(i64), i64]),
    "owm_host_free": (None, [vp]),
    "owm_check_results": (f64, [P(f64), i64, P(f64), i64, P(i64), i64, f32]),
    "owm_synth_config": (C.c_int, [C.c_int, i64, P(SynthSpec), P(u32), P(f64), P(u32), P(i32), P(u64)]),
    "owm_synth_cloud": (C.c_int, [P(SynthSpec), u64, P(f64), P(Bbox), C.c_int]),
    "owm_ctx_create": (C.c_int, [C.c_int, P(vp)]),
    "owm_ctx_destroy": (C.c_int, [vp]),
    "owm_ctx_sync": (C.c_int, [vp]),
    "owm_ctx_stream": (vp, [vp]),
    "owm_ctx_launches": (i64, [vp]),
    "owm_ctx_device_status": (C.c_int, [vp, P(i32)]),
    "owm_ctx_set_profiling": (C.c_int, [vp, C.c_int]),
    "owm_ctx_set_walk_limit": (C.c_int, [vp, i32]),
    "owm_ctx_set_tuning": (C.c_int, [vp, P(Tuning)]),
    "owm_ctx_get_tuning": (C.c_int, [vp, P(Tuning)]),
    "owm_ctx_kernel_times": (C.c_int, [vp, i32, vp, P(f64), P(i64), P(i32)]),
    "owm_cloud_create": (C.c_int, [vp, P(f64), i64, P(Bbox), P(vp)]),
    "owm_cloud_destroy": (C.c_int, [vp]),
    "owm_cloud_size": (i64, [vp]),
    "owm_cloud_bbox": (C.c_int, [vp, P(Bbox)]),
    "owm_cloud_copy_out": (C.c_int, [vp, P(f64), i64]),
    "owm_cloud_parse_xyz": (C.c_int, [vp, C.c_char_p, i64, P(vp)]),
    "owm_cloud_load_xyz": (C.c_int, [vp, C.c_char_p, P(vp)]),
    "owm_tree_build": (C.c_int, [vp, vp, P(TreeCfg), P(vp)]),
    "owm_tree_get_info": (C.c_int, [vp, vp, P(TreeInfo)]),
    "owm_tree_check": (C.c_int, [vp, vp]),
    "owm_tree_destroy": (C.c_int, [vp]),
    "owm_stage1": (C.c_int, [vp, vp, P(Params), P(i64)]),
    "owm_stage2": (C.c_int, [vp, P(i64), i64, f64, P(i64)]),
    "owm_stage3": (C.c_int, [vp, vp, P(Params), P(i64), i64, P(i64), i64, P(i64)]),
    "owm_stage2_noalloc": (C.c_int, [vp, vp, i64, f64, i64, vp, P(i64)]),
    "owm_run": (C.c_int, [vp, vp, P(RunCfg), P(i64), i64, P(i64), P(RunInfo)]),
    "owm_run_host": (C.c_int, [vp, P(f64), i64, P(Bbox), P(RunCfg), P(i64), i64, P(i64), P(RunInfo)]),
    "owm_run_host_submit": (C.c_int, [vp, P(f64), i64, P(Bbox), P(RunCfg), P(i64), i64, P(i64)]),
    "owm_run_host_wait": (C.c_int, [vp, i64, P(i64), P(RunInfo)]),
    "owm_run_submit": (C.c_int, [vp, vp, P(RunCfg), P(i64), i64, P(i64)]),
    "owm_run_wait": (C.c_int, [vp, i64, P(i64), P(RunInfo)]),
    "owm_batch_create": (C.c_int, [vp, P(vp)]),
    "owm_batch_destroy": (C.c_int, [vp]),
    "owm_batch_run": (C.c_int, [vp, P(TileDesc), i32, P(i64), i64, P(i64), P(RunInfo)]),
    "owm_batch_set_graphs": (C.c_int, [vp, C.c_int]),
    "owm_batch_set_leaf_classes": (C.c_int, [vp, i32, P(i64), P(i32)]),
    "owm_server_create": (C.c_int, [C.c_int, P(ServerCfg), P(vp)]),
    "owm_server_destroy": (C.c_int, [vp]),
    "owm_server_submit": (C.c_int, [vp, P(TileDesc), P(i64)]),
    "owm_server_poll": (C.c_int, [vp, i64, P(i64), i64, P(i64), P(f64)]),
    "owm_server_wait": (C.c_int, [vp, i64, P(i64), i64, P(i64), P(f64), f64]),
    "owm_server_get_stats": (C.c_int, [vp, P(ServerStats)]),
    "owm_status_string": (C.c_char_p, [C.c_int]),
    "owm_last_error": (C.c_char_p, []),
    "owm_version": (C.c_int, []),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Loads the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise OSError(f"{p} is missing: build it with fastowm_gb300.build.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
