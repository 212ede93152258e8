"""ORACLE / TEST INFRASTRUCTURE -- Python binding of the CPU oracles.

* ``liboracle.so``      my C restatement of the OWM path (owm_oracle.c) and
                        the project's seeded cloud generator (oracle_synth_*)
* ``_ref/libowmref.so`` the reference's own CPP-TBB-CPU/src/optim3_func.cpp
                        compiled unmodified (ref_runner.cpp + shim/), from the
                        checkout named by $OWM_REFERENCE or from the copies
                        staged under _ref/src by ``make -C oracle REF=...``
* ``librefport.so``     C port of that reference algorithm (owm_refport.c):
                        the timed CPU baseline where the reference cannot be
                        compiled

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_ORACLE = HERE / "liboracle.so"
LIB_REF = HERE / "_ref" / "libowmref.so"
LIB_PORT = HERE / "librefport.so"
# the reference checkout, when one is at hand (no default location)
REF_SRC = Path(os.environ["OWM_REFERENCE"]) if os.environ.get("OWM_REFERENCE") else None
STAGED_SRC = HERE / "_ref" / "src" / "CPP-TBB-CPU"


class OracleParams(C.Structure):
    _fields_ = [("npoints", C.c_int64), ("wsize", C.c_uint32), ("bsize", C.c_uint32), ("overlap", C.c_double),
                ("min_x", C.c_double), ("min_y", C.c_double), ("max_x", C.c_double), ("max_y", C.c_double),
                ("width", C.c_double), ("height", C.c_double), ("density", C.c_double), ("displace", C.c_double),
                ("min_num_points", C.c_uint32), ("ncols", C.c_uint32), ("nrows", C.c_uint32),
                ("ncols_grid", C.c_uint32), ("nrows_grid", C.c_uint32), ("ncells", C.c_int64),
                ("ngrid", C.c_int64)]


class SynthSpec(C.Structure):
    """owm_synth_spec of include/owm_gb300.h."""
    _fields_ = [("n", C.c_int64), ("x0", C.c_double), ("y0", C.c_double), ("x1", C.c_double), ("y1", C.c_double),
                ("amplitude", C.c_double), ("wavelength", C.c_double), ("noise_sigma", C.c_double),
                ("lifted_frac", C.c_double), ("lift_lo", C.c_double), ("lift_hi", C.c_double),
                ("z_quantum", C.c_double), ("tie_free", C.c_int32), ("strips", C.c_int32), ("holes", C.c_int32),
                ("_pad", C.c_int32)]


class RefResult(C.Structure):
    _fields_ = [("n_llp", C.c_int64), ("n_stage3", C.c_int64), ("ncells", C.c_int64), ("ngrid", C.c_int64),
                ("min_num_points", C.c_uint32), ("ncols", C.c_uint32), ("nrows", C.c_uint32),
                ("ncols_grid", C.c_uint32), ("nrows_grid", C.c_uint32), ("displace", C.c_double),
                ("t_tree", C.c_double), ("t_owm", C.c_double), ("t_stage1", C.c_double), ("t_stage2", C.c_double),
                ("t_stage3", C.c_double)]


def build(ref: bool | None = None) -> None:
    """make -C oracle (the reference runner only when its sources exist)."""
    target = "all"
    if ref is False:
        target = "restatement"
    cmd = ["make", "-s", "-C", str(HERE), target]
    if REF_SRC is not None:
        cmd.append(f"REF={REF_SRC}")
    subprocess.run(cmd, check=True)


_o = None
_r = None
_p = None


def _oracle():
    global _o
    if _o is None:
        if not LIB_ORACLE.exists():
            build(ref=False)
        _o = C.CDLL(str(LIB_ORACLE))
        P = C.POINTER
        _o.oracle_params_compute.argtypes = [P(C.c_double), C.c_int64, C.c_uint32, C.c_double, C.c_uint32,
                                             P(OracleParams)]
        _o.oracle_stage1.argtypes = [P(C.c_double), C.c_int64, P(OracleParams), P(C.c_int64), C.c_int]
        _o.oracle_stage2.argtypes = [P(C.c_int64), C.c_int64, C.c_double]
        _o.oracle_stage2.restype = C.c_int64
        _o.oracle_stage3.argtypes = [P(C.c_double), C.c_int64, P(OracleParams), P(C.c_int64), C.c_int64,
                                     P(C.c_int64), C.c_int]
        _o.oracle_stage3.restype = C.c_int64
        _o.oracle_run.argtypes = [P(C.c_double), C.c_int64, P(C.c_double), C.c_uint32, C.c_double, C.c_uint32,
                                  P(C.c_int64), P(C.c_int64), C.c_int]
        _o.oracle_run.restype = C.c_int64
        _o.oracle_window_box.argtypes = [P(OracleParams), C.c_int64, C.c_int64, P(C.c_double)]
        _o.oracle_xyz_parse.argtypes = [C.c_char_p, C.c_int64, P(C.c_double), C.c_int64, P(C.c_int64),
                                        P(C.c_double), P(C.c_int)]
        _o.oracle_cell_box.argtypes = [P(OracleParams), C.c_int64, C.c_int64, P(C.c_double)]
        _o.oracle_synth_config.argtypes = [C.c_int, C.c_int64, P(SynthSpec), P(C.c_uint32), P(C.c_double),
                                           P(C.c_uint32), P(C.c_int32), P(C.c_uint64)]
        _o.oracle_synth_cloud.argtypes = [P(SynthSpec), C.c_uint64, P(C.c_double), P(C.c_double), C.c_int]
    return _o


def _port():
    global _p
    if _p is None:
        if not LIB_PORT.exists():
            build(ref=False)
        _p = C.CDLL(str(LIB_PORT))
        P = C.POINTER
        _p.refport_run.argtypes = [P(C.c_double), C.c_int64, P(C.c_double), C.c_uint32, C.c_double, C.c_uint32,
                                   C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, P(C.c_int64), C.c_int64, P(C.c_int64),
                                   P(C.c_double), P(C.c_double)]
        _p.refport_run.restype = C.c_int64
    return _p


def ref_available() -> bool:
    if LIB_REF.exists():
        return True
    have_src = (STAGED_SRC / "src" / "optim3_func.cpp").exists() or (
        REF_SRC is not None and (REF_SRC / "CPP-TBB-CPU" / "src" / "optim3_func.cpp").exists())
    if have_src:
        try:
            build(ref=True)
        except subprocess.CalledProcessError:
            return False
        return LIB_REF.exists()
    return False


def _ref():
    global _r
    if _r is None:
        if not ref_available():
            raise OSError("reference runner not built (needs the reference sources)")
        _r = C.CDLL(str(LIB_REF))
        P = C.POINTER
        _r.owmref_read_xyz.argtypes = [C.c_char_p, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_int64),
                                       C.POINTER(C.c_double)]
        _r.owmref_run.argtypes = [P(C.c_double), C.c_int64, P(C.c_double), C.c_uint32, C.c_uint32, C.c_double,
                                  C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_int),
                                  C.c_int64, P(C.c_int), C.c_int64, P(RefResult)]
        _r.owmref_check_results.argtypes = [C.c_char_p, P(C.c_double), C.c_int64, P(C.c_int), C.c_int64, C.c_float]
        _r.owmref_check_results.restype = C.c_double
    return _r


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _q(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def synth_config(config: int, tile: int = 0):
    """The project's workload config (the same source as the GPU library's
    owm_synth_config): (spec, wsize, overlap, bsize, max_number, seed)."""
    spec = SynthSpec()
    w, b, m = C.c_uint32(), C.c_uint32(), C.c_int32()
    o, seed = C.c_double(), C.c_uint64()
    if _oracle().oracle_synth_config(config, tile, C.byref(spec), C.byref(w), C.byref(o), C.byref(b), C.byref(m),
                                     C.byref(seed)) != 0:
        raise ValueError(f"no workload config {config}")
    return spec, w.value, o.value, b.value, m.value, seed.value


def synth_cloud(spec: SynthSpec, seed: int, nthreads: int = 0, out: np.ndarray | None = None):
    """The seeded cloud, bit-identical to the GPU library's owm_synth_cloud:
    (xyz (n, 3) float64, bbox array [min_x, min_y, max_x, max_y])."""
    xyz = out if out is not None else np.empty((spec.n, 3), dtype=np.float64)
    bb = np.zeros(4, dtype=np.float64)  # owm_bbox: min_x, min_y, max_x, max_y
    if _oracle().oracle_synth_cloud(C.byref(spec), seed, _d(xyz), _d(bb), nthreads) != 0:
        raise ValueError("bad synthetic cloud spec")
    return xyz, bb


def _bbox_arr(bbox) -> np.ndarray:
    if hasattr(bbox, "min_x"):
        return np.array([bbox.min_x, bbox.min_y, bbox.max_x, bbox.max_y], dtype=np.float64)
    return np.asarray(bbox, dtype=np.float64)


def params(bbox, n: int, W: int, O: float, B: int) -> OracleParams:
    p = OracleParams()
    bb = _bbox_arr(bbox)
    if _oracle().oracle_params_compute(_d(bb), n, W, O, B, C.byref(p)) != 0:
        raise ValueError("bad oracle params")
    return p


def stage1(xyz, p: OracleParams, nthreads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(xyz, dtype=np.float64)
    out = np.empty(p.ncells, dtype=np.int64)
    if _oracle().oracle_stage1(_d(a), a.shape[0], C.byref(p), _q(out), nthreads) != 0:
        raise RuntimeError("oracle stage1 failed")
    return out


def stage2(win_min, overlap: float) -> np.ndarray:
    w = np.array(win_min, dtype=np.int64)
    n = _oracle().oracle_stage2(_q(w), w.size, overlap)
    return w[:n].copy()


def stage3(xyz, p: OracleParams, llp, nthreads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(xyz, dtype=np.float64)
    l = np.ascontiguousarray(llp, dtype=np.int64)
    out = np.empty(max(p.ngrid, 1), dtype=np.int64)
    n = _oracle().oracle_stage3(_d(a), a.shape[0], C.byref(p), _q(l), l.size, _q(out), nthreads)
    if n < 0:
        raise RuntimeError("oracle stage3 failed")
    return out[:n].copy()


def run(xyz, bbox, W: int, O: float, B: int, nthreads: int = 0):
    """Restatement of the whole path: (seeds = stage-3 ids ++ LLPs, n_llp)."""
    a = np.ascontiguousarray(xyz, dtype=np.float64)
    p = params(bbox, a.shape[0], W, O, B)
    out = np.empty(p.ncells + max(p.ngrid, 0) + 1, dtype=np.int64)
    nllp = C.c_int64()
    n = _oracle().oracle_run(_d(a), a.shape[0], _d(_bbox_arr(bbox)), W, O, B, _q(out), C.byref(nllp), nthreads)
    if n < 0:
        raise RuntimeError("oracle run failed")
    return out[:n].copy(), nllp.value


def window_box(p: OracleParams, ii: int, jj: int) -> np.ndarray:
    b = np.empty(4, dtype=np.float64)
    _oracle().oracle_window_box(C.byref(p), ii, jj, _d(b))
    return b


def ref_run(xyz, bbox, W: int, O: float, B: int, policy: int = 1, min_radius: float = 0.1, max_number: int = 32,
            level: int = 5, nthreads: int = 1, memo_a: bool = False, loops: int = 1, want_win: bool = True):
    """The reference's own CPU path: returns (seeds, n_llp, win_min or None, RefResult)."""
    a = np.ascontiguousarray(xyz, dtype=np.float64)
    p = params(bbox, a.shape[0], W, O, B)
    win = np.empty(max(p.ncells, 1), dtype=np.int32) if want_win else None
    seeds = np.empty(p.ncells + max(p.ngrid, 0) + 1, dtype=np.int32)
    res = RefResult()
    rc = _ref().owmref_run(_d(a), a.shape[0], _d(_bbox_arr(bbox)), W, B, O, policy, min_radius, max_number, level,
                           nthreads, 1 if memo_a else 0, loops,
                           win.ctypes.data_as(C.POINTER(C.c_int)) if want_win else None, win.size if want_win else 0,
                           seeds.ctypes.data_as(C.POINTER(C.c_int)), seeds.size, C.byref(res))
    if rc != 0:
        raise RuntimeError(f"reference run failed ({rc})")
    n = res.n_llp + res.n_stage3
    return seeds[:n].astype(np.int64), res.n_llp, (win.astype(np.int64) if want_win else None), res


def port_run(xyz, bbox, W: int, O: float, B: int, policy: int = 1, max_number: int = 32, min_radius: float = 0.1,
             level: int = 5, nthreads: int = 1):
    """C port of the reference algorithm: (seeds = stage-3 ids ++ LLPs, n_llp, t_tree s, t_owm s)."""
    a = np.ascontiguousarray(xyz, dtype=np.float64)
    p = params(bbox, a.shape[0], W, O, B)
    out = np.empty(p.ncells + max(p.ngrid, 0) + 1, dtype=np.int64)
    nllp, tt, to = C.c_int64(), C.c_double(), C.c_double()
    n = _port().refport_run(_d(a), a.shape[0], _d(_bbox_arr(bbox)), W, O, B, policy, max_number, min_radius, level, nthreads,
                            _q(out), out.size, C.byref(nllp), C.byref(tt), C.byref(to))
    if n < 0:
        raise RuntimeError("reference port run failed")
    return out[:n].copy(), nllp.value, tt.value, to.value


def xyz_parse(text: bytes):
    """readXYZfile's rules on .xyz text (oracle_xyz_parse): (points [n, 3],
    bbox (min_x, min_y, max_x, max_y), has_header), or None where the loader
    fails."""
    o = _oracle()
    cap = text.count(b"\n") + 2
    out = np.empty((cap, 3), dtype=np.float64)
    n = C.c_int64()
    bb = np.zeros(4, dtype=np.float64)
    hh = C.c_int()
    rc = o.oracle_xyz_parse(bytes(text), len(text), _d(out), cap, C.byref(n), _d(bb), C.byref(hh))
    if rc != 0:
        return None
    return out[: n.value].copy(), tuple(bb.tolist()), bool(hh.value)


def ref_check_results(gold_path: str, xyz, ids, displace: float) -> float:
    """The reference's own check_results on a gold file (percentage)."""
    a = np.ascontiguousarray(xyz, dtype=np.float64)
    i = np.ascontiguousarray(ids, dtype=np.int32)
    return _ref().owmref_check_results(str(gold_path).encode(), _d(a), a.shape[0],
                                        i.ctypes.data_as(C.POINTER(C.c_int)), i.size, displace)


def ref_read_xyz(path: str, cap: int):
    """The reference's own readXYZfile on a header file (its name must carry
    one of the reference's header names, e.g. ...ArzuaH.xyz): (points, bbox)
    or None where it fails."""
    r = _ref()
    out = np.empty((cap, 3), dtype=np.float64)
    n = C.c_int64()
    bb = np.zeros(4, dtype=np.float64)
    rc = r.owmref_read_xyz(str(path).encode(), _d(out), cap, C.byref(n), _d(bb))
    if rc != 0:
        return None
    return out[: n.value].copy(), tuple(bb.tolist())
