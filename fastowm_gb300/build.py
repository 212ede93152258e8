"""Build recipe of the native library ``fastowm_gb300/libowm_gb300.so``.

Compiles every ``csrc/*.cu`` for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``), every ``csrc/*.cpp`` with g++ and every
``csrc/*.c`` with gcc, in parallel, into ``fastowm_gb300/_build/`` and links one shared library in the
package directory.  Host code is compiled with ``-ffp-contract=off`` so the
parameter arithmetic and the synthetic generator give the same bits on
x86-64 and aarch64.  Rebuilds only what changed (sources or headers newer
than the object).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT = PKG / "_build"
LIB = PKG / "libowm_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libowm_gb300.so")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _compile(cmd: list[str]) -> tuple[list[str], int, str]:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    return cmd, r.returncode, r.stdout


def build(verbose: bool = False, jobs: int | None = None, force: bool = False) -> Path:
    """Compile and link; returns the library path."""
    nvcc = _nvcc()
    OUT.mkdir(exist_ok=True)
    deps = _headers()
    cmds, objs = [], []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OUT / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            cmds.append([nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OUT / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            cmds.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread",
                         "-I", str(INCLUDE), "-I", str(Path(nvcc).resolve().parent.parent / "include"),
                         "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.c")):
        obj = OUT / (src.stem + ".c.o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            cmds.append(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-pthread", "-D_GNU_SOURCE",
                         "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    workers = jobs or min(8, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        for cmd, rc, out in ex.map(_compile, cmds):
            if verbose or rc:
                sys.stderr.write(" ".join(cmd) + "\n" + out)
            if rc:
                raise RuntimeError(f"compile failed: {cmd[-3]}")
    if force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [nvcc, "-shared", *ARCH, "-o", str(LIB), *map(str, objs), "-lpthread", "-lm"]
        _, rc, out = _compile(cmd)
        if verbose or rc:
            sys.stderr.write(" ".join(cmd) + "\n" + out)
        if rc:
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
