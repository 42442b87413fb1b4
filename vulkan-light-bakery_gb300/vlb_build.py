"""Builds libvlb.so (sm_103a kernels + host C++ behind the C ABI) in-tree.

Each translation unit compiles in parallel; an object is rebuilt only when a
source or header is newer.  Output: vulkan-light-bakery_gb300/_build/libvlb.so
(git-ignored).  Also builds the oracle under oracle/_build (and the reference
header shim under oracle/_ref when the reference checkout exists) -- those are
test infrastructure, built here only so one call prepares a machine.  The
shim needs the reference checkout: set VLB_REFERENCE_DIR to its root (no
default; without it the shim is skipped and the tests use the committed
fixtures alone).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libvlb.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
_REF_DIR = os.environ.get("VLB_REFERENCE_DIR")
REFERENCE = Path(_REF_DIR) if _REF_DIR else None


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


BOUNDS_BUILD = PKG / "_build_bounds"


def build_library(verbose: bool = False, extra_nvcc: list[str] | None = None, bounds_check: bool = False) -> Path:
    """bounds_check: the bounds-check variant (-DVLB_BOUNDS_CHECK: every
    data-dependent device index is checked and counted instead of used) in
    _build_bounds/libvlb.so; load it with VLB_LIB."""
    build = BOUNDS_BUILD if bounds_check else BUILD
    lib_path = build / "libvlb.so"
    defs = ["-DVLB_BOUNDS_CHECK"] if bounds_check else []
    build.mkdir(exist_ok=True)
    nvcc = _nvcc()
    inc = _cuda_home() / "include"
    # every object also depends on this file (its compiler flags)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [REPO / "include" / "vlb.h", Path(__file__)]
    jobs = []
    for cu in sorted(CSRC.glob("*.cu")):
        obj = build / (cu.stem + ".o")
        # -fmad=false: device arithmetic exactly as written (explicit fmaf stays fused), so a ray's
        # FP32 decisions do not depend on how a build schedules or allocates registers
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
               "-ffp-contract=off", *defs, *(extra_nvcc or []), "-c", str(cu), "-o", str(obj)]
        jobs.append((obj, [cu, *headers], cmd))
    for cpp in sorted(CSRC.glob("*.cpp")):
        obj = build / (cpp.stem + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", *defs, f"-I{inc}", "-c", str(cpp),
               "-o", str(obj)]
        jobs.append((obj, [cpp, *headers], cmd))
    todo = [(o, c) for o, d, c in jobs if _stale(o, d)]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        for _ in ex.map(lambda oc: _run(oc[1]), todo):
            pass
    objs = [str(o) for o, _, _ in jobs]
    if todo or not lib_path.exists():
        tmp = build / "libvlb.so.tmp"
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
        os.replace(tmp, lib_path)
    if verbose:
        print(f"built {lib_path} ({len(todo)} objects rebuilt)")
    return lib_path


def build_oracle(verbose: bool = False) -> Path:
    src = REPO / "oracle" / "vlb_oracle.cpp"
    out = REPO / "oracle" / "_build" / "liboracle.so"
    out.parent.mkdir(exist_ok=True)
    if _stale(out, [src]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-shared", "-o", str(out),
              str(src)])
    hdr = REFERENCE / "shaders" / "sh_common.h" if REFERENCE else None
    if hdr is not None and hdr.exists():
        shim = REPO / "oracle" / "ref_shim.cpp"
        ref = REPO / "oracle" / "_ref" / "libshref.so"
        ref.parent.mkdir(exist_ok=True)
        if _stale(ref, [shim, hdr]):
            _run(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-shared",
                  f"-I{REFERENCE / 'shaders'}", "-o", str(ref), str(shim)])
    if verbose:
        print(f"built {out}")
    return out


CLI = BUILD / "vlb-bake"


def build_cli(verbose: bool = False) -> Path:
    """The vlb-bake executable (cli/vlb_bake.cpp) linked to libvlb.so, found
    next to it at run time."""
    src = PKG / "cli" / "vlb_bake.cpp"
    if _stale(CLI, [src, LIB, REPO / "include" / "vlb.h"]):
        tmp = BUILD / "vlb-bake.tmp"
        _run(["g++", "-O2", "-std=c++17", "-Wall", f"-I{REPO / 'include'}", "-o", str(tmp), str(src),
              f"-L{BUILD}", "-lvlb", "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, CLI)
    if verbose:
        print(f"built {CLI}")
    return CLI


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, verbose)
        f2 = ex.submit(build_oracle, verbose)
        f1.result()
        f2.result()
    build_cli(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
