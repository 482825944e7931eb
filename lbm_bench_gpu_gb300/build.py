"""Build liblbm_gb300.so (sm_103a) in-tree with nvcc.

Each translation unit of ``csrc/`` is compiled in parallel into ``_build/``,
then linked into ``lbm_bench_gpu_gb300/liblbm_gb300.so`` (CUDA runtime linked
statically, so the library has no runtime path dependency).  The C++ host
driver ``lbm_zsc`` is linked against it.

Usage: ``python -m lbm_bench_gpu_gb300.build [--force]``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "liblbm_gb300.so"
DRIVER = PKG / "bin" / "lbm_zsc"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", *ARCH, "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE), "-I", str(CSRC)]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I", str(INCLUDE), "-I", str(CSRC)]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def cuda_include() -> str:
    return str(Path(nvcc()).resolve().parent.parent / "include")


def _sources() -> list[Path]:
    return sorted(p for p in CSRC.iterdir() if p.suffix in (".cu", ".cpp"))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, force: bool) -> tuple[Path, str]:
    obj = BUILD / (src.name + ".o")
    if not force and not _stale(obj, [src, *_headers()]):
        return obj, ""
    if src.suffix == ".cu":
        cmd = [nvcc(), *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXX_FLAGS, "-I", cuda_include(), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA/C++ source and link the shared library; returns its path."""
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    if verbose:
        for _, log in results:
            if log:
                print(log)
    objs = [o for o, _ in results]
    if force or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(LIB), *map(str, objs)]
        subprocess.run(cmd, check=True)
    driver_src = PKG / "driver" / "lbm_zsc.cpp"
    if driver_src.exists() and (force or _stale(DRIVER, [driver_src, LIB, *_headers()])):
        DRIVER.parent.mkdir(exist_ok=True)
        cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", str(INCLUDE), str(driver_src), "-o", str(DRIVER),
               "-L", str(PKG), "-llbm_gb300", "-Wl,-rpath,$ORIGIN/.."]
        subprocess.run(cmd, check=True)
    return LIB


CHECKED_BUILD = PKG / "_build_checked"
CHECKED_LIB = PKG / "liblbm_gb300_checked.so"


def build_checked(force: bool = False) -> Path:
    """The library with ZSC_CHECKED=1 (every global store and cp.async source of
    the step kernel checked against its field; an index outside it sets an error
    bit and the access is skipped), for tests; returns its path."""
    CHECKED_BUILD.mkdir(exist_ok=True)
    srcs = _sources()

    def one(src: Path) -> Path:
        obj = CHECKED_BUILD / (src.name + ".o")
        if not force and not _stale(obj, [src, *_headers()]):
            return obj
        if src.suffix == ".cu":
            cmd = [nvcc(), *NVCC_FLAGS, "-DZSC_CHECKED=1", "-c", str(src), "-o", str(obj)]
        else:
            cmd = ["g++", *CXX_FLAGS, "-I", cuda_include(), "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(one, srcs))
    if force or _stale(CHECKED_LIB, objs):
        subprocess.run([nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(CHECKED_LIB), *map(str, objs)],
                       check=True)
    return CHECKED_LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
