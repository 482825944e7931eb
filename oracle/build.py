"""Build recipe for the test oracles (test infrastructure only).

* ``build_oracle()`` compiles ``oracle/zsc_oracle.c`` (the FP64 restatement)
  into ``oracle/_build/libzsc_oracle.so``.
* ``build_reference()`` compiles the reference's own step kernels for the host
  CPU (``oracle/ref_harness/zsc_ref_cpu.cpp`` + the reference sources, through
  the CUDA/MPI emulation shim) into ``oracle/_ref/libzsc_ref.so``.
* ``build_reference_cuda()`` compiles the reference's own CUDA program
  (``src/main.cu``, unmodified, with its ``src/Makefile`` flags ``-O3
  -use_fast_math``) for sm_103a against a single-rank MPI stub
  (``oracle/ref_harness/mpi_stub/mpi.h``) into ``oracle/_ref/lbm_ref_cuda``:
  the reference's GPU step, timed beside the product as a baseline.  CUDA 13
  no longer declares ``cudaThreadSynchronize``; it is mapped to
  ``cudaDeviceSynchronize`` on the command line.  The same program is also
  built without ``-use_fast_math`` (``oracle/_ref/lbm_ref_cuda_exact``), to
  separate the fast-math share of its differences from this library.

The reference sources are read from ``$LBM_REFERENCE_SRC``, else from the
checkout this recipe was written against (``CHECKOUT_SRC``; this file is the
only one that names it).  Where that directory exists the recipe first stages
an unmodified copy of the files it needs into ``oracle/_ref/src``, and the
reference's sample ``Input/`` files into ``oracle/_ref/Input`` (ignored by git;
a machine without the checkout, such as the GPU host, builds from the staged
copy, and the tests read the staged copy only).  Nothing is
patched: inputs with more bubbles than the reference's MAX_BUBBLES are fed in
as a phi field instead (see ``zr_init``).

* ``build_reference_dump()`` builds the same program with
  ``oracle/ref_harness/field_dump.c`` standing in for ``src/vtksave.c`` (same
  signature; binary phi, rho, u at chosen steps) into
  ``oracle/_ref/lbm_ref_cuda_dump`` and ``oracle/_ref/lbm_ref_cuda_exact_dump``,
  for node-by-node parity with the reference's GPU fields.

Usage: ``python oracle/build.py [oracle|reference|reference_cuda|reference_dump|all]``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
REF_DIR = HERE / "_ref"
REF_STAGE = REF_DIR / "src"
ORACLE_SO = BUILD_DIR / "libzsc_oracle.so"
REF_SO = REF_DIR / "libzsc_ref.so"

CHECKOUT_SRC = "/root/reference/src"
REF_INPUT_STAGE = REF_DIR / "Input"

# Files of the reference that zsc_ref_cpu.cpp includes (src/main.cu:44-74 minus
# the VTK writer).
REFERENCE_FILES = [
    "constants.h", "gridid.c", "init.c", "paramread.c", "logsave.c", "stats.c",
    "mpiupdate.c", "mpiupdate_f.c", "mpiupdate_phi.c", "vgrid.c",
    "init_f.cu", "init_g.cu", "update_phi.cu", "update_rho.cu", "update_velocity.cu",
    "collision_f.cu", "collision_g.cu", "pack_mpi.cu", "pack_mpi_f.cu", "pack_mpi_phi.cu",
    "stream_f.cu", "stream_g.cu", "unpack_mpi.cu", "unpack_mpi_f.cu", "unpack_mpi_phi.cu",
]
# ... and what src/main.cu adds for the GPU program.
REFERENCE_CUDA_FILES = ["main.cu", "vtksave.c"]
REF_CUDA_BIN = REF_DIR / "lbm_ref_cuda"               # src/Makefile's flags
REF_CUDA_EXACT_BIN = REF_DIR / "lbm_ref_cuda_exact"   # the same without -use_fast_math
# The same program with ref_harness/field_dump.c in place of src/vtksave.c:
# binary phi, rho, u at the steps LBM_DUMP_STEPS names, for per-node parity.
REF_DUMP_STAGE = REF_DIR / "src_dump"
REF_CUDA_DUMP_BIN = REF_DIR / "lbm_ref_cuda_dump"
REF_CUDA_EXACT_DUMP_BIN = REF_DIR / "lbm_ref_cuda_exact_dump"

# Deterministic IEEE float arithmetic on x86-64 and aarch64 alike: no
# contraction into fused multiply-adds, no fast-math.
COMMON_FLAGS = ["-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off"]


def _newer(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(s.exists() and s.stat().st_mtime <= t for s in sources)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "zsc_oracle.c"
    BUILD_DIR.mkdir(exist_ok=True)
    if force or not _newer(ORACLE_SO, [src]):
        cmd = ["gcc", *COMMON_FLAGS, "-std=c11", "-D_DEFAULT_SOURCE", str(src), "-o", str(ORACLE_SO), "-lm"]
        subprocess.run(cmd, check=True)
    return ORACLE_SO


def reference_src_dir() -> Path | None:
    """Directory holding the reference sources: the checkout, else the staged copy."""
    env = os.environ.get("LBM_REFERENCE_SRC", CHECKOUT_SRC)
    p = Path(env)
    if all((p / f).exists() for f in REFERENCE_FILES):
        return p
    if all((REF_STAGE / f).exists() for f in REFERENCE_FILES):
        return REF_STAGE
    return None


def stage_reference() -> Path | None:
    """Copy the needed reference files, unmodified, into oracle/_ref/src."""
    p = Path(os.environ.get("LBM_REFERENCE_SRC", CHECKOUT_SRC))
    if not all((p / f).exists() for f in REFERENCE_FILES):
        return REF_STAGE if all((REF_STAGE / f).exists() for f in REFERENCE_FILES) else None
    REF_STAGE.mkdir(parents=True, exist_ok=True)
    for f in REFERENCE_FILES + [f for f in REFERENCE_CUDA_FILES if (p / f).exists()]:
        dst = REF_STAGE / f
        if not dst.exists() or dst.read_bytes() != (p / f).read_bytes():
            shutil.copyfile(p / f, dst)
    sample = p.parent / "Input"
    for f in ("properties.in", "discrete.in"):
        if (sample / f).exists():
            REF_INPUT_STAGE.mkdir(parents=True, exist_ok=True)
            if not (REF_INPUT_STAGE / f).exists() or (REF_INPUT_STAGE / f).read_bytes() != (sample / f).read_bytes():
                shutil.copyfile(sample / f, REF_INPUT_STAGE / f)
    return REF_STAGE


def build_reference(force: bool = False) -> Path | None:
    """Compile the reference's kernels for the CPU; None if its sources are absent."""
    stage_reference()
    src_dir = reference_src_dir()
    if src_dir is None:
        return None
    harness = HERE / "ref_harness" / "zsc_ref_cpu.cpp"
    shim = HERE / "ref_harness" / "ref_shim.h"
    deps = [harness, shim] + [src_dir / f for f in REFERENCE_FILES]
    REF_DIR.mkdir(exist_ok=True)
    if force or not _newer(REF_SO, deps):
        cmd = ["g++", *COMMON_FLAGS, "-std=c++17", "-w", "-fvisibility=hidden", "-include", str(shim),
               "-I", str(src_dir), "-I", str(shim.parent), str(harness), "-o", str(REF_SO), "-lm"]
        subprocess.run(cmd, check=True)
    return REF_SO


def build_reference_cuda(force: bool = False) -> Path | None:
    """Compile the reference's CUDA program for sm_103a; None if its sources or nvcc are absent."""
    stage_reference()
    src_dir = reference_src_dir()
    if src_dir is None or not all((src_dir / f).exists() for f in REFERENCE_CUDA_FILES):
        return None
    deps = [src_dir / f for f in REFERENCE_FILES + REFERENCE_CUDA_FILES]
    REF_DIR.mkdir(exist_ok=True)
    jobs = _nvcc_jobs(src_dir, ((REF_CUDA_BIN, ["-O3", "-use_fast_math"]), (REF_CUDA_EXACT_BIN, ["-O3"])), deps,
                      force)
    if jobs is None:
        return None
    for cmd, job in jobs:
        if job.wait() != 0:
            raise subprocess.CalledProcessError(job.returncode, cmd)
    return REF_CUDA_BIN


def _nvcc_jobs(src_dir: Path, outputs, deps, force: bool):
    """Start one nvcc per (binary, flags) that is out of date; returns the jobs."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        return None
    stub = HERE / "ref_harness" / "mpi_stub" / "mpi.h"
    jobs = []
    for out, flags in outputs:
        if force or not _newer(out, deps + [stub]):
            cmd = [nvcc, *flags, "-gencode", "arch=compute_103a,code=sm_103a", "-w",
                   "-DcudaThreadSynchronize=cudaDeviceSynchronize", "-include", "stdlib.h",
                   "-I", str(stub.parent), "-I", str(src_dir), str(src_dir / "main.cu"), "-o", str(out)]
            jobs.append((cmd, subprocess.Popen(cmd)))
    return jobs


def build_reference_dump(force: bool = False) -> Path | None:
    """The reference's CUDA program with ref_harness/field_dump.c as its VTK
    writer: every other file is the reference's, unmodified, staged into
    oracle/_ref/src_dump.  None if the sources or nvcc are absent."""
    stage_reference()
    src_dir = reference_src_dir()
    if src_dir is None or not all((src_dir / f).exists() for f in REFERENCE_CUDA_FILES):
        return None
    writer = HERE / "ref_harness" / "field_dump.c"
    REF_DUMP_STAGE.mkdir(parents=True, exist_ok=True)
    for f in REFERENCE_FILES + ["main.cu"]:
        dst = REF_DUMP_STAGE / f
        if not dst.exists() or dst.read_bytes() != (src_dir / f).read_bytes():
            shutil.copyfile(src_dir / f, dst)
    dst = REF_DUMP_STAGE / "vtksave.c"
    if not dst.exists() or dst.read_bytes() != writer.read_bytes():
        shutil.copyfile(writer, dst)
    deps = [REF_DUMP_STAGE / f for f in REFERENCE_FILES + REFERENCE_CUDA_FILES]
    jobs = _nvcc_jobs(REF_DUMP_STAGE, ((REF_CUDA_DUMP_BIN, ["-O3", "-use_fast_math"]),
                                       (REF_CUDA_EXACT_DUMP_BIN, ["-O3"])), deps, force)
    if jobs is None:
        return None
    for cmd, job in jobs:
        if job.wait() != 0:
            raise subprocess.CalledProcessError(job.returncode, cmd)
    return REF_CUDA_DUMP_BIN


def main(argv: list[str]) -> int:
    what = argv[1] if len(argv) > 1 else "all"
    if what in ("oracle", "all"):
        print(build_oracle(force=True))
    if what in ("reference", "all"):
        print(build_reference(force=True) or "reference sources not found")
    if what in ("reference_cuda", "all"):
        print(build_reference_cuda(force=True) or "reference sources or nvcc not found")
    if what in ("reference_dump", "all"):
        print(build_reference_dump(force=True) or "reference sources or nvcc not found")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
