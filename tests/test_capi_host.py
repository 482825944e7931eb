"""Host-side checks of liblbm_gb300.so that need no GPU: the library loads and
exports every entry point of include/lbm_gb300.h, parses the reference's input
format like src/paramread.c, derives the same constants, and rejects bad input
with a status code before touching the device."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT

HEADER = ROOT / "include" / "lbm_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(lbm_\w+)\s*\(", text, re.M)))


def test_header_declares_core_entry_points():
    names = declared_functions()
    for n in ("lbm_init", "lbm_step", "lbm_stats", "lbm_destroy", "lbm_strerror", "lbm_read_inputs"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in lbm_gb300.h but not exported"
    from lbm_bench_gpu_gb300 import capi
    assert set(capi.EXPORTS) == set(declared_functions())


def test_read_inputs_matches_reference_parser(golden_manifest, tmp_path):
    from lbm_bench_gpu_gb300 import capi
    case = golden_manifest["sample_ratio"]
    (tmp_path / "properties.in").write_text(case["properties.in"])
    (tmp_path / "discrete.in").write_text(case["discrete.in"])
    p, run, bub = capi.read_inputs(tmp_path)
    assert (p.nx, p.ny, p.nz, p.block_x, p.block_y) == (64, 32, 16, 32, 8)
    assert (p.rhoL, p.rhoH, p.tauRho) == (1.0, 1000.0, 1.0)
    assert p.tauPhi == np.float32(0.7) and p.sigma == np.float32(0.01) and p.Gamma == 400.0 and p.Eo == 10.0
    assert bub.shape == (1, 4) and p.rc0 == 5.0
    d = capi.derive(p)
    for k, v in case["ref_constants"].items():
        mine = getattr(d, {"Wn0": "K0"}.get(k, k))
        assert mine == pytest.approx(v, rel=5e-7, abs=1e-30), k


def test_read_inputs_reference_sample():
    """The reference's own sample Input/ files, as oracle/build.py stages them."""
    from oracle.build import REF_INPUT_STAGE, stage_reference
    stage_reference()
    src = REF_INPUT_STAGE
    if not (src / "properties.in").exists():
        pytest.skip("reference sample inputs not staged (no checkout on this machine)")
    from lbm_bench_gpu_gb300 import capi
    p, run, bub = capi.read_inputs(src)
    assert (run.max_step, run.relax_step, run.save, run.stat) == (1000, 1000, 2000, 100)
    assert (p.nx, p.ny, p.nz) == (128, 128, 128)
    assert p.rhoH == 1000.0 and p.Gamma == 400.0 and p.Eo == 10.0
    assert bub.tolist() == [[64.0, 64.0, 64.0, 10.0]]


def test_missing_and_malformed_inputs(tmp_path):
    from lbm_bench_gpu_gb300 import capi
    with pytest.raises(capi.LbmError) as e:
        capi.read_inputs(tmp_path)
    assert e.value.code == capi.LBM_EIO
    (tmp_path / "properties.in").write_text("maxStep relaxStep save stat\n10 0 1 1\nxmax ymax zmax\n32 32\n")
    (tmp_path / "discrete.in").write_text("nBubbles\n0\nxc yc zc Rc\n")
    with pytest.raises(capi.LbmError) as e:
        capi.read_inputs(tmp_path)
    assert e.value.code == capi.LBM_EIO


def test_discrete_with_missing_rows(tmp_path):
    from lbm_bench_gpu_gb300 import capi, inputs
    inputs.write_inputs(tmp_path, inputs.Inputs(nx=32, ny=32, nz=32,
                                                bubbles=np.array([[1, 2, 3, 4]], np.float32)))
    (tmp_path / "discrete.in").write_text("nBubbles\n3\nxc yc zc Rc\n1 2 3 4\n")
    with pytest.raises(capi.LbmError) as e:
        capi.read_inputs(tmp_path)
    assert e.value.code == capi.LBM_EIO


@pytest.mark.parametrize("change,code", [
    (dict(nx=48), 1),                      # nx not a multiple of 32
    (dict(ny=12), 1),                      # ny not a multiple of 8
    (dict(ny=40, compat=True), 1),         # compat: NY % 32 (src/main.cu:168)
    (dict(block_x=64, block_y=16, compat=True), 1),  # compat: BLOCK_SIZE_X*Y > 512 (src/main.cu:171)
    (dict(tauRho=0.0), 1),
    (dict(rhoH=0.1), 1),                   # rhoH == rhoL: phiStar = 0
    (dict(storage=7, nx=32), 1),           # unknown storage format
    (dict(nz=2), 1),
])
def test_init_rejects_bad_params_without_touching_the_gpu(change, code):
    from lbm_bench_gpu_gb300 import capi
    kw = dict(rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=1.0, width=4.0, sigma=1e-3, Gamma=1.0)
    dims = dict(nx=32, ny=32, nz=32)
    for k in ("nx", "ny", "nz"):
        if k in change:
            dims[k] = change.pop(k)
    kw.update(change)
    storage = kw.pop("storage", None)
    p = capi.make_params(dims["nx"], dims["ny"], dims["nz"], **kw)
    if storage is not None:
        p.storage = storage
    phi = np.zeros(p.nx * p.ny * p.nz, np.float32)
    with pytest.raises(capi.LbmError) as e:
        capi.Lattice.from_fields(p, phi, phi + 0.55)
    assert e.value.code == code


@pytest.mark.parametrize("dims,change", [
    ((1024, 1024, 256), {}),                 # 19 n >= 2^32: beyond 32-bit element indexing
    ((32, 32, 32), dict(width=0.0)),
    ((32, 32, 32), dict(tauPhi=-1.0)),
    ((32, 32, 32), dict(Eo=1.0, rc0=0.0)),   # gravity from Eo needs a positive Rc0
])
def test_init_bubbles_rejects_bad_params_without_touching_the_gpu(dims, change):
    from lbm_bench_gpu_gb300 import capi
    kw = dict(rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=1.0, width=4.0, sigma=1e-3, Gamma=1.0)
    kw.update(change)
    p = capi.make_params(*dims, **kw)
    # validation comes before any CUDA call: here, without a GPU, anything
    # that got past it would fail with a CUDA error code instead
    with pytest.raises(capi.LbmError) as e:
        capi.Lattice.from_bubbles(p, np.zeros((0, 4), np.float32))
    assert e.value.code == capi.LBM_EINVAL


def test_strerror_covers_codes(lib):
    from lbm_bench_gpu_gb300 import capi
    for code in range(8):
        assert lib.lbm_strerror(code).decode()
    assert lib.lbm_strerror(99).decode() == "unknown status"


def test_null_context_is_rejected(lib):
    from lbm_bench_gpu_gb300 import capi
    assert lib.lbm_step(None, 1, C.c_float(0.0)) == capi.LBM_EINVAL
    assert lib.lbm_sync(None) == capi.LBM_EINVAL
    assert lib.lbm_steps_done(None) == -1
    lib.lbm_destroy(None)


def test_bubble_placement_rules():
    from lbm_bench_gpu_gb300 import inputs
    b = inputs.place_bubbles(64, (256, 256, 256), (6.0, 10.0))
    assert b.shape == (64, 4)
    assert np.array_equal(b, inputs.place_bubbles(64, (256, 256, 256), (6.0, 10.0)))  # seeded
    r = b[:, 3]
    assert r.min() >= 6.0 and r.max() <= 10.0
    c = b[:, :3].astype(np.float64)
    d = np.linalg.norm(c[:, None] - c[None], axis=-1)
    gap = d - (r[:, None] + r[None])
    np.fill_diagonal(gap, np.inf)
    assert gap.min() >= 3.0 - 1e-3
    m = r + 4.0 + 1.0
    assert np.all(c[:, 0] >= m) and np.all(c[:, 0] <= 255 - m)
    assert np.all(c[:, 2] >= 1 + m) and np.all(c[:, 2] <= 256 - m)


def test_integration_examples_compile_and_link(lib, tmp_path):
    """The C examples of INTEGRATION.md (the reference's main loop on the C-ABI,
    the adjoint calls and the one-process z-slab loop) compile with -Wall -Werror against the header and
    link against the library: what a maintainer of the reference would build."""
    import re
    import shutil
    import subprocess
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    blocks = re.findall(r"```c\n(.*?)```", (root / "INTEGRATION.md").read_text(), re.S)
    assert len(blocks) >= 2
    cc = shutil.which("cc") or shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    main_c = tmp_path / "main_loop.c"
    main_c.write_text(blocks[0])
    adjoint_c = tmp_path / "adjoint.c"
    adjoint_c.write_text(
        "#include <stdio.h>\n#include \"lbm_gb300.h\"\n"
        "#define CHECK(x) do { int rc_ = (x); if (rc_) { fprintf(stderr, \"%s\\n\", lbm_strerror(rc_)); "
        "return 1; } } while (0)\n"
        "int adjoint_example(lbm_ctx *c, lbm_derived d, float *grad)\n{\n" + blocks[1] + "    return 0;\n}\n")
    # the one-process z-slab loop, inside a function with the main loop's variables
    slab_block = next(b for b in blocks if "lbm_split_z(" in b)
    slab_c = tmp_path / "slabs.c"
    slab_c.write_text(
        "#include <stdio.h>\n#include \"lbm_gb300.h\"\n"
        "#define CHECK(x) do { int rc_ = (x); if (rc_) { fprintf(stderr, \"%s\\n\", lbm_strerror(rc_)); "
        "return 1; } } while (0)\n"
        "int slab_example(lbm_params p, lbm_run run, lbm_derived d, const float *bubbles, int nb)\n{\n"
        "    lbm_stats_out s;\n" + slab_block + "    lbm_destroy(whole);\n    return 0;\n}\n")
    pkg = root / "lbm_bench_gpu_gb300"
    for src in (main_c, adjoint_c, slab_c):
        args = [cc, "-std=c99", "-Wall", "-Werror", str(src), "-I", str(root / "include")]
        if src is main_c:
            args += ["-L", str(pkg), "-llbm_gb300", "-o", str(tmp_path / "main_loop")]
        else:
            args += ["-c", "-o", str(tmp_path / (src.stem + ".o"))]
        r = subprocess.run(args, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_every_context_entry_point_holds_the_context_device():
    """Each C-ABI function that takes a context and queues or waits for its
    work makes the context's device current for the call and gives the caller
    its own current device back (lbm::DeviceGuard / LBM_ON_DEVICE): a caller
    whose thread has another GPU current still reaches the context.  Checked
    on the sources, since one GPU cannot show a device mix-up."""
    import re
    csrc = Path(__file__).resolve().parents[1] / "lbm_bench_gpu_gb300" / "csrc"
    # no device work, or only through other guarded entry points
    no_device_work = {"lbm_state_bytes", "lbm_steps_done", "lbm_stream", "lbm_halo_bytes", "lbm_slab_stats"}
    seen = set()
    for src in sorted(csrc.glob("*.cu")):
        text = src.read_text()
        for m in re.finditer(r'extern "C" [\w\s\*]*?\b(lbm_\w+)\(([^)]*)\)\s*\{', text):
            name, args = m.group(1), m.group(2)
            if "lbm_ctx" not in args or name in no_device_work:
                continue
            depth, i = 1, m.end()
            while depth:
                depth += {"{": 1, "}": -1}.get(text[i], 0)
                i += 1
            body = text[m.end():i]
            assert "LBM_ON_DEVICE" in body or "DeviceGuard" in body, f"{src.name}: {name} does not hold the device"
            seen.add(name)
    for name in ("lbm_step", "lbm_stats", "lbm_get_dist", "lbm_set_dist", "lbm_save_state", "lbm_load_state",
                 "lbm_sync", "lbm_destroy", "lbm_step_adjoint", "lbm_objective", "lbm_init", "lbm_init_bubbles"):
        assert name in seen, name


def test_stats_combine_adds_sums_and_counts_and_takes_maxima(lib):
    """lbm_stats_combine (host only): the per-slab raw statistics of a box add
    up, apart from the two max |u|^2 entries, and the compat means divide by
    the whole box (Pout by nx*ny*nz - vol, src/logsave.c:158-160)."""
    import numpy as np
    from lbm_bench_gpu_gb300 import capi
    p = capi.make_params(32, 8, 12, rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=1.0, width=4.0, sigma=1e-3, Gamma=1.0,
                         Eo=-0.4, rc0=5.0)
    a = np.linspace(1.0, 16.0, 16)
    b = np.linspace(0.5, 40.0, 16)
    a[14] = b[14] = 0.0          # no non-finite nodes
    s = capi.stats_combine(p, 7, np.stack([a, b]))
    r = a + b
    r[0], r[13] = max(a[0], b[0]), max(a[13], b[13])
    n = 32 * 8 * 12
    assert s["step"] == 7
    assert s["vol"] == r[1] and s["vol_full"] == r[12]
    assert s["umax"] == pytest.approx(np.sqrt(r[0])) and s["umax_full"] == pytest.approx(np.sqrt(r[13]))
    assert s["uz_av"] == pytest.approx(r[4] / r[1])
    assert s["p_in"] == pytest.approx(r[5] / r[1]) and s["p_out"] == pytest.approx(r[6] / (n - r[1]))
    assert s["phi_sum"] == r[7] and s["rho_sum"] == r[8] and s["mom_z"] == r[11]


def test_slab_init_rejects_bad_requests_without_touching_the_gpu(lib):
    """lbm_slab_maxabs / lbm_slab_init_bubbles check the slab's planes and the
    16-bit maxima before any CUDA call."""
    import ctypes as C
    from lbm_bench_gpu_gb300 import capi
    lib_ = capi.load()
    BUB = np.array([[30.3, 14.2, 21.7, 9.0], [8.5, 22.1, 40.2, 6.0], [50.0, 8.0, 3.5, 5.0]], np.float32)

    def params(shape, storage):
        return capi.make_params(*shape, storage=storage, rhoL=0.1, rhoH=1.0, tauRho=0.8, tauPhi=0.9, width=4.0,
                                sigma=1e-3, Gamma=1.0, Eo=-0.8, rc0=9.0)

    m = np.zeros(26, np.float32)
    h = C.c_void_p()
    for storage in ("fp32", "fp16"):
        p = params((64, 32, 48), storage)
        for z0, depth in ((-1, 8), (40, 9), (0, 1), (47, 2)):
            assert lib_.lbm_slab_maxabs(C.byref(p), capi.fptr(BUB), 3, z0, depth, capi.fptr(m)) == capi.LBM_EINVAL
            assert lib_.lbm_slab_init_bubbles(C.byref(h), C.byref(p), capi.fptr(BUB), 3, z0, depth,
                                              capi.fptr(m)) == capi.LBM_EINVAL
    # 16-bit storage without the box's maxima
    p = params((64, 32, 48), "fp16")
    assert lib_.lbm_slab_init_bubbles(C.byref(h), C.byref(p), capi.fptr(BUB), 3, 0, 24, None) == capi.LBM_EINVAL
    assert not h.value


def test_integration_per_rank_examples_compile(tmp_path):
    """The per-rank z-slab examples of INTEGRATION.md (the halo exchange over
    MPI, the step with its interior between pack and unpack, the statistics
    reduced over the ranks, each rank's own slab) compile with -Wall -Werror
    against the header, the CUDA runtime header and MPI's declarations."""
    import re
    import shutil
    import subprocess
    root = Path(__file__).resolve().parents[1]
    cc = shutil.which("cc") or shutil.which("gcc")
    cuda_inc = Path("/usr/local/cuda/include")
    if cc is None or not (cuda_inc / "cuda_runtime_api.h").exists():
        pytest.skip("no C compiler or CUDA headers")
    blocks = re.findall(r"```c\n(.*?)```", (root / "INTEGRATION.md").read_text(), re.S)
    rank_blocks = [b for b in blocks if "MPI_Sendrecv" in b or "lbm_slab_maxabs" in b]
    assert len(rank_blocks) == 2
    prelude = (
        "#include <stdio.h>\n#include <cuda_runtime_api.h>\n#include \"lbm_gb300.h\"\n"
        "typedef int MPI_Comm; typedef int MPI_Datatype; typedef int MPI_Op; typedef struct { int s; } MPI_Status;\n"
        "#define MPI_BYTE 1\n#define MPI_FLOAT 2\n#define MPI_DOUBLE 3\n#define MPI_SUM 1\n#define MPI_MAX 2\n"
        "#define MPI_STATUS_IGNORE ((MPI_Status *)0)\n"
        "int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *, int, MPI_Datatype, int, int, MPI_Comm,"
        " MPI_Status *);\n"
        "int MPI_Reduce(const void *, void *, int, MPI_Datatype, MPI_Op, int, MPI_Comm);\n"
        "int MPI_Allreduce(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm);\n"
        "#define CHECK(x) do { int rc_ = (x); if (rc_) { fprintf(stderr, \"%s\\n\", lbm_strerror(rc_)); return 1; } }"
        " while (0)\n")
    src = tmp_path / "ranks.c"
    src.write_text(prelude + "\n".join(rank_blocks))
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-c", str(src), "-I", str(root / "include"),
                        "-I", str(cuda_inc), "-o", str(tmp_path / "ranks.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
