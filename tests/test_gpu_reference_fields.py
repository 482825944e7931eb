"""Node-by-node parity with the reference's own GPU program on this GPU.

oracle/_ref/lbm_ref_cuda_dump is the reference's src/main.cu built for
sm_103a with its src/Makefile flags (-O3 -use_fast_math) and a single-rank MPI
stub, with oracle/ref_harness/field_dump.c standing in for its VTK writer:
at the steps LBM_DUMP_STEPS names it writes the phi, rho, ux, uy, uz arrays it
has just copied back from the device, in full float precision.
oracle/_ref/lbm_ref_cuda_exact_dump is the same program without
-use_fast_math.  Both run relaxStep = 0 and 100 evolution steps with save = 1
from the same properties.in / discrete.in as this library's
lbm_init_bubbles; the fields after 0 (the initial state), 1, 10 and 100
steps are compared node by node:

* C1, the static bubble: 64^3, one bubble R = 12, no gravity;
* the short adjoint workload: 128^3, 8 bubbles R = 10, tau_rho = 0.8,
  gravity -1e-6.

Each run is also compared with the FP64 oracle stepped alongside.  Bounds:
phi and rho within 1e-5 of the field's largest magnitude (the spec bar
for FP32) and u within U_TOL (1e-6) absolute, after 0, 1 and 10 steps of both
cases and after 100 steps of the static bubble.  After 100 steps of the 128^3
bubbly flow under gravity two FP32 programs no longer agree to 1e-5: there the
reference's own build is 1.7e-5 (phi) from the FP64 oracle, this library
1.9e-5, and the two differ by 3.4e-5 from each other (both reference builds
alike, so fast math is not the cause; each program's rounding grows along the
flow).  At that point the bounds are 2.5e-5 (phi, rho) to the FP64 oracle for
this library and 5e-5 to the reference's build, u still within U_TOL.  The
measured errors are in the parity report ($LBM_PARITY_REPORT).
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import REL_TOL, U_TOL, abs_err, rel_err, report

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
BINS = {"fast_math": ROOT / "oracle" / "_ref" / "lbm_ref_cuda_dump",
        "exact": ROOT / "oracle" / "_ref" / "lbm_ref_cuda_exact_dump"}
STEPS = (0, 1, 10, 100)


def cases():
    from lbm_bench_gpu_gb300 import inputs
    c1 = inputs.Inputs(nx=64, ny=64, nz=64, max_step=STEPS[-1] + 1, relax_step=0, save=1, stat=10 ** 9,
                       Eo=0.0, bubbles=np.array([[32.0, 32.0, 32.0, 12.0]], np.float32))
    c4 = inputs.adjoint_short()
    c4.max_step, c4.relax_step, c4.save, c4.stat = STEPS[-1] + 1, 0, 1, 10 ** 9
    return {"static_bubble_64": c1, "adjoint_short_128": c4}


def read_dump(path: Path, shape):
    a = np.fromfile(path, dtype=np.float32)
    n = int(np.prod(shape))
    assert a.size == 5 * n, f"{path.name}: {a.size} floats, expected {5 * n}"
    a = a.reshape((5,) + shape)
    return dict(zip(("phi", "rho", "ux", "uy", "uz"), a))


def errors(got, want):
    e = {k: rel_err(got[k], want[k]) for k in ("phi", "rho")}
    e.update({k: abs_err(got[k], want[k]) for k in ("ux", "uy", "uz")})
    return e


BOUNDS = {"phi": REL_TOL, "rho": REL_TOL, "ux": U_TOL, "uy": U_TOL, "uz": U_TOL}
# 100 steps of the bubbly flow under gravity (see the module text)
GROWN_TO_REF = dict(BOUNDS, phi=5e-5, rho=5e-5)
GROWN_TO_ORACLE = dict(BOUNDS, phi=2.5e-5, rho=2.5e-5)


@pytest.mark.parametrize("build", sorted(BINS))
@pytest.mark.parametrize("name", sorted(cases()))
def test_fields_match_reference_gpu_build(tmp_path, name, build):
    from lbm_bench_gpu_gb300 import capi, inputs
    from oracle.oracle import Oracle
    binary = BINS[build]
    if not binary.exists():
        pytest.skip(f"{binary.name} is not built (reference sources absent at build time)")
    inp = cases()[name]
    inputs.write_inputs(tmp_path, inp)
    env = dict(os.environ, LBM_DUMP_STEPS=",".join(str(s) for s in STEPS))
    r = subprocess.run([str(binary)], cwd=tmp_path, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
    shape = (inp.nz, inp.ny, inp.nx)

    p = capi.make_params(inp.nx, inp.ny, inp.nz, rhoL=inp.rhoL, rhoH=inp.rhoH, tauRho=inp.tauRho,
                         tauPhi=inp.tauPhi, width=inp.width, sigma=inp.sigma, Gamma=inp.Gamma, Eo=inp.Eo,
                         rc0=inp.rc0, compat=True)
    grav = float(capi.derive(p).grav)
    o = Oracle.from_params(p)
    o.init_bubbles(inp.bubbles)
    failures = []
    with capi.Lattice.from_bubbles(p, inp.bubbles) as lat:
        done = 0
        for s in STEPS:
            lat.step(s - done, grav)
            o.step(s - done, grav)
            done = s
            got = lat.fields()
            ref = read_dump(tmp_path / f"data_{s:07d}.f32", shape)
            exact = o.moments()
            grown = s >= 100 and inp.Eo != 0.0
            checks = (
                (f"reference GPU build ({build}) {name} {s} steps", errors(got, ref),
                 GROWN_TO_REF if grown else BOUNDS),
                (f"this library vs FP64 oracle {name} {s} steps", errors(got, exact),
                 GROWN_TO_ORACLE if grown else BOUNDS),
            )
            report(f"reference GPU build ({build}) vs FP64 oracle {name} {s} steps", errors(ref, exact), BOUNDS)
            for what, e, bounds in checks:
                report(what, e, bounds)
                bad = {k: f"{e[k]:.3e} > {bounds[k]:.1e}" for k in e if not e[k] <= bounds[k]}
                if bad:
                    failures.append(f"{what}: {bad}")
    o.close()
    assert not failures, "\n".join(failures)
