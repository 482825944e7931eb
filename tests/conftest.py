"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"

# Tolerances of the FP32 paths against the FP64 oracle, at <= 100 steps:
#  phi, rho: max |a - b| / max |b| <= 1e-5 (relative);
#  distributions: max |a - b| over a set (the 7 f or the 19 g) / max |b| over
#  that set <= 1e-5 (f_1..f_6 ~ Gamma mu / 2 ~ 1e-6 near equilibrium are
#  differences of O(phi) terms, so each alone carries the rounding of phi);
#  u: max |a - b| <= 1e-6 absolute (u is a cancelling sum of O(rho)
#  distributions divided by rho; FP32 stays within 3.5e-7 of FP64 over 100
#  steps on every box the tests run, 256^3 and 512^3 included).
# 16-bit storage (shifted, power-of-two scaled FP16 / BF16; FP32 arithmetic):
#  STORAGE_TOL relative for phi, rho and the distribution sets, U_TOL_STORAGE
#  absolute for u (measured at <= 10 steps: FP16 6e-6, BF16 1.2e-5).
REL_TOL = 1e-5
CS = 1.0 / np.sqrt(3.0)
U_TOL = 1e-6
STORAGE_TOL = {"fp32": REL_TOL, "fp16": 5e-5, "bf16": 5e-4}
U_TOL_STORAGE = {"fp32": U_TOL, "fp16": 1e-5, "bf16": 5e-5}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def lib():
    from lbm_bench_gpu_gb300 import build, capi
    build.build()
    return capi.load()


@pytest.fixture(scope="session")
def golden_manifest():
    return json.loads((GOLDEN / "golden.json").read_text())


def rel_err(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / scale) if scale > 0 else float(np.abs(a - b).max())


def abs_err(a, b) -> float:
    return float(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)).max())


def report(what: str, errors: dict, bounds: dict, info: dict | None = None) -> None:
    """Append the measured errors of one comparison to the JSON-lines file named
    by $LBM_PARITY_REPORT (if set), so that tolerances can be set from data."""
    path = os.environ.get("LBM_PARITY_REPORT")
    if not path:
        return
    rec = {"what": what, "errors": {k: float(v) for k, v in errors.items()},
           "bounds": {k: float(v) for k, v in bounds.items()}}
    if info:
        rec["info"] = {k: float(v) for k, v in info.items()}
    with open(path, "a") as fh:
        fh.write(json.dumps(rec) + "\n")


def assert_fields_close(got: dict, want: dict, rel=REL_TOL, utol=U_TOL, what=""):
    errs = {k: rel_err(got[k], want[k]) for k in ("phi", "rho")}
    errs.update({k: abs_err(got[k], want[k]) for k in ("ux", "uy", "uz")})
    report(what, errs, {"phi": rel, "rho": rel, "ux": utol, "uy": utol, "uz": utol})
    for k in ("phi", "rho"):
        assert errs[k] <= rel, f"{what} {k}: relative error {errs[k]:.3e} > {rel:.1e}"
    for k in ("ux", "uy", "uz"):
        assert errs[k] <= utol, f"{what} {k}: absolute error {errs[k]:.3e} > {utol:.3e}"


def assert_state_close(lat, o, rel=REL_TOL, utol=U_TOL, what="", failures=None):
    """The lattice's phi, rho, u and all 26 streamed distributions against the
    oracle's, node by node (compared in C without float64 copies, so it scales
    to 512^3): phi and rho within `rel` of the field's largest magnitude, the
    7 f and the 19 g within `rel` of their set's largest magnitude (as the
    small-box tests compare them), u within `utol` absolute.  With a `failures` list the
    violations are appended to it instead of raised (the caller asserts once
    every comparison has been made and reported)."""
    from lbm_bench_gpu_gb300 import capi
    f, g = lat.dist()
    mom = np.empty((5,) + lat.shape, np.float32)
    capi.check(capi.load().lbm_stats(lat._h, None, *[capi.fptr(mom[a]) for a in range(5)]), "lbm_stats")
    res = o.compare(f, g, mom)
    del f, g, mom
    errs, bounds, info = {}, {}, {}
    for k in ("phi", "rho"):
        d, m = res[k]
        errs[k], bounds[k] = (d / m if m > 0 else d), rel
    for k in ("ux", "uy", "uz"):
        errs[k], bounds[k] = res[k][0], utol
    for name, fields in (("f", [f"f{i}" for i in range(7)]), ("g", [f"g{i}" for i in range(19)])):
        d = max(res[k][0] for k in fields)
        m = max(res[k][1] for k in fields)
        errs[name], bounds[name] = (d / m if m > 0 else d), rel
        for k in fields:   # per field, for the report only: |max diff|, max |ref|
            info[k + "_abs"], info[k + "_max"] = res[k]
    report(what, errs, bounds, info)
    bad = {k: f"{errs[k]:.3e} > {bounds[k]:.1e}" for k in errs if not errs[k] <= bounds[k]}
    if failures is not None:
        if bad:
            failures.append(f"{what}: {bad}")
    else:
        assert not bad, f"{what}: {bad}"
    return errs


def write_case(tmp_path, inp):
    from lbm_bench_gpu_gb300 import inputs
    inputs.write_inputs(tmp_path, inp)
    return tmp_path
