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
#  phi, rho and the distributions: max |a - b| / max |b| <= 1e-5 (relative);
#  u: max |a - b| <= 1e-5 * c_s, c_s = 1/sqrt(3) the lattice sound speed.
#  (u is a cancelling sum of O(rho) distributions divided by rho, so its FP32
#  rounding error scales with the distributions, not with |u| ~ 1e-4.)
REL_TOL = 1e-5
CS = 1.0 / np.sqrt(3.0)
U_TOL = 1e-5 * CS


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


def report(what: str, errors: dict, bounds: dict) -> None:
    """Append the measured errors of one comparison to the JSON-lines file named
    by $LBM_PARITY_REPORT (if set), so that tolerances can be set from data."""
    path = os.environ.get("LBM_PARITY_REPORT")
    if not path:
        return
    rec = {"what": what, "errors": {k: float(v) for k, v in errors.items()},
           "bounds": {k: float(v) for k, v in bounds.items()}}
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
    to 512^3): phi, rho and each distribution within `rel` of the field's
    largest magnitude, u within `utol` absolute.  With a `failures` list the
    violations are appended to it instead of raised (the caller asserts once
    every comparison has been made and reported)."""
    from lbm_bench_gpu_gb300 import capi
    f, g = lat.dist()
    mom = np.empty((5,) + lat.shape, np.float32)
    capi.check(capi.load().lbm_stats(lat._h, None, *[capi.fptr(mom[a]) for a in range(5)]), "lbm_stats")
    res = o.compare(f, g, mom)
    del f, g, mom
    errs, bounds = {}, {}
    for k, (d, m) in res.items():
        if k in ("ux", "uy", "uz"):
            errs[k], bounds[k] = d, utol
        else:
            errs[k], bounds[k] = (d / m if m > 0 else d), rel
    report(what, errs, bounds)
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
