"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
from __future__ import annotations

import json
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


def assert_fields_close(got: dict, want: dict, rel=REL_TOL, utol=U_TOL, what=""):
    for k in ("phi", "rho"):
        e = rel_err(got[k], want[k])
        assert e <= rel, f"{what} {k}: relative error {e:.3e} > {rel:.1e}"
    for k in ("ux", "uy", "uz"):
        e = abs_err(got[k], want[k])
        assert e <= utol, f"{what} {k}: absolute error {e:.3e} > {utol:.3e}"


def write_case(tmp_path, inp):
    from lbm_bench_gpu_gb300 import inputs
    inputs.write_inputs(tmp_path, inp)
    return tmp_path
