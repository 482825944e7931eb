"""The checked build (ZSC_CHECKED=1: every global store and cp.async source of
the step kernel checked against its field before the access; an index outside
it sets an error bit that lbm_sync reports) runs the step on boxes of one tile,
two tiles and with interior tiles, in every storage format, without an error
and with the product build's results to FP32 rounding (the checks change how
the compiler contracts multiply-adds, so not bit for bit)."""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [((32, 8, 12), [[15.7, 4.2, 6.4, 3.0], [7.5, 2.2, 3.1, 2.0]]),
         ((64, 32, 48), [[31.7, 16.2, 24.4, 10.0], [16.0, 8.0, 13.0, 6.0]]),
         ((128, 32, 16), [[50.3, 15.8, 8.4, 6.0], [97.1, 9.2, 7.7, 4.5]])]
KW = dict(rhoL=0.1, rhoH=1.0, tauRho=0.8, tauPhi=0.9, width=4.0, sigma=1e-3, Gamma=1.0)

RUN = r"""
import sys
import numpy as np
from lbm_bench_gpu_gb300 import capi
sys.path.insert(0, sys.argv[2])
from test_gpu_checked import CASES, KW, run_all
np.savez(sys.argv[1], **run_all(capi))
"""


def run_all(capi) -> dict:
    out = {}
    for storage in ("fp32", "fp16", "bf16"):
        for shape, bub in CASES:
            p = capi.make_params(*shape, storage=storage, **KW)
            with capi.Lattice.from_bubbles(p, np.array(bub, np.float32)) as lat:
                lat.step(5, -2e-5)     # odd and even steps, the first one from the streamed state
                lat.sync()             # raises if the checked build flagged an index
                for k, v in lat.fields().items():
                    out[f"{storage}_{shape[0]}x{shape[1]}x{shape[2]}_{k}"] = v
    return out


def test_checked_build_flags_nothing_and_matches(lib, tmp_path):
    from lbm_bench_gpu_gb300 import build, capi
    checked = build.build_checked()
    npz = tmp_path / "checked.npz"
    env = dict(os.environ, LBM_GB300_LIB=str(checked))
    root = Path(__file__).resolve().parents[1]
    r = subprocess.run([sys.executable, "-c", RUN, str(npz), str(Path(__file__).parent)], cwd=root, env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    got = np.load(npz)
    want = run_all(capi)
    assert set(got.files) == set(want)
    from conftest import REL_TOL, U_TOL, rel_err
    for k, v in want.items():
        if k.endswith(("_phi", "_rho")):
            assert rel_err(got[k], v) <= REL_TOL, k      # the parity suite's tolerances
        else:
            assert float(np.abs(got[k].astype(np.float64) - v).max()) <= U_TOL, k
