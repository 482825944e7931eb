"""Storage-precision study: FP32, FP16 and BF16 storage against the FP64 oracle
after 10 000 steps.

Box: 64^3 with 4 seeded bubbles (radii U[6, 10], surface gap >= 3), the
physics of the bubbly benchmark (rhoH = 1, rhoL = 0.1, sigma = 1e-3, W = 4,
tau_rho = 0.7, Gamma = 1, tau_phi = 1, gravity -1e-6) -- the 256^3 / 512^3
boxes of the benchmark take the FP64 oracle hours for 10 000 steps.
Reported per format: phi L2 error (||phi - phi_ref||_2 / ||phi_ref||_2 and the
RMS), relative drift of sum(phi) and sum(rho) against the oracle, and the
largest distance between matching heavy-phase (phi > 0) centroids.  The
report is also written to $LBM_REPORT_DIR/precision_study.json when that
variable names a directory.
Bar: relative phi L2 error <= 1e-3 for FP32 and FP16 storage.  BF16 (8-bit
mantissa) is reported, with a looser sanity bound: its phi error after 10 000
steps is ~2e-2 relative, driven by the rounding of the momentum set g (the
oracle's storage-rounding emulation, tests/test_oracle_rounding.py, splits it:
FP16 f_1..f_6 with BF16 g stay at 2.1e-2, BF16 f_1..f_6 with FP16 g reach
5.3e-4)."""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

STEPS = int(os.environ.get("LBM_PRECISION_STEPS", "10000"))


def centroids(phi: np.ndarray) -> np.ndarray:
    """Centroids (z, y, x) of the connected phi > 0 regions, sorted."""
    from scipy import ndimage
    lab, n = ndimage.label(phi > 0)
    if n == 0:
        return np.zeros((0, 3))
    c = np.array(ndimage.center_of_mass(phi > 0, lab, range(1, n + 1)))
    return c[np.lexsort(c.T[::-1])]


def centroid_error(ref: np.ndarray, got: np.ndarray) -> float:
    """Largest distance (max norm, lattice units) from a reference centroid to
    the nearest centroid of the other run: independent of the order in which
    two nearly level bubbles sort."""
    if len(ref) == 0 or len(got) != len(ref):
        return float("inf")
    d = np.abs(ref[:, None, :] - got[None, :, :]).max(axis=2)
    return float(d.min(axis=1).max())


def test_storage_precision_10k_steps(lib):
    pytest.importorskip("scipy")
    from lbm_bench_gpu_gb300 import capi, inputs
    inp = inputs.bubbly(64, 4, r_range=(6.0, 10.0), gravity=-1e-6)
    base = dict(rhoL=inp.rhoL, rhoH=inp.rhoH, tauRho=inp.tauRho, tauPhi=inp.tauPhi, width=inp.width,
                sigma=inp.sigma, Gamma=inp.Gamma, Eo=inp.Eo, rc0=inp.rc0)
    p32 = capi.make_params(64, 64, 64, **base)
    grav = float(capi.derive(p32).grav)

    o = Oracle.from_params(p32)
    o.init_bubbles(inp.bubbles)
    o.step(STEPS, grav)
    ref = o.moments()
    ref_stats = o.stats()
    ref_c = centroids(ref["phi"])

    report = {"box": "64^3, 4 bubbles R~U[6,10], gravity -1e-6", "steps": STEPS, "formats": {}}
    for storage in ("fp32", "fp16", "bf16"):
        p = capi.make_params(64, 64, 64, storage=storage, **base)
        with capi.Lattice.from_bubbles(p, inp.bubbles) as lat:
            lat.step(STEPS, grav)
            s, f = lat.stats(fields=True)
        d = f["phi"].astype(np.float64) - ref["phi"]
        cg = centroids(f["phi"])
        cerr = centroid_error(ref_c, cg)
        report["formats"][storage] = {
            "phi_l2_rel": float(np.linalg.norm(d) / np.linalg.norm(ref["phi"])),
            "phi_rms": float(np.sqrt((d ** 2).mean())),
            "phi_maxabs": float(np.abs(d).max()),
            "mass_phi_drift_rel": abs(s["phi_sum"] - ref_stats["phi_sum"]) / abs(ref_stats["phi_sum"]),
            "mass_rho_drift_rel": abs(s["rho_sum"] - ref_stats["rho_sum"]) / abs(ref_stats["rho_sum"]),
            "centroid_err_max": cerr,
            "bubbles": int(len(cg)),
        }
    out = Path(os.environ.get("LBM_REPORT_DIR", ""))
    if os.environ.get("LBM_REPORT_DIR") and out.is_dir():
        (out / "precision_study.json").write_text(json.dumps(report, indent=1))
    print(json.dumps(report))
    for storage, r in report["formats"].items():
        assert r["phi_l2_rel"] <= (1e-3 if storage != "bf16" else 5e-2), (storage, r)
        assert r["bubbles"] == len(ref_c), (storage, r)


def test_laplace_jump_by_storage(lib):
    """Static bubble (64^3, R = 12, centred, no gravity, 1000 relaxation steps):
    the Laplace pressure jump Pin - Pout of FP32, FP16 and BF16 storage against
    the FP64 oracle.  Bars: FP32 and FP16 within 1e-3 relative of the oracle's
    jump, BF16 within 2e-2 (reported in the printed report)."""
    from lbm_bench_gpu_gb300 import capi, inputs
    inp = inputs.static_bubble(64, 12.0)
    kw = dict(rhoL=inp.rhoL, rhoH=inp.rhoH, tauRho=inp.tauRho, tauPhi=inp.tauPhi, width=inp.width,
              sigma=inp.sigma, Gamma=inp.Gamma, Eo=0.0, rc0=inp.rc0)
    o = Oracle.from_params(capi.make_params(64, 64, 64, **kw))
    o.init_bubbles(inp.bubbles)
    o.step(inp.relax_step, 0.0)
    ref = o.stats()
    report = {"oracle": {"p_dif": ref["p_dif"], "p_err": ref["p_err"]}}
    for storage in ("fp32", "fp16", "bf16"):
        p = capi.make_params(64, 64, 64, storage=storage, **kw)
        with capi.Lattice.from_bubbles(p, inp.bubbles) as lat:
            lat.step(inp.relax_step, 0.0)
            s, _ = lat.stats()
        report[storage] = {"p_dif": s["p_dif"], "p_err": s["p_err"],
                           "p_dif_rel_err": abs(s["p_dif"] - ref["p_dif"]) / abs(ref["p_dif"])}
    print(json.dumps(report))
    out = Path(os.environ.get("LBM_REPORT_DIR", ""))
    if os.environ.get("LBM_REPORT_DIR") and out.is_dir():
        (out / "laplace_by_storage.json").write_text(json.dumps(report, indent=1))
    assert report["fp32"]["p_dif_rel_err"] <= 1e-3
    assert report["fp16"]["p_dif_rel_err"] <= 1e-3
    assert report["bf16"]["p_dif_rel_err"] <= 2e-2
