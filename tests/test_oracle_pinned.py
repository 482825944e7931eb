"""The FP64 oracle against the reference itself (CPU, no GPU needed).

Two pins:
 * the committed golden fixtures (outputs of the reference's own kernels,
   made by tests/golden/make_golden.py) -- always available;
 * the reference's kernels compiled for the CPU (oracle/_ref), on fresh
   seeded inputs -- where the reference sources are available.
"""
from __future__ import annotations

import json
import re
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN, assert_fields_close, rel_err

# The reference prints its statistics with 7 significant digits from float
# accumulators; quantities near zero are compared to this absolute bound.
PRINT_TOL = 6e-7
from oracle.oracle import Oracle, RefCPU, ref_lib


def oracle_for_dir(d):
    from lbm_bench_gpu_gb300 import capi
    p, run, bub = capi.read_inputs(d)
    o = Oracle.from_params(p)
    o.init_bubbles(bub)
    return o, p, run, bub


@pytest.mark.parametrize("name", ["relax32", "overlap_ghost32", "sample_ratio"])
def test_oracle_matches_golden(name, golden_manifest, lib, tmp_path):
    case = golden_manifest[name]
    (tmp_path / "properties.in").write_text(case["properties.in"])
    (tmp_path / "discrete.in").write_text(case["discrete.in"])
    o, p, _, _ = oracle_for_dir(tmp_path)
    ref = np.load(GOLDEN / f"{name}.npz")
    m0 = o.moments()
    # initial fields: bubble phi (float vs double evaluation) and rho, u
    assert rel_err(m0["phi"], ref["init_phi"]) < 1e-6
    assert rel_err(m0["rho"], ref["init_rho"]) < 1e-6
    o.step(case["steps"], case["grav"])
    m = o.moments()
    want = {k: ref[k] for k in ("phi", "rho", "ux", "uy", "uz")}
    # the reference is FP32: compare it to the FP64 oracle at the stated tolerance
    assert_fields_close(want, m, what=f"golden {name}")


def _parse_stats(text):
    lines = [l for l in text.splitlines() if l and not l.startswith("#")]
    return [list(map(float, l.split())) for l in lines]


def _parse_runlog(text):
    vals = {}
    for l in text.splitlines():
        m = re.match(r"(.+?)\s*=\s*(\S+)", l)
        if m:
            vals[m.group(1).strip()] = float(m.group(2))
    return vals


@pytest.mark.parametrize("name", ["relax32", "overlap_ghost32"])
def test_oracle_stats_match_reference_text(name, golden_manifest, lib, tmp_path):
    """stats.c / logsave.c quantities (printed with 7 digits by the reference)."""
    case = golden_manifest[name]
    (tmp_path / "properties.in").write_text(case["properties.in"])
    (tmp_path / "discrete.in").write_text(case["discrete.in"])
    o, p, _, _ = oracle_for_dir(tmp_path)
    s0 = o.stats()
    o.step(case["steps"], case["grav"])
    s = o.stats()
    rows = _parse_stats(case["relax_stats.out"])
    step, ux, uy, uz, umax, vef, ref_r = rows[-1]
    assert step == case["steps"]
    # per-node u differs by FP32 rounding; the printed value has 7 digits
    assert abs(s["umax"] - umax) <= 1e-6 * umax + PRINT_TOL
    assert s["vol"] / s0["vol"] == pytest.approx(vef, rel=1e-6)
    assert s["ref"] == pytest.approx(ref_r, rel=1e-6)
    # mean u over phi >= 0 is a cancelling sum (the reference accumulates it in
    # float): compare at the per-node velocity tolerance
    for mine, theirs in ((s["ux_av"], ux), (s["uy_av"], uy), (s["uz_av"], uz)):
        assert abs(mine - theirs) <= 1e-4 * abs(theirs) + PRINT_TOL
    log = _parse_runlog(case["runlog.out"])
    # The reference sums ~3e4 pressures in a float accumulator
    # (src/logsave.c:139-143): its Pin - Pout carries ~1e-3 relative rounding
    # error (test_reference_pressure_replay reproduces its digits exactly).
    assert s["p_dif"] == pytest.approx(log["(Pin - Pout)"], rel=1e-3)
    assert s["p_err"] == pytest.approx(log["Laplace Error"], rel=1e-3)
    # the reference prints max |u|^2 under "Parasitic Velocity" (src/logsave.c:249, no sqrt)
    assert abs(s["umax"] ** 2 - log["Parasitic Velocity"]) <= 2 * s["umax"] * PRINT_TOL


def test_oracle_constants_match_reference(golden_manifest):
    case = golden_manifest["sample_ratio"]
    with tempfile.TemporaryDirectory() as d:
        Path(d, "properties.in").write_text(case["properties.in"])
        Path(d, "discrete.in").write_text(case["discrete.in"])
        from lbm_bench_gpu_gb300 import capi
        p, _, _ = capi.read_inputs(d)
    c = Oracle.from_params(p).constants()
    for k, v in case["ref_constants"].items():
        assert c[k] == pytest.approx(v, rel=2e-6), k


needs_ref = pytest.mark.skipif(ref_lib() is None, reason="reference sources not available")


@needs_ref
@pytest.mark.parametrize("steps,grav,tau", [(1, 0.0, 0.7), (7, -3e-5, 0.9)])
def test_oracle_matches_reference_kernels(tmp_path, lib, steps, grav, tau):
    from lbm_bench_gpu_gb300 import inputs
    b = inputs.place_bubbles(3, (32, 32, 40), (4.0, 6.0), seed=7)
    inp = inputs.Inputs(nx=32, ny=32, nz=40, tauRho=tau, tauPhi=0.8, bubbles=b)
    inputs.write_inputs(tmp_path, inp)
    ref = RefCPU(tmp_path)
    o, p, _, _ = oracle_for_dir(tmp_path)
    ref.step(steps, grav)
    o.step(steps, grav)
    assert_fields_close(ref.fields(), o.moments(), what="reference kernels")
    fr, gr = ref.dist()
    fo, go = o.dist()
    assert rel_err(fr, fo) < 1e-5
    assert rel_err(gr, go) < 1e-5


@needs_ref
def test_reference_rejects_like_main(tmp_path):
    from lbm_bench_gpu_gb300 import inputs
    inputs.write_inputs(tmp_path, inputs.Inputs(nx=48, ny=32, nz=8,
                                                bubbles=np.array([[8, 8, 4, 2]], np.float32)))
    with pytest.raises(RuntimeError):
        RefCPU(tmp_path)


def test_oracle_conserves_phi_and_rho():
    """Sum phi is conserved exactly by collision and eta-streaming; check drift."""
    o = Oracle(32, 32, 32, rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=1.0, width=4.0, sigma=1e-3, Gamma=1.0)
    o.init_bubbles(np.array([[16, 15, 17, 7], [5.5, 25, 8, 3.5]], np.float32))
    s0 = o.stats()
    o.step(20, -1e-5)
    s = o.stats()
    assert abs(s["phi_sum"] - s0["phi_sum"]) <= 1e-10 * abs(s0["phi_sum"])
    assert abs(s["rho_sum"] - s0["rho_sum"]) <= 1e-10 * abs(s0["rho_sum"])


def _pressure_f32(phi, rho, c):
    """Pressure of src/logsave.c:95-137 evaluated in float32 (periodic stencil)."""
    f32 = np.float32

    def P(dx, dy, dz):
        return np.roll(phi, (-dz, -dy, -dx), axis=(0, 1, 2))

    p00 = phi
    p01, p02, p03, p04, p05, p06 = P(1, 0, 0), P(-1, 0, 0), P(0, 1, 0), P(0, -1, 0), P(0, 0, 1), P(0, 0, -1)
    p07, p08, p09, p10 = P(1, 1, 0), P(-1, -1, 0), P(1, -1, 0), P(-1, 1, 0)
    p11, p12, p13, p14 = P(1, 0, 1), P(-1, 0, -1), P(1, 0, -1), P(-1, 0, 1)
    p15, p16, p17, p18 = P(0, 1, 1), P(0, -1, -1), P(0, 1, -1), P(0, -1, 1)
    inv6, inv12 = f32(1.0 / 6.0), f32(1.0 / 12.0)
    lap = (p07 + p08 + p09 + p10 + p11 + p12 + p13 + p14 + p15 + p16 + p17 + p18
           + f32(2) * (p01 + p02 + p03 + p04 + p05 + p06 - f32(12) * p00)) * inv6
    gx = (f32(2) * (p01 - p02) + p07 - p08 + p09 - p10 + p11 - p12 + p13 - p14) * inv12
    gy = (f32(2) * (p03 - p04) + p07 - p08 + p10 - p09 + p15 - p16 + p17 - p18) * inv12
    gz = (f32(2) * (p05 - p06) + p11 - p12 + p14 - p13 + p15 - p16 + p18 - p17) * inv12
    a, k, pss = f32(c["alpha"]), f32(c["kappa"]), f32(c["phiStarSq"])
    ph2 = phi * phi
    return a * (ph2 * (f32(3) * ph2 - f32(2) * pss) - pss * pss) - k * (phi * lap - f32(0.5) * (gx * gx + gy * gy + gz * gz)) \
        + f32(1.0 / 3.0) * rho


def test_reference_pressure_replay(golden_manifest, lib, tmp_path):
    """Replaying src/logsave.c's float32 loop (i outer, j, k inner; borders in x
    and y skipped) on the reference's own arrays reproduces its printed
    Pin - Pout to all 7 digits -- pins the formula, the region and the quirks
    the oracle and lbm_stats restate in FP64."""
    case = golden_manifest["relax32"]
    (tmp_path / "properties.in").write_text(case["properties.in"])
    (tmp_path / "discrete.in").write_text(case["discrete.in"])
    from lbm_bench_gpu_gb300 import capi
    p, _, _ = capi.read_inputs(tmp_path)
    c = Oracle.from_params(p).constants()
    ref = np.load(GOLDEN / "relax32.npz")
    phi, rho = ref["phi"].astype(np.float32), ref["rho"].astype(np.float32)
    pres = _pressure_f32(phi, rho, c)
    nz, ny, nx = phi.shape
    f32 = np.float32
    s_in = s_out = vol = f32(0)
    P_ = pres.transpose(2, 1, 0)
    F_ = phi.transpose(2, 1, 0)
    for i in range(1, nx - 1):
        for j in range(1, ny - 1):
            for v, ph in zip(P_[i, j], F_[i, j]):
                if ph >= 0:
                    s_in = f32(s_in + v)
                    vol = f32(vol + 1)
                else:
                    s_out = f32(s_out + v)
    dp = f32(s_in / vol) - f32(s_out / (f32(nx * ny * nz) - vol))
    want = _parse_runlog(case["runlog.out"])["(Pin - Pout)"]
    assert float(dp) == pytest.approx(want, rel=5e-7)
