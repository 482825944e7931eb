"""The oracle's storage-rounding emulation (zo_round / zo_set_rounding), used
to split a 16-bit format's error between the f and g sets in precision
studies: its FP16 rounding is IEEE binary16 round-to-nearest-even from the
FP32 value (numpy's float16 conversion), its BF16 rounding keeps the upper 16
bits of the FP32 value rounded to nearest even, and a run with FP32 rounding
stays within FP32 resolution of the unrounded FP64 run."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Oracle, round_to

PHYS = dict(rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=1.0, width=4.0, sigma=1e-3, Gamma=1.0)


def values():
    rng = np.random.default_rng(20261204)
    x = rng.standard_normal(100_000) * 10.0 ** rng.integers(-9, 6, 100_000)
    edge = [0.0, -0.0, 65504.0, 65519.9, 65520.0, 1e5, -7e-8, 2.0 ** -25, 1.5 * 2.0 ** -24, 6.1e-5, 1.0 + 2.0 ** -11]
    return np.concatenate([x, edge])


def test_fp16_rounding_is_ieee_binary16():
    x = values()
    with np.errstate(over="ignore"):
        want = x.astype(np.float32).astype(np.float16).astype(np.float64)
    got = round_to("fp16", x)
    assert np.array_equal(got, want)


def test_bf16_rounding_keeps_the_upper_half_of_fp32():
    x = values()
    u = x.astype(np.float32).view(np.uint32)
    want = ((u + np.uint32(0x7FFF) + ((u >> 16) & np.uint32(1))) & np.uint32(0xFFFF0000)).view(np.float32)
    assert np.array_equal(round_to("bf16", x), want.astype(np.float64))
    assert np.array_equal(round_to("fp32", x), x.astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("fmt,bound", [("fp32", 1e-6), ("bf16", 5e-2)])
def test_rounded_run_stays_near_the_fp64_run(fmt, bound):
    bub = np.array([[16.3, 15.2, 14.7, 7.0]], np.float32)
    runs = []
    for rounding in ("none", fmt):
        o = Oracle(32, 32, 32, **PHYS)
        o.init_bubbles(bub)
        o.set_rounding(f0=rounding, f=rounding, g=rounding, g_shift=np.full(19, 0.0))
        o.step(20, -1e-5)
        runs.append(o.moments()["phi"])
        o.close()
    err = np.linalg.norm(runs[1] - runs[0]) / np.linalg.norm(runs[0])
    assert 0.0 < err < bound


def test_bf16_phi_error_comes_from_the_momentum_set():
    """Which 16-bit set drives BF16's phi error: with the momentum set g in
    BF16 (f_1..f_6 in FP16) phi ends far further from the FP64 run than with
    f_1..f_6 in BF16 (g in FP16), while f in BF16 drives the drift of sum(phi).
    24^3, one bubble rising under gravity, 1000 steps, the library's shifts and
    scales (64^3 x 10 000 steps: phi L2 2.1e-2 vs 5.3e-4, drift of sum(phi)
    1.3e-6 vs 5.5e-5)."""
    bub = np.array([[12.3, 11.2, 10.7, 6.0]], np.float32)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)

    def run(f_fmt, g_fmt):
        o = Oracle(24, 24, 24, **PHYS)
        o.init_bubbles(bub)
        if f_fmt != "none":
            shift = w * o.moments()["rho"].mean()
            fs = 32768.0 if f_fmt == "fp16" else 1.0
            gs = 65536.0 if g_fmt == "fp16" else 1.0
            o.set_rounding(f0="fp32", f=f_fmt, f_scale=fs, g=g_fmt, g_scale=gs, g_shift=shift)
        o.step(1000, -2e-5)
        out = (o.moments()["phi"], o.stats()["phi_sum"])
        o.close()
        return out

    phi64, sum64 = run("none", "none")
    errs = {}
    for f_fmt, g_fmt in (("fp16", "bf16"), ("bf16", "fp16")):
        phi, s = run(f_fmt, g_fmt)
        errs[(f_fmt, g_fmt)] = (np.linalg.norm(phi - phi64) / np.linalg.norm(phi64), abs(s - sum64) / abs(sum64))
    g_bf16, f_bf16 = errs[("fp16", "bf16")], errs[("bf16", "fp16")]
    assert g_bf16[0] > 5 * f_bf16[0], errs
    assert f_bf16[1] > 5 * g_bf16[1], errs
