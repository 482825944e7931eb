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
