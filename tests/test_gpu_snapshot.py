"""Checkpoint / resume through lbm_save_state / lbm_load_state: a context
restored from a snapshot steps on bit for bit like the one that was saved, in
every storage format, from the freshly initialised state (streamed f) and from
the middle of a run (an odd step pending in the AA layout)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHYS = dict(rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=1.0, width=4.0, sigma=1e-3, Gamma=1.0)
BUB = np.array([[31.6, 15.3, 12.4, 7.0], [10.2, 24.0, 5.5, 4.0]], np.float32)
GRAV = -2e-5


def params(storage):
    from lbm_bench_gpu_gb300 import capi
    return capi.make_params(64, 32, 24, storage=storage, **PHYS)


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("before", [0, 7])
def test_resume_is_bit_identical(lib, storage, before):
    from lbm_bench_gpu_gb300 import capi
    p = params(storage)
    with capi.Lattice.from_bubbles(p, BUB) as a:
        if before:
            a.step(before, GRAV)
        stats_at_save, _ = a.stats()
        snap = a.save_state()
        a.step(6, GRAV)
        want, want_dist = a.fields(), a.dist()
    with capi.Lattice.from_bubbles(p, BUB) as b:
        b.step(3, GRAV)                         # whatever it held is replaced
        b.load_state(snap)
        assert b.steps == before
        stats_loaded, _ = b.stats()
        assert stats_loaded == stats_at_save
        b.step(6, GRAV)
        got, got_dist = b.fields(), b.dist()
    for k in want:
        assert np.array_equal(got[k], want[k]), k
    for x, y in zip(got_dist, want_dist):
        assert np.array_equal(x, y)


def test_load_rejects_other_boxes_formats_and_garbage(lib):
    from lbm_bench_gpu_gb300 import capi
    with capi.Lattice.from_bubbles(params("fp32"), BUB) as a:
        snap = a.save_state()
    with capi.Lattice.from_bubbles(params("fp16"), BUB) as b:
        with pytest.raises(capi.LbmError) as e:
            b.load_state(snap)
        assert e.value.code == capi.LBM_EINVAL
    other = capi.make_params(32, 32, 24, storage="fp32", **PHYS)
    with capi.Lattice.from_bubbles(other, np.array([[15.5, 15.5, 12.0, 6.0]], np.float32)) as c:
        with pytest.raises(capi.LbmError) as e:
            c.load_state(snap)
        assert e.value.code == capi.LBM_EINVAL
        bad = snap.copy()
        bad[:8] = 0
        with pytest.raises(capi.LbmError) as e:
            c.load_state(bad)
        assert e.value.code == capi.LBM_EINVAL
