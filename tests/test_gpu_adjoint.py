"""lbm_step_adjoint (GPU, FP32 with FP64 sums) against the FP64 CPU adjoint
of the oracle (itself checked against FP64 finite differences in
test_adjoint_oracle.py).  Tolerances: J 1e-5 relative; dJ/dgrav 1e-3
relative; dJ/dphi0 max |error| <= 2e-3 max |dJ/dphi0| (the FP32 adjoint sums
~20 terms per node and step)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

KW = dict(rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=0.9, width=4.0, sigma=1e-3, Gamma=1.0)
SHAPE = (16, 32, 32)


def fields():
    o = Oracle(32, 32, 16, **KW)
    pg = o.bubble_phi(np.array([[15.5, 16.3, 8.4, 6.0], [5.0, 6.0, 12.0, 3.5]], np.float32))
    return pg[1:-1].copy(), np.full(SHAPE, 0.55)


@pytest.mark.parametrize("objective,window,T", [("light_uz_mean", 5, 12), ("light_z_centroid", 1, 10)])
def test_gpu_adjoint_matches_oracle(lib, objective, window, T):
    from lbm_bench_gpu_gb300 import capi
    phi0, rho0 = fields()
    grav = -3e-5
    p = capi.make_params(32, 32, 16, **KW)
    o = Oracle.from_params(p)
    o.init(phi0.astype(np.float32).astype(np.float64), rho0)
    J, dg, lf, lg = o.adjoint(T, grav, objective, window)
    lphi, _ = o.init_adjoint(phi0.astype(np.float32).astype(np.float64), lf, lg)
    with capi.Lattice.from_fields(p, phi0.astype(np.float32), rho0.astype(np.float32)) as lat:
        r = lat.adjoint(T, grav, objective, window)
        assert lat.steps == 0
    assert r["adjoint_steps"] == T
    assert r["J"] == pytest.approx(J, rel=1e-5)
    assert r["dJ_dgrav"] == pytest.approx(dg, rel=1e-3)
    err = np.abs(r["dJ_dphi0"] - lphi).max()
    assert err <= 2e-3 * np.abs(lphi).max(), err / np.abs(lphi).max()


@pytest.mark.parametrize("device_slots", [3, 5])
def test_host_checkpoint_tier_does_not_change_the_gradient(lib, device_slots):
    """A second checkpoint tier in pinned host memory (segment starts kept on
    the host during the first sweep, each segment reversed with the device
    slots; with 3 device slots the host copies run on the main stream, with 5
    on a copy stream beside the compute): the same trajectory, so J and the
    gradients are identical; with 3 device slots in fewer forward steps than
    one tier takes."""
    from lbm_bench_gpu_gb300 import capi
    phi0, rho0 = fields()
    p = capi.make_params(32, 32, 16, **KW)
    snap = 26 * 4 * 32 * 32 * 16
    dev = (device_slots + 0.5) * snap
    with capi.Lattice.from_fields(p, phi0.astype(np.float32), rho0.astype(np.float32)) as lat:
        one = lat.adjoint(20, -3e-5, "light_uz_mean", 6, checkpoint_bytes=dev)
        two = lat.adjoint(20, -3e-5, "light_uz_mean", 6, checkpoint_bytes=dev, host_checkpoint_bytes=4.5 * snap)
        again = lat.adjoint(20, -3e-5, "light_uz_mean", 6, checkpoint_bytes=dev, host_checkpoint_bytes=4.5 * snap)
        assert lat.steps == 0
    assert one["host_slots"] == 0 and two["host_slots"] == 3 and two["slots"] == device_slots
    assert two["forward_steps"] == capi.adjoint_forward_steps(20, device_slots, 4)
    if device_slots == 3:
        assert two["forward_steps"] < one["forward_steps"]
    for r in (two, again):
        assert r["J"] == one["J"] and r["dJ_dgrav"] == one["dJ_dgrav"]
        assert np.array_equal(r["dJ_dphi0"], one["dJ_dphi0"])


def test_checkpoint_budget_does_not_change_the_gradient(lib):
    """3 slots for 20 steps forces recomputation (binomial schedule); the
    trajectory is deterministic, so J and the gradients are identical."""
    from lbm_bench_gpu_gb300 import capi
    phi0, rho0 = fields()
    p = capi.make_params(32, 32, 16, **KW)
    with capi.Lattice.from_fields(p, phi0.astype(np.float32), rho0.astype(np.float32)) as lat:
        full = lat.adjoint(20, -3e-5, "light_uz_mean", 6)
        snap = 26 * 4 * 32 * 32 * 16
        tight = lat.adjoint(20, -3e-5, "light_uz_mean", 6, checkpoint_bytes=3.5 * snap)
    assert full["slots"] == 21 and tight["slots"] == 3
    assert full["forward_steps"] == 20 and tight["forward_steps"] > 20
    # the planner runs the same schedule without stepping
    assert tight["forward_steps"] == capi.adjoint_forward_steps(20, 3)
    assert full["forward_steps"] == capi.adjoint_forward_steps(20, 21)
    assert tight["J"] == full["J"] and tight["dJ_dgrav"] == full["dJ_dgrav"]
    assert np.array_equal(tight["dJ_dphi0"], full["dJ_dphi0"])


def test_adjoint_needs_initial_state(lib):
    from lbm_bench_gpu_gb300 import capi
    phi0, rho0 = fields()
    p = capi.make_params(32, 32, 16, **KW)
    with capi.Lattice.from_fields(p, phi0.astype(np.float32), rho0.astype(np.float32)) as lat:
        lat.step(1)
        with pytest.raises(capi.LbmError) as e:
            lat.adjoint(5, -3e-5)
        assert e.value.code == capi.LBM_ESTATE


def test_objective_alone_matches_adjoint_J(lib):
    """lbm_objective runs the same forward states as lbm_step_adjoint, so J
    agrees to the rounding of its FP64 sum (the adjoint adds the window's terms
    in reverse step order); central differences of it agree with dJ/dgrav to
    FP32 trajectory noise (5e-3 relative at h = 1e-5 on a 16 x 32 x 32 box)."""
    from lbm_bench_gpu_gb300 import capi
    phi0, rho0 = fields()
    p = capi.make_params(32, 32, 16, **KW)
    grav = -3e-5
    with capi.Lattice.from_fields(p, phi0.astype(np.float32), rho0.astype(np.float32)) as lat:
        r = lat.adjoint(12, grav, "light_uz_mean", 5, want_phi0=False)
        J = lat.objective(12, grav, "light_uz_mean", 5)
        h = 1e-5
        fd = (lat.objective(12, grav + h, "light_uz_mean", 5) - lat.objective(12, grav - h, "light_uz_mean", 5)) / (2 * h)
        assert lat.steps == 0
    assert J == pytest.approx(r["J"], rel=1e-14)
    assert fd == pytest.approx(r["dJ_dgrav"], rel=5e-3)


def test_workspace_is_kept_between_calls_and_released(lib):
    """The context keeps the adjoint workspace and checkpoint pool: a call with
    a smaller budget after a larger one reuses the larger pool and gives the
    same results as on a fresh pool; lbm_adjoint_release returns the memory."""
    import torch
    from lbm_bench_gpu_gb300 import capi
    phi0, rho0 = fields()
    p = capi.make_params(32, 32, 16, **KW)
    snap = 26 * 4 * 32 * 32 * 16
    with capi.Lattice.from_fields(p, phi0.astype(np.float32), rho0.astype(np.float32)) as lat:
        tight = lat.adjoint(20, -3e-5, "light_uz_mean", 6, checkpoint_bytes=3.5 * snap)
        full = lat.adjoint(20, -3e-5, "light_uz_mean", 6)
        held = torch.cuda.mem_get_info()[0]
        again = lat.adjoint(20, -3e-5, "light_uz_mean", 6, checkpoint_bytes=3.5 * snap)
        assert torch.cuda.mem_get_info()[0] == held     # nothing allocated
        J = lat.objective(20, -3e-5, "light_uz_mean", 6)
        assert torch.cuda.mem_get_info()[0] == held
        lat.adjoint_release()
        assert torch.cuda.mem_get_info()[0] - held >= 21 * snap
        after = lat.adjoint(20, -3e-5, "light_uz_mean", 6, checkpoint_bytes=3.5 * snap)
        assert lat.steps == 0
    assert tight["slots"] == again["slots"] == after["slots"] == 3 and full["slots"] == 21
    for r in (again, after):
        assert r["forward_steps"] == tight["forward_steps"]
        assert r["J"] == tight["J"] and r["dJ_dgrav"] == tight["dJ_dgrav"]
        assert np.array_equal(r["dJ_dphi0"], tight["dJ_dphi0"])
    assert J == pytest.approx(tight["J"], rel=1e-14)


# 16-bit states: the adjoint reads the forward state (checkpoints included)
# in its storage format and layout; its arithmetic and lambda stay FP32.  The
# gradient then follows the 16-bit trajectory, whose error against the FP64
# oracle is the storage's: bounds (J, dJ/dgrav, dJ/dphi0 of its max) FP16
# 1e-4 / 1e-3 / 1e-3, BF16 1e-3 / 1e-2 / 1e-2 (measured: FP16 4.2e-5 / 1.8e-7 /
# 4.6e-5, BF16 2.7e-5 / 2.7e-7 / 4.1e-4).
ADJ_STORAGE_BOUNDS = {"fp16": (1e-4, 1e-3, 1e-3), "bf16": (1e-3, 1e-2, 1e-2)}


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_gpu_adjoint_16bit_state_matches_oracle(lib, storage):
    from conftest import report
    from lbm_bench_gpu_gb300 import capi
    o0 = Oracle(64, 32, 16, **KW)
    pg = o0.bubble_phi(np.array([[40.5, 16.3, 8.4, 6.0], [12.0, 9.0, 7.0, 4.5]], np.float32))
    phi0, rho0 = pg[1:-1].astype(np.float32), np.full((16, 32, 64), 0.55, np.float32)
    T, window, grav = 12, 5, -3e-5
    o = Oracle(64, 32, 16, **KW)
    o.init(phi0.astype(np.float64), rho0.astype(np.float64))
    J, dg, lf, lg = o.adjoint(T, grav, "light_uz_mean", window)
    lphi, _ = o.init_adjoint(phi0.astype(np.float64), lf, lg)
    p = capi.make_params(64, 32, 16, storage=storage, **KW)
    with capi.Lattice.from_fields(p, phi0, rho0) as lat:
        # few slots: the state is recomputed from 16-bit checkpoints
        r = lat.adjoint(T, grav, "light_uz_mean", window, checkpoint_bytes=4.5 * 54 * 64 * 32 * 16)
    bj, bg, bp = ADJ_STORAGE_BOUNDS[storage]
    e = {"J": abs(r["J"] - J) / abs(J), "dJ_dgrav": abs(r["dJ_dgrav"] - dg) / abs(dg),
         "dJ_dphi0": float(np.abs(r["dJ_dphi0"] - lphi).max() / np.abs(lphi).max())}
    report(f"adjoint {storage} state vs FP64 oracle adjoint", e, {"J": bj, "dJ_dgrav": bg, "dJ_dphi0": bp})
    assert r["slots"] < T + 1
    assert e["J"] <= bj and e["dJ_dgrav"] <= bg and e["dJ_dphi0"] <= bp, e
