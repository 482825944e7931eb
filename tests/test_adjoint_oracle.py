"""The FP64 CPU adjoint (oracle/zsc_oracle.c) against FP64 central finite
differences of the FP64 forward step.  Checks dJ/dgrav and dJ/dphi0 at probe
nodes with |phi| well away from 0 (the gravity mask H(phi > 0) is not
differentiable there)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Oracle

KW = dict(rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=0.9, width=4.0, sigma=1e-3, Gamma=1.0)
SHAPE = (16, 32, 32)   # nz, ny, nx


@pytest.fixture(scope="module")
def setup():
    o = Oracle(32, 32, 16, **KW)
    pg = o.bubble_phi(np.array([[15.5, 16.3, 8.4, 6.0]], np.float32))
    return o, pg[1:-1].copy(), np.full(SHAPE, 0.55)


@pytest.mark.parametrize("objective,window", [("light_uz_mean", 5), ("light_z_centroid", 1)])
def test_oracle_adjoint_matches_fd(setup, objective, window):
    o, phi0, rho0 = setup
    T, grav = 12, -3e-5
    o.init(phi0, rho0)
    J, dg, lf, lg = o.adjoint(T, grav, objective, window)
    o.init(phi0, rho0)
    assert o.objective(T, grav, objective, window) == pytest.approx(J, rel=1e-14)
    h = 1e-3 * abs(grav)
    o.init(phi0, rho0)
    jp = o.objective(T, grav + h, objective, window)
    o.init(phi0, rho0)
    jm = o.objective(T, grav - h, objective, window)
    assert dg == pytest.approx((jp - jm) / (2 * h), rel=1e-6)

    lphi, _ = o.init_adjoint(phi0, lf, lg)
    rng = np.random.default_rng(3)
    probes = [tuple(int(rng.integers(0, s)) for s in SHAPE) for _ in range(8)]
    probes = [p for p in probes if abs(phi0[p]) > 0.05][:6]
    assert len(probes) >= 4
    for node in probes:
        hp = 1e-6
        p1 = phi0.copy()
        p1[node] += hp
        o.init(p1, rho0)
        jp = o.objective(T, grav, objective, window)
        p1[node] -= 2 * hp
        o.init(p1, rho0)
        jm = o.objective(T, grav, objective, window)
        fd = (jp - jm) / (2 * hp)
        # FD roundoff ~1e-16 |J| / h limits the comparison at ~1e-4 relative
        assert abs(lphi[node] - fd) <= 3e-4 * abs(fd) + 1e-16 * abs(J) / hp, node


def test_adjoint_step_dot_product(setup):
    """One step of the FP64 adjoint is the transpose of the step's Jacobian:
    <J v, w> = <v, J^T w> for random v, w at a moving state with gravity.
    J v is the central difference of the FP64 step (eps = 1e-4 on v ~ 1e-3: a
    1e-7 perturbation keeps both the truncation error, ~1e-14, and the
    roundoff, ~1e-16 * 0.05 / 1e-7, far below the bar; the heavy set
    H(phi > 0) of the base state is replayed, so the map is smooth); bar 1e-9
    relative."""
    o, phi0, rho0 = setup
    grav = -3e-5
    o.init(phi0, rho0)
    o.step(5, grav)
    f, g = o.dist()
    rng = np.random.default_rng(11)
    vf, vg = rng.standard_normal(f.shape) * 1e-3, rng.standard_normal(g.shape) * 1e-3
    wf, wg = rng.standard_normal(f.shape), rng.standard_normal(g.shape)
    eps = 1e-4
    o.heavy_mask("record", 1)
    o.set_dist(f, g)
    o.step(1, grav)
    out = []
    for sgn in (1, -1):
        o.heavy_mask("replay")
        o.set_dist(f + sgn * eps * vf, g + sgn * eps * vg)
        o.step(1, grav)
        out.append(o.dist())
    o.heavy_mask("off")
    jvf = (out[0][0] - out[1][0]) / (2 * eps)
    jvg = (out[0][1] - out[1][1]) / (2 * eps)
    lhs = float((jvf * wf).sum() + (jvg * wg).sum())
    o.set_dist(f, g)
    lf, lg, _ = o.adjoint_apply(grav, wf, wg)
    rhs = float((vf * lf).sum() + (vg * lg).sum())
    assert rhs == pytest.approx(lhs, rel=1e-9)
