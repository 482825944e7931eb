"""lbm_step_adjoint (GPU: FP32 arithmetic, FP64 sums) against FP64 central
finite differences of the oracle's forward run.

Box 64^3, 2 bubbles of radius 10, tau_rho = 0.8, gravity -1e-6,
T = 400 steps, J = light-phase mean u_z over the last 100 states (the short
adjoint workload's objective on a box the FP64 oracle runs in seconds).

The gravity term is switched on by H(phi > 0) (src/collision_f.cu:96), so
J is only piecewise smooth in the force and in phi0: a node whose phi crosses
zero under the perturbation makes J jump, and plain FP64 differences scatter
by ~2e-4 relative with no convergence in h (1e-6 .. 1e-8).  The discrete
adjoint differentiates the map with the heavy set held fixed, so the finite
differences here replay the heavy set of the unperturbed run (the oracle's
heavy-node log); the plain differences are printed beside them.

* dJ/dgrav: h = 1e-6 on the force; bar 1e-4 relative.
* dJ/dphi0: h = 1e-5 on 8 seeded random nodes among those with |dJ/dphi0|
  above 10% of its maximum (the interface shells, where the gradient lives);
  bar 1e-4 relative per node.

FP32 finite differences of the GPU's own forward run cannot check 1e-4 at
all: the FP32 trajectories for g + h and g - h differ by rounding noise of
about 7e-4 of J at this horizon."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

T, WINDOW, OBJ = 400, 100, "light_uz_mean"


def setup():
    from lbm_bench_gpu_gb300 import capi, inputs
    inp = inputs.Inputs(nx=64, ny=64, nz=64, tauRho=0.8, relax_step=0, max_step=T + 1,
                        bubbles=np.array([[24.3, 30.1, 22.6, 10.0], [40.2, 34.7, 43.9, 10.0]], np.float32))
    inp.Eo = inputs.eo_for_gravity(-1e-6, 10.0, inp.sigma)
    p = capi.make_params(64, 64, 64, rhoL=inp.rhoL, rhoH=inp.rhoH, tauRho=inp.tauRho, tauPhi=inp.tauPhi,
                         width=inp.width, sigma=inp.sigma, Gamma=inp.Gamma, Eo=inp.Eo, rc0=inp.rc0)
    grav = float(capi.derive(p).grav)
    o = Oracle.from_params(p)
    phi0 = o.bubble_phi(inp.bubbles)[1:-1].astype(np.float32)
    rho0 = np.full(phi0.shape, 0.5 * (inp.rhoL + inp.rhoH), np.float32)
    return p, grav, o, phi0, rho0


def J64(o, phi, rho, grav):
    o.init(phi.astype(np.float64), rho.astype(np.float64))
    return o.objective(T, grav, OBJ, WINDOW)


def test_gpu_adjoint_vs_fp64_finite_differences(lib):
    from lbm_bench_gpu_gb300 import capi
    p, grav, o, phi0, rho0 = setup()
    with capi.Lattice.from_fields(p, phi0, rho0) as lat:
        r = lat.adjoint(T, grav, OBJ, WINDOW)
    h = 1e-6
    free = (J64(o, phi0, rho0, grav + h) - J64(o, phi0, rho0, grav - h)) / (2 * h)
    o.heavy_mask("record", T)
    J = J64(o, phi0, rho0, grav)
    o.heavy_mask("replay")
    assert r["J"] == pytest.approx(J, rel=1e-4)
    fd = (J64(o, phi0, rho0, grav + h) - J64(o, phi0, rho0, grav - h)) / (2 * h)
    err_g = abs(r["dJ_dgrav"] - fd) / abs(fd)
    print(f"dJ/dgrav adjoint {r['dJ_dgrav']!r} fd64 frozen {fd!r} (rel err {err_g:.3e}); "
          f"fd64 plain {free!r} (rel err {abs(r['dJ_dgrav'] - free) / abs(free):.3e})")

    g0 = r["dJ_dphi0"]
    big = np.flatnonzero(np.abs(g0) > 0.1 * np.abs(g0).max())
    nodes = np.random.default_rng(20261203).choice(big, size=8, replace=False)
    hp = 1e-5
    errs = []
    for k in nodes:
        vals = []
        for sgn in (1, -1):
            ph = phi0.astype(np.float64)
            ph.flat[k] += sgn * hp
            o.init(ph, rho0.astype(np.float64))
            vals.append(o.objective(T, grav, OBJ, WINDOW))
        fdk = (vals[0] - vals[1]) / (2 * hp)
        errs.append(abs(float(g0.flat[k]) - fdk) / abs(fdk))
    o.heavy_mask("off")
    print(f"dJ/dphi0 on {len(nodes)} nodes (frozen heavy set): rel err max {max(errs):.3e} "
          f"median {np.median(errs):.3e}")
    assert err_g <= 1e-4
    assert max(errs) <= 1e-4
