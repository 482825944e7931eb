"""GPU path (liblbm_gb300.so through its C-ABI) against the FP64 oracle and the
reference's own outputs.  Tolerances: see conftest (1e-5 relative for phi,
rho and the distribution sets; 1e-6 absolute for u) at <= 100 steps."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, REL_TOL, STORAGE_TOL, U_TOL, U_TOL_STORAGE, assert_fields_close, rel_err

pytestmark = pytest.mark.gpu

PHYS = dict(rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=1.0, width=4.0, sigma=1e-3, Gamma=1.0)


def make(nx, ny, nz, **kw):
    from lbm_bench_gpu_gb300 import capi
    args = dict(PHYS)
    args.update(kw)
    return capi.make_params(nx, ny, nz, **args)   # storage= "fp32" (default), "fp16" or "bf16"


def oracle_for(p, bubbles):
    from oracle.oracle import Oracle
    o = Oracle.from_params(p)
    o.init_bubbles(bubbles)
    return o


def flat_moments(m):
    return {k: v for k, v in m.items()}


BUB32 = np.array([[15.7, 16.2, 16.45, 8.3]], np.float32)


def test_init_matches_oracle(lib):
    from lbm_bench_gpu_gb300 import capi
    p = make(32, 32, 32)
    with capi.Lattice.from_bubbles(p, BUB32) as lat:
        o = oracle_for(p, BUB32)
        assert_fields_close(lat.fields(), o.moments(), what="init")
        f, g = lat.dist()
        fo, go = o.dist()
        assert rel_err(f, fo) <= REL_TOL
        assert rel_err(g, go) <= REL_TOL


def test_init_ghost_planes_from_geometry(lib, golden_manifest, tmp_path):
    """Bubbles reaching the z faces: the initial equilibrium reads ghost planes
    filled from the geometry (src/init.c:41-59), not periodic copies."""
    from lbm_bench_gpu_gb300 import capi
    case = golden_manifest["overlap_ghost32"]
    (tmp_path / "properties.in").write_text(case["properties.in"])
    (tmp_path / "discrete.in").write_text(case["discrete.in"])
    p, _, bub = capi.read_inputs(tmp_path)
    with capi.Lattice.from_bubbles(p, bub) as lat:
        o = oracle_for(p, bub)
        f, g = lat.dist()
        fo, go = o.dist()
        assert rel_err(f, fo) <= REL_TOL and rel_err(g, go) <= REL_TOL
        # a periodic-ghost initialisation differs measurably on this input
        from oracle.oracle import Oracle
        o2 = Oracle.from_params(p)
        pg = o2.bubble_phi(bub)
        o2.init(pg[1:-1], np.full(o2.shape, 0.5 * (o2.rhoH + o2.rhoL)))
        assert rel_err(o2.dist()[0], fo) > 1e-3


@pytest.mark.parametrize("shape", [(32, 32, 32), (64, 32, 48), (32, 8, 40), (96, 16, 33)])
@pytest.mark.parametrize("steps,grav", [(1, 0.0), (2, -2e-5), (3, 0.0), (10, -2e-5)])
def test_steps_match_oracle(lib, shape, steps, grav):
    from lbm_bench_gpu_gb300 import capi, inputs
    nx, ny, nz = shape
    m = min(shape)
    b = np.array([[nx / 2 - 0.3, ny / 2 + 0.2, nz / 2 + 0.4, m / 3], [nx / 4, ny / 4, nz / 4 + 1, m / 5]],
                 np.float32)
    p = make(nx, ny, nz, tauRho=0.8, tauPhi=0.9)
    with capi.Lattice.from_bubbles(p, b) as lat:
        o = oracle_for(p, b)
        lat.step(steps, grav)
        o.step(steps, grav)
        assert lat.steps == steps
        assert_fields_close(lat.fields(), o.moments(), what=f"{shape} {steps} steps")
        f, g = lat.dist()
        fo, go = o.dist()
        assert rel_err(f, fo) <= REL_TOL, "f"
        assert rel_err(g, go) <= REL_TOL, "g"


def test_100_steps_with_gravity(lib):
    from lbm_bench_gpu_gb300 import capi
    p = make(64, 64, 64)
    b = np.array([[31.6, 30.2, 33.4, 10.5], [12.0, 50.0, 20.0, 5.0]], np.float32)
    with capi.Lattice.from_bubbles(p, b) as lat:
        o = oracle_for(p, b)
        for chunk in (1, 9, 40, 50):   # several lbm_step calls, odd and even lengths
            lat.step(chunk, -1e-5)
            o.step(chunk, -1e-5)
        assert_fields_close(lat.fields(), o.moments(), what="100 steps")
        f, g = lat.dist()
        fo, go = o.dist()
        assert rel_err(f, fo) <= REL_TOL and rel_err(g, go) <= REL_TOL


@pytest.mark.parametrize("name", ["relax32", "overlap_ghost32", "sample_ratio"])
def test_gpu_matches_reference_golden(lib, name, golden_manifest, tmp_path):
    """Straight against the reference's own kernels' outputs (FP32 both)."""
    from lbm_bench_gpu_gb300 import capi
    case = golden_manifest[name]
    (tmp_path / "properties.in").write_text(case["properties.in"])
    (tmp_path / "discrete.in").write_text(case["discrete.in"])
    p, _, bub = capi.read_inputs(tmp_path)
    ref = np.load(GOLDEN / f"{name}.npz")
    with capi.Lattice.from_bubbles(p, bub) as lat:
        init = lat.fields()
        assert rel_err(init["phi"], ref["init_phi"]) <= 1e-6
        lat.step(case["steps"], case["grav"])
        got = lat.fields()
    want = {k: ref[k] for k in ("phi", "rho", "ux", "uy", "uz")}
    assert_fields_close(got, want, rel=2 * REL_TOL, utol=U_TOL, what=f"golden {name}")


def random_state(shape, seed, p):
    """A smooth random state near equilibrium with non-zero velocity."""
    from oracle.oracle import Oracle
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    phi = 0.45 * np.tanh(2.0 * np.sin(2 * np.pi * x / nx + rng.uniform(0, 6)) * np.cos(2 * np.pi * z / nz)
                         + np.cos(2 * np.pi * y / ny))
    o = Oracle.from_params(p)
    o.init(phi, np.full(shape, 0.55) + 0.01 * np.sin(2 * np.pi * z / nz))
    f, g = o.dist()
    g = g * (1.0 + 0.02 * rng.standard_normal(g.shape))
    f = f + 1e-3 * rng.standard_normal(f.shape)
    return f, g


@pytest.mark.parametrize("steps", [1, 2, 5])
def test_random_state_parity(lib, steps):
    """Arbitrary (non-equilibrium, moving) states set through lbm_set_dist."""
    from lbm_bench_gpu_gb300 import capi
    from oracle.oracle import Oracle
    p = make(32, 16, 24, tauRho=0.65, tauPhi=0.75)
    f, g = random_state((24, 16, 32), 5, p)
    f32, g32 = f.astype(np.float32), g.astype(np.float32)
    with capi.Lattice.from_fields(p, np.zeros((24, 16, 32), np.float32), np.full((24, 16, 32), 0.55, np.float32)) as lat:
        lat.set_dist(f32, g32)
        f_back, g_back = lat.dist()
        assert np.array_equal(f_back, f32) and np.array_equal(g_back, g32)   # exact round trip
        o = Oracle.from_params(p)
        o.init(np.zeros((24, 16, 32)), np.full((24, 16, 32), 0.55))
        o.set_dist(f32.astype(np.float64), g32.astype(np.float64))
        lat.step(steps, 3e-5)
        o.step(steps, 3e-5)
        assert_fields_close(lat.fields(), o.moments(), what="random state")
        f1, g1 = lat.dist()
        fo, go = o.dist()
        assert rel_err(f1, fo) <= REL_TOL and rel_err(g1, go) <= REL_TOL


def test_stats_match_oracle(lib):
    from lbm_bench_gpu_gb300 import capi
    p = make(64, 64, 64, Eo=-0.4, rc0=10.0)
    b = np.array([[31.6, 30.2, 33.4, 10.0], [12.0, 50.0, 20.0, 5.0]], np.float32)
    with capi.Lattice.from_bubbles(p, b) as lat:
        o = oracle_for(p, b)
        for s_gpu, s_or in ((lat.stats()[0], o.stats()),):
            assert s_gpu["vol"] == s_or["vol"]
        lat.step(20, -1e-6)
        o.step(20, -1e-6)
        s, _ = lat.stats()
        so = o.stats()
    assert s["step"] == 20
    assert s["vol"] == pytest.approx(so["vol"], abs=2)      # nodes at phi ~ 0 may flip sign
    assert s["vol_full"] == pytest.approx(so["vol_full"], abs=2)
    assert s["phi_sum"] == pytest.approx(so["phi_sum"], rel=1e-6)
    assert s["rho_sum"] == pytest.approx(so["rho_sum"], rel=1e-6)
    assert s["umax"] == pytest.approx(so["umax"], abs=U_TOL)
    assert s["p_dif"] == pytest.approx(so["p_dif"], rel=1e-3)
    assert s["ref"] == pytest.approx(so["ref"], rel=1e-3)
    for k in ("mom_x", "mom_y", "mom_z"):
        # a momentum sum over n nodes: 1% of U_TOL per node on average
        assert abs(s[k] - so[k]) <= 1e-2 * U_TOL * so["rho_sum"]
    assert s["nonfinite"] == 0


def test_nan_is_reported(lib):
    """Failure detection: a NaN planted on the host surfaces as LBM_ENAN."""
    from lbm_bench_gpu_gb300 import capi
    p = make(32, 32, 32)
    with capi.Lattice.from_bubbles(p, BUB32) as lat:
        f, g = lat.dist()
        g[3, 5, 6, 7] = np.nan
        lat.set_dist(f, g)
        lat.step(2)
        with pytest.raises(capi.LbmError) as e:
            lat.stats()
        assert e.value.code == capi.LBM_ENAN
        s, _ = lat.stats(allow_nan=True)
        assert s["nonfinite"] > 0


def test_timed_out_wait_is_reported_and_context_stays_usable(lib):
    """Failure detection on the device without a fault: a bounded wait on a
    barrier that nothing completes gives up (the step kernel's wait and error
    flag), the host reads LBM_ETIMEOUT, and the same context then steps and
    matches the oracle."""
    from lbm_bench_gpu_gb300 import capi
    p = make(32, 32, 32)
    with capi.Lattice.from_bubbles(p, BUB32) as lat:
        assert lat.wait_selftest() == capi.LBM_ETIMEOUT
        lat.sync()                                    # the flag was cleared
        lat.step(3, -2e-5)
        o = oracle_for(p, BUB32)
        o.step(3, -2e-5)
        assert_fields_close(lat.fields(), o.moments(), what="after the self-test")


def test_full_size_conservation(lib):
    """256^3, 64 bubbles (the bench workload): sum phi and sum rho stay put."""
    from lbm_bench_gpu_gb300 import capi, inputs
    inp = inputs.bubbly(256, 64)
    p = make(256, 256, 256, Eo=inp.Eo, rc0=inp.rc0)
    with capi.Lattice.from_bubbles(p, inp.bubbles) as lat:
        s0, _ = lat.stats()
        grav = capi.derive(p).grav
        lat.step(50, grav)
        s1, _ = lat.stats()
    assert s1["nonfinite"] == 0
    assert abs(s1["phi_sum"] - s0["phi_sum"]) <= 1e-6 * abs(s0["phi_sum"])
    assert abs(s1["rho_sum"] - s0["rho_sum"]) <= 1e-6 * abs(s0["rho_sum"])
    assert s1["vol"] == pytest.approx(s0["vol"], rel=2e-2)


# 16-bit storage (f_1..f_6 and g in FP16 / BF16 with a shifted, power-of-two
# scaled map; f_0 and all arithmetic FP32).  Tolerances against the FP64
# oracle at 10 steps (conftest): FP16 5e-5 relative (phi, rho, distributions)
# and 1e-5 absolute on u; BF16 (8-bit mantissa) 5e-4 and 5e-5.


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_storage_roundtrip_error_bound(lib, storage):
    """lbm_set_dist -> lbm_get_dist: every value within half a unit in the last
    place of its shifted, scaled 16-bit encoding."""
    from lbm_bench_gpu_gb300 import capi
    p = make(32, 16, 24, tauRho=0.65, tauPhi=0.75, storage=storage)
    f, g = random_state((24, 16, 32), 5, make(32, 16, 24, tauRho=0.65, tauPhi=0.75))
    f32, g32 = f.astype(np.float32), g.astype(np.float32)
    with capi.Lattice.from_fields(p, np.zeros((24, 16, 32), np.float32), np.full((24, 16, 32), 0.55, np.float32)) as lat:
        lat.set_dist(f32, g32)
        fb, gb = lat.dist()
    assert np.array_equal(fb[0], f32[0])                      # f_0 stays FP32
    ulp = 2.0 ** -11 if storage == "fp16" else 2.0 ** -8
    rho_mean = g32.sum(axis=0).mean()
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    for i in range(19):
        dev = np.abs(g32[i] - w[i] * rho_mean).max()
        assert np.abs(gb[i] - g32[i]).max() <= ulp * dev * 1.01 + 1e-9, f"g{i}"
    for i in range(1, 7):
        assert np.abs(fb[i] - f32[i]).max() <= ulp * np.abs(f32[i]).max() * 1.01 + 1e-12, f"f{i}"


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
@pytest.mark.parametrize("steps", [1, 2, 10])
@pytest.mark.parametrize("shape", [(64, 32, 48), (32, 8, 12), (128, 32, 16)])
def test_storage_steps_match_oracle(lib, storage, steps, shape):
    """16-bit storage (two nodes per thread in the step kernel) against the
    FP64 oracle; the 32 x 8 x 12 box is one tile in x and y, so every +-x and
    +-y neighbour of an odd step wraps inside the block's own tile; the
    128 x 32 x 16 box has interior tiles, whose P_f planes come by TMA (the
    tiles at the periodic seam stage them with cp.async)."""
    from lbm_bench_gpu_gb300 import capi
    nx, ny, nz = shape
    if shape == (64, 32, 48):
        b = np.array([[nx / 2 - 0.3, ny / 2 + 0.2, nz / 2 + 0.4, 10.0], [16, 8, 13, 6.0]], np.float32)
    elif shape == (128, 32, 16):
        b = np.array([[50.3, 15.8, 8.4, 6.0], [97.1, 9.2, 7.7, 4.5]], np.float32)
    else:
        b = np.array([[nx / 2 - 0.3, ny / 2 + 0.2, nz / 2 + 0.4, 3.0], [7.5, 2.2, 3.1, 2.0]], np.float32)
    p = make(nx, ny, nz, tauRho=0.8, tauPhi=0.9, storage=storage)
    tol = STORAGE_TOL[storage]
    with capi.Lattice.from_bubbles(p, b) as lat:
        o = oracle_for(make(nx, ny, nz, tauRho=0.8, tauPhi=0.9), b)
        lat.step(steps, -2e-5)
        o.step(steps, -2e-5)
        assert_fields_close(lat.fields(), o.moments(), rel=tol, utol=U_TOL_STORAGE[storage],
                            what=f"{storage} {steps}")
        f, g = lat.dist()
        fo, go = o.dist()
        assert rel_err(f, fo) <= tol and rel_err(g, go) <= tol
