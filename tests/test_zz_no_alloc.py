"""lbm_stats_noalloc: the statistics entry point for callers that cannot
allocate device memory (in-situ monitoring code running inside another
application's time loop, whose device memory belongs to that application's
pool allocator).  The test owns every buffer -- the fields and the 16-double
output -- and checks that the entry point, which allocates nothing, returns
the same statistics as lbm_stats on two calls in a row.  It lives in a file
that pytest collects last, and passes both alone in a fresh process and after
the rest of the suite."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import REL_TOL, U_TOL


def _params(nx=64, ny=64, nz=64, **kw):
    from lbm_bench_gpu_gb300 import capi
    args = dict(rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=1.0, width=4.0, sigma=1e-3, Gamma=1.0, Eo=-0.4, rc0=10.0)
    args.update(kw)
    return capi.make_params(nx, ny, nz, **args)


def test_noalloc_rejects_boxes_beyond_its_scratch(lib):
    """513 x 512 x 512 nodes do not fit the static partial-sum array: rejected
    before any device work (runs without a GPU)."""
    from lbm_bench_gpu_gb300 import capi
    p = capi.make_params(544, 512, 512, rhoL=0.1, rhoH=1.0, tauRho=0.7, tauPhi=1.0, width=4.0, sigma=1e-3,
                         Gamma=1.0)
    fake = C.c_void_p(16)
    rc = lib.lbm_stats_noalloc(C.byref(p), fake, fake, fake, fake, fake, fake, None)
    assert rc == capi.LBM_EINVAL
    assert "LBM_NOALLOC_MAX_NODES" in lib.lbm_last_error().decode()


def test_noalloc_rejects_underivable_physics(lib):
    """Parameters the constants cannot be derived from (zero interface width)
    are rejected with LBM_EINVAL before any device work (runs without a GPU)."""
    from lbm_bench_gpu_gb300 import capi
    p = _params(width=0.0)
    fake = C.c_void_p(16)
    rc = lib.lbm_stats_noalloc(C.byref(p), fake, fake, fake, fake, fake, fake, None)
    assert rc == capi.LBM_EINVAL
    assert "width" in lib.lbm_last_error().decode()


# a cubic box (16 partial rows) and a non-cubic one with many rows (192)
BOXES = {
    "64^3": ((64, 64, 64), [[31.6, 30.2, 33.4, 10.0], [12.0, 50.0, 20.0, 5.0]]),
    "256x128x96": ((256, 128, 96), [[131.6, 60.2, 43.4, 12.0], [40.0, 100.0, 70.0, 7.0], [200.5, 20.0, 15.0, 6.0]]),
}


@pytest.mark.gpu
@pytest.mark.parametrize("box", sorted(BOXES))
def test_noalloc_stats_match_lbm_stats(lib, box):
    import torch
    from lbm_bench_gpu_gb300 import capi

    shape, bub = BOXES[box]
    p = _params(*shape)
    bubbles = np.array(bub, np.float32)
    with capi.Lattice.from_bubbles(p, bubbles) as lat:
        lat.step(12, capi.derive(p).grav)
        want, fields = lat.stats(fields=True)
    n = p.nx * p.ny * p.nz

    dev = torch.device("cuda", 0)
    # the caller's own buffers (allocated here by the test, not by the entry point)
    dfield = {k: torch.from_numpy(fields[k]).to(dev) for k in ("phi", "rho", "ux", "uy", "uz")}
    out = torch.empty(16, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    ptrs = [C.c_void_p(dfield[k].data_ptr()) for k in ("phi", "rho", "ux", "uy", "uz")]

    for call in range(2):
        out.fill_(float("nan"))   # nothing of an earlier call may leak through
        torch.cuda.synchronize()
        rc = lib.lbm_stats_noalloc(C.byref(p), *ptrs, C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == capi.LBM_OK, lib.lbm_last_error().decode()
        torch.cuda.synchronize()
        raw = out.cpu().numpy()

        vol = raw[1]
        got = {
            "umax": np.sqrt(raw[0]), "vol": vol, "ux_av": raw[2] / vol, "uy_av": raw[3] / vol,
            "uz_av": raw[4] / vol, "p_in": raw[5] / vol, "p_out": raw[6] / (n - vol), "phi_sum": raw[7],
            "rho_sum": raw[8], "mom_x": raw[9], "mom_y": raw[10], "mom_z": raw[11], "vol_full": raw[12],
            "umax_full": np.sqrt(raw[13]),
        }
        assert raw[14] == 0 and raw[15] == 0, f"call {call}"
        for k in ("vol", "vol_full", "umax", "umax_full"):
            assert got[k] == want[k], f"call {call}: {k}"
        # same FP64 sums, different block partition: agree far inside REL_TOL
        for k in ("phi_sum", "rho_sum", "p_in", "p_out"):
            assert got[k] == pytest.approx(want[k], rel=1e-3 * REL_TOL), f"call {call}: {k}"
        for k in ("ux_av", "uy_av", "uz_av"):
            assert abs(got[k] - want[k]) <= 1e-3 * U_TOL, f"call {call}: {k}"
        for k in ("mom_x", "mom_y", "mom_z"):
            assert abs(got[k] - want[k]) <= 1e-3 * U_TOL * want["rho_sum"], f"call {call}: {k}"
