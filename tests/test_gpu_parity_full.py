"""Per-node parity at the benchmark's own sizes: the GPU path (through the
C-ABI) against the FP64 oracle on every node of phi, rho, u and all 26
streamed distributions.

These boxes exercise what the small parity boxes do not: the per-box chunk
depth with a ragged last chunk (256^3 FP32: 37 planes per block), thousands of
blocks in several waves of programmatically overlapped launches, and the TMA
staging of the P_f planes on interior tiles at full width (16-bit formats).

* the bubbly-flow workload the bench times: 256^3, 64 bubbles R ~ U[6, 10],
  gap >= 3, seed 20261203, gravity -1e-6, in FP32, FP16 and BF16 storage,
  after 1, 2 and 3 steps;
* the short adjoint workload's physics: 128^3, 8 bubbles R = 10,
  tau_rho = 0.8, after 1, 2, 3 and 10 steps (FP32);
* one step of the 512^3 precision workload (512 bubbles R ~ U[6, 12]) in FP16
  storage (the oracle holds ~61 GB of host memory there; skipped with the
  reason when the host has less free).

Tolerances (tests/conftest.py): FP32 1e-5 relative for phi, rho and the f
and g distribution sets, 1e-6 absolute for u; 16-bit storage STORAGE_TOL and
U_TOL_STORAGE.
"""
from __future__ import annotations

import pytest

from conftest import STORAGE_TOL, U_TOL_STORAGE, assert_state_close

pytestmark = pytest.mark.gpu


def params_for(inp, storage="fp32"):
    from lbm_bench_gpu_gb300 import capi
    return capi.make_params(inp.nx, inp.ny, inp.nz, rhoL=inp.rhoL, rhoH=inp.rhoH, tauRho=inp.tauRho,
                            tauPhi=inp.tauPhi, width=inp.width, sigma=inp.sigma, Gamma=inp.Gamma, Eo=inp.Eo,
                            rc0=inp.rc0, storage=storage, compat=True)


def oracle_for(inp):
    from oracle.oracle import Oracle
    o = Oracle.from_params(params_for(inp))
    o.init_bubbles(inp.bubbles)
    return o


def host_free_bytes() -> float:
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    return float(line.split()[1]) * 1024
    except OSError:
        pass
    return 0.0


def run_lockstep(inp, storages, checkpoints, what):
    """Step the oracle and one lattice per storage format side by side and
    compare every lattice with the oracle after each step count in
    `checkpoints`."""
    from lbm_bench_gpu_gb300 import capi
    grav = float(capi.derive(params_for(inp)).grav)
    o = oracle_for(inp)
    lats = {st: capi.Lattice.from_bubbles(params_for(inp, st), inp.bubbles) for st in storages}
    failures = []
    try:
        done = 0
        for n in checkpoints:
            o.step(n - done, grav)
            for st, lat in lats.items():
                lat.step(n - done, grav)
            done = n
            for st, lat in lats.items():
                assert lat.steps == n
                assert_state_close(lat, o, rel=STORAGE_TOL[st], utol=U_TOL_STORAGE[st], what=f"{what} {st} {n} steps",
                                   failures=failures)
    finally:
        for lat in lats.values():
            lat.close()
        o.close()
    assert not failures, "\n".join(failures)


def test_bench_workload_256_per_node():
    """The bench's 256^3 bubbly workload, all three storage formats, 1-3 steps."""
    from lbm_bench_gpu_gb300 import inputs
    inp = inputs.bubbly(256, 64, r_range=(6.0, 10.0), gravity=-1e-6)
    run_lockstep(inp, ("fp32", "fp16", "bf16"), (1, 2, 3), "256^3 bubbly")


def test_adjoint_workload_128_per_node():
    """The short adjoint workload's box and physics (tau_rho = 0.8), FP32."""
    from lbm_bench_gpu_gb300 import inputs
    inp = inputs.adjoint_short()
    run_lockstep(inp, ("fp32",), (1, 2, 3, 10), "128^3 adjoint physics")


def test_precision_workload_512_fp16_one_step():
    """One FP16 step of the 512^3 precision workload (512 bubbles)."""
    from lbm_bench_gpu_gb300 import inputs
    need = 1.2e11   # oracle state (57 arrays of 134M doubles) + the float32 copies compared
    free = host_free_bytes()
    if free < need:
        pytest.skip(f"host has {free / 1e9:.0f} GB free, the 512^3 oracle needs ~{need / 1e9:.0f} GB")
    inp = inputs.bubbly(512, 512, r_range=(6.0, 12.0), gravity=-1e-6)
    run_lockstep(inp, ("fp16",), (1,), "512^3 bubbly")
