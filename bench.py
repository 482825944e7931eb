#!/usr/bin/env python3
"""Benchmark of the fused ZSC step on GB300.

Workload (default): 256^3 periodic box, 64 bubbles with radii uniform in
[6, 10] placed by seeded rejection sampling (surface gap >= 3), rhoH = 1,
rhoL = 0.1, sigma = 1e-3, W = 4, tau_rho = 0.7, Gamma = 1, tau_phi = 1,
gravity -1e-6 along z, FP32 storage.  A "step" is one lattice Boltzmann
time step over the whole box (one fused kernel launch).  The state
(26 x 4 B x 16.8M nodes = 1.75 GB) is far larger than the 129 MB L2, so no
L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own step (its seven kernels and three
halo exchanges, compiled for the host CPU from the reference sources) on the
host cores, on a slab of the same workload sized so the run stays within a
few minutes.  For N > 1 (torchrun) every rank runs an independent replica of
the workload on its own GPU (the step has no cross-GPU exchange here).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "MLUPS + HBM GB/s (FP32 vs FP16-storage) at 256^3; adjoint-to-forward time ratio"
# algorithmic bytes per lattice update: every distribution read and written once
# (16-bit formats keep the D3Q7 rest population f_0 in FP32)
BYTES_PER_NODE = {"fp32": 26 * 2 * 4, "fp16": 2 * 4 + 25 * 2 * 2, "bf16": 2 * 4 + 25 * 2 * 2}
FALLBACK_HBM_GBS = 6800.0


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--bubbles", type=int, default=64)
    ap.add_argument("--storage", default="fp32")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="time only --storage (not the other formats)")
    ap.add_argument("--stat-every", type=int, default=100, help="lbm_stats cadence inside the e2e run")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint / forward time ratio")
    ap.add_argument("--no-ref-cuda", action="store_true", help="skip timing the reference's own CUDA build")
    ap.add_argument("--ref-cuda-steps", type=int, default=500)
    ap.add_argument("--precision", action="store_true",
                    help="also run the storage-precision study at 256^3 and 512^3 (10k steps per format)")
    ap.add_argument("--precision-steps", type=int, default=10000)
    ap.add_argument("--adjoint-long", action="store_true",
                    help="also run the long-horizon adjoint (256^3, 64 bubbles, T = 20000, FP16 state, 40 GB)")
    return ap.parse_args(argv)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(size: int, nbubbles: int):
    from lbm_bench_gpu_gb300 import inputs
    r_range = (6.0, 10.0) if size <= 256 else (6.0, 12.0)
    return inputs.bubbly(size, nbubbles, r_range=r_range, gravity=-1e-6)


def workload_config(args, inp, world: int) -> dict:
    """The `config` object of the JSON line, shared by both arms."""
    r_range = list((6.0, 10.0) if args.size <= 256 else (6.0, 12.0))
    return {"workload": f"bubbly_{args.size}: {args.size}^3 periodic, {args.bubbles} bubbles R~U{r_range}, gap>=3, "
                        "rhoH=1 rhoL=0.1 sigma=1e-3 W=4 tau_rho=0.7 Gamma=1 tau_phi=1, gravity -1e-6 along z",
            "nx": inp.nx, "ny": inp.ny, "nz": inp.nz, "bubbles": args.bubbles, "storage": args.storage,
            "seed": 20261203, "parallelism": f"replicas x{world}",
            "l2": "state >= 1.5 GB >> 129 MB L2: no flush needed"}


def params_for(inp, storage="fp32", device=0):
    from lbm_bench_gpu_gb300 import capi
    return capi.make_params(inp.nx, inp.ny, inp.nz, rhoL=inp.rhoL, rhoH=inp.rhoH, tauRho=inp.tauRho,
                            tauPhi=inp.tauPhi, width=inp.width, sigma=inp.sigma, Gamma=inp.Gamma, Eo=inp.Eo,
                            rc0=inp.rc0, storage=storage, device=device, compat=True)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def profiled_traffic(storage: str, size: int):
    """dram bytes read + written per step-kernel launch from the committed ncu summary."""
    f = ROOT / "profiles" / f"zsc_step_{storage}_{size}cube.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith("dram_bytes_per_launch"):
            try:
                return float(line.split("=")[1].split()[0])
            except Exception:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None
        self.out = tempfile.NamedTemporaryFile(prefix="clocks_", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_id}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.out, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        self.out.close()

    def summary(self, t_start: float, t_end: float):
        try:
            rows = [l.split(",") for l in Path(self.out.name).read_text().splitlines() if l.strip()]
        except Exception:
            rows = []
        finally:
            try:
                os.unlink(self.out.name)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if len(r) > 2 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].strip().lower().startswith("active"):
                    reasons.add(n)
        # samples under load: clocks above the idle floor
        load = [s for s in sm if s > 0.5 * max(sm)] if sm else []
        return {"sm_mhz": float(np.median(load)) if load else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_identity(device: int) -> str:
    import torch
    props = torch.cuda.get_device_properties(device)
    uuid = getattr(props, "uuid", None)
    if uuid is not None:
        s = str(uuid)
        return s if s.startswith("GPU-") else "GPU-" + s
    return str(device)


def cpu_baseline(inp, budget_s: float = 15.0):
    """The FP64 oracle (C/OpenMP) on the host cores, on the same 256^3 workload,
    timed over as many steps as fit in ~budget_s."""
    from oracle.oracle import Oracle
    from lbm_bench_gpu_gb300 import capi
    p = params_for(inp)
    o = Oracle.from_params(p)
    o.init_bubbles(inp.bubbles)
    grav = float(capi.derive(p).grav)
    t0 = time.perf_counter()
    o.step(1, grav)
    t1 = time.perf_counter() - t0
    n = int(max(1, min(20, budget_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    o.step(n, grav)
    dt = time.perf_counter() - t0
    nodes = inp.nx * inp.ny * inp.nz
    o.close()
    out = {"value": nodes * n / dt / 1e6, "unit": "MLUPS", "cores": Oracle.threads(), "kind": "port",
           "cpu_model": cpu_model(),
           "sample": f"FP64 oracle, full {inp.nx}x{inp.ny}x{inp.nz} box, {n} steps after 1 untimed step "
                     f"({dt:.1f} s)"}
    # the static-bubble case in full: 64^3, one bubble R = 12, 1000 relaxation steps
    from lbm_bench_gpu_gb300 import inputs
    s1 = inputs.static_bubble()
    o = Oracle.from_params(params_for(s1))
    o.init_bubbles(s1.bubbles)
    t0 = time.perf_counter()
    o.step(1000, 0.0)
    dt1 = time.perf_counter() - t0
    o.close()
    out["static_bubble_64"] = {"value": s1.nx * s1.ny * s1.nz * 1000 / dt1 / 1e6, "unit": "MLUPS",
                               "seconds": round(dt1, 2), "sample": "64^3, one bubble R = 12, 1000 steps, in full"}
    return out


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the architecture)."""
    import platform
    import subprocess
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for line in r.stdout.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip() + f" ({platform.machine()})"
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def max_over_ranks(x: float, local: int = 0) -> float:
    """The largest x over the ranks of the process group (x itself without one):
    the job's time is its slowest replica's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = f"cuda:{local}" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def time_storage(inp, storage, local, K, W, sampler=None):
    """Device time (ms) of K fused steps on resident state, CUDA events on the
    context's stream."""
    import torch
    from lbm_bench_gpu_gb300 import capi
    p = params_for(inp, storage, local)
    grav = float(capi.derive(p).grav)
    lat = capi.Lattice.from_bubbles(p, inp.bubbles)
    stream = torch.cuda.ExternalStream(lat.stream, device=local)
    lat.step(W, grav)
    lat.sync()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if sampler:
        sampler.__enter__()
    e0.record(stream)
    lat.step(K, grav)
    e1.record(stream)
    e1.synchronize()
    if sampler:
        sampler.__exit__(None, None, None)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), local)
    s, _ = lat.stats()
    lat.close()
    if s["nonfinite"]:
        raise RuntimeError(f"state went non-finite during the {storage} bench")
    return ms


def run_ours(args, rank, world, local):
    import torch
    from lbm_bench_gpu_gb300 import capi

    torch.cuda.set_device(local)
    inp = workload(args.size, args.bubbles)
    p = params_for(inp, args.storage, local)
    grav = float(capi.derive(p).grav)
    nodes = inp.nx * inp.ny * inp.nz
    K, W = args.steps, args.warmup

    sampler = ClockSampler(gpu_identity(local)) if rank == 0 else None
    ms = time_storage(inp, args.storage, local, K, W, sampler)

    ms_step = ms / K
    value = world * nodes * K / (ms / 1e3) / 1e6
    bpn = BYTES_PER_NODE[args.storage]
    achieved = bpn * nodes / (ms_step / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = profiled_traffic(args.storage, args.size)
    result = {
        "metric": METRIC, "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": round(ms_step, 5), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.storage == "fp32" else f"f32 ({args.storage} storage)", "data": "synthetic",
        "config": workload_config(args, inp, world),
        "hbm_gbs": round(achieved, 1),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "algorithmic_bytes_per_launch": bpn * nodes, "peak_source": peak_kind},
        "gpu_launches": K,
    }
    if sampler:
        result["clocks"] = sampler.summary(0, 0)
    if not args.no_variants:
        variants = {}
        for st in ("fp32", "fp16", "bf16"):
            if st == args.storage:
                continue
            ms_v = time_storage(inp, st, local, K, W)
            b_v = BYTES_PER_NODE[st]
            mlups = world * nodes * K / (ms_v / 1e3) / 1e6
            variants[st] = {"value": round(mlups, 1), "unit": "MLUPS", "ms_per_step": round(ms_v / K, 5),
                            "hbm_gbs": round(b_v * nodes / (ms_v / K / 1e3) / 1e9, 1),
                            "roofline_frac": round(b_v * nodes / (ms_v / K / 1e3) / 1e9 / peak, 4),
                            "bytes_per_node": b_v, "speedup_vs_headline": round(mlups / value, 3)}
        result["storage_variants"] = variants
    if not args.no_e2e:
        # every rank runs its replica's end-to-end sequence; the job's time is
        # the slowest rank's
        result["e2e"] = run_e2e(args, inp, p, grav, local, world)
    if rank == 0 and not args.no_adjoint:
        result["adjoint"] = run_adjoint(local)
        if args.adjoint_long:
            result["adjoint_long"] = run_adjoint(local, long_horizon=True)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(inp)
    if rank == 0 and world == 1 and not args.no_ref_cuda:
        result["reference_cuda"] = run_reference_cuda(inp, args.ref_cuda_steps, local, value)
    if rank == 0 and args.precision:
        result["precision_large"] = run_precision(local, args.precision_steps)
    return result


def heavy_centroids(phi):
    """Centroids (z, y, x) of the connected phi > 0 regions."""
    from scipy import ndimage
    lab, n = ndimage.label(phi > 0)
    if n == 0:
        return np.zeros((0, 3))
    return np.array(ndimage.center_of_mass(phi > 0, lab, range(1, n + 1)))


def run_precision(local, steps):
    """Storage precision at the benchmark's sizes: 256^3 with 64 bubbles R~U[6,10]
    and 512^3 with 512 bubbles R~U[6,12] (gap >= 3, seeded), gravity -1e-6,
    `steps` steps in FP32, FP16 and BF16 storage.  The errors are taken against the
    FP32-storage GPU run: the FP64 oracle would need ~48 minutes of the host per
    10k steps at 256^3, and at 64^3 FP32 storage stays within 1.1e-4 (phi L2) of
    it after 10k steps (tests/test_precision_study.py).  Per format: MLUPS over
    the run (CUDA events), phi L2 relative error, the drift of sum(phi) and
    sum(rho) from their initial values, and the largest distance from a FP32
    heavy-phase centroid to the nearest one of the format."""
    import torch
    from lbm_bench_gpu_gb300 import capi
    out = {"steps": steps, "reference": "FP32-storage GPU run"}
    for size, nb in ((256, 64), (512, 512)):
        inp = workload(size, nb)
        nodes = inp.nx * inp.ny * inp.nz
        res, phis = {}, {}
        for st in ("fp32", "fp16", "bf16"):
            p = params_for(inp, st, local)
            grav = float(capi.derive(p).grav)
            with capi.Lattice.from_bubbles(p, inp.bubbles) as lat:
                s0, _ = lat.stats()
                stream = torch.cuda.ExternalStream(lat.stream, device=local)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                lat.step(steps, grav)
                e1.record(stream)
                e1.synchronize()
                ms = e0.elapsed_time(e1)
                s, f = lat.stats(fields=True)
            phis[st] = f["phi"]
            res[st] = {"mlups": round(nodes * steps / (ms / 1e3) / 1e6, 1),
                       "phi_sum_drift": (s["phi_sum"] - s0["phi_sum"]) / abs(s0["phi_sum"]),
                       "rho_sum_drift": (s["rho_sum"] - s0["rho_sum"]) / abs(s0["rho_sum"]),
                       "nonfinite": s["nonfinite"]}
        ref = phis["fp32"].astype(np.float64)
        cref = heavy_centroids(phis["fp32"])
        for st in ("fp16", "bf16"):
            d = phis[st].astype(np.float64) - ref
            res[st]["phi_l2_rel_vs_fp32"] = float(np.linalg.norm(d) / np.linalg.norm(ref))
            c = heavy_centroids(phis[st])
            res[st]["bubbles"] = [int(len(cref)), int(len(c))]
            if len(c) and len(cref):
                dist = np.sqrt(((cref[:, None, :] - c[None, :, :]) ** 2).sum(-1)).min(1)
                res[st]["centroid_err_max"] = float(dist.max())
            res[st]["speedup_vs_fp32"] = round(res[st]["mlups"] / res["fp32"]["mlups"], 3)
        out[f"{size}^3"] = res
        del phis
    return out


REF_STATS_KEYS = ("ux", "uy", "uz", "Umax", "Vef", "Ref")


def run_reference_cuda(inp, steps, local, ours_mlups):
    """The reference's own CUDA program on this GPU (baseline only).

    oracle/_ref/lbm_ref_cuda is src/main.cu compiled unmodified for sm_103a with
    src/Makefile's -O3 -use_fast_math and a single-rank MPI stub (one rank
    exchanges its z halos with itself: periodic wrap, as here).  It runs the
    same box and physics with the first 20 bubbles of the workload (its
    MAX_BUBBLES, src/constants.h:28; the step's cost does not depend on the
    bubbles), relaxStep = 0 and `steps` evolution steps, stats and VTK output
    outside the loop (its three ASCII VTK files go to /dev/null).  The value is
    its own "Evolution time" (CUDA events around the evolution loop,
    src/main.cu:613-624) per step; every step includes its seven kernels, six
    pack/unpack kernels and three host-staged halo exchanges.  Its final stats.out line is
    compared with lbm_stats of this library after the same steps from the same
    input."""
    import dataclasses
    from lbm_bench_gpu_gb300 import capi, inputs
    binary = ROOT / "oracle" / "_ref" / "lbm_ref_cuda"
    if not binary.exists():
        return {"unavailable": "oracle/_ref/lbm_ref_cuda not built (reference sources absent at build time)"}
    sub = dataclasses.replace(inp, bubbles=inp.bubbles[:20], max_step=steps + 1, relax_step=0,
                              save=10 ** 9, stat=10 ** 9)
    nodes = inp.nx * inp.ny * inp.nz
    with tempfile.TemporaryDirectory() as d:
        inputs.write_inputs(d, sub)
        for name in ("relax_data_00_0000000.vtk", "data_00_0000000.vtk", f"data_00_{steps + 1:07d}.vtk"):
            os.symlink("/dev/null", os.path.join(d, name))
        env = dict(os.environ, CUDA_VISIBLE_DEVICES=os.environ.get("CUDA_VISIBLE_DEVICES", str(local)))
        t0 = time.perf_counter()
        r = subprocess.run([str(binary)], cwd=d, capture_output=True, text=True, timeout=900, env=env)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            return {"unavailable": f"reference CUDA build exited {r.returncode}: {r.stderr.strip()[-200:]}"}
        evo = None
        for line in r.stdout.splitlines():
            if line.startswith("Evolution time"):
                evo = float(line.split(":")[1].split()[0])
        rows = [l.split() for l in Path(d, "stats.out").read_text().splitlines() if l and not l.startswith("#")]
    if evo is None or not rows:
        return {"unavailable": "reference CUDA build printed no evolution time / stats"}
    ref = dict(zip(REF_STATS_KEYS, map(float, rows[-1][1:7])))
    ms_step = evo / steps
    out = {"value": round(nodes / (ms_step / 1e3) / 1e6, 1), "unit": "MLUPS", "ms_per_step": round(ms_step, 4),
           "steps": steps, "speedup_of_ours": round(ours_mlups / (nodes / (ms_step / 1e3) / 1e6), 2),
           "kind": "reference src/main.cu, nvcc -O3 -use_fast_math sm_103a, one rank (MPI stub)",
           "sample": f"{inp.nx}^3, first 20 of the workload's bubbles, {steps} evolution steps, "
                     f"its own CUDA-event evolution time; process wall {wall:.1f} s",
           "final_stats": ref}
    # the same run through this library: moments at the start of the last step, compat stats
    p = params_for(sub, "fp32", local)
    grav = float(capi.derive(p).grav)
    with capi.Lattice.from_bubbles(p, sub.bubbles) as lat:
        s0, _ = lat.stats()
        lat.step(steps, grav)
        s, _ = lat.stats()
    ours = {"ux": s["ux_av"], "uy": s["uy_av"], "uz": s["uz_av"], "Umax": s["umax"],
            "Vef": s["vol"] / s0["vol"], "Ref": s["ref"]}
    out["ours_final_stats"] = ours
    out["stats_rel_diff"] = {k: abs(ours[k] - ref[k]) / max(abs(ref[k]), 1e-30) for k in REF_STATS_KEYS}
    return out


def run_adjoint(local, long_horizon=False):
    """Adjoint / forward wall-time ratio through lbm_step_adjoint.

    short: 128^3, 8 bubbles R = 10, tau_rho = 0.8, gravity -1e-6, T = 2000,
           J = light-phase mean u_z over the last 200 states, FP32 state; the
           workload names no checkpoint budget, so the headline is the
           library's default (the free device memory less a reserve of
           max(4 GiB, 5%)), with a 40 GB
           budget reported beside it;
    long:  256^3, 64 bubbles R ~ U[6, 10], T = 20000, J = final light-phase
           z-centroid, FP16 live state (native FP16 snapshots), 40 GB budget.
    Each budget is called twice on one context: the first call allocates the
    workspace and the checkpoint pool (reported as first_call), the second
    reuses them (the reported ratio); device_GB is the memory the call holds
    (workspace + pool, from the free memory before and after) plus the
    context's state.  The forward time is lbm_step over T steps.  dJ/dgrav is
    compared with central differences of J from lbm_objective (the GPU forward
    run) at h = 1e-6, 5e-7, 2.5e-7 on the force (down to 6.25e-8 on the long
    run, whose J is far from linear over |h| ~ |g|); fd_rel_err uses the
    smallest h and fd_richardson extrapolates the two smallest.  These FP32
    differences carry the trajectory's rounding noise (~7e-4 of J on the short
    run); the 1e-4 check against FP64 differences is
    tests/test_gpu_adjoint_fd64.py."""
    import torch
    from lbm_bench_gpu_gb300 import capi, inputs
    if long_horizon:
        inp = inputs.bubbly(256, 64, gravity=-1e-6, tauRho=0.7)
        T, objective, window, storage = 20000, "light_z_centroid", 1, "fp16"
    else:
        inp = inputs.adjoint_short()
        T, objective, window, storage = 2000, "light_uz_mean", 200, "fp32"
    p = params_for(inp, storage, local)
    grav = float(capi.derive(p).grav)
    n = inp.nx * inp.ny * inp.nz
    esz = 4 if storage == "fp32" else 2
    state_bytes = n * (2 * 4 + 2 * 6 * esz + 19 * esz + 5 * 4)   # f0 A/B, fq A/B, g, moments

    with capi.Lattice.from_bubbles(p, inp.bubbles) as lat:
        phi0 = lat.fields()["phi"]
        rho0 = lat.fields()["rho"]

    def forward_time(g):
        with capi.Lattice.from_bubbles(p, inp.bubbles) as lat:
            lat.sync()
            t0 = time.perf_counter()
            lat.step(T, g)
            lat.sync()
            return time.perf_counter() - t0

    t_fwd = min(forward_time(grav) for _ in range(2))

    def measure(lat, budget, want_phi0, host=0.0):
        lat.adjoint_release()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        first = lat.adjoint(T, grav, objective, window, checkpoint_bytes=budget, want_phi0=want_phi0,
                            host_checkpoint_bytes=host)
        held = free0 - torch.cuda.mem_get_info()[0]
        warm = lat.adjoint(T, grav, objective, window, checkpoint_bytes=budget, want_phi0=want_phi0,
                           host_checkpoint_bytes=host)
        return {"adjoint_s": round(warm["seconds"], 4), "ratio": round(warm["seconds"] / t_fwd, 3),
                "first_call": {"adjoint_s": round(first["seconds"], 4),
                               "ratio": round(first["seconds"] / t_fwd, 3),
                               "same_gradient": first["dJ_dgrav"] == warm["dJ_dgrav"]},
                "slots": warm["slots"], "checkpoint_GB": round(warm["checkpoint_bytes_used"] / 1e9, 2),
                "device_GB": round((held + state_bytes) / 1e9, 2),
                "forward_steps": warm["forward_steps"], "host_slots": warm["host_slots"]}, warm

    with capi.Lattice.from_fields(p, phi0, rho0) as lat:
        lat.sync()
        torch.cuda.synchronize()
        head, r = measure(lat, 40e9 if long_horizon else 0.0, True)
        other = host_tier = None
        if not long_horizon:
            other, r40 = measure(lat, 40e9, False)
            other["same_gradient"] = r40["dJ_dgrav"] == r["dJ_dgrav"]
        else:
            # the same 40 GB of device checkpoints and a second tier of 60 GB
            # of pinned host memory
            host_tier, rh = measure(lat, 40e9, False, host=60e9)
            host_tier["same_gradient"] = rh["dJ_dgrav"] == r["dJ_dgrav"]
        fd = {}
        hs = (1e-6, 5e-7, 2.5e-7) if not long_horizon else (1e-6, 5e-7, 2.5e-7, 1.25e-7, 6.25e-8)
        for h in hs:
            fd[h] = (lat.objective(T, grav + h, objective, window)
                     - lat.objective(T, grav - h, objective, window)) / (2 * h)
    rich = (4 * fd[hs[-1]] - fd[hs[-2]]) / 3
    out = {"workload": ("long: 256^3, 64 bubbles, T=20000, final light-phase z-centroid, FP16 state"
                        if long_horizon else
                        "short: 128^3, 8 bubbles R=10, tau_rho=0.8, T=2000, light-phase mean u_z over the "
                        "last 200 states, FP32 state"),
           "T": T, "forward_s": round(t_fwd, 4),
           "budget": "40 GB" if long_horizon else "library default: free device memory less max(4 GiB, 5%)"}
    out.update(head)
    out.update({"J": r["J"], "dJ_dgrav": r["dJ_dgrav"],
                "fd_dJ_dgrav": {f"{h:g}": v for h, v in fd.items()}, "fd_richardson": rich,
                "fd_rel_err": abs(r["dJ_dgrav"] - fd[hs[-1]]) / abs(fd[hs[-1]]),
                "fd_rel_err_richardson": abs(r["dJ_dgrav"] - rich) / abs(rich),
                "dJ_dphi0_norm": float(np.sqrt((r["dJ_dphi0"].astype(np.float64) ** 2).sum()))})
    if other is not None:
        out["budget_40GB"] = other
    if host_tier is not None:
        out["host_tier_60GB"] = host_tier
    return out


def run_e2e(args, inp, p, grav, local, world: int = 1):
    """Same metric through the C-ABI with host buffers: lbm_init from pinned host
    fields (upload inside the timed region), K steps with lbm_stats every
    `stat_every` steps (scalar diagnostics back to the host, as the reference
    driver does with stats()), and the final phi, rho, u copied back."""
    import torch
    from lbm_bench_gpu_gb300 import capi
    nodes = inp.nx * inp.ny * inp.nz
    K = args.steps
    with capi.Lattice.from_bubbles(p, inp.bubbles) as seed_lat:
        f0 = seed_lat.fields()
    shape = (inp.nz, inp.ny, inp.nx)
    host_in = {k: torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy() for k in f0}
    host_out = {k: torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy() for k in f0}
    for k in f0:
        host_in[k][...] = f0[k]
        # set-up, like the inputs: the output buffers are written once before
        # the timed read-back
        host_out[k].fill(0.0)
    torch.cuda.synchronize()
    import ctypes as C
    n_stats = 0
    t_steps = t_stats = 0.0
    t0 = time.perf_counter()
    lat = capi.Lattice.from_fields(p, host_in["phi"], host_in["rho"], host_in["ux"], host_in["uy"], host_in["uz"])
    t_init = time.perf_counter() - t0
    done = 0
    while done < K:
        n = min(args.stat_every, K - done)
        ta = time.perf_counter()
        lat.step(n, grav)
        lat.sync()
        tb = time.perf_counter()
        done += n
        lat.stats()
        n_stats += 1
        t_steps += tb - ta
        t_stats += time.perf_counter() - tb
    # the final fields (the statistics of step K came with the loop's last call)
    ta = time.perf_counter()
    capi.check(capi.load().lbm_stats(lat._h, None, *[capi.fptr(host_out[k]) for k in
                                                      ("phi", "rho", "ux", "uy", "uz")]), "lbm_stats")
    t_down = time.perf_counter() - ta
    dt = max_over_ranks(time.perf_counter() - t0, local)
    lat.close()
    h2d = world * 5 * nodes * 4                 # every replica's upload and read-back
    d2h = world * (n_stats * 16 * 8 + 5 * nodes * 4)
    return {"value": round(world * nodes * K / dt / 1e6, 1), "unit": "MLUPS",
            "h2d_bytes_per_step": round(h2d / K, 1), "d2h_bytes_per_step": round(d2h / K, 1),
            "breakdown_s": {"init_s": round(t_init, 5), "steps_s": round(t_steps, 5), "stats_s": round(t_stats, 5),
                            "download_s": round(t_down, 5), "total_s": round(dt, 5)},
            "steps_only_mlups": round(world * nodes * K / t_steps / 1e6, 1) if t_steps > 0 else None,
            "what": f"lbm_init from pinned host phi/rho/u (context allocation, upload, initial equilibrium: "
                    f"init_s), {K} x lbm_step (steps_s) with lbm_stats every {args.stat_every} steps and at step "
                    f"{K} (stats_s), the final fields copied back (download_s); wall clock {dt:.3f} s"}


def run_reference(args, rank, world):
    """The reference's own kernels on the host CPU (all threads), on the
    workload's box, or on a slab of it when W + K steps of the full box would
    not fit in about a minute.  Nothing of this library is loaded: the
    reference reads the same properties.in / discrete.in and derives its own
    constants (its paramRead, src/paramread.c:141-170); its phi comes from the
    oracle's restatement of its bubble initialisation (src/init.c:39-59),
    because the workload has more bubbles than its MAX_BUBBLES."""
    from lbm_bench_gpu_gb300 import inputs
    from oracle.oracle import Oracle, RefCPU, ref_lib
    if rank != 0:
        return None
    if ref_lib() is None:
        return {"impl": "reference", "unavailable": "reference sources not staged (oracle/_ref/src missing)"}
    inp = workload(args.size, args.bubbles)
    K, W = args.steps, args.warmup
    o = Oracle(inp.nx, inp.ny, inp.nz, rhoL=inp.rhoL, rhoH=inp.rhoH, tauRho=inp.tauRho, tauPhi=inp.tauPhi,
               width=inp.width, sigma=inp.sigma, Gamma=inp.Gamma, Eo=inp.Eo, rc0=inp.rc0)
    phi_full = o.bubble_phi(inp.bubbles).astype(np.float32)   # (nz+2, ny, nx), reference planes
    o.close()

    def make_ref(nxs, nys, nzs):
        d = tempfile.mkdtemp(prefix="refbench_")
        sub = inputs.Inputs(nx=nxs, ny=nys, nz=nzs, rhoL=inp.rhoL, rhoH=inp.rhoH, tauRho=inp.tauRho,
                            tauPhi=inp.tauPhi, width=inp.width, sigma=inp.sigma, Gamma=inp.Gamma, Eo=inp.Eo,
                            bubbles=inp.bubbles[:1])
        inputs.write_inputs(d, sub)
        z0 = inp.nz // 2 - nzs // 2
        slab = np.ascontiguousarray(phi_full[z0:z0 + nzs + 2, :nys, :nxs])
        return RefCPU(d, phi_override=slab)

    # calibrate: seconds per node-step on a 16-plane slab of the full x-y plane
    ref = make_ref(inp.nx, inp.ny, 16)
    grav = float(ref.constants()["grav"])   # the reference's own derivation from the written inputs
    ref.step(1, grav)
    t0 = time.perf_counter()
    ref.step(2, grav)
    t_node = (time.perf_counter() - t0) / 2 / (inp.nx * inp.ny * 16)
    budget = 60.0
    nodes_per_step = budget / max(1, K + W) / max(t_node, 1e-12)
    nxs, nys = inp.nx, inp.ny
    nzs = int(nodes_per_step // (nxs * nys))
    while nzs < 3 and nys > 32:          # shrink the plane (multiples of 32) before going below 3 planes
        nys = max(32, nys // 2)
        nzs = int(nodes_per_step // (nxs * nys))
    while nzs < 3 and nxs > 32:
        nxs = max(32, nxs // 2)
        nzs = int(nodes_per_step // (nxs * nys))
    nzs = int(max(3, min(inp.nz, nzs)))
    ref = make_ref(nxs, nys, nzs)
    ref.step(W, grav)
    t0 = time.perf_counter()
    ref.step(K, grav)
    dt = time.perf_counter() - t0
    nodes = nxs * nys * nzs
    value = nodes * K / dt / 1e6
    full = (nxs, nys, nzs) == (inp.nx, inp.ny, inp.nz)
    sample = (f"reference kernels (src/*.cu compiled for the host CPU), "
              + (f"the full {inp.nx}^3 box" if full else f"{nxs}x{nys}x{nzs} slab of the {inp.nx}^3 workload")
              + f", {K} steps after {W} warm-up, {dt:.1f} s")
    config = workload_config(args, inp, world)
    if not full:
        config.update({"workload": config["workload"] + f" (slab {nxs}x{nys}x{nzs})", "nx": nxs, "ny": nys,
                       "nz": nzs})
    return {"metric": METRIC, "value": round(value, 2), "unit": "MLUPS", "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": round(dt / K * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": config,
            "cpu_baseline": {"value": round(value, 2), "unit": "MLUPS", "cores": RefCPU.threads(),
                             "kind": "reference", "sample": sample},
            "e2e": {"value": round(value, 2), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main(argv=None):
    args = parse_args(argv)
    rank, world, local = dist_env()
    if args.impl == "reference":
        res = run_reference(args, rank, world)
        if res is not None:
            print(json.dumps(res))
        return 0
    if world > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    res = run_ours(args, rank, world, local)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
