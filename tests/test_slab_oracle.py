"""The domain split over z-slabs on the FP64 oracle, on CPU: each slab holds
planes [z0, z0 + nz) of the periodic box and swaps planes with its two
neighbours three times per step, as the reference's ranks do
(src/vgrid.c:38-52, src/main.cu:496-608): phi after the moments, then the
post-collision f and g before streaming.  The slabs together must reproduce
the whole-box oracle exactly (the same FP64 operations on every node).

* in one process: three slabs of unequal depth, exchanges by copies;
* over two gloo ranks on 127.0.0.1 (standing in for two GPUs): one slab per
  rank, the planes sent with torch.distributed point-to-point messages.
"""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PHYS = dict(rhoL=0.1, rhoH=1.0, tauRho=0.8, tauPhi=0.9, width=4.0, sigma=1e-3, Gamma=1.0)
GRAV = -2e-5


def whole_oracle(nx, ny, nz, bubbles):
    from oracle.oracle import Oracle
    o = Oracle(nx, ny, nz, **PHYS)
    o.init_bubbles(bubbles)
    return o


def make_slabs(o, depths):
    """Slabs of the given depths covering o's box, set to o's current state."""
    from oracle.oracle import SlabOracle
    f, g = o.dist()
    slabs, z0 = [], 0
    for d in depths:
        s = SlabOracle(o.nx, o.ny, d, **PHYS)
        s.set_dist(f[:, z0:z0 + d], g[:, z0:z0 + d])
        slabs.append(s)
        z0 += d
    assert z0 == o.nz
    return slabs


def step_in_process(slabs, grav):
    k = len(slabs)
    for s in slabs:
        s.moments_update()
    planes = [(s.phi_plane(0), s.phi_plane(1)) for s in slabs]
    for i, s in enumerate(slabs):
        s.set_phi_ghost(0, planes[(i - 1) % k][1])   # the last plane of the slab below
        s.set_phi_ghost(1, planes[(i + 1) % k][0])   # the first plane of the slab above
    for s in slabs:
        s.collide(grav)
    planes = [(s.post_plane(0), s.post_plane(1)) for s in slabs]
    for i, s in enumerate(slabs):
        s.set_post_ghost(0, planes[(i - 1) % k][1])
        s.set_post_ghost(1, planes[(i + 1) % k][0])
    for s in slabs:
        s.stream()


def test_three_slabs_reproduce_the_whole_box():
    bub = np.array([[30.3, 14.2, 21.7, 9.0], [8.5, 22.1, 40.2, 6.0]], np.float32)
    o = whole_oracle(64, 32, 48, bub)
    slabs = make_slabs(o, (20, 12, 16))
    for _ in range(6):
        step_in_process(slabs, GRAV)
    o.step(6, GRAV)
    f, g = o.dist()
    m = o.moments()
    z0 = 0
    for s in slabs:
        fs, gs = s.dist()
        ms = s.moments()
        assert np.array_equal(fs, f[:, z0:z0 + s.nz]) and np.array_equal(gs, g[:, z0:z0 + s.nz])
        for k in ("phi", "rho", "ux", "uy", "uz"):
            assert np.array_equal(ms[k], m[k][z0:z0 + s.nz]), k
        z0 += s.nz


def _free_port() -> int:
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


BOX = (32, 32, 24)
BUB2 = np.array([[15.4, 16.2, 12.6, 7.0]], np.float32)
STEPS = 5


def _rank(rank: int, world: int, port: int, out) -> None:
    import torch
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        nx, ny, nz = BOX
        depth = nz // world
        # every rank derives the same initial state; it keeps its own planes
        slab = make_slabs(whole_oracle(nx, ny, nz, BUB2), [depth] * world)[rank]
        below, above = (rank - 1) % world, (rank + 1) % world

        def exchange(first, last, set_ghost):
            # my first plane goes below (tag 0), my last plane above (tag 1)
            r_lo = torch.empty(first.shape, dtype=torch.float64)
            r_hi = torch.empty(first.shape, dtype=torch.float64)
            reqs = [dist.isend(torch.from_numpy(np.ascontiguousarray(first)), below, tag=0),
                    dist.isend(torch.from_numpy(np.ascontiguousarray(last)), above, tag=1),
                    dist.irecv(r_lo, below, tag=1), dist.irecv(r_hi, above, tag=0)]
            for q in reqs:
                q.wait()
            set_ghost(0, r_lo.numpy())
            set_ghost(1, r_hi.numpy())

        for _ in range(STEPS):
            slab.moments_update()
            exchange(slab.phi_plane(0), slab.phi_plane(1), slab.set_phi_ghost)
            slab.collide(GRAV)
            exchange(slab.post_plane(0), slab.post_plane(1), slab.set_post_ghost)
            slab.stream()
        f, g = slab.dist()
        m = slab.moments()
        # gather every rank's planes on rank 0 and compare with the whole box
        parts = [torch.from_numpy(np.concatenate([f.ravel(), g.ravel()] + [m[k].ravel() for k in
                                                                          ("phi", "rho", "ux", "uy", "uz")]))]
        gathered = [torch.empty_like(parts[0]) for _ in range(world)] if rank == 0 else None
        dist.gather(parts[0], gathered, dst=0)
        if rank == 0:
            o = whole_oracle(nx, ny, nz, BUB2)
            o.step(STEPS, GRAV)
            fw, gw = o.dist()
            mw = o.moments()
            worst = 0.0
            for r, t in enumerate(gathered):
                a = t.numpy()
                zs = slice(r * depth, (r + 1) * depth)
                want = np.concatenate([fw[:, zs].ravel(), gw[:, zs].ravel()] + [mw[k][zs].ravel() for k in
                                                                                ("phi", "rho", "ux", "uy", "uz")])
                worst = max(worst, float(np.abs(a - want).max()))
            out["max_abs_diff"] = worst
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_whole_box():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        assert out["max_abs_diff"] == 0.0
