"""The box split in z over slab contexts (lbm_split_z / lbm_slab_step, the
counterpart of the reference's MPI domain split, src/vgrid.c:38-52, and of
its halo exchanges, src/main.cu:496-608), on one GPU: several slab contexts
on the same device stand in for the GPUs of a larger machine, and their
halo planes move by device copies.  Every node computes exactly what the
whole-box step computes, so after the same steps the merged slabs must equal
a whole-box context bit for bit, in every storage format, and the statistics
combined over the slabs must equal the whole box's (FP64 sums in another
order)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHYS = dict(rhoL=0.1, rhoH=1.0, tauRho=0.8, tauPhi=0.9, width=4.0, sigma=1e-3, Gamma=1.0, Eo=-0.8, rc0=9.0)
BUB = np.array([[30.3, 14.2, 21.7, 9.0], [8.5, 22.1, 40.2, 6.0], [50.0, 8.0, 3.5, 5.0]], np.float32)


def params(shape, storage):
    from lbm_bench_gpu_gb300 import capi
    return capi.make_params(*shape, storage=storage, **PHYS)


def assert_same_state(a, b, what):
    fa, ga = a.dist()
    fb, gb = b.dist()
    assert np.array_equal(fa, fb), f"{what}: f"
    assert np.array_equal(ga, gb), f"{what}: g"
    ma, mb = a.fields(), b.fields()
    for k in ma:
        assert np.array_equal(ma[k], mb[k]), f"{what}: {k}"


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("depths", [(16, 16, 16), (20, 12, 16), (24, 24), (48,)])
def test_slabs_step_like_the_whole_box(lib, storage, depths):
    from lbm_bench_gpu_gb300 import capi
    p = params((64, 32, 48), storage)
    grav = float(capi.derive(p).grav)
    with capi.Lattice.from_bubbles(p, BUB) as whole, capi.Lattice.from_bubbles(p, BUB) as ref:
        with capi.Slabs(whole, depths) as slabs:
            slabs.step(4, grav)
            slabs.step(6, grav)       # two calls: an odd number of steps in between
            ref.step(10, grav)
            s = slabs.stats()
            sr, _ = ref.stats()
            slabs.merge_into(whole)
        assert whole.steps == 10
        assert_same_state(whole, ref, f"{storage} {depths}")
    for k in ("vol", "vol_full", "umax", "umax_full", "step", "nonfinite"):
        assert s[k] == sr[k], k
    for k in ("phi_sum", "rho_sum", "mom_x", "mom_y", "mom_z", "ux_av", "uy_av", "uz_av", "p_in", "p_out"):
        assert s[k] == pytest.approx(sr[k], rel=1e-9, abs=1e-15), k


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("depths", [(20, 12, 16), (24, 24)])
def test_slabs_built_on_their_own_equal_the_split(lib, storage, depths):
    """lbm_slab_maxabs + lbm_slab_init_bubbles (each slab from the bubble list,
    the 16-bit maxima reduced over the slabs) give the slabs lbm_split_z makes
    of lbm_init_bubbles's whole box, bit for bit (the bubbles cross the slab
    boundaries and the box's bottom plane), and they step on like it."""
    from lbm_bench_gpu_gb300 import capi
    p = params((64, 32, 48), storage)
    grav = float(capi.derive(p).grav)
    with capi.Lattice.from_bubbles(p, BUB) as ref, capi.Lattice.from_bubbles(p, BUB) as target:
        target.step(3, grav)      # overwritten by the merge
        with capi.Slabs.from_bubbles(p, BUB, depths) as slabs:
            slabs.merge_into(target)
            assert target.steps == 0
            assert_same_state(target, ref, f"init {storage} {depths}")
            slabs.step(7, grav)
            ref.step(7, grav)
            slabs.merge_into(target)
        assert_same_state(target, ref, f"7 steps {storage} {depths}")


def test_slab_rejects_whole_box_calls(lib):
    from lbm_bench_gpu_gb300 import capi
    p = params((64, 32, 48), "fp32")
    with capi.Lattice.from_bubbles(p, BUB) as whole, capi.Slabs(whole, (24, 24)) as slabs:
        lib_ = capi.load()
        assert lib_.lbm_step(slabs.handle(0), 1, 0.0) == capi.LBM_EINVAL
        f = np.empty((7, 24, 32, 64), np.float32)
        assert lib_.lbm_get_dist(slabs.handle(0), capi.fptr(f), None) == capi.LBM_EINVAL
        # a second split of a slab, and depths that do not cover the box
        out = (C.c_void_p * 2)()
        assert lib_.lbm_split_z(slabs.handle(0), 2, (C.c_int * 2)(12, 12), None, out) == capi.LBM_EINVAL
        assert lib_.lbm_split_z(whole._h, 2, (C.c_int * 2)(24, 20), None, out) == capi.LBM_EINVAL
        assert lib_.lbm_split_z(whole._h, 2, (C.c_int * 2)(47, 1), None, out) == capi.LBM_EINVAL
        # the two parts of a step in order, once each
        h = slabs.handle(0)
        assert lib_.lbm_slab_step_boundary(h, 0.0) == capi.LBM_ESTATE
        assert lib_.lbm_slab_step_interior(h, 0.0) == capi.LBM_OK
        assert lib_.lbm_slab_step_interior(h, 0.0) == capi.LBM_ESTATE
        assert lib_.lbm_slab_step_local(h, 0.0) == capi.LBM_ESTATE
        assert lib_.lbm_slab_step(slabs._h, 2, 1, 0.0) == capi.LBM_ESTATE
        assert lib_.lbm_slab_step_interior(whole._h, 0.0) == capi.LBM_EINVAL


@pytest.mark.parametrize("order", ["whole step", "interior while the halo moves"])
@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_halo_pack_unpack_protocol(lib, storage, order):
    """The per-process protocol: each slab packs its halo planes into buffers
    the caller owns (here torch device tensors), the buffers go to the
    neighbours (here a device copy; across processes NCCL or MPI), each slab
    unpacks what it received and steps alone; after an odd step the
    LBM_HALO_POST exchange returns the ghost-plane writes.  Either the whole
    step after the exchange (lbm_slab_step_local), or its interior planes
    between pack and unpack and its boundary planes after
    (lbm_slab_step_interior / lbm_slab_step_boundary)."""
    import torch
    from lbm_bench_gpu_gb300 import capi
    p = params((64, 32, 48), storage)
    grav = float(capi.derive(p).grav)
    lib_ = capi.load()
    dev = torch.device("cuda", 0)
    with capi.Lattice.from_bubbles(p, BUB) as whole, capi.Lattice.from_bubbles(p, BUB) as ref:
        with capi.Slabs(whole, (20, 28)) as slabs:
            hs = [slabs.handle(k) for k in range(2)]

            def pack(phase):
                nbytes = [int(lib_.lbm_halo_bytes(h, phase)) for h in hs]
                assert nbytes[0] == nbytes[1] >= 0
                if nbytes[0] == 0:
                    return None
                send = [(torch.empty(nbytes[0], dtype=torch.uint8, device=dev),
                         torch.empty(nbytes[0], dtype=torch.uint8, device=dev)) for _ in hs]
                for h, (lo, hi) in zip(hs, send):
                    capi.check(lib_.lbm_halo_pack(h, phase, C.c_void_p(lo.data_ptr()), C.c_void_p(hi.data_ptr())),
                               "pack")
                    capi.check(lib_.lbm_sync(h), "sync")
                return send

            def unpack(phase, send):
                if send is None:
                    return
                for k, h in enumerate(hs):
                    below, above = send[(k - 1) % 2], send[(k + 1) % 2]
                    # from below its "hi" buffer, from above its "lo" buffer
                    capi.check(lib_.lbm_halo_unpack(h, phase, C.c_void_p(below[1].data_ptr()),
                                                    C.c_void_p(above[0].data_ptr())), "unpack")
                for h in hs:
                    capi.check(lib_.lbm_sync(h), "sync")

            for _ in range(5):
                if order == "whole step":
                    unpack(capi.LBM_HALO_PRE, pack(capi.LBM_HALO_PRE))
                    for h in hs:
                        capi.check(lib_.lbm_slab_step_local(h, grav), "lbm_slab_step_local")
                else:
                    send = pack(capi.LBM_HALO_PRE)
                    for h in hs:
                        capi.check(lib_.lbm_slab_step_interior(h, grav), "lbm_slab_step_interior")
                    unpack(capi.LBM_HALO_PRE, send)
                    for h in hs:
                        capi.check(lib_.lbm_slab_step_boundary(h, grav), "lbm_slab_step_boundary")
                unpack(capi.LBM_HALO_POST, pack(capi.LBM_HALO_POST))
            ref.step(5, grav)
            slabs.merge_into(whole)
        assert_same_state(whole, ref, f"protocol {storage}")


def test_bench_box_in_two_slabs(lib):
    """256^3, the bench's workload, FP32 and FP16, in two slabs of 128 planes
    (interior tiles staged by TMA, full-size chunking) for 3 steps."""
    from lbm_bench_gpu_gb300 import capi, inputs
    inp = inputs.bubbly(256, 64)
    for storage in ("fp32", "fp16"):
        p = capi.make_params(256, 256, 256, rhoL=inp.rhoL, rhoH=inp.rhoH, tauRho=inp.tauRho, tauPhi=inp.tauPhi,
                             width=inp.width, sigma=inp.sigma, Gamma=inp.Gamma, Eo=inp.Eo, rc0=inp.rc0,
                             storage=storage, compat=True)
        grav = float(capi.derive(p).grav)
        with capi.Lattice.from_bubbles(p, inp.bubbles) as whole, capi.Lattice.from_bubbles(p, inp.bubbles) as ref:
            with capi.Slabs(whole, (128, 128)) as slabs:
                slabs.step(3, grav)
                ref.step(3, grav)
                slabs.merge_into(whole)
            a, b = whole.fields(), ref.fields()
            for k in a:
                assert np.array_equal(a[k], b[k]), f"{storage} {k}"
