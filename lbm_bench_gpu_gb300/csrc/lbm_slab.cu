// lbm_slab.cu -- the box split in z over several contexts (one per GPU): the
// GB300 counterpart of the reference's MPI domain split (src/vgrid.c:38-52)
// and of its halo exchanges (src/pack_mpi*.cu, src/unpack_mpi*.cu,
// src/mpiupdate*.c, called from src/main.cu:496-608).
//
// A slab context's f fields (f_0, f_1..f_6, both halves) hold nz + 4 planes
// (memory plane p + 2 is interior plane p), its g fields nz + 2 (interior
// plane p at p + 1), its moment fields the nz interior planes.  The step
// kernel reads the ghost planes in place of the periodic wrap (Box::zghost).
// What the fused step needs from the neighbours:
//  * before every step, planes -2, -1 and nz, nz + 1 of the seven f fields in
//    the half the step reads (phi at the slab's first and last planes needs
//    their neighbours' phi, which is rebuilt from the f planes around it);
//  * before an odd step, ghost plane -1 of the g fields the odd step reads
//    there (the reversed slots of the directions with c_z = +1, i.e. the
//    c_z = -1 fields) and plane nz of the c_z = +1 fields;
//  * after an odd step, what it wrote into those ghost planes (c_z = -1
//    fields below, c_z = +1 fields above) into the neighbours' boundary
//    planes, where those values belong.
// Even steps read and write g at their own nodes only.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_internal.h"

namespace {

using lbm::cuda_fail;
using lbm::fail;

#define LBM_CUDA(call, what)                               \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

constexpr int kUp[5] = {5, 11, 14, 15, 18};     // g directions with c_z = +1
constexpr int kDown[5] = {6, 12, 13, 16, 17};   // g directions with c_z = -1

// One contiguous run of planes of one field: its first memory plane, the
// number of planes and the element size.
struct Run {
    unsigned char *field;
    long long plane;
    int planes;
    size_t elem;
};

unsigned char *f_field(lbm_ctx *c, int half, int k)   // k = 0: f_0, 1..6: f_k
{
    const size_t nf = (size_t)c->box.nf;
    if (k == 0) return reinterpret_cast<unsigned char *>(c->st.f0 + (size_t)half * nf);
    return static_cast<unsigned char *>(c->st.fq) + ((size_t)half * (lbm::kQf - 1) + (k - 1)) * nf * c->esz;
}
unsigned char *g_field(lbm_ctx *c, int i)
{
    return static_cast<unsigned char *>(c->st.g) + (size_t)i * (size_t)c->box.ng * c->esz;
}

// The runs of one side (0: lo, 1: hi) of a phase, in buffer order, for
// packing (from the slab's planes) or unpacking (into them).
std::vector<Run> runs(lbm_ctx *c, int phase, int side, bool pack)
{
    std::vector<Run> r;
    const int nz = c->box.nz;
    if (phase == LBM_HALO_PRE) {
        // f: pack the two boundary planes, unpack into the two ghost planes
        const long long plane = pack ? (side ? nz : 2) : (side ? nz + 2 : 0);
        for (int k = 0; k < lbm::kQf; k++)
            r.push_back({f_field(c, c->st.f_cur, k), plane, 2, k == 0 ? sizeof(float) : c->esz});
        if (c->st.g_odd_next) {
            // lo: pack plane 0 (memory 1) of the c_z = +1 fields, unpack ghost
            // plane -1 (memory 0) of the c_z = -1 fields; hi: pack plane nz - 1
            // of the c_z = -1 fields, unpack ghost plane nz of the c_z = +1 ones
            const int *set = (side == 0) == pack ? kUp : kDown;
            const long long gp = pack ? (side ? nz : 1) : (side ? nz + 1 : 0);
            for (int j = 0; j < 5; j++) r.push_back({g_field(c, set[j]), gp, 1, c->esz});
        }
    } else if (phase == LBM_HALO_POST) {
        if (c->post_pending) {
            // lo: pack ghost plane -1 of the c_z = -1 fields, unpack into plane
            // 0 the c_z = +1 fields; hi: pack ghost plane nz of the c_z = +1
            // fields, unpack into plane nz - 1 the c_z = -1 fields
            const int *set = (side == 0) == pack ? kDown : kUp;
            const long long gp = pack ? (side ? nz + 1 : 0) : (side ? nz : 1);
            for (int j = 0; j < 5; j++) r.push_back({g_field(c, set[j]), gp, 1, c->esz});
        }
    } else if (phase == LBM_HALO_PHI) {
        if (pack) r.push_back({reinterpret_cast<unsigned char *>(c->st.mom), side ? nz - 1 : 0, 1, sizeof(float)});
        else r.push_back({reinterpret_cast<unsigned char *>(c->phi_ghost), side, 1, sizeof(float)});
    }
    return r;
}

size_t run_bytes(const lbm_ctx *c, const Run &r) { return (size_t)r.planes * (size_t)c->box.nxy * r.elem; }

// Bytes of one side of a phase at the slab's current step.
size_t phase_bytes(lbm_ctx *c, int phase)
{
    size_t b = 0;
    for (const Run &r : runs(c, phase, 0, true)) b += run_bytes(c, r);
    return b;
}

// The largest side buffer any phase needs (f planes plus the g planes of an
// odd step).
size_t max_side_bytes(const lbm_ctx *c)
{
    const size_t nxy = (size_t)c->box.nxy;
    return 2 * nxy * (sizeof(float) + (lbm::kQf - 1) * c->esz) + 5 * nxy * c->esz;
}

int copy_runs(lbm_ctx *c, int phase, int side, bool pack, void *buf)
{
    unsigned char *b = static_cast<unsigned char *>(buf);
    for (const Run &r : runs(c, phase, side, pack)) {
        const size_t bytes = run_bytes(c, r);
        unsigned char *plane = r.field + (size_t)r.plane * (size_t)c->box.nxy * r.elem;
        LBM_CUDA(cudaMemcpyAsync(pack ? (void *)b : (void *)plane, pack ? (const void *)plane : (const void *)b,
                                 bytes, cudaMemcpyDefault, c->stream),
                 pack ? "halo pack" : "halo unpack");
        b += bytes;
    }
    return LBM_OK;
}

int check_slab(const lbm_ctx *c, const char *what)
{
    if (!c) return fail(LBM_EINVAL, std::string(what) + ": NULL context");
    if (!c->box.zghost) return fail(LBM_EINVAL, std::string(what) + ": not a z-slab context (lbm_split_z)");
    return LBM_OK;
}

int check_phase(int phase, const char *what)
{
    if (phase != LBM_HALO_PRE && phase != LBM_HALO_POST && phase != LBM_HALO_PHI)
        return fail(LBM_EINVAL, std::string(what) + ": unknown halo phase");
    return LBM_OK;
}

// The planes of a step.  The interior planes [2, nz - 2) read nothing the
// LBM_HALO_PRE exchange brings (phi of a plane needs the f planes up to two
// away, an odd step's g the planes one away) and write nothing it moves, so
// they can step while the halo planes are in flight; the boundary planes
// [0, 2) and [nz - 2, nz) step after it.  The in-place g update touches every
// memory slot from one node only, so the parts can run as separate launches.
struct Planes {
    int lo, hi;
};
Planes interior(const lbm_ctx *c) { return c->box.nz > 4 ? Planes{2, c->box.nz - 2} : Planes{2, 2}; }
void boundary(const lbm_ctx *c, Planes out[2])
{
    const int nz = c->box.nz, lo_end = nz < 2 ? nz : 2;
    out[0] = Planes{0, lo_end};
    out[1] = Planes{nz - 2 > lo_end ? nz - 2 : lo_end, nz};
}

// Launch the step kernel of the slab's current state over planes [r.lo, r.hi).
int slab_launch(lbm_ctx *c, float grav, bool write_moments, Planes r)
{
    if (r.lo >= r.hi) return LBM_OK;
    const lbm::StepConst k = lbm::step_const(c->d, c->p, grav);
    cudaError_t e = lbm::launch_step(c->box, k, c->q, lbm::state_view(c, c->st.f_cur), c->st.f_streamed,
                                     c->st.g_odd_next, write_moments, c->stream, r.lo, r.hi);
    return e == cudaSuccess ? LBM_OK : cuda_fail(e, "slab step kernel launch");
}

// The state after a step's launches.
void slab_advance(lbm_ctx *c)
{
    const bool odd = c->st.g_odd_next;
    c->st.f_cur = 1 - c->st.f_cur;
    c->st.f_streamed = false;
    c->st.g_odd_next = !odd;
    c->st.steps++;
    c->post_pending = odd;
    c->interior_done = false;
}

// The boundary planes of a step whose interior ran, and the state update.
int slab_finish(lbm_ctx *c, float grav, bool write_moments)
{
    Planes b[2];
    boundary(c, b);
    for (const Planes &r : b)
        if (int rc = slab_launch(c, grav, write_moments, r)) return rc;
    slab_advance(c);
    return LBM_OK;
}

// Halo exchange of one phase between the slabs of one process: every slab
// packs its two sides into its own buffer (after its neighbours finished
// reading that buffer), then unpacks what its neighbours packed.  All writes
// to a slab's memory happen on its own stream.  exchange_pack and
// exchange_unpack are the two halves (a step's interior goes between them).
int exchange_pack(lbm_ctx *const *s, int n, int phase)
{
    for (int k = 0; k < n; k++) {
        lbm_ctx *c = s[k];
        LBM_ON_DEVICE(c->p.device);
        const lbm_ctx *lo = s[(k + n - 1) % n], *hi = s[(k + 1) % n];
        LBM_CUDA(cudaStreamWaitEvent(c->stream, lo->ev_unpack, 0), "halo order");
        LBM_CUDA(cudaStreamWaitEvent(c->stream, hi->ev_unpack, 0), "halo order");
        unsigned char *buf = static_cast<unsigned char *>(c->halo_send);
        if (int rc = copy_runs(c, phase, 0, true, buf)) return rc;
        if (int rc = copy_runs(c, phase, 1, true, buf + c->halo_bytes)) return rc;
        LBM_CUDA(cudaEventRecord(c->ev_pack, c->stream), "halo order");
    }
    return LBM_OK;
}

int exchange_unpack(lbm_ctx *const *s, int n, int phase)
{
    for (int k = 0; k < n; k++) {
        lbm_ctx *c = s[k];
        LBM_ON_DEVICE(c->p.device);
        const lbm_ctx *lo = s[(k + n - 1) % n], *hi = s[(k + 1) % n];
        LBM_CUDA(cudaStreamWaitEvent(c->stream, lo->ev_pack, 0), "halo order");
        LBM_CUDA(cudaStreamWaitEvent(c->stream, hi->ev_pack, 0), "halo order");
        // from below: the lower slab's "hi" side; from above: the upper slab's "lo" side
        const unsigned char *from_lo = static_cast<const unsigned char *>(lo->halo_send) + lo->halo_bytes;
        const unsigned char *from_hi = static_cast<const unsigned char *>(hi->halo_send);
        if (int rc = copy_runs(c, phase, 0, false, const_cast<unsigned char *>(from_lo))) return rc;
        if (int rc = copy_runs(c, phase, 1, false, const_cast<unsigned char *>(from_hi))) return rc;
        LBM_CUDA(cudaEventRecord(c->ev_unpack, c->stream), "halo order");
    }
    if (phase == LBM_HALO_POST)
        for (int k = 0; k < n; k++) s[k]->post_pending = false;
    return LBM_OK;
}

int exchange(lbm_ctx *const *s, int n, int phase)
{
    if (int rc = exchange_pack(s, n, phase)) return rc;
    return exchange_unpack(s, n, phase);
}

int check_slabs(lbm_ctx *const *s, int n, const char *what)
{
    if (!s || n < 1) return fail(LBM_EINVAL, std::string(what) + ": no slabs");
    for (int k = 0; k < n; k++) {
        if (int rc = check_slab(s[k], what)) return rc;
        const lbm_ctx *a = s[k], *b = s[0];
        if (a->box.nx != b->box.nx || a->box.ny != b->box.ny || a->p.storage != b->p.storage ||
            a->nz_total != b->nz_total || a->st.g_odd_next != b->st.g_odd_next || a->st.steps != b->st.steps)
            return fail(LBM_EINVAL, std::string(what) + ": the slabs are not parts of one box at one step");
    }
    int z = s[0]->z0;
    for (int k = 0; k < n; k++) {
        if (s[k]->z0 != z % s[0]->nz_total) return fail(LBM_EINVAL, std::string(what) + ": slabs out of order");
        z += s[k]->box.nz;
    }
    if (z - s[0]->z0 != s[0]->nz_total) return fail(LBM_EINVAL, std::string(what) + ": the slabs do not cover the box");
    return LBM_OK;
}

}  // namespace

extern "C" int lbm_split_z(lbm_ctx *whole, int nslabs, const int *depths, const int *devices, lbm_ctx **slabs)
{
    const lbm::Range nvtx_range("lbm_split_z");
    if (!whole || !depths || !slabs || nslabs < 1) return fail(LBM_EINVAL, "lbm_split_z: bad argument");
    if (whole->box.zghost) return fail(LBM_EINVAL, "lbm_split_z: the context is already a z-slab");
    int total = 0;
    for (int k = 0; k < nslabs; k++) {
        if (depths[k] < 2) return fail(LBM_EINVAL, "lbm_split_z: a slab needs at least 2 planes");
        total += depths[k];
    }
    if (total != whole->box.nz) return fail(LBM_EINVAL, "lbm_split_z: the depths do not sum to the box's nz");
    for (int k = 0; k < nslabs; k++) slabs[k] = nullptr;
    {
        LBM_ON_DEVICE(whole->p.device);
        LBM_CUDA(cudaStreamSynchronize(whole->stream), "lbm_split_z");
    }
    const size_t nxy = (size_t)whole->box.nxy, n = (size_t)whole->box.n;
    int z0 = 0, rc = LBM_OK;
    for (int k = 0; k < nslabs && rc == LBM_OK; k++) {
        lbm_params p = whole->p;
        p.nz = depths[k];
        if (devices) p.device = devices[k];
        LBM_ON_DEVICE(p.device);
        lbm_ctx *c = nullptr;
        if ((rc = lbm::create_context(&c, &p, 1))) break;
        slabs[k] = c;
        c->d = whole->d;
        c->q = whole->q;
        c->z0 = z0;
        c->nz_total = whole->box.nz;
        c->halo_bytes = max_side_bytes(c);
        cudaError_t e = cudaMalloc(&c->halo_send, 2 * c->halo_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&c->phi_ghost, sizeof(float) * 2 * nxy);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_pack, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_unpack, cudaEventDisableTiming);
        // the interior planes of the whole context's current state, copied on
        // the slab's stream (the context streams do not order with the legacy
        // default stream, and a device-to-device cudaMemcpy does not wait)
        const int h = whole->st.f_cur;
        const size_t d = (size_t)depths[k];
        for (int f = 0; f < lbm::kQf && e == cudaSuccess; f++) {
            const size_t es = f == 0 ? sizeof(float) : whole->esz;
            const unsigned char *src = f_field(whole, h, f) + (size_t)z0 * nxy * es;
            e = cudaMemcpyAsync(f_field(c, 0, f) + 2 * nxy * es, src, d * nxy * es, cudaMemcpyDefault, c->stream);
        }
        for (int i = 0; i < lbm::kQg && e == cudaSuccess; i++)
            e = cudaMemcpyAsync(g_field(c, i) + nxy * c->esz, g_field(whole, i) + (size_t)z0 * nxy * whole->esz,
                                d * nxy * c->esz, cudaMemcpyDefault, c->stream);
        for (int a = 0; a < 5 && e == cudaSuccess; a++)
            e = cudaMemcpyAsync(c->st.mom + (size_t)a * c->box.n, whole->st.mom + (size_t)a * n + (size_t)z0 * nxy,
                                d * nxy * sizeof(float), cudaMemcpyDefault, c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_pack, c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_unpack, c->stream);
        // the whole context may be stepped or freed once this returns
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "lbm_split_z");
        c->st.f_cur = 0;
        c->st.f_streamed = whole->st.f_streamed;
        c->st.g_odd_next = whole->st.g_odd_next;
        c->st.steps = whole->st.steps;
        z0 += depths[k];
    }
    if (rc != LBM_OK) {
        for (int k = 0; k < nslabs; k++) {
            lbm_destroy(slabs[k]);
            slabs[k] = nullptr;
        }
    }
    return rc;
}

extern "C" int lbm_merge_z(lbm_ctx *const *slabs, int nslabs, lbm_ctx *whole)
{
    const lbm::Range nvtx_range("lbm_merge_z");
    if (int rc = check_slabs(slabs, nslabs, "lbm_merge_z")) return rc;
    if (!whole || whole->box.zghost) return fail(LBM_EINVAL, "lbm_merge_z: the target is not a whole-box context");
    const lbm_ctx *s0 = slabs[0];
    if (whole->box.nx != s0->box.nx || whole->box.ny != s0->box.ny || whole->box.nz != s0->nz_total ||
        whole->p.storage != s0->p.storage)
        return fail(LBM_EINVAL, "lbm_merge_z: the whole context's box or storage differs from the slabs'");
    for (int k = 0; k < nslabs; k++) {
        if (slabs[k]->post_pending)
            return fail(LBM_ESTATE, "lbm_merge_z: a slab still owes its neighbours the LBM_HALO_POST exchange");
        LBM_ON_DEVICE(slabs[k]->p.device);
        LBM_CUDA(cudaStreamSynchronize(slabs[k]->stream), "lbm_merge_z");
        if (int rc = lbm::device_error(slabs[k])) return rc;
    }
    LBM_ON_DEVICE(whole->p.device);
    LBM_CUDA(cudaStreamSynchronize(whole->stream), "lbm_merge_z");
    const size_t nxy = (size_t)whole->box.nxy, n = (size_t)whole->box.n;
    for (int k = 0; k < nslabs; k++) {
        lbm_ctx *c = slabs[k];
        const size_t d = (size_t)c->box.nz, z0 = (size_t)c->z0;
        const int h = c->st.f_cur;
        // on the whole context's stream, which its next work follows
        for (int f = 0; f < lbm::kQf; f++) {
            const size_t es = f == 0 ? sizeof(float) : c->esz;
            LBM_CUDA(cudaMemcpyAsync(f_field(whole, 0, f) + z0 * nxy * es, f_field(c, h, f) + 2 * nxy * es,
                                     d * nxy * es, cudaMemcpyDefault, whole->stream),
                     "lbm_merge_z");
        }
        for (int i = 0; i < lbm::kQg; i++)
            LBM_CUDA(cudaMemcpyAsync(g_field(whole, i) + z0 * nxy * c->esz, g_field(c, i) + nxy * c->esz,
                                     d * nxy * c->esz, cudaMemcpyDefault, whole->stream),
                     "lbm_merge_z");
        for (int a = 0; a < 5; a++)
            LBM_CUDA(cudaMemcpyAsync(whole->st.mom + (size_t)a * n + z0 * nxy, c->st.mom + (size_t)a * c->box.n,
                                     d * nxy * sizeof(float), cudaMemcpyDefault, whole->stream),
                     "lbm_merge_z");
    }
    // the slabs may step on (and overwrite what was read) once this returns
    LBM_CUDA(cudaStreamSynchronize(whole->stream), "lbm_merge_z");
    whole->q = s0->q;
    whole->st.f_cur = 0;
    whole->st.f_streamed = s0->st.f_streamed;
    whole->st.g_odd_next = s0->st.g_odd_next;
    whole->st.steps = s0->st.steps;
    return LBM_OK;
}

extern "C" long long lbm_halo_bytes(const lbm_ctx *slab, int phase)
{
    if (check_slab(slab, "lbm_halo_bytes") || check_phase(phase, "lbm_halo_bytes")) return -1;
    return (long long)phase_bytes(const_cast<lbm_ctx *>(slab), phase);
}

extern "C" int lbm_halo_pack(lbm_ctx *slab, int phase, void *send_lo, void *send_hi)
{
    if (int rc = check_slab(slab, "lbm_halo_pack")) return rc;
    if (int rc = check_phase(phase, "lbm_halo_pack")) return rc;
    if (phase_bytes(slab, phase) > 0 && (!send_lo || !send_hi)) return fail(LBM_EINVAL, "lbm_halo_pack: NULL buffer");
    LBM_ON_DEVICE(slab->p.device);
    if (int rc = copy_runs(slab, phase, 0, true, send_lo)) return rc;
    return copy_runs(slab, phase, 1, true, send_hi);
}

extern "C" int lbm_halo_unpack(lbm_ctx *slab, int phase, const void *recv_lo, const void *recv_hi)
{
    if (int rc = check_slab(slab, "lbm_halo_unpack")) return rc;
    if (int rc = check_phase(phase, "lbm_halo_unpack")) return rc;
    if (phase_bytes(slab, phase) > 0 && (!recv_lo || !recv_hi))
        return fail(LBM_EINVAL, "lbm_halo_unpack: NULL buffer");
    LBM_ON_DEVICE(slab->p.device);
    if (int rc = copy_runs(slab, phase, 0, false, const_cast<void *>(recv_lo))) return rc;
    if (int rc = copy_runs(slab, phase, 1, false, const_cast<void *>(recv_hi))) return rc;
    if (phase == LBM_HALO_POST) slab->post_pending = false;
    return LBM_OK;
}

extern "C" int lbm_slab_step_interior(lbm_ctx *slab, float grav)
{
    const lbm::Range nvtx_range("lbm_slab_step_interior");
    if (int rc = check_slab(slab, "lbm_slab_step_interior")) return rc;
    if (!std::isfinite(grav)) return fail(LBM_EINVAL, "grav is not finite");
    if (slab->interior_done)
        return fail(LBM_ESTATE, "lbm_slab_step_interior: the boundary part of the last step is missing");
    LBM_ON_DEVICE(slab->p.device);
    if (int rc = slab_launch(slab, grav, true, interior(slab))) return rc;
    slab->interior_done = true;
    return LBM_OK;
}

extern "C" int lbm_slab_step_boundary(lbm_ctx *slab, float grav)
{
    const lbm::Range nvtx_range("lbm_slab_step_boundary");
    if (int rc = check_slab(slab, "lbm_slab_step_boundary")) return rc;
    if (!std::isfinite(grav)) return fail(LBM_EINVAL, "grav is not finite");
    if (!slab->interior_done)
        return fail(LBM_ESTATE, "lbm_slab_step_boundary: lbm_slab_step_interior of this step is missing");
    if (slab->post_pending)
        return fail(LBM_ESTATE, "lbm_slab_step_boundary: the LBM_HALO_POST exchange of the last (odd) step is missing");
    LBM_ON_DEVICE(slab->p.device);
    return slab_finish(slab, grav, true);
}

extern "C" int lbm_slab_step_local(lbm_ctx *slab, float grav)
{
    const lbm::Range nvtx_range("lbm_slab_step_local");
    if (int rc = check_slab(slab, "lbm_slab_step_local")) return rc;
    if (!std::isfinite(grav)) return fail(LBM_EINVAL, "grav is not finite");
    if (slab->post_pending)
        return fail(LBM_ESTATE, "lbm_slab_step_local: the LBM_HALO_POST exchange of the last (odd) step is missing");
    if (slab->interior_done)
        return fail(LBM_ESTATE, "lbm_slab_step_local: the boundary part of the last step is missing");
    LBM_ON_DEVICE(slab->p.device);
    if (int rc = slab_launch(slab, grav, true, interior(slab))) return rc;
    return slab_finish(slab, grav, true);
}

extern "C" int lbm_slab_step(lbm_ctx *const *slabs, int nslabs, int nsteps, float grav)
{
    const lbm::Range nvtx_range("lbm_slab_step");
    if (int rc = check_slabs(slabs, nslabs, "lbm_slab_step")) return rc;
    if (nsteps < 0) return fail(LBM_EINVAL, "nsteps < 0");
    if (!std::isfinite(grav)) return fail(LBM_EINVAL, "grav is not finite");
    for (int k = 0; k < nslabs; k++)
        if (slabs[k]->interior_done)
            return fail(LBM_ESTATE, "lbm_slab_step: a slab is between lbm_slab_step_interior and _boundary");
    for (int k = 0; k < nslabs; k++)
        if (slabs[k]->post_pending) {
            if (int rc = exchange(slabs, nslabs, LBM_HALO_POST)) return rc;
            break;
        }
    for (int t = 0; t < nsteps; t++) {
        const bool wm = t == nsteps - 1;
        // pack the halo planes, step the interiors while the neighbours'
        // planes come in, then the boundary planes
        if (int rc = exchange_pack(slabs, nslabs, LBM_HALO_PRE)) return rc;
        for (int k = 0; k < nslabs; k++) {
            LBM_ON_DEVICE(slabs[k]->p.device);
            if (int rc = slab_launch(slabs[k], grav, wm, interior(slabs[k]))) return rc;
        }
        if (int rc = exchange_unpack(slabs, nslabs, LBM_HALO_PRE)) return rc;
        for (int k = 0; k < nslabs; k++) {
            LBM_ON_DEVICE(slabs[k]->p.device);
            if (int rc = slab_finish(slabs[k], grav, wm)) return rc;
        }
        if (slabs[0]->post_pending)
            if (int rc = exchange(slabs, nslabs, LBM_HALO_POST)) return rc;
    }
    return LBM_OK;
}

extern "C" int lbm_stats_raw(lbm_ctx *c, double *raw)
{
    if (!c || !raw) return fail(LBM_EINVAL, "lbm_stats_raw: NULL argument");
    LBM_ON_DEVICE(c->p.device);
    const float *lo = c->box.zghost ? c->phi_ghost : nullptr;
    const float *hi = c->box.zghost ? c->phi_ghost + c->box.nxy : nullptr;
    cudaError_t e = lbm::launch_stats(c->box, c->d, c->st.mom, c->partials, c->partial_count, c->result, nullptr,
                                      c->stream, lo, hi);
    if (e != cudaSuccess) return cuda_fail(e, "stats kernel launch");
    LBM_CUDA(cudaMemcpyAsync(c->result_host, c->result, sizeof(double) * lbm::kStatsValues, cudaMemcpyDeviceToHost,
                             c->stream),
             "stats copy");
    LBM_CUDA(cudaStreamSynchronize(c->stream), "lbm_stats_raw");
    if (int rc = lbm::device_error(c)) return rc;
    std::memcpy(raw, c->result_host, sizeof(double) * lbm::kStatsValues);
    return LBM_OK;
}

extern "C" int lbm_stats_combine(const lbm_params *p, long long steps, const double *raw, int nraw,
                                 lbm_stats_out *s)
{
    if (!p || !raw || !s || nraw < 1) return fail(LBM_EINVAL, "lbm_stats_combine: bad argument");
    double r[lbm::kStatsValues];
    for (int v = 0; v < lbm::kStatsValues; v++) {
        r[v] = raw[v];
        for (int k = 1; k < nraw; k++) {
            const double x = raw[(size_t)k * lbm::kStatsValues + v];
            r[v] = (v == 0 || v == 13) ? (x > r[v] ? x : r[v]) : r[v] + x;
        }
    }
    return lbm::fill_stats_raw((double)p->nx * p->ny * p->nz, *p, steps, r, s);
}

extern "C" int lbm_slab_stats(lbm_ctx *const *slabs, int nslabs, lbm_stats_out *s)
{
    const lbm::Range nvtx_range("lbm_slab_stats");
    if (int rc = check_slabs(slabs, nslabs, "lbm_slab_stats")) return rc;
    if (!s) return fail(LBM_EINVAL, "lbm_slab_stats: NULL output");
    if (int rc = exchange(slabs, nslabs, LBM_HALO_PHI)) return rc;
    std::vector<double> raw((size_t)nslabs * lbm::kStatsValues);
    for (int k = 0; k < nslabs; k++)
        if (int rc = lbm_stats_raw(slabs[k], raw.data() + (size_t)k * lbm::kStatsValues)) return rc;
    lbm_params box = slabs[0]->p;
    box.nz = slabs[0]->nz_total;
    return lbm_stats_combine(&box, slabs[0]->st.steps, raw.data(), nslabs, s);
}
