// lbm_api.cu -- the C-ABI of liblbm_gb300 (include/lbm_gb300.h).
#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "lbm_internal.h"

namespace {

constexpr double kW[lbm::kQg] = {1.0 / 3,  1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18,
                                 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                                 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};   // src/constants.h:52-54

using lbm::cuda_fail;
using lbm::fail;

#define LBM_CUDA(call, what)                               \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

int validate(const lbm_params *p)
{
    if (!p) return fail(LBM_EINVAL, "params is NULL");
    if (p->nx < 32 || p->ny < 8 || p->nz < 3)
        return fail(LBM_EINVAL, "box too small (need nx >= 32, ny >= 8, nz >= 3)");
    if (p->nx % 32 != 0) return fail(LBM_EINVAL, "nx must be a multiple of 32");
    if (p->ny % 8 != 0) return fail(LBM_EINVAL, "ny must be a multiple of 8");
    if (p->compat) {
        // src/main.cu:167-173
        if (p->ny % 32 != 0) return fail(LBM_EINVAL, "NY is not a multiple of 32");
        if (p->block_x * p->block_y > 512) return fail(LBM_EINVAL, "Too many blocks");
        if (p->nx < p->block_x) return fail(LBM_EINVAL, "BLOCK_SIZE_X is too large");
        if (p->ny < p->block_y) return fail(LBM_EINVAL, "BLOCK_SIZE_Y is too large");
    }
    const double n = (double)p->nx * p->ny * p->nz;
    if (n * lbm::kQg >= 4294967296.0) return fail(LBM_EINVAL, "box too large for 32-bit element indexing");
    if (const char *why = lbm::physics_error(*p)) return fail(LBM_EINVAL, why);
    if (p->storage != LBM_STORAGE_FP32 && p->storage != LBM_STORAGE_FP16 && p->storage != LBM_STORAGE_BF16)
        return fail(LBM_EINVAL, "unknown storage format");
    return LBM_OK;
}

void identity_quant(lbm::Quant &q)
{
    q.f_scale = q.f_inv = q.g_scale = q.g_inv = 1.f;
    for (int i = 0; i < lbm::kQg; i++) q.g_shift[i] = 0.f;
}

// Allocate a context and its buffers; the state is left uninitialised.
int create(lbm_ctx **out, const lbm_params *p) { return lbm::create_context(out, p, 0); }

lbm::StepView view(lbm_ctx *c, int in) { return lbm::state_view(c, in); }

}  // namespace

namespace lbm {
// Allocate a context and its buffers; the state is left uninitialised.  With
// zghost the context is a z-slab: its f fields carry two ghost planes below
// and above, its g fields one (p->nz >= 2 interior planes).
int create_context(lbm_ctx **out, const lbm_params *p, int zghost)
{
    if (!out) return fail(LBM_EINVAL, "out is NULL");
    *out = nullptr;
    if (zghost) {
        if (!p || p->nz < 2) return fail(LBM_EINVAL, "a z-slab needs at least 2 planes");
        lbm_params q = *p;
        q.nz = 3;   // the checks of a whole box, apart from its depth
        if (int rc = validate(&q)) return rc;
    } else if (int rc = validate(p)) {
        return rc;
    }
    lbm_ctx *c = new (std::nothrow) lbm_ctx();
    if (!c) return fail(LBM_ENOMEM, "host allocation");
    c->p = *p;
    lbm::derive(c->p, c->d);
    if (c->p.Eo == 0.f) {
        c->d.gravity = 0.f;
        c->d.grav = 0.f;
    }
    identity_quant(c->q);
    c->esz = lbm::storage_bytes(p->storage);
    c->box.nx = p->nx;
    c->box.ny = p->ny;
    c->box.nz = p->nz;
    c->box.nxy = (long long)p->nx * p->ny;
    c->box.n = c->box.nxy * p->nz;
    c->box.zghost = zghost ? 1 : 0;
    c->box.nf = c->box.nxy * (p->nz + (zghost ? 4 : 0));
    c->box.ng = c->box.nxy * (p->nz + (zghost ? 2 : 0));
    const size_t n = (size_t)c->box.n, nf = (size_t)c->box.nf, ng = (size_t)c->box.ng;
    c->partial_count = lbm::stats_partial_count(c->box);
    // the device buffers, 256-byte aligned pieces of one allocation (the TMA
    // tensor maps need 16-byte aligned field bases)
    const size_t sizes[7] = {sizeof(float) * 2 * nf, c->esz * 2 * (lbm::kQf - 1) * nf, c->esz * lbm::kQg * ng,
                             sizeof(float) * 5 * n, sizeof(double) * lbm::kStatsValues * c->partial_count,
                             sizeof(double) * lbm::kStatsValues, sizeof(int)};
    size_t offs[7], total = 0;
    for (int k = 0; k < 7; k++) {
        offs[k] = total;
        total += (sizes[k] + 255) & ~(size_t)255;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->arena, total);
    if (e == cudaSuccess) {
        unsigned char *a = static_cast<unsigned char *>(c->arena);
        c->st.f0 = reinterpret_cast<float *>(a + offs[0]);
        c->st.fq = a + offs[1];
        c->st.g = a + offs[2];
        c->st.mom = reinterpret_cast<float *>(a + offs[3]);
        c->partials = reinterpret_cast<double *>(a + offs[4]);
        c->result = reinterpret_cast<double *>(a + offs[5]);
        c->err = reinterpret_cast<int *>(a + offs[6]);
    }
    if (e == cudaSuccess) e = cudaMallocHost(&c->result_host, sizeof(double) * lbm::kStatsValues);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->err, 0, sizeof(int), c->stream);
    if (e != cudaSuccess) {
        lbm_destroy(c);
        return cuda_fail(e, "context allocation");
    }
    *out = c;
    return LBM_OK;
}
}  // namespace lbm

namespace {

// Stats reduction of the mom arrays into c->result_host (synchronises).
int reduce_stats(lbm_ctx *c)
{
    cudaError_t e = lbm::launch_stats(c->box, c->d, c->st.mom, c->partials, c->partial_count, c->result, nullptr,
                                      c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "stats kernel launch");
    LBM_CUDA(cudaMemcpyAsync(c->result_host, c->result, sizeof(double) * lbm::kStatsValues, cudaMemcpyDeviceToHost,
                             c->stream),
             "stats copy");
    LBM_CUDA(cudaStreamSynchronize(c->stream), "stats");
    return LBM_OK;
}

// Load streamed FP32 distributions tf (7 x n) and tg (19 x n) into the state
// (half 0, natural g layout), choosing the 16-bit storage map from the data.
// c->st.mom must already hold the fields (for the mean density).  maxabs_in
// (26 floats: |f_k| and |g_i - shift_i| maxima) replaces the maxima of this
// context's data (a z-slab takes the maxima of the whole box, reduced over
// its slabs); maxabs_out receives this context's maxima (zeros for FP32).
int load_state(lbm_ctx *c, const float *tf, const float *tg, const float *maxabs_in = nullptr,
               float *maxabs_out = nullptr)
{
    if (maxabs_out)
        for (int k = 0; k < lbm::kQf + lbm::kQg; k++) maxabs_out[k] = 0.f;
    identity_quant(c->q);
    if (c->p.storage != LBM_STORAGE_FP32) {
        int rc = reduce_stats(c);
        if (rc) return rc;
        const double rho_mean = c->result_host[8] / (double)c->box.n;
        float shift[lbm::kQg];
        for (int i = 0; i < lbm::kQg; i++) shift[i] = (float)(kW[i] * rho_mean);
        float *shift_dev = nullptr;
        unsigned *bits_dev = nullptr;
        unsigned bits[lbm::kQf + lbm::kQg];
        cudaError_t e = cudaMalloc(&shift_dev, sizeof(shift));
        if (e == cudaSuccess) e = cudaMalloc(&bits_dev, sizeof(bits));
        if (e == cudaSuccess) e = cudaMemcpyAsync(shift_dev, shift, sizeof(shift), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = lbm::launch_field_maxabs(c->box, tf, tg, shift_dev, bits_dev, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(bits, bits_dev, sizeof(bits), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cudaFree(shift_dev);
        cudaFree(bits_dev);
        if (e != cudaSuccess) return cuda_fail(e, "storage map");
        for (int k = 0; k < lbm::kQf + lbm::kQg; k++) {
            if (maxabs_out) std::memcpy(&maxabs_out[k], &bits[k], sizeof(float));
            if (maxabs_in) std::memcpy(&bits[k], &maxabs_in[k], sizeof(float));
        }
        // Scales: powers of two that put a generous bound on each field at
        // 2^12, leaving 16x headroom below the FP16 maximum (65504).  The bound
        // covers the flow developing later: |u| up to 0.1 moves g_i by about
        // 3 w_i rho |u| and f_i by about phiStar |u| / (tauPhi (1 - eta)).
        // BF16 has the FP32 exponent range and keeps scale 1.
        // One scale per set, the smallest of its fields' (scaling by a power
        // of two changes no rounding of normal FP16 numbers).
        const bool fp16 = c->p.storage == LBM_STORAGE_FP16;
        auto pick = [&](float maxabs, double bound) -> float {
            double m = std::max((double)maxabs, bound);
            if (!fp16 || !(m > 0.0) || !std::isfinite(m)) return 1.f;
            int ex = (int)std::floor(std::log2(4096.0 / m));
            ex = std::max(-60, std::min(60, ex));
            return std::ldexp(1.f, ex);
        };
        const double fbound = 0.1 * std::fabs((double)c->d.phiStar) * c->d.invTauPhi * c->d.invEta2;
        float fs = INFINITY, gs = INFINITY;
        for (int a = 0; a < lbm::kQf - 1; a++) {
            float m;
            std::memcpy(&m, &bits[a + 1], sizeof(float));
            fs = std::min(fs, pick(m, fbound));
        }
        for (int i = 0; i < lbm::kQg; i++) {
            float m;
            std::memcpy(&m, &bits[lbm::kQf + i], sizeof(float));
            c->q.g_shift[i] = shift[i];
            gs = std::min(gs, pick(m, 0.3 * kW[i] * std::fabs(rho_mean)));
        }
        c->q.f_scale = fs;
        c->q.f_inv = 1.f / fs;
        c->q.g_scale = gs;
        c->q.g_inv = 1.f / gs;
    }
    lbm::StepView v = view(c, 0);
    LBM_CUDA(lbm::launch_quantize(c->box, c->q, c->p.storage, tf, tg, c->st.f0, const_cast<void *>(v.fq_in),
                                  c->st.g, c->stream),
             "quantize kernel");
    LBM_CUDA(cudaStreamSynchronize(c->stream), "load state");
    c->st.f_cur = 0;
    c->st.f_streamed = true;
    c->st.g_odd_next = false;
    return LBM_OK;
}

// Equilibrium from the fields in c->st.mom into the state.  FP32 storage
// holds the streamed FP32 distributions as they are, so the equilibrium is
// written straight into half 0; the 16-bit formats go through FP32 scratch,
// from which the storage map is chosen.
int init_from_mom(lbm_ctx *c, const float *ghost_lo, const float *ghost_hi, const float *maxabs_in = nullptr,
                  float *maxabs_out = nullptr)
{
    if (maxabs_out)
        for (int k = 0; k < lbm::kQf + lbm::kQg; k++) maxabs_out[k] = 0.f;
    const size_t n = (size_t)c->box.n;
    if (c->p.storage == LBM_STORAGE_FP32) {
        identity_quant(c->q);
        const lbm::StepView v = view(c, 0);
        LBM_CUDA(lbm::launch_equilibrium(c->box, c->d, c->p.Gamma, c->st.mom, c->st.mom + n, ghost_lo, ghost_hi,
                                         c->st.f0, static_cast<float *>(const_cast<void *>(v.fq_in)),
                                         static_cast<float *>(c->st.g), c->stream),
                 "equilibrium kernel");
        LBM_CUDA(cudaStreamSynchronize(c->stream), "init");
        c->st.f_cur = 0;
        c->st.f_streamed = true;
        c->st.g_odd_next = false;
        c->st.steps = 0;
        return LBM_OK;
    }
    float *tmp = nullptr;
    LBM_CUDA(cudaMalloc(&tmp, sizeof(float) * (lbm::kQf + lbm::kQg) * n), "init scratch");
    cudaError_t e = lbm::launch_equilibrium(c->box, c->d, c->p.Gamma, c->st.mom, c->st.mom + n, ghost_lo, ghost_hi,
                                            tmp, tmp + n, tmp + lbm::kQf * n, c->stream);
    int rc = e == cudaSuccess ? load_state(c, tmp, tmp + lbm::kQf * n, maxabs_in, maxabs_out)
                              : cuda_fail(e, "equilibrium kernel");
    cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    c->st.steps = 0;
    return rc;
}

}  // namespace

namespace lbm {
// The step kernel's error flag (it stays set): bit 1 a bounded wait gave up
// (LBM_ETIMEOUT), bit 2 a shared-memory stage was misaligned, bit 4 a checked
// build found a global index outside its field (LBM_ECUDA).
int device_error(lbm_ctx *c)
{
    int flag = 0;
    // on the context's stream, after the kernels that set it
    LBM_CUDA(cudaMemcpyAsync(&flag, c->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "error flag");
    LBM_CUDA(cudaStreamSynchronize(c->stream), "error flag");
    if (flag & 4) return fail(LBM_ECUDA, "a checked build found a global index outside its field");
    if (flag & 2) return fail(LBM_ECUDA, "a step kernel's shared-memory stage was misaligned for TMA");
    if (flag) return fail(LBM_ETIMEOUT, "a step kernel timed out waiting for its staged data");
    return LBM_OK;
}

}  // namespace lbm

namespace {
using lbm::device_error;
int fill_stats(const lbm_ctx *c, const double *r, lbm_stats_out *s)
{
    return lbm::fill_stats_raw((double)c->box.n, c->p, c->st.steps, r, s);
}
}  // namespace

namespace lbm {
int fail(int code, const std::string &msg)
{
    set_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    return fail(e == cudaErrorMemoryAllocation ? LBM_ENOMEM : LBM_ECUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace lbm

extern "C" int lbm_init(lbm_ctx **out, const lbm_params *p, const float *phi0, const float *rho0, const float *ux0,
                        const float *uy0, const float *uz0, const float *phi_ghost)
{
    const lbm::Range nvtx_range("lbm_init");
    if (!phi0 || !rho0) return fail(LBM_EINVAL, "phi0 and rho0 are required");
    if (!out) return fail(LBM_EINVAL, "out is NULL");
    if (int rc0 = validate(p)) return rc0;   // before any CUDA call
    LBM_ON_DEVICE(p->device);
    lbm_ctx *c = nullptr;
    int rc = create(&c, p);
    if (rc) return rc;
    const size_t n = (size_t)c->box.n, bytes = sizeof(float) * n;
    float *mom = c->st.mom;
    float *ghost = nullptr;
    // The at-rest equilibrium reads phi and rho only (src/init_f.cu,
    // src/init_g.cu), so u goes up on a second stream while the FP32
    // equilibrium runs; the 16-bit storage map reads all five fields first.
    cudaStream_t side = nullptr;
    cudaEvent_t u_done = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&u_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMemcpyAsync(mom, phi0, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(mom + n, rho0, bytes, cudaMemcpyHostToDevice, c->stream);
    const float *u[3] = {ux0, uy0, uz0};
    for (int a = 0; a < 3 && e == cudaSuccess; a++) {
        if (u[a]) e = cudaMemcpyAsync(mom + (2 + a) * n, u[a], bytes, cudaMemcpyHostToDevice, side);
        else e = cudaMemsetAsync(mom + (2 + a) * n, 0, bytes, side);
    }
    if (e == cudaSuccess) e = cudaEventRecord(u_done, side);
    if (e == cudaSuccess && c->p.storage != LBM_STORAGE_FP32) e = cudaStreamWaitEvent(c->stream, u_done, 0);
    if (e == cudaSuccess && phi_ghost) {
        e = cudaMalloc(&ghost, sizeof(float) * 2 * c->box.nxy);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ghost, phi_ghost, sizeof(float) * 2 * c->box.nxy, cudaMemcpyHostToDevice, c->stream);
    }
    auto release_side = [&]() {
        if (side) cudaStreamSynchronize(side);
        if (u_done) cudaEventDestroy(u_done);
        if (side) cudaStreamDestroy(side);
    };
    if (e != cudaSuccess) {
        cudaStreamSynchronize(c->stream);
        release_side();
        if (ghost) cudaFree(ghost);
        lbm_destroy(c);
        return cuda_fail(e, "lbm_init");
    }
    rc = init_from_mom(c, ghost, ghost ? ghost + c->box.nxy : nullptr);
    // the context's later work follows u's upload
    const cudaError_t ew = cudaStreamWaitEvent(c->stream, u_done, 0);
    if (ew != cudaSuccess && !rc) rc = cuda_fail(ew, "lbm_init");
    release_side();
    if (ghost) cudaFree(ghost);
    if (rc) {
        lbm_destroy(c);
        return rc;
    }
    *out = c;
    return LBM_OK;
}

namespace {

// The initial state of a created context from the bubble list (src/init.c:39-59,
// src/init_f.cu, src/init_g.cu): phi from the bubbles on the box's planes and on
// the planes just below and above it (from the geometry, as the reference's
// ghost planes), rho = (rhoH + rhoL) / 2, u = 0, the at-rest equilibrium.  The
// box's plane 0 is plane z0 of the bubbles' frame (a slab of a larger box).
int init_bubbles_into(lbm_ctx *c, const float *bubbles, int nbubbles, int z0, const float *maxabs_in,
                      float *maxabs_out)
{
    const size_t n = (size_t)c->box.n, nxy = (size_t)c->box.nxy;
    float *phig = nullptr, *bub = nullptr;
    float *mom = c->st.mom;
    cudaError_t e = cudaMalloc(&phig, sizeof(float) * nxy * (c->box.nz + 2));
    if (e == cudaSuccess && nbubbles > 0) e = cudaMalloc(&bub, sizeof(float) * 4 * nbubbles);
    if (e == cudaSuccess && nbubbles > 0)
        e = cudaMemcpyAsync(bub, bubbles, sizeof(float) * 4 * nbubbles, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = lbm::launch_bubble_phi(c->box, bub, nbubbles, c->d.phiStar, c->p.width, z0, phig, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(mom, phig + nxy, sizeof(float) * n, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = lbm::launch_fill(mom + n, (long long)n, 0.5f * (c->p.rhoH + c->p.rhoL), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(mom + 2 * n, 0, sizeof(float) * 3 * n, c->stream);
    const int rc = e == cudaSuccess
                       ? init_from_mom(c, phig, phig + nxy * (c->box.nz + 1), maxabs_in, maxabs_out)
                       : cuda_fail(e, "bubble initial state");
    cudaStreamSynchronize(c->stream);
    if (phig) cudaFree(phig);
    if (bub) cudaFree(bub);
    return rc;
}

// Checks of a slab request of the whole box p, before any CUDA call.
int check_slab_request(const lbm_params *p, const float *bubbles, int nbubbles, int z0, int depth)
{
    if (nbubbles < 0 || (nbubbles > 0 && !bubbles)) return fail(LBM_EINVAL, "bad bubble list");
    if (int rc = validate(p)) return rc;
    if (depth < 2 || z0 < 0 || z0 + depth > p->nz)
        return fail(LBM_EINVAL, "slab planes outside the box (need depth >= 2 and 0 <= z0, z0 + depth <= nz)");
    return LBM_OK;
}

// A created context holding the box's planes [z0, z0 + depth) as a whole box of
// its own (no ghost planes), initialised from the bubbles.
int slab_as_box(lbm_ctx **out, const lbm_params *p, const float *bubbles, int nbubbles, int z0, int depth,
                const float *maxabs_in, float *maxabs_out)
{
    lbm_params q = *p;
    q.nz = depth;
    lbm_ctx *c = nullptr;
    if (int rc = lbm::create_context(&c, &q, 0)) return rc;
    if (int rc = init_bubbles_into(c, bubbles, nbubbles, z0, maxabs_in, maxabs_out)) {
        lbm_destroy(c);
        return rc;
    }
    *out = c;
    return LBM_OK;
}

}  // namespace

extern "C" int lbm_init_bubbles(lbm_ctx **out, const lbm_params *p, const float *bubbles, int nbubbles)
{
    const lbm::Range nvtx_range("lbm_init_bubbles");
    if (nbubbles < 0 || (nbubbles > 0 && !bubbles)) return fail(LBM_EINVAL, "bad bubble list");
    if (!out) return fail(LBM_EINVAL, "out is NULL");
    if (int rc0 = validate(p)) return rc0;   // before any CUDA call
    LBM_ON_DEVICE(p->device);
    lbm_ctx *c = nullptr;
    int rc = create(&c, p);
    if (rc) return rc;
    if ((rc = init_bubbles_into(c, bubbles, nbubbles, 0, nullptr, nullptr))) {
        lbm_destroy(c);
        return rc;
    }
    *out = c;
    return LBM_OK;
}

extern "C" int lbm_slab_maxabs(const lbm_params *p, const float *bubbles, int nbubbles, int z0, int depth,
                               float *maxabs)
{
    const lbm::Range nvtx_range("lbm_slab_maxabs");
    if (!maxabs) return fail(LBM_EINVAL, "lbm_slab_maxabs: maxabs is NULL");
    if (int rc = check_slab_request(p, bubbles, nbubbles, z0, depth)) return rc;
    LBM_ON_DEVICE(p->device);
    lbm_ctx *c = nullptr;
    if (int rc = slab_as_box(&c, p, bubbles, nbubbles, z0, depth, nullptr, maxabs)) return rc;
    lbm_destroy(c);
    return LBM_OK;
}

extern "C" int lbm_slab_init_bubbles(lbm_ctx **out, const lbm_params *p, const float *bubbles, int nbubbles, int z0,
                                     int depth, const float *maxabs)
{
    const lbm::Range nvtx_range("lbm_slab_init_bubbles");
    if (!out) return fail(LBM_EINVAL, "out is NULL");
    *out = nullptr;
    if (int rc = check_slab_request(p, bubbles, nbubbles, z0, depth)) return rc;
    if (p->storage != LBM_STORAGE_FP32 && !maxabs)
        return fail(LBM_EINVAL, "lbm_slab_init_bubbles: 16-bit storage needs the box's maxima (lbm_slab_maxabs)");
    LBM_ON_DEVICE(p->device);
    lbm_ctx *box = nullptr;
    if (int rc = slab_as_box(&box, p, bubbles, nbubbles, z0, depth, maxabs, nullptr)) return rc;
    lbm_ctx *slab = nullptr;
    const int device = p->device;
    const int rc = lbm_split_z(box, 1, &depth, &device, &slab);
    lbm_destroy(box);
    if (rc) return rc;
    slab->z0 = z0;
    slab->nz_total = p->nz;
    *out = slab;
    return LBM_OK;
}

extern "C" int lbm_step(lbm_ctx *c, int nsteps, float grav)
{
    const lbm::Range nvtx_range("lbm_step");
    if (!c) return fail(LBM_EINVAL, "context is NULL");
    if (nsteps < 0) return fail(LBM_EINVAL, "nsteps < 0");
    if (!std::isfinite(grav)) return fail(LBM_EINVAL, "grav is not finite");
    if (c->box.zghost) return fail(LBM_EINVAL, "lbm_step: a z-slab steps with lbm_slab_step / lbm_slab_step_local");
    LBM_ON_DEVICE(c->p.device);
    const lbm::StepConst k = lbm::step_const(c->d, c->p, grav);
    for (int s = 0; s < nsteps; s++) {
        const int in = c->st.f_cur;
        cudaError_t e = lbm::launch_step(c->box, k, c->q, view(c, in), c->st.f_streamed, c->st.g_odd_next,
                                         s == nsteps - 1, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
        c->st.f_cur = 1 - in;
        c->st.f_streamed = false;
        c->st.g_odd_next = !c->st.g_odd_next;
        c->st.steps++;
    }
    return LBM_OK;
}

extern "C" int lbm_stats(lbm_ctx *c, lbm_stats_out *s, float *phi, float *rho, float *ux, float *uy, float *uz)
{
    const lbm::Range nvtx_range("lbm_stats");
    if (!c) return fail(LBM_EINVAL, "context is NULL");
    if (s && c->box.zghost) return fail(LBM_EINVAL, "lbm_stats: the statistics of z-slabs come from lbm_slab_stats");
    LBM_ON_DEVICE(c->p.device);
    const size_t n = (size_t)c->box.n, bytes = sizeof(float) * n;
    if (s) {
        cudaError_t e = lbm::launch_stats(c->box, c->d, c->st.mom, c->partials, c->partial_count, c->result,
                                          nullptr, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "stats kernel launch");
        LBM_CUDA(cudaMemcpyAsync(c->result_host, c->result, sizeof(double) * lbm::kStatsValues,
                                 cudaMemcpyDeviceToHost, c->stream),
                 "stats copy");
    }
    float *dst[5] = {phi, rho, ux, uy, uz};
    for (int a = 0; a < 5; a++)
        if (dst[a])
            LBM_CUDA(cudaMemcpyAsync(dst[a], c->st.mom + a * n, bytes, cudaMemcpyDeviceToHost, c->stream),
                     "field copy");
    LBM_CUDA(cudaStreamSynchronize(c->stream), "lbm_stats");
    if (int rc = device_error(c)) return rc;
    if (!s) return LBM_OK;
    return fill_stats(c, c->result_host, s);
}

extern "C" int lbm_stats_fields(lbm_ctx *c, lbm_stats_out *s, const float *phi, const float *rho, const float *ux,
                                const float *uy, const float *uz)
{
    if (!c || !s) return fail(LBM_EINVAL, "lbm_stats_fields: NULL context or output");
    if (!phi || !rho || !ux || !uy || !uz) return fail(LBM_EINVAL, "lbm_stats_fields: every field is required");
    if (c->box.zghost) return fail(LBM_EINVAL, "lbm_stats_fields: not available on a z-slab context");
    LBM_ON_DEVICE(c->p.device);
    const size_t n = (size_t)c->box.n, bytes = sizeof(float) * n;
    float *tmp = nullptr;
    LBM_CUDA(cudaMalloc(&tmp, 5 * bytes), "lbm_stats_fields scratch");
    const float *src[5] = {phi, rho, ux, uy, uz};
    cudaError_t e = cudaSuccess;
    for (int a = 0; a < 5 && e == cudaSuccess; a++)
        e = cudaMemcpyAsync(tmp + a * n, src[a], bytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = lbm::launch_stats(c->box, c->d, tmp, c->partials, c->partial_count, c->result, nullptr, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->result_host, c->result, sizeof(double) * lbm::kStatsValues, cudaMemcpyDeviceToHost,
                            c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(e, "lbm_stats_fields");
    return fill_stats(c, c->result_host, s);
}

extern "C" int lbm_pressure(lbm_ctx *c, float *p)
{
    if (!c || !p) return fail(LBM_EINVAL, "lbm_pressure: NULL argument");
    if (c->box.zghost) return fail(LBM_EINVAL, "lbm_pressure: not available on a z-slab context");
    LBM_ON_DEVICE(c->p.device);
    const size_t n = (size_t)c->box.n;
    float *tmp = nullptr;
    LBM_CUDA(cudaMalloc(&tmp, sizeof(float) * n), "lbm_pressure scratch");
    cudaError_t e = lbm::launch_pressure(c->box, c->d, c->st.mom, tmp, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p, tmp, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    return e == cudaSuccess ? LBM_OK : cuda_fail(e, "lbm_pressure");
}

extern "C" int lbm_device_name(int device, char *name, int len, double *total_bytes)
{
    cudaDeviceProp prop;
    LBM_CUDA(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    if (name && len > 0) {
        std::strncpy(name, prop.name, (size_t)len - 1);
        name[len - 1] = '\0';
    }
    if (total_bytes) *total_bytes = (double)prop.totalGlobalMem;
    return LBM_OK;
}

namespace lbm {
// lbm_stats_out from the 16 raw stats values of a box of n nodes (the
// reference's formulas of src/stats.c:60-91 and src/logsave.c:152-167, in FP64).
int fill_stats_raw(double n, const lbm_params &p, long long steps, const double *r, lbm_stats_out *s)
{
    std::memset(s, 0, sizeof(*s));
    s->step = steps;
    s->umax = std::sqrt(r[0]);
    s->vol = r[1];
    s->ux_av = r[1] > 0 ? r[2] / r[1] : 0.0;
    s->uy_av = r[1] > 0 ? r[3] / r[1] : 0.0;
    s->uz_av = r[1] > 0 ? r[4] / r[1] : 0.0;
    s->ref = std::pow(r[1] * 0.75 / M_PI, 1.0 / 3.0);
    const double vol_out = n - r[1];
    s->p_in = r[1] > 0 ? r[5] / r[1] : 0.0;
    s->p_out = vol_out > 0 ? r[6] / vol_out : 0.0;
    s->p_dif = s->p_in - s->p_out;
    s->p_err = p.rc0 > 0.f ? 0.5 * (2.0 * p.sigma / p.rc0 - s->p_dif) * p.rc0 / p.sigma : 0.0;
    s->phi_sum = r[7];
    s->rho_sum = r[8];
    s->mom_x = r[9];
    s->mom_y = r[10];
    s->mom_z = r[11];
    s->vol_full = r[12];
    s->umax_full = std::sqrt(r[13]);
    s->nonfinite = (long long)r[14];
    if (s->nonfinite > 0) return fail(LBM_ENAN, std::to_string(s->nonfinite) + " non-finite nodes");
    return LBM_OK;
}
}  // namespace lbm

extern "C" int lbm_get_dist(lbm_ctx *c, float *f, float *g)
{
    const lbm::Range nvtx_range("lbm_get_dist");
    if (!c) return fail(LBM_EINVAL, "context is NULL");
    if (!f && !g) return LBM_OK;
    if (c->box.zghost) return fail(LBM_EINVAL, "lbm_get_dist: not available on a z-slab context");
    LBM_ON_DEVICE(c->p.device);
    const size_t n = (size_t)c->box.n;
    float *tmp = nullptr;
    const size_t count = (f ? lbm::kQf : 0) + (g ? lbm::kQg : 0);
    LBM_CUDA(cudaMalloc(&tmp, sizeof(float) * count * n), "lbm_get_dist scratch");
    float *tf = f ? tmp : nullptr;
    float *tg = g ? tmp + (f ? lbm::kQf * n : 0) : nullptr;
    cudaError_t e = lbm::launch_stream_out(c->box, c->d.eta, c->q, view(c, c->st.f_cur), c->st.f_streamed,
                                           c->st.g_odd_next, tf, tg, c->stream);
    if (e == cudaSuccess && f)
        e = cudaMemcpyAsync(f, tf, sizeof(float) * lbm::kQf * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && g)
        e = cudaMemcpyAsync(g, tg, sizeof(float) * lbm::kQg * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(e, "lbm_get_dist");
    return LBM_OK;
}

extern "C" int lbm_set_dist(lbm_ctx *c, const float *f, const float *g)
{
    const lbm::Range nvtx_range("lbm_set_dist");
    if (!c || !f || !g) return fail(LBM_EINVAL, "NULL argument");
    if (c->box.zghost) return fail(LBM_EINVAL, "lbm_set_dist: not available on a z-slab context");
    LBM_ON_DEVICE(c->p.device);
    const size_t n = (size_t)c->box.n;
    LBM_CUDA(cudaStreamSynchronize(c->stream), "lbm_set_dist");
    float *tmp = nullptr;
    LBM_CUDA(cudaMalloc(&tmp, sizeof(float) * (lbm::kQf + lbm::kQg) * n), "lbm_set_dist scratch");
    float *tf = tmp, *tg = tmp + lbm::kQf * n;
    cudaError_t e = cudaMemcpyAsync(tf, f, sizeof(float) * lbm::kQf * n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tg, g, sizeof(float) * lbm::kQg * n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = lbm::launch_moments(c->box, tf, tg, c->st.mom, c->stream);
    const int rc = e == cudaSuccess ? load_state(c, tf, tg) : cuda_fail(e, "lbm_set_dist");
    cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    return rc;
}

// ---- state snapshots (checkpoint / resume) ----
// Layout of a snapshot (host memory, this machine's byte order): the header,
// then f_0 (n floats) and f_1..f_6 (6 n storage elements) of the current half,
// g (19 n, AA layout as stored), the five moment fields (5 n floats).
namespace {
struct SnapshotHeader {
    char magic[8];            // "LBMSTATE"
    int version;              // 1
    int nx, ny, nz, storage;
    int f_streamed, g_odd_next;
    long long steps;
    lbm::Quant q;             // the 16-bit storage map
};
constexpr char kSnapMagic[8] = {'L', 'B', 'M', 'S', 'T', 'A', 'T', 'E'};

size_t snapshot_payload(const lbm_ctx *c)
{
    const size_t n = (size_t)c->box.n;
    return sizeof(float) * n + c->esz * (lbm::kQf - 1 + lbm::kQg) * n + sizeof(float) * 5 * n;
}
}  // namespace

extern "C" long long lbm_state_bytes(const lbm_ctx *c)
{
    return c ? (long long)(sizeof(SnapshotHeader) + snapshot_payload(c)) : -1;
}

extern "C" int lbm_save_state(lbm_ctx *c, void *buf)
{
    const lbm::Range nvtx_range("lbm_save_state");
    if (!c || !buf) return fail(LBM_EINVAL, "lbm_save_state: NULL argument");
    if (c->box.zghost) return fail(LBM_EINVAL, "lbm_save_state: not available on a z-slab context");
    LBM_ON_DEVICE(c->p.device);
    SnapshotHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kSnapMagic, sizeof(h.magic));
    h.version = 1;
    h.nx = c->box.nx;
    h.ny = c->box.ny;
    h.nz = c->box.nz;
    h.storage = c->p.storage;
    h.f_streamed = c->st.f_streamed ? 1 : 0;
    h.g_odd_next = c->st.g_odd_next ? 1 : 0;
    h.steps = c->st.steps;
    h.q = c->q;
    unsigned char *d = static_cast<unsigned char *>(buf);
    std::memcpy(d, &h, sizeof(h));
    d += sizeof(h);
    const size_t n = (size_t)c->box.n, b0 = sizeof(float) * n, bq = c->esz * (lbm::kQf - 1) * n,
                 bg = c->esz * lbm::kQg * n, bm = sizeof(float) * 5 * n;
    const lbm::StepView v = view(c, c->st.f_cur);
    LBM_CUDA(cudaMemcpyAsync(d, v.f0_in, b0, cudaMemcpyDeviceToHost, c->stream), "lbm_save_state");
    LBM_CUDA(cudaMemcpyAsync(d + b0, v.fq_in, bq, cudaMemcpyDeviceToHost, c->stream), "lbm_save_state");
    LBM_CUDA(cudaMemcpyAsync(d + b0 + bq, c->st.g, bg, cudaMemcpyDeviceToHost, c->stream), "lbm_save_state");
    LBM_CUDA(cudaMemcpyAsync(d + b0 + bq + bg, c->st.mom, bm, cudaMemcpyDeviceToHost, c->stream), "lbm_save_state");
    LBM_CUDA(cudaStreamSynchronize(c->stream), "lbm_save_state");
    return device_error(c);
}

extern "C" int lbm_load_state(lbm_ctx *c, const void *buf)
{
    const lbm::Range nvtx_range("lbm_load_state");
    if (!c || !buf) return fail(LBM_EINVAL, "lbm_load_state: NULL argument");
    if (c->box.zghost) return fail(LBM_EINVAL, "lbm_load_state: not available on a z-slab context");
    SnapshotHeader h;
    std::memcpy(&h, buf, sizeof(h));
    if (std::memcmp(h.magic, kSnapMagic, sizeof(h.magic)) != 0 || h.version != 1)
        return fail(LBM_EINVAL, "lbm_load_state: not a state snapshot of this format");
    if (h.nx != c->box.nx || h.ny != c->box.ny || h.nz != c->box.nz || h.storage != c->p.storage)
        return fail(LBM_EINVAL, "lbm_load_state: the snapshot's box or storage format differs from the context's");
    if (h.steps < 0) return fail(LBM_EINVAL, "lbm_load_state: bad step count");
    LBM_ON_DEVICE(c->p.device);
    const unsigned char *d = static_cast<const unsigned char *>(buf) + sizeof(h);
    const size_t n = (size_t)c->box.n, b0 = sizeof(float) * n, bq = c->esz * (lbm::kQf - 1) * n,
                 bg = c->esz * lbm::kQg * n, bm = sizeof(float) * 5 * n;
    if (int rc = lbm_sync(c)) return rc;
    const lbm::StepView v = view(c, 0);
    LBM_CUDA(cudaMemcpyAsync(c->st.f0, d, b0, cudaMemcpyHostToDevice, c->stream), "lbm_load_state");
    LBM_CUDA(cudaMemcpyAsync(const_cast<void *>(v.fq_in), d + b0, bq, cudaMemcpyHostToDevice, c->stream),
             "lbm_load_state");
    LBM_CUDA(cudaMemcpyAsync(c->st.g, d + b0 + bq, bg, cudaMemcpyHostToDevice, c->stream), "lbm_load_state");
    LBM_CUDA(cudaMemcpyAsync(c->st.mom, d + b0 + bq + bg, bm, cudaMemcpyHostToDevice, c->stream), "lbm_load_state");
    LBM_CUDA(cudaStreamSynchronize(c->stream), "lbm_load_state");
    c->st.f_cur = 0;
    c->st.f_streamed = h.f_streamed != 0;
    c->st.g_odd_next = h.g_odd_next != 0;
    c->st.steps = h.steps;
    c->q = h.q;
    return LBM_OK;
}

extern "C" long long lbm_steps_done(const lbm_ctx *c) { return c ? c->st.steps : -1; }

extern "C" void *lbm_stream(const lbm_ctx *c) { return c ? (void *)c->stream : nullptr; }

extern "C" int lbm_sync(lbm_ctx *c)
{
    if (!c) return fail(LBM_EINVAL, "context is NULL");
    LBM_ON_DEVICE(c->p.device);
    LBM_CUDA(cudaStreamSynchronize(c->stream), "lbm_sync");
    return device_error(c);
}

extern "C" int lbm_wait_selftest(lbm_ctx *c)
{
    if (!c) return fail(LBM_EINVAL, "context is NULL");
    LBM_ON_DEVICE(c->p.device);
    if (int rc = lbm_sync(c)) return rc;
    LBM_CUDA(lbm::launch_wait_selftest(c->err, c->stream), "wait self-test launch");
    LBM_CUDA(cudaStreamSynchronize(c->stream), "wait self-test");
    const int rc = device_error(c);
    LBM_CUDA(cudaMemsetAsync(c->err, 0, sizeof(int), c->stream), "clear error flag");
    LBM_CUDA(cudaStreamSynchronize(c->stream), "clear error flag");
    if (rc == LBM_OK) return fail(LBM_ESTATE, "lbm_wait_selftest: the bounded wait did not give up");
    return rc;
}

extern "C" void lbm_destroy(lbm_ctx *c)
{
    if (!c) return;
    const lbm::DeviceGuard device_guard(c->p.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->arena);   // st.f0, st.fq, st.g, st.mom, partials, result, err
    cudaFree(c->adj_work);
    cudaFree(c->adj_slots);
    if (c->adj_host) cudaFreeHost(c->adj_host);
    cudaFree(c->halo_send);
    cudaFree(c->phi_ghost);
    if (c->ev_pack) cudaEventDestroy(c->ev_pack);
    if (c->ev_unpack) cudaEventDestroy(c->ev_unpack);
    if (c->result_host) cudaFreeHost(c->result_host);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}
