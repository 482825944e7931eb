// lbm_internal.h -- shared definitions of liblbm_gb300 (not part of the C-ABI).
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>

#include "lbm_gb300.h"
#include <nvtx3/nvToolsExt.h>   // header-only; no-ops unless a profiler is attached

namespace lbm {

// D3Q7 (f) and D3Q19 (g) lattice vectors in the reference order
// (src/stream_f.cu:52-59, src/stream_g.cu:56-76).
// f: 0 rest, 1 +x, 2 -x, 3 +y, 4 -y, 5 +z, 6 -z
// g: 0 rest, 1..6 as f, 7 (+x+y), 8 (-x-y), 9 (+x-y), 10 (-x+y), 11 (+x+z),
//    12 (-x-z), 13 (+x-z), 14 (-x+z), 15 (+y+z), 16 (-y-z), 17 (+y-z), 18 (-y+z)
constexpr int kQf = 7;
constexpr int kQg = 19;

// Scalars the step needs, all FP32 (src/constants.h:81-85 plus grav_d).
struct StepConst {
    float eta, eta2;                          // ZSC streaming interpolation
    float alpha4, kappa, phiStarSq, Gamma;    // chemical potential
    float invTauPhi, invTauPhiOne, invEta2;   // D3Q7 relaxation
    float invTauRhoOne, K0, K1, K2, KC0, KC1, KC2;  // D3Q19 relaxation + forcing
    float grav;                               // body force on phi > 0 nodes
};

// Box of interior nodes, periodic in x and y.  In z it is periodic too, or a
// z-slab of a larger box (zghost = 1): then the state's fields carry ghost
// planes the neighbouring slabs fill, two below and two above the slab for
// f_0..f_6 (nz + 4 planes, field length nf) and one below and one above for
// g (nz + 2 planes, field length ng); the moment fields hold the nz planes.
struct Box {
    int nx, ny, nz;
    long long nxy, n;
    int zghost = 0;
    long long nf = 0, ng = 0;   // elements per f / g field (n when periodic)
};

// Affine map of the 16-bit storage formats, one power-of-two scale per set:
//   stored f_k = f_k * f_scale                   (k = 1..6; f_0 stays FP32)
//   stored g_i = (g_i - g_shift[i]) * g_scale     (g_shift[i] = w_i * mean rho)
// A power of two makes the map exact, and one scale per set lets the step
// fold it into its collision constants.  For FP32 storage the map is the
// identity and is not applied.
struct Quant {
    float f_scale, f_inv;
    float g_scale, g_inv;
    float g_shift[kQg];
};

// Device buffers of one context (element type of fq and g: the storage type,
// float / __half / __nv_bfloat16):
//  f0     : 2 x n floats        D3Q7 rest population, A/B
//  fq     : 2 x 6 x n           D3Q7 f_1..f_6, A/B
//  g      : 19 x n              D3Q19 in the in-place AA layout
//  mom    : 5 x n floats        phi, rho, ux, uy, uz as the reference's arrays hold them
// f holds post-collision values, except right after init / lbm_set_dist
// (f_streamed), when it holds streamed values.  FP32 storage keeps f0, fq and
// g in the natural layout; the 16-bit formats keep them in the pair layout
// (storage_index in lattice.cuh); mom is always natural.
struct State {
    float *f0 = nullptr;
    void *fq = nullptr;
    void *g = nullptr;
    float *mom = nullptr;
    int f_cur = 0;            // which half of f0 / fq holds the current values
    bool f_streamed = true;
    bool g_odd_next = false;  // the next step reads g in the AA "odd" layout
    long long steps = 0;
};

// The state buffers one step reads and writes.
struct StepView {
    int storage;              // LBM_STORAGE_*
    const float *f0_in;
    float *f0_out;
    const void *fq_in;        // 6 arrays of n elements
    void *fq_out;
    void *g;                  // 19 arrays of n elements, written (and read when g_in is NULL)
    const void *g_in;         // g read by the step when it is not g (a checkpoint), else NULL
    float *mom;
    int *err;                 // device flag a kernel sets when a bounded wait gives up
};

size_t storage_bytes(int storage);   // bytes per element of fq / g

// A forward state as the step kernel stores it (the context's current half or
// a checkpoint slot): f_0 FP32, f_1..f_6 and g in the storage type.
struct NativeState {
    int storage;              // LBM_STORAGE_*
    const float *f0;          // n floats
    const void *fq;           // 6 x n: streamed f_1..f_6 when f_streamed, else post-collision P
    const void *g;            // 19 x n, AA layout
    bool f_streamed;
    bool g_odd;               // g in the reversed layout (the next step is odd)
};

// Buffers of one adjoint step (FP32, n elements per field).
struct AdjointBuffers {
    const float *phi;                  // phi of s^n
    const float *lf_in, *lg_in;        // lambda^{n+1} (f part without its stencil term)
    const float *lst_in;               //   stencil term of lambda^{n+1}, common to the 7 f fields
    float *lf_out, *lg_out, *lst_out;  // lambda^n
    float4 *lsrc;                      // scratch per node: (lambda_lap, mu lambda_F)
    double *dgrav;                     // per-warp running sums of the dJ/dgrav terms
    const double *ab;                  // objective sums of s^n
};

void set_error(const std::string &msg);
const std::string &last_error();

// Host-side derivation of the constants (src/paramread.c:141-170).
void derive(const lbm_params &p, lbm_derived &d);
// Why p's physical parameters cannot be derived from (nullptr: they can).
const char *physics_error(const lbm_params &p);
StepConst step_const(const lbm_derived &d, const lbm_params &p, float grav);

// Kernel launchers (defined in the .cu files); all return the cudaError_t of the launch.
// phi of planes -1 .. nz of the box from the bubble list, the box's plane 0
// being plane z0 of the bubbles' frame (0 for a whole box).
cudaError_t launch_bubble_phi(const Box &b, const float *bubbles_dev, int nbubbles, float phiStar, float width,
                              int z0, float *phi_ghosted, cudaStream_t s);
// At-rest equilibrium into FP32 arrays f_0 (n), f_1..f_6 (6 x n) and g (19 x n),
// streamed natural layout.
cudaError_t launch_equilibrium(const Box &b, const lbm_derived &d, float Gamma, const float *phi, const float *rho,
                               const float *ghost_lo, const float *ghost_hi, float *f0, float *fq, float *g,
                               cudaStream_t s);
cudaError_t launch_fill(float *p, long long n, float v, cudaStream_t s);
// One step of the state in v; a z-slab (Box::zghost) may step planes
// [zlo, zhi) of it only (zhi < 0: all), a periodic box steps whole.
cudaError_t launch_step(const Box &b, const StepConst &c, const Quant &q, const StepView &v, bool f_streamed,
                        bool odd, bool write_moments, cudaStream_t s, int zlo = 0, int zhi = -1);
// One block whose bounded mbarrier wait gives up and sets *err (the step's wait).
cudaError_t launch_wait_selftest(int *err, cudaStream_t s);
// State (post-collision / AA layout, any storage) -> streamed FP32 f (7 x n) and g (19 x n).
cudaError_t launch_stream_out(const Box &b, float eta, const Quant &q, const StepView &v, bool f_streamed, bool odd,
                              float *f_out, float *g_out, cudaStream_t s);
// Streamed FP32 f, g -> state half 0 (natural g slots, the storage's layout), applying the storage map.
cudaError_t launch_quantize(const Box &b, const Quant &q, int storage, const float *f, const float *g, float *f0,
                            void *fq, void *gq, cudaStream_t s);
// Per-field max |x - shift| of the 7 f and 19 g FP32 arrays (26 floats at out, device).
cudaError_t launch_field_maxabs(const Box &b, const float *f, const float *g, const float *g_shift_dev,
                                unsigned *out_bits, cudaStream_t s);
cudaError_t launch_moments(const Box &b, const float *f, const float *g, float *mom, cudaStream_t s);
// phi_lo / phi_hi: the phi planes below and above a z-slab (NULL: periodic z).
cudaError_t launch_stats(const Box &b, const lbm_derived &d, const float *mom, double *partials,
                         size_t partial_count, double *result, unsigned long long *counters, cudaStream_t s,
                         const float *phi_lo = nullptr, const float *phi_hi = nullptr);
size_t stats_partial_count(const Box &b);
// Pressure field (n floats) of the mom arrays (src/vtksave.c:63-127).
cudaError_t launch_pressure(const Box &b, const lbm_derived &d, const float *mom, float *out, cudaStream_t s);

// Adjoint (zsc_adjoint.cu).  acc[0] accumulates J, acc[1] dJ/dgrav (FP64).
// All adjoint kernels run on one grid of 32 x 8 column tiles, each block
// marching a few z planes; adjoint_blocks is its block count (the length of
// the dgrav array, and half the length of the objective partials).
size_t adjoint_blocks(const Box &b);
// Length of the dgrav array: one running sum per warp of the local kernel's grid.
size_t adjoint_dgrav_parts(const Box &b);
cudaError_t launch_adjoint_phi(const Box &b, float eta, const Quant &q, const NativeState &st, float *phi,
                               cudaStream_t s);
cudaError_t launch_objective(const Box &b, int objective, float phiStar, double scale, const Quant &q,
                             const NativeState &st, const float *phi, double *partials, double *ab, double *acc,
                             cudaStream_t s);
cudaError_t launch_source_init(const Box &b, int objective, double scale, const double *ab, float phiStar,
                               const Quant &q, const NativeState &st, const float *phi, float *lf, float *lg,
                               float *lst, cudaStream_t s);
cudaError_t launch_adjoint_step(const Box &b, const StepConst &c, float phiStar, const Quant &q,
                                const NativeState &st, const AdjointBuffers &a, bool add_source, int objective,
                                double scale, cudaStream_t s);
// acc[1] = sum of the per-warp dgrav sums.
cudaError_t launch_dgrav_fold(const Box &b, const double *dgrav, double *acc, cudaStream_t s);
cudaError_t launch_init_adjoint(const Box &b, const lbm_derived &d, float Gamma, const float *phi0, const float *lf,
                                const float *lst, const float *lg, float *lphi0, float *llap, cudaStream_t s);

// Number of doubles produced by launch_stats in `result`.
constexpr int kStatsValues = 16;

}  // namespace lbm

// One simulation context (the opaque lbm_ctx of the C-ABI).
struct lbm_ctx {
    lbm_params p;
    lbm_derived d;
    lbm::Box box;
    cudaStream_t stream = nullptr;
    lbm::State st;
    lbm::Quant q;
    size_t esz = 4;                // bytes per element of fq / g
    double *partials = nullptr;    // stats scratch: per-block partial sums
    size_t partial_count = 0;
    double *result = nullptr;      // stats result (device)
    double *result_host = nullptr; // pinned copy
    int *err = nullptr;            // device error flag of the kernels (0 = none)
    // one device allocation holding st.f0, st.fq, st.g, st.mom, partials,
    // result and err (one cudaMalloc per context instead of seven)
    void *arena = nullptr;
    // adjoint workspace, kept between lbm_step_adjoint / lbm_objective calls
    // (freeing tens of GB costs ~0.4 ms per GB) until lbm_adjoint_release or
    // lbm_destroy: the work buffers as one arena, and the checkpoint pool
    void *adj_work = nullptr;
    size_t adj_work_bytes = 0;
    void *adj_slots = nullptr;
    size_t adj_slot_bytes = 0;
    void *adj_host = nullptr;          // pinned host checkpoints (the second tier)
    size_t adj_host_bytes = 0;
    // z-slab contexts (lbm_split_z): planes [z0, z0 + nz) of a box of
    // nz_total planes, the device buffers the halo exchange packs into (one
    // per side, halo_bytes each), the phi planes around the slab for the
    // statistics, events that order the exchange across the slabs' streams,
    // and whether the last step was odd (its ghost-plane g writes still have
    // to reach the neighbours)
    int z0 = 0, nz_total = 0;
    bool interior_done = false;    // lbm_slab_step_interior ran, the boundary part of the step not yet
    void *halo_send = nullptr;
    size_t halo_bytes = 0;
    float *phi_ghost = nullptr;
    cudaEvent_t ev_pack = nullptr, ev_unpack = nullptr;
    bool post_pending = false;
};

namespace lbm {
// The buffers of a step that reads half `in` of f.
inline StepView state_view(lbm_ctx *c, int in)
{
    const int out = 1 - in;
    unsigned char *fq = static_cast<unsigned char *>(c->st.fq);
    StepView v;
    v.storage = c->p.storage;
    const size_t nf = (size_t)c->box.nf;
    v.f0_in = c->st.f0 + (size_t)in * nf;
    v.f0_out = c->st.f0 + (size_t)out * nf;
    v.fq_in = fq + (size_t)in * (kQf - 1) * nf * c->esz;
    v.fq_out = fq + (size_t)out * (kQf - 1) * nf * c->esz;
    v.g = c->st.g;
    v.g_in = nullptr;
    v.mom = c->st.mom;
    v.err = c->err;
    return v;
}
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
// Allocate a context (zghost: a z-slab with ghost planes, lbm_split_z).
int create_context(lbm_ctx **out, const lbm_params *p, int zghost);
// The kernels' error flag as a status (LBM_ETIMEOUT, LBM_ECUDA) after a sync.
int device_error(lbm_ctx *c);
// lbm_stats_out from the raw statistics of a box of n nodes.
int fill_stats_raw(double n, const lbm_params &p, long long steps, const double *raw, lbm_stats_out *s);

// Makes `device` current for the length of a C-ABI call and gives the caller
// its own current device back afterwards.  Every entry point that queues or
// waits for work of a context holds one, so a caller whose thread has another
// GPU current (a second context, or torch's current device) still reaches the
// context's stream and memory.  If the caller's device cannot be read (no
// context on this thread yet), the context's device stays current.
class DeviceGuard {
public:
    explicit DeviceGuard(int device)
    {
        have_prev_ = cudaGetDevice(&prev_) == cudaSuccess;
        if (have_prev_ && prev_ == device) return;
        err_ = cudaSetDevice(device);
        changed_ = err_ == cudaSuccess && have_prev_;
    }
    ~DeviceGuard()
    {
        if (changed_) cudaSetDevice(prev_);
    }
    cudaError_t error() const { return err_; }
    DeviceGuard(const DeviceGuard &) = delete;
    DeviceGuard &operator=(const DeviceGuard &) = delete;

private:
    int prev_ = 0;
    bool have_prev_ = false;
    bool changed_ = false;
    cudaError_t err_ = cudaSuccess;
};

// NVTX range over a C-ABI call (host side: the calls queue work on the
// context's stream), for timelines of the library's work.
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};
}  // namespace lbm

// Holds the context device for the rest of the enclosing C-ABI call; returns
// the call's CUDA status if the device cannot be made current.
#define LBM_ON_DEVICE(dev)                                                            \
    const lbm::DeviceGuard lbm_device_guard_(dev);                                    \
    do {                                                                              \
        if (lbm_device_guard_.error() != cudaSuccess)                                 \
            return lbm::cuda_fail(lbm_device_guard_.error(), "cudaSetDevice");       \
    } while (0)
