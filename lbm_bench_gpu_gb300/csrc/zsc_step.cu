// zsc_step.cu -- one fused sm_103a kernel per ZSC lattice Boltzmann step.
//
// One launch does what the reference does with seven kernels (plus six
// pack/unpack kernels) and three host-staged halo exchanges per step (src/main.cu:496-608):
//   update_phi / update_rho / update_velocity   (moments)
//   collision_f (D3Q7 phi) / collision_g (D3Q19 momentum, forcing)
//   stream_f (ZSC eta-interpolated) / stream_g (plain)
//   pack/unpack + mpiUpdate* halos -> periodic index wrap
//
// Storage:
//  * f (D3Q7) is kept post-collision, A/B: step n reads P^{n-1} and rebuilds
//    the streamed value on the fly, f_i(x) = eta P_i(x - c_i) + (1-eta) P_i(x)
//    (src/stream_f.cu:52-59 turned from push into pull), and writes P^n.
//  * g (D3Q19) is streamed in place with the AA pattern: even steps read and
//    write the node's own slots (direction reversed on write); odd steps read
//    the reversed slots of the upstream neighbours and write the downstream
//    neighbours' natural slots.  Each thread reads and writes the same 19
//    locations, so the update is race-free in one buffer.
//  * Storage type ST of f_1..f_6 and g: float, or __half / __nv_bfloat16 with a
//    per-field affine map (stored = (value - shift) * scale; shift = w_i mean(rho)
//    for g).  f_0 ~ phi is bimodal (+-phiStar), so no shift centres it: it stays
//    FP32 in every format.  Arithmetic is FP32 throughout.
//
// Work decomposition: a block owns a TX x TY column tile and marches a chunk
// of tz planes in z.  The phi stencil (19-point Laplacian and gradient,
// src/collision_f.cu:61-94) needs phi on a one-node ring around the tile, and
// phi = sum f needs P^{n-1} one node further out, so each plane of P^{n-1} is
// staged in shared memory on the tile plus two halo rows and one 16-byte
// chunk of halo columns on each side.
//
// Memory pipeline: the global reads go through asynchronous copies into
// shared-memory stages (L2-cached, no registers held while in flight):
//   - the 19 g rows of the next plane (2 stages; odd steps stage one extra
//     chunk per row so the +-x shifted reads stay 16-byte aligned),
//   - the 7 P_f planes three planes ahead (4 stages),
// so a block always has about one plane of the step's input in flight while it
// computes the current plane.  The P_f planes (tile + ragged halo, periodic
// wrap) and the odd step's shifted g rows are cp.async 16-byte chunks: warps
// 0-3 queue P_f, warps 4-7 queue g, each thread with chunk coordinates fixed
// for the whole block; with nx a multiple of 32 no chunk straddles the seam.
// In the even step the g tile goes by one TMA tensor copy per plane (4-d
// tensor map x, y, z, field; box 32 x 8 x 1 x 19) completing on an mbarrier;
// the odd step stages its shifted g rows with cp.async only.  For 16-bit
// storage the P_f planes of interior tiles also come by TMA (a 3-d f_0 box and
// a 4-d f_1..f_6 box per plane).  The mbarrier waits are bounded and report a
// timeout through an error flag.
#include <cuda.h>   // CUtensorMap (the encoder is fetched from the driver at run time)
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <cstring>
#include <type_traits>
#include <utility>

#include "lattice.cuh"

namespace lbm {
namespace {

#ifndef ZSC_TILE_Y
#define ZSC_TILE_Y 8
#endif
constexpr int TX = 32;              // tile width in x (one warp per row)
constexpr int TY = ZSC_TILE_Y;      // tile height in y
constexpr int NT = TX * TY;         // threads per block
constexpr int FR = TY + 4;          // staged P_f rows: y in [y0 - 2, y0 + TY + 2)
constexpr int W0 = TX + 8;          // staged f_0 row (floats): x in [x0 - 4, x0 + 36)
constexpr int RW = TX + 2;          // phi ring width (tile + one-node ring)
constexpr int RH = TY + 2;
constexpr int RING = 2 * RW + 2 * TY;
// 16-bit storage keeps its fields in the pair layout: 32-bit word w of a row
// holds nodes x = w and x = w + nx/2.  A tile is TXW words (32 nodes) wide and
// its phi ring holds float2 words (node w in .x, node w + nx/2 in .y).
constexpr int TXW = TX / 2;
constexpr int RWP = TXW + 2;
constexpr int RINGP = 2 * RWP + 2 * TY;
constexpr int NG = 2;               // g stages
static_assert(RING <= NT, "one ring node per thread at most");
static_assert(TX == 32 && TY == 8, "issuer roles assume a 32 x 8 tile");

constexpr float kInv6 = 0.16666666666666666667f;

// 16-bit storage: two nodes per thread (128 threads per 32-node x 8 tile), the
// two nodes of one 32-bit word of the pair layout (A = x in .x, B = x + nx/2 in
// .y of every packed f32x2 value), both nodes' 16-bit values converted and
// stored as one 32-bit word.
template <typename ST>
constexpr bool use_pair() { return sizeof(ST) == 2; }
template <typename ST>
constexpr int threads_of() { return use_pair<ST>() ? NT / 2 : NT; }

// Packed FP32 (f32x2: two lanes per instruction, each rounded as FP32) in the
// D3Q19 collision: 32-36 fewer warp instructions per 32 nodes, FP16 storage
// 38.6k -> 39.6k MLUPS at 256^3.  (Packing the eta-blends, the stencil sums
// and rho as well saved no instructions — forming the register pairs costs
// what the packed operations save — and was slower.)
#ifndef ZSC_PACKED
#define ZSC_PACKED 1
#endif
#ifndef ZSC_TMA_G
#define ZSC_TMA_G 1
#endif
// Odd steps stage their shifted g rows with cp.async: one TMA tensor copy per
// direction (19 per plane, interior tiles) measured slower (256^3: FP16 one
// node per thread 33.7k vs 36.2k, two nodes per thread 39.5k vs 41.9k, pair
// layout 41.9k vs 45.5k; FP32 26.7k vs 27.2k MLUPS), and one 1-d bulk copy
// (cp.async.bulk) per shifted row, 152 per plane, slower still (FP16 36.8k vs
// 42.3k, FP32 26.5k vs 27.6k).
// the P_f planes by TMA on interior tiles (f_0 box W0 x FR, f_1..f_6 box
// W x FR x 6), for the 16-bit formats: measured at 256^3 (same GPU, 500
// steps), FP16 36 250 -> 37 060 MLUPS, while FP32 drops 27 110 -> 26 560 with
// it (its per-thread cp.async spreads the twice larger planes better; again
// 27 200 -> 26 640 with the current kernel); 2 = all formats
#ifndef ZSC_TMA_F
#define ZSC_TMA_F 1
#endif
constexpr bool kUseTma = ZSC_TMA_G != 0;
constexpr bool kUseTmaF = ZSC_TMA_F != 0;
template <typename ST>
constexpr bool use_tma_f() { return kUseTmaF && (sizeof(ST) == 2 || ZSC_TMA_F == 2); }
constexpr float kInv12 = 0.08333333333333333333f;

template <int I>
struct Dir {
    static constexpr int value = I;
};

// Staging geometry implied by the element size.  FP32 (two blocks per SM)
// stages 4 P_f planes and 4 phi planes; the 16-bit formats fit four blocks per
// SM into the shared memory with 3 + 3 and g rows one chunk narrower (the odd
// step's shifted rows need one extra chunk on one side only).
template <typename ST>
struct Geo {
    static constexpr bool kSmall = sizeof(ST) == 2;
    static constexpr int E = 16 / (int)sizeof(ST);   // elements per 16-byte chunk
    static constexpr int W = TX + 2 * E;             // staged P_f row: x in [x0 - E, x0 + TX + E)
    static constexpr int GW = kSmall ? TX + E : TX + 2 * E;   // staged g row
    static constexpr int GX0 = kSmall ? 0 : E;       // g row column of x0 (even step: E)
    static constexpr int NF = kSmall ? 3 : 4;        // P_f stages
    static constexpr int NPHI = kSmall ? 3 : 4;      // phi planes
    static constexpr int CR = W / E;                 // chunks per staged row
    static constexpr int CM = TX / E;                // chunks covering [x0, x0 + TX)
    static constexpr int G_STAGE = kQg * TY * GW * (int)sizeof(ST);           // bytes
    static constexpr int F0_BYTES = FR * W0 * 4;
    static constexpr int F_STAGE = F0_BYTES + (kQf - 1) * FR * W * (int)sizeof(ST);
    static constexpr int PHI_STAGE = sizeof(ST) == 2 ? RH * RWP * 8 : RH * RW * 4;
    static constexpr int G_OFF = 0;
    static constexpr int F_OFF = NG * G_STAGE;
    static constexpr int PHI_OFF = F_OFF + NF * F_STAGE;
    static constexpr int MBAR_OFF = PHI_OFF + NPHI * PHI_STAGE;   // mbarriers: 2 g stages, then NF P_f stages
    static constexpr int SMEM = MBAR_OFF + 8 * (NG + NF);
    static constexpr int G_TMA_BYTES = kQg * TY * TX * (int)sizeof(ST);   // one plane's tile, 19 fields
    static constexpr int TPD = TY * CM;              // g issuer threads per direction
    static constexpr int D = (NT / 2) / TPD;         // directions per pass of the g issuers
    static_assert(G_STAGE % 16 == 0 && F_STAGE % 16 == 0 && F0_BYTES % 16 == 0, "16-byte aligned stages");
    static_assert(G_STAGE % 128 == 0 && G_TMA_BYTES <= G_STAGE, "TMA destinations: 128-byte aligned, inside a stage");
    static_assert(E + TX <= GW, "even-step rows staged from column E fit a g row");
    static_assert(MBAR_OFF % 8 == 0, "8-byte aligned mbarriers");
    static_assert(F_OFF % 128 == 0 && F_STAGE % 128 == 0 && F0_BYTES % 128 == 0, "P_f TMA destinations 128-byte aligned");
    static_assert(FR * (W0 / 4) <= NT / 2 && FR * CR <= NT / 2, "P_f issuers fit in warps 0-3");
    static_assert(D * TPD == NT / 2, "g issuers cover whole directions");
};

template <typename ST>
struct StepPtrs {
    const float *f0in;
    float *f0out;
    const ST *fin[kQf - 1];   // f_1 .. f_6
    ST *fout[kQf - 1];
    const ST *gin[kQg];       // g read (== g for the in-place AA update)
    ST *g[kQg];               // g written
    float *mom[5];
    int *err;                 // set when a bounded wait gives up
};

__device__ __forceinline__ int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// 16-byte global -> shared copy, cached in L2 only; completes asynchronously.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

// Checked builds (ZSC_CHECKED=1, a separate library for testing): every global
// store and cp.async source is checked against its field's extent first; an
// index out of range sets bit 4 of the context's error flag and the access is
// skipped, in place of the memory checker.  Other builds compile the checks away.
#ifndef ZSC_CHECKED
#define ZSC_CHECKED 0
#endif
__device__ __forceinline__ bool in_field(long long idx, int count, long long n, int *err)
{
#if ZSC_CHECKED
    if (idx < 0 || idx + count > n) {
        atomicOr(err, 4);
        return false;
    }
#endif
    return true;
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---- mbarrier + TMA (bulk tensor copy) ----
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// One poll of an mbarrier phase: the thread sleeps until the phase completes
// or kSuspendNs pass (so a waiting warp takes no issue slots), then reports
// whether it completed.
constexpr unsigned kSuspendNs = 100000;
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned phase)
{
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(phase), "r"(kSuspendNs)
        : "memory");
    return done != 0;
}
// Bounded wait for phase `phase` of an mbarrier: false after kWaitLimit polls
// (at most kWaitLimit * kSuspendNs = 2 s).
constexpr unsigned kWaitLimit = 20000;
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned phase, unsigned limit = kWaitLimit)
{
    for (unsigned it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// Programmatic dependent launch: a step grid lets the next step's grid be
// scheduled as soon as all its own blocks have started (so the next grid's
// blocks take the SMs this grid's tail frees), and a block waits for the
// previous grid's completion and memory before it first touches the state.
// Measured (MLUPS, without -> with): 256^3 FP32 27 197 -> 27 433, FP16
// 41 935 -> 42 287; 128^3 FP32 24 476 -> 24 852, FP16 33 558 -> 35 194.
#ifndef ZSC_PDL
#define ZSC_PDL 1
#endif
__device__ __forceinline__ void pdl_launch_dependents()
{
#if ZSC_PDL
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
#endif
}
__device__ __forceinline__ void pdl_wait()
{
#if ZSC_PDL
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
#endif
}

// One warp waits, bounded, on a fresh mbarrier that nothing arrives at (no
// copy is issued against it, so nothing is in flight when the block exits):
// the wait gives up and the error flag is set as in the step kernel.
__global__ void wait_selftest_kernel(int *err, unsigned limit)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    const bool done = mbar_wait(&bar, 0, limit);
    if (__syncthreads_or(!done) && threadIdx.x == 0) atomicOr(err, 1);
}
// Order this thread's earlier generic-proxy shared-memory accesses (made
// visible to it by a barrier) before a following TMA write to the same bytes.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// f(Dir<i>) for i = I, I + D, I + 2D, ... < 19
template <int I, int D, typename F>
__device__ __forceinline__ void for_dirs_from(F &&f)
{
    if constexpr (I < kQg) {
        f(Dir<I>{});
        for_dirs_from<I + D, D>(f);
    }
}

// The 16-bit storage map folded into the step's constants.  The step works on
// stored values: a stored f_k is f_k f_scale, so phi = f_0 + f_inv sum_k f_k
// and the outputs f_scale P_k come from f_scale-scaled collision terms; a
// stored g_i is (g_i - shift_i) g_scale, so rho = g_inv sum_i s_i + sum_i
// shift_i (the shifts cancel in the momentum's opposite-pair differences),
// and with bb = 1 - 1/tauRho the stored output is
//   (bb g_i + eq_i - shift_i) g_scale = bb s_i + g_scale eq_i + (bb - 1) shift_i g_scale,
// i.e. the FP32 collision with g_scale-scaled constants plus one constant per
// weight class (g_scale g_inv = 1 exactly: both are powers of two).
struct StepMap {
    float f_inv, Af, Cf;                  // f_inv; f_scale Gamma / (2 tauPhi); f_scale invTauPhi invEta2
    float g_inv, rho_shift;               // g_inv; sum of the shifts
    float K0, K1, K2, KC0, KC1, KC2;      // g_scale x the collision constants
    float k0, k1, k2;                     // (bb - 1) shift g_scale: rest, face, edge classes
};

StepMap step_map(const StepConst &c, const Quant &q)
{
    StepMap m;
    m.f_inv = q.f_inv;
    m.Af = 0.5f * c.Gamma * c.invTauPhi * q.f_scale;
    m.Cf = c.invTauPhi * c.invEta2 * q.f_scale;
    m.g_inv = q.g_inv;
    float rs = 0.f;
    for (int i = 0; i < kQg; i++) rs += q.g_shift[i];
    m.rho_shift = rs;
    m.K0 = c.K0 * q.g_scale;
    m.K1 = c.K1 * q.g_scale;
    m.K2 = c.K2 * q.g_scale;
    m.KC0 = c.KC0 * q.g_scale;
    m.KC1 = c.KC1 * q.g_scale;
    m.KC2 = c.KC2 * q.g_scale;
    const float bm1 = c.invTauRhoOne - 1.f;
    m.k0 = bm1 * q.g_shift[0] * q.g_scale;
    m.k1 = bm1 * q.g_shift[1] * q.g_scale;
    m.k2 = bm1 * q.g_shift[7] * q.g_scale;
    return m;
}

// TMA: on even steps the g tile comes by one tensor copy per plane (gmap) in
// the dense layout [field][TY][TX]; odd steps stage their shifted rows with
// cp.async into [dir][TY][W].  Without TMA gmap is unused.
// The box as the step kernel sees it (the field lengths of a z-slab follow
// from nz and ZG).
struct StepBox {
    int nx, ny, nz;
    long long nxy, n;
};

__device__ __forceinline__ unsigned node_index(const StepBox &b, int x, int y, int z)
{
    return (unsigned)x + (unsigned)b.nx * ((unsigned)y + (unsigned)b.ny * (unsigned)z);
}

// ZG: the box is a z-slab whose fields carry ghost planes (Box::zghost): a
// separate instance, so the periodic kernels keep their registers.
template <typename ST, bool STREAMED, bool ODD, bool TMA, bool ZG>
__global__ void __launch_bounds__(threads_of<ST>(), Fmt<ST>::kMinBlocks)
zsc_step_kernel(const StepPtrs<ST> P, const StepBox b, const StepConst c, const StepMap m, const int tz,
                const int write_moments, const int zlo, const int zhi, const __grid_constant__ CUtensorMap gmap,
                const __grid_constant__ CUtensorMap f0map, const __grid_constant__ CUtensorMap fqmap)
{
    using Gm = Geo<ST>;
    using Fm = Fmt<ST>;
    constexpr int E = Gm::E, W = Gm::W, GW = Gm::GW, GX0 = Gm::GX0, CR = Gm::CR, CM = Gm::CM;
    constexpr int NF = Gm::NF, NPHI = Gm::NPHI;
    extern __shared__ __align__(128) unsigned char smem[];
    ST *const G = reinterpret_cast<ST *>(smem + Gm::G_OFF);            // [NG][19][TY][GW]
    unsigned char *const F = smem + Gm::F_OFF;                          // [NF]{f0 [FR][W0]; fq [6][FR][W]}
    float *const PHI = reinterpret_cast<float *>(smem + Gm::PHI_OFF);   // [NPHI][RH][RW] (pairs: float2 [RWP])
    constexpr int G_ELEMS = kQg * TY * GW;                              // per stage

    constexpr bool PAIR = use_pair<ST>();
    constexpr int XPT = PAIR ? 2 : 1;          // x nodes per thread (block TX / XPT x TY)
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * (TX / XPT) + tx;
    int bid = blockIdx.x;
    const int ntx = b.nx / TX, nty = b.ny / TY;
    const int bx = bid % ntx;
    bid /= ntx;
    const int by = bid % nty;
    bid /= nty;
    // a z-slab launch may cover planes [zlo, zhi) only (its interior while the
    // halo planes are in flight, then its boundary planes)
    const int z0 = (ZG ? zlo : 0) + bid * tz;
    const int nzc = min(tz, (ZG ? zhi : b.nz) - z0);   // planes of this chunk
    const int x0 = bx * TX, y0 = by * TY;
    const int x = x0 + XPT * tx, y = y0 + ty;   // (first) node of the thread

    // memory plane of P_f plane p and of g plane p: periodic wrap, or in a
    // z-slab the ghost-extended fields (two planes below the slab for f, one
    // for g; the moment fields have none)
    constexpr bool zg = ZG;
    // elements of an f / g field (checked builds test indices against them)
    const long long nf = b.nxy * (b.nz + (zg ? 4 : 0)), ng = b.nxy * (b.nz + (zg ? 2 : 0));
    auto zf = [&](int p) { return zg ? p + 2 : wrap(p, b.nz); };
    auto zgm = [&](int p) { return zg ? p + 1 : wrap(p, b.nz); };
    auto zg0 = [&](int p) { return zg ? p + 1 : p; };   // a plane of the box itself

    uint64_t *const mbar = reinterpret_cast<uint64_t *>(smem + Gm::MBAR_OFF);
    constexpr bool g_tma = TMA && !ODD;   // the even step's g tile: one TMA copy per plane
    // P_f planes by TMA: the staged rows y0 - 2 .. y0 + TY + 1 and columns
    // x0 - 4 .. x0 + TX + 3 (f_0) / x0 - E .. x0 + TX + E - 1 (f_1..f_6) inside the box
    const bool tile_tma_f = TMA && use_tma_f<ST>() && x0 - 4 >= 0 && x0 - E >= 0 && x0 + TX + 4 <= b.nx &&
                            x0 + TX + E <= b.nx && y0 - 2 >= 0 && y0 + TY + 2 <= b.ny;
    if constexpr (TMA) {
        // a TMA destination must be 128-byte aligned (uniform check: every
        // thread returns before any wait or barrier)
        if (smem_u32(G) & 127u) {
            if (tid == 0) atomicOr(P.err, 2);
            return;
        }
        if (tid == 0) {
            for (int k = 0; k < NG + NF; k++) mbar_init(&mbar[k], 1);
            mbar_init_fence();
        }
        __syncthreads();
    }

    // Halo ring node (16-bit: ring word) handled by this thread (if any): top
    // row, bottom row, left column, right column of the (RWX) x (TY+2) phi tile.
    constexpr int RWX = PAIR ? RWP : RW;
    const bool has_ring = tid < (PAIR ? RINGP : RING);
    int rlx = 0, rly = 0;
    if (tid < RWX) {
        rlx = tid;
        rly = 0;
    } else if (tid < 2 * RWX) {
        rlx = tid - RWX;
        rly = TY + 1;
    } else if (tid < 2 * RWX + TY) {
        rlx = 0;
        rly = tid - 2 * RWX + 1;
    } else if (has_ring) {
        rlx = RWX - 1;
        rly = tid - 2 * RWX - TY + 1;
    }
    // Pair layout: staged words that came round the periodic x seam hold their
    // two nodes swapped (word w - nx/2 of the row is word w's neighbour pair in
    // the other order).  Tiles at the left seam (x0 = 0) see that in the staged
    // columns left of the tile, tiles at the right seam right of it.
    const bool seam_l = x0 == 0, seam_r = x0 + TX == b.nx;

    // P_f stage of plane p (p >= z0 - 2): planes z0 - 2 + m go to stage m % NF
    // for their (m / NF)-th use; f_0 part and f_1..f_6 part
    auto fslot = [&](int p) { return (unsigned)(p - z0 + 2) % (unsigned)NF; };
    auto fstage = [&](int p) { return F + fslot(p) * Gm::F_STAGE; };
    auto f0part = [&](unsigned char *st) { return reinterpret_cast<float *>(st); };
    auto fqpart = [&](unsigned char *st) { return reinterpret_cast<ST *>(st + Gm::F0_BYTES); };

    // ---- staging roles, fixed per thread for the whole chunk ----
    // Warps 0-3 queue P_f: thread t owns staged row t / (chunks per row), chunk
    // t % (chunks per row), of f_0 (FP32 geometry) and of f_1..f_6 (ST geometry).
    const bool f0_issuer = tid < FR * (W0 / 4);
    const bool fq_issuer = tid < FR * CR;
    int f0_xy = 0, f0_dst = 0, fq_xy = 0, fq_dst = 0;
    if (f0_issuer) {
        const int r = tid / (W0 / 4), k = tid - r * (W0 / 4);
        f0_xy = wrap(x0 - 4 + 4 * k, b.nx) + b.nx * wrap(y0 - 2 + r, b.ny);
        f0_dst = r * W0 + 4 * k;
    }
    if (fq_issuer) {
        const int r = tid / CR, k = tid - r * CR;
        fq_xy = wrap(x0 - E + E * k, b.nx) + b.nx * wrap(y0 - 2 + r, b.ny);
        fq_dst = r * W + E * k;
    }
    // Warps 4-7 queue the g rows: thread owns row g_r, chunk g_k of every D-th
    // direction starting at g_q (uniform per warp).
    const int gt = PAIR ? tid : tid - NT / 2;   // with 128 threads every thread also queues g
    const bool g_issuer = gt >= 0;
    const int g_q = gt / Gm::TPD;
    const int g_r = (gt % Gm::TPD) / CM, g_k = gt % CM;
    int g_row_0 = 0, g_row_p = 0, g_row_m = 0, g_x_lo = 0, g_x_hi = 0, g_x_wrap = 0;
    if (g_issuer) {
        g_row_0 = b.nx * (y0 + g_r);
        g_row_p = b.nx * wrap(y0 + g_r - 1, b.ny);   // directions with c_y = +1 read row y - 1
        g_row_m = b.nx * wrap(y0 + g_r + 1, b.ny);   // c_y = -1 reads row y + 1
        g_x_lo = wrap(x0 - E + E * g_k, b.nx);        // c_x = +1 reads x - 1: chunks from x0 - E
        g_x_hi = x0 + E * g_k;                         // c_x <= 0: chunks from x0
        g_x_wrap = wrap(x0 + TX, b.nx);                // c_x = -1 also needs x0 + TX
    }

    // P_f stage p's mbarrier and the phase of plane p's use of it
    auto fbar = [&](int p) { return &mbar[NG + fslot(p)]; };
    auto fphase = [&](int p) { return ((unsigned)(p - z0 + 2) / (unsigned)NF) & 1u; };
    // phi slot of plane p (planes z0 - 1 + m go to slot m % NPHI)
    auto pslot = [&](int p) { return (int)((unsigned)(p - z0 + 1) % (unsigned)NPHI); };

    // Queue the 7 P_f planes of plane p (tile + halo) into its stage.
    auto issue_f = [&](int p) {
        if (tile_tma_f) {
            if (tid == 32) {   // lane 0 of warp 1 (warp 0 issues the g copies)
                unsigned char *st = fstage(p);
                const int zp = zf(p);
                fence_proxy_async();
                mbar_expect_tx(fbar(p), (unsigned)Gm::F_STAGE);
                tma_load_3d(f0part(st), &f0map, x0 - 4, y0 - 2, zp, fbar(p));
                tma_load_4d(fqpart(st), &fqmap, x0 - E, y0 - 2, zp, 0, fbar(p));
            }
            return;
        }
        const unsigned zb = (unsigned)zf(p) * (unsigned)b.nxy;
        unsigned char *st = fstage(p);
        if (f0_issuer && in_field((long long)zb + f0_xy, 4, nf, P.err))
            cp_async16(f0part(st) + f0_dst, P.f0in + (zb + (unsigned)f0_xy));
        if (fq_issuer) {
            ST *dst = fqpart(st) + fq_dst;
            const unsigned base = zb + (unsigned)fq_xy;
#pragma unroll
            for (int a = 0; a < kQf - 1; a++)
                if (in_field(base, E, nf, P.err)) cp_async16(dst + a * FR * W, P.fin[a] + base);
        }
    };

    // Call f(Dir<i>) for the directions this g issuer owns (compile-time
    // direction numbers; the branch is uniform per warp).
    auto for_my_dirs = [&](auto &&f) {
        if constexpr (Gm::D == 2) {
            if (g_q == 0) for_dirs_from<0, 2>(f);
            else for_dirs_from<1, 2>(f);
        } else {
            static_assert(Gm::D == 4, "two or four directions per pass");
            if (g_q == 0) for_dirs_from<0, 4>(f);
            else if (g_q == 1) for_dirs_from<1, 4>(f);
            else if (g_q == 2) for_dirs_from<2, 4>(f);
            else for_dirs_from<3, 4>(f);
        }
    };

    // Queue the 19 g rows the nodes of plane z read, into g stage s.  Even
    // steps read the node's own slots; odd steps read direction i of node x
    // from the reversed slot of x - c_i (AA pattern).
    auto issue_g = [&](int z, int s) {
        if constexpr (TMA && !ODD) {
            if (tid == 0) {
                fence_proxy_async();
                mbar_expect_tx(&mbar[s], (unsigned)Gm::G_TMA_BYTES);
                tma_load_4d(G + s * G_ELEMS, &gmap, x0, y0, zg0(z), 0, &mbar[s]);
            }
            return;
        }
        if (!g_issuer) return;
        ST *dst = G + s * G_ELEMS + g_r * GW;
        if (!ODD) {
            const unsigned base = (unsigned)zg0(z) * (unsigned)b.nxy + (unsigned)(g_row_0 + g_x_hi);
            for_my_dirs([&](auto d) {
                constexpr int i = decltype(d)::value;
                if (in_field(base, E, ng, P.err)) cp_async16(dst + i * TY * GW + E + E * g_k, P.gin[i] + base);
            });
        } else {
            const unsigned zb0 = (unsigned)zg0(z) * (unsigned)b.nxy;
            const unsigned zbp = (unsigned)zgm(z - 1) * (unsigned)b.nxy;   // c_z = +1 reads z - 1
            const unsigned zbm = (unsigned)zgm(z + 1) * (unsigned)b.nxy;   // c_z = -1 reads z + 1
            for_my_dirs([&](auto d) {
                constexpr int i = decltype(d)::value;
                constexpr int cx = kCx(i), cy = kCy(i), cz = kCz(i);
                const unsigned zb = cz > 0 ? zbp : (cz < 0 ? zbm : zb0);
                const int row = cy > 0 ? g_row_p : (cy < 0 ? g_row_m : g_row_0);
                const ST *src = P.gin[kOpp(i)] + (zb + (unsigned)row);
                ST *d_row = dst + i * TY * GW;
                const long long r0 = (long long)zb + row;   // row start in the field
                if (cx > 0) {
                    // columns 0 .. TX + E - 1 hold x0 - E .. x0 + TX - 1
                    if (in_field(r0 + g_x_lo, E, ng, P.err)) cp_async16(d_row + E * g_k, src + g_x_lo);
                    if (g_k == 0 && in_field(r0 + x0 + TX - E, E, ng, P.err))
                        cp_async16(d_row + TX, src + (x0 + TX - E));
                } else {
                    // columns GX0 .. hold x0 .. x0 + TX (+ E for cx < 0)
                    if (in_field(r0 + g_x_hi, E, ng, P.err)) cp_async16(d_row + GX0 + E * g_k, src + g_x_hi);
                    if (cx < 0 && g_k == 0 && in_field(r0 + g_x_wrap, E, ng, P.err))
                        cp_async16(d_row + TX + GX0, src + g_x_wrap);
                }
            });
        }
    };

    // Streamed D3Q7 values at ring-tile position (lx, ly) of plane p (f_1..f_6
    // in stored units) and phi (src/update_phi.cu:42-43), from the staged planes.
    auto phi_at = [&](int p, int lx, int ly, float(&f)[kQf]) -> float {
        const int row = ly + 1;
        const int c0 = lx + 3;          // f_0 column: x - (x0 - 4)
        const int cq = lx - 1 + E;      // f_1..f_6 column: x - (x0 - E)
        unsigned char *S1 = fstage(p);
        auto raw = [&](unsigned char *S, int a, int rr, int cc) {
            return Fm::load(fqpart(S)[(a * FR + rr) * W + cc]);
        };
        // eta P(x - c) + (1 - eta) P(x), in stored units
        auto blend = [&](unsigned char *Su, int a, int ru, int cu) {
            return c.eta * raw(Su, a, ru, cu) + c.eta2 * raw(S1, a, row, cq);
        };
        f[0] = f0part(S1)[row * W0 + c0];
        if (STREAMED) {
#pragma unroll
            for (int a = 0; a < kQf - 1; a++) f[a + 1] = raw(S1, a, row, cq);
        } else {
            unsigned char *S0 = fstage(p - 1), *S2 = fstage(p + 1);
            f[1] = blend(S1, 0, row, cq - 1);
            f[2] = blend(S1, 1, row, cq + 1);
            f[3] = blend(S1, 2, row - 1, cq);
            f[4] = blend(S1, 3, row + 1, cq);
            f[5] = blend(S0, 4, row, cq);
            f[6] = blend(S2, 5, row, cq);
        }
        if constexpr (Fm::kMapped) return fmaf(m.f_inv, f[1] + f[2] + f[3] + f[4] + f[5] + f[6], f[0]);
        else return f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6];
    };

    // phi of plane p on the tile + ring into phi slot s; the streamed f of the
    // thread's own node(s) is returned in fo.
    auto build_plane = [&](int p, int s, float(&fo)[XPT][kQf]) {
        float *ph = PHI + s * (RH * RW);
#pragma unroll
        for (int k = 0; k < XPT; k++)
            ph[(ty + 1) * RW + XPT * tx + k + 1] = phi_at(p, XPT * tx + k + 1, ty + 1, fo[k]);
        if (has_ring) {
            float tmp[kQf];
            ph[rly * RW + rlx] = phi_at(p, rlx, rly, tmp);
        }
    };

    // Pair layout (16-bit storage): the same for the two nodes of a word at
    // once.  Ring word column lx (0 = row word x0/2 - 1) is staged f_0 word
    // column lx + 1 (f_0 rows start at word x0/2 - 2) and f_1..f_6 word column
    // lx + 3 (rows start at word x0/2 - 4); a word that came round the x seam
    // is swapped back on read.
    using T2 = typename Fm::T2;
    // byte_perm selectors of the staged columns a word position reads, fixed
    // per thread: fq columns cq - 1, cq, cq + 1 and the f_0 column.  The own
    // word (cq = tx + 4) only reads across the seam at the tile's edge words.
    struct Sel {
        unsigned m, c, p;
        bool f0;
    };
    auto sel_of = [&](int lx) {
        const int cq = lx + 3, c0 = lx + 1;
        auto q = [&](int cw) { return (seam_l && cw < 4) || (seam_r && cw >= TXW + 4) ? kSwap : kKeep; };
        Sel r;
        r.m = q(cq - 1);
        r.c = q(cq);
        r.p = q(cq + 1);
        r.f0 = (seam_l && c0 < 2) || (seam_r && c0 >= TXW + 2);
        return r;
    };
    const Sel sel_own = {seam_l && tx == 0 ? kSwap : kKeep, kKeep, seam_r && tx == TXW - 1 ? kSwap : kKeep, false};
    const Sel sel_ring = sel_of(rlx);
    auto fq_word = [&](unsigned char *S, int a, int rr, int cw, unsigned sel) -> float2 {
        const T2 v = reinterpret_cast<const T2 *>(fqpart(S))[(a * FR + rr) * (W / 2) + cw];
        return Fm::load2(Fm::perm2(v, sel));
    };
    auto phi_pair = [&](int p, int lx, int ly, const Sel &sw, float2(&f)[kQf]) -> float2 {
        using namespace pk;
        const int row = ly + 1, c0 = lx + 1, cq = lx + 3;
        unsigned char *S1 = fstage(p);
        const float2 v0 = reinterpret_cast<const float2 *>(f0part(S1))[row * (W0 / 2) + c0];
        f[0] = sw.f0 ? make_float2(v0.y, v0.x) : v0;
        if (STREAMED) {
#pragma unroll
            for (int a = 0; a < kQf - 1; a++) f[a + 1] = fq_word(S1, a, row, cq, sw.c);
        } else {
            unsigned char *S0 = fstage(p - 1), *S2 = fstage(p + 1);
            // eta P(x - c) + (1 - eta) P(x), in stored units
            auto blend = [&](unsigned char *Su, int a, int ru, int cu, unsigned su) {
                return fma(splat(c.eta), fq_word(Su, a, ru, cu, su), mul(splat(c.eta2), fq_word(S1, a, row, cq, sw.c)));
            };
            f[1] = blend(S1, 0, row, cq - 1, sw.m);
            f[2] = blend(S1, 1, row, cq + 1, sw.p);
            f[3] = blend(S1, 2, row - 1, cq, sw.c);
            f[4] = blend(S1, 3, row + 1, cq, sw.c);
            f[5] = blend(S0, 4, row, cq, sw.c);
            f[6] = blend(S2, 5, row, cq, sw.c);
        }
        return fma(splat(m.f_inv), add(add(add(add(add(f[1], f[2]), f[3]), f[4]), f[5]), f[6]), f[0]);
    };
    auto build_pair = [&](int p, int s, float2(&fo)[kQf]) {
        float2 *ph = reinterpret_cast<float2 *>(PHI) + s * (RH * RWP);
        ph[(ty + 1) * RWP + tx + 1] = phi_pair(p, tx + 1, ty + 1, sel_own, fo);
        if (has_ring) {
            float2 tmp[kQf];
            ph[rly * RWP + rlx] = phi_pair(p, rlx, rly, sel_ring, tmp);
        }
    };

    // Neighbour offsets in x and y are fixed for the thread; z per plane.
    const int o_xm = (x == 0) ? b.nx - 1 : -1;
    const int o_xp = (x == b.nx - 1) ? -(b.nx - 1) : 1;
    const int o_ym = (y == 0) ? (b.ny - 1) * b.nx : -b.nx;
    const int o_yp = (y == b.ny - 1) ? -(b.ny - 1) * b.nx : b.nx;

    float fcur[XPT][kQf], fnext[XPT][kQf];   // one node per thread (FP32)
    float2 fcur2[kQf], fnext2[kQf];           // pair layout (16-bit storage)

    pdl_launch_dependents();
    pdl_wait();   // the previous step's writes are complete and visible

    // prologue: P_f planes z0-2 .. z0+1 (with 3 stages: z0+1 after the first
    // build), g of plane z0; phi of z0-1 and z0
    constexpr int kAhead = NF - 1;   // P_f planes past z0 - 2 staged before the first build
    issue_f(z0 - 2);
    issue_f(z0 - 1);
    issue_f(z0);
    if (kAhead >= 3) issue_f(z0 + 1);
    issue_g(z0, 0);
    cp_async_commit();
    cp_async_wait_all();
    bool late = false;
    if (tile_tma_f) {
        for (int p = z0 - 2; p <= z0 - 2 + kAhead; p++) late |= !mbar_wait(fbar(p), fphase(p));
    }
    __syncthreads();
    if constexpr (PAIR) {
        float2 tmp[kQf];
        build_pair(z0 - 1, pslot(z0 - 1), tmp);
    } else {
        float tmp[XPT][kQf];
        build_plane(z0 - 1, pslot(z0 - 1), tmp);
    }
    if (kAhead < 3) {
        // the stage of plane z0 - 2 is free once every thread has built z0 - 1
        __syncthreads();
        issue_f(z0 + 1);
        cp_async_commit();
        cp_async_wait_all();
        if (tile_tma_f) late |= !mbar_wait(fbar(z0 + 1), fphase(z0 + 1));
        __syncthreads();
    }
    if constexpr (PAIR) build_pair(z0, pslot(z0), fcur2);
    else build_plane(z0, pslot(z0), fcur);
    __syncthreads();
    issue_f(z0 + 2);
    cp_async_commit();

    for (int j = 0; j < nzc; ++j) {
        const int z = z0 + j;
        cp_async_wait_all();
        __syncthreads();
        if (j + 1 < nzc) {
            issue_g(z + 1, (j + 1) & 1);
            if (kAhead >= 3) issue_f(z + 3);
        }
        cp_async_commit();
        // P_f plane z + 2 is first read here (a late copy only spoils values:
        // the uniform exit below comes before anything is stored)
        if (tile_tma_f) late |= !mbar_wait(fbar(z + 2), fphase(z + 2));
        if constexpr (PAIR) build_pair(z + 1, pslot(z + 1), fnext2);
        else build_plane(z + 1, pslot(z + 1), fnext);
        if constexpr (TMA) {
            // g of plane z: stage j & 1, its (j >> 1)-th use (cp.async tiles
            // were complete at the barrier above)
            if (g_tma) late |= !mbar_wait(&mbar[j & 1], (unsigned)(j >> 1) & 1u);
            if (__syncthreads_or(late)) {
                if (tid == 0) atomicOr(P.err, 1);
                // copies still in flight: wait for them (bounded) before leaving
                if (g_tma && j + 1 < nzc) mbar_wait(&mbar[(j + 1) & 1], (unsigned)((j + 1) >> 1) & 1u);
                if (kAhead >= 3 && tile_tma_f && j + 1 < nzc) mbar_wait(fbar(z + 3), fphase(z + 3));
                return;
            }
        } else {
            __syncthreads();
        }
        // with 3 P_f stages plane z + 3 goes into plane z's stage, free now
        // that every thread has built phi of z + 1
        if (kAhead < 3) {
            if (j + 1 < nzc) issue_f(z + 3);
            cp_async_commit();
        }

        const float *S0 = PHI + pslot(z - 1) * (RH * RW);   // plane z - 1
        const float *S1 = PHI + pslot(z) * (RH * RW);       // plane z
        const float *S2 = PHI + pslot(z + 1) * (RH * RW);   // plane z + 1
        if constexpr (!PAIR) {
        const int lx = tx + 1, ly = ty + 1;
        auto at = [&](const float *S, int yy, int xx) { return S[yy * RW + xx]; };

        // 19-point stencil, src/collision_f.cu:61-94 (e/w = x+-1, n/s = y+-1,
        // t/b = z+-1)
        const float pc = at(S1, ly, lx);
        const float pe = at(S1, ly, lx + 1), pw = at(S1, ly, lx - 1);
        const float pn = at(S1, ly + 1, lx), ps = at(S1, ly - 1, lx);
        const float pt = at(S2, ly, lx), pb = at(S0, ly, lx);
        const float pen = at(S1, ly + 1, lx + 1), pws = at(S1, ly - 1, lx - 1);
        const float pes = at(S1, ly - 1, lx + 1), pwn = at(S1, ly + 1, lx - 1);
        const float pet = at(S2, ly, lx + 1), pwb = at(S0, ly, lx - 1);
        const float peb = at(S0, ly, lx + 1), pwt = at(S2, ly, lx - 1);
        const float pnt = at(S2, ly + 1, lx), psb = at(S0, ly - 1, lx);
        const float pnb = at(S0, ly + 1, lx), pst = at(S2, ly - 1, lx);

        const float lap = (pen + pws + pes + pwn + pet + pwb + peb + pwt + pnt + psb + pnb + pst
                           + 2.f * (pe + pw + pn + ps + pt + pb - 12.f * pc)) * kInv6;
        const float mu = c.alpha4 * pc * (pc * pc - c.phiStarSq) - c.kappa * lap;
        // the edge differences each gradient component shares with another
        const float d_en = pen - pws, d_es = pes - pwn, d_et = pet - pwb, d_eb = peb - pwt;
        const float d_nt = pnt - psb, d_nb = pnb - pst;
        const float mu12 = mu * kInv12;
        const float Fx = mu12 * (2.f * (pe - pw) + d_en + d_es + d_et + d_eb);
        const float Fy = mu12 * (2.f * (pn - ps) + d_en - d_es + d_nt + d_nb);
        float Fz = mu12 * (2.f * (pt - pb) + d_et - d_eb + d_nt - d_nb);
        if (pc > 0.f) Fz += c.grav;

        // D3Q19 values of this node from the staged rows (AA pattern), in
        // stored units
        const ST *Gs = G + (j & 1) * G_ELEMS;
        float g[kQg];
#pragma unroll
        for (int i = 0; i < kQg; i++)
            g[i] = Fm::load((TMA && !ODD) ? Gs[(i * TY + ty) * TX + tx]
                            : Gs[(i * TY + ty) * GW + (!ODD || kCx(i) > 0 ? E : GX0) + tx - (ODD ? kCx(i) : 0)]);

        // moments: src/update_rho.cu:46-50, src/update_velocity.cu:47-59
        float rho = g[0];
#pragma unroll
        for (int i = 1; i < kQg; i++) rho += g[i];
        if constexpr (Fm::kMapped) rho = fmaf(m.g_inv, rho, m.rho_shift);
        const float invRho = 1.0f / rho;
        float invRhoG = invRho;   // 1 / rho on physical momentum differences
        if constexpr (Fm::kMapped) invRhoG = invRho * m.g_inv;
        // momentum from the pair differences each component shares
        const float d7 = g[7] - g[8], d9 = g[9] - g[10], d11 = g[11] - g[12], d13 = g[13] - g[14];
        const float d15 = g[15] - g[16], d17 = g[17] - g[18];
        const float ux = ((g[1] - g[2]) + d7 + d9 + d11 + d13) * invRhoG;
        const float uy = ((g[3] - g[4]) + d7 - d9 + d15 + d17) * invRhoG;
        const float uz = ((g[5] - g[6]) + d11 - d13 + d15 - d17) * invRhoG;
        const unsigned id = node_index(b, x, y, z);   // moment fields
        const unsigned idf = id + (zg ? 2u * (unsigned)b.nxy : 0u), idg = id + (zg ? (unsigned)b.nxy : 0u);
        if (write_moments && in_field(id, 1, b.n, P.err)) {
            P.mom[0][id] = pc;
            P.mom[1][id] = rho;
            P.mom[2][id] = ux;
            P.mom[3][id] = uy;
            P.mom[4][id] = uz;
        }

        // force-shifted velocity, src/collision_f.cu:100-102
        const float usx = ux + 0.5f * Fx * invRho;
        const float usy = uy + 0.5f * Fy * invRho;
        const float usz = uz + 0.5f * Fz * invRho;

        // D3Q7 collision, src/collision_f.cu:105-114 (A/B store)
        {
            const float Af = 0.5f * c.Gamma * c.invTauPhi * mu;
            const float a = c.invTauPhiOne;
            if (in_field(idf, 1, nf, P.err)) P.f0out[idf] = a * fcur[0][0] - 6.0f * Af + c.invTauPhi * pc;
            // f_1..f_6 in stored units: terms scaled by f_scale
            const float Afk = Fm::kMapped ? m.Af * mu : Af;
            const float Cf = (Fm::kMapped ? m.Cf : c.invTauPhi * c.invEta2) * pc;
            auto put = [&](int k, float v) {
                if (in_field(idf, 1, nf, P.err)) P.fout[k][idf] = Fm::store(v);
            };
            put(0, a * fcur[0][1] + Afk + Cf * usx);
            put(1, a * fcur[0][2] + Afk - Cf * usx);
            put(2, a * fcur[0][3] + Afk + Cf * usy);
            put(3, a * fcur[0][4] + Afk - Cf * usy);
            put(4, a * fcur[0][5] + Afk + Cf * usz);
            put(5, a * fcur[0][6] + Afk - Cf * usz);
        }

        // D3Q19 collision with forcing, src/collision_g.cu:111-196; in stored
        // units for 16-bit storage (StepMap)
        {
            constexpr bool M = Fm::kMapped;
            const float bb = c.invTauRhoOne;
            const float K1 = M ? m.K1 : c.K1, K2 = M ? m.K2 : c.K2, KC1 = M ? m.KC1 : c.KC1, KC2 = M ? m.KC2 : c.KC2;
            const float phimu3 = 3.f * pc * mu;
            const float temp1 = K1 * (phimu3 + rho * (1.f - 1.5f * (usx * usx + usy * usy + usz * usz)));
            const float UF = usx * Fx + usy * Fy + usz * Fz;
            const float vx = usx * 3.f, vy = usy * 3.f, vz = usz * 3.f;
            const float vsq6 = (vx * vx + vy * vy + vz * vz) * kInv6;
            float qv[kQg];
            qv[0] = bb * g[0] + (M ? m.K0 : c.K0) * (rho - 6.f * pc * mu - rho * vsq6) - (M ? m.KC0 : c.KC0) * UF;
            if constexpr (M) qv[0] += m.k0;
#if ZSC_PACKED
            {
                // two +- direction pairs per packed (f32x2) evaluation:
                //   eq1 = t + hKr w^2 + KC w G,  qv(+-) = bb g(+-) + (eq1 +- eq2)
                const float2 bb2 = make_float2(bb, bb), neg = make_float2(-1.f, -1.f), pm = make_float2(1.f, -1.f);
                auto quad = [&](float2 W, float2 G, float2 E2, float t, float hKr, float KC, int p1, int m1, int p2,
                                int m2) {
                    const float2 WG = __fmul2_rn(W, G), WW = __fmul2_rn(W, W);
                    float2 E1 = __ffma2_rn(make_float2(hKr, hKr), WW, make_float2(t, t));
                    E1 = __ffma2_rn(make_float2(KC, KC), WG, E1);
                    const float2 P = __fadd2_rn(E1, E2), Mn = __ffma2_rn(E2, neg, E1);
                    const float2 QP = __ffma2_rn(bb2, make_float2(g[p1], g[p2]), P);
                    const float2 QM = __ffma2_rn(bb2, make_float2(g[m1], g[m2]), Mn);
                    qv[p1] = QP.x;
                    qv[p2] = QP.y;
                    qv[m1] = QM.x;
                    qv[m2] = QM.y;
                };
                const float K1r = K1 * rho, hK1r = 0.5f * K1r;
                float t1 = temp1 - KC1 * UF;
                if constexpr (M) t1 += m.k1;
                {
                    // faces x and y packed, eq2 = w (K1r + KC1 G)
                    const float2 W = make_float2(vx, vy), G = make_float2(Fx, Fy);
                    const float2 E2 = __fmul2_rn(W, __ffma2_rn(make_float2(KC1, KC1), G, make_float2(K1r, K1r)));
                    quad(W, G, E2, t1, hK1r, KC1, 1, 2, 3, 4);
                }
                {
                    const float eq1 = t1 + hK1r * vz * vz + KC1 * (vz * Fz);
                    const float eq2 = vz * (K1r + KC1 * Fz);
                    qv[5] = bb * g[5] + eq1 + eq2;
                    qv[6] = bb * g[6] + eq1 - eq2;
                }
                const float K2r = K2 * rho, hK2r = 0.5f * K2r;
                float t2 = K2 * (phimu3 + rho * (1.f - vsq6)) - KC2 * UF;
                if constexpr (M) t2 += m.k2;
                // edges (a + b, a - b) packed, eq2 = K2r w + KC2 G
                auto edges = [&](float va, float vb, float Fa, float Fb, int p1, int m1, int p2, int m2) {
                    const float2 W = __ffma2_rn(make_float2(vb, vb), pm, make_float2(va, va));
                    const float2 G = __ffma2_rn(make_float2(Fb, Fb), pm, make_float2(Fa, Fa));
                    const float2 E2 = __ffma2_rn(make_float2(K2r, K2r), W, __fmul2_rn(make_float2(KC2, KC2), G));
                    quad(W, G, E2, t2, hK2r, KC2, p1, m1, p2, m2);
                };
                edges(vx, vy, Fx, Fy, 7, 8, 9, 10);
                edges(vx, vz, Fx, Fz, 11, 12, 13, 14);
                edges(vy, vz, Fy, Fz, 15, 16, 17, 18);
            }
#else
            {
                const float K1r = K1 * rho, hK1r = 0.5f * K1r;
                float t1 = temp1 - KC1 * UF;
                if constexpr (M) t1 += m.k1;
                float eq1 = t1 + hK1r * vx * vx + KC1 * (vx * Fx);
                float eq2 = vx * (K1r + KC1 * Fx);
                qv[1] = bb * g[1] + eq1 + eq2;
                qv[2] = bb * g[2] + eq1 - eq2;
                eq1 = t1 + hK1r * vy * vy + KC1 * (vy * Fy);
                eq2 = vy * (K1r + KC1 * Fy);
                qv[3] = bb * g[3] + eq1 + eq2;
                qv[4] = bb * g[4] + eq1 - eq2;
                eq1 = t1 + hK1r * vz * vz + KC1 * (vz * Fz);
                eq2 = vz * (K1r + KC1 * Fz);
                qv[5] = bb * g[5] + eq1 + eq2;
                qv[6] = bb * g[6] + eq1 - eq2;
            }
            {
                const float K2r = K2 * rho, hK2r = 0.5f * K2r;
                float t2 = K2 * (phimu3 + rho * (1.f - vsq6)) - KC2 * UF;
                if constexpr (M) t2 += m.k2;
                auto pair = [&](float w, float Gf, int ip, int im) {
                    const float eq1 = t2 + hK2r * w * w + KC2 * (w * Gf);
                    const float eq2 = K2r * w + KC2 * Gf;
                    qv[ip] = bb * g[ip] + eq1 + eq2;
                    qv[im] = bb * g[im] + eq1 - eq2;
                };
                pair(vx + vy, Fx + Fy, 7, 8);
                pair(vx - vy, Fx - Fy, 9, 10);
                pair(vx + vz, Fx + Fz, 11, 12);
                pair(vx - vz, Fx - Fz, 13, 14);
                pair(vy + vz, Fy + Fz, 15, 16);
                pair(vy - vz, Fy - Fz, 17, 18);
            }
#endif
            auto enc = [&](int, float v) -> ST { return Fm::store(v); };
            if (!ODD) {
                // even: own node, reversed slots
#pragma unroll
                for (int i = 0; i < kQg; i++)
                    if (in_field(idg, 1, ng, P.err)) P.g[kOpp(i)][idg] = enc(i, qv[i]);
            } else {
                // odd: downstream neighbour x + c_i, natural slot i (in a
                // z-slab the planes just outside it are ghost planes)
                const int o_zm = (z == 0 && !zg) ? (b.nz - 1) * (int)b.nxy : -(int)b.nxy;
                const int o_zp = (z == b.nz - 1 && !zg) ? -(b.nz - 1) * (int)b.nxy : (int)b.nxy;
                auto off = [&](int i) {
                    return (kCx(i) > 0 ? o_xp : kCx(i) < 0 ? o_xm : 0) + (kCy(i) > 0 ? o_yp : kCy(i) < 0 ? o_ym : 0)
                           + (kCz(i) > 0 ? o_zp : kCz(i) < 0 ? o_zm : 0);
                };
#pragma unroll
                for (int i = 0; i < kQg; i++)
                    if (in_field((long long)idg + off(i), 1, ng, P.err)) P.g[i][idg + off(i)] = enc(i, qv[i]);
            }
        }

        } else {
            // Two nodes per thread, the two of one pair-layout word w = x0/2 + tx:
            // A = (w, y, z) in the .x lanes, B = (w + nx/2, y, z) in the .y lanes of
            // packed FP32; 16-bit storage only, so g and f_1..f_6 are in stored
            // units (StepMap) and each store writes both nodes.  Their x
            // neighbours are the neighbouring words' nodes, so every stencil point
            // is one float2 of the phi ring.
            using namespace pk;
            const float2 *Q0 = reinterpret_cast<const float2 *>(PHI) + pslot(z - 1) * (RH * RWP);   // plane z - 1
            const float2 *Q1 = reinterpret_cast<const float2 *>(PHI) + pslot(z) * (RH * RWP);       // plane z
            const float2 *Q2 = reinterpret_cast<const float2 *>(PHI) + pslot(z + 1) * (RH * RWP);   // plane z + 1
            const int lx = tx + 1, ly = ty + 1;
            auto at = [&](const float2 *S, int yy, int xx) { return S[yy * RWP + xx]; };
            const float2 pc = at(Q1, ly, lx);
            const float2 pe = at(Q1, ly, lx + 1), pw = at(Q1, ly, lx - 1);
            const float2 pn = at(Q1, ly + 1, lx), ps = at(Q1, ly - 1, lx);
            const float2 pt = at(Q2, ly, lx), pb = at(Q0, ly, lx);
            const float2 pen = at(Q1, ly + 1, lx + 1), pws = at(Q1, ly - 1, lx - 1);
            const float2 pes = at(Q1, ly - 1, lx + 1), pwn = at(Q1, ly + 1, lx - 1);
            const float2 pet = at(Q2, ly, lx + 1), pwb = at(Q0, ly, lx - 1);
            const float2 peb = at(Q0, ly, lx + 1), pwt = at(Q2, ly, lx - 1);
            const float2 pnt = at(Q2, ly + 1, lx), psb = at(Q0, ly - 1, lx);
            const float2 pnb = at(Q0, ly + 1, lx), pst = at(Q2, ly - 1, lx);

            float2 se = add(add(add(pen, pws), add(pes, pwn)), add(add(pet, pwb), add(peb, pwt)));
            se = add(se, add(add(pnt, psb), add(pnb, pst)));
            const float2 sf = add(add(add(pe, pw), add(pn, ps)), add(pt, pb));
            const float2 lap = mul(fma(splat(2.f), fma(splat(-12.f), pc, sf), se), splat(kInv6));
            const float2 mu =
                fma(splat(-c.kappa), lap, mul(mul(splat(c.alpha4), pc), add(mul(pc, pc), splat(-c.phiStarSq))));
            const float2 d_en = sub(pen, pws), d_es = sub(pes, pwn), d_et = sub(pet, pwb), d_eb = sub(peb, pwt);
            const float2 d_nt = sub(pnt, psb), d_nb = sub(pnb, pst);
            const float2 mu12 = mul(mu, splat(kInv12));
            const float2 Fx = mul(mu12, add(add(fma(splat(2.f), sub(pe, pw), d_en), add(d_es, d_et)), d_eb));
            const float2 Fy = mul(mu12, add(add(fma(splat(2.f), sub(pn, ps), d_en), sub(d_nt, d_es)), d_nb));
            float2 Fz = mul(mu12, sub(add(fma(splat(2.f), sub(pt, pb), d_et), sub(d_nt, d_eb)), d_nb));
            if (pc.x > 0.f) Fz.x += c.grav;
            if (pc.y > 0.f) Fz.y += c.grav;

            // D3Q19 values of both nodes from the staged rows (AA pattern); an
            // odd step's x-shifted direction reads the neighbouring word, which
            // came round the x seam (swapped) for the first / last word of a
            // seam tile
            const ST *Gs = G + (j & 1) * G_ELEMS;
            const bool wrap_l = seam_l && tx == 0, wrap_r = seam_r && tx == TXW - 1;
            const unsigned sel_l = wrap_l ? kSwap : kKeep, sel_r = wrap_r ? kSwap : kKeep;
            float2 g[kQg];
#pragma unroll
            for (int i = 0; i < kQg; i++) {
                if (TMA && !ODD) {
                    g[i] = Fm::load2(*reinterpret_cast<const T2 *>(Gs + (i * TY + ty) * TX + 2 * tx));
                } else if (!ODD) {
                    g[i] = Fm::load2(*reinterpret_cast<const T2 *>(Gs + (i * TY + ty) * GW + E + 2 * tx));
                } else if (kCx(i) == 0) {
                    g[i] = Fm::load2(*reinterpret_cast<const T2 *>(Gs + (i * TY + ty) * GW + GX0 + 2 * tx));
                } else {
                    const T2 v = *reinterpret_cast<const T2 *>(Gs + (i * TY + ty) * GW + (kCx(i) > 0 ? E : GX0) + 2 * tx
                                                               - 2 * kCx(i));
                    g[i] = Fm::load2(Fm::perm2(v, kCx(i) > 0 ? sel_l : sel_r));
                }
            }

            // moments (stored units: rho = g_inv sum + sum of shifts)
            float2 rho = g[0];
#pragma unroll
            for (int i = 1; i < kQg; i++) rho = add(rho, g[i]);
            rho = fma(splat(m.g_inv), rho, splat(m.rho_shift));
            const float2 invRho = make_float2(1.0f / rho.x, 1.0f / rho.y);
            const float2 invRhoG = mul(invRho, splat(m.g_inv));
            const float2 d7 = sub(g[7], g[8]), d9 = sub(g[9], g[10]), d11 = sub(g[11], g[12]);
            const float2 d13 = sub(g[13], g[14]), d15 = sub(g[15], g[16]), d17 = sub(g[17], g[18]);
            const float2 ux = mul(add(add(add(add(sub(g[1], g[2]), d7), d9), d11), d13), invRhoG);
            const float2 uy = mul(add(add(sub(add(sub(g[3], g[4]), d7), d9), d15), d17), invRhoG);
            const float2 uz = mul(sub(add(sub(add(sub(g[5], g[6]), d11), d13), d15), d17), invRhoG);
            // element index of the word (its A half) in every pair-layout field
            const unsigned id = node_index(b, x, y, z);
            const unsigned idf = id + (zg ? 2u * (unsigned)b.nxy : 0u), idg = id + (zg ? (unsigned)b.nxy : 0u);
            const int half = b.nx / 2;
            if (write_moments) {
                // the moment fields are in the natural layout: A and B apart
                const unsigned ia = node_index(b, x0 / 2 + tx, y, z), ib = ia + (unsigned)half;
                const float2 mv[5] = {pc, rho, ux, uy, uz};
#pragma unroll
                for (int k = 0; k < 5; k++) {
                    if (in_field(ia, 1, b.n, P.err)) P.mom[k][ia] = mv[k].x;
                    if (in_field(ib, 1, b.n, P.err)) P.mom[k][ib] = mv[k].y;
                }
            }
            const float2 hinv = mul(splat(0.5f), invRho);
            const float2 usx = fma(Fx, hinv, ux), usy = fma(Fy, hinv, uy), usz = fma(Fz, hinv, uz);

            // D3Q7 collision (A/B store), f_1..f_6 in stored units
            {
                const float2 a2 = splat(c.invTauPhiOne);
                auto fc = [&](int k) { return fcur2[k]; };
                const float2 Af = mul(splat(0.5f * c.Gamma * c.invTauPhi), mu);
                if (in_field(idf, 2, nf, P.err))
                    *reinterpret_cast<float2 *>(P.f0out + idf) =
                        fma(a2, fc(0), fma(splat(-6.f), Af, mul(splat(c.invTauPhi), pc)));
                const float2 Afk = mul(splat(m.Af), mu), Cf = mul(splat(m.Cf), pc);
                const float2 cux = mul(Cf, usx), cuy = mul(Cf, usy), cuz = mul(Cf, usz);
                auto put2 = [&](int k, float2 v) {
                    if (in_field(idf, 2, nf, P.err)) *reinterpret_cast<T2 *>(P.fout[k] + idf) = Fm::store2(v);
                };
                put2(0, fma(a2, fc(1), add(Afk, cux)));
                put2(1, fma(a2, fc(2), sub(Afk, cux)));
                put2(2, fma(a2, fc(3), add(Afk, cuy)));
                put2(3, fma(a2, fc(4), sub(Afk, cuy)));
                put2(4, fma(a2, fc(5), add(Afk, cuz)));
                put2(5, fma(a2, fc(6), sub(Afk, cuz)));
            }

            // D3Q19 collision with forcing (the one-node formulas, StepMap constants)
            {
                const float2 bb = splat(c.invTauRhoOne);
                const float2 phimu3 = mul(mul(splat(3.f), pc), mu);
                const float2 usq = fma(usx, usx, fma(usy, usy, mul(usz, usz)));
                const float2 temp1 = mul(splat(m.K1), fma(rho, fma(splat(-1.5f), usq, splat(1.f)), phimu3));
                const float2 UF = fma(usx, Fx, fma(usy, Fy, mul(usz, Fz)));
                const float2 vx = mul(usx, splat(3.f)), vy = mul(usy, splat(3.f)), vz = mul(usz, splat(3.f));
                const float2 vsq6 = mul(fma(vx, vx, fma(vy, vy, mul(vz, vz))), splat(kInv6));
                float2 qv[kQg];
                qv[0] = fma(bb, g[0],
                            fma(splat(m.K0), sub(fma(splat(-6.f), mul(pc, mu), rho), mul(rho, vsq6)),
                                fma(splat(-m.KC0), UF, splat(m.k0))));
                const float2 K1r = mul(splat(m.K1), rho), hK1r = mul(splat(0.5f), K1r);
                const float2 t1 = fma(splat(-m.KC1), UF, add(temp1, splat(m.k1)));
                auto face = [&](float2 w, float2 Gf, int ip, int im) {
                    const float2 eq1 = fma(splat(m.KC1), mul(w, Gf), fma(mul(hK1r, w), w, t1));
                    const float2 eq2 = mul(w, fma(splat(m.KC1), Gf, K1r));
                    qv[ip] = add(fma(bb, g[ip], eq1), eq2);
                    qv[im] = sub(fma(bb, g[im], eq1), eq2);
                };
                face(vx, Fx, 1, 2);
                face(vy, Fy, 3, 4);
                face(vz, Fz, 5, 6);
                const float2 K2r = mul(splat(m.K2), rho), hK2r = mul(splat(0.5f), K2r);
                const float2 t2 =
                    fma(splat(-m.KC2), UF, fma(splat(m.K2), fma(rho, sub(splat(1.f), vsq6), phimu3), splat(m.k2)));
                auto edge = [&](float2 w, float2 Gf, int ip, int im) {
                    const float2 eq1 = fma(splat(m.KC2), mul(w, Gf), fma(mul(hK2r, w), w, t2));
                    const float2 eq2 = fma(K2r, w, mul(splat(m.KC2), Gf));
                    qv[ip] = add(fma(bb, g[ip], eq1), eq2);
                    qv[im] = sub(fma(bb, g[im], eq1), eq2);
                };
                edge(add(vx, vy), add(Fx, Fy), 7, 8);
                edge(sub(vx, vy), sub(Fx, Fy), 9, 10);
                edge(add(vx, vz), add(Fx, Fz), 11, 12);
                edge(sub(vx, vz), sub(Fx, Fz), 13, 14);
                edge(add(vy, vz), add(Fy, Fz), 15, 16);
                edge(sub(vy, vz), sub(Fy, Fz), 17, 18);
                if (!ODD) {
                    // even: own nodes, reversed slots
#pragma unroll
                    for (int i = 0; i < kQg; i++)
                        if (in_field(idg, 2, ng, P.err))
                            *reinterpret_cast<T2 *>(P.g[kOpp(i)] + idg) = Fm::store2(qv[i]);
                } else {
                    // odd: downstream neighbours x + c_i, natural slot i.  Both
                    // nodes of the word move to the neighbouring word together;
                    // past the x seam (word nx/2 - 1 -> 0 and back) the pair
                    // lands swapped.
                    const int o_zm = (z == 0 && !zg) ? (b.nz - 1) * (int)b.nxy : -(int)b.nxy;
                    const int o_zp = (z == b.nz - 1 && !zg) ? -(b.nz - 1) * (int)b.nxy : (int)b.nxy;
                    const int o_wp = wrap_r ? -2 * (half - 1) : 2;   // element offset of word w + 1
                    const int o_wm = wrap_l ? 2 * (half - 1) : -2;   // ... of word w - 1
#pragma unroll
                    for (int i = 0; i < kQg; i++) {
                        const int o = (kCx(i) > 0 ? o_wp : kCx(i) < 0 ? o_wm : 0) +
                                      (kCy(i) > 0 ? o_yp : kCy(i) < 0 ? o_ym : 0) +
                                      (kCz(i) > 0 ? o_zp : kCz(i) < 0 ? o_zm : 0);
                        T2 h = Fm::store2(qv[i]);
                        if (kCx(i) != 0) h = Fm::perm2(h, kCx(i) > 0 ? sel_r : sel_l);
                        if (in_field((long long)idg + o, 2, ng, P.err)) *reinterpret_cast<T2 *>(P.g[i] + idg + o) = h;
                    }
                }
            }
        }

        if constexpr (PAIR) {
#pragma unroll
            for (int i = 0; i < kQf; i++) fcur2[i] = fnext2[i];
        } else {
#pragma unroll
            for (int k = 0; k < XPT; k++)
#pragma unroll
                for (int i = 0; i < kQf; i++) fcur[k][i] = fnext[k][i];
        }
    }
}

template <typename ST, bool S, bool O, bool T, bool Z>
cudaError_t configure()
{
    static bool done = false;   // per template instance, per process
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(zsc_step_kernel<ST, S, O, T, Z>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Geo<ST>::SMEM);
    // all of the unified L1 / shared storage as shared memory: the resident
    // blocks per SM the launch bounds ask for need it
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(zsc_step_kernel<ST, S, O, T, Z>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) done = true;
    return e;
}

// cuTensorMapEncodeTiled from the driver (no link-time dependency on it).
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled tensor_map_encoder()
{
    static const EncodeTiled fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return EncodeTiled(nullptr);
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

template <typename ST>
constexpr CUtensorMapDataType tensor_type()
{
    if constexpr (std::is_same<ST, float>::value) return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    else if constexpr (std::is_same<ST, __half>::value) return CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    else return CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
}

// The 19 g arrays at g (n elements each) as one 4-d tensor (x, y, z, field),
// read in boxes of one plane's tile in all fields (32 x 8 x 1 x 19, the even
// step).  Strides are multiples of 16 bytes (nx is a multiple of 32); the base
// must be 16-byte aligned (a cudaMalloc pointer, or a checkpoint slot offset by
// whole fields).
template <typename ST>
bool encode_g_map(const Box &b, const ST *g, CUtensorMap *map)
{
    const EncodeTiled encode = tensor_map_encoder();
    if (!encode) return false;
    const cuuint64_t es = sizeof(ST);
    const cuuint64_t dims[4] = {(cuuint64_t)b.nx, (cuuint64_t)b.ny, (cuuint64_t)(b.ng / b.nxy), (cuuint64_t)kQg};
    const cuuint64_t strides[3] = {(cuuint64_t)b.nx * es, (cuuint64_t)b.nxy * es, (cuuint64_t)b.ng * es};
    const cuuint32_t box[4] = {(cuuint32_t)TX, (cuuint32_t)TY, 1u, (cuuint32_t)kQg};
    const cuuint32_t elem[4] = {1u, 1u, 1u, 1u};
    if ((reinterpret_cast<uintptr_t>(g) & 15u) != 0) return false;
    return encode(map, tensor_type<ST>(), 4, const_cast<ST *>(g), dims, strides, box, elem,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The P_f planes: f_0 (FP32) as a 3-d tensor read in W0 x FR boxes, f_1..f_6
// (six consecutive arrays) as a 4-d tensor (x, y, z, field) read in
// W x FR x 1 x 6 boxes, both from x0 - 4 / x0 - E and y0 - 2.
template <typename ST>
bool encode_f_maps(const Box &b, const float *f0, const ST *fq, CUtensorMap *f0map, CUtensorMap *fqmap)
{
    const EncodeTiled encode = tensor_map_encoder();
    if (!encode) return false;
    if ((reinterpret_cast<uintptr_t>(f0) & 15u) != 0 || (reinterpret_cast<uintptr_t>(fq) & 15u) != 0) return false;
    const cuuint32_t elem[4] = {1u, 1u, 1u, 1u};
    const cuuint64_t dims0[3] = {(cuuint64_t)b.nx, (cuuint64_t)b.ny, (cuuint64_t)(b.nf / b.nxy)};
    const cuuint64_t strides0[2] = {(cuuint64_t)b.nx * 4, (cuuint64_t)b.nxy * 4};
    const cuuint32_t box0[3] = {(cuuint32_t)W0, (cuuint32_t)FR, 1u};
    if (encode(f0map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(f0), dims0, strides0, box0, elem,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const cuuint64_t es = sizeof(ST);
    const cuuint64_t dims[4] = {(cuuint64_t)b.nx, (cuuint64_t)b.ny, (cuuint64_t)(b.nf / b.nxy), (cuuint64_t)(kQf - 1)};
    const cuuint64_t strides[3] = {(cuuint64_t)b.nx * es, (cuuint64_t)b.nxy * es, (cuuint64_t)b.nf * es};
    const cuuint32_t box[4] = {(cuuint32_t)Geo<ST>::W, (cuuint32_t)FR, 1u, (cuuint32_t)(kQf - 1)};
    return encode(fqmap, tensor_type<ST>(), 4, const_cast<ST *>(fq), dims, strides, box, elem,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Planes per block.  The blocks of one launch all march the same number of
// planes, so the step takes about ceil(blocks / resident slots) "waves" of
// (tz + prologue) planes; pick the chunk depth that minimises that product
// (e.g. 256^3 FP32: 37 planes -> 1792 blocks = 5.9 waves of 304 slots, instead
// of 32 planes -> 6.7 waves with a 74%-full last wave).
template <typename ST>
int choose_tz(const Box &b)
{
    static int slots = 0;   // per storage type, per process
    if (slots == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zsc_step_kernel<ST, false, false, false, false>,
                                                      threads_of<ST>(), Geo<ST>::SMEM);
        slots = sms * per_sm > 0 ? sms * per_sm : 1;
    }
    const long long tiles = (long long)(b.nx / TX) * (b.ny / TY);
    constexpr int kPrologue = 3;   // extra planes each block stages and rebuilds
    int best = 32;
    long long best_cost = -1;
    for (int tz = 4; tz <= 64; tz++) {
        const long long chunks = (b.nz + tz - 1) / tz;
        const long long waves = (tiles * chunks + slots - 1) / slots;
        const long long cost = waves * (tz + kPrologue);
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = tz;
        }
    }
    return best;
}

// A step launch with programmatic stream serialization (the kernel orders
// itself after the previous grid with griddepcontrol.wait).
template <typename... KArgs, typename... Args>
cudaError_t launch_step_kernel(void (*kernel)(KArgs...), unsigned nblocks, dim3 block, int smem, cudaStream_t s,
                               Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nblocks, 1, 1);
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = ZSC_PDL ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <typename ST, bool ZG>
cudaError_t launch_typed(const Box &b, const StepConst &c, const Quant &q, const StepView &v, bool f_streamed,
                         bool odd, bool write_moments, cudaStream_t s, int zlo, int zhi)
{
    const StepMap m = step_map(c, q);
    StepPtrs<ST> P;
    P.f0in = v.f0_in;
    P.f0out = v.f0_out;
    const ST *fin = static_cast<const ST *>(v.fq_in);
    ST *fout = static_cast<ST *>(v.fq_out);
    ST *g = static_cast<ST *>(v.g);
    const ST *gin = static_cast<const ST *>(v.g_in ? v.g_in : v.g);
    for (int a = 0; a < kQf - 1; a++) {
        P.fin[a] = fin + (size_t)a * b.nf;
        P.fout[a] = fout + (size_t)a * b.nf;
    }
    for (int i = 0; i < kQg; i++) {
        P.gin[i] = gin + (size_t)i * b.ng;
        P.g[i] = g + (size_t)i * b.ng;
    }
    for (int i = 0; i < 5; i++) P.mom[i] = v.mom + (size_t)i * b.n;
    P.err = v.err;
    cudaError_t e = configure<ST, true, false, false, ZG>();
    if (e == cudaSuccess) e = configure<ST, false, true, false, ZG>();
    if (e == cudaSuccess) e = configure<ST, false, false, false, ZG>();
    if (e == cudaSuccess) e = configure<ST, true, false, true, ZG>();
    if (e == cudaSuccess) e = configure<ST, false, false, true, ZG>();
    if (e == cudaSuccess) e = configure<ST, false, true, true, ZG>();
    if (e != cudaSuccess) return e;
    // staging by TMA when the driver encodes every map the step needs: the g
    // tile (even steps) and the P_f planes (if enabled)
    CUtensorMap gmap, f0map, fqmap;
    std::memset(&gmap, 0, sizeof(gmap));
    std::memset(&f0map, 0, sizeof(f0map));
    std::memset(&fqmap, 0, sizeof(fqmap));
    const bool need_g = !odd;
    bool tma = kUseTma && (need_g || use_tma_f<ST>());
    if (tma && need_g) tma = encode_g_map<ST>(b, gin, &gmap);
    if (tma && use_tma_f<ST>()) tma = encode_f_maps<ST>(b, P.f0in, fin, &f0map, &fqmap);
    Box range = b;   // the chunk depth for the planes this launch covers
    range.nz = zhi - zlo;
    const int tz = choose_tz<ST>(range);
    const int nchunks = (range.nz + tz - 1) / tz;
    const unsigned nblocks = (unsigned)((b.nx / TX) * (b.ny / TY) * nchunks);
    const dim3 block(TX / (use_pair<ST>() ? 2 : 1), TY, 1);
    const int wm = write_moments ? 1 : 0;
    constexpr int smem = Geo<ST>::SMEM;
    const StepBox kb{b.nx, b.ny, b.nz, b.nxy, b.n};
    auto go = [&](auto kernel) {
        return launch_step_kernel(kernel, nblocks, block, smem, s, P, kb, c, m, tz, wm, zlo, zhi, gmap, f0map,
                                  fqmap);
    };
    if (f_streamed) {
        if (odd) return cudaErrorInvalidValue;  // the streamed initial state is always read by an even step
        return tma ? go(zsc_step_kernel<ST, true, false, true, ZG>) : go(zsc_step_kernel<ST, true, false, false, ZG>);
    }
    if (odd)
        return tma ? go(zsc_step_kernel<ST, false, true, true, ZG>) : go(zsc_step_kernel<ST, false, true, false, ZG>);
    return tma ? go(zsc_step_kernel<ST, false, false, true, ZG>) : go(zsc_step_kernel<ST, false, false, false, ZG>);
}

template <typename ST>
cudaError_t launch_typed(const Box &b, const StepConst &c, const Quant &q, const StepView &v, bool f_streamed,
                         bool odd, bool write_moments, cudaStream_t s, int zlo, int zhi)
{
    if (b.zghost) return launch_typed<ST, true>(b, c, q, v, f_streamed, odd, write_moments, s, zlo, zhi);
    return launch_typed<ST, false>(b, c, q, v, f_streamed, odd, write_moments, s, 0, b.nz);
}

}  // namespace

cudaError_t launch_wait_selftest(int *err, cudaStream_t s)
{
    wait_selftest_kernel<<<1, 32, 0, s>>>(err, 64);
    return cudaGetLastError();
}

cudaError_t launch_step(const Box &b, const StepConst &c, const Quant &q, const StepView &v, bool f_streamed,
                        bool odd, bool write_moments, cudaStream_t s, int zlo, int zhi)
{
    if (b.nx % TX != 0 || b.ny % TY != 0) return cudaErrorInvalidValue;
    if (zhi < 0) zhi = b.nz;
    // a periodic box steps whole; a z-slab any nonempty range of its planes
    if (zlo < 0 || zhi > b.nz || zlo >= zhi || (!b.zghost && (zlo != 0 || zhi != b.nz)))
        return cudaErrorInvalidValue;
    switch (v.storage) {
    case LBM_STORAGE_FP32: return launch_typed<float>(b, c, q, v, f_streamed, odd, write_moments, s, zlo, zhi);
    case LBM_STORAGE_FP16: return launch_typed<__half>(b, c, q, v, f_streamed, odd, write_moments, s, zlo, zhi);
    case LBM_STORAGE_BF16:
        return launch_typed<__nv_bfloat16>(b, c, q, v, f_streamed, odd, write_moments, s, zlo, zhi);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace lbm
