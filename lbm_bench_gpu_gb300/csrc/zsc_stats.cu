// zsc_stats.cu -- statistics of the phi, rho, u arrays in FP64.
//
// Replaces the host loops of src/stats.c:39-58 and the pressure part of
// src/logsave.c:63-150.  One pass over the five arrays: per-thread
// compensated float sums (a float pair hi + lo updated with Knuth's two-sum,
// products split exactly with an FMA), which hold ~48 bits like an FP64 sum
// at FP32 throughput (GB300's FP64 rate is a small fraction of its FP32 rate);
// FP64 warp-shuffle reductions per block into a partials array, then one block
// folds the partials in a fixed order (deterministic for a given box).
//
// Partial / result layout (doubles):
//   0 max |u|^2 (compat)    1 #phi>=0 (compat)   2..4 sum u over phi>=0 (compat)
//   5 sum p over phi>=0     6 sum p over phi<0 (compat)
//   7 sum phi   8 sum rho   9..11 sum rho u   12 #phi>=0   13 max |u|^2
//   14 #non-finite nodes    15 unused
// "compat" skips the planes x = 0, nx-1 and y = 0, ny-1 like the reference.
#include "lbm_internal.h"

namespace lbm {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 152 * 8;
constexpr float kInv6 = 0.16666666666666666667f;
constexpr float kInv12 = 0.08333333333333333333f;

constexpr float kCsSq = 0.33333333333333333333f;   // src/constants.h:48

struct StatsConst {
    float alpha, kappa, phiStarSq;
};

// row index of (y, z)
__device__ __forceinline__ int kk_row(int y, int z, int ny) { return y + ny * z; }

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide reduction of acc[0..kStatsValues) (entries 0 and 13 by max, the
// rest by sum); thread 0 writes the result to out.
__device__ void block_reduce(double (&acc)[kStatsValues], double *out)
{
    __shared__ double red[kThreads / 32][kStatsValues];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v < kStatsValues; v++) {
        const double r = (v == 0 || v == 13) ? warp_max(acc[v]) : warp_sum(acc[v]);
        if (lane == 0) red[warp][v] = r;
    }
    __syncthreads();
    if (threadIdx.x < kStatsValues) {
        const int v = threadIdx.x;
        double r = red[0][v];
        for (int w = 1; w < kThreads / 32; w++) r = (v == 0 || v == 13) ? fmax(r, red[w][v]) : r + red[w][v];
        out[v] = r;
    }
}

// Compensated float accumulator: the sum is hi + lo.  The _rn intrinsics keep
// the compiler from contracting the two-sum's operations into FMAs, which
// would break the exact error terms.
struct Sum2 {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        const float s = __fadd_rn(hi, x);
        const float bp = __fsub_rn(s, hi);
        lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp)));
        hi = s;
    }
    // a * b exactly (the product's rounding error from an FMA)
    __device__ __forceinline__ void add_product(float a, float b)
    {
        const float p = __fmul_rn(a, b);
        add(p);
        lo = __fadd_rn(lo, fmaf(a, b, -p));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// One block works on whole x-rows (row r = y + ny z, grid-stride over rows);
// |u|^2 and the pressure are evaluated in float as the reference does
// (src/stats.c:45, src/logsave.c:94-137); sums are compensated, counts exact.
// phi_lo / phi_hi: the phi planes just below and above a z-slab (NULL for a
// periodic box, whose z neighbours wrap).
__global__ void __launch_bounds__(kThreads) stats_kernel(Box b, StatsConst c, const float *__restrict__ phi,
                                                         const float *__restrict__ rho, const float *__restrict__ ux,
                                                         const float *__restrict__ uy, const float *__restrict__ uz,
                                                         double *__restrict__ partials,
                                                         const float *__restrict__ phi_lo = nullptr,
                                                         const float *__restrict__ phi_hi = nullptr)
{
    Sum2 sum[kStatsValues];
    unsigned cnt_in = 0, cnt_all = 0, cnt_bad = 0;
    float umax_c = 0.f, umax_all = 0.f;

    const int nx = b.nx, ny = b.ny, nz = b.nz;
    const int rows = ny * nz;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int k = r / ny, j = r - k * ny;
        const bool row_in = j >= 1 && j <= ny - 2;   // reference region in y
        const int jn = j == ny - 1 ? 0 : j + 1, js = j == 0 ? ny - 1 : j - 1;
        const int kt = k == nz - 1 ? 0 : k + 1, kb = k == 0 ? nz - 1 : k - 1;
        const size_t row_c = (size_t)r * nx;
        const size_t row_n = ((size_t)kk_row(jn, k, ny)) * nx, row_s = ((size_t)kk_row(js, k, ny)) * nx;
        // the planes above and below: the neighbouring slab's at a slab's edge
        const float *pt = (k == nz - 1 && phi_hi) ? phi_hi : phi + (size_t)kt * b.nxy;
        const float *pb = (k == 0 && phi_lo) ? phi_lo : phi + (size_t)kb * b.nxy;
        const float *rt = pt + (size_t)j * nx, *rb = pb + (size_t)j * nx;
        const float *rnt = pt + (size_t)jn * nx, *rsb = pb + (size_t)js * nx;
        const float *rnb = pb + (size_t)jn * nx, *rst = pt + (size_t)js * nx;
        for (int i = threadIdx.x; i < nx; i += blockDim.x) {
            const size_t t = row_c + i;
            const float ph = phi[t], rh = rho[t], vx = ux[t], vy = uy[t], vz = uz[t];
            if (!(isfinite(ph) && isfinite(rh) && isfinite(vx) && isfinite(vy) && isfinite(vz))) {
                cnt_bad++;
                continue;
            }
            const float u2 = vx * vx + vy * vy + vz * vz;
            sum[7].add(ph);
            sum[8].add(rh);
            sum[9].add_product(rh, vx);
            sum[10].add_product(rh, vy);
            sum[11].add_product(rh, vz);
            if (ph >= 0.f) cnt_all++;
            umax_all = fmaxf(umax_all, u2);
            if (!row_in || i < 1 || i > nx - 2) continue;
            umax_c = fmaxf(umax_c, u2);

            const int ie = i == nx - 1 ? 0 : i + 1, iw = i == 0 ? nx - 1 : i - 1;
            const float p01 = phi[row_c + ie], p02 = phi[row_c + iw], p03 = phi[row_n + i], p04 = phi[row_s + i];
            const float p05 = rt[i], p06 = rb[i], p07 = phi[row_n + ie], p08 = phi[row_s + iw];
            const float p09 = phi[row_s + ie], p10 = phi[row_n + iw], p11 = rt[ie], p12 = rb[iw];
            const float p13 = rb[ie], p14 = rt[iw], p15 = rnt[i], p16 = rsb[i];
            const float p17 = rnb[i], p18 = rst[i];
            const float lap = (p07 + p08 + p09 + p10 + p11 + p12 + p13 + p14 + p15 + p16 + p17 + p18
                               + 2.f * (p01 + p02 + p03 + p04 + p05 + p06 - 12.f * ph)) * kInv6;
            const float gx = (2.f * (p01 - p02) + p07 - p08 + p09 - p10 + p11 - p12 + p13 - p14) * kInv12;
            const float gy = (2.f * (p03 - p04) + p07 - p08 + p10 - p09 + p15 - p16 + p17 - p18) * kInv12;
            const float gz = (2.f * (p05 - p06) + p11 - p12 + p14 - p13 + p15 - p16 + p18 - p17) * kInv12;
            const float ph2 = ph * ph;
            const float pres = c.alpha * (ph2 * (3.f * ph2 - 2.f * c.phiStarSq) - c.phiStarSq * c.phiStarSq)
                               - c.kappa * (ph * lap - 0.5f * (gx * gx + gy * gy + gz * gz)) + kCsSq * rh;
            if (ph >= 0.f) {
                cnt_in++;
                sum[2].add(vx);
                sum[3].add(vy);
                sum[4].add(vz);
                sum[5].add(pres);
            } else {
                sum[6].add(pres);
            }
        }
    }
    double acc[kStatsValues];
#pragma unroll
    for (int v = 0; v < kStatsValues; v++) acc[v] = sum[v].value();
    acc[0] = umax_c;
    acc[1] = cnt_in;
    acc[12] = cnt_all;
    acc[13] = umax_all;
    acc[14] = cnt_bad;
    acc[15] = 0.0;
    block_reduce(acc, partials + (size_t)blockIdx.x * kStatsValues);
}

__global__ void __launch_bounds__(kThreads) fold_kernel(const double *__restrict__ partials, int nparts,
                                                        double *__restrict__ out)
{
    double acc[kStatsValues];
#pragma unroll
    for (int v = 0; v < kStatsValues; v++) acc[v] = 0.0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
#pragma unroll
        for (int v = 0; v < kStatsValues; v++) {
            const double x = partials[(size_t)p * kStatsValues + v];
            acc[v] = (v == 0 || v == 13) ? fmax(acc[v], x) : acc[v] + x;
        }
    }
    block_reduce(acc, out);
}

// Pressure of every node (src/vtksave.c:63-127): the same float expression as
// the stats, periodic neighbours.  One thread per node of a row-major grid.
__global__ void __launch_bounds__(kThreads) pressure_kernel(Box b, StatsConst c, const float *__restrict__ phi,
                                                            const float *__restrict__ rho, float *__restrict__ out)
{
    const int nx = b.nx, ny = b.ny, nz = b.nz;
    const int rows = ny * nz;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int k = r / ny, j = r - k * ny;
        const int jn = j == ny - 1 ? 0 : j + 1, js = j == 0 ? ny - 1 : j - 1;
        const int kt = k == nz - 1 ? 0 : k + 1, kb = k == 0 ? nz - 1 : k - 1;
        const size_t row_c = (size_t)r * nx;
        const size_t row_n = ((size_t)kk_row(jn, k, ny)) * nx, row_s = ((size_t)kk_row(js, k, ny)) * nx;
        const size_t row_t = ((size_t)kk_row(j, kt, ny)) * nx, row_b = ((size_t)kk_row(j, kb, ny)) * nx;
        const size_t row_nt = ((size_t)kk_row(jn, kt, ny)) * nx, row_sb = ((size_t)kk_row(js, kb, ny)) * nx;
        const size_t row_nb = ((size_t)kk_row(jn, kb, ny)) * nx, row_st = ((size_t)kk_row(js, kt, ny)) * nx;
        for (int i = threadIdx.x; i < nx; i += blockDim.x) {
            const size_t t = row_c + i;
            const float ph = phi[t];
            const int ie = i == nx - 1 ? 0 : i + 1, iw = i == 0 ? nx - 1 : i - 1;
            const float p01 = phi[row_c + ie], p02 = phi[row_c + iw], p03 = phi[row_n + i], p04 = phi[row_s + i];
            const float p05 = phi[row_t + i], p06 = phi[row_b + i], p07 = phi[row_n + ie], p08 = phi[row_s + iw];
            const float p09 = phi[row_s + ie], p10 = phi[row_n + iw], p11 = phi[row_t + ie], p12 = phi[row_b + iw];
            const float p13 = phi[row_b + ie], p14 = phi[row_t + iw], p15 = phi[row_nt + i], p16 = phi[row_sb + i];
            const float p17 = phi[row_nb + i], p18 = phi[row_st + i];
            const float lap = (p07 + p08 + p09 + p10 + p11 + p12 + p13 + p14 + p15 + p16 + p17 + p18
                               + 2.f * (p01 + p02 + p03 + p04 + p05 + p06 - 12.f * ph)) * kInv6;
            const float gx = (2.f * (p01 - p02) + p07 - p08 + p09 - p10 + p11 - p12 + p13 - p14) * kInv12;
            const float gy = (2.f * (p03 - p04) + p07 - p08 + p10 - p09 + p15 - p16 + p17 - p18) * kInv12;
            const float gz = (2.f * (p05 - p06) + p11 - p12 + p14 - p13 + p15 - p16 + p18 - p17) * kInv12;
            const float ph2 = ph * ph;
            out[t] = c.alpha * (ph2 * (3.f * ph2 - 2.f * c.phiStarSq) - c.phiStarSq * c.phiStarSq)
                     - c.kappa * (ph * lap - 0.5f * (gx * gx + gy * gy + gz * gz)) + kCsSq * rho[t];
        }
    }
}

unsigned stats_blocks(const Box &b)
{
    long long blocks = (long long)b.ny * b.nz;   // one x-row per block and pass
    if (blocks > kMaxBlocks) blocks = kMaxBlocks;
    return (unsigned)(blocks < 1 ? 1 : blocks);
}

}  // namespace

size_t stats_partial_count(const Box &b) { return stats_blocks(b); }

cudaError_t launch_stats(const Box &b, const lbm_derived &d, const float *mom, double *partials,
                         size_t partial_count, double *result, unsigned long long *, cudaStream_t s,
                         const float *phi_lo, const float *phi_hi)
{
    const unsigned blocks = stats_blocks(b);
    if (partial_count < blocks) return cudaErrorInvalidValue;
    StatsConst c{d.alpha, d.kappa, d.phiStarSq};
    stats_kernel<<<blocks, kThreads, 0, s>>>(b, c, mom, mom + b.n, mom + 2 * b.n, mom + 3 * b.n, mom + 4 * b.n,
                                             partials, phi_lo, phi_hi);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    fold_kernel<<<1, kThreads, 0, s>>>(partials, (int)blocks, result);
    return cudaGetLastError();
}

cudaError_t launch_pressure(const Box &b, const lbm_derived &d, const float *mom, float *out, cudaStream_t s)
{
    StatsConst c{d.alpha, d.kappa, d.phiStarSq};
    long long blocks = (long long)b.ny * b.nz;
    if (blocks > 152 * 16) blocks = 152 * 16;
    pressure_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(b, c, mom, mom + b.n, out);
    return cudaGetLastError();
}

}  // namespace lbm

// ---------------------------------------------------------------------------
// lbm_stats_noalloc: the same reduction for callers that must not allocate
// device memory.
//
// Who needs it: code that inspects the fields of a simulation it does not own
// -- an in-situ analysis or monitoring hook called from inside another
// program's time loop.  There the device memory usually belongs to the host
// application's own pool allocator, and cudaMalloc / cudaFree are off limits:
// they would take memory outside the application's budget and they
// synchronise the whole device, stalling the work already queued.  Such a
// caller hands over the five field arrays and a 16-double output buffer it
// already owns; this entry point adds nothing to them.
//
// The per-block partial sums live in a fixed array in the library's static
// device memory (1 MiB, reserved on every GPU that loads the library until the
// process exits).  One block reduces 16384 nodes, so the array holds the
// partials of at most 512^3 nodes; larger boxes are rejected.  Every row the
// final fold reads is written earlier in the same call, so no part of the
// array has to be cleared between calls.  All calls share the array: two calls
// whose kernels overlap on the GPU (different streams, or different host
// threads on one device) race on it and must be ordered by the caller.
// ---------------------------------------------------------------------------
#include <mutex>

namespace lbm {
namespace {

constexpr int kNoAllocNodesPerBlock = kThreads * 64;
constexpr long long kNoAllocMaxNodes = LBM_NOALLOC_MAX_NODES;
constexpr int kNoAllocRows = (int)(kNoAllocMaxNodes / kNoAllocNodesPerBlock);
static_assert(kNoAllocMaxNodes % kNoAllocNodesPerBlock == 0, "whole rows");

static __device__ __align__(256) double g_noalloc_partials[kNoAllocRows * kStatsValues];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device` (which must be current).
// Looked up on the first call per device; later calls reuse it.  A
// cudaDeviceReset of that device ends the context that holds the array, so a
// process that resets a device must not call lbm_stats_noalloc on it again.
cudaError_t noalloc_scratch(int device, double **out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[device] = static_cast<double *>(p);
    }
    *out = g_noalloc_ptr[device];
    return cudaSuccess;
}

}  // namespace
}  // namespace lbm

extern "C" int lbm_stats_noalloc(const lbm_params *p, const float *phi, const float *rho, const float *ux,
                                 const float *uy, const float *uz, double *raw_out, void *stream)
{
    if (!p || !phi || !rho || !ux || !uy || !uz || !raw_out) {
        lbm::set_error("lbm_stats_noalloc: NULL argument");
        return LBM_EINVAL;
    }
    if (p->nx < 3 || p->ny < 3 || p->nz < 3) {
        lbm::set_error("lbm_stats_noalloc: box must be at least 3 nodes in each direction");
        return LBM_EINVAL;
    }
    const long long n = (long long)p->nx * p->ny * p->nz;
    if (n > lbm::kNoAllocMaxNodes) {
        lbm::set_error("lbm_stats_noalloc: box of " + std::to_string(n) +
                       " nodes exceeds the no-allocation limit of LBM_NOALLOC_MAX_NODES = 512^3 nodes");
        return LBM_EINVAL;
    }
    if (p->device < 0 || p->device >= lbm::kMaxDevices) {
        lbm::set_error("lbm_stats_noalloc: device ordinal out of range");
        return LBM_EINVAL;
    }
    if (const char *why = lbm::physics_error(*p)) {
        lbm::set_error(std::string("lbm_stats_noalloc: ") + why);
        return LBM_EINVAL;
    }
    // the caller's current device is given back on return (when it can be read)
    int prev = 0;
    const bool have_prev = cudaGetDevice(&prev) == cudaSuccess;
    const bool switch_device = !have_prev || prev != p->device;
    cudaError_t e = switch_device ? cudaSetDevice(p->device) : cudaSuccess;
    double *scratch = nullptr;
    if (e == cudaSuccess) e = lbm::noalloc_scratch(p->device, &scratch);
    if (e == cudaSuccess) {
        lbm_derived d;
        lbm::derive(*p, d);
        lbm::Box b;
        b.nx = p->nx;
        b.ny = p->ny;
        b.nz = p->nz;
        b.nxy = (long long)p->nx * p->ny;
        b.n = n;
        const unsigned blocks = (unsigned)((n + lbm::kNoAllocNodesPerBlock - 1) / lbm::kNoAllocNodesPerBlock);
        const cudaStream_t s = static_cast<cudaStream_t>(stream);
        lbm::StatsConst c{d.alpha, d.kappa, d.phiStarSq};
        lbm::stats_kernel<<<blocks, lbm::kThreads, 0, s>>>(b, c, phi, rho, ux, uy, uz, scratch);
        e = cudaGetLastError();
        if (e == cudaSuccess) {
            lbm::fold_kernel<<<1, lbm::kThreads, 0, s>>>(scratch, (int)blocks, raw_out);
            e = cudaGetLastError();
        }
    }
    if (switch_device && have_prev) cudaSetDevice(prev);
    if (e != cudaSuccess) {
        lbm::set_error(std::string("lbm_stats_noalloc: ") + cudaGetErrorString(e));
        return LBM_ECUDA;
    }
    return LBM_OK;
}
