// zsc_init.cu -- initial condition kernels.
//
// bubble_phi_kernel   : src/init.c:39-59 (phi from the bubble list, on the GPU)
// equilibrium_kernel  : src/init_f.cu:42-79 and src/init_g.cu:46-93
#include "lbm_internal.h"

namespace lbm {
namespace {

constexpr float kW0 = 0.33333333333333333333f;  // src/constants.h:52-54
constexpr float kW1 = 0.05555555555555555556f;
constexpr float kW2 = 0.02777777777777777778f;
constexpr float kInv6 = 0.16666666666666666667f;

// phi on nx * ny * (nz + 2) nodes: plane kk is the reference's plane
// k = kk + kk0 (the two ghost planes included; kk0 = z0 for a z-slab starting
// at plane z0 of a larger box, as a rank of the reference sets its own planes
// from the bubble list), x and y 0-based.  For each bubble in file
// order, nodes with R <= Rc + width take phiStar * tanh(2 (Rc - R) / width),
// the others keep -phiStar; the last bubble that covers a node wins.  The
// distance and the comparison use round-to-nearest float operations without
// contraction, so the covered set is the one the reference's host code gets.
__global__ void bubble_phi_kernel(Box b, const float *__restrict__ bubbles, int nbubbles, float phiStar,
                                  float width, int kk0, float *__restrict__ phig)
{
    const long long total = b.nxy * (long long)(b.nz + 2);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % b.nx);
        const int j = (int)((t / b.nx) % b.ny);
        const int kk = (int)(t / b.nxy);
        float v = -phiStar;
        for (int m = 0; m < nbubbles; m++) {
            const float xc = __ldg(bubbles + 4 * m + 0), yc = __ldg(bubbles + 4 * m + 1);
            const float zc = __ldg(bubbles + 4 * m + 2), rc = __ldg(bubbles + 4 * m + 3);
            const float dx = __fsub_rn((float)i, xc);
            const float dy = __fsub_rn((float)j, yc);
            const float dz = __fsub_rn((float)(kk + kk0), zc);
            const float s = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            const float R = __fsqrt_rn(s);
            if (R <= __fadd_rn(rc, width)) v = phiStar * tanhf(__fdiv_rn(2.f * __fsub_rn(rc, R), width));
        }
        phig[t] = v;
    }
}

// The same phi, per tile of 32 x 8 x 4 nodes of the ghosted grid: the block
// first lists, in file order, the bubbles that can reach the tile (the
// distance from the centre to the tile's box, in double, against
// Rc + width + 0.01, which no rounding of the float test can exceed), then
// makes the float test of bubble_phi_kernel for those only, so the node set
// and the last covering bubble are the same.  A tile reached by more than
// kTileBubbles bubbles tests them all.
constexpr int BTX = 32, BTY = 8, BTZ = 4, kTileBubbles = 1024;

__global__ void __launch_bounds__(BTX * BTY) bubble_phi_tiled_kernel(Box b, const float *__restrict__ bubbles,
                                                                     int nbubbles, float phiStar, float width,
                                                                     int kk0, float *__restrict__ phig)
{
    __shared__ int list[kTileBubbles];
    __shared__ int warp_off[BTY];
    __shared__ int count, overflow;
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int x0 = blockIdx.x * BTX, y0 = blockIdx.y * BTY, k0 = blockIdx.z * BTZ;
    const int k1 = min(k0 + BTZ, b.nz + 2) - 1;
    if (lane == 0 && warp == 0) {
        count = 0;
        overflow = 0;
    }
    __syncthreads();
    for (int base = 0; base < nbubbles; base += BTX * BTY) {
        const int m = base + warp * BTX + lane;
        bool hit = false;
        if (m < nbubbles) {
            const double xc = bubbles[4 * m + 0], yc = bubbles[4 * m + 1], zc = bubbles[4 * m + 2];
            const double reach = (double)bubbles[4 * m + 3] + (double)width + 0.01;
            const double dx = fmax(fmax((double)x0 - xc, xc - (double)(x0 + BTX - 1)), 0.0);
            const double dy = fmax(fmax((double)y0 - yc, yc - (double)(y0 + BTY - 1)), 0.0);
            const double dz = fmax(fmax((double)(k0 + kk0) - zc, zc - (double)(k1 + kk0)), 0.0);
            hit = dx * dx + dy * dy + dz * dz <= reach * reach;
        }
        const unsigned ballot = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) warp_off[warp] = __popc(ballot);
        __syncthreads();
        if (lane == 0 && warp == 0) {   // exclusive prefix over the warps, in bubble order
            int run = count;
            for (int w = 0; w < BTY; w++) {
                const int c = warp_off[w];
                warp_off[w] = run;
                run += c;
            }
            count = run;
        }
        __syncthreads();
        if (hit) {
            const int pos = warp_off[warp] + __popc(ballot & ((1u << lane) - 1u));
            if (pos < kTileBubbles) list[pos] = m;
            else overflow = 1;
        }
        __syncthreads();
    }
    const bool every = overflow != 0;
    const int nlist = every ? nbubbles : min(count, kTileBubbles);
    const int i = x0 + lane, j = y0 + warp;
    for (int kk = k0; kk <= k1; kk++) {
        float v = -phiStar;
        for (int q = 0; q < nlist; q++) {
            const int m = every ? q : list[q];
            const float xc = __ldg(bubbles + 4 * m + 0), yc = __ldg(bubbles + 4 * m + 1);
            const float zc = __ldg(bubbles + 4 * m + 2), rc = __ldg(bubbles + 4 * m + 3);
            const float dx = __fsub_rn((float)i, xc);
            const float dy = __fsub_rn((float)j, yc);
            const float dz = __fsub_rn((float)(kk + kk0), zc);
            const float s = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            const float R = __fsqrt_rn(s);
            if (R <= __fadd_rn(rc, width)) v = phiStar * tanhf(__fdiv_rn(2.f * __fsub_rn(rc, R), width));
        }
        phig[(size_t)kk * (size_t)b.nxy + (size_t)j * (size_t)b.nx + (size_t)i] = v;
    }
}

// At-rest equilibrium from phi and rho.  z neighbours outside [0, nz) come
// from ghost_lo / ghost_hi (nx*ny each) when given, else by periodic wrap.
__global__ void equilibrium_kernel(Box b, float alpha4, float kappa, float phiStarSq, float Gamma,
                                   const float *__restrict__ phi, const float *__restrict__ rho,
                                   const float *__restrict__ ghost_lo, const float *__restrict__ ghost_hi,
                                   float *__restrict__ f0, float *__restrict__ fq, float *__restrict__ g)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % b.nx);
        const int j = (int)((t / b.nx) % b.ny);
        const int k = (int)(t / b.nxy);
        const int ie = i == b.nx - 1 ? 0 : i + 1, iw = i == 0 ? b.nx - 1 : i - 1;
        const int jn = j == b.ny - 1 ? 0 : j + 1, js = j == 0 ? b.ny - 1 : j - 1;
        auto P = [&](int x, int y, int z) -> float {
            if (z < 0) return ghost_lo ? ghost_lo[x + b.nx * y] : phi[x + b.nx * (y + (long long)b.ny * (b.nz - 1))];
            if (z >= b.nz) return ghost_hi ? ghost_hi[x + b.nx * y] : phi[x + b.nx * y];
            return phi[x + b.nx * (y + (long long)b.ny * z)];
        };
        const int kt = k + 1, kb = k - 1;
        const float phin = phi[t];
        const float lap = (P(ie, jn, k) + P(iw, js, k) + P(ie, js, k) + P(iw, jn, k) + P(ie, j, kt) + P(iw, j, kb)
                           + P(ie, j, kb) + P(iw, j, kt) + P(i, jn, kt) + P(i, js, kb) + P(i, jn, kb) + P(i, js, kt)
                           + 2.f * (P(ie, j, k) + P(iw, j, k) + P(i, jn, k) + P(i, js, k) + P(i, j, kt) + P(i, j, kb)
                                    - 12.f * phin)) * kInv6;
        const float mu = alpha4 * phin * (phin * phin - phiStarSq) - kappa * lap;
        const float Af = 0.5f * Gamma * mu;
        f0[t] = phin - 3.f * Gamma * mu;
        for (int q = 1; q < kQf; q++) fq[(q - 1) * b.n + t] = Af;
        const float rhon = rho[t];
        const float Ag1 = kW1 * (3.f * phin * mu + rhon);
        const float Ag2 = kW2 * (3.f * phin * mu + rhon);
        g[t] = kW0 * (rhon - 6.f * phin * mu);
        for (int q = 1; q < 7; q++) g[q * b.n + t] = Ag1;
        for (int q = 7; q < kQg; q++) g[q * b.n + t] = Ag2;
    }
}

__global__ void fill_kernel(float *p, long long n, float v)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        p[t] = v;
}

unsigned grid_for(long long n)
{
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    return (unsigned)(blocks < 1 ? 1 : blocks);
}

}  // namespace

cudaError_t launch_bubble_phi(const Box &b, const float *bubbles_dev, int nbubbles, float phiStar, float width,
                              int z0, float *phi_ghosted, cudaStream_t s)
{
    if (b.nx % BTX == 0 && b.ny % BTY == 0) {
        const dim3 grid((unsigned)(b.nx / BTX), (unsigned)(b.ny / BTY), (unsigned)((b.nz + 2 + BTZ - 1) / BTZ));
        bubble_phi_tiled_kernel<<<grid, dim3(BTX, BTY), 0, s>>>(b, bubbles_dev, nbubbles, phiStar, width, z0,
                                                                 phi_ghosted);
    } else {
        bubble_phi_kernel<<<grid_for(b.nxy * (b.nz + 2)), 256, 0, s>>>(b, bubbles_dev, nbubbles, phiStar, width,
                                                                        z0, phi_ghosted);
    }
    return cudaGetLastError();
}

cudaError_t launch_equilibrium(const Box &b, const lbm_derived &d, float Gamma, const float *phi, const float *rho,
                               const float *ghost_lo, const float *ghost_hi, float *f0, float *fq, float *g,
                               cudaStream_t s)
{
    equilibrium_kernel<<<grid_for(b.n), 256, 0, s>>>(b, d.alpha4, d.kappa, d.phiStarSq, Gamma, phi, rho, ghost_lo,
                                                      ghost_hi, f0, fq, g);
    return cudaGetLastError();
}

cudaError_t launch_fill(float *p, long long n, float v, cudaStream_t s)
{
    fill_kernel<<<grid_for(n), 256, 0, s>>>(p, n, v);
    return cudaGetLastError();
}

}  // namespace lbm
