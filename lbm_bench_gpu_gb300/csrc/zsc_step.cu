// zsc_step.cu -- one fused sm_103a kernel per ZSC lattice Boltzmann step.
//
// One launch does what the reference does with nine kernels and three
// host-staged halo exchanges per step (src/main.cu:416-507):
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
//
// Work decomposition: a block owns a TX x TY column tile and marches a chunk
// of TZ planes in z.  The phi stencil (19-point Laplacian and gradient,
// src/collision_f.cu:61-94) needs phi on a one-node ring around the tile, and
// phi = sum f needs P^{n-1} one node further out, so each plane of P^{n-1} is
// staged in shared memory on the tile plus two halo rows and four halo columns.
//
// Memory pipeline: every global read goes through cp.async (16-byte chunks,
// L2-cached, no registers held while in flight) into shared-memory stages:
//   - the 19 g rows of the next plane (2 stages; odd steps stage 36-wide rows
//     so the +-x shifted reads stay 16-byte aligned),
//   - the 7 P_f planes three planes ahead (4 stages),
// so a block always has about one plane of the step's input in flight while it
// computes the current plane.  Periodic wrap is applied per 16-byte chunk: with
// nx a multiple of 32 no chunk straddles the seam.  DRAM sees each
// distribution once per step (26 x 8 B = 208 B per node in FP32); the halo
// re-reads of neighbouring tiles are served by L2.
#include "lbm_internal.h"

namespace lbm {
namespace {

#ifndef ZSC_TILE_Y
#define ZSC_TILE_Y 8
#endif
#ifndef ZSC_MIN_BLOCKS
#define ZSC_MIN_BLOCKS 2
#endif
constexpr int TX = 32;              // tile width in x (one warp per row)
constexpr int TY = ZSC_TILE_Y;      // tile height in y
constexpr int NT = TX * TY;         // threads per block
constexpr int GW = 40;              // staged row width: x in [x0 - 4, x0 + 36)
constexpr int FR = TY + 4;          // staged P_f rows: y in [y0 - 2, y0 + TY + 2)
constexpr int RW = TX + 2;          // phi ring width (tile + one-node ring)
constexpr int RH = TY + 2;
constexpr int RING = 2 * RW + 2 * TY;
constexpr int NG = 2;               // g stages
constexpr int NF = 4;               // P_f stages
constexpr int NPHI = 4;             // phi planes
constexpr int G_STAGE = kQg * TY * GW;
constexpr int F_STAGE = kQf * FR * GW;
constexpr int PHI_STAGE = RH * RW;
constexpr size_t kSmemBytes = sizeof(float) * (NG * G_STAGE + NF * F_STAGE + NPHI * PHI_STAGE);
static_assert(RING <= NT, "one ring node per thread at most");

constexpr float kInv6 = 0.16666666666666666667f;
constexpr float kInv12 = 0.08333333333333333333f;

// D3Q19 lattice vectors and opposite directions (reference order).
__host__ __device__ constexpr int kCx(int i)
{
    return (i == 1 || i == 7 || i == 9 || i == 11 || i == 13) ? 1
           : (i == 2 || i == 8 || i == 10 || i == 12 || i == 14) ? -1 : 0;
}
__host__ __device__ constexpr int kCy(int i)
{
    return (i == 3 || i == 7 || i == 10 || i == 15 || i == 17) ? 1
           : (i == 4 || i == 8 || i == 9 || i == 16 || i == 18) ? -1 : 0;
}
__host__ __device__ constexpr int kCz(int i)
{
    return (i == 5 || i == 11 || i == 14 || i == 15 || i == 18) ? 1
           : (i == 6 || i == 12 || i == 13 || i == 16 || i == 17) ? -1 : 0;
}
__host__ __device__ constexpr int kOpp(int i) { return i == 0 ? 0 : ((i & 1) ? i + 1 : i - 1); }

template <int I>
struct Dir {
    static constexpr int value = I;
};

struct StepPtrs {
    const float *fin[kQf];
    float *fout[kQf];
    float *g[kQg];
    float *mom[5];
};

// Offsets (in elements, within one array) from a node to its periodic
// neighbours.
struct Nbr {
    int xm, xp, ym, yp, zm, zp;
};

__device__ __forceinline__ Nbr neighbours(const Box &b, int x, int y, int z)
{
    Nbr o;
    o.xm = (x == 0) ? b.nx - 1 : -1;
    o.xp = (x == b.nx - 1) ? -(b.nx - 1) : 1;
    o.ym = (y == 0) ? (b.ny - 1) * b.nx : -b.nx;
    o.yp = (y == b.ny - 1) ? -(b.ny - 1) * b.nx : b.nx;
    const int nxy = (int)b.nxy;
    o.zm = (z == 0) ? (b.nz - 1) * nxy : -nxy;
    o.zp = (z == b.nz - 1) ? -(b.nz - 1) * nxy : nxy;
    return o;
}

__device__ __forceinline__ unsigned node_index(const Box &b, int x, int y, int z)
{
    return (unsigned)x + (unsigned)b.nx * ((unsigned)y + (unsigned)b.ny * (unsigned)z);
}

__device__ __forceinline__ int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// 16-byte global -> shared copy, cached in L2 only; completes asynchronously.
__device__ __forceinline__ void cp_async16(float *smem, const float *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <bool STREAMED, bool ODD>
__global__ void __launch_bounds__(NT, ZSC_MIN_BLOCKS)
zsc_step_kernel(const StepPtrs P, const Box b, const StepConst c, const int tz, const int write_moments)
{
    extern __shared__ __align__(16) float smem[];
    float *const G = smem;                    // [NG][19][TY][GW]
    float *const F = G + NG * G_STAGE;        // [NF][7][FR][GW]
    float *const PHI = F + NF * F_STAGE;      // [NPHI][RH][RW]

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * TX + tx;
    int bid = blockIdx.x;
    const int ntx = b.nx / TX, nty = b.ny / TY;
    const int bx = bid % ntx;
    bid /= ntx;
    const int by = bid % nty;
    bid /= nty;
    const int z0 = bid * tz;
    const int nzc = min(tz, b.nz - z0);       // planes of this chunk
    const int x0 = bx * TX, y0 = by * TY;
    const int x = x0 + tx, y = y0 + ty;

    // Halo ring node handled by this thread (if any): top row, bottom row,
    // left column, right column of the (TX+2) x (TY+2) phi tile.
    const bool has_ring = tid < RING;
    int rlx = 0, rly = 0;
    if (tid < RW) {
        rlx = tid;
        rly = 0;
    } else if (tid < 2 * RW) {
        rlx = tid - RW;
        rly = TY + 1;
    } else if (tid < 2 * RW + TY) {
        rlx = 0;
        rly = tid - 2 * RW + 1;
    } else if (has_ring) {
        rlx = TX + 1;
        rly = tid - 2 * RW - TY + 1;
    }

    // P_f stage of plane p (p >= z0 - 2)
    auto fslot = [&](int p) { return F + ((p - z0 + 4) & (NF - 1)) * F_STAGE; };

    // ---- staging roles, fixed per thread for the whole chunk ----
    // Warps 0-3 queue the 7 P_f planes: thread t < FR * GW/4 owns staged row
    // t / (GW/4), 16-byte chunk t % (GW/4), of every array.
    constexpr int kFChunks = FR * (GW / 4);
    static_assert(kFChunks <= NT / 2, "P_f issuers fit in the first half of the block");
    const bool f_issuer = tid < kFChunks;
    int f_xy = 0, f_dst = 0;
    if (f_issuer) {
        const int r = tid / (GW / 4), k = tid - r * (GW / 4);
        f_xy = wrap(x0 - 4 + 4 * k, b.nx) + b.nx * wrap(y0 - 2 + r, b.ny);
        f_dst = r * GW + 4 * k;
    }
    // Warps 4-7 queue the g rows: thread owns row g_r, chunk g_k of every
    // second direction (g_hi: odd or even directions; uniform per warp).
    static_assert(TX == 32 && TY == 8, "g issuer mapping: 8 rows x 8 chunks per direction, two halves");
    const int gt = tid - NT / 2;
    const bool g_issuer = gt >= 0;
    const int g_hi = (gt >> 6) & 1;
    const int g_r = (gt & 63) >> 3, g_k = gt & 7;
    int g_row_0 = 0, g_row_p = 0, g_row_m = 0, g_x_lo = 0, g_x_hi = 0, g_x_wrap = 0;
    if (g_issuer) {
        g_row_0 = b.nx * (y0 + g_r);
        g_row_p = b.nx * wrap(y0 + g_r - 1, b.ny);   // directions with c_y = +1 read row y - 1
        g_row_m = b.nx * wrap(y0 + g_r + 1, b.ny);   // c_y = -1 reads row y + 1
        g_x_lo = wrap(x0 - 4 + 4 * g_k, b.nx);        // c_x = +1 reads x - 1: chunks from x0 - 4
        g_x_hi = x0 + 4 * g_k;                         // c_x <= 0: chunks from x0
        g_x_wrap = wrap(x0 + TX, b.nx);                // c_x = -1 also needs x0 + 32
    }

    // Queue the 7 P_f planes of plane p (tile + halo) into its stage.
    auto issue_f = [&](int p) {
        if (!f_issuer) return;
        const unsigned base = (unsigned)wrap(p, b.nz) * (unsigned)b.nxy + (unsigned)f_xy;
        float *dst = fslot(p) + f_dst;
#pragma unroll
        for (int arr = 0; arr < kQf; arr++) cp_async16(dst + arr * FR * GW, P.fin[arr] + base);
    };

    // Call f(direction) for the directions this g issuer owns (compile-time
    // direction numbers; the branch is uniform per warp).
    auto for_my_dirs = [&](auto &&f) {
        if (g_hi == 0) {
            f(Dir<0>{}); f(Dir<2>{}); f(Dir<4>{}); f(Dir<6>{}); f(Dir<8>{});
            f(Dir<10>{}); f(Dir<12>{}); f(Dir<14>{}); f(Dir<16>{}); f(Dir<18>{});
        } else {
            f(Dir<1>{}); f(Dir<3>{}); f(Dir<5>{}); f(Dir<7>{}); f(Dir<9>{});
            f(Dir<11>{}); f(Dir<13>{}); f(Dir<15>{}); f(Dir<17>{});
        }
    };

    // Queue the 19 g rows the nodes of plane z read, into g stage s.  Even
    // steps read the node's own slots; odd steps read direction i of node x
    // from the reversed slot of x - c_i (AA pattern).
    auto issue_g = [&](int z, int s) {
        if (!g_issuer) return;
        float *dst = G + s * G_STAGE + g_r * GW;
        if (!ODD) {
            const unsigned base = (unsigned)z * (unsigned)b.nxy + (unsigned)(g_row_0 + g_x_hi);
            for_my_dirs([&](auto d) {
                constexpr int i = decltype(d)::value;
                cp_async16(dst + i * TY * GW + 4 + 4 * g_k, P.g[i] + base);
            });
        } else {
            const unsigned zb0 = (unsigned)z * (unsigned)b.nxy;
            const unsigned zbp = (unsigned)wrap(z - 1, b.nz) * (unsigned)b.nxy;   // c_z = +1 reads z - 1
            const unsigned zbm = (unsigned)wrap(z + 1, b.nz) * (unsigned)b.nxy;   // c_z = -1 reads z + 1
            for_my_dirs([&](auto d) {
                constexpr int i = decltype(d)::value;
                constexpr int cx = kCx(i), cy = kCy(i), cz = kCz(i);
                const unsigned zb = cz > 0 ? zbp : (cz < 0 ? zbm : zb0);
                const int row = cy > 0 ? g_row_p : (cy < 0 ? g_row_m : g_row_0);
                const float *src = P.g[kOpp(i)] + (zb + (unsigned)row);
                float *d_row = dst + i * TY * GW;
                if (cx > 0) {
                    cp_async16(d_row + 4 * g_k, src + g_x_lo);
                    if (g_k == 0) cp_async16(d_row + 32, src + (x0 + 28));
                } else {
                    cp_async16(d_row + 4 + 4 * g_k, src + g_x_hi);
                    if (cx < 0 && g_k == 0) cp_async16(d_row + 36, src + g_x_wrap);
                }
            });
        }
    };

    // Streamed D3Q7 values at ring-tile position (lx, ly) of plane p and their
    // sum phi (src/update_phi.cu:42-43), from the staged planes.
    auto phi_at = [&](int p, int lx, int ly, float(&f)[kQf]) -> float {
        const int col = lx + 3, row = ly + 1;
        const float *S1 = fslot(p);
        auto at = [&](const float *S, int arr, int rr, int cc) { return S[(arr * FR + rr) * GW + cc]; };
        if (STREAMED) {
#pragma unroll
            for (int i = 0; i < kQf; i++) f[i] = at(S1, i, row, col);
        } else {
            const float *S0 = fslot(p - 1), *S2 = fslot(p + 1);
            const float eta = c.eta, eta2 = c.eta2;
            f[0] = at(S1, 0, row, col);
            f[1] = eta * at(S1, 1, row, col - 1) + eta2 * at(S1, 1, row, col);
            f[2] = eta * at(S1, 2, row, col + 1) + eta2 * at(S1, 2, row, col);
            f[3] = eta * at(S1, 3, row - 1, col) + eta2 * at(S1, 3, row, col);
            f[4] = eta * at(S1, 4, row + 1, col) + eta2 * at(S1, 4, row, col);
            f[5] = eta * at(S0, 5, row, col) + eta2 * at(S1, 5, row, col);
            f[6] = eta * at(S2, 6, row, col) + eta2 * at(S1, 6, row, col);
        }
        return f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6];
    };

    // phi of plane p on the tile + ring into phi slot s; the streamed f of the
    // thread's own node is returned in fo.
    auto build_plane = [&](int p, int s, float(&fo)[kQf]) {
        float *ph = PHI + s * PHI_STAGE;
        ph[(ty + 1) * RW + tx + 1] = phi_at(p, tx + 1, ty + 1, fo);
        if (has_ring) {
            float tmp[kQf];
            ph[rly * RW + rlx] = phi_at(p, rlx, rly, tmp);
        }
    };

    float fcur[kQf], fnext[kQf];

    // prologue: P_f planes z0-2 .. z0+1, g of plane z0; phi of z0-1 and z0
    issue_f(z0 - 2);
    issue_f(z0 - 1);
    issue_f(z0);
    issue_f(z0 + 1);
    issue_g(z0, 0);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    {
        float tmp[kQf];
        build_plane(z0 - 1, 0, tmp);
    }
    build_plane(z0, 1, fcur);
    __syncthreads();
    issue_f(z0 + 2);
    cp_async_commit();

    for (int j = 0; j < nzc; ++j) {
        const int z = z0 + j;
        cp_async_wait_all();
        __syncthreads();
        if (j + 1 < nzc) {
            issue_g(z + 1, (j + 1) & 1);
            issue_f(z + 3);
        }
        cp_async_commit();
        build_plane(z + 1, (j + 2) & 3, fnext);
        __syncthreads();

        const float *S0 = PHI + (j & 3) * PHI_STAGE;        // plane z - 1
        const float *S1 = PHI + ((j + 1) & 3) * PHI_STAGE;  // plane z
        const float *S2 = PHI + ((j + 2) & 3) * PHI_STAGE;  // plane z + 1
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
        const float Fx = mu * (2.f * (pe - pw) + pen - pws + pes - pwn + pet - pwb + peb - pwt) * kInv12;
        const float Fy = mu * (2.f * (pn - ps) + pen - pws + pwn - pes + pnt - psb + pnb - pst) * kInv12;
        float Fz = mu * (2.f * (pt - pb) + pet - pwb + pwt - peb + pnt - psb + pst - pnb) * kInv12;
        if (pc > 0.f) Fz += c.grav;

        // D3Q19 values of this node from the staged rows (AA pattern)
        const float *Gs = G + (j & 1) * G_STAGE;
        float g[kQg];
#pragma unroll
        for (int i = 0; i < kQg; i++) g[i] = Gs[(i * TY + ty) * GW + 4 + tx - (ODD ? kCx(i) : 0)];

        // moments: src/update_rho.cu:46-50, src/update_velocity.cu:47-59
        float rho = g[0];
#pragma unroll
        for (int i = 1; i < kQg; i++) rho += g[i];
        const float invRho = 1.0f / rho;
        const float ux = (g[1] - g[2] + g[7] - g[8] + g[9] - g[10] + g[11] - g[12] + g[13] - g[14]) * invRho;
        const float uy = (g[3] - g[4] + g[7] - g[8] - g[9] + g[10] + g[15] - g[16] + g[17] - g[18]) * invRho;
        const float uz = (g[5] - g[6] + g[11] - g[12] - g[13] + g[14] + g[15] - g[16] - g[17] + g[18]) * invRho;
        const unsigned id = node_index(b, x, y, z);
        if (write_moments) {
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
            const float Cf = c.invTauPhi * c.invEta2 * pc;
            const float a = c.invTauPhiOne;
            P.fout[0][id] = a * fcur[0] - 6.0f * Af + c.invTauPhi * pc;
            P.fout[1][id] = a * fcur[1] + Af + Cf * usx;
            P.fout[2][id] = a * fcur[2] + Af - Cf * usx;
            P.fout[3][id] = a * fcur[3] + Af + Cf * usy;
            P.fout[4][id] = a * fcur[4] + Af - Cf * usy;
            P.fout[5][id] = a * fcur[5] + Af + Cf * usz;
            P.fout[6][id] = a * fcur[6] + Af - Cf * usz;
        }

        // D3Q19 collision with forcing, src/collision_g.cu:232-313
        {
            const float bb = c.invTauRhoOne;
            const float K1 = c.K1, K2 = c.K2, KC1 = c.KC1, KC2 = c.KC2;
            const float phimu3 = 3.f * pc * mu;
            const float temp1 = K1 * (phimu3 + rho * (1.f - 1.5f * (usx * usx + usy * usy + usz * usz)));
            const float UF = usx * Fx + usy * Fy + usz * Fz;
            const float vx = usx * 3.f, vy = usy * 3.f, vz = usz * 3.f;
            const float vsq6 = (vx * vx + vy * vy + vz * vz) * kInv6;
            float q[kQg];
            q[0] = bb * g[0] + c.K0 * (rho - 6.f * pc * mu - rho * vsq6) - c.KC0 * UF;
            {
                const float K1r = K1 * rho;
                float eq1 = temp1 + K1r * vx * vx * 0.5f + KC1 * (vx * Fx - UF);
                float eq2 = vx * (K1r + KC1 * Fx);
                q[1] = bb * g[1] + eq1 + eq2;
                q[2] = bb * g[2] + eq1 - eq2;
                eq1 = temp1 + K1r * vy * 0.5f * vy + KC1 * (vy * Fy - UF);
                eq2 = vy * (K1r + KC1 * Fy);
                q[3] = bb * g[3] + eq1 + eq2;
                q[4] = bb * g[4] + eq1 - eq2;
                eq1 = temp1 + K1r * vz * 0.5f * vz + KC1 * (vz * Fz - UF);
                eq2 = vz * (K1r + KC1 * Fz);
                q[5] = bb * g[5] + eq1 + eq2;
                q[6] = bb * g[6] + eq1 - eq2;
            }
            {
                const float K2r = K2 * rho;
                const float temp2 = K2 * (phimu3 + rho * (1.f - vsq6));
                auto pair = [&](float w, float Gf, int ip, int im) {
                    const float eq1 = temp2 + K2r * w * 0.5f * w + KC2 * (w * Gf - UF);
                    const float eq2 = K2r * w + KC2 * Gf;
                    q[ip] = bb * g[ip] + eq1 + eq2;
                    q[im] = bb * g[im] + eq1 - eq2;
                };
                pair(vx + vy, Fx + Fy, 7, 8);
                pair(vx - vy, Fx - Fy, 9, 10);
                pair(vx + vz, Fx + Fz, 11, 12);
                pair(vx - vz, Fx - Fz, 13, 14);
                pair(vy + vz, Fy + Fz, 15, 16);
                pair(vy - vz, Fy - Fz, 17, 18);
            }
            if (!ODD) {
                // even: own node, reversed slots
#pragma unroll
                for (int i = 0; i < kQg; i++) P.g[kOpp(i)][id] = q[i];
            } else {
                // odd: downstream neighbour x + c_i, natural slot i
                const Nbr o = neighbours(b, x, y, z);
                auto off = [&](int i) {
                    return (kCx(i) > 0 ? o.xp : kCx(i) < 0 ? o.xm : 0) + (kCy(i) > 0 ? o.yp : kCy(i) < 0 ? o.ym : 0)
                           + (kCz(i) > 0 ? o.zp : kCz(i) < 0 ? o.zm : 0);
                };
#pragma unroll
                for (int i = 0; i < kQg; i++) P.g[i][id + off(i)] = q[i];
            }
        }

#pragma unroll
        for (int i = 0; i < kQf; i++) fcur[i] = fnext[i];
    }
}

template <bool S, bool O>
cudaError_t configure()
{
    static bool done = false;   // per template instance, per process
    if (done) return cudaSuccess;
    const cudaError_t e =
        cudaFuncSetAttribute(zsc_step_kernel<S, O>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
    if (e == cudaSuccess) done = true;
    return e;
}

// Planes per block.  The blocks of one launch all march the same number of
// planes, so the step takes about ceil(blocks / resident slots) "waves" of
// (tz + prologue) planes; pick the chunk depth that minimises that product
// (e.g. 256^3: 37 planes -> 1792 blocks = 5.9 waves of 304 slots, instead of
// 32 planes -> 6.7 waves with a 74%-full last wave).
int choose_tz(const Box &b)
{
    static int slots = 0;
    if (slots == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zsc_step_kernel<false, false>, NT, kSmemBytes);
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

}  // namespace

cudaError_t launch_step(const Box &b, const StepConst &c, const float *f_in, float *f_out, float *g, float *mom,
                        bool f_streamed, bool odd, bool write_moments, cudaStream_t s)
{
    if (b.nx % TX != 0 || b.ny % TY != 0) return cudaErrorInvalidValue;
    StepPtrs P;
    for (int i = 0; i < kQf; i++) {
        P.fin[i] = f_in + (size_t)i * b.n;
        P.fout[i] = f_out + (size_t)i * b.n;
    }
    for (int i = 0; i < kQg; i++) P.g[i] = g + (size_t)i * b.n;
    for (int i = 0; i < 5; i++) P.mom[i] = mom + (size_t)i * b.n;
    cudaError_t e = configure<true, false>();
    if (e == cudaSuccess) e = configure<false, true>();
    if (e == cudaSuccess) e = configure<false, false>();
    if (e != cudaSuccess) return e;
    const int tz = choose_tz(b);
    const int nchunks = (b.nz + tz - 1) / tz;
    const unsigned nblocks = (unsigned)((b.nx / TX) * (b.ny / TY) * nchunks);
    const dim3 block(TX, TY, 1);
    const int wm = write_moments ? 1 : 0;
    if (f_streamed) {
        if (odd) return cudaErrorInvalidValue;  // the streamed initial state is always read by an even step
        zsc_step_kernel<true, false><<<nblocks, block, kSmemBytes, s>>>(P, b, c, tz, wm);
    } else if (odd) {
        zsc_step_kernel<false, true><<<nblocks, block, kSmemBytes, s>>>(P, b, c, tz, wm);
    } else {
        zsc_step_kernel<false, false><<<nblocks, block, kSmemBytes, s>>>(P, b, c, tz, wm);
    }
    return cudaGetLastError();
}

}  // namespace lbm
