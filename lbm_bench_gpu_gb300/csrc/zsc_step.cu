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
// The phi stencil (19-point Laplacian and gradient, src/collision_f.cu:61-94)
// needs phi on a one-node halo, and phi = sum f needs P^{n-1} one node further
// out.  Each block owns a TX x TY column tile and marches a chunk of TZ planes
// in z; phi of the tile plus a one-node ring is rebuilt per plane into a
// four-plane shared-memory ring buffer, so DRAM sees each distribution once
// per step (read + write = 26 x 8 B = 208 B per node in FP32) and the halo
// re-reads are served by L1/L2.
#include "lbm_internal.h"

namespace lbm {
namespace {

constexpr int TX = 32;            // tile width in x (one warp per row)
constexpr int TY = 8;             // tile height in y
constexpr int TZ = 32;            // planes per block
constexpr int NT = TX * TY;       // threads per block
constexpr int RW = TX + 2;        // phi ring buffer row width (tile + 1 halo)
constexpr int RH = TY + 2;
constexpr int RING = 2 * RW + 2 * TY;  // halo nodes around the tile
static_assert(RING <= NT, "one halo node per thread at most");

constexpr float kInv6 = 0.16666666666666666667f;
constexpr float kInv12 = 0.08333333333333333333f;

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

__device__ __forceinline__ float ldg(const float *p) { return __ldg(p); }

// Streamed D3Q7 values at node (x, y, z) and their sum phi
// (src/update_phi.cu:42-43).  STREAMED: f holds streamed values (initial
// state).  Otherwise f holds P^{n-1} and the ZSC interpolated streaming
// (src/stream_f.cu:52-59) is applied while reading.
template <bool STREAMED>
__device__ __forceinline__ float phi_at(const StepPtrs &P, const Box &b, const StepConst &c, int x, int y, int z,
                                        float (&f)[kQf])
{
    const unsigned id = node_index(b, x, y, z);
    if (STREAMED) {
#pragma unroll
        for (int i = 0; i < kQf; i++) f[i] = ldg(P.fin[i] + id);
    } else {
        const Nbr o = neighbours(b, x, y, z);
        const float eta = c.eta, eta2 = c.eta2;
        f[0] = ldg(P.fin[0] + id);
        f[1] = eta * ldg(P.fin[1] + (id + o.xm)) + eta2 * ldg(P.fin[1] + id);
        f[2] = eta * ldg(P.fin[2] + (id + o.xp)) + eta2 * ldg(P.fin[2] + id);
        f[3] = eta * ldg(P.fin[3] + (id + o.ym)) + eta2 * ldg(P.fin[3] + id);
        f[4] = eta * ldg(P.fin[4] + (id + o.yp)) + eta2 * ldg(P.fin[4] + id);
        f[5] = eta * ldg(P.fin[5] + (id + o.zm)) + eta2 * ldg(P.fin[5] + id);
        f[6] = eta * ldg(P.fin[6] + (id + o.zp)) + eta2 * ldg(P.fin[6] + id);
    }
    return f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6];
}

template <bool STREAMED, bool ODD>
__global__ void __launch_bounds__(NT, 2)
zsc_step_kernel(const StepPtrs P, const Box b, const StepConst c, const int write_moments)
{
    __shared__ float sphi[4][RH][RW];

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * TX + tx;
    int bid = blockIdx.x;
    const int ntx = b.nx / TX, nty = b.ny / TY;
    const int bx = bid % ntx;
    bid /= ntx;
    const int by = bid % nty;
    bid /= nty;
    const int z0 = bid * TZ;
    const int zend = min(z0 + TZ, b.nz);

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
    int rx = x0 + rlx - 1, ry = y0 + rly - 1;
    rx = rx < 0 ? rx + b.nx : (rx >= b.nx ? rx - b.nx : rx);
    ry = ry < 0 ? ry + b.ny : (ry >= b.ny ? ry - b.ny : ry);

    auto wrapz = [&](int z) { return z < 0 ? z + b.nz : (z >= b.nz ? z - b.nz : z); };

    float fcur[kQf], fnext[kQf];

    // phi of plane z on the tile + ring into ring-buffer slot s; the streamed
    // f of the thread's own node is returned in fo.
    auto build_plane = [&](int z, int s, float (&fo)[kQf]) {
        sphi[s][ty + 1][tx + 1] = phi_at<STREAMED>(P, b, c, x, y, z, fo);
        if (has_ring) {
            float tmp[kQf];
            sphi[s][rly][rlx] = phi_at<STREAMED>(P, b, c, rx, ry, z, tmp);
        }
    };

    {
        float tmp[kQf];
        build_plane(wrapz(z0 - 1), 0, tmp);
    }
    build_plane(z0, 1, fcur);

    for (int z = z0; z < zend; ++z) {
        const int j = z - z0;
        build_plane(wrapz(z + 1), (j + 2) & 3, fnext);
        __syncthreads();

        const float(*S0)[RW] = sphi[j & 3];        // plane z - 1
        const float(*S1)[RW] = sphi[(j + 1) & 3];  // plane z
        const float(*S2)[RW] = sphi[(j + 2) & 3];  // plane z + 1
        const int lx = tx + 1, ly = ty + 1;

        // 19-point stencil, src/collision_f.cu:61-94 (e/w = x+-1, n/s = y+-1,
        // t/b = z+-1)
        const float pc = S1[ly][lx];
        const float pe = S1[ly][lx + 1], pw = S1[ly][lx - 1];
        const float pn = S1[ly + 1][lx], ps = S1[ly - 1][lx];
        const float pt = S2[ly][lx], pb = S0[ly][lx];
        const float pen = S1[ly + 1][lx + 1], pws = S1[ly - 1][lx - 1];
        const float pes = S1[ly - 1][lx + 1], pwn = S1[ly + 1][lx - 1];
        const float pet = S2[ly][lx + 1], pwb = S0[ly][lx - 1];
        const float peb = S0[ly][lx + 1], pwt = S2[ly][lx - 1];
        const float pnt = S2[ly + 1][lx], psb = S0[ly - 1][lx];
        const float pnb = S0[ly + 1][lx], pst = S2[ly - 1][lx];

        const float lap = (pen + pws + pes + pwn + pet + pwb + peb + pwt + pnt + psb + pnb + pst
                           + 2.f * (pe + pw + pn + ps + pt + pb - 12.f * pc)) * kInv6;
        const float mu = c.alpha4 * pc * (pc * pc - c.phiStarSq) - c.kappa * lap;
        const float Fx = mu * (2.f * (pe - pw) + pen - pws + pes - pwn + pet - pwb + peb - pwt) * kInv12;
        const float Fy = mu * (2.f * (pn - ps) + pen - pws + pwn - pes + pnt - psb + pnb - pst) * kInv12;
        float Fz = mu * (2.f * (pt - pb) + pet - pwb + pwt - peb + pnt - psb + pst - pnb) * kInv12;
        if (pc > 0.f) Fz += c.grav;

        // D3Q19 values of this node (AA pattern)
        const unsigned id = node_index(b, x, y, z);
        const Nbr o = neighbours(b, x, y, z);
        float g[kQg];
        if (!ODD) {
#pragma unroll
            for (int i = 0; i < kQg; i++) g[i] = P.g[i][id];
        } else {
            g[0] = P.g[0][id];
            g[1] = P.g[2][id + o.xm];
            g[2] = P.g[1][id + o.xp];
            g[3] = P.g[4][id + o.ym];
            g[4] = P.g[3][id + o.yp];
            g[5] = P.g[6][id + o.zm];
            g[6] = P.g[5][id + o.zp];
            g[7] = P.g[8][id + o.xm + o.ym];
            g[8] = P.g[7][id + o.xp + o.yp];
            g[9] = P.g[10][id + o.xm + o.yp];
            g[10] = P.g[9][id + o.xp + o.ym];
            g[11] = P.g[12][id + o.xm + o.zm];
            g[12] = P.g[11][id + o.xp + o.zp];
            g[13] = P.g[14][id + o.xm + o.zp];
            g[14] = P.g[13][id + o.xp + o.zm];
            g[15] = P.g[16][id + o.ym + o.zm];
            g[16] = P.g[15][id + o.yp + o.zp];
            g[17] = P.g[18][id + o.ym + o.zp];
            g[18] = P.g[17][id + o.yp + o.zm];
        }

        // moments: src/update_rho.cu:46-50, src/update_velocity.cu:47-59
        float rho = g[0];
#pragma unroll
        for (int i = 1; i < kQg; i++) rho += g[i];
        const float invRho = 1.0f / rho;
        const float ux = (g[1] - g[2] + g[7] - g[8] + g[9] - g[10] + g[11] - g[12] + g[13] - g[14]) * invRho;
        const float uy = (g[3] - g[4] + g[7] - g[8] - g[9] + g[10] + g[15] - g[16] + g[17] - g[18]) * invRho;
        const float uz = (g[5] - g[6] + g[11] - g[12] - g[13] + g[14] + g[15] - g[16] - g[17] + g[18]) * invRho;
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
                auto pair = [&](float w, float G, int ip, int im) {
                    const float eq1 = temp2 + K2r * w * 0.5f * w + KC2 * (w * G - UF);
                    const float eq2 = K2r * w + KC2 * G;
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
                P.g[0][id] = q[0];
                P.g[2][id] = q[1];
                P.g[1][id] = q[2];
                P.g[4][id] = q[3];
                P.g[3][id] = q[4];
                P.g[6][id] = q[5];
                P.g[5][id] = q[6];
                P.g[8][id] = q[7];
                P.g[7][id] = q[8];
                P.g[10][id] = q[9];
                P.g[9][id] = q[10];
                P.g[12][id] = q[11];
                P.g[11][id] = q[12];
                P.g[14][id] = q[13];
                P.g[13][id] = q[14];
                P.g[16][id] = q[15];
                P.g[15][id] = q[16];
                P.g[18][id] = q[17];
                P.g[17][id] = q[18];
            } else {
                // odd: downstream neighbour x + c_i, natural slot i
                P.g[0][id] = q[0];
                P.g[1][id + o.xp] = q[1];
                P.g[2][id + o.xm] = q[2];
                P.g[3][id + o.yp] = q[3];
                P.g[4][id + o.ym] = q[4];
                P.g[5][id + o.zp] = q[5];
                P.g[6][id + o.zm] = q[6];
                P.g[7][id + o.xp + o.yp] = q[7];
                P.g[8][id + o.xm + o.ym] = q[8];
                P.g[9][id + o.xp + o.ym] = q[9];
                P.g[10][id + o.xm + o.yp] = q[10];
                P.g[11][id + o.xp + o.zp] = q[11];
                P.g[12][id + o.xm + o.zm] = q[12];
                P.g[13][id + o.xp + o.zm] = q[13];
                P.g[14][id + o.xm + o.zp] = q[14];
                P.g[15][id + o.yp + o.zp] = q[15];
                P.g[16][id + o.ym + o.zm] = q[16];
                P.g[17][id + o.yp + o.zm] = q[17];
                P.g[18][id + o.ym + o.zp] = q[18];
            }
        }

#pragma unroll
        for (int i = 0; i < kQf; i++) fcur[i] = fnext[i];
    }
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
    const int nchunks = (b.nz + TZ - 1) / TZ;
    const unsigned nblocks = (unsigned)((b.nx / TX) * (b.ny / TY) * nchunks);
    const dim3 block(TX, TY, 1);
    const int wm = write_moments ? 1 : 0;
    if (f_streamed) {
        if (odd) return cudaErrorInvalidValue;  // the streamed initial state is always read by an even step
        zsc_step_kernel<true, false><<<nblocks, block, 0, s>>>(P, b, c, wm);
    } else if (odd) {
        zsc_step_kernel<false, true><<<nblocks, block, 0, s>>>(P, b, c, wm);
    } else {
        zsc_step_kernel<false, false><<<nblocks, block, 0, s>>>(P, b, c, wm);
    }
    return cudaGetLastError();
}

}  // namespace lbm
