// zsc_adjoint.cu -- discrete adjoint of the fused ZSC step (no counterpart in
// the reference).
//
// The forward step maps the streamed state s^n = (f^n, g^n) to s^{n+1}:
//   moments phi = sum f, rho = sum g, u = sum c g / rho;
//   lap, grad: 19-point stencils of phi (src/collision_f.cu:61-94);
//   mu = alpha4 phi (phi^2 - phiStar^2) - kappa lap;  F = mu grad (+ grav on phi > 0);
//   u* = u + F / (2 rho);  P = collision_f, Q = collision_g (src/collision_*.cu);
//   f'_i(x) = eta P_i(x - c_i) + (1 - eta) P_i(x);  g'_i(x) = Q_i(x - c_i).
// Its transpose, applied to lambda^{n+1} = dJ/ds^{n+1}:
//   stream:   lP_i(x) = eta lf'_i(x + c_i) + (1 - eta) lf'_i(x);  lQ_i(x) = lg'_i(x + c_i)
//   collision (local): direct terms (1 - 1/tau) lP, lQ plus the adjoints of
//             phi, mu, rho, u*, F, UF, 3 phi mu; dJ/dgrav += lambda_Fz H(phi > 0)
//   stencil:  lambda_phi += L[lambda_lap] - sum_k D_k[lambda_grad_k]
//             (the Laplacian stencil is symmetric, the gradient antisymmetric)
//   moments:  lf_i += lambda_phi;  lg_i += lambda_rho + c_i . lambda_m
// The stencil part is kept as a separate field lst (the same for all seven f
// populations) and added when lambda is read.  All per-node arithmetic is FP32;
// the objective sums and the gradient with respect to gravity are FP64.
#include "lbm_internal.h"

namespace lbm {
namespace {

constexpr int kThreads = 256;
constexpr float kInv6 = 0.16666666666666666667f;
constexpr float kInv12 = 0.08333333333333333333f;
constexpr float kW0 = 0.33333333333333333333f, kW1 = 0.05555555555555555556f, kW2 = 0.02777777777777777778f;

__constant__ int aCf[kQf][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
__constant__ int aCg[kQg][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                {0, 0, 1},  {0, 0, -1},  {1, 1, 0},  {-1, -1, 0}, {1, -1, 0},
                                {-1, 1, 0}, {1, 0, 1},   {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
                                {0, 1, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};

struct Coord {
    int x, y, z;
};

__device__ __forceinline__ Coord coord(const Box &b, long long t)
{
    Coord c;
    c.x = (int)(t % b.nx);
    c.y = (int)((t / b.nx) % b.ny);
    c.z = (int)(t / b.nxy);
    return c;
}

__device__ __forceinline__ long long at(const Box &b, Coord c, int dx, int dy, int dz)
{
    int x = c.x + dx, y = c.y + dy, z = c.z + dz;
    x = x < 0 ? x + b.nx : (x >= b.nx ? x - b.nx : x);
    y = y < 0 ? y + b.ny : (y >= b.ny ? y - b.ny : y);
    z = z < 0 ? z + b.nz : (z >= b.nz ? z - b.nz : z);
    return x + (long long)b.nx * (y + (long long)b.ny * z);
}

// 19-point Laplacian and gradient of field p at c (src/collision_f.cu:61-94).
__device__ __forceinline__ void stencil(const Box &b, const float *__restrict__ p, Coord c, float &lap, float &gx,
                                        float &gy, float &gz)
{
    auto P = [&](int dx, int dy, int dz) { return p[at(b, c, dx, dy, dz)]; };
    const float pc = P(0, 0, 0);
    const float pe = P(1, 0, 0), pw = P(-1, 0, 0), pn = P(0, 1, 0), ps = P(0, -1, 0), pt = P(0, 0, 1),
                pb = P(0, 0, -1);
    const float pen = P(1, 1, 0), pws = P(-1, -1, 0), pes = P(1, -1, 0), pwn = P(-1, 1, 0);
    const float pet = P(1, 0, 1), pwb = P(-1, 0, -1), peb = P(1, 0, -1), pwt = P(-1, 0, 1);
    const float pnt = P(0, 1, 1), psb = P(0, -1, -1), pnb = P(0, 1, -1), pst = P(0, -1, 1);
    lap = (pen + pws + pes + pwn + pet + pwb + peb + pwt + pnt + psb + pnb + pst
           + 2.f * (pe + pw + pn + ps + pt + pb - 12.f * pc)) * kInv6;
    gx = (2.f * (pe - pw) + pen - pws + pes - pwn + pet - pwb + peb - pwt) * kInv12;
    gy = (2.f * (pn - ps) + pen - pws + pwn - pes + pnt - psb + pnb - pst) * kInv12;
    gz = (2.f * (pt - pb) + pet - pwb + pwt - peb + pnt - psb + pst - pnb) * kInv12;
}

__device__ __forceinline__ double block_sum(double v, double *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kThreads / 32; w++) r += red[w];
    __syncthreads();
    return r;
}

// phi = sum f of the streamed state.
__global__ void phi_kernel(Box b, const float *__restrict__ F, float *__restrict__ phi)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        float s = F[t];
        for (int i = 1; i < kQf; i++) s += F[i * b.n + t];
        phi[t] = s;
    }
}

// Objective sums of one streamed state: A = sum w q, B = sum w, with
// w = (phiStar - phi) / (2 phiStar) and q = u_z (objective 0) or the reference
// plane index z + 1 (objective 1); per-block partials.
__global__ void __launch_bounds__(kThreads) objective_kernel(Box b, int objective, float phiStar,
                                                             const float *__restrict__ phi,
                                                             const float *__restrict__ G,
                                                             double *__restrict__ partials)
{
    __shared__ double red[kThreads / 32];
    double A = 0.0, B = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        const double w = ((double)phiStar - phi[t]) / (2.0 * phiStar);
        double q;
        if (objective == 0) {
            float rho = 0.f, mz = 0.f;
            for (int i = 0; i < kQg; i++) {
                const float gi = G[i * b.n + t];
                rho += gi;
                mz += aCg[i][2] * gi;
            }
            q = (double)mz / rho;
        } else {
            q = (double)(t / b.nxy + 1);
        }
        A += w * q;
        B += w;
    }
    A = block_sum(A, red);
    B = block_sum(B, red);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = A;
        partials[2 * blockIdx.x + 1] = B;
    }
}

// ab[0..1] = sums of the partials; acc[0] (J) += scale * A / B.
__global__ void objective_fold_kernel(const double *__restrict__ partials, int nparts, double scale,
                                      double *__restrict__ ab, double *__restrict__ acc)
{
    __shared__ double red[kThreads / 32];
    double A = 0.0, B = 0.0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) {
        A += partials[2 * p];
        B += partials[2 * p + 1];
    }
    A = block_sum(A, red);
    B = block_sum(B, red);
    if (threadIdx.x == 0) {
        ab[0] = A;
        ab[1] = B;
        acc[0] += scale * A / B;
    }
}

// d(scale * A / B)/d(state) at node t into lf, lg.
__device__ __forceinline__ void objective_source(const Box &b, long long t, int objective, double scale,
                                                 const double *ab, float phiStar, float ph, float rho, float mz,
                                                 float &dphi, float &drho, float &dmz)
{
    const double A = ab[0], B = ab[1];
    const double ratio = A / B;
    const double dw = -1.0 / (2.0 * phiStar);
    const double w = ((double)phiStar - ph) / (2.0 * phiStar);
    if (objective == 0) {
        const double uz = (double)mz / rho;
        dphi = (float)(scale * dw * (uz - ratio) / B);
        const double duz = scale * w / B;
        dmz = (float)(duz / rho);
        drho = (float)(-duz * uz / rho);
    } else {
        dphi = (float)(scale * dw * ((double)(t / b.nxy + 1) - ratio) / B);
        drho = 0.f;
        dmz = 0.f;
    }
}

// lambda^T: only the objective source of the final state.
__global__ void source_init_kernel(Box b, int objective, double scale, const double *__restrict__ ab,
                                   float phiStar, const float *__restrict__ phi, const float *__restrict__ G,
                                   float *__restrict__ lf, float *__restrict__ lg, float *__restrict__ lst)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        float rho = 0.f, mz = 0.f;
        for (int i = 0; i < kQg; i++) {
            const float gi = G[i * b.n + t];
            rho += gi;
            mz += aCg[i][2] * gi;
        }
        float dphi, drho, dmz;
        objective_source(b, t, objective, scale, ab, phiStar, phi[t], rho, mz, dphi, drho, dmz);
        for (int i = 0; i < kQf; i++) lf[i * b.n + t] = dphi;
        for (int i = 0; i < kQg; i++) lg[i * b.n + t] = drho + aCg[i][2] * dmz;
        lst[t] = 0.f;
    }
}

struct AdjIn {
    const float *F, *G, *phi;              // streamed s^n and its phi
    const float *lf, *lg, *lst;            // lambda^{n+1} (lf without its stencil part lst)
    float *lf_out, *lg_out;                // lambda^n without its stencil part
    float *llap, *lgrad;                   // lambda of lap and grad (3 x n) at every node
    double *dgrav_partials;                // per block
    const double *ab;                      // objective sums of s^n (when add_source)
    double scale;
    int objective, add_source;
};

// The local part of one adjoint step (see the file comment).
__global__ void __launch_bounds__(kThreads) adjoint_local_kernel(Box b, StepConst c, float phiStar, AdjIn a)
{
    __shared__ double red[kThreads / 32];
    double dg = 0.0;
    const long long n = b.n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const Coord cd = coord(b, t);
        float lap, gr[3];
        stencil(b, a.phi, cd, lap, gr[0], gr[1], gr[2]);
        const float ph = a.phi[t];
        float g[kQg], rh = 0.f, m[3] = {0.f, 0.f, 0.f};
        for (int i = 0; i < kQg; i++) {
            g[i] = a.G[i * n + t];
            rh += g[i];
            m[0] += aCg[i][0] * g[i];
            m[1] += aCg[i][1] * g[i];
            m[2] += aCg[i][2] * g[i];
        }
        const float inv = 1.0f / rh;
        const float u[3] = {m[0] * inv, m[1] * inv, m[2] * inv};
        const float mu = c.alpha4 * ph * (ph * ph - c.phiStarSq) - c.kappa * lap;
        float F[3] = {mu * gr[0], mu * gr[1], mu * gr[2]};
        const bool heavy = ph > 0.f;
        if (heavy) F[2] += c.grav;
        const float us[3] = {u[0] + 0.5f * F[0] * inv, u[1] + 0.5f * F[1] * inv, u[2] + 0.5f * F[2] * inv};
        const float v[3] = {3.f * us[0], 3.f * us[1], 3.f * us[2]};
        const float vsq6 = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * kInv6;
        const float Cf = c.invTauPhi * c.invEta2 * ph;

        // stream adjoint
        float lP[kQf], lQ[kQg];
        lP[0] = a.lf[t] + a.lst[t];
        const float lst_here = a.lst[t];
        for (int i = 1; i < kQf; i++) {
            const long long dn = at(b, cd, aCf[i][0], aCf[i][1], aCf[i][2]);
            lP[i] = c.eta * (a.lf[i * n + dn] + a.lst[dn]) + c.eta2 * (a.lf[i * n + t] + lst_here);
        }
        for (int i = 0; i < kQg; i++) lQ[i] = a.lg[i * n + at(b, cd, aCg[i][0], aCg[i][1], aCg[i][2])];

        // D3Q7 collision
        float lphi = 0.f, lmu = 0.f, lus[3] = {0.f, 0.f, 0.f}, lF[3] = {0.f, 0.f, 0.f}, lrho = 0.f;
        {
            const float lAf = -6.f * lP[0] + lP[1] + lP[2] + lP[3] + lP[4] + lP[5] + lP[6];
            float lCf = 0.f;
            for (int k = 0; k < 3; k++) {
                const float d = lP[1 + 2 * k] - lP[2 + 2 * k];
                lCf += us[k] * d;
                lus[k] += Cf * d;
            }
            lphi += c.invTauPhi * lP[0] + c.invTauPhi * c.invEta2 * lCf;
            lmu += 0.5f * c.Gamma * c.invTauPhi * lAf;
        }
        // D3Q19 collision with forcing
        float ls = 0.f, lvsq6 = 0.f, lUF = 0.f, lv[3] = {0.f, 0.f, 0.f};
        {
            ls += -2.f * c.K0 * lQ[0];
            lrho += c.K0 * (1.f - vsq6) * lQ[0];
            lvsq6 += -c.K0 * rh * lQ[0];
            lUF += -c.KC0 * lQ[0];
            float ltemp1 = 0.f;
            for (int k = 0; k < 3; k++) {
                const float S = lQ[1 + 2 * k] + lQ[2 + 2 * k], A = lQ[1 + 2 * k] - lQ[2 + 2 * k];
                ltemp1 += S;
                lrho += 0.5f * c.K1 * v[k] * v[k] * S + c.K1 * v[k] * A;
                lv[k] += c.K1 * rh * v[k] * S + c.KC1 * F[k] * S + (c.K1 * rh + c.KC1 * F[k]) * A;
                lF[k] += c.KC1 * v[k] * (S + A);
                lUF += -c.KC1 * S;
            }
            ls += c.K1 * ltemp1;
            lrho += c.K1 * (1.f - vsq6) * ltemp1;
            lvsq6 += -c.K1 * rh * ltemp1;
            // pairs (7,8) x+y, (9,10) x-y, (11,12) x+z, (13,14) x-z, (15,16) y+z, (17,18) y-z
            const int PA[6] = {0, 0, 0, 0, 1, 1}, PB[6] = {1, 1, 2, 2, 2, 2};
            const float SG[6] = {1.f, -1.f, 1.f, -1.f, 1.f, -1.f};
            float ltemp2 = 0.f;
#pragma unroll
            for (int p = 0; p < 6; p++) {
                const int ia = PA[p], ib = PB[p];
                const float sg = SG[p];
                const float w = v[ia] + sg * v[ib], Gs = F[ia] + sg * F[ib];
                const float S = lQ[7 + 2 * p] + lQ[8 + 2 * p], A = lQ[7 + 2 * p] - lQ[8 + 2 * p];
                ltemp2 += S;
                lrho += 0.5f * c.K2 * w * w * S + c.K2 * w * A;
                const float lw = c.K2 * rh * w * S + c.KC2 * Gs * S + c.K2 * rh * A;
                const float lG = c.KC2 * w * S + c.KC2 * A;
                lUF += -c.KC2 * S;
                lv[ia] += lw;
                lv[ib] += sg * lw;
                lF[ia] += lG;
                lF[ib] += sg * lG;
            }
            ls += c.K2 * ltemp2;
            lrho += c.K2 * (1.f - vsq6) * ltemp2;
            lvsq6 += -c.K2 * rh * ltemp2;
        }
        for (int k = 0; k < 3; k++) lv[k] += lvsq6 * v[k] * (1.f / 3.f);
        for (int k = 0; k < 3; k++) {
            lus[k] += lUF * F[k] + 3.f * lv[k];
            lF[k] += lUF * us[k];
        }
        lphi += 3.f * mu * ls;
        lmu += 3.f * ph * ls;
        float lm[3];
        for (int k = 0; k < 3; k++) {
            lF[k] += 0.5f * lus[k] * inv;
            lrho += -0.5f * lus[k] * F[k] * inv * inv;
            lm[k] = lus[k] * inv;
            lrho += -lus[k] * u[k] * inv;
        }
        for (int k = 0; k < 3; k++) lmu += gr[k] * lF[k];
        if (heavy) dg += lF[2];
        a.lgrad[t] = mu * lF[0];
        a.lgrad[n + t] = mu * lF[1];
        a.lgrad[2 * n + t] = mu * lF[2];
        lphi += c.alpha4 * (3.f * ph * ph - c.phiStarSq) * lmu;
        a.llap[t] = -c.kappa * lmu;
        if (a.add_source) {
            float dphi, drho, dmz;
            objective_source(b, t, a.objective, a.scale, a.ab, phiStar, ph, rh, m[2], dphi, drho, dmz);
            lphi += dphi;
            lrho += drho;
            lm[2] += dmz;
        }
        a.lf_out[t] = c.invTauPhiOne * lP[0] + lphi;
        for (int i = 1; i < kQf; i++) a.lf_out[i * n + t] = c.invTauPhiOne * lP[i] + lphi;
        for (int i = 0; i < kQg; i++)
            a.lg_out[i * n + t] =
                c.invTauRhoOne * lQ[i] + lrho + aCg[i][0] * lm[0] + aCg[i][1] * lm[1] + aCg[i][2] * lm[2];
    }
    dg = block_sum(dg, red);
    if (threadIdx.x == 0) a.dgrav_partials[blockIdx.x] = dg;
}

// lst = L[llap] - sum_k D_k[lgrad_k]: the transposed stencils.
__global__ void adjoint_stencil_kernel(Box b, const float *__restrict__ llap, const float *__restrict__ lgrad,
                                       float *__restrict__ lst)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        const Coord cd = coord(b, t);
        float l1, d0, d1, d2, gxv, gyv, gzv;
        stencil(b, llap, cd, l1, d0, d1, d2);
        stencil(b, lgrad, cd, d0, gxv, d1, d2);
        stencil(b, lgrad + b.n, cd, d0, d1, gyv, d2);
        stencil(b, lgrad + 2 * b.n, cd, d0, d1, d2, gzv);
        lst[t] = l1 - gxv - gyv - gzv;
    }
}

// acc[1] (dJ/dgrav) += sum of the partials.
__global__ void sum_fold_kernel(const double *__restrict__ partials, int nparts, double *__restrict__ acc)
{
    __shared__ double red[kThreads / 32];
    double s = 0.0;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) s += partials[p];
    s = block_sum(s, red);
    if (threadIdx.x == 0) acc[1] += s;
}

// dJ/dphi0 through the initial equilibrium (src/init_f.cu:57-78,
// src/init_g.cu:69-91), local part; llap receives lambda of the Laplacian.
__global__ void init_adjoint_kernel(Box b, float alpha4, float kappa, float phiStarSq, float Gamma,
                                    const float *__restrict__ phi0, const float *__restrict__ lf,
                                    const float *__restrict__ lst, const float *__restrict__ lg,
                                    float *__restrict__ lphi0, float *__restrict__ llap)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        const Coord cd = coord(b, t);
        float lap, gx, gy, gz;
        stencil(b, phi0, cd, lap, gx, gy, gz);
        const float ph = phi0[t];
        const float mu = alpha4 * ph * (ph * ph - phiStarSq) - kappa * lap;
        const float add = lst[t];
        const float l0 = lf[t] + add;
        float lfs = 0.f, lga = 0.f, lgd = 0.f;
        for (int i = 1; i < kQf; i++) lfs += lf[i * b.n + t] + add;
        for (int i = 1; i < 7; i++) lga += lg[i * b.n + t];
        for (int i = 7; i < kQg; i++) lgd += lg[i * b.n + t];
        const float lg0 = lg[t];
        const float lmu = -3.f * Gamma * l0 + 0.5f * Gamma * lfs - 6.f * kW0 * ph * lg0 + 3.f * kW1 * ph * lga
                          + 3.f * kW2 * ph * lgd;
        float lphi = l0 - 6.f * kW0 * mu * lg0 + 3.f * kW1 * mu * lga + 3.f * kW2 * mu * lgd;
        lphi += alpha4 * (3.f * ph * ph - phiStarSq) * lmu;
        llap[t] = -kappa * lmu;
        lphi0[t] = lphi;
    }
}

__global__ void init_adjoint_stencil_kernel(Box b, const float *__restrict__ llap, float *__restrict__ lphi0)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        float l1, d0, d1, d2;
        stencil(b, llap, coord(b, t), l1, d0, d1, d2);
        lphi0[t] += l1;
    }
}

unsigned grid_for(long long n)
{
    long long blocks = (n + kThreads - 1) / kThreads;
    if (blocks > 152 * 8) blocks = 152 * 8;
    return (unsigned)(blocks < 1 ? 1 : blocks);
}

}  // namespace

size_t adjoint_partial_count(const Box &b) { return grid_for(b.n); }

cudaError_t launch_phi(const Box &b, const float *F, float *phi, cudaStream_t s)
{
    phi_kernel<<<grid_for(b.n), kThreads, 0, s>>>(b, F, phi);
    return cudaGetLastError();
}

cudaError_t launch_objective(const Box &b, int objective, float phiStar, double scale, const float *phi,
                             const float *G, double *partials, double *ab, double *acc, cudaStream_t s)
{
    const unsigned blocks = grid_for(b.n);
    objective_kernel<<<blocks, kThreads, 0, s>>>(b, objective, phiStar, phi, G, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    objective_fold_kernel<<<1, kThreads, 0, s>>>(partials, (int)blocks, scale, ab, acc);
    return cudaGetLastError();
}

cudaError_t launch_source_init(const Box &b, int objective, double scale, const double *ab, float phiStar,
                               const float *phi, const float *G, float *lf, float *lg, float *lst, cudaStream_t s)
{
    source_init_kernel<<<grid_for(b.n), kThreads, 0, s>>>(b, objective, scale, ab, phiStar, phi, G, lf, lg, lst);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_step(const Box &b, const StepConst &c, float phiStar, const AdjointBuffers &a,
                                bool add_source, int objective, double scale, double *acc, cudaStream_t s)
{
    const unsigned blocks = grid_for(b.n);
    AdjIn in;
    in.F = a.F;
    in.G = a.G;
    in.phi = a.phi;
    in.lf = a.lf_in;
    in.lg = a.lg_in;
    in.lst = a.lst_in;
    in.lf_out = a.lf_out;
    in.lg_out = a.lg_out;
    in.llap = a.llap;
    in.lgrad = a.lgrad;
    in.dgrav_partials = a.partials;
    in.ab = a.ab;
    in.scale = scale;
    in.objective = objective;
    in.add_source = add_source ? 1 : 0;
    adjoint_local_kernel<<<blocks, kThreads, 0, s>>>(b, c, phiStar, in);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sum_fold_kernel<<<1, kThreads, 0, s>>>(a.partials, (int)blocks, acc);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    adjoint_stencil_kernel<<<grid_for(b.n), kThreads, 0, s>>>(b, a.llap, a.lgrad, a.lst_out);
    return cudaGetLastError();
}

cudaError_t launch_init_adjoint(const Box &b, const lbm_derived &d, float Gamma, const float *phi0, const float *lf,
                                const float *lst, const float *lg, float *lphi0, float *llap, cudaStream_t s)
{
    init_adjoint_kernel<<<grid_for(b.n), kThreads, 0, s>>>(b, d.alpha4, d.kappa, d.phiStarSq, Gamma, phi0, lf, lst,
                                                           lg, lphi0, llap);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    init_adjoint_stencil_kernel<<<grid_for(b.n), kThreads, 0, s>>>(b, llap, lphi0);
    return cudaGetLastError();
}

}  // namespace lbm
