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
// populations) and added when lambda is read.
//
// The forward state is read where the step kernel keeps it (a checkpoint slot
// or the context's buffers): f_0 FP32, f_1..f_6 post-collision (the eta-blend
// is redone on read), g in the AA layout, 16-bit formats mapped back to FP32.
// The collision's Jacobian needs g only through rho and the momentum, and f
// only through phi, so only phi is materialised (the stencil needs it at the
// neighbours).  Per step:
//   adjoint_phi_kernel     s^n -> phi                          ~32 B/node (FP32)
//   adjoint_local_kernel   lambda^{n+1}, s^n, phi -> lambda^n   ~320 B/node
//                          and (lambda_lap, mu lambda_F) as one float4
//   adjoint_stencil_kernel float4 -> lst                        ~20 B/node
// All per-node arithmetic is FP32; the objective sums and dJ/dgrav are FP64.
// Every kernel runs on one grid: 32 x 8 column tiles, each block marching
// kPlanes (4) consecutive z planes (so the z neighbours of one plane are the
// block's previous and next planes, mostly L1 hits), except the local kernel,
// whose blocks take kLocalPlanes (2) planes gridDim.z apart (with consecutive
// planes the compiler keeps more values live across iterations and spills),
// with the next plane's rows prefetched into L2.  Measured at 128^3 (T = 2000,
// 40 GB): 1, 2, 4 local planes -> adjoint/forward 4.06, 3.99, 4.09 (and, later,
// 3.92, 3.81, 3.87; at 256^3 with an FP16 state, T = 400: 6.21, 6.07, 6.12);
// 8 and 16 stencil planes are slower.  32-bit node indices (n * 19 < 2^32 is checked at
// init).
#include <algorithm>
#include <type_traits>

#include "lattice.cuh"

namespace lbm {
namespace {

constexpr int TXA = 32, TYA = 8, NTA = TXA * TYA;
#ifndef ZSC_ADJ_PLANES
#define ZSC_ADJ_PLANES 4
#endif
// Resident blocks per SM the local kernel's launch bounds ask for: 3 (80
// registers) for an FP32 state, 4 (64 registers, ~100 bytes spilled) for a
// 16-bit state, whose two-byte gathers leave more latency to hide.  Measured
// (adjoint / forward wall time): 256^3 FP16 state, T = 400, 40 GB: 2, 3, 4
// blocks -> 6.18, 6.07, 5.79; 128^3 FP32 state, T = 2000, 40 GB: 4.03, 3.81,
// 3.92.  ZSC_ADJ_MIN_BLOCKS overrides both.
template <typename ST>
constexpr int adj_min_blocks()
{
#ifdef ZSC_ADJ_MIN_BLOCKS
    return ZSC_ADJ_MIN_BLOCKS;
#else
    return sizeof(ST) == 2 ? 4 : 3;
#endif
}
#ifndef ZSC_ADJ_LOCAL_PLANES
#define ZSC_ADJ_LOCAL_PLANES 2
#endif
constexpr int kPlanes = ZSC_ADJ_PLANES;
constexpr int kLocalPlanes = ZSC_ADJ_LOCAL_PLANES;   // planes per block of the local kernel
constexpr float kInv6 = 0.16666666666666666667f;
constexpr float kInv12 = 0.08333333333333333333f;
constexpr float kW0 = 0.33333333333333333333f, kW1 = 0.05555555555555555556f, kW2 = 0.02777777777777777778f;

// Node indices of the 3 x 3 x 3 neighbourhood of (x, y, z), periodic.
struct Nb {
    unsigned X[3], Y[3], Z[3];
    __device__ __forceinline__ unsigned at(int dx, int dy, int dz) const { return X[dx + 1] + Y[dy + 1] + Z[dz + 1]; }
};

__device__ __forceinline__ Nb neighbourhood(const Box &b, int x, int y, int z)
{
    Nb r;
    const unsigned nx = (unsigned)b.nx, nxy = (unsigned)b.nxy;
    r.X[0] = x == 0 ? nx - 1 : x - 1;
    r.X[1] = x;
    r.X[2] = x == b.nx - 1 ? 0 : x + 1;
    r.Y[0] = (y == 0 ? b.ny - 1 : y - 1) * nx;
    r.Y[1] = y * nx;
    r.Y[2] = (y == b.ny - 1 ? 0 : y + 1) * nx;
    r.Z[0] = (z == 0 ? b.nz - 1 : z - 1) * nxy;
    r.Z[1] = z * nxy;
    r.Z[2] = (z == b.nz - 1 ? 0 : z + 1) * nxy;
    return r;
}

// The same neighbourhood as element indices of the state's fields (FP32:
// the node indices; 16-bit storage: the pair layout, see storage_index).
template <typename ST>
__device__ __forceinline__ Nb state_neighbourhood(const Box &b, int x, int y, int z)
{
    Nb r = neighbourhood(b, x, y, z);
    if constexpr (sizeof(ST) == 2) {
        const unsigned h = (unsigned)b.nx >> 1;
#pragma unroll
        for (int k = 0; k < 3; k++) r.X[k] = r.X[k] < h ? 2u * r.X[k] : 2u * (r.X[k] - h) + 1u;
    }
    return r;
}

__device__ __forceinline__ unsigned node_index_of(const Box &b, int x, int y, int z)
{
    return (unsigned)x + (unsigned)b.nx * ((unsigned)y + (unsigned)b.ny * (unsigned)z);
}

// index of the node at sign * c_i from the centre of p
__device__ __forceinline__ unsigned dir_at(const Nb &p, int i, int sign)
{
    return p.at(sign * kCx(i), sign * kCy(i), sign * kCz(i));
}

// 19-point Laplacian and gradient of field v at the centre of p
// (src/collision_f.cu:61-94), the stencil points taken in D3Q19 order.
__device__ __forceinline__ void stencil19(const float *__restrict__ v, const Nb &p, float &lap, float &gx, float &gy,
                                          float &gz)
{
    float s[kQg];
#pragma unroll
    for (int i = 0; i < kQg; i++) s[i] = __ldg(v + dir_at(p, i, 1));
    lap = (s[7] + s[8] + s[9] + s[10] + s[11] + s[12] + s[13] + s[14] + s[15] + s[16] + s[17] + s[18]
           + 2.f * (s[1] + s[2] + s[3] + s[4] + s[5] + s[6] - 12.f * s[0])) * kInv6;
    gx = (2.f * (s[1] - s[2]) + s[7] - s[8] + s[9] - s[10] + s[11] - s[12] + s[13] - s[14]) * kInv12;
    gy = (2.f * (s[3] - s[4]) + s[7] - s[8] + s[10] - s[9] + s[15] - s[16] + s[17] - s[18]) * kInv12;
    gz = (2.f * (s[5] - s[6]) + s[11] - s[12] + s[14] - s[13] + s[15] - s[16] + s[18] - s[17]) * kInv12;
}

// Per-field base pointers of a state (kernel parameters: a field's address is
// one multiply-add on the node index).
struct GFields {
    const void *f[kQg];       // g, AA layout
};
struct FQFields {
    const void *f[kQf - 1];   // f_1 .. f_6
};

// Streamed g_i at the centre of p, FP32.
template <typename ST, bool ODD>
__device__ __forceinline__ float g_streamed(const GFields &g, const Quant &q, const Nb &p, int i)
{
    const ST v = ODD ? static_cast<const ST *>(g.f[kOpp(i)])[dir_at(p, i, -1)]
                     : static_cast<const ST *>(g.f[i])[p.at(0, 0, 0)];
    if constexpr (Fmt<ST>::kMapped)
        return Fmt<ST>::load(v) * q.g_inv + q.g_shift[i];
    else
        return Fmt<ST>::load(v);
}

// rho and momentum of the streamed g at the centre of p.
template <typename ST, bool ODD>
__device__ __forceinline__ void g_moments(const GFields &g, const Quant &q, const Nb &p, float &rho, float m[3])
{
    rho = 0.f;
    m[0] = m[1] = m[2] = 0.f;
#pragma unroll
    for (int i = 0; i < kQg; i++) {
        const float gi = g_streamed<ST, ODD>(g, q, p, i);
        rho += gi;
        if (kCx(i)) m[0] += kCx(i) * gi;
        if (kCy(i)) m[1] += kCy(i) * gi;
        if (kCz(i)) m[2] += kCz(i) * gi;
    }
}

__device__ __forceinline__ double block_sum(double v, double *red)
{
    const int tid = threadIdx.y * TXA + threadIdx.x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (tid == 0)
        for (int w = 0; w < NTA / 32; w++) r += red[w];
    __syncthreads();
    return r;
}

__device__ __forceinline__ unsigned block_id() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }

// phi = sum of the streamed f of a native state.
template <typename ST>
__global__ void __launch_bounds__(NTA) adjoint_phi_kernel(Box b, float eta, Quant q, const float *__restrict__ f0,
                                                          const FQFields fq, int f_streamed,
                                                          float *__restrict__ phi)
{
    const float eta2 = 1.f - eta;
    const int x = blockIdx.x * TXA + threadIdx.x, y = blockIdx.y * TYA + threadIdx.y;
    for (int z = blockIdx.z * kPlanes, z_end = min(b.nz, z + kPlanes); z < z_end; z++) {
        const Nb p = state_neighbourhood<ST>(b, x, y, z);
        const unsigned ts = p.at(0, 0, 0);
        float s = f0[ts];
#pragma unroll
        for (int i = 1; i < kQf; i++) {
            const ST *a = static_cast<const ST *>(fq.f[i - 1]);
            const float inv = Fmt<ST>::kMapped ? q.f_inv : 1.f;
            const float here = Fmt<ST>::load(a[ts]) * inv;
            s += f_streamed ? here : eta * (Fmt<ST>::load(a[dir_at(p, i, -1)]) * inv) + eta2 * here;
        }
        phi[node_index_of(b, x, y, z)] = s;
    }
}

// Objective sums of one state: A = sum w q, B = sum w, with
// w = (phiStar - phi) / (2 phiStar) and q = u_z (objective 0) or the reference
// plane index z + 1 (objective 1); per-block partials.
template <typename ST, bool ODD>
__global__ void __launch_bounds__(NTA) objective_kernel(Box b, int objective, float phiStar, Quant q,
                                                        const GFields g, const float *__restrict__ phi,
                                                        double *__restrict__ partials)
{
    __shared__ double red[NTA / 32];
    const float half_inv = 0.5f / phiStar;
    double A = 0.0, B = 0.0;
    const int x = blockIdx.x * TXA + threadIdx.x, y = blockIdx.y * TYA + threadIdx.y;
    for (int z = blockIdx.z * kPlanes, z_end = min(b.nz, z + kPlanes); z < z_end; z++) {
        const float w = (phiStar - phi[node_index_of(b, x, y, z)]) * half_inv;
        float qv;
        if (objective == 0) {
            float rho, m[3];
            g_moments<ST, ODD>(g, q, state_neighbourhood<ST>(b, x, y, z), rho, m);
            qv = m[2] / rho;
        } else {
            qv = (float)(z + 1);
        }
        A += (double)(w * qv);
        B += (double)w;
    }
    A = block_sum(A, red);
    B = block_sum(B, red);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        partials[2 * block_id()] = A;
        partials[2 * block_id() + 1] = B;
    }
}

// ab[0..1] = sums of the partials, ab[2] = A / B, ab[3] = scale / B;
// acc[0] (J) += scale * A / B.
__global__ void __launch_bounds__(NTA) objective_fold_kernel(const double *__restrict__ partials, int nparts,
                                                             double scale, double *__restrict__ ab,
                                                             double *__restrict__ acc)
{
    __shared__ double red[NTA / 32];
    double A = 0.0, B = 0.0;
    for (int p = threadIdx.y * TXA + threadIdx.x; p < nparts; p += NTA) {
        A += partials[2 * p];
        B += partials[2 * p + 1];
    }
    A = block_sum(A, red);
    B = block_sum(B, red);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        ab[0] = A;
        ab[1] = B;
        ab[2] = A / B;
        ab[3] = scale / B;
        acc[0] += scale * A / B;
    }
}

// Per-launch coefficients of the objective's derivative: J += scale A / B
// gives dJ/dw = scale (q - A/B) / B and dJ/dq = scale w / B, with
// dw/dphi = -1 / (2 phiStar).
struct SourceCoef {
    float ratio;    // A / B
    float s_over_b; // scale / B
    float half_inv; // 1 / (2 phiStar)
};

__device__ __forceinline__ SourceCoef source_coef(const double *ab, float phiStar)
{
    SourceCoef k;
    k.ratio = (float)ab[2];
    k.s_over_b = (float)ab[3];
    k.half_inv = 0.5f / phiStar;
    return k;
}

// d(scale * A / B)/d(state) at a node of plane z (FP32 per node).
__device__ __forceinline__ void objective_source(int z, int objective, const SourceCoef &k, float phiStar, float ph,
                                                 float rho, float mz, float &dphi, float &drho, float &dmz)
{
    const float w = (phiStar - ph) * k.half_inv;
    if (objective == 0) {
        const float inv = 1.0f / rho;
        const float uz = mz * inv;
        dphi = -k.half_inv * k.s_over_b * (uz - k.ratio);
        const float duz = k.s_over_b * w;
        dmz = duz * inv;
        drho = -duz * uz * inv;
    } else {
        dphi = -k.half_inv * k.s_over_b * ((float)(z + 1) - k.ratio);
        drho = 0.f;
        dmz = 0.f;
    }
}

// lambda^T: only the objective source of the final state.
template <typename ST, bool ODD>
__global__ void __launch_bounds__(NTA) source_init_kernel(Box b, int objective, double scale,
                                                          const double *__restrict__ ab, float phiStar, Quant q,
                                                          const GFields g, const float *__restrict__ phi,
                                                          float *__restrict__ lf, float *__restrict__ lg,
                                                          float *__restrict__ lst)
{
    const unsigned n = (unsigned)b.n;
    const SourceCoef k = source_coef(ab, phiStar);
    const int x = blockIdx.x * TXA + threadIdx.x, y = blockIdx.y * TYA + threadIdx.y;
    for (int z = blockIdx.z * kPlanes, z_end = min(b.nz, z + kPlanes); z < z_end; z++) {
        const unsigned t = node_index_of(b, x, y, z);
        float rho, m[3];
        g_moments<ST, ODD>(g, q, state_neighbourhood<ST>(b, x, y, z), rho, m);
        float dphi, drho, dmz;
        objective_source(z, objective, k, phiStar, phi[t], rho, m[2], dphi, drho, dmz);
#pragma unroll
        for (int i = 0; i < kQf; i++) lf[i * n + t] = dphi;
#pragma unroll
        for (int i = 0; i < kQg; i++) lg[i * n + t] = drho + kCz(i) * dmz;
        lst[t] = 0.f;
    }
}

struct AdjIn {
    // per-field base pointers (kernel parameters: a field's address is one
    // multiply-add on the node index, with no i * n on the load's path)
    const void *g_f[kQg];                  // the state's g fields
    const float *lf_f[kQf], *lg_f[kQg];    // lambda^{n+1}
    float *lf_o[kQf], *lg_o[kQg];          // lambda^n
    const void *g;                         // native g of s^n
    const float *phi;                      // phi of s^n
    const float *lf, *lg, *lst;            // lambda^{n+1} (lf without its stencil part lst)
    float *lf_out, *lg_out;                // lambda^n without its stencil part
    float4 *lsrc;                          // (lambda_lap, mu lambda_F) at every node
    double *dgrav;                         // per warp of each block, accumulated over steps
    const double *ab;                      // objective sums of s^n (when add_source)
    double scale;
    int objective, add_source;
};

// L2 prefetch of the block's tile rows of plane z in every field the local
// kernel reads (lambda_g, lambda_f, lst, g, phi): one bulk prefetch per row
// (128 B of floats, 32 storage elements of g), about 1.5 per thread.  The
// kernel is latency-bound on its neighbour gathers; with the rows already on
// their way to L2 they hit there.  The blocks of neighbouring tiles and planes
// (which run at the same time) prefetch the halo rows.
template <typename ST>
__device__ __forceinline__ void prefetch_plane(const Box &b, const AdjIn &a, int z)
{
    constexpr int kFields = kQg + kQf + 1 + kQg + 1;
    const unsigned n = (unsigned)b.n;
    const int tid = threadIdx.y * TXA + threadIdx.x;
    for (int r = tid; r < kFields * TYA; r += NTA) {
        const int field = r / TYA;
        const unsigned node =
            (unsigned)z * (unsigned)b.nxy + (blockIdx.y * TYA + (unsigned)(r % TYA)) * (unsigned)b.nx + blockIdx.x * TXA;
        const void *src;
        unsigned bytes = TXA * sizeof(float);
        if (field < kQg) {
            src = a.lg + field * n + node;
        } else if (field < kQg + kQf) {
            src = a.lf + (field - kQg) * n + node;
        } else if (field == kQg + kQf) {
            src = a.lst + node;
        } else if (field < 2 * kQg + kQf + 1) {
            // the tile row's nodes in the state's layout: FP32 the node range;
            // pair layout the 32 words holding them (and the other half's)
            unsigned first = node, count = TXA;
            if constexpr (sizeof(ST) == 2) {
                const unsigned h = (unsigned)b.nx >> 1, x0 = blockIdx.x * TXA;
                first = node - x0 + 2u * (x0 < h ? x0 : x0 - h);
                count = 2 * TXA;
            }
            src = static_cast<const ST *>(a.g) + (field - kQg - kQf - 1) * n + first;
            bytes = count * sizeof(ST);
        } else {
            src = a.phi + node;
        }
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(src), "r"(bytes) : "memory");
    }
}

// The local part of one adjoint step (see the file comment).
template <typename ST, bool ODD>
__global__ void __launch_bounds__(NTA, adj_min_blocks<ST>()) adjoint_local_kernel(Box b, StepConst c, float phiStar, Quant q, AdjIn a)
{
    double dg = 0.0;
    const int x = blockIdx.x * TXA + threadIdx.x, y = blockIdx.y * TYA + threadIdx.y;
    if (blockIdx.z < (unsigned)b.nz) prefetch_plane<ST>(b, a, blockIdx.z);
    for (int z = blockIdx.z; z < b.nz; z += gridDim.z) {
        if (z + (int)gridDim.z < b.nz) prefetch_plane<ST>(b, a, z + gridDim.z);
        const Nb p = neighbourhood(b, x, y, z);
        const unsigned t = p.at(0, 0, 0);
        float lap, gr[3];
        stencil19(a.phi, p, lap, gr[0], gr[1], gr[2]);
        const float ph = __ldg(a.phi + t);
        float rh = 0.f, m[3] = {0.f, 0.f, 0.f};
        const Nb ps = state_neighbourhood<ST>(b, x, y, z);
#pragma unroll
        for (int i = 0; i < kQg; i++) {
            const ST v = ODD ? static_cast<const ST *>(a.g_f[kOpp(i)])[dir_at(ps, i, -1)]
                             : static_cast<const ST *>(a.g_f[i])[ps.at(0, 0, 0)];
            float gi = Fmt<ST>::load(v);
            if constexpr (Fmt<ST>::kMapped) gi = gi * q.g_inv + q.g_shift[i];
            rh += gi;
            if (kCx(i)) m[0] += kCx(i) * gi;
            if (kCy(i)) m[1] += kCy(i) * gi;
            if (kCz(i)) m[2] += kCz(i) * gi;
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
        const float lst_here = __ldg(a.lst + t);
        lP[0] = __ldg(a.lf_f[0] + t) + lst_here;
#pragma unroll
        for (int i = 1; i < kQf; i++) {
            const unsigned dn = dir_at(p, i, 1);
            lP[i] = c.eta * (__ldg(a.lf_f[i] + dn) + __ldg(a.lst + dn)) + c.eta2 * (__ldg(a.lf_f[i] + t) + lst_here);
        }
#pragma unroll
        for (int i = 0; i < kQg; i++) lQ[i] = __ldg(a.lg_f[i] + dir_at(p, i, 1));

        // D3Q7 collision
        float lphi = 0.f, lmu = 0.f, lus[3] = {0.f, 0.f, 0.f}, lF[3] = {0.f, 0.f, 0.f}, lrho = 0.f;
        {
            const float lAf = -6.f * lP[0] + lP[1] + lP[2] + lP[3] + lP[4] + lP[5] + lP[6];
            float lCf = 0.f;
#pragma unroll
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
#pragma unroll
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
            constexpr int PA[6] = {0, 0, 0, 0, 1, 1}, PB[6] = {1, 1, 2, 2, 2, 2};
            constexpr float SG[6] = {1.f, -1.f, 1.f, -1.f, 1.f, -1.f};
            float ltemp2 = 0.f;
#pragma unroll
            for (int pp = 0; pp < 6; pp++) {
                const int ia = PA[pp], ib = PB[pp];
                const float sg = SG[pp];
                const float w = v[ia] + sg * v[ib], Gs = F[ia] + sg * F[ib];
                const float S = lQ[7 + 2 * pp] + lQ[8 + 2 * pp], A = lQ[7 + 2 * pp] - lQ[8 + 2 * pp];
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
#pragma unroll
        for (int k = 0; k < 3; k++) lv[k] += lvsq6 * v[k] * (1.f / 3.f);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            lus[k] += lUF * F[k] + 3.f * lv[k];
            lF[k] += lUF * us[k];
        }
        lphi += 3.f * mu * ls;
        lmu += 3.f * ph * ls;
        float lm[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            lF[k] += 0.5f * lus[k] * inv;
            lrho += -0.5f * lus[k] * F[k] * inv * inv;
            lm[k] = lus[k] * inv;
            lrho += -lus[k] * u[k] * inv;
        }
#pragma unroll
        for (int k = 0; k < 3; k++) lmu += gr[k] * lF[k];
        if (heavy) dg += lF[2];
        lphi += c.alpha4 * (3.f * ph * ph - c.phiStarSq) * lmu;
        a.lsrc[t] = make_float4(-c.kappa * lmu, mu * lF[0], mu * lF[1], mu * lF[2]);
        if (a.add_source) {
            float dphi, drho, dmz;
            objective_source(z, a.objective, source_coef(a.ab, phiStar), phiStar, ph, rh, m[2], dphi, drho, dmz);
            lphi += dphi;
            lrho += drho;
            lm[2] += dmz;
        }
#pragma unroll
        for (int i = 0; i < kQf; i++) a.lf_o[i][t] = c.invTauPhiOne * lP[i] + lphi;
#pragma unroll
        for (int i = 0; i < kQg; i++) {
            float o = c.invTauRhoOne * lQ[i] + lrho;
            if (kCx(i)) o += kCx(i) * lm[0];
            if (kCy(i)) o += kCy(i) * lm[1];
            if (kCz(i)) o += kCz(i) * lm[2];
            a.lg_o[i][t] = o;
        }
    }
    // per-warp sums into the warp's own slot: no block barrier, so warps that
    // finish early leave at once (with a block reduction here they waited for
    // the block's slowest warp: 1.5 barrier stalls per issued instruction at
    // 160^3 with an FP16 state), and the FP64 sums stay in a fixed order
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dg += __shfl_down_sync(0xffffffffu, dg, o);
    if (threadIdx.x == 0) a.dgrav[block_id() * (NTA / 32) + threadIdx.y] += dg;
}

// lst = L[lambda_lap] - sum_k D_k[lambda_grad_k]: the transposed stencils.
// Laplacian weights: 2/6 on faces, 1/6 on edges, -4 at the centre; gradient
// component k: c_ik times 2/12 on faces, 1/12 on edges.
//
// The block marches its kPlanes planes with a ring of three planes of the
// float4 source in shared memory, each on the tile plus a one-node ring
// (34 x 10), split into its four components so that a node reads the 49
// scalars it needs (lambda_lap at 19 points, each gradient component at the
// 10 points with c_k != 0) without bank conflicts.  Plane z + 2 is read into
// registers before plane z is computed (its loads overlap the computation) and
// stored into the slot plane z - 1 frees; each thread's staging coordinates
// are computed once.
constexpr int SW = TXA + 2, SH = TYA + 2, SPLANE = SW * SH;

__global__ void __launch_bounds__(NTA) adjoint_stencil_kernel(Box b, const float4 *__restrict__ lsrc,
                                                              float *__restrict__ lst)
{
    __shared__ float sm[3][4][SPLANE];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TXA + tx;
    const int x0 = blockIdx.x * TXA, y0 = blockIdx.y * TYA;
    const int z_begin = blockIdx.z * kPlanes, z_end = min(b.nz, z_begin + kPlanes);
    const unsigned nx = (unsigned)b.nx;
    // the (up to two) ring-tile nodes this thread stages, as in-plane offsets
    // (periodic in x and y), fixed for the block
    auto xy_of = [&](int e) {
        const int r = e / SW, c = e - r * SW;
        int gx = x0 - 1 + c, gy = y0 - 1 + r;
        gx = gx < 0 ? gx + b.nx : (gx >= b.nx ? gx - b.nx : gx);
        gy = gy < 0 ? gy + b.ny : (gy >= b.ny ? gy - b.ny : gy);
        return (unsigned)gy * nx + (unsigned)gx;
    };
    const int e0 = tid, e1 = tid + NTA;
    const bool two = e1 < SPLANE;
    const unsigned xy0 = xy_of(e0), xy1 = two ? xy_of(e1) : 0u;
    float4 v0, v1;
    auto fetch = [&](int z) {   // plane z into registers (its loads stay in flight)
        const int zw = z < 0 ? z + b.nz : (z >= b.nz ? z - b.nz : z);
        const unsigned zo = (unsigned)zw * (unsigned)b.nxy;
        v0 = __ldg(lsrc + zo + xy0);
        if (two) v1 = __ldg(lsrc + zo + xy1);
    };
    auto put = [&](int z) {     // ... and into its ring slot, components apart
        const int slot = (z + 3) % 3;
        sm[slot][0][e0] = v0.x;
        sm[slot][1][e0] = v0.y;
        sm[slot][2][e0] = v0.z;
        sm[slot][3][e0] = v0.w;
        if (two) {
            sm[slot][0][e1] = v1.x;
            sm[slot][1][e1] = v1.y;
            sm[slot][2][e1] = v1.z;
            sm[slot][3][e1] = v1.w;
        }
    };
    for (int z = z_begin - 1; z <= min(z_begin + 1, z_end); z++) {
        fetch(z);
        put(z);
    }
    __syncthreads();
    const int cell = (ty + 1) * SW + tx + 1;
    for (int z = z_begin; z < z_end; z++) {
        // plane z + 2 is read from memory while plane z is computed
        const bool next = z + 2 <= z_end;
        if (next) fetch(z + 2);
        float lface = 0.f, ledge = 0.f, dface = 0.f, dedge = 0.f;
#pragma unroll
        for (int i = 1; i < kQg; i++) {
            const int slot = (z + kCz(i) + 3) % 3;
            const int at = cell + kCy(i) * SW + kCx(i);
            const float lx = sm[slot][0][at];
            float d = 0.f;
            if (kCx(i)) d += kCx(i) * sm[slot][1][at];
            if (kCy(i)) d += kCy(i) * sm[slot][2][at];
            if (kCz(i)) d += kCz(i) * sm[slot][3][at];
            if (i < 7) {
                lface += lx;
                dface += d;
            } else {
                ledge += lx;
                dedge += d;
            }
        }
        const float c0 = sm[z % 3][0][cell];
        const float L = (ledge + 2.f * (lface - 12.f * c0)) * kInv6;
        const float D = (2.f * dface + dedge) * kInv12;
        lst[(unsigned)z * (unsigned)b.nxy + (unsigned)(y0 + ty) * nx + (unsigned)(x0 + tx)] = L - D;
        __syncthreads();          // plane z - 1's slot is free (z + 2 takes it)
        if (next) put(z + 2);
        __syncthreads();
    }
}

// acc[1] (dJ/dgrav) = sum of the per-warp sums.
__global__ void __launch_bounds__(NTA) dgrav_fold_kernel(const double *__restrict__ parts, int nparts,
                                                         double *__restrict__ acc)
{
    __shared__ double red[NTA / 32];
    double s = 0.0;
    for (int p = threadIdx.y * TXA + threadIdx.x; p < nparts; p += NTA) s += parts[p];
    s = block_sum(s, red);
    if (threadIdx.x == 0 && threadIdx.y == 0) acc[1] = s;
}

// dJ/dphi0 through the initial equilibrium (src/init_f.cu:57-78,
// src/init_g.cu:69-91), local part; llap receives lambda of the Laplacian.
__global__ void __launch_bounds__(NTA) init_adjoint_kernel(Box b, float alpha4, float kappa, float phiStarSq,
                                                           float Gamma, const float *__restrict__ phi0,
                                                           const float *__restrict__ lf,
                                                           const float *__restrict__ lst,
                                                           const float *__restrict__ lg, float *__restrict__ lphi0,
                                                           float *__restrict__ llap)
{
    const unsigned n = (unsigned)b.n;
    const int x = blockIdx.x * TXA + threadIdx.x, y = blockIdx.y * TYA + threadIdx.y;
    for (int z = blockIdx.z * kPlanes, z_end = min(b.nz, z + kPlanes); z < z_end; z++) {
        const Nb p = neighbourhood(b, x, y, z);
        const unsigned t = p.at(0, 0, 0);
        float lap, gx, gy, gz;
        stencil19(phi0, p, lap, gx, gy, gz);
        const float ph = phi0[t];
        const float mu = alpha4 * ph * (ph * ph - phiStarSq) - kappa * lap;
        const float add = lst[t];
        const float l0 = lf[t] + add;
        float lfs = 0.f, lga = 0.f, lgd = 0.f;
        for (int i = 1; i < kQf; i++) lfs += lf[i * n + t] + add;
        for (int i = 1; i < 7; i++) lga += lg[i * n + t];
        for (int i = 7; i < kQg; i++) lgd += lg[i * n + t];
        const float lg0 = lg[t];
        const float lmu = -3.f * Gamma * l0 + 0.5f * Gamma * lfs - 6.f * kW0 * ph * lg0 + 3.f * kW1 * ph * lga
                          + 3.f * kW2 * ph * lgd;
        float lphi = l0 - 6.f * kW0 * mu * lg0 + 3.f * kW1 * mu * lga + 3.f * kW2 * mu * lgd;
        lphi += alpha4 * (3.f * ph * ph - phiStarSq) * lmu;
        llap[t] = -kappa * lmu;
        lphi0[t] = lphi;
    }
}

__global__ void __launch_bounds__(NTA) init_adjoint_stencil_kernel(Box b, const float *__restrict__ llap,
                                                                   float *__restrict__ lphi0)
{
    const int x = blockIdx.x * TXA + threadIdx.x, y = blockIdx.y * TYA + threadIdx.y;
    for (int z = blockIdx.z * kPlanes, z_end = min(b.nz, z + kPlanes); z < z_end; z++) {
        const Nb p = neighbourhood(b, x, y, z);
        float l1, d0, d1, d2;
        stencil19(llap, p, l1, d0, d1, d2);
        lphi0[p.at(0, 0, 0)] += l1;
    }
}

dim3 adjoint_grid(const Box &b)
{
    return dim3((unsigned)(b.nx / TXA), (unsigned)(b.ny / TYA), (unsigned)((b.nz + kPlanes - 1) / kPlanes));
}

// the local kernel's grid (its blocks take planes gridDim.z apart)
dim3 local_grid(const Box &b)
{
    return dim3((unsigned)(b.nx / TXA), (unsigned)(b.ny / TYA), (unsigned)((b.nz + kLocalPlanes - 1) / kLocalPlanes));
}

size_t blocks_of(const dim3 &g) { return (size_t)g.x * g.y * g.z; }

const dim3 kBlock(TXA, TYA);

// fn(ST{}, std::integral_constant<bool, ODD>{}) for the state's storage type and g layout.
template <typename Fn>
cudaError_t dispatch(const NativeState &st, Fn &&fn)
{
    auto with = [&](auto tag) { return st.g_odd ? fn(tag, std::true_type{}) : fn(tag, std::false_type{}); };
    switch (st.storage) {
    case LBM_STORAGE_FP32: return with(float{});
    case LBM_STORAGE_FP16: return with(__half{});
    case LBM_STORAGE_BF16: return with(__nv_bfloat16{});
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

// per-field pointers of a native state
GFields g_fields(const Box &b, const NativeState &st)
{
    GFields r;
    const size_t stride = (size_t)b.n * storage_bytes(st.storage);
    for (int i = 0; i < kQg; i++) r.f[i] = static_cast<const unsigned char *>(st.g) + (size_t)i * stride;
    return r;
}
FQFields fq_fields(const Box &b, const NativeState &st)
{
    FQFields r;
    const size_t stride = (size_t)b.n * storage_bytes(st.storage);
    for (int i = 0; i < kQf - 1; i++) r.f[i] = static_cast<const unsigned char *>(st.fq) + (size_t)i * stride;
    return r;
}

size_t adjoint_dgrav_parts(const Box &b) { return blocks_of(local_grid(b)) * (NTA / 32); }

size_t adjoint_blocks(const Box &b)
{
    return std::max(blocks_of(adjoint_grid(b)), blocks_of(local_grid(b)));
}

cudaError_t launch_adjoint_phi(const Box &b, float eta, const Quant &q, const NativeState &st, float *phi,
                               cudaStream_t s)
{
    NativeState even = st;
    even.g_odd = false;   // phi does not read g
    return dispatch(even, [&](auto tag, auto) {
        using ST = decltype(tag);
        adjoint_phi_kernel<ST><<<adjoint_grid(b), kBlock, 0, s>>>(b, eta, q, st.f0, fq_fields(b, st),
                                                                 st.f_streamed ? 1 : 0, phi);
        return cudaGetLastError();
    });
}

cudaError_t launch_objective(const Box &b, int objective, float phiStar, double scale, const Quant &q,
                             const NativeState &st, const float *phi, double *partials, double *ab, double *acc,
                             cudaStream_t s)
{
    cudaError_t e = dispatch(st, [&](auto tag, auto odd) {
        using ST = decltype(tag);
        objective_kernel<ST, decltype(odd)::value><<<adjoint_grid(b), kBlock, 0, s>>>(
            b, objective, phiStar, q, g_fields(b, st), phi, partials);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    objective_fold_kernel<<<1, kBlock, 0, s>>>(partials, (int)blocks_of(adjoint_grid(b)), scale, ab, acc);
    return cudaGetLastError();
}

cudaError_t launch_source_init(const Box &b, int objective, double scale, const double *ab, float phiStar,
                               const Quant &q, const NativeState &st, const float *phi, float *lf, float *lg,
                               float *lst, cudaStream_t s)
{
    return dispatch(st, [&](auto tag, auto odd) {
        using ST = decltype(tag);
        source_init_kernel<ST, decltype(odd)::value><<<adjoint_grid(b), kBlock, 0, s>>>(
            b, objective, scale, ab, phiStar, q, g_fields(b, st), phi, lf, lg, lst);
        return cudaGetLastError();
    });
}

cudaError_t launch_adjoint_step(const Box &b, const StepConst &c, float phiStar, const Quant &q,
                                const NativeState &st, const AdjointBuffers &a, bool add_source, int objective,
                                double scale, cudaStream_t s)
{
    AdjIn in;
    in.g = st.g;
    in.phi = a.phi;
    in.lf = a.lf_in;
    in.lg = a.lg_in;
    in.lst = a.lst_in;
    in.lf_out = a.lf_out;
    in.lg_out = a.lg_out;
    const size_t n = (size_t)b.n, esz = storage_bytes(st.storage);
    for (int i = 0; i < kQg; i++) {
        in.g_f[i] = static_cast<const unsigned char *>(st.g) + (size_t)i * n * esz;
        in.lg_f[i] = a.lg_in + (size_t)i * n;
        in.lg_o[i] = a.lg_out + (size_t)i * n;
    }
    for (int i = 0; i < kQf; i++) {
        in.lf_f[i] = a.lf_in + (size_t)i * n;
        in.lf_o[i] = a.lf_out + (size_t)i * n;
    }
    in.lsrc = a.lsrc;
    in.dgrav = a.dgrav;
    in.ab = a.ab;
    in.scale = scale;
    in.objective = objective;
    in.add_source = add_source ? 1 : 0;
    cudaError_t e = dispatch(st, [&](auto tag, auto odd) {
        adjoint_local_kernel<decltype(tag), decltype(odd)::value>
            <<<local_grid(b), kBlock, 0, s>>>(b, c, phiStar, q, in);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    adjoint_stencil_kernel<<<adjoint_grid(b), kBlock, 0, s>>>(b, a.lsrc, a.lst_out);
    return cudaGetLastError();
}

cudaError_t launch_dgrav_fold(const Box &b, const double *dgrav, double *acc, cudaStream_t s)
{
    dgrav_fold_kernel<<<1, kBlock, 0, s>>>(dgrav, (int)adjoint_dgrav_parts(b), acc);
    return cudaGetLastError();
}

cudaError_t launch_init_adjoint(const Box &b, const lbm_derived &d, float Gamma, const float *phi0, const float *lf,
                                const float *lst, const float *lg, float *lphi0, float *llap, cudaStream_t s)
{
    init_adjoint_kernel<<<adjoint_grid(b), kBlock, 0, s>>>(b, d.alpha4, d.kappa, d.phiStarSq, Gamma, phi0, lf, lst,
                                                           lg, lphi0, llap);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    init_adjoint_stencil_kernel<<<adjoint_grid(b), kBlock, 0, s>>>(b, llap, lphi0);
    return cudaGetLastError();
}

}  // namespace lbm
