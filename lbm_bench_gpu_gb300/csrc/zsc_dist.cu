// zsc_dist.cu -- conversion between the kernel's storage and the reference's
// streamed distributions (the lower halves of f_i / g_i after a step).
//
//  stream_out_kernel: f stored post-collision -> streamed value
//                     f_i(x) = eta P_i(x - c_i) + (1 - eta) P_i(x)
//                     (src/stream_f.cu:52-59); g in AA layout -> natural
//                     layout (after an even step the value for direction i at
//                     x sits in the reversed slot of the upstream node).
//  moments_kernel   : phi, rho, u from streamed f and g
//                     (src/update_phi.cu:42-43, src/update_rho.cu:46-50,
//                     src/update_velocity.cu:47-59).
#include "lbm_internal.h"

namespace lbm {
namespace {

__constant__ int kCf[kQf][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
__constant__ int kCg[kQg][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                {0, 0, 1},  {0, 0, -1},  {1, 1, 0},  {-1, -1, 0}, {1, -1, 0},
                                {-1, 1, 0}, {1, 0, 1},   {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
                                {0, 1, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
__constant__ int kOpp[kQg] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};

__device__ __forceinline__ long long shifted(const Box &b, int x, int y, int z, int dx, int dy, int dz)
{
    x += dx;
    y += dy;
    z += dz;
    x = x < 0 ? x + b.nx : (x >= b.nx ? x - b.nx : x);
    y = y < 0 ? y + b.ny : (y >= b.ny ? y - b.ny : y);
    z = z < 0 ? z + b.nz : (z >= b.nz ? z - b.nz : z);
    return x + (long long)b.nx * (y + (long long)b.ny * z);
}

// odd: the next step is odd, i.e. the last step was even and g is in the
// reversed layout.
__global__ void stream_out_kernel(Box b, float eta, const float *__restrict__ fs, int f_streamed,
                                  const float *__restrict__ g, int odd, float *__restrict__ fo,
                                  float *__restrict__ go)
{
    const float eta2 = 1.f - eta;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(t % b.nx), y = (int)((t / b.nx) % b.ny), z = (int)(t / b.nxy);
        if (fo) {
            fo[t] = fs[t];
            for (int i = 1; i < kQf; i++) {
                if (f_streamed) {
                    fo[i * b.n + t] = fs[i * b.n + t];
                } else {
                    const long long up = shifted(b, x, y, z, -kCf[i][0], -kCf[i][1], -kCf[i][2]);
                    fo[i * b.n + t] = eta * fs[i * b.n + up] + eta2 * fs[i * b.n + t];
                }
            }
        }
        if (go) {
            for (int i = 0; i < kQg; i++) {
                if (!odd) {
                    go[i * b.n + t] = g[i * b.n + t];
                } else {
                    const long long up = shifted(b, x, y, z, -kCg[i][0], -kCg[i][1], -kCg[i][2]);
                    go[i * b.n + t] = g[kOpp[i] * b.n + up];
                }
            }
        }
    }
}

__global__ void moments_kernel(Box b, const float *__restrict__ f, const float *__restrict__ g,
                               float *__restrict__ mom)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        float q[kQg];
        for (int i = 0; i < kQg; i++) q[i] = g[i * b.n + t];
        float phi = f[t];
        for (int i = 1; i < kQf; i++) phi += f[i * b.n + t];
        float rho = q[0];
        for (int i = 1; i < kQg; i++) rho += q[i];
        const float inv = 1.0f / rho;
        mom[t] = phi;
        mom[b.n + t] = rho;
        mom[2 * b.n + t] = (q[1] - q[2] + q[7] - q[8] + q[9] - q[10] + q[11] - q[12] + q[13] - q[14]) * inv;
        mom[3 * b.n + t] = (q[3] - q[4] + q[7] - q[8] - q[9] + q[10] + q[15] - q[16] + q[17] - q[18]) * inv;
        mom[4 * b.n + t] = (q[5] - q[6] + q[11] - q[12] - q[13] + q[14] + q[15] - q[16] - q[17] + q[18]) * inv;
    }
}

unsigned grid_for(long long n)
{
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    return (unsigned)(blocks < 1 ? 1 : blocks);
}

}  // namespace

cudaError_t launch_stream_out(const Box &b, float eta, const float *f_state, bool f_streamed, const float *g,
                              bool odd, float *f_out, float *g_out, cudaStream_t s)
{
    stream_out_kernel<<<grid_for(b.n), 256, 0, s>>>(b, eta, f_state, f_streamed ? 1 : 0, g, odd ? 1 : 0, f_out,
                                                    g_out);
    return cudaGetLastError();
}

cudaError_t launch_moments(const Box &b, const float *f, const float *g, float *mom, cudaStream_t s)
{
    moments_kernel<<<grid_for(b.n), 256, 0, s>>>(b, f, g, mom);
    return cudaGetLastError();
}

}  // namespace lbm
