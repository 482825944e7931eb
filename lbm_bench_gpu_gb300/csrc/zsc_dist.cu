// zsc_dist.cu -- conversion between the kernel's storage and the reference's
// streamed FP32 distributions (the lower halves of f_i / g_i after a step).
//
//  stream_out_kernel: state -> streamed FP32.  f is stored post-collision, so
//                     f_i(x) = eta P_i(x - c_i) + (1 - eta) P_i(x)
//                     (src/stream_f.cu:52-59); g in the AA layout is read from
//                     the reversed slot of the upstream node when the next step
//                     is odd; 16-bit storage is mapped back to FP32.
//  quantize_kernel  : streamed FP32 -> state (its layout, storage map).
//  maxabs_kernel    : per-field max |value - shift|, to choose the 16-bit scales.
//  moments_kernel   : phi, rho, u from streamed f and g
//                     (src/update_phi.cu:42-43, src/update_rho.cu:46-50,
//                     src/update_velocity.cu:47-59).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "lattice.cuh"

namespace lbm {
namespace {

__constant__ int kCf[kQf][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
__constant__ int kCg[kQg][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                {0, 0, 1},  {0, 0, -1},  {1, 1, 0},  {-1, -1, 0}, {1, -1, 0},
                                {-1, 1, 0}, {1, 0, 1},   {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
                                {0, 1, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
__constant__ int kOppTab[kQg] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__half v) { return __half2float(v); }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
template <typename ST>
__device__ __forceinline__ ST from_f(float v);
template <>
__device__ __forceinline__ float from_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half from_f<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// node index of (x + dx, y + dy, z + dz), periodic; its x in *xo
__device__ __forceinline__ long long shifted(const Box &b, int x, int y, int z, int dx, int dy, int dz, int *xo)
{
    x += dx;
    y += dy;
    z += dz;
    x = x < 0 ? x + b.nx : (x >= b.nx ? x - b.nx : x);
    y = y < 0 ? y + b.ny : (y >= b.ny ? y - b.ny : y);
    z = z < 0 ? z + b.nz : (z >= b.nz ? z - b.nz : z);
    *xo = x;
    return x + (long long)b.nx * (y + (long long)b.ny * z);
}

// odd: the next step is odd, i.e. the last step was even and g is in the
// reversed layout.
template <typename ST>
__global__ void stream_out_kernel(Box b, float eta, Quant q, const float *__restrict__ f0, const ST *__restrict__ fq,
                                  int f_streamed, const ST *__restrict__ g, int odd, float *__restrict__ fo,
                                  float *__restrict__ go)
{
    const float eta2 = 1.f - eta;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(t % b.nx), y = (int)((t / b.nx) % b.ny), z = (int)(t / b.nxy);
        const unsigned st = storage_index<ST>(b, (unsigned)t, x);   // this node in the state's layout
        int ux = 0;
        if (fo) {
            fo[t] = f0[st];
            for (int i = 1; i < kQf; i++) {
                const float inv = q.f_inv;
                const ST *a = fq + (i - 1) * b.n;
                if (f_streamed) {
                    fo[i * b.n + t] = to_f(a[st]) * inv;
                } else {
                    const long long up = shifted(b, x, y, z, -kCf[i][0], -kCf[i][1], -kCf[i][2], &ux);
                    fo[i * b.n + t] = eta * (to_f(a[storage_index<ST>(b, (unsigned)up, ux)]) * inv)
                                      + eta2 * (to_f(a[st]) * inv);
                }
            }
        }
        if (go) {
            for (int i = 0; i < kQg; i++) {
                float v;
                if (!odd) {
                    v = to_f(g[i * b.n + st]);
                } else {
                    const long long up = shifted(b, x, y, z, -kCg[i][0], -kCg[i][1], -kCg[i][2], &ux);
                    v = to_f(g[kOppTab[i] * b.n + storage_index<ST>(b, (unsigned)up, ux)]);
                }
                go[i * b.n + t] = v * q.g_inv + q.g_shift[i];
            }
        }
    }
}

template <typename ST>
__global__ void quantize_kernel(Box b, Quant q, const float *__restrict__ f, const float *__restrict__ g,
                                float *__restrict__ f0, ST *__restrict__ fq, ST *__restrict__ gq)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        const unsigned st = storage_index<ST>(b, (unsigned)t, (int)(t % b.nx));
        f0[st] = f[t];
        for (int i = 1; i < kQf; i++) fq[(i - 1) * b.n + st] = from_f<ST>(f[i * b.n + t] * q.f_scale);
        for (int i = 0; i < kQg; i++) gq[i * b.n + st] = from_f<ST>((g[i * b.n + t] - q.g_shift[i]) * q.g_scale);
    }
}

// out_bits[field] = bits of max |x - shift| (non-negative floats order like
// their bit patterns, so an unsigned atomicMax is exact); fields 0..6 are f,
// 7..25 are g.
__global__ void maxabs_kernel(Box b, const float *__restrict__ f, const float *__restrict__ g,
                              const float *__restrict__ g_shift, unsigned *__restrict__ out_bits)
{
    const int field = blockIdx.y;
    const float *src = field < kQf ? f + field * b.n : g + (field - kQf) * b.n;
    const float shift = field < kQf ? 0.f : g_shift[field - kQf];
    float m = 0.f;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(src[t] - shift));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out_bits + field, __float_as_uint(m));
}

__global__ void moments_kernel(Box b, const float *__restrict__ f, const float *__restrict__ g,
                               float *__restrict__ mom)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < b.n;
         t += (long long)gridDim.x * blockDim.x) {
        float qv[kQg];
        for (int i = 0; i < kQg; i++) qv[i] = g[i * b.n + t];
        float phi = f[t];
        for (int i = 1; i < kQf; i++) phi += f[i * b.n + t];
        float rho = qv[0];
        for (int i = 1; i < kQg; i++) rho += qv[i];
        const float inv = 1.0f / rho;
        mom[t] = phi;
        mom[b.n + t] = rho;
        mom[2 * b.n + t] = (qv[1] - qv[2] + qv[7] - qv[8] + qv[9] - qv[10] + qv[11] - qv[12] + qv[13] - qv[14]) * inv;
        mom[3 * b.n + t] = (qv[3] - qv[4] + qv[7] - qv[8] - qv[9] + qv[10] + qv[15] - qv[16] + qv[17] - qv[18]) * inv;
        mom[4 * b.n + t] = (qv[5] - qv[6] + qv[11] - qv[12] - qv[13] + qv[14] + qv[15] - qv[16] - qv[17] + qv[18]) * inv;
    }
}

unsigned grid_for(long long n)
{
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    return (unsigned)(blocks < 1 ? 1 : blocks);
}

template <typename ST>
cudaError_t stream_out_typed(const Box &b, float eta, const Quant &q, const StepView &v, bool f_streamed, bool odd,
                             float *f_out, float *g_out, cudaStream_t s)
{
    stream_out_kernel<ST><<<grid_for(b.n), 256, 0, s>>>(b, eta, q, v.f0_in, static_cast<const ST *>(v.fq_in),
                                                        f_streamed ? 1 : 0, static_cast<const ST *>(v.g), odd ? 1 : 0,
                                                        f_out, g_out);
    return cudaGetLastError();
}

template <typename ST>
cudaError_t quantize_typed(const Box &b, const Quant &q, const float *f, const float *g, float *f0, void *fq, void *gq,
                           cudaStream_t s)
{
    quantize_kernel<ST><<<grid_for(b.n), 256, 0, s>>>(b, q, f, g, f0, static_cast<ST *>(fq), static_cast<ST *>(gq));
    return cudaGetLastError();
}

}  // namespace

size_t storage_bytes(int storage) { return storage == LBM_STORAGE_FP32 ? 4 : 2; }

cudaError_t launch_stream_out(const Box &b, float eta, const Quant &q, const StepView &v, bool f_streamed, bool odd,
                              float *f_out, float *g_out, cudaStream_t s)
{
    switch (v.storage) {
    case LBM_STORAGE_FP32: return stream_out_typed<float>(b, eta, q, v, f_streamed, odd, f_out, g_out, s);
    case LBM_STORAGE_FP16: return stream_out_typed<__half>(b, eta, q, v, f_streamed, odd, f_out, g_out, s);
    case LBM_STORAGE_BF16: return stream_out_typed<__nv_bfloat16>(b, eta, q, v, f_streamed, odd, f_out, g_out, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_quantize(const Box &b, const Quant &q, int storage, const float *f, const float *g, float *f0,
                            void *fq, void *gq, cudaStream_t s)
{
    switch (storage) {
    case LBM_STORAGE_FP32: return quantize_typed<float>(b, q, f, g, f0, fq, gq, s);
    case LBM_STORAGE_FP16: return quantize_typed<__half>(b, q, f, g, f0, fq, gq, s);
    case LBM_STORAGE_BF16: return quantize_typed<__nv_bfloat16>(b, q, f, g, f0, fq, gq, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_field_maxabs(const Box &b, const float *f, const float *g, const float *g_shift_dev,
                                unsigned *out_bits, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out_bits, 0, sizeof(unsigned) * (kQf + kQg), s);
    if (e != cudaSuccess) return e;
    long long blocks = (b.n + 255) / 256;
    if (blocks > 152 * 4) blocks = 152 * 4;
    maxabs_kernel<<<dim3((unsigned)blocks, kQf + kQg), 256, 0, s>>>(b, f, g, g_shift_dev, out_bits);
    return cudaGetLastError();
}

cudaError_t launch_moments(const Box &b, const float *f, const float *g, float *mom, cudaStream_t s)
{
    moments_kernel<<<grid_for(b.n), 256, 0, s>>>(b, f, g, mom);
    return cudaGetLastError();
}

}  // namespace lbm
