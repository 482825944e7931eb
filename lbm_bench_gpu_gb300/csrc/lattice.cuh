// lattice.cuh -- lattice vectors of the reference's D3Q7 / D3Q19 order and the
// storage element formats, shared by the step and adjoint kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "lbm_internal.h"

namespace lbm {

// D3Q19 lattice vectors and opposite directions (reference order,
// src/stream_g.cu:58-76; the first seven are the D3Q7 set, src/stream_f.cu:54-59).
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

// Storage formats: element conversions, and the resident blocks per SM the
// step kernel's launch bounds ask for.  FP32 stages 108 KB of shared memory
// per block (2 blocks of 256 threads per SM, 128 registers); the 16-bit
// formats stage 54 KB per block of 128 threads, 4 blocks per SM (128
// registers).
template <typename ST>
struct Fmt;
template <>
struct Fmt<float> {
    static constexpr int kMinBlocks = 2;
    static constexpr bool kMapped = false;
    using T2 = float2;   // (unused: FP32 keeps one node per thread)
    __device__ static float load(float v) { return v; }
    __device__ static float store(float v) { return v; }
    __device__ static float2 load2(float2 v) { return v; }
    __device__ static float2 store2(float2 v) { return v; }
    __device__ static float2 swap2(float2 v) { return make_float2(v.y, v.x); }
    __device__ static float2 perm2(float2 v, unsigned) { return v; }
};
template <>
struct Fmt<__half> {
    static constexpr int kMinBlocks = 4;
    static constexpr bool kMapped = true;
    using T2 = __half2;   // two adjacent nodes, one 32-bit word
    __device__ static float load(__half v) { return __half2float(v); }
    __device__ static __half store(float v) { return __float2half_rn(v); }
    __device__ static float2 load2(__half2 v) { return __half22float2(v); }
    __device__ static __half2 store2(float2 v) { return __float22half2_rn(v); }
    __device__ static __half2 swap2(__half2 v) { return __lowhigh2highlow(v); }
    // the word's two halves in the order selector sel gives (kKeep / kSwap)
    __device__ static __half2 perm2(__half2 v, unsigned sel)
    {
        const unsigned w = __byte_perm(*reinterpret_cast<const unsigned *>(&v), 0u, sel);
        return *reinterpret_cast<const __half2 *>(&w);
    }
};
template <>
struct Fmt<__nv_bfloat16> {
    static constexpr int kMinBlocks = 4;
    static constexpr bool kMapped = true;
    using T2 = __nv_bfloat162;
    __device__ static float load(__nv_bfloat16 v) { return __bfloat162float(v); }
    __device__ static __nv_bfloat16 store(float v) { return __float2bfloat16_rn(v); }
    __device__ static float2 load2(__nv_bfloat162 v) { return __bfloat1622float2(v); }
    __device__ static __nv_bfloat162 store2(float2 v) { return __float22bfloat162_rn(v); }
    __device__ static __nv_bfloat162 swap2(__nv_bfloat162 v) { return __lowhigh2highlow(v); }
    __device__ static __nv_bfloat162 perm2(__nv_bfloat162 v, unsigned sel)
    {
        const unsigned w = __byte_perm(*reinterpret_cast<const unsigned *>(&v), 0u, sel);
        return *reinterpret_cast<const __nv_bfloat162 *>(&w);
    }
};

// Element index of node (x, row start t - x) in a field of the state: FP32
// storage keeps the natural layout; the 16-bit formats keep the pair layout,
// in which 32-bit word w of a row holds nodes x = w and x = w + nx/2 (so that
// a step moving both nodes of a word by one node in x moves a whole word).
// f_0 of a 16-bit state is in the pair layout too (float2 words).
template <typename ST>
__device__ __forceinline__ unsigned storage_index(const Box &b, unsigned t, int x)
{
    if constexpr (sizeof(ST) == 2) {
        const int h = b.nx >> 1;
        return t - (unsigned)x + (x < h ? 2u * (unsigned)x : 2u * (unsigned)(x - h) + 1u);
    } else {
        return t;
    }
}

// __byte_perm selectors: a 32-bit word as it is, or with its 16-bit halves swapped.
constexpr unsigned kKeep = 0x3210u, kSwap = 0x1032u;

// Packed FP32 (f32x2): two lanes per instruction, each rounded as FP32.
namespace pk {
__device__ __forceinline__ float2 splat(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, splat(-1.f), a); }
}  // namespace pk

}  // namespace lbm
