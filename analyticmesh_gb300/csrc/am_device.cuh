// am_device.cuh -- device helpers shared by the engine's kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "am_internal.h"

namespace am {

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
    using type = float4;
};
template <>
struct Vec4<double> {
    using type = double4;
};
template <typename T>
using vec4_t = typename Vec4<T>::type;

template <typename T>
__device__ __forceinline__ vec4_t<T> ld4(const T *p)
{
    return *reinterpret_cast<const vec4_t<T> *>(p);
}
template <typename T>
__device__ __forceinline__ void st4(T *p, vec4_t<T> v)
{
    *reinterpret_cast<vec4_t<T> *>(p) = v;
}

// ---------------------------------------------------------------- keys
__device__ __forceinline__ int key_bit(const uint32_t *key, int k) { return (key[k >> 5] >> (k & 31)) & 1; }

// 64-bit mix (splitmix64 finaliser)
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Hash of a packed key = sum over words of mix64(word, position).  Additive,
// so flipping one bit updates it in O(1).
__host__ __device__ __forceinline__ uint64_t word_term(uint32_t w, int pos)
{
    return mix64(((uint64_t)(uint32_t)pos << 32) | (uint64_t)w);
}

__device__ __forceinline__ uint64_t flip_hash(uint64_t h, uint32_t word, int k)
{
    const int pos = k >> 5;
    return h - word_term(word, pos) + word_term(word ^ (1u << (k & 31)), pos);
}

// slot value: [fingerprint 32][tag 1][id 31]; tag 1 = candidate of the
// current wave, 0 = committed region
__device__ __forceinline__ uint32_t fp_of(uint64_t h) { return (uint32_t)(h >> 32); }
__device__ __forceinline__ unsigned long long slot_value(uint32_t fp, int cand, uint32_t id)
{
    return ((unsigned long long)fp << 32) | ((unsigned long long)(cand ? 1u : 0u) << 31) | (id & 0x7fffffffu);
}

// ---------------------------------------------------------------- warp
__device__ __forceinline__ int warp_sum(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------- 3x3
// Cramer's rule for A x + b = 0 with rows (r0, r1, r2) -- the reference's
// solve_3x3 (backend/inc/kernel.h:553-571).  Returns the determinant.
template <typename S>
__device__ __forceinline__ S det3(S a0, S a1, S a2, S a3, S a4, S a5, S a6, S a7, S a8)
{
    return a0 * (a4 * a8 - a5 * a7) - a1 * (a3 * a8 - a5 * a6) + a2 * (a3 * a7 - a4 * a6);
}

template <typename S>
__device__ __forceinline__ S solve3(const S *r0, const S *r1, const S *r2, S *x)
{
    const S d0 = det3<S>(r0[0], r0[1], r0[2], r1[0], r1[1], r1[2], r2[0], r2[1], r2[2]);
    const S d1 = det3<S>(-r0[3], r0[1], r0[2], -r1[3], r1[1], r1[2], -r2[3], r2[1], r2[2]);
    const S d2 = det3<S>(r0[0], -r0[3], r0[2], r1[0], -r1[3], r1[2], r2[0], -r2[3], r2[2]);
    const S d3 = det3<S>(r0[0], r0[1], -r0[3], r1[0], r1[1], -r1[3], r2[0], r2[1], -r2[3]);
    x[0] = d1 / d0;
    x[1] = d2 / d0;
    x[2] = d3 / d0;
    return d0;
}

// get_i_j (backend/inc/kernel.h:607-622): pair index x -> (i, j), i > j,
// along anti-diagonals of i + j, clamped to ij_max - 1.
__device__ __forceinline__ void get_i_j(int x, int ij_max, int &i, int &j)
{
    const int k = x / 2;
    const int a = (int)ceilf(sqrtf(2 * k + 2.25f) - 1.5f);
    const int r = x - a * (a + 1);
    const int A = 2 * a + r / (a + 1);
    const int B = r % (a + 1);
    i = (A + 1) / 2 + B + 1;
    j = A + 1 - i;
    i = i < ij_max ? i : ij_max - 1;
    j = j < ij_max ? j : ij_max - 1;
}

} // namespace am
