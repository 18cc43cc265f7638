// Device-side helpers shared by the kernel translation units.
#pragma once

#include <cstdint>

#include "pdpd_internal.h"

namespace pdpd {

// 32-byte aligned FP64 payload element (x, y, z, w).
struct __align__(32) Vec4d {
    double x, y, z, w;
};
struct __align__(16) Vec2d {
    double x, y;
};

// riscv_mix64_m2 (reference include/dpd/core/hash.hpp:20-30), full 64-bit form.
__device__ __forceinline__ uint64_t mix64_m2(uint64_t x)
{
    const uint64_t C = 0xd392d2a7ull;
    x = x ^ (x >> 32);
    x = x * C;
    x = x ^ (x >> 32);
    x = x * C;
    x = x ^ (x >> 32);
    return x;
}

// get_t_hash (hash.hpp:61-65).
__device__ __forceinline__ uint64_t t_hash(uint32_t t, uint64_t seed)
{
    return mix64_m2(seed + mix64_m2((uint64_t)t));
}

// hash_rng_sym (hash.hpp:81-88): the low 32 bits of mix64_m2((min | max << 32) ^ t_hash),
// evaluated with 32-bit integer operations.  With x = hi:lo and a 32-bit constant C,
// x ^= x >> 32 only changes lo (lo ^= hi), and x *= C gives lo' = lo*C and
// hi' = hi*C + umulhi(lo, C) (mod 2^32).  The final x ^= x >> 32 leaves lo ^ hi in the
// low word, which is all the caller keeps.
__device__ __forceinline__ uint32_t hash_rng_sym(uint32_t th_lo, uint32_t th_hi, uint32_t a,
                                                 uint32_t b)
{
    const uint32_t C = 0xd392d2a7u;
    uint32_t lo = min(a, b) ^ th_lo;
    uint32_t hi = max(a, b) ^ th_hi;
    lo ^= hi;
    uint32_t lo2 = lo * C;
    uint32_t hi2 = hi * C + __umulhi(lo, C);
    lo2 ^= hi2;
    uint32_t lo3 = lo2 * C;
    uint32_t hi3 = hi2 * C + __umulhi(lo2, C);
    return lo3 ^ hi3;
}

// dpd_maths_core::default_hash (dpd_maths_core.hpp:55-79): u = (float)(int32)h * 2^-32,
// uniform on [-0.5, 0.5).
__device__ __forceinline__ float hash_u(uint32_t th_lo, uint32_t th_hi, uint32_t a, uint32_t b)
{
    uint32_t h = hash_rng_sym(th_lo, th_hi, a, b);
    return __int2float_rn((int)h) * 2.3283064365386962890625e-10f;
}

// MIN_DISTANCE_CUTOFF_SQR (dpd_state.hpp:138-139): 1e-9f squared in single precision.
__device__ __forceinline__ float min_dist_sqr_f()
{
    return 0.000000001f * 0.000000001f;
}

__device__ __forceinline__ int wrap_index(int i, int L)
{
    i %= L;
    return i < 0 ? i + L : i;
}

__device__ __forceinline__ void decode_cell(uint32_t local, const int32_t L[3], int &cx, int &cy,
                                            int &cz)
{
    uint32_t yz = (uint32_t)L[1] * (uint32_t)L[2];
    cx = (int)(local / yz);
    uint32_t r = local - (uint32_t)cx * yz;
    cy = (int)(r / (uint32_t)L[2]);
    cz = (int)(r - (uint32_t)cy * (uint32_t)L[2]);
}

}  // namespace pdpd
