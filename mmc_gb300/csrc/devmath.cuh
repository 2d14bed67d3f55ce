// Device math for the photon engine.  exp/log/sincos(2*pi*u) are the
// project's own routines (Cody-Waite argument reduction with truncated Taylor /
// atanh series, Cody & Waite, "Software Manual for the Elementary Functions",
// 1980); every operation is an explicit IEEE-rounded op or fmaf, and the file
// is compiled with -fmad=false, so the CPU oracle (oracle/mmc_oracle.c, same
// sequence) reproduces each photon bit for bit.
#pragma once
#include <cstdint>

namespace mmcgb {

#define MMC_LN2_HI 0.693145751953125f
#define MMC_LN2_LO 1.42860682030941723212e-6f
#define MMC_LOG2E 1.44269504088896340736f

__device__ __forceinline__ float mmc_expf(float x) {
    if (x < -104.f) return 0.f;
    if (x > 88.7f) return __int_as_float(0x7F800000);
    float k = rintf(x * MMC_LOG2E);
    float r = fmaf(k, -MMC_LN2_HI, x);
    r = fmaf(k, -MMC_LN2_LO, r);
    float p = 1.f / 5040.f;
    p = fmaf(p, r, 1.f / 720.f);
    p = fmaf(p, r, 1.f / 120.f);
    p = fmaf(p, r, 1.f / 24.f);
    p = fmaf(p, r, 1.f / 6.f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.f);
    p = fmaf(p, r, 1.f);
    int ki = (int)k;
    if (ki < -125) {
        p = p * 5.42101086242752217e-20f;
        ki += 64;
    }
    return p * __int_as_float((ki + 127) << 23);
}

__device__ __forceinline__ float mmc_logf(float x) {
    uint32_t b = __float_as_uint(x);
    int e = (int)((b >> 23) & 0xFF) - 127;
    float m = __uint_as_float((b & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    float s = __fdiv_rn(m - 1.f, m + 1.f);
    float z = s * s;
    float p = 1.f / 11.f;
    p = fmaf(p, z, 1.f / 9.f);
    p = fmaf(p, z, 1.f / 7.f);
    p = fmaf(p, z, 1.f / 5.f);
    p = fmaf(p, z, 1.f / 3.f);
    p = fmaf(p, z, 1.f);
    float lm = 2.f * s * p;
    float fe = (float)e;
    return fmaf(fe, MMC_LN2_HI, fmaf(fe, MMC_LN2_LO, lm));
}

__device__ __forceinline__ void mmc_sincos2pi(float u, float& sv, float& cv) {
    float q = rintf(u * 4.f);
    float f = u - q * 0.25f;
    float x = f * 6.28318530717958647692f;
    float z = x * x;
    float ps = 1.f / 362880.f;
    ps = fmaf(ps, z, -1.f / 5040.f);
    ps = fmaf(ps, z, 1.f / 120.f);
    ps = fmaf(ps, z, -1.f / 6.f);
    ps = fmaf(ps * z, x, x);
    float pc = -1.f / 3628800.f;
    pc = fmaf(pc, z, 1.f / 40320.f);
    pc = fmaf(pc, z, -1.f / 720.f);
    pc = fmaf(pc, z, 1.f / 24.f);
    pc = fmaf(pc, z, -0.5f);
    pc = fmaf(pc, z, 1.f);
    int qi = ((int)q) & 3;
    sv = (qi == 0) ? ps : (qi == 1) ? pc : (qi == 2) ? -ps : -pc;
    cv = (qi == 0) ? pc : (qi == 1) ? -ps : (qi == 2) ? -pc : ps;
}

// xorshift128+ with the reference's float extraction (src/mmc_core.cl:517-531).
__device__ __forceinline__ float rng_next(unsigned long long& t0, unsigned long long& t1) {
    unsigned long long s1 = t0;
    const unsigned long long s0 = t1;
    t0 = s0;
    s1 ^= s1 << 23;
    t1 = s1 ^ s0 ^ (s1 >> 18) ^ (s0 >> 5);
    unsigned long long r = t1 + s0;
    uint32_t lo = (uint32_t)r;
    return __uint_as_float(0x3F800000u | (lo >> 9)) - 1.0f;
}

// One xorshift128+ step giving two floats in [0,1): the return value from the
// low 32 bits of the output (as rng_next) and `hi` from its high 32 bits.
__device__ __forceinline__ float rng_next_pair(unsigned long long& t0, unsigned long long& t1, float& hi) {
    unsigned long long s1 = t0;
    const unsigned long long s0 = t1;
    t0 = s0;
    s1 ^= s1 << 23;
    t1 = s1 ^ s0 ^ (s1 >> 18) ^ (s0 >> 5);
    const unsigned long long r = t1 + s0;
    hi = __uint_as_float(0x3F800000u | ((uint32_t)(r >> 32) >> 9)) - 1.0f;
    return __uint_as_float(0x3F800000u | ((uint32_t)r >> 9)) - 1.0f;
}

__host__ __device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Per-photon initial state from (seed, global photon index).
__host__ __device__ __forceinline__ void rng_seed(unsigned long long seed, unsigned long long pid,
                                                  unsigned long long& t0, unsigned long long& t1) {
    unsigned long long base = splitmix64(seed ^ 0x6D6D63676233ull) + 2ull * pid * 0x9E3779B97F4A7C15ull;
    t0 = splitmix64(base);
    t1 = splitmix64(base + 0x9E3779B97F4A7C15ull);
    if ((t0 | t1) == 0) t1 = 1;
}

}  // namespace mmcgb
