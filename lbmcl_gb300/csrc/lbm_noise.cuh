// lbm_noise.cuh -- seeded Gaussian perturbation of the initial populations.
//
// Two N(0,1) samples per (seed, site, pair): Philox4x32-10 (Salmon, Moraes,
// Dror, Shaw, SC'11) on the counter (site_lo, site_hi, pair, block); each
// 32-bit output word is one attempt of Marsaglia's polar method (its low and
// high 16 bits give the uniform pair), so one block offers four attempts and
// a warp rarely needs a second block; an accepted attempt gives both
// normals.  Populations 2m and 2m+1 of a site take the two samples of pair m.
// The natural logarithm is summed from the atanh series.  Every
// floating-point step is an explicit IEEE single-precision operation (no
// contraction, no library transcendental), so a CPU implementation of the
// same recipe gets the same bits.  Single precision because FP64 runs at a
// small fraction of the FP32 rate on GB300 and the samples only perturb the
// initial state.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lbm {

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c[0];
        const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]);
        const uint32_t lo1 = 0xCD9E8D57u * c[2];
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]);
        const uint32_t n0 = hi1 ^ c[1] ^ k0;
        const uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// ln(x), x finite and > 0, single precision: x = m 2^e, m in
// [sqrt(1/2), sqrt(2)), ln m = 2 s sum_{k=0..6} s^(2k) / (2k+1), s = (m-1)/(m+1).
__device__ __forceinline__ float series_logf(float x)
{
    unsigned bits = __float_as_uint(x);
    int e = (int)((bits >> 23) & 0xff);
    if (e == 0) {
        x = __fmul_rn(x, 16777216.0f);  // 2^24, exact
        bits = __float_as_uint(x);
        e = (int)((bits >> 23) & 0xff) - 24;
    }
    e -= 127;
    bits = (bits & 0x007fffffu) | 0x3f800000u;
    float m = __uint_as_float(bits);
    if (m > 1.41421354f) {
        m = __fmul_rn(m, 0.5f);
        e += 1;
    }
    const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const float s2 = __fmul_rn(s, s);
    // 1 / (2k + 1), folded at compile time to the correctly rounded floats
    constexpr float inv_odd[7] = {1.0f / 1.0f, 1.0f / 3.0f, 1.0f / 5.0f,  1.0f / 7.0f,
                                  1.0f / 9.0f, 1.0f / 11.0f, 1.0f / 13.0f};
    float acc = inv_odd[6];
#pragma unroll
    for (int k = 5; k >= 0; --k) acc = __fadd_rn(inv_odd[k], __fmul_rn(s2, acc));
    const float ln2 = 0.693147182f;
    return __fadd_rn(__fmul_rn((float)e, ln2), __fmul_rn(__fmul_rn(2.0f, s), acc));
}

// uniform in (-1, 1) from 16 random bits: (a + 1/2) / 2^15 - 1, exact
__device__ __forceinline__ float sym_uniform16(uint32_t a)
{
    return __fsub_rn(__fmul_rn(__fadd_rn((float)a, 0.5f), 1.0f / 32768.0f), 1.0f);
}

// The two samples of pair `pair` of a site (at most 64 attempts).
__device__ __forceinline__ void gauss_pair(uint64_t seed, uint64_t site, uint32_t pair, float &z0, float &z1)
{
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (uint32_t block = 0; block < 16; ++block) {
        uint32_t c[4] = {(uint32_t)site, (uint32_t)(site >> 32), pair, block};
        philox4x32_10(c, k0, k1);
        // the first accepted attempt of the four, found by selects; the
        // logarithm, division and square root then run once
        float v1 = 0.0f, v2 = 0.0f, s = 0.0f;
        bool found = false;
#pragma unroll
        for (int a = 3; a >= 0; --a) {
            const float w1 = sym_uniform16(c[a] & 0xffffu);
            const float w2 = sym_uniform16(c[a] >> 16);
            const float sa = __fadd_rn(__fmul_rn(w1, w1), __fmul_rn(w2, w2));
            const bool ok = sa < 1.0f && sa != 0.0f;
            v1 = ok ? w1 : v1;
            v2 = ok ? w2 : v2;
            s = ok ? sa : s;
            found |= ok;
        }
        if (found) {
            const float t = __fdiv_rn(__fmul_rn(-2.0f, series_logf(s)), s);
            const float r = __fsqrt_rn(t);
            z0 = __fmul_rn(v1, r);
            z1 = __fmul_rn(v2, r);
            return;
        }
    }
    z0 = 0.0f;
    z1 = 0.0f;
}

// The sample of population q of a site.
__device__ __forceinline__ float gauss(uint64_t seed, uint64_t site, uint32_t q)
{
    float z0, z1;
    gauss_pair(seed, site, q >> 1, z0, z1);
    return (q & 1u) ? z1 : z0;
}

}  // namespace lbm
