// lbm_noise.cuh -- seeded Gaussian perturbation of the initial populations.
//
// N(0,1) samples per (seed, site): Philox4x32-10 (Salmon, Moraes, Dror,
// Shaw, SC'11) on the counter (site_lo, site_hi, block, 0) gives four 32-bit
// words; each pair of words is one Box-Muller draw (Box and Muller, 1958):
// a radius sqrt(-2 ln u1) from 23 bits of the first word, an angle from 24
// bits of the second, and the pair (r cos theta, r sin theta).  Block g
// feeds sample pairs 2g and 2g+1; populations 2m and 2m+1 of a site take
// pair m.  The logarithm is summed from the atanh series, sine and cosine
// from their Taylor series on a quarter turn.  Every floating-point step is
// an explicit IEEE single-precision operation (no contraction, no library
// transcendental), so a CPU implementation of the same recipe gets the same
// bits.  Single precision because FP64 runs at a small fraction of the FP32
// rate on GB300 and the samples only perturb the initial state.
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

// cos and sin of the angle 2 pi (k / 4 + 1 / 8 + x / (2 pi)), x in
// (-pi/4, pi/4), k in 0..3: the quarter turn k, then pi/4 + x from the Taylor
// series of cos x (to x^10) and sin x (to x^9) and the rotation by pi/4.
__device__ __forceinline__ void quarter_turn_cs(uint32_t k, float x, float &c, float &s)
{
    const float x2 = __fmul_rn(x, x);
    float sp = 1.0f / 362880.0f;
    sp = __fadd_rn(-1.0f / 5040.0f, __fmul_rn(x2, sp));
    sp = __fadd_rn(1.0f / 120.0f, __fmul_rn(x2, sp));
    sp = __fadd_rn(-1.0f / 6.0f, __fmul_rn(x2, sp));
    const float sn = __fadd_rn(x, __fmul_rn(__fmul_rn(x, x2), sp));
    float cp = -1.0f / 3628800.0f;
    cp = __fadd_rn(1.0f / 40320.0f, __fmul_rn(x2, cp));
    cp = __fadd_rn(-1.0f / 720.0f, __fmul_rn(x2, cp));
    cp = __fadd_rn(1.0f / 24.0f, __fmul_rn(x2, cp));
    cp = __fadd_rn(-0.5f, __fmul_rn(x2, cp));
    const float cs = __fadd_rn(1.0f, __fmul_rn(x2, cp));
    const float h = 0.707106781f;  // sqrt(1/2)
    const float c0 = __fmul_rn(h, __fsub_rn(cs, sn)), s0 = __fmul_rn(h, __fadd_rn(cs, sn));
    c = (k == 0) ? c0 : (k == 1) ? -s0 : (k == 2) ? -c0 : s0;
    s = (k == 0) ? s0 : (k == 1) ? c0 : (k == 2) ? -s0 : -c0;
}

// One Box-Muller pair from two 32-bit words: u1 = (w0 >> 9 + 1/2) / 2^23 in
// (0, 1) (exact), the angle's quarter turn from the top two bits of w1 and
// its offset in the quarter from the next 22, (f + 1/2) / 2^22 (exact).
__device__ __forceinline__ void box_muller(uint32_t w0, uint32_t w1, float &z0, float &z1)
{
    const float u1 = __fmul_rn(__fadd_rn((float)(w0 >> 9), 0.5f), 1.0f / 8388608.0f);
    const float r = __fsqrt_rn(__fmul_rn(-2.0f, series_logf(u1)));
    const float fq = __fmul_rn(__fadd_rn((float)((w1 >> 8) & 0x3fffffu), 0.5f), 1.0f / 4194304.0f);
    const float x = __fmul_rn(__fsub_rn(fq, 0.5f), 1.57079637f);  // (fq - 1/2) pi/2
    float c, s;
    quarter_turn_cs(w1 >> 30, x, c, s);
    z0 = __fmul_rn(r, c);
    z1 = __fmul_rn(r, s);
}

// The four samples of block g of a site: pairs 2g (z[0], z[1]) and 2g + 1
// (z[2], z[3]).
__device__ __forceinline__ void gauss_block(uint64_t seed, uint64_t site, uint32_t g, float (&z)[4])
{
    uint32_t c[4] = {(uint32_t)site, (uint32_t)(site >> 32), g, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    box_muller(c[0], c[1], z[0], z[1]);
    box_muller(c[2], c[3], z[2], z[3]);
}

}  // namespace lbm
