// lbm_noise.cuh -- seeded Gaussian perturbation of the initial populations.
//
// N(0,1) samples per (seed, site): Philox4x32-10 (Salmon, Moraes, Dror,
// Shaw, SC'11) on the counter (site_lo, site_hi, block, 0) gives four 32-bit
// words; each pair of words is one Box-Muller draw (Box and Muller, 1958):
// a radius sqrt(-2 ln u1) from 23 bits of the first word, an angle from 24
// bits of the second, and the pair (r cos theta, r sin theta).  Block g
// feeds sample pairs 2g and 2g+1; populations 2m and 2m+1 of a site take
// pair m.  The logarithm is summed from the atanh series, sine and cosine
// from their Taylor series on a quarter turn (Horner steps as fused
// multiply-adds).  Every floating-point step is an explicit IEEE
// single-precision operation or fma (no contraction left to the compiler, no
// library transcendental), so a CPU implementation of the same recipe gets
// the same bits.  Single precision because FP64 runs at a small fraction of the FP32
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

// The exponent / mantissa split of the logarithm: x = m 2^e with m in
// [sqrt(1/2), sqrt(2)); returns m and the float of e.
__device__ __forceinline__ void log_split(float x, float &m, float &fe)
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
    m = __uint_as_float(bits);
    if (m > 1.41421354f) {
        m = __fmul_rn(m, 0.5f);
        e += 1;
    }
    fe = (float)e;
}

// Both Box-Muller draws of a Philox block at once on packed FP32 pairs
// (lane .x from words 0, 1; lane .y from words 2, 3).  Every product that
// feeds a sum is an explicit fused multiply-add (one rounding, the CPU's
// fmaf), every other operation an IEEE add / multiply (lane-wise, as the
// scalar ones), division and square root per lane: no step is left for the
// compiler to fuse, so the CPU recipe gives the same bits.
__device__ __forceinline__ float2 nz_f2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 nz_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 nz_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 nz_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// ln x = e ln 2 + 2 s (1 + s^2/3 + ... + s^12/13), s = (m-1)/(m+1)
// (|s| <= 0.1716: truncation below 1e-9)
__device__ __forceinline__ float2 series_logf2(float2 x)
{
    float2 m, fe;
    log_split(x.x, m.x, fe.x);
    log_split(x.y, m.y, fe.y);
    const float2 num = nz_add(m, nz_f2(-1.0f)), den = nz_add(m, nz_f2(1.0f));
    const float2 s = make_float2(__fdiv_rn(num.x, den.x), __fdiv_rn(num.y, den.y));
    const float2 s2 = nz_mul(s, s);
    // 1 / (2k + 1), folded at compile time to the correctly rounded floats
    constexpr float inv_odd[7] = {1.0f / 1.0f, 1.0f / 3.0f, 1.0f / 5.0f,  1.0f / 7.0f,
                                  1.0f / 9.0f, 1.0f / 11.0f, 1.0f / 13.0f};
    float2 acc = nz_f2(inv_odd[6]);
#pragma unroll
    for (int k = 5; k >= 0; --k) acc = nz_fma(s2, acc, nz_f2(inv_odd[k]));
    const float ln2 = 0.693147182f;
    return nz_fma(nz_mul(nz_f2(2.0f), s), acc, nz_mul(fe, nz_f2(ln2)));
}

// cos and sin of the angle 2 pi (k / 4 + 1 / 8) + x, x in (-pi/4, pi/4), k in
// 0..3: the Taylor series of cos x (to x^10) and sin x (to x^9), the rotation
// by pi/4 to pi/4 + x, then the quarter turn k (per lane).
__device__ __forceinline__ void quarter_turn_cs2(uint32_t k0, uint32_t k1, float2 x, float2 &c, float2 &s)
{
    const float2 x2 = nz_mul(x, x);
    float2 sp = nz_f2(1.0f / 362880.0f);
    sp = nz_fma(x2, sp, nz_f2(-1.0f / 5040.0f));
    sp = nz_fma(x2, sp, nz_f2(1.0f / 120.0f));
    sp = nz_fma(x2, sp, nz_f2(-1.0f / 6.0f));
    const float2 sn = nz_fma(nz_mul(x, x2), sp, x);
    float2 cp = nz_f2(-1.0f / 3628800.0f);
    cp = nz_fma(x2, cp, nz_f2(1.0f / 40320.0f));
    cp = nz_fma(x2, cp, nz_f2(-1.0f / 720.0f));
    cp = nz_fma(x2, cp, nz_f2(1.0f / 24.0f));
    cp = nz_fma(x2, cp, nz_f2(-0.5f));
    const float2 cs = nz_fma(x2, cp, nz_f2(1.0f));
    const float2 h = nz_f2(0.707106781f);  // sqrt(1/2)
    const float2 c0 = nz_mul(h, nz_add(cs, make_float2(-sn.x, -sn.y))), s0 = nz_mul(h, nz_add(cs, sn));
    c.x = (k0 == 0) ? c0.x : (k0 == 1) ? -s0.x : (k0 == 2) ? -c0.x : s0.x;
    s.x = (k0 == 0) ? s0.x : (k0 == 1) ? c0.x : (k0 == 2) ? -s0.x : -c0.x;
    c.y = (k1 == 0) ? c0.y : (k1 == 1) ? -s0.y : (k1 == 2) ? -c0.y : s0.y;
    s.y = (k1 == 0) ? s0.y : (k1 == 1) ? c0.y : (k1 == 2) ? -s0.y : -c0.y;
}

// Two Box-Muller pairs from the four words: u1 = (w >> 9 + 1/2) / 2^23 in
// (0, 1) (exact), the angle's quarter turn from the top two bits of the
// partner word and its offset in the quarter from the next 22,
// (f + 1/2) / 2^22 (exact); r = sqrt(-2 ln u1), samples (r cos, r sin).
__device__ __forceinline__ void box_muller2(const uint32_t (&w)[4], float (&z)[4])
{
    const float2 u1 = nz_mul(nz_add(make_float2((float)(w[0] >> 9), (float)(w[2] >> 9)), nz_f2(0.5f)),
                             nz_f2(1.0f / 8388608.0f));
    const float2 l2 = nz_mul(nz_f2(-2.0f), series_logf2(u1));
    const float2 r = make_float2(__fsqrt_rn(l2.x), __fsqrt_rn(l2.y));
    const float2 fq = nz_mul(nz_add(make_float2((float)((w[1] >> 8) & 0x3fffffu), (float)((w[3] >> 8) & 0x3fffffu)),
                                    nz_f2(0.5f)),
                             nz_f2(1.0f / 4194304.0f));
    const float2 x = nz_mul(nz_add(fq, nz_f2(-0.5f)), nz_f2(1.57079637f));  // (fq - 1/2) pi/2
    float2 c, s;
    quarter_turn_cs2(w[1] >> 30, w[3] >> 30, x, c, s);
    const float2 zc = nz_mul(r, c), zs = nz_mul(r, s);
    z[0] = zc.x;
    z[1] = zs.x;
    z[2] = zc.y;
    z[3] = zs.y;
}

// The four samples of block g of a site: pairs 2g (z[0], z[1]) and 2g + 1
// (z[2], z[3]).
__device__ __forceinline__ void gauss_block(uint64_t seed, uint64_t site, uint32_t g, float (&z)[4])
{
    uint32_t c[4] = {(uint32_t)site, (uint32_t)(site >> 32), g, 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    box_muller2(c, z);
}

}  // namespace lbm
