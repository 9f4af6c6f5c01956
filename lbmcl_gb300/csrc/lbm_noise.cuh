// lbm_noise.cuh -- seeded Gaussian perturbation of the initial populations.
//
// N(0,1) sample for (seed, site, q): Philox4x32-10 (Salmon, Moraes, Dror,
// Shaw, SC'11) on the counter (site_lo, site_hi, q, attempt), two 53-bit
// uniforms per block, Marsaglia's polar method, and a natural logarithm
// summed from the atanh series.  Every floating-point step is an explicit
// IEEE double operation (no contraction, no library transcendental), so a
// CPU implementation of the same recipe gets the same bits.
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

// ln(x), x finite and > 0: x = m 2^e, m in [sqrt(1/2), sqrt(2)),
// ln m = 2 s sum_{k=0..11} s^(2k) / (2k+1), s = (m-1)/(m+1).
__device__ __forceinline__ double series_log(double x)
{
    long long bits = __double_as_longlong(x);
    int e = (int)((bits >> 52) & 0x7ff);
    if (e == 0) {
        x = __dmul_rn(x, 18014398509481984.0);  // 2^54, exact
        bits = __double_as_longlong(x);
        e = (int)((bits >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    bits = (bits & 0x000fffffffffffffll) | 0x3ff0000000000000ll;
    double m = __longlong_as_double(bits);
    if (m > 1.4142135623730951) {
        m = __dmul_rn(m, 0.5);
        e += 1;
    }
    const double s = __ddiv_rn(__dsub_rn(m, 1.0), __dadd_rn(m, 1.0));
    const double s2 = __dmul_rn(s, s);
    // 1 / (2k + 1), k = 0 .. 11, folded at compile time to the correctly
    // rounded doubles (the values an IEEE division yields at run time)
    constexpr double inv_odd[12] = {1.0 / 1.0,  1.0 / 3.0,  1.0 / 5.0,  1.0 / 7.0,  1.0 / 9.0,  1.0 / 11.0,
                                    1.0 / 13.0, 1.0 / 15.0, 1.0 / 17.0, 1.0 / 19.0, 1.0 / 21.0, 1.0 / 23.0};
    double acc = inv_odd[11];
#pragma unroll
    for (int k = 10; k >= 0; --k) acc = __dadd_rn(inv_odd[k], __dmul_rn(s2, acc));
    const double ln2 = 0.6931471805599453;
    return __dadd_rn(__dmul_rn((double)e, ln2), __dmul_rn(__dmul_rn(2.0, s), acc));
}

__device__ __forceinline__ double sym_uniform(uint32_t a, uint32_t b)
{
    const unsigned long long m = ((unsigned long long)(a >> 5) << 26) | (unsigned long long)(b >> 6);
    const double u01 = __dmul_rn(__dadd_rn((double)m, 0.5), 1.0 / 9007199254740992.0);
    return __dsub_rn(__dmul_rn(2.0, u01), 1.0);
}

__device__ __forceinline__ double gauss(uint64_t seed, uint64_t site, uint32_t q)
{
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (uint32_t attempt = 0; attempt < 64; ++attempt) {
        uint32_t c[4] = {(uint32_t)site, (uint32_t)(site >> 32), q, attempt};
        philox4x32_10(c, k0, k1);
        const double v1 = sym_uniform(c[0], c[1]);
        const double v2 = sym_uniform(c[2], c[3]);
        const double s = __dadd_rn(__dmul_rn(v1, v1), __dmul_rn(v2, v2));
        if (s >= 1.0 || s == 0.0) continue;
        const double t = __ddiv_rn(__dmul_rn(-2.0, series_log(s)), s);
        return __dmul_rn(v1, __dsqrt_rn(t));
    }
    return 0.0;
}

}  // namespace lbm
