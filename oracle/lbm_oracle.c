/*
 * lbm_oracle.c -- CPU oracle for LBMCL's D3Q19 BGK lid-driven-cavity step.
 *
 * TEST INFRASTRUCTURE ONLY (see lbm_oracle.h): the checker for the CUDA
 * library and the timed CPU baseline, never part of the product path.
 */
#include "lbm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define LBMO_Q 19

/* D3Q19 velocity set in the reference's ordering (kernels.cl:131-205):
 * 0 rest; 1..6 = +x,+y,-x,-y,-z,+z; 7..18 the edge directions. */
static const int LBMO_EX[LBMO_Q] = {0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0};
static const int LBMO_EY[LBMO_Q] = {0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1};
static const int LBMO_EZ[LBMO_Q] = {0, 0, 0, 0, 0, -1, 1, 0, 0, 0, 0, -1, -1, -1, -1, 1, 1, 1, 1};
/* opposite direction S_i (kernels.cl:208-226) */
static const int LBMO_OPP[LBMO_Q] = {0, 3, 4, 1, 2, 6, 5, 9, 10, 7, 8, 17, 18, 15, 16, 13, 14, 11, 12};

/* Cell-type predicates (common.h:23-66). */
static inline int lbmo_is_moving_init(int ct) { return ct & LBMO_FRONT; }
static inline int lbmo_is_fluid(int ct) { return ct == LBMO_FLUID; }
static inline int lbmo_is_wall(int ct) { return ct == LBMO_WALL; }
static inline int lbmo_is_boundary(int ct)
{
    return ct & (LBMO_LEFT | LBMO_RIGHT | LBMO_BOTTOM | LBMO_TOP | LBMO_BACK | LBMO_FRONT);
}
static inline int lbmo_is_moving(int ct) { return ct & LBMO_MOVING; }
static inline int lbmo_is_store_macro(int ct) { return lbmo_is_fluid(ct) || lbmo_is_moving(ct); }
static inline int lbmo_is_collision(int ct) { return lbmo_is_fluid(ct) || lbmo_is_moving(ct); }
static inline int lbmo_is_bounceback(int ct) { return lbmo_is_boundary(ct) && !(ct & LBMO_MOVING); }

int lbmo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static double lbmo_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* kernels.cl:236-266: face flags on the first interior layer, WALL on the
 * outer layer, CORNER for the four BACK corners, MOVING on the bare FRONT face,
 * FLUID elsewhere. */
int lbmo_cell_type(int dim, int x, int y, int z)
{
    int ct = LBMO_NONE;
    if (x == 1) ct |= LBMO_LEFT;
    if (x == dim - 2) ct |= LBMO_RIGHT;
    if (y == 1) ct |= LBMO_BOTTOM;
    if (y == dim - 2) ct |= LBMO_TOP;
    if (z == 1) ct |= LBMO_BACK;
    if (z == dim - 2) ct |= LBMO_FRONT;
    if (x == 0 || x == dim - 1 || y == 0 || y == dim - 1 || z == 0 || z == dim - 1) ct = LBMO_WALL;
    if (ct == (LBMO_LEFT | LBMO_BACK | LBMO_BOTTOM) || ct == (LBMO_RIGHT | LBMO_BACK | LBMO_BOTTOM) ||
        ct == (LBMO_LEFT | LBMO_BACK | LBMO_TOP) || ct == (LBMO_RIGHT | LBMO_BACK | LBMO_TOP))
        ct = LBMO_CORNER;
    if (ct == LBMO_FRONT) ct |= LBMO_MOVING;
    if (ct == LBMO_NONE) ct = LBMO_FLUID;
    return ct;
}

/* ---------------------------------------------------------------------------
 * Seeded noise.  Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
 * numbers: as easy as 1, 2, 3", SC'11): 10 rounds of two 32x32->64
 * multiplications with the published multipliers and Weyl key increments.
 * ------------------------------------------------------------------------- */
void lbmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        const uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ln(x) for finite x > 0 in single precision: x = m 2^e with m in
 * [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s), s = (m-1)/(m+1), summed as the odd
 * series 2 s (1 + s^2/3 + ... + s^12/13) (|s| <= 0.1716: truncation below
 * 1e-9) by Horner steps with fused multiply-adds.  IEEE float + - * / and
 * fmaf (one rounding, as the GPU's fma) only. */
float lbmo_logf(float x)
{
    uint32_t bits;
    memcpy(&bits, &x, sizeof bits);
    int e = (int)((bits >> 23) & 0xff);
    if (e == 0) { /* subnormal: scale by 2^24 exactly */
        x = x * 16777216.0f;
        memcpy(&bits, &x, sizeof bits);
        e = (int)((bits >> 23) & 0xff) - 24;
    }
    e -= 127;
    bits = (bits & 0x007fffffu) | 0x3f800000u; /* m in [1,2) */
    float m;
    memcpy(&m, &bits, sizeof m);
    if (m > 1.41421354f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    static const float inv_odd[7] = {1.0f / 1.0f, 1.0f / 3.0f, 1.0f / 5.0f, 1.0f / 7.0f,
                                     1.0f / 9.0f, 1.0f / 11.0f, 1.0f / 13.0f};
    float acc = inv_odd[6];
    for (int k = 5; k >= 0; --k) acc = fmaf(s2, acc, inv_odd[k]);
    const float ln2 = 0.693147182f;
    return fmaf(2.0f * s, acc, (float)e * ln2);
}

double lbmo_log(double x) { return (double)lbmo_logf((float)x); }

/* cos and sin of 2 pi (k/4 + 1/8) + x, x in (-pi/4, pi/4), k in 0..3:
 * Taylor series of cos x (to x^10) and sin x (to x^9) by Horner steps with
 * fused multiply-adds, the rotation by pi/4 to pi/4 + x, then the quarter
 * turn k.  IEEE float + - * and fmaf only. */
static void lbmo_quarter_turn_cs(uint32_t k, float x, float *c, float *s)
{
    const float x2 = x * x;
    float sp = 1.0f / 362880.0f;
    sp = fmaf(x2, sp, -1.0f / 5040.0f);
    sp = fmaf(x2, sp, 1.0f / 120.0f);
    sp = fmaf(x2, sp, -1.0f / 6.0f);
    const float sn = fmaf(x * x2, sp, x);
    float cp = -1.0f / 3628800.0f;
    cp = fmaf(x2, cp, 1.0f / 40320.0f);
    cp = fmaf(x2, cp, -1.0f / 720.0f);
    cp = fmaf(x2, cp, 1.0f / 24.0f);
    cp = fmaf(x2, cp, -0.5f);
    const float cs = fmaf(x2, cp, 1.0f);
    const float h = 0.707106781f; /* sqrt(1/2) */
    const float c0 = h * (cs - sn), s0 = h * (cs + sn);
    *c = (k == 0) ? c0 : (k == 1) ? -s0 : (k == 2) ? -c0 : s0;
    *s = (k == 0) ? s0 : (k == 1) ? c0 : (k == 2) ? -s0 : -c0;
}

/* One Box-Muller pair from two 32-bit words: u1 = ((w0 >> 9) + 1/2) / 2^23
 * in (0, 1), r = sqrt(-2 ln u1); the angle's quarter turn from the top two
 * bits of w1, its offset x = (fq - 1/2) pi/2 from the next 22 bits,
 * fq = (f + 1/2) / 2^22 (both uniforms exact in float). */
static void lbmo_box_muller(uint32_t w0, uint32_t w1, float z[2])
{
    const float u1 = ((float)(w0 >> 9) + 0.5f) * (1.0f / 8388608.0f);
    const float r = sqrtf(-2.0f * lbmo_logf(u1));
    const float fq = ((float)((w1 >> 8) & 0x3fffffu) + 0.5f) * (1.0f / 4194304.0f);
    const float x = (fq - 0.5f) * 1.57079637f;
    float c, s;
    lbmo_quarter_turn_cs(w1 >> 30, x, &c, &s);
    z[0] = r * c;
    z[1] = r * s;
}

/* Two standard normals for (seed, site, pair) by the Box-Muller transform:
 * Philox4x32-10 on the counter (site_lo, site_hi, pair >> 1, 0); words 0, 1
 * give pair 2g, words 2, 3 pair 2g + 1 of block g.  Single precision, IEEE
 * + - * / sqrt and fmaf only. */
void lbmo_gauss_pairf(uint64_t seed, uint64_t site, uint32_t pair, float z[2])
{
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const uint32_t ctr[4] = {(uint32_t)site, (uint32_t)(site >> 32), pair >> 1, 0u};
    uint32_t r[4];
    lbmo_philox4x32_10(ctr, key, r);
    const int w = 2 * (int)(pair & 1u);
    lbmo_box_muller(r[w], r[w + 1], z);
}

/* The sample of population q of a site: element q & 1 of pair q >> 1. */
float lbmo_gaussf(uint64_t seed, uint64_t site, uint32_t q)
{
    float z[2];
    lbmo_gauss_pairf(seed, site, q >> 1, z);
    return z[q & 1u];
}

double lbmo_gauss(uint64_t seed, uint64_t site, uint32_t q) { return (double)lbmo_gaussf(seed, site, q); }

/* ---- precision-generic body, instantiated for float and double ---------- */
#define REAL float
#define SFX(name) name##_f32
#include "lbm_oracle_body.h"
#undef REAL
#undef SFX

#define REAL double
#define SFX(name) name##_f64
#include "lbm_oracle_body.h"
#undef REAL
#undef SFX
