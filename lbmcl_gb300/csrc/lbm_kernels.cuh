// lbm_kernels.cuh -- the sm_103a kernels of one lattice handle.
//
//   pull_kernel<S, MODE>  one fused pull-stream + collide iteration
//                         (replaces kernels.cl:321-425); MODE_REDUCE reuses
//                         its gather to form FP64 mass / energy partials
//   init_kernel<S>        initial state (replaces kernels.cl:277-318)
//   dump_f_kernel<S,T>    reference post-stream buffer R_t in CSoA order
//   load_f_kernel<S,T>    the inverse of dump_f_kernel
//   sum_partials_kernel   deterministic final pass of the reductions
//
// Work decomposition of the pull kernel: one thread owns V = 16 / sizeof(S)
// consecutive x-sites of one interior row (y, z in [1, dim-2]).  Each of the 19
// populations is read with one aligned 16-byte load from its source row; the
// ten populations with e_x != 0 need one more element just outside the
// vector, read with one scalar load (the neighbouring thread's vector, so an
// L1/L2 hit).  Results are written with one aligned 16-byte store per
// population.  No shared memory, no shuffles in the step itself.
#pragma once

#include <string.h>

#include <type_traits>

#include "lbm_device.cuh"
#include "lbm_noise.cuh"


namespace lbm {

template <class S> struct Compute { using type = float; };
template <> struct Compute<double> { using type = double; };
template <class S> __host__ __device__ constexpr bool is_dev16() { return sizeof(S) == 2; }

// 16-byte vector load / store (ld.global.nc.v4 / st.global.v4).
template <class S, int V>
__device__ __forceinline__ void load_vec(const S *__restrict__ p, S (&out)[V])
{
    static_assert(V * sizeof(S) == 16 || V * sizeof(S) == 8 || V * sizeof(S) == 4, "4-, 8- or 16-byte vectors");
    if constexpr (V * sizeof(S) == 16) {
        const uint4 r = __ldg(reinterpret_cast<const uint4 *>(p));
        memcpy(out, &r, 16);
    } else if constexpr (V * sizeof(S) == 8) {
        const uint2 r = __ldg(reinterpret_cast<const uint2 *>(p));
        memcpy(out, &r, 8);
    } else {
        const unsigned r = __ldg(reinterpret_cast<const unsigned *>(p));
        memcpy(out, &r, 4);
    }
}
template <class S, int V>
__device__ __forceinline__ void store_vec(S *__restrict__ p, const S (&in)[V])
{
    if constexpr (V * sizeof(S) == 16) {
        uint4 r;
        memcpy(&r, in, 16);
        *reinterpret_cast<uint4 *>(p) = r;
    } else {
        uint2 r;
        memcpy(&r, in, 8);
        *reinterpret_cast<uint2 *>(p) = r;
    }
}
template <class S> __device__ __forceinline__ S load_one(const S *__restrict__ p)
{
    if constexpr (sizeof(S) == 2) {
        const unsigned short v = __ldg(reinterpret_cast<const unsigned short *>(p));
        S s;
        memcpy(&s, &v, 2);
        return s;
    } else {
        return __ldg(p);
    }
}
template <class S> __device__ __forceinline__ S zero_elem()
{
    S s;
    memset(&s, 0, sizeof(S));
    return s;
}

// One storage element from lane +-delta (up: from the lower lane).
template <class S> __device__ __forceinline__ S shfl_elem(S v, int delta, bool up, unsigned mask = 0xffffffffu)
{
    if constexpr (sizeof(S) == 2) {
        unsigned short u;
        memcpy(&u, &v, 2);
        const int r = up ? __shfl_up_sync(mask, (int)u, delta) : __shfl_down_sync(mask, (int)u, delta);
        const unsigned short ur = (unsigned short)r;
        S o;
        memcpy(&o, &ur, 2);
        return o;
    } else {
        return up ? __shfl_up_sync(mask, v, delta) : __shfl_down_sync(mask, v, delta);
    }
}

// Pull one population for the V sites x0..x0+V-1 of a row: the values at
// x - EX.  `row` points at x = 0 of the source row.
template <class S, int V, int EX>
__device__ __forceinline__ void gather_row(const S *__restrict__ row, int x0, int dim, S (&out)[V])
{
    S v[V];
    load_vec<S, V>(row + x0, v);
    if constexpr (EX == 0) {
#pragma unroll
        for (int k = 0; k < V; ++k) out[k] = v[k];
    } else if constexpr (EX == 1) {
        out[0] = (x0 > 0) ? load_one(row + x0 - 1) : zero_elem<S>();
#pragma unroll
        for (int k = 1; k < V; ++k) out[k] = v[k - 1];
    } else {
#pragma unroll
        for (int k = 0; k < V - 1; ++k) out[k] = v[k + 1];
        out[V - 1] = (x0 + V < dim) ? load_one(row + x0 + V) : zero_elem<S>();
    }
}

template <int V> struct MapWord;
template <> struct MapWord<2> { using type = unsigned short; };
template <> struct MapWord<4> { using type = unsigned int; };
template <> struct MapWord<8> { using type = unsigned long long; };

template <class T> __device__ __forceinline__ T nan_of();
template <> __device__ __forceinline__ float nan_of<float>() { return __int_as_float(0x7fc00000); }
template <> __device__ __forceinline__ double nan_of<double>() { return __longlong_as_double(0x7ff8000000000000ll); }

template <class S, int V, int I>
__device__ __forceinline__ void gather_pop(const S *__restrict__ fin, size_t n, size_t rowoff, int dim, int x0,
                                           S (&out)[V])
{
    const ptrdiff_t shift = (ptrdiff_t)ez_of(I) * dim * dim + (ptrdiff_t)ey_of(I) * dim;
    gather_row<S, V, ex_of(I)>(fin + (size_t)I * n + rowoff - shift, x0, dim, out);
}

template <class S, int V, int I>
__device__ __forceinline__ void gather_all(const S *__restrict__ fin, size_t n, size_t rowoff, int dim, int x0,
                                           S (&fs)[Q][V])
{
    gather_pop<S, V, I>(fin, n, rowoff, dim, x0, fs[I]);
    if constexpr (I + 1 < Q) gather_all<S, V, I + 1>(fin, n, rowoff, dim, x0, fs);
}

// ---------------------------------------------------------------------------
// Site updates.  f holds the 19 pulled (pre-collision) values of one site.
// ---------------------------------------------------------------------------
struct SiteOut {
    bool macro;      // FLUID or MOVING: stores rho/u on macro iterations
    bool bad;        // density <= 0 or NaN on a FLUID / MOVING site
    double r, ux, uy, uz;
};

// Exact-order FP32 / FP64 site update.  COLLIDE = false only forms moments.
// sf: rho and u in the Sailfish summation order (block-uniform).
template <class T, bool COLLIDE>
__device__ __forceinline__ void site_exact(T (&f)[Q], uint8_t b, T lidv, T inv_tau, const Weights<T> &W,
                                           SiteOut &o, bool sf)
{
    using O = X<T>;
    o.macro = false;
    o.bad = false;
    if (b == 0) {  // FLUID
        T r, ux, uy, uz;
        if (sf) moments_sailfish(f, r, ux, uy, uz);
        else moments_exact(f, r, ux, uy, uz);
        o.macro = true;
        o.bad = !(r > (T)0);
        o.r = r; o.ux = ux; o.uy = uy; o.uz = uz;
        if (COLLIDE) relax_exact(f, r, ux, uy, uz, inv_tau, W);
        return;
    }
    if (b & M_WALL) return;
    // sources that are walls hold the site's initial equilibrium
#pragma unroll
    for (int i = 0; i < Q; ++i)
        if (wall_sourced(i, b)) f[i] = (b & M_FRONT) ? init_eq_exact(i, lidv, W) : W.w[wclass_of(i)];
    if (b == M_FRONT) {
        // moving lid (kernels.cl:343-349, 355, 362-367, 393-398)
        f[5] = f[6]; f[11] = f[17]; f[12] = f[18]; f[13] = f[15]; f[14] = f[16];
        T r;
        if (sf) {
            r = rho_sailfish(f);
        } else {
            r = f[0];
#pragma unroll
            for (int i = 1; i < Q; ++i) r = O::add(r, f[i]);
        }
        o.macro = true;
        o.bad = !(r > (T)0);
        o.r = r; o.ux = lidv; o.uy = 0; o.uz = 0;
        if (COLLIDE) {
            const T c15 = O::mul((T)1.5, O::add(O::add(O::mul(lidv, lidv), (T)0), (T)0));
            const T rw[3] = {O::mul(r, W.w[0]), O::mul(r, W.w[1]), O::mul(r, W.w[2])};
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                const T eu = ex_of(i) > 0 ? lidv : (ex_of(i) < 0 ? -lidv : (T)0);
                f[i] = O::mul(rw[wclass_of(i)], eq_bracket_exact(eu, c15));
            }
        }
        return;
    }
    if (b & M_CORNER) return;  // corners only propagate
    if (COLLIDE) {
        // full-way bounce-back of the nine opposite pairs (kernels.cl:400-408)
        T g[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) g[i] = f[opp_of(i)];
#pragma unroll
        for (int i = 0; i < Q; ++i) f[i] = g[i];
    }
}

// ---------------------------------------------------------------------------
// 16-bit deviation site update.  D holds s (f - w) as FP32.  Written for a
// low instruction count (the 16-bit kernels move half the bytes per site, so
// issue rate, not HBM, limits them otherwise): moments from opposite-pair sums
// and differences, and the BGK update of each opposite pair (i, -i) with
// e_i . u = +-a as
//     D'_(+-) = (1 - w) D_(+-) + K_c (drho + rho (4.5 a^2 - 1.5 u^2)) +- 3 K_c rho a,
// K_c = omega s w_c.  Every operation is an explicit IEEE intrinsic, so the
// result does not depend on where the compiler inlines it.
// ---------------------------------------------------------------------------
struct DevK {
    float keep;   // 1 - omega
    float k[3];   // omega * s * w_c
    float k3[3];  // 3 omega s w_c
    float inv_s;
};

__device__ __forceinline__ DevK make_devk(float omega, float s, float inv_s)
{
    DevK K;
    K.keep = __fsub_rn(1.0f, omega);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float w = c == 0 ? (1.0f / 3.0f) : (c == 1 ? (1.0f / 18.0f) : (1.0f / 36.0f));
        K.k[c] = __fmul_rn(__fmul_rn(omega, s), w);
        K.k3[c] = __fmul_rn(3.0f, K.k[c]);
    }
    K.inv_s = inv_s;
    return K;
}

__device__ __forceinline__ void relax_pair_dev(float &dp, float &dm, float a, int c, float rho, float drho, float c15,
                                               const DevK &K)
{
    const float p = __fmaf_rn(__fmul_rn(4.5f, a), a, -c15);
    const float X = __fmaf_rn(rho, p, drho);
    const float lin = __fmul_rn(__fmul_rn(K.k3[c], rho), a);
    dp = __fmaf_rn(K.keep, dp, __fmaf_rn(K.k[c], X, lin));
    dm = __fmaf_rn(K.keep, dm, __fmaf_rn(K.k[c], X, -lin));
}

// Moments of a FLUID site in deviation form (D = s (f - w)): drho = rho - 1,
// rho, u; the forward's own arithmetic, also the adjoint's linearisation point.
__device__ __forceinline__ void moments_dev(const float (&D)[Q], float inv_s, float &drho, float &rho, float &ux,
                                            float &uy, float &uz)
{
    const float s13 = __fadd_rn(D[1], D[3]), d13 = __fsub_rn(D[1], D[3]);
    const float s24 = __fadd_rn(D[2], D[4]), d24 = __fsub_rn(D[2], D[4]);
    const float s56 = __fadd_rn(D[5], D[6]), d65 = __fsub_rn(D[6], D[5]);
    const float s79 = __fadd_rn(D[7], D[9]), d79 = __fsub_rn(D[7], D[9]);         // e7 = (+1,+1, 0)
    const float s810 = __fadd_rn(D[8], D[10]), d810 = __fsub_rn(D[8], D[10]);     // e8 = (-1,+1, 0)
    const float s1117 = __fadd_rn(D[11], D[17]), d1117 = __fsub_rn(D[11], D[17]); // e11 = (+1, 0,-1)
    const float s1218 = __fadd_rn(D[12], D[18]), d1218 = __fsub_rn(D[12], D[18]); // e12 = ( 0,+1,-1)
    const float s1315 = __fadd_rn(D[13], D[15]), d1513 = __fsub_rn(D[15], D[13]); // e15 = (+1, 0,+1)
    const float s1416 = __fadd_rn(D[14], D[16]), d1614 = __fsub_rn(D[16], D[14]); // e16 = ( 0,+1,+1)
    const float sd = __fadd_rn(__fadd_rn(D[0], s1416),
                               __fadd_rn(__fadd_rn(__fadd_rn(s13, s24), __fadd_rn(s56, s79)),
                                         __fadd_rn(__fadd_rn(s810, s1117), __fadd_rn(s1218, s1315))));
    const float jx = __fadd_rn(__fsub_rn(__fadd_rn(d13, d79), d810), __fadd_rn(d1117, d1513));
    const float jy = __fadd_rn(__fadd_rn(__fadd_rn(d24, d79), d810), __fadd_rn(d1218, d1614));
    const float jz = __fadd_rn(__fsub_rn(__fsub_rn(d65, d1117), d1218), __fadd_rn(d1513, d1614));
    drho = __fmul_rn(sd, inv_s);
    rho = __fadd_rn(1.0f, drho);
    const float kk = __fmul_rn(inv_s, __fdividef(1.0f, rho));
    ux = __fmul_rn(jx, kk);
    uy = __fmul_rn(jy, kk);
    uz = __fmul_rn(jz, kk);
}

// The BGK update of fluid_dev for one site from its moments.
__device__ __forceinline__ void relax_dev(float (&D)[Q], float drho, float rho, float ux, float uy, float uz,
                                          const DevK &K)
{
    const float c15 = __fmul_rn(1.5f, __fmaf_rn(ux, ux, __fmaf_rn(uy, uy, __fmul_rn(uz, uz))));
    D[0] = __fmaf_rn(K.keep, D[0], __fmul_rn(K.k[0], __fmaf_rn(rho, -c15, drho)));
    relax_pair_dev(D[1], D[3], ux, 1, rho, drho, c15, K);
    relax_pair_dev(D[2], D[4], uy, 1, rho, drho, c15, K);
    relax_pair_dev(D[6], D[5], uz, 1, rho, drho, c15, K);
    relax_pair_dev(D[7], D[9], __fadd_rn(ux, uy), 2, rho, drho, c15, K);
    relax_pair_dev(D[8], D[10], __fsub_rn(uy, ux), 2, rho, drho, c15, K);
    relax_pair_dev(D[11], D[17], __fsub_rn(ux, uz), 2, rho, drho, c15, K);
    relax_pair_dev(D[12], D[18], __fsub_rn(uy, uz), 2, rho, drho, c15, K);
    relax_pair_dev(D[15], D[13], __fadd_rn(ux, uz), 2, rho, drho, c15, K);
    relax_pair_dev(D[16], D[14], __fadd_rn(uy, uz), 2, rho, drho, c15, K);
}

// FLUID site in deviation form.
template <bool COLLIDE>
__device__ __forceinline__ void fluid_dev(float (&D)[Q], const DevK &K, SiteOut &o)
{
    float drho, rho, ux, uy, uz;
    moments_dev(D, K.inv_s, drho, rho, ux, uy, uz);
    o.macro = true;
    o.bad = !(rho > 0.0f);
    o.r = rho; o.ux = ux; o.uy = uy; o.uz = uz;
    if (COLLIDE) relax_dev(D, drho, rho, ux, uy, uz, K);
}

// Two FLUID sites at once on packed FP32 pairs (lane .x one site, .y the
// other): the operations of moments_dev / fluid_dev in the same order and
// rounding (add/mul/fma .rn on f32x2), so each lane's result is bit for bit
// the scalar one, in fewer arithmetic instructions.  RELAX2: the BGK update
// packed too (its constants then live as register pairs), else per lane with
// the scalar relax_pair_dev.
__device__ __forceinline__ float2 f2_(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }  // exact: a + (-b)
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ void relax_pair_dev2(float2 &dp, float2 &dm, float2 a, int c, float2 rho, float2 drho,
                                                float2 c15, const DevK &K)
{
    const float2 p = fma2(mul2(f2_(4.5f), a), a, neg2(c15));
    const float2 X = fma2(rho, p, drho);
    const float2 lin = mul2(mul2(f2_(K.k3[c]), rho), a);
    dp = fma2(f2_(K.keep), dp, fma2(f2_(K.k[c]), X, lin));
    dm = fma2(f2_(K.keep), dm, fma2(f2_(K.k[c]), X, neg2(lin)));
}

template <bool COLLIDE, bool RELAX2>
__device__ __forceinline__ void fluid_dev2(float2 (&D)[Q], const DevK &K, SiteOut &o0, SiteOut &o1)
{
    const float2 s13 = add2(D[1], D[3]), d13 = sub2(D[1], D[3]);
    const float2 s24 = add2(D[2], D[4]), d24 = sub2(D[2], D[4]);
    const float2 s56 = add2(D[5], D[6]), d65 = sub2(D[6], D[5]);
    const float2 s79 = add2(D[7], D[9]), d79 = sub2(D[7], D[9]);
    const float2 s810 = add2(D[8], D[10]), d810 = sub2(D[8], D[10]);
    const float2 s1117 = add2(D[11], D[17]), d1117 = sub2(D[11], D[17]);
    const float2 s1218 = add2(D[12], D[18]), d1218 = sub2(D[12], D[18]);
    const float2 s1315 = add2(D[13], D[15]), d1513 = sub2(D[15], D[13]);
    const float2 s1416 = add2(D[14], D[16]), d1614 = sub2(D[16], D[14]);
    const float2 sd = add2(add2(D[0], s1416), add2(add2(add2(s13, s24), add2(s56, s79)),
                                                   add2(add2(s810, s1117), add2(s1218, s1315))));
    const float2 jx = add2(sub2(add2(d13, d79), d810), add2(d1117, d1513));
    const float2 jy = add2(add2(add2(d24, d79), d810), add2(d1218, d1614));
    const float2 jz = add2(sub2(sub2(d65, d1117), d1218), add2(d1513, d1614));
    const float2 drho = mul2(sd, f2_(K.inv_s));
    const float2 rho = add2(f2_(1.0f), drho);
    const float2 kk = mul2(f2_(K.inv_s), make_float2(__fdividef(1.0f, rho.x), __fdividef(1.0f, rho.y)));
    const float2 ux = mul2(jx, kk), uy = mul2(jy, kk), uz = mul2(jz, kk);
    o0.macro = o1.macro = true;
    o0.bad = !(rho.x > 0.0f);
    o1.bad = !(rho.y > 0.0f);
    o0.r = rho.x; o0.ux = ux.x; o0.uy = uy.x; o0.uz = uz.x;
    o1.r = rho.y; o1.ux = ux.y; o1.uy = uy.y; o1.uz = uz.y;
    if (!COLLIDE) return;
    if constexpr (RELAX2) {
        const float2 c15 = mul2(f2_(1.5f), fma2(ux, ux, fma2(uy, uy, mul2(uz, uz))));
        D[0] = fma2(f2_(K.keep), D[0], mul2(f2_(K.k[0]), fma2(rho, neg2(c15), drho)));
        relax_pair_dev2(D[1], D[3], ux, 1, rho, drho, c15, K);
        relax_pair_dev2(D[2], D[4], uy, 1, rho, drho, c15, K);
        relax_pair_dev2(D[6], D[5], uz, 1, rho, drho, c15, K);
        relax_pair_dev2(D[7], D[9], add2(ux, uy), 2, rho, drho, c15, K);
        relax_pair_dev2(D[8], D[10], sub2(uy, ux), 2, rho, drho, c15, K);
        relax_pair_dev2(D[11], D[17], sub2(ux, uz), 2, rho, drho, c15, K);
        relax_pair_dev2(D[12], D[18], sub2(uy, uz), 2, rho, drho, c15, K);
        relax_pair_dev2(D[15], D[13], add2(ux, uz), 2, rho, drho, c15, K);
        relax_pair_dev2(D[16], D[14], add2(uy, uz), 2, rho, drho, c15, K);
    } else {
        float L[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) L[i] = D[i].x;
        relax_dev(L, drho.x, rho.x, ux.x, uy.x, uz.x, K);
#pragma unroll
        for (int i = 0; i < Q; ++i) D[i].x = L[i];
#pragma unroll
        for (int i = 0; i < Q; ++i) L[i] = D[i].y;
        relax_dev(L, drho.y, rho.y, ux.y, uy.y, uz.y, K);
#pragma unroll
        for (int i = 0; i < Q; ++i) D[i].y = L[i];
    }
}

// Any site in deviation form (walls, faces, corners, lid, fluid).
template <bool COLLIDE>
__device__ __forceinline__ void site_dev(float (&D)[Q], uint8_t b, float lidv, const DevK &K, float s, SiteOut &o)
{
    o.macro = false;
    o.bad = false;
    if (b == 0) {
        fluid_dev<COLLIDE>(D, K, o);
        return;
    }
    if (b & M_WALL) return;
#pragma unroll
    for (int i = 0; i < Q; ++i)
        if (wall_sourced(i, b)) {
            if (b & M_FRONT) {
                const float eu = ex_of(i) > 0 ? lidv : (ex_of(i) < 0 ? -lidv : 0.0f);
                D[i] = deq_scaled(i, 0.0f, 1.0f, eu, 1.5f * lidv * lidv, s);
            } else {
                D[i] = 0.0f;
            }
        }
    if (b == M_FRONT) {
        // moving lid: wall-sourced -z populations take their +z opposites, then
        // the site is set to the equilibrium at its density and the lid velocity
        D[5] = D[6]; D[11] = D[17]; D[12] = D[18]; D[13] = D[15]; D[14] = D[16];
        float sd = 0.0f;
#pragma unroll
        for (int i = 0; i < Q; ++i) sd += D[i];
        const float drho = sd * K.inv_s;
        const float rho = 1.0f + drho;
        o.macro = true;
        o.bad = !(rho > 0.0f);
        o.r = rho; o.ux = lidv; o.uy = 0.0f; o.uz = 0.0f;
        if (COLLIDE) {
            const float c15 = 1.5f * lidv * lidv;
#pragma unroll
            for (int i = 0; i < Q; ++i) D[i] = deq_scaled(i, drho, rho, proj_fast(i, lidv, 0.0f, 0.0f), c15, s);
        }
        return;
    }
    if (b & M_CORNER) return;
    if (COLLIDE) {
        float g[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) g[i] = D[opp_of(i)];
#pragma unroll
        for (int i = 0; i < Q; ++i) D[i] = g[i];
    }
}

// Block reduction of (mass, energy) in double, written to partials[2*block]
// (partials already offset by the launch's first block).
__device__ __forceinline__ void block_reduce_write(double m, double e, double *partials)
{
    // warp shuffles: the reductions are the only place this code uses them
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        m += __shfl_down_sync(0xffffffffu, m, off);
        e += __shfl_down_sync(0xffffffffu, e, off);
    }
    __shared__ double sm[2][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sm[0][warp] = m; sm[1][warp] = e; }
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        m = lane < nw ? sm[0][lane] : 0.0;
        e = lane < nw ? sm[1][lane] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            m += __shfl_down_sync(0xffffffffu, m, off);
            e += __shfl_down_sync(0xffffffffu, e, off);
        }
        if (lane == 0) {
            partials[2 * blockIdx.x] = m;
            partials[2 * blockIdx.x + 1] = e;
        }
    }
}

// Block sum of v added to acc[blockIdx.x] (one writer per slot and launch, so
// successive launches with the same grid accumulate deterministically).
__device__ __forceinline__ void block_reduce_add(double v, double *acc)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    __shared__ double sm[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? sm[lane] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) acc[blockIdx.x] += v;
    }
}

// ---------------------------------------------------------------------------
// The fused pull-stream + collide iteration.
// ---------------------------------------------------------------------------
template <class C>
__device__ __forceinline__ void store_macro(const StepArgs &a, size_t id, const SiteOut &o)
{
    C *rho = static_cast<C *>(a.rho);
    C *u = static_cast<C *>(a.u);
    rho[id] = (C)o.r;
    u[id] = (C)o.ux;
    u[a.n + id] = (C)o.uy;
    u[2 * a.n + id] = (C)o.uz;
}

// The adjoint's linearisation point of one site (MODE_STEP_ADJ): u of a
// FLUID site, rho (then 0, 0) of a MOVING site, in the three planes at a.u.
template <class C>
__device__ __forceinline__ void store_adj(const StepArgs &a, size_t id, const SiteOut &o, bool moving)
{
    C *u = static_cast<C *>(a.u);
    u[id] = moving ? (C)o.r : (C)o.ux;
    u[a.n + id] = (C)o.uy;
    u[2 * a.n + id] = (C)o.uz;
}

// rho / u (MODE_STEP_MACRO) or the FLUID linearisation point (MODE_STEP_ADJ)
// of two neighbouring FLUID-or-not sites (id even) with one 2-element vector
// store per field when both store, else per site
template <class C> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };
template <class C, int MODE>
__device__ __forceinline__ void store_macro_pair(const StepArgs &a, size_t id, bool s0, bool s1, const SiteOut &o0,
                                                 const SiteOut &o1)
{
    static_assert(MODE == MODE_STEP_MACRO || MODE == MODE_STEP_ADJ, "storing modes");
    if (s0 && s1) {
        using V2 = typename Vec2<C>::type;
        C *u = static_cast<C *>(a.u);
        if (MODE == MODE_STEP_MACRO) {
            C *rho = static_cast<C *>(a.rho);
            *reinterpret_cast<V2 *>(rho + id) = V2{(C)o0.r, (C)o1.r};
        }
        *reinterpret_cast<V2 *>(u + id) = V2{(C)o0.ux, (C)o1.ux};
        *reinterpret_cast<V2 *>(u + a.n + id) = V2{(C)o0.uy, (C)o1.uy};
        *reinterpret_cast<V2 *>(u + 2 * a.n + id) = V2{(C)o0.uz, (C)o1.uz};
        return;
    }
    if (MODE == MODE_STEP_MACRO) {
        if (s0) store_macro<C>(a, id, o0);
        if (s1) store_macro<C>(a, id + 1, o1);
    } else {
        if (s0) store_adj<C>(a, id, o0, false);
        if (s1) store_adj<C>(a, id + 1, o1, false);
    }
}

__device__ __forceinline__ void accumulate(const SiteOut &o, double &m, double &e)
{
    m += o.r;
    e += 0.5 * o.r * (o.ux * o.ux + o.uy * o.uy + o.uz * o.uz);
}

// Any mix of site kinds (face rows): per-site, map-driven update.
template <class S, int MODE, int V>
__device__ __forceinline__ void update_general(S (&fs)[Q][V], typename MapWord<V>::type mw, const StepArgs &a,
                                               int y, int z, int x0, size_t site0, double &red_m, double &red_e)
{
    using C = typename Compute<S>::type;
    constexpr bool DEV = is_dev16<S>();
    const int dim = a.dim;
    const bool lid_row = (z == dim - 2);
    const C *lid = static_cast<const C *>(a.lid);
    const Weights<C> W = make_weights<C>();
    const C inv_tau = (C)a.inv_tau;
    const DevK K = make_devk(a.omega_f, Dev16<S>::scale, Dev16<S>::inv_scale);
    bool bad = false;
#pragma unroll
    for (int k = 0; k < V; ++k) {
        const uint8_t b = (uint8_t)(mw >> (8 * k));
        const C lidv = lid_row ? lid[(size_t)y * dim + x0 + k] : (C)0;
        SiteOut o;
        if constexpr (DEV) {
            float D[Q];
#pragma unroll
            for (int i = 0; i < Q; ++i) D[i] = Dev16<S>::to_f(fs[i][k]);
            site_dev<MODE != MODE_REDUCE>(D, b, (float)lidv, K, Dev16<S>::scale, o);
#pragma unroll
            for (int i = 0; i < Q; ++i) fs[i][k] = Dev16<S>::from_f(D[i]);
        } else {
            C f[Q];
#pragma unroll
            for (int i = 0; i < Q; ++i) f[i] = fs[i][k];
            site_exact<C, MODE != MODE_REDUCE>(f, b, lidv, inv_tau, W, o, a.sailfish != 0);
#pragma unroll
            for (int i = 0; i < Q; ++i) fs[i][k] = f[i];
        }
        bad |= o.bad;
        if (MODE == MODE_STEP_MACRO && o.macro) store_macro<C>(a, site0 + k, o);
        if (MODE == MODE_STEP_ADJ && o.macro) store_adj<C>(a, site0 + k, o, b != 0);
        if (MODE == MODE_REDUCE && o.macro) accumulate(o, red_m, red_e);
    }
    if (bad) atomicOr(a.status, 1);
}

// Instruction form of the all-FLUID pairs of the 16-bit kernels (the same
// bits either way): 0 = two scalar site updates, 1 = packed FP32x2 moments
// and scalar BGK updates, 2 = packed throughout.  Chosen per storage type by
// measurement at 512^3 (the packed forms change the register allocation at
// the 168-register cap, which decides).
#ifndef LBM_DEV16_FORM_F16
#define LBM_DEV16_FORM_F16 0
#endif
#ifndef LBM_DEV16_FORM_BF16
#define LBM_DEV16_FORM_BF16 2
#endif
template <class S> __host__ __device__ constexpr int dev16_form()
{
    return sizeof(S) != 2 ? 0 : (std::is_same<S, __half>::value ? LBM_DEV16_FORM_F16 : LBM_DEV16_FORM_BF16);
}

// Update the V sites x0..x0+V-1 of row (y, z) in place: fs holds their pulled
// populations on entry and their post-collision populations on exit.  Stores
// rho / u (MODE_STEP_MACRO) or accumulates the reduction sums (MODE_REDUCE).
template <class S, int MODE, int V, bool FLUID_ONLY = false>
__device__ __forceinline__ void update_vector(S (&fs)[Q][V], typename MapWord<V>::type mw, const StepArgs &a,
                                              int y, int z, int x0, size_t site0, double &red_m, double &red_e)
{
    using C = typename Compute<S>::type;
    constexpr bool DEV = is_dev16<S>();
    const int dim = a.dim;
    const Weights<C> W = make_weights<C>();
    const C inv_tau = (C)a.inv_tau;
    bool bad = false;

    const DevK K = make_devk(a.omega_f, Dev16<S>::scale, Dev16<S>::inv_scale);
    if constexpr (!DEV) {
        if (FLUID_ONLY) {
#pragma unroll
            for (int k = 0; k < V; k += 2) {
                SiteOut o[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    C f[Q];
#pragma unroll
                    for (int i = 0; i < Q; ++i) f[i] = fs[i][k + h];
                    site_exact<C, MODE != MODE_REDUCE>(f, 0, (C)0, inv_tau, W, o[h], a.sailfish != 0);
#pragma unroll
                    for (int i = 0; i < Q; ++i) fs[i][k + h] = f[i];
                }
                // x in [2, dim-3] is FLUID; the row ends are walls / faces
                const bool f0 = (unsigned)(x0 + k - 2) <= (unsigned)(dim - 5);
                const bool f1 = (unsigned)(x0 + k - 1) <= (unsigned)(dim - 5);
                bad |= (f0 && o[0].bad) || (f1 && o[1].bad);
                if constexpr (MODE == MODE_STEP_MACRO || MODE == MODE_STEP_ADJ)
                    store_macro_pair<C, MODE>(a, site0 + k, f0, f1, o[0], o[1]);
                if (MODE == MODE_REDUCE) {
                    if (f0) accumulate(o[0], red_m, red_e);
                    if (f1) accumulate(o[1], red_m, red_e);
                }
            }
            if (bad) atomicOr(a.status, 1);
            return;
        }
    }
    if constexpr (DEV) {
        if (FLUID_ONLY || mw == 0) {
            // all V sites FLUID (the bulk of the lattice): no per-site branches,
            // two sites per step so the output converts as packed pairs
#pragma unroll
            for (int k = 0; k < V; k += 2) {
                SiteOut o0, o1;
                if constexpr (dev16_form<S>() == 0) {
                    float D0[Q], D1[Q];
#pragma unroll
                    for (int i = 0; i < Q; ++i) {
                        D0[i] = Dev16<S>::to_f(fs[i][k]);
                        D1[i] = Dev16<S>::to_f(fs[i][k + 1]);
                    }
                    fluid_dev<MODE != MODE_REDUCE>(D0, K, o0);
                    fluid_dev<MODE != MODE_REDUCE>(D1, K, o1);
                    if (MODE != MODE_REDUCE) {
#pragma unroll
                        for (int i = 0; i < Q; ++i) Dev16<S>::from_f2(D0[i], D1[i], fs[i][k], fs[i][k + 1]);
                    }
                } else {
                    float2 D[Q];
#pragma unroll
                    for (int i = 0; i < Q; ++i)
                        D[i] = make_float2(Dev16<S>::to_f(fs[i][k]), Dev16<S>::to_f(fs[i][k + 1]));
                    fluid_dev2<MODE != MODE_REDUCE, dev16_form<S>() == 2>(D, K, o0, o1);
                    if (MODE != MODE_REDUCE) {
#pragma unroll
                        for (int i = 0; i < Q; ++i) Dev16<S>::from_f2(D[i].x, D[i].y, fs[i][k], fs[i][k + 1]);
                    }
                }
                // in an interior row, x in [2, dim-3] is FLUID; the row ends are walls / faces
                const bool f0 = !FLUID_ONLY || (unsigned)(x0 + k - 2) <= (unsigned)(dim - 5);
                const bool f1 = !FLUID_ONLY || (unsigned)(x0 + k - 1) <= (unsigned)(dim - 5);
                bad |= (f0 && o0.bad) || (f1 && o1.bad);
                if constexpr (MODE == MODE_STEP_MACRO || MODE == MODE_STEP_ADJ)
                    store_macro_pair<C, MODE>(a, site0 + k, f0, f1, o0, o1);
                if (MODE == MODE_REDUCE) {
                    if (f0) accumulate(o0, red_m, red_e);
                    if (f1) accumulate(o1, red_m, red_e);
                }
            }
            if (bad) atomicOr(a.status, 1);
            return;
        }
    }
    if constexpr (!FLUID_ONLY) update_general<S, MODE, V>(fs, mw, a, y, z, x0, site0, red_m, red_e);
}


// Bounce-back of the x-face site x = xf of an interior row (y, z in
// [2, dim-3]): its output population i is its pulled input of the opposite
// direction, and an input whose source is the wall (x = 0 or dim-1) is the
// site's initial equilibrium w_i (kernels.cl:400-408 with the fixed
// wall-sourced slots; interior rows are never on the lid).  Reloaded from
// the input buffer, so the interior fast path can run on every lane first.
template <class S, int V>
__device__ __forceinline__ void face_fix(const StepArgs &a, size_t rowoff, int xf, int k, S (&fs)[Q][V])
{
    using C = typename Compute<S>::type;
    const S *__restrict__ fin = static_cast<const S *>(a.fin);
    const int dim = a.dim;
    const Weights<C> W = make_weights<C>();
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const int j = opp_of(i);
        const int sx = xf - ex_of(j);
        S v;
        if (sx == 0 || sx == dim - 1) {
            if constexpr (is_dev16<S>()) v = zero_elem<S>();
            else v = (S)W.w[wclass_of(j)];
        } else {
            const ptrdiff_t shift = (ptrdiff_t)ez_of(j) * dim * dim + (ptrdiff_t)ey_of(j) * dim;
            v = load_one(fin + (size_t)j * a.n + rowoff - shift + sx);
        }
        fs[i][k] = v;
    }
}

template <class S, int MODE, int V, bool INTERIOR>
__device__ __forceinline__ void pull_vector(const StepArgs &a, int xv, int y, int z, double &red_m, double &red_e)
{
    const int dim = a.dim;
    const int x0 = xv * V;
    const size_t rowoff = (size_t)z * dim * dim + (size_t)y * dim;
    const size_t site0 = rowoff + (size_t)x0;
    typename MapWord<V>::type mw = 0;
    if (!INTERIOR) mw = __ldg(reinterpret_cast<const typename MapWord<V>::type *>(a.map + site0));
    const S *__restrict__ fin = static_cast<const S *>(a.fin);
    S fs[Q][V];
    gather_all<S, V, 0>(fin, a.n, rowoff, dim, x0, fs);
    update_vector<S, MODE, V, INTERIOR>(fs, mw, a, y, z, x0, site0, red_m, red_e);
    if (INTERIOR && MODE != MODE_REDUCE) {
        // the walls (x = 0, dim-1) hold values nobody reads; the faces bounce back
        if (x0 == 0) face_fix<S, V>(a, rowoff, 1, 1, fs);
        if (x0 + V == dim) face_fix<S, V>(a, rowoff, dim - 2, V - 2, fs);
    }
    if (MODE != MODE_REDUCE) {
        S *__restrict__ fout = static_cast<S *>(a.fout);
#pragma unroll
        for (int i = 0; i < Q; ++i) store_vec<S, V>(fout + (size_t)i * a.n + site0, fs[i]);
    }
}

// ---------------------------------------------------------------------------
// Direct variant: every thread loads its V sites' populations with VB-byte
// vector loads straight from HBM (V = VB / sizeof(S)).  One iteration is two
// launches over disjoint sets of whole rows:
//   ROWS_INTERIOR  the (dim-4)^2 rows with y, z in [2, dim-3]: branch-free
//                  FLUID update on every lane, the two x-face sites of each
//                  row patched afterwards by face_fix (no map read)
//   ROWS_FACES     the 4 (dim-3) rows with y or z in {1, dim-2}: the general,
//                  map-driven site update
// Each launch gets its own register allocation, and rows stay whole, so no
// 32-byte sector is shared between the two launches.
// ---------------------------------------------------------------------------
enum { ROWS_INTERIOR = 0, ROWS_FACES = 1 };

// face row index -> (y, z): plane z = 1, plane z = dim-2, then rows y = 1 and
// y = dim-2 of the planes 2 .. dim-3
__device__ __forceinline__ void decode_face_row(int dim, unsigned br, int &y, int &z)
{
    const unsigned side = (unsigned)(dim - 2);
    if (br < side) {
        z = 1;
        y = 1 + (int)br;
    } else if (br < 2 * side) {
        z = dim - 2;
        y = 1 + (int)(br - side);
    } else {
        const unsigned k = br - 2 * side;
        z = 2 + (int)(k / 2);
        y = (k & 1) ? dim - 2 : 1;
    }
}

// Launch bounds of the iteration kernels: the largest block each is compiled
// for and the blocks of that size that must fit an SM, i.e. the register cap
// 65536 / (threads n).  Measured at 512^3 on GB300: 16-bit storage runs
// fastest at 128-thread blocks with three per SM (168 registers, no spills:
// 84,448 MLUPS against 82,201 at 128 registers, which spill 88 bytes); FP32
// with 8-byte vectors at 85 registers (256 x 3); FP64 is FP64-throughput bound
// and left uncapped.  lbm_init clamps block_threads to max_threads.
#ifndef LBM_MINB_16
#define LBM_MINB_16 3
#endif
#ifndef LBM_MAXT_16
#define LBM_MAXT_16 128
#endif
#ifndef LBM_MINB_32_V16
#define LBM_MINB_32_V16 2
#endif
#ifndef LBM_MINB_32_V8
#define LBM_MINB_32_V8 3
#endif
#ifndef LBM_MINB_64
#define LBM_MINB_64 1
#endif
template <class S, int VB> constexpr int min_blocks()
{
    return sizeof(S) == 2 ? LBM_MINB_16
         : sizeof(S) == 4 ? (VB == 16 ? LBM_MINB_32_V16 : LBM_MINB_32_V8)
                          : LBM_MINB_64;
}
template <class S> constexpr int max_threads() { return sizeof(S) == 2 ? LBM_MAXT_16 : 256; }

template <class S, int MODE, int VB, int ROWS>
__global__ void __launch_bounds__(max_threads<S>(), min_blocks<S, VB>()) pull_kernel(StepArgs a)
{
    constexpr int V = VB / (int)sizeof(S);
    const unsigned g = blockIdx.x * blockDim.x + threadIdx.x;
    double red_m = 0.0, red_e = 0.0;
    const unsigned nrows = ROWS == ROWS_INTERIOR ? (unsigned)(a.dim - 4) * (unsigned)(a.dim - 4)
                                                 : 4u * (unsigned)(a.dim - 3);
    if (g < nrows * (unsigned)a.nvx) {
        const int dim = a.dim;
        const unsigned row = g / (unsigned)a.nvx;
        const int xv = (int)(g - row * (unsigned)a.nvx);
        int y, z;
        if (ROWS == ROWS_INTERIOR) {
            y = 2 + (int)(row % (unsigned)(dim - 4));
            z = 2 + (int)(row / (unsigned)(dim - 4));
        } else {
            decode_face_row(dim, row, y, z);
        }
        pull_vector<S, MODE, V, ROWS == ROWS_INTERIOR>(a, xv, y, z, red_m, red_e);
    }
    if (MODE == MODE_REDUCE) block_reduce_write(red_m, red_e, a.partials + 2 * (size_t)a.partial_base);
}

// ---------------------------------------------------------------------------
// AA pattern: one lattice updated in place, two kinds of iteration.
//   A-form buffer: f(s, i) = R(s, i), the post-stream value of slot (s, i)
//   B-form buffer: f(s, opp i) = P_i(s), the post-collision value of site s
// A-step (A-form -> B-form): every site reads its own 19 slots and writes its
// post-collision populations to its own opposite slots; aligned vectors, no
// neighbour.  B-step (B-form -> A-form): site s reads g_i = f(s - e_i, opp i)
// (the pull of the two-lattice kernel, from the opposite population) and
// writes P_i(s) to f(s + e_i, i).  Each slot is read and written by one site
// per step, reads first, so the update is race-free in place.  The B-step's
// x-shifted stores are realigned in registers: a lane's aligned destination
// vector takes one element from its neighbour lane (warp shuffle); the
// element that crosses a warp boundary is stored by its own lane as a
// scalar, and the receiving lane stores the rest of its vector element-wise.
// Lanes of wall sites compute garbage that lands only in wall slots whose
// source is a wall (or outside the lattice) and in wall-sourced slots of
// boundary sites: slots that no iteration and no dump reads.
// ---------------------------------------------------------------------------
// out[k] (site x0 + k) to position x0 + k + EX of a row (`row` at x = 0).
// Every lane of the warp calls this (the shuffles); inactive lanes store
// nothing.
template <class S, int V, int EX>
__device__ __forceinline__ void store_row_shifted(S *__restrict__ row, int x0, int dim, const S (&out)[V],
                                                  bool active, int lane)
{
    if constexpr (EX == 0) {
        if (active) store_vec<S, V>(row + x0, out);
    } else if constexpr (EX == 1) {
        const S prev = shfl_elem(out[V - 1], 1, true);
        if (!active) return;
        S v[V];
        v[0] = prev;
#pragma unroll
        for (int k = 1; k < V; ++k) v[k] = out[k - 1];
        if (lane != 0 || x0 == 0) {
            store_vec<S, V>(row + x0, v);  // at a row start v[0] is a wall slot's don't-care
        } else {
#pragma unroll
            for (int k = 1; k < V; ++k) row[x0 + k] = v[k];
        }
        if (lane == 31 && x0 + V < dim) row[x0 + V] = out[V - 1];
    } else {
        const S next = shfl_elem(out[0], 1, false);
        if (!active) return;
        S v[V];
#pragma unroll
        for (int k = 0; k < V - 1; ++k) v[k] = out[k + 1];
        v[V - 1] = next;
        if (lane != 31 || x0 + V == dim) {
            store_vec<S, V>(row + x0, v);  // at a row end v[V-1] is a wall slot's don't-care
        } else {
#pragma unroll
            for (int k = 0; k < V - 1; ++k) row[x0 + k] = v[k];
        }
        if (lane == 0 && x0 > 0) row[x0 - 1] = out[0];
    }
}

// The pre-collision populations of V sites from the one lattice.
template <class S, int V, int I, int PHASE>
__device__ __forceinline__ void gather_aa(const S *__restrict__ f, size_t n, size_t rowoff, int dim, int x0,
                                          S (&fs)[Q][V])
{
    if constexpr (PHASE == 0) {
        load_vec<S, V>(f + (size_t)I * n + rowoff + x0, fs[I]);
    } else {
        const ptrdiff_t shift = (ptrdiff_t)ez_of(I) * dim * dim + (ptrdiff_t)ey_of(I) * dim;
        gather_row<S, V, ex_of(I)>(f + (size_t)opp_of(I) * n + rowoff - shift, x0, dim, fs[I]);
    }
    if constexpr (I + 1 < Q) gather_aa<S, V, I + 1, PHASE>(f, n, rowoff, dim, x0, fs);
}

// Bounce-back of the x-face site xf of an interior row (see face_fix): its
// output i is its input opp(i), a wall-sourced input being the constant.
template <class S, int V, int PHASE>
__device__ __forceinline__ void face_fix_aa(const StepArgs &a, size_t rowoff, int xf, int k, S (&fs)[Q][V])
{
    using C = typename Compute<S>::type;
    const S *__restrict__ f = static_cast<const S *>(a.fout);
    const int dim = a.dim;
    const Weights<C> W = make_weights<C>();
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const int j = opp_of(i);
        const int sx = xf - ex_of(j);
        S v;
        if (sx == 0 || sx == dim - 1) {
            if constexpr (is_dev16<S>()) v = zero_elem<S>();
            else v = (S)W.w[wclass_of(j)];
        } else if constexpr (PHASE == 0) {
            v = load_one(f + (size_t)j * a.n + rowoff + xf);  // own slot j
        } else {
            const ptrdiff_t shift = (ptrdiff_t)ez_of(j) * dim * dim + (ptrdiff_t)ey_of(j) * dim;
            v = load_one(f + (size_t)i * a.n + rowoff - shift + sx);  // f(s - e_j, opp j)
        }
        fs[i][k] = v;
    }
}

template <class S, int MODE, int V, bool INTERIOR, int PHASE>
__device__ __forceinline__ void aa_vector(const StepArgs &a, bool active, int xv, int y, int z, double &red_m,
                                          double &red_e)
{
    const int dim = a.dim;
    const int x0 = xv * V;
    const size_t rowoff = (size_t)z * dim * dim + (size_t)y * dim;
    const size_t site0 = rowoff + (size_t)x0;
    S *__restrict__ f = static_cast<S *>(a.fout);
    S fs[Q][V];
    if (active) {
        typename MapWord<V>::type mw = 0;
        if (!INTERIOR) mw = __ldg(reinterpret_cast<const typename MapWord<V>::type *>(a.map + site0));
        gather_aa<S, V, 0, PHASE>(f, a.n, rowoff, dim, x0, fs);
        update_vector<S, MODE, V, INTERIOR>(fs, mw, a, y, z, x0, site0, red_m, red_e);
        if (INTERIOR && MODE != MODE_REDUCE) {
            if (x0 == 0) face_fix_aa<S, V, PHASE>(a, rowoff, 1, 1, fs);
            if (x0 + V == dim) face_fix_aa<S, V, PHASE>(a, rowoff, dim - 2, V - 2, fs);
        }
    }
    if constexpr (MODE != MODE_REDUCE) {
        if constexpr (PHASE == 0) {
            if (active) {
#pragma unroll
                for (int i = 0; i < Q; ++i) store_vec<S, V>(f + (size_t)opp_of(i) * a.n + site0, fs[i]);
            }
        } else {
            const int lane = (int)(threadIdx.x & 31);
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                const ptrdiff_t shift = (ptrdiff_t)ez_of(i) * dim * dim + (ptrdiff_t)ey_of(i) * dim;
                S *row = f + (size_t)i * a.n + (size_t)((ptrdiff_t)rowoff + shift);
                if (ex_of(i) == 1) store_row_shifted<S, V, 1>(row, x0, dim, fs[i], active, lane);
                else if (ex_of(i) == -1) store_row_shifted<S, V, -1>(row, x0, dim, fs[i], active, lane);
                else store_row_shifted<S, V, 0>(row, x0, dim, fs[i], active, lane);
            }
        }
    }
}

// One AA iteration (or reduction pass) over the rows of one kind; a.fout is
// the lattice, PHASE 0 = A-step, 1 = B-step.  Same row split and register
// caps as pull_kernel.
template <class S, int MODE, int VB, int ROWS, int PHASE>
__global__ void __launch_bounds__(max_threads<S>(), min_blocks<S, VB>()) aa_kernel(StepArgs a)
{
    constexpr int V = VB / (int)sizeof(S);
    const unsigned g = blockIdx.x * blockDim.x + threadIdx.x;
    double red_m = 0.0, red_e = 0.0;
    const unsigned nrows = ROWS == ROWS_INTERIOR ? (unsigned)(a.dim - 4) * (unsigned)(a.dim - 4)
                                                 : 4u * (unsigned)(a.dim - 3);
    const bool active = g < nrows * (unsigned)a.nvx;
    int y = 2, z = 2, xv = 0;
    if (active) {
        const int dim = a.dim;
        const unsigned row = g / (unsigned)a.nvx;
        xv = (int)(g - row * (unsigned)a.nvx);
        if (ROWS == ROWS_INTERIOR) {
            y = 2 + (int)(row % (unsigned)(dim - 4));
            z = 2 + (int)(row / (unsigned)(dim - 4));
        } else {
            decode_face_row(dim, row, y, z);
        }
    }
    aa_vector<S, MODE, V, ROWS == ROWS_INTERIOR, PHASE>(a, active, xv, y, z, red_m, red_e);
    if (MODE == MODE_REDUCE) block_reduce_write(red_m, red_e, a.partials + 2 * (size_t)a.partial_base);
}

// ---------------------------------------------------------------------------
// Staged variant.  Persistent CTAs walk "row groups" (R consecutive interior
// rows of one z-plane).  For each group one thread issues 19 cp.async.bulk
// copies -- the R source rows of every population, which are contiguous in
// the SoA layout -- into one stage of a shared-memory ring, completing on
// that stage's mbarrier.  The ring keeps `stages` groups in flight while the
// CTA's threads update the current group from shared memory (the +-x shifted
// values are neighbouring shared-memory elements) and store the results with
// vector stores.  Every mbarrier wait is bounded: on expiry the kernel sets
// bit 1 of the status word, stops issuing copies, drains what it issued
// (again bounded) and returns.
// ---------------------------------------------------------------------------
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// one arrival (release semantics at CTA scope: this thread's earlier shared
// memory accesses are visible to the threads that wait for the phase)
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t k = 0; k < limit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Pull one population for V sites from a shared-memory row (values at x - EX).
template <class S, int V, int EX>
__device__ __forceinline__ void gather_smem(const S *row, int x0, int dim, S (&out)[V])
{
    static_assert((V * sizeof(S)) % 8 == 0, "8-byte multiples");
    S v[V];
    if constexpr (V * sizeof(S) == 8) {
        const uint2 r = *reinterpret_cast<const uint2 *>(row + x0);
        memcpy(v, &r, 8);
    } else {
#pragma unroll
        for (int c = 0; c < (int)(V * sizeof(S) / 16); ++c) {
            const uint4 r = *reinterpret_cast<const uint4 *>(reinterpret_cast<const char *>(row + x0) + 16 * c);
            memcpy(reinterpret_cast<char *>(v) + 16 * c, &r, 16);
        }
    }
    if constexpr (EX == 0) {
#pragma unroll
        for (int k = 0; k < V; ++k) out[k] = v[k];
    } else if constexpr (EX == 1) {
        out[0] = (x0 > 0) ? row[x0 - 1] : zero_elem<S>();
#pragma unroll
        for (int k = 1; k < V; ++k) out[k] = v[k - 1];
    } else {
#pragma unroll
        for (int k = 0; k < V - 1; ++k) out[k] = v[k + 1];
        out[V - 1] = (x0 + V < dim) ? row[x0 + V] : zero_elem<S>();
    }
}

template <class S, int V, int I>
__device__ __forceinline__ void gather_all_smem(const S *stage, int rowlen, int r, int dim, int x0, S (&fs)[Q][V])
{
    gather_smem<S, V, ex_of(I)>(stage + (size_t)I * rowlen + (size_t)r * dim, x0, dim, fs[I]);
    if constexpr (I + 1 < Q) gather_all_smem<S, V, I + 1>(stage, rowlen, r, dim, x0, fs);
}

template <class S, int V>
__device__ __forceinline__ void store_global(S *p, const S (&in)[V])
{
    if constexpr (V * sizeof(S) == 8) {
        uint2 r;
        memcpy(&r, in, 8);
        *reinterpret_cast<uint2 *>(p) = r;
    } else {
#pragma unroll
        for (int c = 0; c < (int)(V * sizeof(S) / 16); ++c) {
            uint4 r;
            memcpy(&r, reinterpret_cast<const char *>(in) + 16 * c, 16);
            *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(p) + 16 * c) = r;
        }
    }
}

// group g -> plane z, first row y0, rows in this group
__device__ __forceinline__ void decode_group(const StepArgs &a, unsigned g, int &z, int &y0, int &reff)
{
    z = 1 + (int)(g / (unsigned)a.gpp);
    y0 = 1 + (int)(g % (unsigned)a.gpp) * a.rows;
    reff = min(a.rows, a.dim - 1 - y0);
}

template <class S>
__device__ __forceinline__ void issue_group(const StepArgs &a, S *stage, uint64_t *bar, unsigned g)
{
    int z, y0, reff;
    decode_group(a, g, z, y0, reff);
    const int dim = a.dim;
    const uint32_t bytes = (uint32_t)reff * (uint32_t)dim * (uint32_t)sizeof(S);
    const size_t rowlen = (size_t)a.rows * dim;
    mbar_expect_tx(bar, (uint32_t)Q * bytes);
    const S *fin = static_cast<const S *>(a.fin);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const S *src = fin + (size_t)i * a.n + (size_t)(z - ez_of(i)) * dim * dim + (size_t)(y0 - ey_of(i)) * dim;
        bulk_copy_g2s(stage + (size_t)i * rowlen, src, bytes, bar);
    }
}

template <class S, int MODE>
__global__ void __launch_bounds__(256) pull_staged_kernel(StepArgs a)
{
    constexpr int V = 4;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem_raw);
    S *ring = reinterpret_cast<S *>(smem_raw + 128);
    const int dim = a.dim;
    const int ns = a.stages;
    const int rowlen = a.rows * dim;
    const size_t stage_elems = (size_t)Q * rowlen;
    const unsigned G = a.ngroups;
    const int nvx = dim / V;

    if (threadIdx.x == 0) {
        for (int s = 0; s < ns; ++s) mbar_init(&bars[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    unsigned issued = 0;  // groups issued by thread 0 (only thread 0 tracks it)
    if (threadIdx.x == 0) {
        for (int s = 0; s < ns; ++s) {
            const unsigned g = blockIdx.x + (unsigned)s * gridDim.x;
            if (g < G) {
                issue_group<S>(a, ring + (size_t)s * stage_elems, &bars[s], g);
                ++issued;
            }
        }
    }

    bool err = false;
    unsigned k = 0, fail_k = 0xffffffffu;
    double red_m = 0.0, red_e = 0.0;
    S *__restrict__ fout = static_cast<S *>(a.fout);
    for (;; ++k) {
        const unsigned g = blockIdx.x + k * gridDim.x;
        if (g >= G) break;
        const int s = (int)(k % (unsigned)ns);
        const uint32_t parity = (k / (unsigned)ns) & 1u;
        if (!err) {
            err = !mbar_wait_bounded(&bars[s], parity, kWaitLimit);
            if (err) fail_k = k;
        }
        if (!err) {
            int z, y0, reff;
            decode_group(a, g, z, y0, reff);
            const S *stage = ring + (size_t)s * stage_elems;
            for (int v = threadIdx.x; v < reff * nvx; v += blockDim.x) {
                const int r = v / nvx;
                const int x0 = (v - r * nvx) * V;
                const int y = y0 + r;
                const size_t site0 = (size_t)z * dim * dim + (size_t)y * dim + x0;
                const typename MapWord<V>::type mw =
                    __ldg(reinterpret_cast<const typename MapWord<V>::type *>(a.map + site0));
                S fs[Q][V];
                gather_all_smem<S, V, 0>(stage, rowlen, r, dim, x0, fs);
                update_vector<S, MODE, V>(fs, mw, a, y, z, x0, site0, red_m, red_e);
#pragma unroll
                for (int i = 0; i < Q; ++i) store_global<S, V>(fout + (size_t)i * a.n + site0, fs[i]);
            }
        }
        __syncthreads();  // stage s fully read before it is refilled
        if (threadIdx.x == 0 && !err) {
            const unsigned gn = g + (unsigned)ns * gridDim.x;
            if (gn < G) {
                issue_group<S>(a, ring + (size_t)s * stage_elems, &bars[s], gn);
                ++issued;
            }
        }
    }
    if (err) {
        atomicOr(a.status, 2);
        // drain the copies this CTA issued and never consumed (bounded)
        if (threadIdx.x == 0) {
            for (unsigned j = fail_k; j < issued; ++j)
                mbar_wait_bounded(&bars[j % (unsigned)ns], (j / (unsigned)ns) & 1u, kWaitLimit);
        }
    }
}

// ---------------------------------------------------------------------------
// Initial state.  Writes P_{-1} such that S(P_{-1}) is the reference's initial
// buffer R_0 (kernels.cl:303-317 plus the optional noise): the slot of site s
// feeding direction i holds R_0(s + e_i)[i].  Also writes the byte map and the
// initial rho / u (kernels.cl:290-300).
// ---------------------------------------------------------------------------

template <class C>
__device__ __forceinline__ C lid_at(const InitArgs &a, int x, int y)
{
    return static_cast<const C *>(a.lid)[(size_t)y * a.dim + x];
}

// The population slots a site's initial state writes (all but those that
// noise_kernel owns): P_{-1} slots pulled into the site (or, in A-form, its
// own R_0 slots).
template <class S>
__device__ __forceinline__ void init_site_pops(const InitArgs &a, int x, int y, int z, size_t id, uint8_t b)
{
    using C = typename Compute<S>::type;
    const int dim = a.dim;
    const C qn = nan_of<C>();
    S *f = static_cast<S *>(a.f);
    const Weights<C> W = make_weights<C>();
    const bool noisy = a.noise_sigma != 0.0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        C val = qn;  // walls hold NaN (kernels.cl:312, 316)
        if (a.in_place) {
            // A-form: the site's own R_0 slots, its initial equilibrium
            if (noisy && b == 0) continue;
            if (!(b & M_WALL)) {
                const C lv = (b & M_FRONT) ? lid_at<C>(a, x, y) : (C)0;
                if constexpr (is_dev16<S>()) {
                    float d = 0.0f;
                    if (b & M_FRONT) {
                        const float eu = ex_of(i) > 0 ? (float)lv : (ex_of(i) < 0 ? -(float)lv : 0.0f);
                        d = deq_scaled(i, 0.0f, 1.0f, eu, 1.5f * (float)lv * (float)lv, 1.0f);
                    }
                    val = d * Dev16<S>::scale;
                } else {
                    val = (b & M_FRONT) ? init_eq_exact<C>(i, lv, W) : W.w[wclass_of(i)];
                }
            }
        } else if (!(b & M_WALL)) {
            const int tx = x + ex_of(i), ty = y + ey_of(i), tz = z + ez_of(i);
            const uint8_t tb = pack_cell(dim, tx, ty, tz);
            if (noisy && tb == 0) continue;
            if (!(tb & M_WALL)) {
                const C lv = (tb & M_FRONT) ? lid_at<C>(a, tx, ty) : (C)0;
                if constexpr (is_dev16<S>()) {
                    // deviation of the equilibrium at rho = 1
                    float d = 0.0f;
                    if (tb & M_FRONT) {
                        const float eu = ex_of(i) > 0 ? (float)lv : (ex_of(i) < 0 ? -(float)lv : 0.0f);
                        d = deq_scaled(i, 0.0f, 1.0f, eu, 1.5f * (float)lv * (float)lv, 1.0f);
                    }
                    val = d * Dev16<S>::scale;
                } else {
                    val = (tb & M_FRONT) ? init_eq_exact<C>(i, lv, W) : W.w[wclass_of(i)];
                }
            }
        }
        if constexpr (is_dev16<S>()) {
            f[(size_t)i * a.n + id] = Dev16<S>::from_f((float)val);
        } else {
            f[(size_t)i * a.n + id] = (S)val;
        }
    }
}

// Four values of type T at p (4-element aligned) with one or two vector
// stores.
template <class T> __device__ __forceinline__ void store4(T *p, const T (&v)[4])
{
    if constexpr (sizeof(T) == 8) {
        reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
    } else if constexpr (sizeof(T) == 4) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
        uint2 r;
        memcpy(&r, v, 8);
        *reinterpret_cast<uint2 *>(p) = r;
    }
}

// Grid: blockIdx.y = z-plane, x-blocks over the plane's dim^2 / 4 groups of
// four consecutive x-sites (dim % 4 == 0; 32-bit index arithmetic inside a
// plane).  Each thread writes its four sites' map bytes, rho and u with one
// vector store per field; the population slots of sites whose neighbours
// are all FLUID take a branch-free path (nothing with noise, the rest state
// without), the others init_site_pops.
template <class S>
__global__ void init_kernel(InitArgs a)
{
    using C = typename Compute<S>::type;
    const int dim = a.dim;
    const unsigned nq = (unsigned)dim / 4u;
    const unsigned pi = blockIdx.x * blockDim.x + threadIdx.x;
    if (pi >= nq * (unsigned)dim) return;
    const int y = (int)(pi / nq), x0 = 4 * (int)(pi - (unsigned)y * nq), z = (int)blockIdx.y;
    const size_t id0 = (size_t)z * dim * dim + (size_t)y * dim + (size_t)x0;
    uint8_t b[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) b[k] = pack_cell(dim, x0 + k, y, z);
    uint32_t mw;
    memcpy(&mw, b, 4);
    *reinterpret_cast<uint32_t *>(a.map + id0) = mw;
    const C qn = nan_of<C>();
    C r[4], ux[4], u0[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const bool store = (b[k] == 0) || (b[k] == M_FRONT);
        r[k] = store ? (C)1 : qn;
        ux[k] = store ? ((b[k] & M_FRONT) ? lid_at<C>(a, x0 + k, y) : (C)0) : qn;
        u0[k] = store ? (C)0 : qn;
    }
    C *u = static_cast<C *>(a.u);
    store4<C>(static_cast<C *>(a.rho) + id0, r);
    store4<C>(u + id0, ux);
    store4<C>(u + a.n + id0, u0);
    store4<C>(u + 2 * a.n + id0, u0);

    // With noise, noise_kernel writes every slot whose value belongs to a
    // FLUID site (the slots streaming into it, or its own in A-form); this
    // kernel writes the others.
    const bool noisy = a.noise_sigma != 0.0;
    const bool bulk = y >= 3 && z >= 3 && y <= dim - 4 && z <= dim - 4;
    if (bulk && x0 >= 3 && x0 + 3 <= dim - 4) {
        // every site and all its neighbours are FLUID: the rest state
        if (!noisy) {
            S *f = static_cast<S *>(a.f);
            const Weights<C> W = make_weights<C>();
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                S v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if constexpr (is_dev16<S>()) v[k] = Dev16<S>::from_f(0.0f);
                    else v[k] = (S)W.w[wclass_of(i)];
                }
                store4<S>(f + (size_t)i * a.n + id0, v);
            }
        }
        return;
    }
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int x = x0 + k;
        if (bulk && x >= 3 && x <= dim - 4) {
            if (!noisy) {
                S *f = static_cast<S *>(a.f);
                const Weights<C> W = make_weights<C>();
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    if constexpr (is_dev16<S>()) f[(size_t)i * a.n + id0 + k] = Dev16<S>::from_f(0.0f);
                    else f[(size_t)i * a.n + id0 + k] = (S)W.w[wclass_of(i)];
                }
            }
            continue;
        }
        init_site_pops<S>(a, x, y, z, id0 + k, b[k]);
    }
}


// Seeded N(0, sigma^2) noise on the initial populations of the FLUID sites
// (x, y, z in [2, dim-3]), run after init_kernel: the thread of FLUID site t
// draws its five sample blocks (populations 4g .. 4g+3 <- block g) and writes the
// 19 slots (t - e_q, q) of P_{-1} that stream into t (in place: t's own
// slots (t, q)), each slot having this one writer: the equilibrium at rest
// (w_q; deviation 0) plus sigma z.  sigma z is one single-precision product
// (sigma rounded to float) for FP32 and 16-bit storage, a double product for
// FP64 storage: GB300's FP64 pipe would otherwise bound this kernel.
template <class S>
__global__ void noise_kernel(InitArgs a)
{
    using C = typename Compute<S>::type;
    const int dim = a.dim;
    const unsigned m = (unsigned)(dim - 4);
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;  // grid: blockIdx.y = z - 2
    if (k >= m * m) return;
    const size_t x = 2 + k % m, y = 2 + k / m, z = 2 + (size_t)blockIdx.y;
    const size_t t = x + y * (size_t)dim + z * (size_t)dim * dim;
    S *f = static_cast<S *>(a.f);
    const Weights<C> W = make_weights<C>();
#pragma unroll
    for (int g = 0; g < (Q + 3) / 4; ++g) {
        float zb[4];
        gauss_block(a.seed, t, (uint32_t)g, zb);
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const int q = 4 * g + h;
            if (q >= Q) break;
            const float zq = zb[h];
            const ptrdiff_t sh = a.in_place ? 0
                               : (ptrdiff_t)ex_of(q) + (ptrdiff_t)ey_of(q) * dim + (ptrdiff_t)ez_of(q) * dim * dim;
            S *dst = f + (size_t)q * a.n + (size_t)((ptrdiff_t)t - sh);
            if constexpr (is_dev16<S>()) {
                *dst = Dev16<S>::from_f(__fmul_rn(__fmul_rn(a.noise_sigma_f, zq), Dev16<S>::scale));
            } else if constexpr (sizeof(C) == 4) {
                *dst = (S)__fadd_rn(W.w[wclass_of(q)], __fmul_rn(a.noise_sigma_f, zq));
            } else {
                *dst = (S)X<C>::add(W.w[wclass_of(q)], (C)__dmul_rn(a.noise_sigma, (double)zq));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Dump / load of the reference's post-stream buffer R_t in CSoA order.
// Output element o <-> (site id, q): o = (((id >> sd) * 19 + q) << sd) + (id & (2^sd - 1))
// (kernels.cl:64).  Chunked by output index so any stride works.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void decode_csoa(size_t o, int sd, size_t n, size_t &id, int &q)
{
    if (sd < 0) {  // pure SoA of a non-power-of-two lattice: o = q * n + id
        q = (int)(o / n);
        id = o - (size_t)q * n;
        return;
    }
    const size_t smask = ((size_t)1 << sd) - 1;
    const size_t lane = o & smask;
    const size_t t = o >> sd;
    q = (int)(t % Q);
    id = ((t / Q) << sd) | lane;
}

// the value of population q held in slot (at, qs)
template <class S, class C>
__device__ __forceinline__ C stored_value(const S *f, size_t n, int qs, size_t at, int q)
{
    const S v = f[(size_t)qs * n + at];
    if constexpr (is_dev16<S>()) {
        return (C)(wf_of(q) + Dev16<S>::to_f(v) * Dev16<S>::inv_scale);
    } else {
        return (C)v;
    }
}


template <class S, class T>
__global__ void dump_f_kernel(DumpArgs a)
{
    using C = typename Compute<S>::type;
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.count) return;
    size_t id;
    int q;
    decode_csoa(a.o0 + k, a.sd, a.n, id, q);
    const int dim = a.dim;
    const int x = (int)(id % dim), y = (int)((id / dim) % dim), z = (int)(id / ((size_t)dim * dim));
    const uint8_t b = a.map[id];
    const int sx = x - ex_of(q), sy = y - ey_of(q), sz = z - ez_of(q);
    const bool in = sx >= 0 && sy >= 0 && sz >= 0 && sx < dim && sy < dim && sz < dim;
    const size_t src = in ? (size_t)sx + (size_t)sy * dim + (size_t)sz * dim * dim : 0;
    const bool src_wall = !in || (a.map[src] & M_WALL);
    const S *f = static_cast<const S *>(a.f);
    // where R(id, q) lives: P(src, q) (two-lattice), f(id, q) (AA A-form),
    // f(src, opp q) (AA B-form)
    const int qs = a.layout == LAYOUT_AA_B ? opp_of(q) : q;
    const size_t at = a.layout == LAYOUT_AA_A ? id : src;
    T val;
    if (b & M_WALL) {
        val = src_wall ? (T)nan_of<C>() : (T)stored_value<S, C>(f, a.n, qs, at, q);
    } else if (src_wall) {
        const Weights<C> W = make_weights<C>();
        C lv = (b & M_FRONT) ? static_cast<const C *>(a.lid)[(size_t)y * dim + x] : (C)0;
        val = (T)((b & M_FRONT) ? init_eq_exact<C>(q, lv, W) : W.w[wclass_of(q)]);
    } else {
        val = (T)stored_value<S, C>(f, a.n, qs, at, q);
    }
    static_cast<T *>(a.buf)[k] = val;
}

template <class S, class T>
__global__ void load_f_kernel(DumpArgs a)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.count) return;
    size_t id;
    int q;
    decode_csoa(a.o0 + k, a.sd, a.n, id, q);
    const int dim = a.dim;
    const int x = (int)(id % dim), y = (int)((id / dim) % dim), z = (int)(id / ((size_t)dim * dim));
    const int sx = x - ex_of(q), sy = y - ey_of(q), sz = z - ez_of(q);
    if (sx < 0 || sy < 0 || sz < 0 || sx >= dim || sy >= dim || sz >= dim) return;
    const size_t src = (size_t)sx + (size_t)sy * dim + (size_t)sz * dim * dim;
    if (a.map[src] & M_WALL) return;
    const T v = static_cast<const T *>(a.buf)[k];
    S *f = static_cast<S *>(a.f);
    const size_t slot = (size_t)(a.layout == LAYOUT_AA_B ? opp_of(q) : q) * a.n + (a.layout == LAYOUT_AA_A ? id : src);
    if constexpr (is_dev16<S>()) {
        f[slot] = Dev16<S>::from_f(((float)v - wf_of(q)) * Dev16<S>::scale);
    } else {
        f[slot] = (S)v;
    }
}

}  // namespace lbm
