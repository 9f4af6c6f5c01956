// lbm_adjoint.cuh -- hand-written adjoint of the D3Q19 BGK cavity iteration.
//
// Written in the reference's post-stream form.  With R_k the buffer iteration
// k+1 reads (kernels.cl:339-341) and C the local collision with its boundary
// rules (kernels.cl:343-418),
//     R_{k+1} = S C(R_k),   S: slot (s, i) <- site s - e_i, slot i.
// For a loss J(R_T), the adjoint a_k = dJ/dR_k obeys
//     a_k(s, .) = J_C(R_k(s))^T b(s),   b_i(s) = a_{k+1}(s + e_i, i),
// i.e. "pull from s + e_i (reverse streaming), then apply the transposed
// local Jacobian" -- the same data movement as the forward step with the
// shifts reversed.  Walls never compute and their adjoint stays 0, which makes
// b_i = 0 wherever the forward pushed into a wall.  Slots whose forward source
// is a wall hold constants; their adjoint is never pulled again.
//
// Transposed Jacobians of C at a site with pre-collision g (R_k(s)):
//  FLUID   (BGK, omega = 1/tau): with rho, u of g, p_i = 1 + 3 e.u + 4.5 (e.u)^2
//          - 1.5 u^2, feq_i = w_i rho p_i,
//            B0 = sum_i b_i w_i p_i,
//            G  = sum_i b_i w_i (3 + 9 e_i.u) e_i - 3 u sum_i b_i w_i,
//            a_j = (1 - omega) b_j + omega (B0 - G.u + G.e_j),
//          and dJ/domega += sum_i b_i (feq_i - g_i).
//  MOVING  (lid, kernels.cl:343-349, 393-398): out_i = w_i rho p_i(lid) with
//          rho over g after the -z replacements, so
//            a_j = m_j sum_i b_i w_i p_i,  m_j = 0 for j in {5,11,12,13,14},
//            2 for j in {6,15,16,17,18}, 1 otherwise,
//          and dJ/dlid(x,y) += sum_i b_i w_i rho (3 e_ix + (9 e_ix^2 - 3) lid).
//  bounce-back: a_j = b_opp(j);  CORNER: a_j = b_j;  WALL: a = 0.
#pragma once

#include <cuda.h>

#include "lbm_kernels.cuh"

namespace lbm {

struct AdjArgs {
    const void *fwd;     // forward state Q_k (the P buffer iteration k+1 reads from)
    const void *ain;     // a_{k+1}, adjoint type, post-stream layout [q][z][y][x]
    void *aout;          // a_k
    const uint8_t *map;
    const void *lid;     // forward macro type, dim*dim
    double *grad_lid;    // dim*dim, += per column (MOVING sites)
    double *tau_acc;     // per block: += dJ/domega of this launch's sites
    const void *target;  // loss: u_x target on the plane, adjoint type, [x + z*dim]
    double *loss_part;   // loss: per block partial sums
    int dim;
    int nvx;
    unsigned nvec;
    size_t n;
    double omega;        // 1/tau in the forward's precision
    double dloss;        // loss-gradient seed scale (dJ/dL * 2 / M)
    int plane_y;         // loss plane
    unsigned tau_base;   // first tau_acc slot of this launch
};

template <class S> struct AdjType { using type = float; };
template <> struct AdjType<double> { using type = double; };

// forward storage element -> value in the adjoint precision
template <class S, class A> __device__ __forceinline__ A fwd_value(S v, int i)
{
    if constexpr (is_dev16<S>()) return (A)(wf_of(i) + Dev16<S>::to_f(v) * Dev16<S>::inv_scale);
    else return (A)v;
}

template <class A>
__device__ __forceinline__ void moments_plain(const A (&g)[Q], A &rho, A &ux, A &uy, A &uz)
{
    rho = 0;
    A jx = 0, jy = 0, jz = 0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        rho += g[i];
        if (ex_of(i)) jx += ex_of(i) > 0 ? g[i] : -g[i];
        if (ey_of(i)) jy += ey_of(i) > 0 ? g[i] : -g[i];
        if (ez_of(i)) jz += ez_of(i) > 0 ? g[i] : -g[i];
    }
    const A inv = (A)1 / rho;
    ux = jx * inv;
    uy = jy * inv;
    uz = jz * inv;
}

template <class A> __device__ __forceinline__ A w_of(int i)
{
    return wclass_of(i) == 0 ? (A)1 / (A)3 : (wclass_of(i) == 1 ? (A)1 / (A)18 : (A)1 / (A)36);
}

// MOVING site with density rho (of g after the -z replacements).
template <class A>
__device__ __forceinline__ void adjoint_moving_rho(A (&b)[Q], A rho, A lid, A &dlid)
{
    const A c15 = (A)1.5 * lid * lid;
    A s = 0, dl = 0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const A ex = (A)ex_of(i);
        const A eu = ex * lid;
        const A w = w_of<A>(i);
        s += b[i] * w * ((A)1 + (A)3 * eu + (A)4.5 * eu * eu - c15);
        dl += b[i] * w * rho * ((A)3 * ex + ((A)9 * ex * ex - (A)3) * lid);
    }
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        const bool zero = (j == 5 || j == 11 || j == 12 || j == 13 || j == 14);
        const bool twice = (j == 6 || j == 15 || j == 16 || j == 17 || j == 18);
        b[j] = zero ? (A)0 : (twice ? (A)2 * s : s);
    }
    dlid += dl;
}

// MOVING site.
template <class A>
__device__ __forceinline__ void adjoint_moving(const A (&g)[Q], A (&b)[Q], A lid, A &dlid)
{
    A rho = 0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const bool replaced = (i == 5 || i == 11 || i == 12 || i == 13 || i == 14);
        rho += replaced ? g[opp_of(i)] : g[i];
    }
    adjoint_moving_rho<A>(b, rho, lid, dlid);
}

// FLUID adjoint written around opposite pairs (i, i') with e_i.u = +-a:
//   p_(+-) = base +- 3a, base = 1 + 4.5 a^2 - 1.5 u^2
//   B0 = sum_c w_c sum_pairs (s base + 3 a d),   s = b+ + b-, d = b+ - b-
//   G  = sum_c w_c sum_pairs e_i (3 d + 9 a s) - 3 u SB,  SB = sum_c w_c sum s
//   a_(+-) = (1 - omega) b_(+-) + omega (B0 - G.u) +- omega G.e_i
//   dJ/domega += rho B0 - sum_i b_i g_i
// e_i . u as a signed sum of the non-zero terms (chosen at compile time: no
// multiplications by the 0 / +-1 components)
template <class A> __device__ __forceinline__ A proj_sum(int i, A ux, A uy, A uz)
{
    A s = 0;
    bool first = true;
    if (ex_of(i)) { s = ex_of(i) > 0 ? ux : -ux; first = false; }
    if (ey_of(i)) { s = first ? (ey_of(i) > 0 ? uy : -uy) : (ey_of(i) > 0 ? s + uy : s - uy); first = false; }
    if (ez_of(i)) s = first ? (ez_of(i) > 0 ? uz : -uz) : (ez_of(i) > 0 ? s + uz : s - uz);
    return s;
}

template <class A>
__device__ __forceinline__ A adjoint_fluid_core(A (&b)[Q], A ux, A uy, A uz, A omega)
{
    const A c0 = (A)1 - (A)1.5 * (ux * ux + uy * uy + uz * uz);
    // per weight class accumulators: rest (0), axis (1), edge (2)
    A B[3] = {b[0] * c0, 0, 0}, SB[3] = {b[0], 0, 0};
    A Gx[3] = {0, 0, 0}, Gy[3] = {0, 0, 0}, Gz[3] = {0, 0, 0};
    // (i, i') pairs with e_i listed first
    constexpr int P[9][2] = {{1, 3}, {2, 4}, {6, 5}, {7, 9}, {8, 10}, {11, 17}, {12, 18}, {15, 13}, {16, 14}};
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int i = P[k][0], j = P[k][1];
        const int c = wclass_of(i);
        const A aa = proj_sum<A>(i, ux, uy, uz);
        const A sm = b[i] + b[j], df = b[i] - b[j];
        B[c] += sm * (c0 + (A)4.5 * aa * aa) + (A)3 * aa * df;
        SB[c] += sm;
        const A q = (A)3 * df + (A)9 * aa * sm;
        if (ex_of(i)) Gx[c] += ex_of(i) > 0 ? q : -q;
        if (ey_of(i)) Gy[c] += ey_of(i) > 0 ? q : -q;
        if (ez_of(i)) Gz[c] += ez_of(i) > 0 ? q : -q;
    }
    // class weights: rest, axis (population 1), edge (population 7)
    const A w0 = w_of<A>(0), w1 = w_of<A>(1), w2 = w_of<A>(7);
    const A B0 = w0 * B[0] + w1 * B[1] + w2 * B[2];
    const A sb = w0 * SB[0] + w1 * SB[1] + w2 * SB[2];
    const A gx = w1 * Gx[1] + w2 * Gx[2] - (A)3 * ux * sb;
    const A gy = w1 * Gy[1] + w2 * Gy[2] - (A)3 * uy * sb;
    const A gz = w1 * Gz[1] + w2 * Gz[2] - (A)3 * uz * sb;
    const A keep = (A)1 - omega;
    const A oc = omega * (B0 - (gx * ux + gy * uy + gz * uz));
    b[0] = keep * b[0] + oc;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int i = P[k][0], j = P[k][1];
        A ge = 0;
        if (ex_of(i)) ge += ex_of(i) > 0 ? gx : -gx;
        if (ey_of(i)) ge += ey_of(i) > 0 ? gy : -gy;
        if (ez_of(i)) ge += ez_of(i) > 0 ? gz : -gz;
        const A t = omega * ge;
        b[i] = keep * b[i] + (oc + t);
        b[j] = keep * b[j] + (oc - t);
    }
    return B0;
}

// A FLUID site's pre-collision populations g (adjoint type) and its moments
// as the forward's collision formed them from the stored values v: the
// deviation-form sums for 16-bit storage (moments_dev), the reference's
// summation order for FP32 / FP64 (moments_exact).
template <class S, class A>
__device__ __forceinline__ void forward_point(const S (&v)[Q], A (&g)[Q], A &rho, A &ux, A &uy, A &uz)
{
    if constexpr (is_dev16<S>()) {
        float D[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) D[i] = Dev16<S>::to_f(v[i]);
        float drho, r, x, y, z;
        moments_dev(D, Dev16<S>::inv_scale, drho, r, x, y, z);
        rho = (A)r;
        ux = (A)x;
        uy = (A)y;
        uz = (A)z;
#pragma unroll
        for (int i = 0; i < Q; ++i) g[i] = (A)(wf_of(i) + D[i] * Dev16<S>::inv_scale);
    } else {
        using C = typename Compute<S>::type;
        C f[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) f[i] = (C)v[i];
        C r, x, y, z;
        moments_exact(f, r, x, y, z);
        rho = (A)r;
        ux = (A)x;
        uy = (A)y;
        uz = (A)z;
#pragma unroll
        for (int i = 0; i < Q; ++i) g[i] = (A)f[i];
    }
}

// FLUID site at the forward's point: the core, and dw += dJ/domega term
// rho B0 - sum_i b_i g_i (b before the update).
template <class A>
__device__ __forceinline__ void adjoint_fluid_point(const A (&g)[Q], A (&b)[Q], A rho, A ux, A uy, A uz, A omega,
                                                    A &dw)
{
    A bg = 0;
#pragma unroll
    for (int i = 0; i < Q; ++i) bg += b[i] * g[i];
    const A B0 = adjoint_fluid_core<A>(b, ux, uy, uz, omega);
    dw += rho * B0 - bg;
}

// Any site kind from the forward's stored linearisation point (MODE_STEP_ADJ
// planes m0, m1, m2: u of a FLUID site, rho of a MOVING site): the adjoint
// without the tau term, which needs the full populations.
template <class A>
__device__ __forceinline__ void adjoint_site_macro(A (&b)[Q], uint8_t b8, A m0, A m1, A m2, A lidv, A omega,
                                                   A &dlid)
{
    if (b8 == 0) {
        adjoint_fluid_core<A>(b, m0, m1, m2, omega);
        return;
    }
    if (b8 & M_WALL) {
#pragma unroll
        for (int i = 0; i < Q; ++i) b[i] = (A)0;
        return;
    }
    if (b8 == M_FRONT) {
        adjoint_moving_rho<A>(b, m0, lidv, dlid);
        return;
    }
    if (!(b8 & M_CORNER)) {
        A t[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) t[i] = b[opp_of(i)];
#pragma unroll
        for (int i = 0; i < Q; ++i) b[i] = t[i];
    }
}

// Any site kind (face rows), map-driven, from the stored forward values v of
// its pulled populations: FLUID at the forward's point; otherwise g gets the
// wall-sourced constants.
template <class S, class A, class C>
__device__ __forceinline__ void adjoint_general(const S (&v)[Q], A (&b)[Q], uint8_t b8, C lidv, A omega,
                                                const Weights<C> &W, A &dw, A &dlid)
{
    if (b8 & M_WALL) {
#pragma unroll
        for (int i = 0; i < Q; ++i) b[i] = (A)0;
        return;
    }
    if (b8 == 0) {
        A g[Q], rho, ux, uy, uz;
        forward_point<S, A>(v, g, rho, ux, uy, uz);
        adjoint_fluid_point<A>(g, b, rho, ux, uy, uz, omega, dw);
        return;
    }
    if (b8 == M_FRONT) {
        A g[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i)
            g[i] = wall_sourced(i, b8) ? (A)init_eq_exact<C>(i, lidv, W) : fwd_value<S, A>(v[i], i);
        adjoint_moving<A>(g, b, (A)lidv, dlid);
    } else if (!(b8 & M_CORNER)) {
        A t[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) t[i] = b[opp_of(i)];
#pragma unroll
        for (int i = 0; i < Q; ++i) b[i] = t[i];
    }
}

// Adjoint of the x-face site xf of an interior row (bounce-back): a_j =
// b_opp(j) = a_{k+1}(s - e_j, opp(j)), reloaded from the input adjoint.
template <class A, int V>
__device__ __forceinline__ void adjoint_face_fix(const AdjArgs &a, size_t rowoff, int xf, int k, A (&bs)[Q][V])
{
    const A *ain = static_cast<const A *>(a.ain);
    const int dim = a.dim;
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        const int o = opp_of(j);
        const ptrdiff_t shift = (ptrdiff_t)ez_of(j) * dim * dim + (ptrdiff_t)ey_of(j) * dim;
        bs[j][k] = load_one(ain + (size_t)o * a.n + rowoff - shift + (xf - ex_of(j)));
    }
}

// One adjoint step a_{k+1} -> a_k over the rows of one kind (ROWS_INTERIOR:
// y, z in [2, dim-3], branch-free FLUID adjoint then the row ends patched;
// ROWS_FACES: the general path).  V = VB / sizeof(A) sites per thread.
// register cap of the adjoint kernels: 128 (two 256-thread blocks per SM)
// for the FP32 adjoint, uncapped for FP64
#ifndef LBM_ADJ_MINB
#define LBM_ADJ_MINB 2
#endif

// MACRO = false: a.fwd is the forward state Q_k (its pull gives the
// pre-collision populations); MACRO = true: a.fwd holds the three planes the
// MODE_STEP_ADJ iteration from Q_k stored (compute type), and no tau term is
// formed.
template <class S, class A, int VB, int ROWS, bool MACRO>
__global__ void __launch_bounds__(256, sizeof(A) == 8 ? 1 : LBM_ADJ_MINB) adjoint_kernel(AdjArgs a)
{
    using C = typename Compute<S>::type;
    constexpr int V = VB / (int)sizeof(A);
    const int dim = a.dim;
    const int nvx = dim / V;
    const unsigned nrows = ROWS == ROWS_INTERIOR ? (unsigned)(dim - 4) * (unsigned)(dim - 4) : 4u * (unsigned)(dim - 3);
    const unsigned g0 = blockIdx.x * blockDim.x + threadIdx.x;
    A dw = 0;
    if (g0 < nrows * (unsigned)nvx) {
        const unsigned row = g0 / (unsigned)nvx;
        const int xv = (int)(g0 - row * (unsigned)nvx);
        int y, z;
        if (ROWS == ROWS_INTERIOR) {
            y = 2 + (int)(row % (unsigned)(dim - 4));
            z = 2 + (int)(row / (unsigned)(dim - 4));
        } else {
            decode_face_row(dim, row, y, z);
        }
        const int x0 = xv * V;
        const size_t rowoff = (size_t)z * dim * dim + (size_t)y * dim;
        const size_t site0 = rowoff + (size_t)x0;

        // reverse streaming: slot i of site s takes a_{k+1}(s + e_i, i)
        const A *ain = static_cast<const A *>(a.ain);
        A bs[Q][V];
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const ptrdiff_t shift = (ptrdiff_t)ez_of(i) * dim * dim + (ptrdiff_t)ey_of(i) * dim;
            const A *src = ain + (size_t)i * a.n + rowoff + shift;
            if (ex_of(i) == 1) gather_row<A, V, -1>(src, x0, dim, bs[i]);
            else if (ex_of(i) == -1) gather_row<A, V, 1>(src, x0, dim, bs[i]);
            else gather_row<A, V, 0>(src, x0, dim, bs[i]);
        }
        const A omega = (A)a.omega;
        // forward values: the pulled populations R_k(s), or the stored
        // linearisation point (three planes, same element type as A)
        S fsv[MACRO ? 1 : Q][MACRO ? 1 : V];
        C mv[MACRO ? 3 : 1][MACRO ? V : 1];
        if constexpr (MACRO) {
            const C *m = static_cast<const C *>(a.fwd);
#pragma unroll
            for (int c = 0; c < 3; ++c) load_vec<C, V>(m + (size_t)c * a.n + site0, mv[c]);
        } else {
            const S *fwd = static_cast<const S *>(a.fwd);
            gather_all<S, V, 0>(fwd, a.n, rowoff, dim, x0, fsv);
        }

        if (ROWS == ROWS_INTERIOR) {
#pragma unroll
            for (int k = 0; k < V; ++k) {
                A b[Q];
#pragma unroll
                for (int i = 0; i < Q; ++i) b[i] = bs[i][k];
                if constexpr (MACRO) {
                    adjoint_fluid_core<A>(b, (A)mv[0][k], (A)mv[1][k], (A)mv[2][k], omega);
                } else {
                    S v[Q];
#pragma unroll
                    for (int i = 0; i < Q; ++i) v[i] = fsv[i][k];
                    A g[Q], rho, ux, uy, uz;
                    forward_point<S, A>(v, g, rho, ux, uy, uz);
                    A d = 0;
                    adjoint_fluid_point<A>(g, b, rho, ux, uy, uz, omega, d);
                    // x in [2, dim-3] is FLUID; the row ends are patched below
                    if ((unsigned)(x0 + k - 2) <= (unsigned)(dim - 5)) dw += d;
                }
#pragma unroll
                for (int i = 0; i < Q; ++i) bs[i][k] = b[i];
            }
            if (x0 == 0) {
#pragma unroll
                for (int i = 0; i < Q; ++i) bs[i][0] = (A)0;
                adjoint_face_fix<A, V>(a, rowoff, 1, 1, bs);
            }
            if (x0 + V == dim) {
#pragma unroll
                for (int i = 0; i < Q; ++i) bs[i][V - 1] = (A)0;
                adjoint_face_fix<A, V>(a, rowoff, dim - 2, V - 2, bs);
            }
        } else {
            const typename MapWord<V>::type mw =
                __ldg(reinterpret_cast<const typename MapWord<V>::type *>(a.map + site0));
            const C *lid = static_cast<const C *>(a.lid);
            const Weights<C> W = make_weights<C>();
#pragma unroll
            for (int k = 0; k < V; ++k) {
                const uint8_t b8 = (uint8_t)(mw >> (8 * k));
                A b[Q];
#pragma unroll
                for (int i = 0; i < Q; ++i) b[i] = bs[i][k];
                const C lidv = (b8 & M_FRONT) ? lid[(size_t)y * dim + x0 + k] : (C)0;
                A dl = 0;
                if constexpr (MACRO) {
                    adjoint_site_macro<A>(b, b8, (A)mv[0][k], (A)mv[1][k], (A)mv[2][k], (A)lidv, omega, dl);
                } else {
                    S v[Q];
#pragma unroll
                    for (int i = 0; i < Q; ++i) v[i] = fsv[i][k];
                    adjoint_general<S, A, C>(v, b, b8, lidv, omega, W, dw, dl);
                }
                if (b8 == M_FRONT) a.grad_lid[(size_t)y * dim + x0 + k] += (double)dl;
#pragma unroll
                for (int i = 0; i < Q; ++i) bs[i][k] = b[i];
            }
        }
        A *aout = static_cast<A *>(a.aout);
#pragma unroll
        for (int i = 0; i < Q; ++i) store_vec<A, V>(aout + (size_t)i * a.n + site0, bs[i]);
    }
    if constexpr (!MACRO) block_reduce_add((double)dw, a.tau_acc + a.tau_base);
}

// ---------------------------------------------------------------------------
// Two adjoint steps per launch, a_{k+1} -> a_k -> a_{k-1}, for the FP32
// adjoint (forward storage FP32, FP16 or BF16).
//
// A block owns a tile of ADJ2_TX x ADJ2_TY columns of [1, dim-2]^2 and a chunk
// of z-planes, and marches the chunk in z.  Step A computes a_k, one thread
// per site, on the tile plus a one-site ring in x and y (the ext tile,
// ADJ2_EX x ADJ2_EY = the block), plane by plane, into shared memory; step B,
// one plane behind, computes a_{k-1} on the tile from the shared a_k and
// writes it.  a_k never reaches global memory, so a pair of steps moves
// a_{k+1} in, Q_k and Q_{k-1} in, a_{k-1} out: 2 x 76 + 2 x 19 x sizeof(S)
// bytes per site instead of twice 2 x 76 + 19 x sizeof(S).
//
// Step B at plane q reads population i of a_k at plane q + ez_i, x + ex_i,
// y + ey_i.  Populations 0, 5 and 6 have no x, y offset: the same thread
// computed them, so they stay in registers, a short history per plane.  The
// other 16 live in shared memory for the planes still to be read: with step
// B one plane behind and one barrier per plane, the writer of plane p+1 runs
// alongside the readers of plane p-1, so a population needs 2, 3 or 4 plane
// slots for ez_i = +1, 0, -1 (48 slots, 48 KB); with step B two planes
// behind (ADJ2_LAG) 3, 4 or 5 (64 slots, 64 KB).
// Sums for tau and the lid gradient count a site once: step A's
// contributions only on the block's own tile and planes.
//
// Element offsets are 32-bit (i * n + site < 2^32: 19 dim^3 < 2^32, dim <=
// 609); larger lattices take the one-step kernels.
// ---------------------------------------------------------------------------
constexpr int ADJ2_EX = 32, ADJ2_EY = 8;                    // block = ext tile
constexpr int ADJ2_TX = ADJ2_EX - 2, ADJ2_TY = ADJ2_EY - 2;  // owned tile
// Tile height of the stored-point variant (MACRO): 8 rows; 16 rows (512
// threads, two blocks per SM, a ring of 18% of the sites instead of 30%)
// measured slower
#ifndef LBM_ADJ2M_EY
#define LBM_ADJ2M_EY 8
#endif
template <bool MACRO> __host__ __device__ constexpr int adj2_ey() { return MACRO ? LBM_ADJ2M_EY : ADJ2_EY; }
// Planes step B runs behind step A: 1 = one block barrier per plane between
// them; 2 = an mbarrier whose arrival (after step A of plane p) and wait
// (after step B of plane p - 2) enclose step B's work, so a block's warps
// drift by up to one plane instead of meeting at every barrier; each
// population then needs one more plane slot.  Lag 2 measured slower at
// 256^3 FP16 (stored points 0.647 against 0.622 ms per backward iteration,
// full states 0.907 against 0.715): the barrier stalls go, but three blocks
// per SM instead of four leave the kernel as bound by load latency as
// before (ncu: long-scoreboard 5.4 stalls per issue either way).
#ifndef LBM_ADJ2_LAG
#define LBM_ADJ2_LAG 1
#endif
constexpr int ADJ2_LAG = LBM_ADJ2_LAG;
static_assert(ADJ2_LAG == 1 || ADJ2_LAG == 2, "step B lags step A by one or two planes");
__host__ __device__ constexpr bool adj2_in_regs(int i) { return i == 0 || i == 5 || i == 6; }
__host__ __device__ constexpr int adj2_depth(int i)
{
    return adj2_in_regs(i) ? 0 : (ez_of(i) == 1 ? 1 + ADJ2_LAG : (ez_of(i) == 0 ? 2 + ADJ2_LAG : 3 + ADJ2_LAG));
}
// first plane slot of each population; used through a constexpr local, so
// that every index is an immediate (a call at run time would recurse)
struct Adj2Layout {
    int base[Q + 1];
};
__host__ __device__ constexpr Adj2Layout adj2_layout()
{
    Adj2Layout l{};
    for (int i = 0; i < Q; ++i) l.base[i + 1] = l.base[i] + adj2_depth(i);
    return l;
}
constexpr int ADJ2_SLOTS = adj2_layout().base[Q];
// plane slots, then (lag 2) the mbarrier
template <bool MACRO> __host__ __device__ constexpr size_t adj2_smem_bytes()
{
    return (size_t)ADJ2_SLOTS * ADJ2_EX * adj2_ey<MACRO>() * sizeof(float) + (ADJ2_LAG == 2 ? 16 : 0);
}
static_assert(ADJ2_SLOTS == 32 + 16 * ADJ2_LAG, "plane slots of the two-step adjoint");
// the largest dim whose 19 dim^3 element offsets fit 32 bits
constexpr int ADJ2_MAX_DIM = 609;

struct Adj2Args {
    const void *fwd_a;   // Q_k, forward state of step A
    const void *fwd_b;   // Q_{k-1}, forward state of step B
    const float *ain;    // a_{k+1}
    float *aout;         // a_{k-1}
    const uint8_t *map;
    const void *lid;     // forward macro type, dim*dim
    double *grad_lid;    // dim*dim
    double *tau_acc;     // per block
    int dim;
    int ntx, nty;        // tiles in x and y
    int zc;              // planes per chunk
    float omega;
    // per-population element offsets from a site (mod 2^32): i n + e_i
    // (reverse streaming), i n - e_i (forward pull), i n (own slot); kernel
    // parameters, so the unrolled loops take them as constant operands
    unsigned off_up[Q], off_down[Q], off_own[Q];
    int *status;         // bit 1: a bounded wait expired (the launch's results are invalid)
};

#ifndef LBM_ADJ2_MINB
#define LBM_ADJ2_MINB 3
#endif
// resident blocks per SM of the MACRO variant: with lag 1 (48 KB of slots)
// four (64 registers, no spills; 2% faster than three at 256^3 FP16); with
// lag 2 (64 KB) three fit
#ifndef LBM_ADJ2M_MINB
#define LBM_ADJ2M_MINB (ADJ2_LAG == 2 ? 24 / LBM_ADJ2M_EY : 32 / LBM_ADJ2M_EY)
#endif

// a_k(s) of one site of step A or B: b = the reverse-streamed adjoint, v =
// the stored forward values of its pulled populations; d, l = its tau and
// lid terms.
template <class S>
__device__ __forceinline__ void adjoint_site(const S (&v)[Q], uint8_t b8, float lidv, float omega,
                                             const Weights<float> &W, float (&b)[Q], float &d, float &l)
{
    if (b8 == 0) {
        float g[Q], rho, ux, uy, uz;
        forward_point<S, float>(v, g, rho, ux, uy, uz);
        adjoint_fluid_point<float>(g, b, rho, ux, uy, uz, omega, d);
    } else {
        adjoint_general<S, float, float>(v, b, b8, lidv, omega, W, d, l);
    }
}
// the stored values of a site's forward pull from its step's Q
template <class S>
__device__ __forceinline__ void adjoint_pull(const S *__restrict__ fwd, const unsigned (&off)[Q], unsigned site,
                                             S (&v)[Q])
{
#pragma unroll
    for (int i = 0; i < Q; ++i) v[i] = load_one(fwd + (site + off[i]));
}

// MACRO = true: fwd_a / fwd_b hold the three MODE_STEP_ADJ planes (float) of
// Q_k / Q_{k-1} instead of the states, and no tau term is formed.
//
// Iteration p: step A at plane p (p <= zi1), then step B at plane
// q = p - ADJ2_LAG (q in [zi0, zi1)).  Step B at plane q reads population i
// of a_k at plane q + ez_i.  Lag 1: a block barrier between them.  Lag 2:
// every thread arrives on the mbarrier after step A(p) and waits for the
// phase after step B(p - 2), whose planes p-1 .. p-3 were complete at the
// previous wait; a warp can then run at most one plane ahead of the slowest
// (step A(p+1) while another is in step B(p-2)), which the plane slots'
// depths 3 / 4 / 5 allow for.
template <class S, bool MACRO>
__global__ void __launch_bounds__(ADJ2_EX * adj2_ey<MACRO>(), MACRO ? LBM_ADJ2M_MINB : LBM_ADJ2_MINB)
    adjoint2_kernel(Adj2Args a)
{
    extern __shared__ float adj2_smem[];  // [ADJ2_SLOTS][EY][ADJ2_EX], then the mbarrier
    constexpr int EY = adj2_ey<MACRO>(), TY = EY - 2;
    constexpr int PL = ADJ2_EX * EY;
    constexpr int LAG = ADJ2_LAG;
    constexpr Adj2Layout LAY = adj2_layout();
    // slot depth of a population with ez = +1, 0, -1
    constexpr int DP = 1 + LAG, D0 = 2 + LAG, DM = 3 + LAG;
    uint64_t *bar = reinterpret_cast<uint64_t *>(adj2_smem + ADJ2_SLOTS * PL);
    const int dim = a.dim;
    const unsigned plane = (unsigned)dim * (unsigned)dim;
    const int lx = (int)threadIdx.x % ADJ2_EX, ly = (int)threadIdx.x / ADJ2_EX;
    int t = (int)blockIdx.x;
    const int tx = t % a.ntx;
    t /= a.ntx;
    const int ty = t % a.nty, tz = t / a.nty;
    const int xi0 = 1 + tx * ADJ2_TX, yi0 = 1 + ty * TY, zi0 = 1 + tz * a.zc;
    const int zi1 = min(zi0 + a.zc, dim - 1);  // owned planes [zi0, zi1)
    const int x = xi0 - 1 + lx, y = yi0 - 1 + ly;
    const bool in_dom = x < dim && y < dim;
    const bool owned = lx >= 1 && lx <= ADJ2_TX && ly >= 1 && ly <= TY && x <= dim - 2 && y <= dim - 2;
    // block-uniform: every site of the ext tile / owned tile in x, y is FLUID
    // on the planes [2, dim-3]
    const bool ext_fluid = xi0 - 1 >= 2 && xi0 + ADJ2_EX - 2 <= dim - 3 && yi0 - 1 >= 2 && yi0 + EY - 2 <= dim - 3;
    const bool own_fluid = xi0 >= 2 && xi0 + ADJ2_TX - 1 <= dim - 3 && yi0 >= 2 && yi0 + TY - 1 <= dim - 3;
    const S *fwd_a = static_cast<const S *>(a.fwd_a);
    const S *fwd_b = static_cast<const S *>(a.fwd_b);
    const float *lid = static_cast<const float *>(a.lid);
    const Weights<float> W = make_weights<float>();
    const float omega = a.omega;
    float dw = 0.f, dl = 0.f;
    const unsigned col = (unsigned)y * (unsigned)dim + (unsigned)x;
    // register-held populations of a_k by plane (index k: plane p - k as of
    // step A of plane p): 6 (ez = +1) back to p - LAG + 1, 0 back to p - LAG,
    // 5 (ez = -1) back to p - LAG - 1
    float h6[LAG], h0[LAG + 1], h5[LAG + 2];
#pragma unroll
    for (int k = 0; k < LAG; ++k) h6[k] = 0.f;
#pragma unroll
    for (int k = 0; k <= LAG; ++k) h0[k] = 0.f;
#pragma unroll
    for (int k = 0; k <= LAG + 1; ++k) h5[k] = 0.f;
    if constexpr (LAG == 2) {
        if (threadIdx.x == 0) mbar_init(bar, blockDim.x);
        __syncthreads();
    }
    uint32_t phase = 0;

    for (int p = zi0 - 1; p <= zi1 - 1 + LAG; ++p) {
#pragma unroll
        for (int k = LAG - 1; k > 0; --k) h6[k] = h6[k - 1];
#pragma unroll
        for (int k = LAG; k > 0; --k) h0[k] = h0[k - 1];
#pragma unroll
        for (int k = LAG + 1; k > 0; --k) h5[k] = h5[k - 1];
        // ---- step A: a_k at (x, y, p) of the ext tile
        if (p <= zi1) {
            float b[Q];
            const unsigned site = (unsigned)p * plane + col;
            uint8_t b8 = M_WALL;
            if (in_dom) b8 = (ext_fluid && p >= 2 && p <= dim - 3) ? (uint8_t)0 : __ldg(a.map + site);
            if (b8 & M_WALL) {
#pragma unroll
                for (int i = 0; i < Q; ++i) b[i] = 0.f;
            } else {
#pragma unroll
                for (int i = 0; i < Q; ++i) b[i] = __ldg(a.ain + (site + a.off_up[i]));
                float d = 0.f, l = 0.f;
                const float lidv = (b8 & M_FRONT) ? lid[col] : 0.f;
                if constexpr (MACRO) {
                    const float *m = static_cast<const float *>(a.fwd_a);
                    adjoint_site_macro<float>(b, b8, __ldg(m + site), __ldg(m + (site + a.off_own[1])),
                                              __ldg(m + (site + a.off_own[2])), lidv, omega, l);
                } else {
                    S v[Q];
                    adjoint_pull<S>(fwd_a, a.off_down, site, v);
                    adjoint_site<S>(v, b8, lidv, omega, W, b, d, l);
                }
                if (owned && p >= zi0 && p < zi1) {
                    dw += d;
                    dl += l;
                }
            }
            const int mp = p % DP, m0 = p % D0, mm = p % DM;
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                if (adj2_in_regs(i)) continue;
                const int slot = LAY.base[i] + (ez_of(i) == 1 ? mp : (ez_of(i) == 0 ? m0 : mm));
                adj2_smem[slot * PL + threadIdx.x] = b[i];
            }
            h0[0] = b[0];
            h5[0] = b[5];
            h6[0] = b[6];
        }
        // ---- step B: a_{k-1} at (x, y, q) of the owned tile.  Its forward
        // values do not depend on step A: loaded before the barrier (lag 1),
        // they arrive while the block waits there.
        const int q = p - LAG;
        const bool do_b = owned && q >= zi0 && q < zi1;
        const unsigned site_b = (unsigned)q * plane + col;
        float mb[3];
        S vb[MACRO ? 1 : Q];
        uint8_t b8b = 0;
        if (do_b) {  // owned sites are never walls
            b8b = (own_fluid && q >= 2 && q <= dim - 3) ? (uint8_t)0 : __ldg(a.map + site_b);
            if constexpr (MACRO) {
                const float *m = static_cast<const float *>(a.fwd_b);
                mb[0] = __ldg(m + site_b);
                mb[1] = __ldg(m + (site_b + a.off_own[1]));
                mb[2] = __ldg(m + (site_b + a.off_own[2]));
            } else {
                adjoint_pull<S>(fwd_b, a.off_down, site_b, vb);
            }
        }
        if constexpr (LAG == 1) __syncthreads();
        else mbar_arrive(bar);
        if (do_b) {
            const unsigned site = site_b;
            const uint8_t b8 = b8b;
            // plane q + ez_i of population i
            const int mp = (q + 1) % DP, m0 = q % D0, mm = (q + DM - 1) % DM;
            float b[Q];
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                if (adj2_in_regs(i)) continue;
                const int slot = LAY.base[i] + (ez_of(i) == 1 ? mp : (ez_of(i) == 0 ? m0 : mm));
                b[i] = adj2_smem[slot * PL + (ly + ey_of(i)) * ADJ2_EX + (lx + ex_of(i))];
            }
            b[0] = h0[LAG];
            b[5] = h5[LAG + 1];
            b[6] = h6[LAG - 1];
            float d = 0.f, l = 0.f;
            const float lidv = (b8 & M_FRONT) ? lid[col] : 0.f;
            if constexpr (MACRO) adjoint_site_macro<float>(b, b8, mb[0], mb[1], mb[2], lidv, omega, l);
            else adjoint_site<S>(vb, b8, lidv, omega, W, b, d, l);
            dw += d;
            dl += l;
#pragma unroll
            for (int i = 0; i < Q; ++i) a.aout[site + a.off_own[i]] = b[i];
        }
        if constexpr (LAG == 2) {
            // bounded: on expiry flag the launch and leave the loop (every
            // thread then expires at this or the next phase and reaches the
            // block reduction below)
            if (!mbar_wait_bounded(bar, phase & 1u, kWaitLimit)) {
                atomicOr(a.status, 2);
                break;
            }
            ++phase;
        }
    }
    // one MOVING site per column, in one chunk: a single writer per column
    if (owned && zi0 <= dim - 2 && dim - 2 < zi1) a.grad_lid[col] += (double)dl;
    if constexpr (!MACRO) block_reduce_add((double)dw, a.tau_acc);
}

// ---------------------------------------------------------------------------
// The stored-point two-step adjoint with its inputs staged by TMA.
//
// Same tiles, z-chunks, plane slots and per-site arithmetic as
// adjoint2_kernel<S, true>, but no thread loads its inputs from global
// memory: for every plane p one thread issues 25 tiled TMA loads
// (cp.async.bulk.tensor) of 40 x 8 floats into one stage of a two-stage
// shared-memory ring -- the 19 populations of a_{k+1} at (x + e_ix, y + e_iy,
// p + e_iz), the three point planes of Q_k at plane p (step A) and those of
// Q_{k-1} at plane p - 1 (step B) -- completing on that stage's mbarrier.
// The stage of plane p + 2 is issued as soon as every thread has read the
// stage of plane p (the block barrier between step A and step B), so the
// loads of the next plane are in flight while the block computes.
//
// Boxes start at xs = the ext tile's first x - 1 rounded down to a multiple
// of 4 (16 bytes: the TMA alignment of the innermost coordinate); 40 columns
// cover the 34 that the tile reads.  Coordinates outside the lattice (x or y
// in {-4 .. -1} or >= dim, planes -1 and dim) are filled with zeros by the
// TMA unit; no site that reads them is a non-wall site.
//
// Waits on the stage barriers are bounded.  Every thread folds its wait's
// outcome into the block barrier (__syncthreads_or), so an expired wait
// stops the whole block before step B writes anything; it sets bit 1 of the
// status word, the issuing thread drains the copies still in flight (again
// bounded) and the block returns.
// ---------------------------------------------------------------------------
constexpr int ADJ2T_BW = 40;                         // box columns (floats)
constexpr int ADJ2T_NB = Q + 6;                      // boxes per stage
constexpr int ADJ2T_BOX = ADJ2T_BW * ADJ2_EY;        // floats per box
constexpr int ADJ2T_STAGE = ADJ2T_NB * ADJ2T_BOX;    // floats per stage
constexpr int ADJ2T_NS = 2;                          // stages
constexpr size_t adj2t_smem_bytes()
{
    return (size_t)ADJ2T_NS * ADJ2T_STAGE * sizeof(float) + (size_t)ADJ2_SLOTS * ADJ2_EX * ADJ2_EY * sizeof(float) +
           (size_t)ADJ2T_NS * sizeof(uint64_t);
}
static_assert((ADJ2T_BOX * sizeof(float)) % 128 == 0, "TMA destinations stay 128-byte aligned");

// One 4-D tiled TMA load (coordinates x, y, z, w; x fastest) into shared
// memory, completing on bar.  x * 4 bytes must be a multiple of 16.
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int x, int y, int z, int w,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_addr(bar))
        : "memory");
}

// map_a: a_{k+1} as (dim, dim, dim, 19) floats; map_pa / map_pb: the point
// planes of Q_k / Q_{k-1} as (dim, dim, dim, 3) floats; all with 40 x 8 x 1
// x 1 boxes.  (A template so that every translation unit that includes
// this header can hold it.)
template <int NS>
__global__ void __launch_bounds__(ADJ2_EX *ADJ2_EY, 2)
    adjoint2_tma_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_pa,
                        const __grid_constant__ CUtensorMap map_pb, Adj2Args a)
{
    static_assert(NS == ADJ2T_NS, "two stages");
    static_assert(ADJ2_LAG == 1, "the staged kernel runs step B one plane behind step A");
    extern __shared__ __align__(128) unsigned char adj2t_raw[];
    float *stages = reinterpret_cast<float *>(adj2t_raw);
    float *slots = stages + ADJ2T_NS * ADJ2T_STAGE;
    constexpr int EY = ADJ2_EY, TY = EY - 2;
    constexpr int PL = ADJ2_EX * EY;
    uint64_t *full = reinterpret_cast<uint64_t *>(slots + ADJ2_SLOTS * PL);
    constexpr Adj2Layout LAY = adj2_layout();
    constexpr int DP = 2, D0 = 3, DM = 4;  // plane slots of a population with ez = +1, 0, -1
    const int dim = a.dim;
    const unsigned plane = (unsigned)dim * (unsigned)dim;
    const int lx = (int)threadIdx.x % ADJ2_EX, ly = (int)threadIdx.x / ADJ2_EX;
    int t = (int)blockIdx.x;
    const int tx = t % a.ntx;
    t /= a.ntx;
    const int ty = t % a.nty, tz = t / a.nty;
    const int xi0 = 1 + tx * ADJ2_TX, yi0 = 1 + ty * TY, zi0 = 1 + tz * a.zc;
    const int zi1 = min(zi0 + a.zc, dim - 1);  // owned planes [zi0, zi1)
    const int x = xi0 - 1 + lx, y = yi0 - 1 + ly;
    const bool in_dom = x < dim && y < dim;
    const bool owned = lx >= 1 && lx <= ADJ2_TX && ly >= 1 && ly <= TY && x <= dim - 2 && y <= dim - 2;
    const bool ext_fluid = xi0 - 1 >= 2 && xi0 + ADJ2_EX - 2 <= dim - 3 && yi0 - 1 >= 2 && yi0 + EY - 2 <= dim - 3;
    const bool own_fluid = xi0 >= 2 && xi0 + ADJ2_TX - 1 <= dim - 3 && yi0 >= 2 && yi0 + TY - 1 <= dim - 3;
    // box origin in x (16-byte aligned; -4 for the first tile column) and the
    // box column of this thread's site
    const int xs = ((xi0 - 2) >> 2) * 4;
    const int col0 = lx + (xi0 - 1 - xs);
    const int ybox = yi0 - 1;  // box row 0 = the ext tile's first row
    const float *lid = static_cast<const float *>(a.lid);
    const float omega = a.omega;
    float dl = 0.f;
    const unsigned col = (unsigned)y * (unsigned)dim + (unsigned)x;
    // register-held populations of a_k (0: planes p, p - 1; 5: p .. p - 2);
    // population 6 of step B is the current step A's
    float h0[2] = {0.f, 0.f}, h5[3] = {0.f, 0.f, 0.f};

    const int p0 = zi0 - 1;
    const int np = zi1 - p0 + 1;  // step A at planes p0 .. zi1, step B one behind
    // stage j (plane p0 + j) into ring slot j % 2; thread 0 only (warp 0 has
    // no step-B sites, so the issue stays off the block's critical path)
    auto issue = [&](int j) {
        const int p = p0 + j;
        float *st = stages + (j & 1) * ADJ2T_STAGE;
        uint64_t *bar = &full[j & 1];
        mbar_expect_tx(bar, (uint32_t)(ADJ2T_STAGE * sizeof(float)));
#pragma unroll
        for (int i = 0; i < Q; ++i) tma_load_4d(st + i * ADJ2T_BOX, &map_a, xs, ybox + ey_of(i), p + ez_of(i), i, bar);
#pragma unroll
        for (int c = 0; c < 3; ++c) tma_load_4d(st + (Q + c) * ADJ2T_BOX, &map_pa, xs, ybox, p, c, bar);
#pragma unroll
        for (int c = 0; c < 3; ++c) tma_load_4d(st + (Q + 3 + c) * ADJ2T_BOX, &map_pb, xs, ybox, p - 1, c, bar);
    };
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_fence_init();
        for (int k = 0; k < min(ADJ2T_NS, np); ++k) issue(k);
    }
    __syncthreads();

    int j = 0;
    bool err = false;
    for (; j < np; ++j) {
        const int p = p0 + j;
        const float *st = stages + (j & 1) * ADJ2T_STAGE;
        const bool bad = !mbar_wait_bounded(&full[j & 1], (uint32_t)(j >> 1) & 1u, kWaitLimit);
        h5[2] = h5[1];
        h5[1] = h5[0];
        h0[1] = h0[0];
        // ---- step A: a_k at (x, y, p) of the ext tile (p <= zi1 always)
        {
            float b[Q];
            const unsigned site = (unsigned)p * plane + col;
            uint8_t b8 = M_WALL;
            if (in_dom) b8 = (ext_fluid && p >= 2 && p <= dim - 3) ? (uint8_t)0 : __ldg(a.map + site);
            if (b8 & M_WALL) {
#pragma unroll
                for (int i = 0; i < Q; ++i) b[i] = 0.f;
            } else {
                const float *row = st + ly * ADJ2T_BW + col0;
#pragma unroll
                for (int i = 0; i < Q; ++i) b[i] = row[i * ADJ2T_BOX + ex_of(i)];
                float l = 0.f;
                const float lidv = (b8 & M_FRONT) ? lid[col] : 0.f;
                adjoint_site_macro<float>(b, b8, row[Q * ADJ2T_BOX], row[(Q + 1) * ADJ2T_BOX],
                                          row[(Q + 2) * ADJ2T_BOX], lidv, omega, l);
                if (owned && p >= zi0 && p < zi1) dl += l;
            }
            const int mp = p % DP, m0 = p % D0, mm = p % DM;
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                if (adj2_in_regs(i)) continue;
                const int slot = LAY.base[i] + (ez_of(i) == 1 ? mp : (ez_of(i) == 0 ? m0 : mm));
                slots[slot * PL + threadIdx.x] = b[i];
            }
            h0[0] = b[0];
            h5[0] = b[5];
            const float b6 = b[6];
            // ---- step B's inputs: its points (from this stage) and its map
            const int q = p - 1;
            const bool do_b = owned && q >= zi0 && q < zi1;
            const unsigned site_b = (unsigned)q * plane + col;
            float mb[3];
            uint8_t b8b = 0;
            {
                const float *row = st + ly * ADJ2T_BW + col0;
                mb[0] = row[(Q + 3) * ADJ2T_BOX];
                mb[1] = row[(Q + 4) * ADJ2T_BOX];
                mb[2] = row[(Q + 5) * ADJ2T_BOX];
            }
            if (do_b) b8b = (own_fluid && q >= 2 && q <= dim - 3) ? (uint8_t)0 : __ldg(a.map + site_b);
            // every thread has read stage j and written its plane slots
            if (__syncthreads_or(bad)) {
                err = true;
                break;
            }
            if (threadIdx.x == 0 && j + ADJ2T_NS < np) issue(j + ADJ2T_NS);
            // ---- step B: a_{k-1} at (x, y, q) of the owned tile
            if (do_b) {
                const int mq = (q + 1) % DP, m0q = q % D0, mmq = (q + DM - 1) % DM;
                float bb[Q];
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    if (adj2_in_regs(i)) continue;
                    const int slot = LAY.base[i] + (ez_of(i) == 1 ? mq : (ez_of(i) == 0 ? m0q : mmq));
                    bb[i] = slots[slot * PL + (ly + ey_of(i)) * ADJ2_EX + (lx + ex_of(i))];
                }
                bb[0] = h0[1];
                bb[5] = h5[2];
                bb[6] = b6;
                float l = 0.f;
                const float lidv = (b8b & M_FRONT) ? lid[col] : 0.f;
                adjoint_site_macro<float>(bb, b8b, mb[0], mb[1], mb[2], lidv, omega, l);
                dl += l;
#pragma unroll
                for (int i = 0; i < Q; ++i) a.aout[site_b + a.off_own[i]] = bb[i];
            }
        }
    }
    if (err) {
        if (threadIdx.x == 0) {
            atomicOr(a.status, 2);
            // drain what was issued and not consumed (stages j .. j + 1; bounded)
            for (int k = j; k < min(j + ADJ2T_NS, np); ++k)
                mbar_wait_bounded(&full[k & 1], (uint32_t)(k >> 1) & 1u, kWaitLimit);
        }
        return;
    }
    // one MOVING site per column, in one chunk: a single writer per column
    if (owned && zi0 <= dim - 2 && dim - 2 < zi1) a.grad_lid[col] += (double)dl;
}

// Seed of the backward sweep: a_T = dJ/dR_T for the mid-plane loss
//   J = (1/M) sum over the FLUID sites of plane y = plane_y of (u_x - target)^2,
// dJ/dR_T(s, i) = (2/M) (u_x - target) (e_ix - u_x) / rho; zero elsewhere.
// a.dloss carries the factor dJ_total/dJ * 2 / M.  Also writes the loss
// partials (sum of squared differences) when loss_part != NULL.
template <class S, class A>
__global__ void __launch_bounds__(256) loss_seed_kernel(AdjArgs a)
{
    const int dim = a.dim;
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    double sq = 0.0;
    if (id < a.n) {
        const int x = (int)(id % dim), y = (int)((id / dim) % dim), z = (int)(id / ((size_t)dim * dim));
        const bool on = y == a.plane_y && pack_cell(dim, x, y, z) == 0;
        A *aout = static_cast<A *>(a.aout);
        A out[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) out[i] = (A)0;
        if (on) {
            const S *fwd = static_cast<const S *>(a.fwd);
            A g[Q];
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                const size_t src = id - (ptrdiff_t)ex_of(i) - (ptrdiff_t)ey_of(i) * dim - (ptrdiff_t)ez_of(i) * dim * dim;
                g[i] = fwd_value<S, A>(fwd[(size_t)i * a.n + src], i);
            }
            A rho, ux, uy, uz;
            moments_plain(g, rho, ux, uy, uz);
            const A tgt = static_cast<const A *>(a.target)[(size_t)x + (size_t)z * dim];
            const A diff = ux - tgt;
            sq = (double)diff * (double)diff;
            const A d = (A)a.dloss * diff / rho;
#pragma unroll
            for (int i = 0; i < Q; ++i) out[i] = d * ((A)ex_of(i) - ux);
        }
        if (aout) {
#pragma unroll
            for (int i = 0; i < Q; ++i) aout[(size_t)i * a.n + id] = out[i];
        }
    }
    if (a.loss_part) block_reduce_write(sq, 0.0, a.loss_part);
}

// Lid sensitivity of an initial state made by the init kernel: the FRONT
// sites (x, y in [1, dim-2], z = dim-2) start at the equilibrium at rho = 1
// and u = (lid, 0, 0) (kernels.cl:292-308); dR_0(s,i)/dlid =
// w_i (3 e_ix + (9 e_ix^2 - 3) lid).
template <class S, class A>
__global__ void lid_init_grad_kernel(AdjArgs a)
{
    using C = typename Compute<S>::type;
    const int dim = a.dim;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= dim * dim) return;
    const int x = k % dim, y = k / dim;
    if (x < 1 || y < 1 || x > dim - 2 || y > dim - 2) return;
    const size_t id = (size_t)x + (size_t)y * dim + (size_t)(dim - 2) * dim * dim;
    const A *a0 = static_cast<const A *>(a.ain);
    const A lid = (A) static_cast<const C *>(a.lid)[k];
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const A ex = (A)ex_of(i);
        s += (double)(a0[(size_t)i * a.n + id] * w_of<A>(i) * ((A)3 * ex + ((A)9 * ex * ex - (A)3) * lid));
    }
    a.grad_lid[k] += s;
}

// Adjoint buffer (post-stream layout) -> CSoA order of the F dumps, in the
// dump element type T.
template <class A, class T>
__global__ void export_adjoint_kernel(const A *__restrict__ adj, T *__restrict__ out, size_t o0, size_t count, int sd,
                                      size_t n)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    size_t id;
    int q;
    decode_csoa(o0 + k, sd, n, id, q);
    out[k] = (T)adj[(size_t)q * n + id];
}

// Launchers of the FP64 adjoint over FP32 / 16-bit storage (their own
// translation unit, lbm_adjoint_f64.cu): prec is the storage lbm_precision.
cudaError_t launch_adjoint_step_a64(int prec, const AdjArgs &a, unsigned gi, unsigned gf, unsigned block,
                                    cudaStream_t s, bool macro);
cudaError_t launch_loss_seed_a64(int prec, const AdjArgs &a, unsigned grid, unsigned block, cudaStream_t s);
cudaError_t launch_lid_init_grad_a64(int prec, const AdjArgs &a, cudaStream_t s);

}  // namespace lbm
