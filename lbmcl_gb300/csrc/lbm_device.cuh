// lbm_device.cuh -- device-side building blocks of the D3Q19 BGK lid-driven
// cavity on sm_103a: lattice constants, the packed cell map, exact-order and
// 16-bit-deviation site updates, and the pull gather of one x-vector.
//
// Layout in HBM (one handle):
//   populations  two buffers, structure of arrays f[q][z][y][x] (x fastest),
//                19 * dim^3 elements each, element = float | double | 16-bit
//   map          uint8 [dim^3] (bits below)
//   rho, u       macro type [dim^3] and [3][dim^3] (planar, kernels.cl:68-70)
//
// State convention.  The buffers hold the POST-COLLISION populations P of
// each site.  The reference stores the post-stream buffer R instead
// (kernels.cl:420-424 pushes into f_stream).  R_t = S(P_{t-1}), where S pulls
// P[s - e_i][i] into slot (s, i); a slot whose source is a wall keeps the
// reference's fixed value (its initial equilibrium, kernels.cl:303-317, never
// overwritten because walls never push, kernels.cl:421).  One iteration
// P_t = C(S(P_{t-1})) is one fused pull-stream + collide pass.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace lbm {

constexpr int Q = 19;

// D3Q19 velocity set in the reference's ordering (kernels.cl:131-205):
// 0 rest; 1..6 = +x,+y,-x,-y,-z,+z; 7..18 edges.
__host__ __device__ constexpr int ex_of(int i)
{
    return (i == 1 || i == 7 || i == 10 || i == 11 || i == 15) ? 1
         : (i == 3 || i == 8 || i == 9 || i == 13 || i == 17) ? -1 : 0;
}
__host__ __device__ constexpr int ey_of(int i)
{
    return (i == 2 || i == 7 || i == 8 || i == 12 || i == 16) ? 1
         : (i == 4 || i == 9 || i == 10 || i == 14 || i == 18) ? -1 : 0;
}
__host__ __device__ constexpr int ez_of(int i)
{
    return (i == 6 || i == 15 || i == 16 || i == 17 || i == 18) ? 1
         : (i == 5 || i == 11 || i == 12 || i == 13 || i == 14) ? -1 : 0;
}
// opposite direction (kernels.cl:208-226)
__host__ __device__ constexpr int opp_of(int i)
{
    return i == 0 ? 0 : i == 1 ? 3 : i == 2 ? 4 : i == 3 ? 1 : i == 4 ? 2 : i == 5 ? 6 : i == 6 ? 5
         : i == 7 ? 9 : i == 8 ? 10 : i == 9 ? 7 : i == 10 ? 8 : i == 11 ? 17 : i == 12 ? 18
         : i == 13 ? 15 : i == 14 ? 16 : i == 15 ? 13 : i == 16 ? 14 : i == 17 ? 11 : 12;
}
// weight class: 0 rest (1/3), 1 axis (1/18), 2 edge (1/36)  (kernels.cl:110-128)
__host__ __device__ constexpr int wclass_of(int i) { return i == 0 ? 0 : (i <= 6 ? 1 : 2); }

// ---------------------------------------------------------------------------
// Packed cell map.  One byte per site instead of the reference's int
// (kernels.cl:236-266 / common.h:7-20).  The face bits stay set on corners so
// that every non-wall site knows which of its pull sources are walls.
//   WALL    -> 0x80
//   CORNER  -> its three face bits | 0x40      (reference: CORNER only)
//   FLUID   -> 0
//   MOVING  -> FRONT bit alone                 (reference: FRONT | MOVING)
//   others  -> face bits (bounce-back sites)
// ---------------------------------------------------------------------------
constexpr uint8_t M_LEFT = 0x01, M_RIGHT = 0x02, M_BOTTOM = 0x04, M_TOP = 0x08;
constexpr uint8_t M_BACK = 0x10, M_FRONT = 0x20, M_CORNER = 0x40, M_WALL = 0x80;
constexpr uint8_t M_FACES = 0x3f;

__host__ __device__ inline uint8_t pack_cell(int dim, int x, int y, int z)
{
    if (x == 0 || y == 0 || z == 0 || x == dim - 1 || y == dim - 1 || z == dim - 1) return M_WALL;
    uint8_t b = 0;
    if (x == 1) b |= M_LEFT;
    if (x == dim - 2) b |= M_RIGHT;
    if (y == 1) b |= M_BOTTOM;
    if (y == dim - 2) b |= M_TOP;
    if (z == 1) b |= M_BACK;
    if (z == dim - 2) b |= M_FRONT;
    // the four BACK corners (kernels.cl:254-260)
    if ((b & M_BACK) && !(b & M_FRONT) && (b & (M_LEFT | M_RIGHT)) && (b & (M_BOTTOM | M_TOP)))
        b |= M_CORNER;
    return b;
}

// Reference int cell type of a packed byte (common.h:7-20 values).
__host__ __device__ inline int unpack_cell(uint8_t b)
{
    if (b & M_WALL) return 0x008;
    if (b & M_CORNER) return 0x004;
    if (b == 0) return 0x001;
    int ct = 0;
    if (b & M_LEFT) ct |= 0x010;
    if (b & M_RIGHT) ct |= 0x020;
    if (b & M_TOP) ct |= 0x040;
    if (b & M_BOTTOM) ct |= 0x080;
    if (b & M_FRONT) ct |= 0x100;
    if (b & M_BACK) ct |= 0x200;
    if (ct == 0x100) ct |= 0x002;
    return ct;
}

// Is the pull source of population i of a site with byte b a wall?
__host__ __device__ constexpr bool wall_sourced(int i, uint8_t b)
{
    return (ex_of(i) == 1 && (b & M_LEFT)) || (ex_of(i) == -1 && (b & M_RIGHT)) ||
           (ey_of(i) == 1 && (b & M_BOTTOM)) || (ey_of(i) == -1 && (b & M_TOP)) ||
           (ez_of(i) == 1 && (b & M_BACK)) || (ez_of(i) == -1 && (b & M_FRONT));
}

// ---------------------------------------------------------------------------
// IEEE operations that the compiler may not contract into FMAs: the FP32 and
// FP64 modes evaluate every expression in the reference's operand order
// (kernels.cl:270-273, 352-418), so they agree bit for bit with the oracle.
// ---------------------------------------------------------------------------
template <class T> struct X;
template <> struct X<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
template <> struct X<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};

template <class T> struct Weights {
    T w[3];
};

// Lattice weights evaluated in T like the reference's constants
// (kernels.cl:110-128 with -cl-single-precision-constant for float).
template <class T> __host__ __device__ inline Weights<T> make_weights()
{
    Weights<T> W;
    W.w[0] = (T)1.0 / (T)3.0;
    W.w[1] = (T)1.0 / (T)18.0;
    W.w[2] = (T)1.0 / (T)36.0;
    return W;
}

// Signed projection e_i . u of the exact-order evaluation.  The reference
// forms ((ux*ex) + (uy*ey)) + (uz*ez) with integer e in {-1,0,1}; the products
// are exact and the additions of zeros are exact, so the value equals one
// signed sum of the non-zero terms (only the sign of a zero can differ, which
// no later operation observes).  Opposite directions give exact negatives.
template <class T>
__device__ __forceinline__ T signed_pair(int sp, int sq, T p, T q)
{
    using O = X<T>;
    // (p*sp) + (q*sq) for sp, sq in {-1, +1}, as one IEEE operation
    return (sp > 0 && sq > 0) ? O::add(p, q)
         : (sp < 0 && sq < 0) ? -O::add(p, q)
         : (sp < 0)           ? O::sub(q, p)
                              : O::sub(p, q);
}

template <class T>
__device__ __forceinline__ T proj_exact(int i, T ux, T uy, T uz)
{
    const int a = ex_of(i), b = ey_of(i), c = ez_of(i);
    if (a != 0 && b != 0) return signed_pair(a, b, ux, uy);
    if (a != 0 && c != 0) return signed_pair(a, c, ux, uz);
    if (b != 0 && c != 0) return signed_pair(b, c, uy, uz);
    if (a != 0) return a > 0 ? ux : -ux;
    if (b != 0) return b > 0 ? uy : -uy;
    if (c != 0) return c > 0 ? uz : -uz;
    return (T)0;
}

// The bracket of the equilibrium, ((1 + 3 eu) + (4.5 eu) eu) - 1.5 u2
// (kernels.cl:308, 397, 416), for eu = proj and c15 = 1.5 u2.
template <class T>
__device__ __forceinline__ T eq_bracket_exact(T eu, T c15)
{
    using O = X<T>;
    return O::sub(O::add(O::add((T)1.0, O::mul((T)3.0, eu)), O::mul(O::mul((T)4.5, eu), eu)), c15);
}

// BGK relaxation of a fluid or moving site in place: f_i += inv_tau (feq_i - f_i)
// with feq_i = (rho w_i) * bracket_i  (kernels.cl:270-273, 412-418).
// Opposite directions i, j share their products: e_j.u = -e_i.u exactly, so
// 3 e_j.u = -(3 e_i.u) and (4.5 e_j.u) e_j.u = (4.5 e_i.u) e_i.u bit for bit
// (round-to-nearest is symmetric), and 1 + 3 e_j.u is 1 - 3 e_i.u; the rest
// population's bracket ((1 + 3 * 0) + (4.5 * 0) * 0) - 1.5 u2 is 1 - 1.5 u2.
// Three FP64 operations fewer per pair than the reference's per-direction
// evaluation, with identical results.
template <class T>
__device__ __forceinline__ void relax_exact(T (&f)[Q], T r, T ux, T uy, T uz, T inv_tau, const Weights<T> &W)
{
    using O = X<T>;
    const T u2 = O::add(O::add(O::mul(ux, ux), O::mul(uy, uy)), O::mul(uz, uz));
    const T c15 = O::mul((T)1.5, u2);
    const T rw0 = O::mul(r, W.w[0]), rw1 = O::mul(r, W.w[1]), rw2 = O::mul(r, W.w[2]);
    f[0] = O::add(f[0], O::mul(inv_tau, O::sub(O::mul(rw0, O::sub((T)1.0, c15)), f[0])));
#pragma unroll
    for (int i = 1; i < Q; ++i) {
        const int j = opp_of(i);
        if (j < i) continue;
        const T rw = wclass_of(i) == 1 ? rw1 : rw2;
        const T eu = proj_exact(i, ux, uy, uz);
        const T t3 = O::mul((T)3.0, eu);
        const T sq = O::mul(O::mul((T)4.5, eu), eu);
        const T fi = O::mul(rw, O::sub(O::add(O::add((T)1.0, t3), sq), c15));
        const T fj = O::mul(rw, O::sub(O::add(O::sub((T)1.0, t3), sq), c15));
        f[i] = O::add(f[i], O::mul(inv_tau, O::sub(fi, f[i])));
        f[j] = O::add(f[j], O::mul(inv_tau, O::sub(fj, f[j])));
    }
}

// Density in the Sailfish order (kernels.cl:352-354), left to right.
template <class T> __device__ __forceinline__ T rho_sailfish(const T (&f)[Q])
{
    using O = X<T>;
    constexpr int ord[Q] = {5, 11, 12, 14, 13, 0, 1, 2, 7, 8, 4, 10, 9, 6, 15, 16, 18, 17, 3};
    T r = f[ord[0]];
#pragma unroll
    for (int k = 1; k < Q; ++k) r = O::add(r, f[ord[k]]);
    return r;
}

// Density and velocity in the Sailfish order (kernels.cl:352-354, 368-375):
// each momentum a left-to-right chain of signed terms, then / rho.
template <class T>
__device__ __forceinline__ void moments_sailfish(const T (&f)[Q], T &r, T &ux, T &uy, T &uz)
{
    using O = X<T>;
    r = rho_sailfish(f);
    T s = O::sub(f[11], f[13]);
    s = O::add(s, f[1]); s = O::add(s, f[7]); s = O::sub(s, f[8]); s = O::add(s, f[10]);
    s = O::sub(s, f[9]); s = O::add(s, f[15]); s = O::sub(s, f[17]); s = O::sub(s, f[3]);
    ux = O::div(s, r);
    s = O::sub(f[12], f[14]);
    s = O::add(s, f[2]); s = O::add(s, f[7]); s = O::add(s, f[8]); s = O::sub(s, f[4]);
    s = O::sub(s, f[10]); s = O::sub(s, f[9]); s = O::add(s, f[16]); s = O::sub(s, f[18]);
    uy = O::div(s, r);
    s = O::sub(-f[5], f[11]);
    s = O::sub(s, f[12]); s = O::sub(s, f[14]); s = O::sub(s, f[13]); s = O::add(s, f[6]);
    s = O::add(s, f[15]); s = O::add(s, f[16]); s = O::add(s, f[18]); s = O::add(s, f[17]);
    uz = O::div(s, r);
}

// Density (kernels.cl:355) and momentum sums (kernels.cl:376-378) in the
// reference's summation order.
template <class T>
__device__ __forceinline__ void moments_exact(const T (&f)[Q], T &r, T &ux, T &uy, T &uz)
{
    using O = X<T>;
    r = f[0];
#pragma unroll
    for (int i = 1; i < Q; ++i) r = O::add(r, f[i]);
    const T px = O::add(O::add(O::add(O::add(f[1], f[7]), f[10]), f[11]), f[15]);
    const T mx = O::add(O::add(O::add(O::add(f[3], f[8]), f[9]), f[13]), f[17]);
    const T py = O::add(O::add(O::add(O::add(f[2], f[7]), f[8]), f[12]), f[16]);
    const T my = O::add(O::add(O::add(O::add(f[4], f[9]), f[10]), f[14]), f[18]);
    const T pz = O::add(O::add(O::add(O::add(f[6], f[15]), f[16]), f[17]), f[18]);
    const T mz = O::add(O::add(O::add(O::add(f[5], f[11]), f[12]), f[13]), f[14]);
    ux = O::div(O::sub(px, mx), r);
    uy = O::div(O::sub(py, my), r);
    uz = O::div(O::sub(pz, mz), r);
}

// Equilibrium of a site at rest density 1 moving with (lid, 0, 0): the value
// initialize() gives a FRONT site (kernels.cl:292-308) and the fixed value of
// its wall-sourced slots.
template <class T>
__device__ __forceinline__ T init_eq_exact(int i, T lid, const Weights<T> &W)
{
    using O = X<T>;
    const T c15 = O::mul((T)1.5, O::mul(lid, lid));
    const T eu = ex_of(i) > 0 ? lid : (ex_of(i) < 0 ? -lid : (T)0);
    return O::mul(W.w[wclass_of(i)], eq_bracket_exact(eu, c15));
}

// ---------------------------------------------------------------------------
// 16-bit deviation storage: a population is held as D = s (f - w) in FP16
// (s = 2^15) or BF16 (s = 1); all arithmetic is FP32 with FMAs.
// ---------------------------------------------------------------------------
template <class H> struct Dev16 {  // not a 16-bit type: unused placeholders
    static constexpr float scale = 1.0f;
    static constexpr float inv_scale = 1.0f;
};
template <> struct Dev16<__half> {
    static constexpr float scale = 32768.0f;
    static constexpr float inv_scale = 1.0f / 32768.0f;
    static __device__ __forceinline__ float to_f(__half h) { return __half2float(h); }
    static __device__ __forceinline__ __half from_f(float v) { return __float2half_rn(v); }
    static __device__ __forceinline__ void from_f2(float a, float b, __half &ha, __half &hb)
    {
        const __half2 h = __floats2half2_rn(a, b);  // one packed conversion
        ha = __low2half(h);
        hb = __high2half(h);
    }
};
template <> struct Dev16<__nv_bfloat16> {
    static constexpr float scale = 1.0f;
    static constexpr float inv_scale = 1.0f;
    static __device__ __forceinline__ float to_f(__nv_bfloat16 h) { return __bfloat162float(h); }
    static __device__ __forceinline__ __nv_bfloat16 from_f(float v) { return __float2bfloat16_rn(v); }
    static __device__ __forceinline__ void from_f2(float a, float b, __nv_bfloat16 &ha, __nv_bfloat16 &hb)
    {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        ha = __low2bfloat16(h);
        hb = __high2bfloat16(h);
    }
};

__host__ __device__ constexpr float wf_of(int i)
{
    return wclass_of(i) == 0 ? (1.0f / 3.0f) : (wclass_of(i) == 1 ? (1.0f / 18.0f) : (1.0f / 36.0f));
}

// e_i . u for the deviation kernels (plain FP32, contraction allowed).
__device__ __forceinline__ float proj_fast(int i, float ux, float uy, float uz)
{
    float s = 0.0f;
    if (ex_of(i) > 0) s += ux;
    if (ex_of(i) < 0) s -= ux;
    if (ey_of(i) > 0) s += uy;
    if (ey_of(i) < 0) s -= uy;
    if (ez_of(i) > 0) s += uz;
    if (ez_of(i) < 0) s -= uz;
    return s;
}

// Scaled equilibrium deviation s (feq_i - w_i) = s w_i (drho + rho (3 eu + 4.5 eu^2 - 1.5 u2)).
__device__ __forceinline__ float deq_scaled(int i, float drho, float rho, float eu, float c15, float s)
{
    const float p = fmaf(4.5f * eu, eu, fmaf(3.0f, eu, -c15));
    return (s * wf_of(i)) * fmaf(rho, p, drho);
}

// Pull-kernel variants: plain iteration, iteration that also stores rho/u,
// moments-only pass that writes FP64 reduction partials, and iteration that
// stores the adjoint's linearisation point of its input (three planes at
// StepArgs::u: u_x, u_y, u_z of FLUID sites; rho, 0, 0 of MOVING sites).
enum { MODE_STEP = 0, MODE_STEP_MACRO = 1, MODE_REDUCE = 2, MODE_STEP_ADJ = 3 };

// ---------------------------------------------------------------------------
// Per-launch parameters.
// ---------------------------------------------------------------------------
struct StepArgs {
    const void *fin;     // P_{t-1}
    void *fout;          // P_t
    const uint8_t *map;
    const void *lid;     // per-column lid u_x, macro type, dim*dim
    void *rho;           // macro type
    void *u;             // macro type, 3 planes
    int *status;         // bit 0: a density <= 0 or NaN was seen
    double *partials;    // reduction partials, 2 per block
    int dim;
    int nvx;             // x-vectors per row = dim / V
    unsigned nvec;       // vectors in the interior rows = nvx * (dim-2)^2
    unsigned partial_base;  // first reduction-partial slot of this launch
    size_t n;            // dim^3
    double inv_tau;      // 1/tau in the compute precision (rounded by the host)
    float omega_f;       // 1/tau as float, deviation kernels
    // staged variant
    int rows;            // rows per group
    int gpp;             // groups per z-plane = ceil((dim-2) / rows)
    unsigned ngroups;    // gpp * (dim-2)
    int stages;          // ring depth
    // AA variant: fin == fout is the one lattice; 0 = A-step, 1 = B-step
    int aa_phase;
    int sailfish;        // 1: rho and u summed in the Sailfish order (FP32 / FP64)
};

// Initial-state kernel arguments.
struct InitArgs {
    void *f;
    uint8_t *map;
    const void *lid;
    void *rho, *u;
    int dim;
    size_t n;
    uint64_t seed;
    double noise_sigma;
    float noise_sigma_f;  // noise_sigma rounded to float (FP32 / 16-bit storage)
    int in_place;         // 1: the AA kernels' one lattice in A-form (f(s, i) = R_0(s, i));
                          // 0: P_{-1} of the two-lattice kernels
};

// F dump / load kernel arguments (output element range [o0, o0 + count)).
struct DumpArgs {
    void *f;              // the current buffer
    const uint8_t *map;
    const void *lid;
    void *buf;            // staging, T elements
    size_t o0, count;     // output range [o0, o0 + count)
    int dim, sd;          // sd = log2(stride), -1 for SoA of a non-power-of-two lattice
    size_t n;
    int layout;           // LAYOUT_PULL: P of the two-lattice kernels; LAYOUT_AA_A / _B: the
                          // AA lattice in A-form / B-form
};
enum { LAYOUT_PULL = -1, LAYOUT_AA_A = 0, LAYOUT_AA_B = 1 };

}  // namespace lbm
