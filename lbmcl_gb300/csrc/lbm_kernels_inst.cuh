// lbm_kernels_inst.cuh -- instantiates the kernels of one storage type.
// Included by lbm_kernels_<type>.cu with LBM_S (element type), LBM_T (F-dump
// element type) and LBM_SFX (launcher suffix) defined.
#include "lbm_kernels.cuh"
#include "lbm_launch.h"

namespace lbm {

#define LBM_CAT2(a, b) a##b
#define LBM_CAT(a, b) LBM_CAT2(a, b)

// One iteration (or reduction pass) of the direct variant with VB-byte
// vectors: the interior-row launch, then the face-row launch.  *nparts gets
// the number of reduction partial slots the two launches use.
// passes: bit 0 the interior-row launch, bit 1 the face-row launch (on
// stream sf when given).
template <int VB>
static cudaError_t launch_direct(int mode, const StepArgs &a0, unsigned block, cudaStream_t s, unsigned *nparts,
                                 int passes = 3, cudaStream_t sf = nullptr)
{
    constexpr int V = VB / (int)sizeof(LBM_S);
    StepArgs a = a0;
    a.nvx = a0.dim / V;
    const size_t m = (size_t)(a.dim - 4);
    const unsigned gi = (unsigned)((m * m * (size_t)a.nvx + block - 1) / block);
    const unsigned gf = (unsigned)(((size_t)4 * (a.dim - 3) * (size_t)a.nvx + block - 1) / block);
    for (int pass = 0; pass < 2; ++pass) {
        if (!(passes & (1 << pass))) continue;
        if (pass == 1 && sf) s = sf;
        const unsigned grid = pass == 0 ? gi : gf;
        if (grid == 0) continue;
        a.partial_base = pass == 0 ? 0u : gi;
        if (pass == 0) {
            switch (mode) {
            case MODE_STEP: pull_kernel<LBM_S, MODE_STEP, VB, ROWS_INTERIOR><<<grid, block, 0, s>>>(a); break;
            case MODE_STEP_MACRO:
                pull_kernel<LBM_S, MODE_STEP_MACRO, VB, ROWS_INTERIOR><<<grid, block, 0, s>>>(a);
                break;
            case MODE_REDUCE: pull_kernel<LBM_S, MODE_REDUCE, VB, ROWS_INTERIOR><<<grid, block, 0, s>>>(a); break;
            case MODE_STEP_ADJ: pull_kernel<LBM_S, MODE_STEP_ADJ, VB, ROWS_INTERIOR><<<grid, block, 0, s>>>(a); break;
            default: return cudaErrorInvalidValue;
            }
        } else {
            switch (mode) {
            case MODE_STEP: pull_kernel<LBM_S, MODE_STEP, VB, ROWS_FACES><<<grid, block, 0, s>>>(a); break;
            case MODE_STEP_MACRO: pull_kernel<LBM_S, MODE_STEP_MACRO, VB, ROWS_FACES><<<grid, block, 0, s>>>(a); break;
            case MODE_REDUCE: pull_kernel<LBM_S, MODE_REDUCE, VB, ROWS_FACES><<<grid, block, 0, s>>>(a); break;
            case MODE_STEP_ADJ: pull_kernel<LBM_S, MODE_STEP_ADJ, VB, ROWS_FACES><<<grid, block, 0, s>>>(a); break;
            default: return cudaErrorInvalidValue;
            }
        }
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (nparts) *nparts = gi + gf;
    return cudaSuccess;
}

// One AA iteration (or reduction pass) of phase PHASE: interior rows, then
// face rows, as launch_direct.
template <int VB, int PHASE>
static cudaError_t launch_aa_phase(int mode, const StepArgs &a0, unsigned block, cudaStream_t s, unsigned *nparts)
{
    constexpr int V = VB / (int)sizeof(LBM_S);
    StepArgs a = a0;
    a.nvx = a0.dim / V;
    const size_t m = (size_t)(a.dim - 4);
    const unsigned gi = (unsigned)((m * m * (size_t)a.nvx + block - 1) / block);
    const unsigned gf = (unsigned)(((size_t)4 * (a.dim - 3) * (size_t)a.nvx + block - 1) / block);
    for (int pass = 0; pass < 2; ++pass) {
        const unsigned grid = pass == 0 ? gi : gf;
        if (grid == 0) continue;
        a.partial_base = pass == 0 ? 0u : gi;
        if (pass == 0) {
            switch (mode) {
            case MODE_STEP: aa_kernel<LBM_S, MODE_STEP, VB, ROWS_INTERIOR, PHASE><<<grid, block, 0, s>>>(a); break;
            case MODE_STEP_MACRO:
                aa_kernel<LBM_S, MODE_STEP_MACRO, VB, ROWS_INTERIOR, PHASE><<<grid, block, 0, s>>>(a);
                break;
            case MODE_REDUCE: aa_kernel<LBM_S, MODE_REDUCE, VB, ROWS_INTERIOR, PHASE><<<grid, block, 0, s>>>(a); break;
            default: return cudaErrorInvalidValue;
            }
        } else {
            switch (mode) {
            case MODE_STEP: aa_kernel<LBM_S, MODE_STEP, VB, ROWS_FACES, PHASE><<<grid, block, 0, s>>>(a); break;
            case MODE_STEP_MACRO:
                aa_kernel<LBM_S, MODE_STEP_MACRO, VB, ROWS_FACES, PHASE><<<grid, block, 0, s>>>(a);
                break;
            case MODE_REDUCE: aa_kernel<LBM_S, MODE_REDUCE, VB, ROWS_FACES, PHASE><<<grid, block, 0, s>>>(a); break;
            default: return cudaErrorInvalidValue;
            }
        }
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (nparts) *nparts = gi + gf;
    return cudaSuccess;
}

// AA variant: 8-byte vectors for FP32 (its fastest two-lattice width), 16-byte
// otherwise; a.aa_phase picks the A- or B-step.
cudaError_t LBM_CAT(launch_aa_, LBM_SFX)(int mode, const StepArgs &a, unsigned block, cudaStream_t s,
                                         unsigned *nparts)
{
    constexpr int VB = sizeof(LBM_S) == 4 ? 8 : 16;
    return a.aa_phase ? launch_aa_phase<VB, 1>(mode, a, block, s, nparts)
                      : launch_aa_phase<VB, 0>(mode, a, block, s, nparts);
}

cudaError_t LBM_CAT(launch_pull_, LBM_SFX)(int mode, const StepArgs &a, unsigned block, cudaStream_t s,
                                           unsigned *nparts)
{
    return launch_direct<16>(mode, a, block, s, nparts);
}

// One iteration (MODE_STEP or MODE_STEP_ADJ) of the direct variant (VB =
// 16) or the narrow one (VB = 8) with the face-row launch on stream sf, so
// that the two launches can run side by side.
cudaError_t LBM_CAT(launch_split_, LBM_SFX)(int vb, int mode, const StepArgs &a, unsigned block, cudaStream_t s,
                                            cudaStream_t sf)
{
    if (mode != MODE_STEP && mode != MODE_STEP_ADJ) return cudaErrorInvalidValue;
    if (vb == 16) return launch_direct<16>(mode, a, block, s, nullptr, 3, sf);
    if constexpr (sizeof(LBM_S) < 8) {
        if (vb == 8) return launch_direct<8>(mode, a, block, s, nullptr, 3, sf);
    }
    return cudaErrorInvalidValue;
}

cudaError_t LBM_CAT(launch_narrow_, LBM_SFX)(int mode, const StepArgs &a, unsigned block, cudaStream_t s)
{
    if constexpr (sizeof(LBM_S) < 8) {
        if (mode == MODE_REDUCE) return cudaErrorInvalidValue;
        return launch_direct<8>(mode, a, block, s, nullptr);
    } else {
        return cudaErrorInvalidValue;  // one double per 8 bytes: no narrow variant
    }
}

cudaError_t LBM_CAT(launch_staged_, LBM_SFX)(int mode, const StepArgs &a, unsigned grid, unsigned block,
                                             size_t smem, cudaStream_t s)
{
    if (grid == 0) return cudaSuccess;
    switch (mode) {
    case MODE_STEP: pull_staged_kernel<LBM_S, MODE_STEP><<<grid, block, smem, s>>>(a); break;
    case MODE_STEP_MACRO: pull_staged_kernel<LBM_S, MODE_STEP_MACRO><<<grid, block, smem, s>>>(a); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

const void *LBM_CAT(staged_kernel_ptr_, LBM_SFX)(int mode)
{
    switch (mode) {
    case MODE_STEP: return (const void *)pull_staged_kernel<LBM_S, MODE_STEP>;
    case MODE_STEP_MACRO: return (const void *)pull_staged_kernel<LBM_S, MODE_STEP_MACRO>;
    default: return nullptr;
    }
}

cudaError_t LBM_CAT(launch_init_, LBM_SFX)(const InitArgs &a, cudaStream_t s)
{
    const unsigned block = 256;
    // four consecutive x-sites per thread (dim % 4 == 0)
    const dim3 grid((unsigned)(((size_t)a.dim * a.dim / 4 + block - 1) / block), (unsigned)a.dim);
    init_kernel<LBM_S><<<grid, block, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || a.noise_sigma == 0.0 || a.dim < 5) return e;
    const size_t m = (size_t)(a.dim - 4);
    noise_kernel<LBM_S><<<dim3((unsigned)((m * m + block - 1) / block), (unsigned)m), block, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t LBM_CAT(launch_dump_, LBM_SFX)(const DumpArgs &a, cudaStream_t s)
{
    const unsigned block = 256;
    const size_t grid = (a.count + block - 1) / block;
    if (grid == 0) return cudaSuccess;
    dump_f_kernel<LBM_S, LBM_T><<<(unsigned)grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t LBM_CAT(launch_load_, LBM_SFX)(const DumpArgs &a, cudaStream_t s)
{
    const unsigned block = 256;
    const size_t grid = (a.count + block - 1) / block;
    if (grid == 0) return cudaSuccess;
    load_f_kernel<LBM_S, LBM_T><<<(unsigned)grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace lbm
