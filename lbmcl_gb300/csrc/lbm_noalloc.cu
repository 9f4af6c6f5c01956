// lbm_noalloc.cu -- lbm_reduce_noalloc: mass and kinetic energy of a lattice
// state that lives in the caller's own device memory, computed without any
// device allocation.
//
// Why: some callers cannot call cudaMalloc -- processes whose device memory
// is owned by another allocator (a framework's caching pool, a fixed arena
// sized once at start-up in a real-time loop) or that have already committed
// all of it, so a further cudaMalloc would fail or escape the owner's
// accounting.  They can still hand this library device pointers to buffers
// they own.
//
// How: the block partial sums that lbm_reduce keeps in a handle-owned buffer
// live here in one file-scope __device__ array of fixed size, which every GPU
// that loads the library holds until the process exits.  A grid-stride
// variant of the reduction kernel caps the number of blocks per launch so the
// partials always fit.  On the first call on a device, with that device
// current, the host looks up the array's device address once with
// cudaGetSymbolAddress and passes it to the kernels; the host-side symbol is
// only a stand-in and is never handed to a kernel.  The address is kept for
// the life of the process (a cudaDeviceReset would invalidate it).
#include <algorithm>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "lbm.h"
#include "lbm_kernels.cuh"
#include "lbm_launch.h"

namespace {

constexpr unsigned kBlocks = LBM_NOALLOC_MAX_BLOCKS;  // per launch (interior rows, face rows)
constexpr unsigned kThreads = 256;
constexpr int kMaxDevices = 64;

// Layout: [0, 4*kBlocks) block partials (mass, energy) of the two launches,
// then the two final sums, then the status word (as a double slot).
constexpr size_t kSumSlot = 4 * (size_t)kBlocks;
constexpr size_t kStatusSlot = kSumSlot + 2;
constexpr size_t kScratchDoubles = kStatusSlot + 2;
static_assert(kScratchDoubles * sizeof(double) == LBM_NOALLOC_SCRATCH_BYTES, "scratch size stated in lbm.h");

static __device__ __align__(256) double g_reduce_scratch[kScratchDoubles];

std::mutex g_setup_mu;
double *g_scratch_ptr[kMaxDevices] = {};

// failures are reported through lbm_last_error(), like every other entry point
int fail(int code, const char *fmt, ...)
{
    char buf[400];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    lbm::set_last_error(buf);
    return code;
}

// Grid-stride reduction over the rows of one kind (see pull_kernel): each
// block accumulates any number of vectors and writes one partial pair.
template <class S, int ROWS>
__global__ void __launch_bounds__(kThreads) reduce_noalloc_kernel(lbm::StepArgs a)
{
    constexpr int V = 16 / (int)sizeof(S);
    const int dim = a.dim;
    const size_t nrows = ROWS == lbm::ROWS_INTERIOR ? (size_t)(dim - 4) * (size_t)(dim - 4) : 4 * (size_t)(dim - 3);
    const size_t total = nrows * (size_t)a.nvx;
    double m = 0.0, e = 0.0;
    for (size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
        const size_t row = g / (size_t)a.nvx;
        const int xv = (int)(g - row * (size_t)a.nvx);
        int y, z;
        if (ROWS == lbm::ROWS_INTERIOR) {
            y = 2 + (int)(row % (size_t)(dim - 4));
            z = 2 + (int)(row / (size_t)(dim - 4));
        } else {
            lbm::decode_face_row(dim, (unsigned)row, y, z);
        }
        lbm::pull_vector<S, lbm::MODE_REDUCE, V, ROWS == lbm::ROWS_INTERIOR>(a, xv, y, z, m, e);
    }
    lbm::block_reduce_write(m, e, a.partials + 2 * (size_t)a.partial_base);
}

__global__ void sum_noalloc_kernel(const double *__restrict__ partials, int nblocks, double *__restrict__ out)
{
    double m = 0.0, e = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        m += partials[2 * i];
        e += partials[2 * i + 1];
    }
    __shared__ double sm[2][kThreads];
    sm[0][threadIdx.x] = m;
    sm[1][threadIdx.x] = e;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sm[0][threadIdx.x] += sm[0][threadIdx.x + w];
            sm[1][threadIdx.x] += sm[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sm[0][0];
        out[1] = sm[1][0];
    }
}

template <class S>
cudaError_t launch_reduce(const lbm::StepArgs &a0, cudaStream_t s, unsigned *nparts)
{
    lbm::StepArgs a = a0;
    const size_t ni = (size_t)(a.dim - 4) * (size_t)(a.dim - 4) * (size_t)a.nvx;
    const size_t nf = 4 * (size_t)(a.dim - 3) * (size_t)a.nvx;
    const unsigned gi = (unsigned)std::min<size_t>(kBlocks, (ni + kThreads - 1) / kThreads);
    const unsigned gf = (unsigned)std::min<size_t>(kBlocks, (nf + kThreads - 1) / kThreads);
    if (gi > 0) {
        a.partial_base = 0;
        reduce_noalloc_kernel<S, lbm::ROWS_INTERIOR><<<gi, kThreads, 0, s>>>(a);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (gf > 0) {
        a.partial_base = gi;
        reduce_noalloc_kernel<S, lbm::ROWS_FACES><<<gf, kThreads, 0, s>>>(a);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    *nparts = gi + gf;
    return cudaSuccess;
}

}  // namespace

extern "C" int lbm_reduce_noalloc(const void *f, const uint8_t *map, const void *lid, int dim, int precision,
                                  void *stream, double out[3])
{
    if (!f || !map || !lid || !out) return fail(LBM_EINVAL, "lbm_reduce_noalloc: NULL argument");
    if (precision < LBM_FP32 || precision > LBM_BF16)
        return fail(LBM_EINVAL, "lbm_reduce_noalloc: unknown precision %d", precision);
    const int mult = (precision == LBM_FP16 || precision == LBM_BF16) ? 8 : 4;
    if (dim < 4 || dim % mult != 0 || dim > LBM_NOALLOC_MAX_DIM)
        return fail(LBM_EINVAL,
                    "lbm_reduce_noalloc: dim %d must be in [4, %d] and a multiple of %d for this precision", dim,
                    LBM_NOALLOC_MAX_DIM, mult);
    // the kernels read f with 16-byte vectors, the map in words of one byte
    // per site of a vector, the lid as the macro type: a misaligned pointer
    // (an offset view into a pool) would fault the caller's context
    const size_t sb = precision == LBM_FP64 ? 8 : (precision == LBM_FP32 ? 4 : 2);
    const size_t map_align = 16 / sb, lid_align = precision == LBM_FP64 ? 8 : 4;
    if ((uintptr_t)f % 16 != 0 || (uintptr_t)map % map_align != 0 || (uintptr_t)lid % lid_align != 0)
        return fail(LBM_EINVAL,
                    "lbm_reduce_noalloc: misaligned buffer (f needs 16-byte, map %zu-byte, lid %zu-byte alignment)",
                    map_align, lid_align);

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(LBM_ECUDA, "lbm_reduce_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(LBM_EINVAL, "lbm_reduce_noalloc: device %d not supported", dev);
    double *scratch = nullptr;
    {
        // once per device, with that device current
        std::lock_guard<std::mutex> lock(g_setup_mu);
        if (!g_scratch_ptr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_reduce_scratch);
            if (e != cudaSuccess)
                return fail(LBM_ECUDA, "lbm_reduce_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            g_scratch_ptr[dev] = static_cast<double *>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int *status = reinterpret_cast<int *>(scratch + kStatusSlot);

    lbm::StepArgs a = {};
    a.fin = f;
    a.fout = nullptr;
    a.map = map;
    a.lid = lid;
    a.status = status;
    a.partials = scratch;
    a.dim = dim;
    a.nvx = dim / (int)(16 / sb);
    a.n = (size_t)dim * dim * dim;

    // the status word keeps the previous call's value: clear it
    e = cudaMemsetAsync(status, 0, sizeof(int), s);
    if (e != cudaSuccess) return fail(LBM_ECUDA, "lbm_reduce_noalloc: cudaMemsetAsync: %s", cudaGetErrorString(e));
    unsigned nparts = 0;
    switch (precision) {
    case LBM_FP32: e = launch_reduce<float>(a, s, &nparts); break;
    case LBM_FP64: e = launch_reduce<double>(a, s, &nparts); break;
    case LBM_FP16: e = launch_reduce<__half>(a, s, &nparts); break;
    default: e = launch_reduce<__nv_bfloat16>(a, s, &nparts); break;
    }
    if (e != cudaSuccess) return fail(LBM_ECUDA, "lbm_reduce_noalloc: launch: %s", cudaGetErrorString(e));
    sum_noalloc_kernel<<<1, kThreads, 0, s>>>(scratch, (int)nparts, scratch + kSumSlot);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(LBM_ECUDA, "lbm_reduce_noalloc: launch: %s", cudaGetErrorString(e));
    double sums[2];
    int st = 0;
    e = cudaMemcpyAsync(sums, scratch + kSumSlot, sizeof sums, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, status, sizeof st, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(LBM_ECUDA, "lbm_reduce_noalloc: %s", cudaGetErrorString(e));
    const double d4 = (double)(dim - 4);
    out[0] = sums[0];
    out[1] = sums[1];
    out[2] = d4 * d4 * d4 + d4 * d4;
    if (st & 1) return fail(LBM_EDIVERGED, "lbm_reduce_noalloc: a density <= 0 or NaN was seen");
    return LBM_OK;
}
