/*
 * lbm.h -- C ABI of the GB300 (sm_103a) D3Q19 BGK lid-driven-cavity library.
 *
 * This is the drop-in boundary that replaces the reference's OpenCL kernel ABI
 * and its host plumbing:
 *   - initialize(f_stream, f_collide, density, u, map)      kernels.cl:277-282
 *   - compute(f_stream, f_collide, density, u, map, update)  kernels.cl:321-327
 *   - the -D macro set DIM/STRIDE/VISCOSITY/VELOCITY/FP_*     lbmcl.hpp:131-156
 *   - buffer creation and the ping-pong enqueue loop          lbmcl.hpp:392-521
 *   - the blocking read-backs behind the dumps                lbmcl.hpp:159-334
 *   - OpenCL event timing                                     lbmcl.hpp:548-620
 *
 * Conventions
 *   - Every function returns an lbm_status; nothing calls exit().  The text of
 *     the last failure on the calling thread is lbm_last_error().
 *   - A handle owns all device memory and one CUDA stream.  lbm_step is
 *     asynchronous on that stream; lbm_dump, lbm_load, lbm_sync, lbm_timing
 *     and lbm_reduce synchronise it.  Use one handle per host thread.
 *   - Every call on a handle runs on the handle's device (lbm_config.device)
 *     and leaves the caller's current device as it found it; lbm_init makes
 *     the handle's device current.
 *   - Host buffers passed in are caller-owned; the library never keeps them.
 *   - Iteration labels follow the reference host (lbmcl.hpp:435-520): after
 *     lbm_step has run t iterations in total, an F dump holds the buffer that
 *     iteration t wrote (what iteration t+1 would read), and the RHO / U
 *     dumps hold the moments last stored, i.e. those iteration k computed
 *     from its input when k was the last iteration with k % macro_every == 0.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_ABI_VERSION 1

typedef struct lbm_handle lbm_t;

/* Status codes. */
typedef enum lbm_status {
    LBM_OK = 0,
    LBM_EINVAL = 1,    /* bad argument: dim, sizes, NULL, unknown enum        */
    LBM_ENOMEM = 2,    /* device allocation failed or exceeds max_device_bytes */
    LBM_ECUDA = 3,     /* a CUDA runtime call failed (no device, launch error) */
    LBM_ESTATE = 4,    /* call not valid in the handle's current state         */
    LBM_EDIVERGED = 5, /* a site's density became <= 0 or NaN (lbm_sync)       */
    LBM_ETIMEOUT = 6   /* a kernel's bounded wait expired (staged iteration
                          kernel, two-step adjoint): the handle's results are
                          not valid; the flag stays set on the handle        */
} lbm_status;

/* Population storage.  FP32/FP64 reproduce the reference's float / double
 * builds (-F, lbm_options.hpp:214-216).  FP16/BF16 store the deviation
 * f_i - w_i in 16 bits and do all arithmetic in FP32. */
typedef enum lbm_precision {
    LBM_FP32 = 0,
    LBM_FP64 = 1,
    LBM_FP16 = 2,
    LBM_BF16 = 3
} lbm_precision;

/* What lbm_dump copies out / lbm_load copies in. */
typedef enum lbm_what {
    LBM_DUMP_F = 0,       /* populations, CSoA with the handle's stride (kernels.cl:64);
                             float (FP32/FP16/BF16 handles) or double (FP64): dim^3*19 values */
    LBM_DUMP_RHO = 1,     /* density, dim^3 values of the macro type                      */
    LBM_DUMP_U = 2,       /* velocity, planar ux,uy,uz: 3*dim^3 values (kernels.cl:68-70) */
    LBM_DUMP_MAP = 3,     /* reference cell types as int32 (common.h:7-20): dim^3 values  */
    LBM_DUMP_MAP_U8 = 4,  /* the packed byte map the kernels read: dim^3 bytes            */
    LBM_DUMP_F_RAW = 5    /* the raw internal population buffer (binary checkpoint); the
                             slots of wall sites hold unspecified values                  */
} lbm_what;

typedef struct lbm_config {
    int dim;                   /* cube edge incl. the wall layer (DIM); >= 4, multiple of 8
                                  for FP16/BF16, of 4 otherwise                             */
    double viscosity;          /* nu; tau = 3 nu + 0.5 (kernels.cl:61)                      */
    double velocity;           /* lid u_x along +x (VELOCITY, kernels.cl:57)                */
    int precision;             /* lbm_precision                                             */
    int stride;                /* CSoA stride of F dumps (-s); power of two <= dim^3;
                                  0 means dim^3 (pure SoA)                                  */
    int block_threads;         /* CUDA threads per block (from -w); 0 = tuned default       */
    uint64_t seed;             /* noise seed                                                */
    double noise_sigma;        /* std-dev of the N(0, sigma^2) noise added to every
                                  population of FLUID sites after initialisation; 0 = none;
                                  sigma z is a float product (sigma rounded to float) for
                                  FP32 and 16-bit storage, a double product for FP64     */
    const double *lid_profile; /* optional host array dim*dim: lid u_x of column (x,y)
                                  at lid_profile[x + y*dim]; NULL = velocity everywhere    */
    double tau;                /* > 0 overrides the viscosity                               */
    size_t max_device_bytes;   /* > 0: refuse (LBM_ENOMEM) when the handle would need
                                  more device memory than this                              */
    int device;                /* CUDA device ordinal                                       */
    int profile_steps;         /* 1: one CUDA event pair per iteration (reference's
                                  per-kernel events); 0: one pair per lbm_step call         */
    int kernel;                /* lbm_kernel: iteration kernel variant; 0 = the tuned default
                                  (NARROW for FP32, DIRECT otherwise)                       */
    int stages;                /* TMA-staged kernel: pipeline depth (0 = tuned default)    */
    int adjoint_steps;         /* adjoint steps per launch of the backward sweep: 0 = tuned
                                  default (2 for the FP32 adjoint on lattices that fill the
                                  GPU, about 128^3 and up; else 1), 1, or 2 (FP32 adjoint,
                                  dim <= 609)                                               */
    int adjoint_max_states;    /* > 0: at most this many recomputed state buffers in the
                                  backward sweep (fewer than checkpoint_every - 1 makes it
                                  checkpoint segments recursively); 0 = as many as fit     */
    int graph_iterations;      /* lbm_step replays runs of this many plain iterations as
                                  one captured CUDA graph (launch-bound small lattices);
                                  0 = default 16, 1 = launch every kernel directly; an
                                  even number, at most 256                                  */
    int adjoint_full_states;   /* backward sweep without a tau gradient: 0 = recompute each
                                  segment storing only the adjoint's linearisation point
                                  per iteration (u of FLUID sites, rho of lid sites: 3
                                  planes); 1 = store the full states, as with a tau
                                  gradient                                                  */
    int adjoint_fp64;          /* 1: the adjoint in FP64 arithmetic for FP32 / FP16 / BF16
                                  storage too (one step per launch), e.g. to measure the
                                  FP32 adjoint's rounding on the same trajectory; 0: FP64
                                  only for FP64 storage                                     */
    int order;                 /* summation order of rho and u (FP32 / FP64 storage):
                                  LBM_ORDER_REFERENCE (the reference's active order,
                                  kernels.cl:355, 376-378) or LBM_ORDER_SAILFISH (its
                                  compiled-out Sailfish order, kernels.cl:352-354,
                                  368-375); the gradient calls need the reference order   */
    int adjoint_kernel;        /* data movement of the FP32 adjoint's two-step kernel in
                                  the stored-point sweep: 0 = tuned default (DIRECT),
                                  LBM_KERNEL_DIRECT = per-thread loads from HBM,
                                  LBM_KERNEL_STAGED = each plane's inputs staged in shared
                                  memory by tiled TMA loads (dim % 4 == 0); the same
                                  per-site arithmetic                                      */
    int adjoint_tail_segments; /* lbm_adjoint_forward also records the linearisation
                                  points of its last checkpoint segments, so that a backward
                                  sweep without a tau gradient does not recompute them:
                                  0 = as many segments as fit in the device memory left
                                  beyond what the sweep itself needs, n > 0 = at most n,
                                  -1 = none; the gradients are the same bit for bit       */
} lbm_config;

/* Iteration kernel variants (same results, different data movement). */
typedef enum lbm_kernel {
    LBM_KERNEL_AUTO = 0,
    LBM_KERNEL_DIRECT = 1,   /* per-thread 16-byte vector loads straight from HBM        */
    LBM_KERNEL_STAGED = 2,   /* persistent CTAs; whole source rows staged in shared
                                memory by cp.async.bulk (TMA) through an mbarrier ring   */
    LBM_KERNEL_NARROW = 3,   /* as DIRECT with 8-byte vectors (fewer registers)          */
    LBM_KERNEL_AA = 4        /* one lattice updated in place, alternating a local step and
                                a neighbour step (AA pattern): half the population memory;
                                LBM_DUMP_F_RAW then holds the current step's layout, and
                                the lbm_adjoint_* calls are not available                 */
} lbm_kernel;

/* Summation orders of rho and u (lbm_config.order). */
typedef enum lbm_order {
    LBM_ORDER_REFERENCE = 0, /* kernels.cl:355, 376-378 (the reference's active path)   */
    LBM_ORDER_SAILFISH = 1   /* kernels.cl:352-354, 368-375 (CALCULATION_ORDER_SAILFISH) */
} lbm_order;

/* Fill *c with the reference CLI defaults (lbm_options.hpp:83-101):
 * dim 8, nu 0.0089, u 0.05, FP32, stride 32. */
void lbm_config_default(lbm_config *c);

/* Allocate the lattice and run the initialisation kernel (replaces
 * kernels.cl:277-318 + lbmcl.hpp:392-482, 494-498). */
int lbm_init(lbm_t **h, const lbm_config *c);

/* Enqueue nsteps iterations (replaces kernels.cl:321-425 + lbmcl.hpp:505-511).
 * Iteration it (1-based, counted over the handle's life) stores rho and u
 * when macro_every != 0 && it % macro_every == 0 (lbmcl.hpp:436). */
int lbm_step(lbm_t *h, int nsteps, int macro_every);

/* Copy `what` into the caller's host buffer dst of `bytes` bytes (must be
 * exactly the size of that quantity).  Synchronous. */
int lbm_dump(lbm_t *h, int what, void *dst, size_t bytes);

/* Replace the populations by a host array in the LBM_DUMP_F layout (or
 * LBM_DUMP_F_RAW).  The slots whose source is a wall keep the reference's
 * fixed values.  Synchronous. */
int lbm_load(lbm_t *h, int what, const void *src, size_t bytes);

/* Byte size of `what` for this handle (0 for an unknown `what`). */
size_t lbm_size(const lbm_t *h, int what);

/* Wait for the stream; LBM_EDIVERGED once a non-finite or non-positive
 * density has been seen by a kernel. */
int lbm_sync(lbm_t *h);

/* Elapsed times, milliseconds: total = from the initialisation kernel's start
 * to the end of the last enqueued work (lbmcl.hpp:548-556); kernels = sum of
 * step-kernel time (lbmcl.hpp:562-574). */
int lbm_timing(lbm_t *h, double *total_ms, double *kernels_ms);

/* Iterations run so far. */
int lbm_iteration(const lbm_t *h, int64_t *it);

/* Name of the CUDA device the handle runs on (replaces the CL_DEVICE_NAME
 * query of lbmcl.hpp:626 and lbmcl.hpp:651). */
const char *lbm_device_name(const lbm_t *h);

/* The handle's CUDA stream (cudaStream_t), for callers that time or order
 * their own work against it.  (Iterations may run their face-row launches
 * on a second internal stream; that work is always joined back into this
 * stream, so ordering against it orders against everything the handle
 * enqueued.) */
void *lbm_stream(lbm_t *h);

/* FP64 sums over the sites that store macros (FLUID and MOVING) of the
 * current state (what the next iteration would read): out[0] = mass
 * sum(rho), out[1] = kinetic energy sum(rho |u|^2 / 2), out[2] = number of
 * such sites.  Moments as kernels.cl:352-380 defines them.  Synchronous. */
int lbm_reduce(lbm_t *h, double out[3]);

/* ---------------------------------------------------------------------------
 * Gradients (new; the reference has no adjoint).
 *
 * Loss: J = mean over the FLUID sites of the plane y = plane_y of
 * (u_x - target(x, z))^2, u_x the velocity of the buffer the next iteration
 * would read (the post-stream state R_T after T iterations).  Controls: the
 * per-column lid velocity, tau, and the initial populations R_0 (the state
 * the adjoint forward starts from, in the LBM_DUMP_F layout).
 * ------------------------------------------------------------------------- */

/* Set the loss plane (2 <= plane_y <= dim-3) and the u_x target,
 * target_ux[x + z*dim] (NULL: zero). */
int lbm_adjoint_set_loss(lbm_t *h, int plane_y, const double *target_ux);

/* Run `iterations` iterations from the current state (as lbm_step without
 * macro output), keeping a checkpoint of the state every `checkpoint_every`
 * iterations (1 = the whole trajectory), and return the loss of the final
 * state.  Device memory: ceil(iterations / checkpoint_every) states here,
 * checkpoint_every - 1 more on the first lbm_adjoint_backward.  Synchronous. */
int lbm_adjoint_forward(lbm_t *h, int iterations, int checkpoint_every, double *loss);

/* Backward sweep of the last lbm_adjoint_forward, scaled by dloss (dL/dJ for
 * a caller's outer loss L): hand-written adjoint kernels, each checkpoint
 * segment recomputed with the forward kernel.  Without grad_tau the segments
 * are recomputed storing only the velocity (FLUID) and density (lid sites) of
 * each iteration, which is all the adjoint of the lid and of the initial
 * populations needs (lbm_config.adjoint_full_states).  Any output may be NULL:
 *   grad_tau   dL/dtau
 *   grad_lid   dim*dim doubles, dL/dlid at [x + y*dim]
 *   grad_f0    dL/dR_0 in the LBM_DUMP_F layout and type (grad_f0_bytes =
 *              lbm_size(h, LBM_DUMP_F)); when R_0 is the state lbm_init made,
 *              its dependence on the lid is included in grad_lid.
 * Adjoint arithmetic: FP64 for an FP64 handle or with adjoint_fp64, FP32
 * otherwise.  Synchronous. */
int lbm_adjoint_backward(lbm_t *h, double dloss, double *grad_tau, double *grad_lid, void *grad_f0,
                         size_t grad_f0_bytes);

void lbm_destroy(lbm_t *h);

const char *lbm_last_error(void);

/* ---------------------------------------------------------------------------
 * lbm_reduce_noalloc -- no counterpart in the reference.
 *
 * The sums of lbm_reduce (out[0] mass, out[1] kinetic energy, out[2] number
 * of FLUID and MOVING sites) for a lattice state held in the caller's own
 * device memory, computed without allocating anything.  It is meant for
 * callers that cannot call cudaMalloc: processes whose device memory belongs
 * to another allocator (a framework's caching pool, a fixed arena sized once
 * at start-up in a real-time loop), or whose device memory is already fully
 * committed, so that a further cudaMalloc would fail or would bypass the
 * owner's accounting.  Such callers cannot create a handle (lbm_init
 * allocates) but can pass pointers to buffers they own.
 *
 *   f      the populations in the LBM_DUMP_F_RAW layout of `precision`
 *          (19 planes of dim^3 storage elements; the post-collision state
 *          a handle holds after its last iteration); 16-byte aligned
 *   map    the byte map (LBM_DUMP_MAP_U8), dim^3 bytes; aligned to 16 /
 *          (storage element size) bytes (4 for FP32, 2 for FP64, 8 for
 *          FP16 / BF16)
 *   lid    the lid u_x of each column, dim*dim values of the macro type
 *          (double for LBM_FP64, float otherwise), aligned to that type
 *   stream cudaStream_t to run on (NULL: the legacy default stream); the call
 *          returns after the stream has finished the reduction
 * All three buffers must be on the calling thread's current device.  A
 * misaligned pointer is rejected with LBM_EINVAL before anything runs.
 *
 * The block partial sums live in one fixed __device__ array of
 * LBM_NOALLOC_SCRATCH_BYTES (32 KiB + 32 B) that every GPU which loads the
 * library holds until the process exits; a launch uses at most
 * LBM_NOALLOC_MAX_BLOCKS blocks per row kind so the partials always fit, and
 * dim is limited to LBM_NOALLOC_MAX_DIM (larger: LBM_EINVAL).  The first call
 * on a device looks up that array's device address (cudaGetSymbolAddress)
 * with the device current and keeps it for the life of the process, so the
 * entry point must not be used on a device after cudaDeviceReset there.
 * Every call reuses the same array, which keeps the last call's contents (the
 * status word is cleared at the start of each call), so calls that overlap on
 * the GPU -- on different streams, or from several host threads -- race and
 * must be serialised by the caller.  Returns LBM_EDIVERGED (with out filled)
 * when a density <= 0 or NaN was seen.
 * ------------------------------------------------------------------------- */
#define LBM_NOALLOC_MAX_BLOCKS 1024
#define LBM_NOALLOC_MAX_DIM 2048
#define LBM_NOALLOC_SCRATCH_BYTES ((4 * LBM_NOALLOC_MAX_BLOCKS + 4) * 8)
int lbm_reduce_noalloc(const void *f, const uint8_t *map, const void *lid, int dim, int precision, void *stream,
                       double out[3]);

#ifdef __cplusplus
}
#endif
#endif
