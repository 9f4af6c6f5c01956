/*
 * ref_shim.cpp -- compiles the reference's own OpenCL kernel source
 * (kernels.cl, active SCRATCH path) as host C++ so that the CPU oracle can be
 * pinned against it.  TEST INFRASTRUCTURE ONLY.
 *
 * Built by oracle/Makefile (target `ref`) straight from the reference tree
 * (REF=<path to the LBMCL checkout>, which holds kernels.cl and common.h);
 * nothing of the reference is copied into this repository.  Output goes to
 * oracle/_ref/ and is never committed.
 *
 * The OpenCL C keywords are mapped to nothing, get_global_id() reads a
 * per-thread index set by the loops over sites below, and the compile-time
 * macros the reference host passes with -D (lbmcl.hpp:131-156) become
 * run-time globals.  VELOCITY may additionally read a per-column lid array,
 * which is valid wherever the reference uses it because x and y are in scope
 * there (kernels.cl:284-293, 329-363).
 */
#include <cmath>
#include <cstddef>
#include <vector>

#if defined(FP_SINGLE)
typedef float shim_real;
#elif defined(FP_DOUBLE)
typedef double shim_real;
#else
#error "build with -DFP_SINGLE or -DFP_DOUBLE"
#endif

static int g_dim = 8;
static int g_sdiv = 0;
static int g_smod = 0;
static shim_real g_visc = 0;
static shim_real g_vel = 0;
static const shim_real *g_lid = nullptr;
static std::vector<shim_real> g_lid_store;
static thread_local int g_gid[3];

static inline int get_global_id(int d) { return g_gid[d]; }

#define DIM g_dim
#define LWS 1
#define STRIDE_DIV g_sdiv
#define STRIDE_MOD g_smod
#define VISCOSITY g_visc
#define VELOCITY (g_lid ? g_lid[(x) + (y) * g_dim] : g_vel)
#define __kernel static
#define __global
#define restrict __restrict__

#include "kernels.cl"

extern "C" {

void ref_configure(int dim, int stride_log2, double viscosity, double velocity, const double *lid)
{
    g_dim = dim;
    g_sdiv = stride_log2;
    g_smod = (1 << stride_log2) - 1;
    g_visc = (shim_real)viscosity;
    g_vel = (shim_real)velocity;
    if (lid) {
        g_lid_store.assign(lid, lid + (size_t)dim * dim);
        g_lid = g_lid_store.data();
    } else {
        g_lid = nullptr;
    }
}

void ref_initialize(real_t *f_stream, real_t *f_collide, real_t *density, real_t *u, int *map)
{
    for (int z = 0; z < g_dim; ++z)
        for (int y = 0; y < g_dim; ++y)
            for (int x = 0; x < g_dim; ++x) {
                g_gid[0] = x; g_gid[1] = y; g_gid[2] = z;
                initialize(f_stream, f_collide, density, u, map);
            }
}

// One reference step over the z-planes [z0, z1), the planes split over the
// OpenMP threads: every site pushes into distinct slots (kernels.cl:420-424),
// so the planes are independent; get_global_id reads a thread-local index.
void ref_compute_slab(real_t *f_stream, const real_t *f_collide, real_t *density, real_t *u,
                      const int *map, int update_macro, int z0, int z1)
{
#pragma omp parallel for schedule(static)
    for (int z = z0; z < z1; ++z)
        for (int y = 0; y < g_dim; ++y)
            for (int x = 0; x < g_dim; ++x) {
                g_gid[0] = x; g_gid[1] = y; g_gid[2] = z;
                compute(f_stream, f_collide, density, u, map, update_macro);
            }
}

void ref_compute(real_t *f_stream, const real_t *f_collide, real_t *density, real_t *u,
                 const int *map, int update_macro)
{
    ref_compute_slab(f_stream, f_collide, density, u, map, update_macro, 0, g_dim);
}

int ref_real_size(void) { return (int)sizeof(real_t); }

}  // extern "C"
