/*
 * lbm_oracle.h -- CPU oracle for LBMCL's D3Q19 BGK lid-driven-cavity step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: only the tests, the
 * smoke check and the CPU-baseline leg of bench.py load it.  The product
 * library (liblbm_gb300.so) never links or calls it, and nothing here is a
 * fallback for the CUDA path.
 *
 * It restates, in plain C, the active ("SCRATCH") path of the reference's
 * kernels.cl in the reference's own push formulation and operation order:
 *   - cell typing           kernels.cl:236-266, common.h:7-66
 *   - initialize            kernels.cl:277-318
 *   - compute (one step)    kernels.cl:321-425
 *   - CSoA index            kernels.cl:64-67, lbmcl.hpp:19
 *   - host ping-pong order  lbmcl.hpp:435-467, lbmcl.hpp:505-520
 * Three run-time extensions that the reference does not have are added in the
 * same place the reference's compile-time macros sit: the relaxation time and
 * lid velocity are run-time values (kernels.cl:57,61 take them as -D macros),
 * the lid velocity may vary per (x,y) column, and seeded Gaussian noise may be
 * added to the populations of FLUID sites after initialisation.
 *
 * Precision: every function exists as _f32 (float) and _f64 (double).  Build
 * with -ffp-contract=off and without -ffast-math so that each + - * / is one
 * IEEE operation, as in the reference run without -cl-fast-relaxed-math.
 */
#ifndef LBM_ORACLE_H
#define LBM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Cell-type flags, same values as the reference (common.h:7-20). */
#define LBMO_NONE   0x000
#define LBMO_FLUID  0x001
#define LBMO_MOVING 0x002
#define LBMO_CORNER 0x004
#define LBMO_WALL   0x008
#define LBMO_LEFT   0x010
#define LBMO_RIGHT  0x020
#define LBMO_TOP    0x040
#define LBMO_BOTTOM 0x080
#define LBMO_FRONT  0x100
#define LBMO_BACK   0x200

typedef struct lbmo_params {
    int dim;                 /* cube edge including the wall layer (DIM)         */
    int stride_log2;         /* CSoA stride = 1 << stride_log2 (STRIDE_DIV)      */
    double viscosity;        /* nu; tau = 3 nu + 0.5 evaluated in the precision  */
    double velocity;         /* lid u_x (VELOCITY), used when lid == NULL        */
    const double *lid;       /* optional per-column lid u_x, lid[x + y*dim]      */
    uint64_t seed;           /* noise seed                                        */
    double noise_sigma;      /* 0: no noise; FP32 adds (float)sigma * z in float,
                              * FP64 adds sigma * z in double                    */
    int threads;             /* OpenMP threads, 0: runtime default                */
    int order;               /* 0: the reference's summation order of rho and u
                              * (kernels.cl:355, 376-378); 1: its compiled-out
                              * Sailfish order (kernels.cl:352-354, 368-375)    */
} lbmo_params;

/* Reference cell type of site (x,y,z) (kernels.cl:236-266). */
int lbmo_cell_type(int dim, int x, int y, int z);

/* Standard normal sample for (seed, site, q): Philox4x32-10 counter stream,
 * Box-Muller transform (block g of a site gives pairs 2g and 2g+1:
 * populations 4g .. 4g+3), a self-contained natural logarithm, sine and
 * cosine.  Computed with IEEE single-precision + - * / sqrt only, so the GPU
 * library reproduces it bit for bit.  lbmo_gauss returns the same value
 * widened to double; lbmo_gauss_pairf gives both samples of one pair. */
void lbmo_gauss_pairf(uint64_t seed, uint64_t site, uint32_t pair, float z[2]);
float lbmo_gaussf(uint64_t seed, uint64_t site, uint32_t q);
double lbmo_gauss(uint64_t seed, uint64_t site, uint32_t q);

/* Philox4x32-10 block (Salmon et al., SC'11), exposed for known-answer tests. */
void lbmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Natural logarithm used by lbmo_gaussf (x > 0, finite); lbmo_log widens it. */
float lbmo_logf(float x);
double lbmo_log(double x);

/* initialize (kernels.cl:277-318), then noise on FLUID sites of both buffers. */
void lbmo_init_f32(const lbmo_params *p, float *f_stream, float *f_collide,
                   float *rho, float *u, int *map);
void lbmo_init_f64(const lbmo_params *p, double *f_stream, double *f_collide,
                   double *rho, double *u, int *map);

/* compute (kernels.cl:321-425) over the z-planes [z0, z1): reads f_collide,
 * pushes into f_stream.  z0 = 0, z1 = dim is the whole lattice. */
void lbmo_compute_f32(const lbmo_params *p, float *f_stream, const float *f_collide,
                      float *rho, float *u, const int *map, int update_macro,
                      int z0, int z1);
void lbmo_compute_f64(const lbmo_params *p, double *f_stream, const double *f_collide,
                      double *rho, double *u, const int *map, int update_macro,
                      int z0, int z1);

/* The host loop of lbmcl.hpp:505-520 for iterations 1..n (no file output):
 * step `it` reads the buffer the previous step wrote, update_macro =
 * (every != 0 && it % every == 0).  On return *which = 0 if the newest state
 * is in fa (the initial f_collide), 1 if in fb.  Returns wall seconds of the
 * step loop. */
double lbmo_run_f32(const lbmo_params *p, int first_it, int n, int every,
                    float *fa, float *fb, float *rho, float *u, const int *map,
                    int *which);
double lbmo_run_f64(const lbmo_params *p, int first_it, int n, int every,
                    double *fa, double *fb, double *rho, double *u, const int *map,
                    int *which);

/* Number of OpenMP threads a parallel region would use (1 without OpenMP). */
int lbmo_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
