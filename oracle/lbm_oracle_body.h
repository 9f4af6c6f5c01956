/*
 * lbm_oracle_body.h -- precision-generic body of the CPU oracle.
 * Included twice by lbm_oracle.c with REAL = float / double and SFX(name)
 * appending _f32 / _f64.  TEST INFRASTRUCTURE ONLY (see lbm_oracle.h).
 *
 * Every arithmetic expression below keeps the reference's operand order
 * (kernels.cl), so that with -ffp-contract=off the results are bit-identical
 * to the reference kernel source compiled for the CPU.
 */

/* CSoA index of (site id, q) (kernels.cl:64). */
static inline size_t SFX(csoa)(size_t id, int q, int sd)
{
    const size_t smod = ((size_t)1 << sd) - 1;
    return ((((id >> sd) * (size_t)LBMO_Q) + (size_t)q) << sd) + (id & smod);
}

/* Lid u_x seen by column (x,y): the VELOCITY macro (kernels.cl:57), or the
 * optional per-column profile. */
static inline REAL SFX(lid_at)(const lbmo_params *p, int x, int y)
{
    if (p->lid) return (REAL)p->lid[(size_t)x + (size_t)y * (size_t)p->dim];
    return (REAL)p->velocity;
}

/* Equilibrium f_i = (rho w_i)(1 + 3 eu + 4.5 eu eu - 1.5 u2) with
 * eu = ux ex + uy ey + uz ez, in the reference's operand order
 * (kernels.cl:307-308, 396-397, 415-416). */
static inline REAL SFX(feq)(int i, REAL rho, REAL ux, REAL uy, REAL uz, REAL u2,
                            const REAL *w)
{
    const REAL eu = ((ux * (REAL)LBMO_EX[i]) + (uy * (REAL)LBMO_EY[i])) + (uz * (REAL)LBMO_EZ[i]);
    return (rho * w[i]) * ((((REAL)1.0 + ((REAL)3.0 * eu)) + (((REAL)4.5 * eu) * eu)) - ((REAL)1.5 * u2));
}

/* Lattice weights OMEGA_i (kernels.cl:110-128), evaluated in REAL as the
 * reference's single-precision-constant build does. */
static inline void SFX(weights)(REAL *w)
{
    for (int i = 0; i < LBMO_Q; ++i) {
        const int n2 = LBMO_EX[i] * LBMO_EX[i] + LBMO_EY[i] * LBMO_EY[i] + LBMO_EZ[i] * LBMO_EZ[i];
        w[i] = (n2 == 0) ? ((REAL)1.0 / (REAL)3.0)
             : (n2 == 1) ? ((REAL)1.0 / (REAL)18.0)
                         : ((REAL)1.0 / (REAL)36.0);
    }
}

void SFX(lbmo_init)(const lbmo_params *p, REAL *f_stream, REAL *f_collide,
                    REAL *rho, REAL *u, int *map)
{
    const int dim = p->dim;
    const int sd = p->stride_log2;
    const size_t n = (size_t)dim * dim * dim;
    REAL w[LBMO_Q];
    SFX(weights)(w);
    const REAL qnan = (REAL)NAN;

    /* kernels.cl:277-318 */
#pragma omp parallel for schedule(static) if (p->threads != 1) num_threads(p->threads > 0 ? p->threads : lbmo_max_threads())
    for (int z = 0; z < dim; ++z) {
        for (int y = 0; y < dim; ++y) {
            for (int x = 0; x < dim; ++x) {
                const size_t id = (size_t)x + (size_t)y * dim + (size_t)z * dim * dim;
                const int ct = lbmo_cell_type(dim, x, y, z);
                map[id] = ct;
                const REAL r0 = (REAL)1.0;
                const int mv = lbmo_is_moving_init(ct);
                const REAL ux = mv ? SFX(lid_at)(p, x, y) : (REAL)0.0;
                const REAL uy = (REAL)0.0;
                const REAL uz = (REAL)0.0;
                const int sm = lbmo_is_store_macro(ct);
                rho[id] = sm ? r0 : qnan;
                u[0 * n + id] = sm ? ux : qnan;
                u[1 * n + id] = sm ? uy : qnan;
                u[2 * n + id] = sm ? uz : qnan;
                const REAL u2 = ((ux * ux) + (uy * uy)) + (uz * uz);
                /* seeded perturbation of FLUID populations, both buffers:
                 * populations 2m and 2m+1 take the two samples of pair m */
                float z[LBMO_Q + 1];
                const int noisy = p->noise_sigma != 0.0 && ct == LBMO_FLUID;
                if (noisy)
                    for (int m = 0; m < (LBMO_Q + 1) / 2; ++m) lbmo_gauss_pairf(p->seed, id, (uint32_t)m, z + 2 * m);
                for (int i = 0; i < LBMO_Q; ++i) {
                    REAL fi = SFX(feq)(i, r0, ux, uy, uz, u2, w);
                    if (lbmo_is_wall(ct)) fi = qnan;
                    /* sigma z: a float product (sigma rounded to float) for
                     * FP32, a double product for FP64 */
                    if (noisy)
                        fi = fi + (sizeof(REAL) == 4 ? (REAL)((float)p->noise_sigma * z[i])
                                                     : (REAL)(p->noise_sigma * (double)z[i]));
                    f_collide[SFX(csoa)(id, i, sd)] = fi;
                    f_stream[SFX(csoa)(id, i, sd)] = fi;
                }
            }
        }
    }
}

void SFX(lbmo_compute)(const lbmo_params *p, REAL *f_stream, const REAL *f_collide,
                       REAL *rho, REAL *u, const int *map, int update_macro,
                       int z0, int z1)
{
    const int dim = p->dim;
    const int sd = p->stride_log2;
    const size_t n = (size_t)dim * dim * dim;
    REAL w[LBMO_Q];
    SFX(weights)(w);
    /* TAU and INV_TAU (kernels.cl:61-62), in REAL */
    const REAL tau = ((REAL)3.0 * (REAL)p->viscosity) + (REAL)0.5;
    const REAL inv_tau = (REAL)1.0 / tau;

#pragma omp parallel for schedule(static) if (p->threads != 1) num_threads(p->threads > 0 ? p->threads : lbmo_max_threads())
    for (int z = z0; z < z1; ++z) {
        for (int y = 0; y < dim; ++y) {
            for (int x = 0; x < dim; ++x) {
                const size_t id = (size_t)x + (size_t)y * dim + (size_t)z * dim * dim;
                const int ct = map[id];
                /* a WALL site computes nothing observable and never pushes
                 * (kernels.cl:421) */
                if (lbmo_is_wall(ct)) continue;

                REAL f[LBMO_Q];
                for (int i = 0; i < LBMO_Q; ++i) f[i] = f_collide[SFX(csoa)(id, i, sd)];

                /* moving lid: wall-sourced -z populations take their +z
                 * opposites (kernels.cl:343-349) */
                if (lbmo_is_moving(ct)) {
                    f[5] = f[6];
                    f[11] = f[17];
                    f[12] = f[18];
                    f[13] = f[15];
                    f[14] = f[16];
                }

                /* density, index order (kernels.cl:355), or the Sailfish
                 * order (kernels.cl:352-354) */
                REAL r;
                if (p->order == 1) {
                    r = f[5] + f[11] + f[12] + f[14] + f[13] + f[0] + f[1] + f[2] + f[7] + f[8] + f[4] +
                        f[10] + f[9] + f[6] + f[15] + f[16] + f[18] + f[17] + f[3];
                } else {
                    r = f[0];
                    for (int i = 1; i < LBMO_Q; ++i) r = r + f[i];
                }

                REAL ux, uy, uz;
                if (lbmo_is_moving(ct)) {
                    ux = SFX(lid_at)(p, x, y);
                    uy = (REAL)0.0;
                    uz = (REAL)0.0;
                } else if (p->order == 1) {
                    /* kernels.cl:368-375, left to right */
                    ux = (f[11] - f[13] + f[1] + f[7] - f[8] + f[10] - f[9] + f[15] - f[17] - f[3]) / r;
                    uy = (f[12] - f[14] + f[2] + f[7] + f[8] - f[4] - f[10] - f[9] + f[16] - f[18]) / r;
                    uz = (-f[5] - f[11] - f[12] - f[14] - f[13] + f[6] + f[15] + f[16] + f[18] + f[17]) / r;
                } else {
                    /* kernels.cl:376-378 */
                    ux = ((f[1] + f[7] + f[10] + f[11] + f[15]) - (f[3] + f[8] + f[9] + f[13] + f[17])) / r;
                    uy = ((f[2] + f[7] + f[8] + f[12] + f[16]) - (f[4] + f[9] + f[10] + f[14] + f[18])) / r;
                    uz = ((f[6] + f[15] + f[16] + f[17] + f[18]) - (f[5] + f[11] + f[12] + f[13] + f[14])) / r;
                }

                /* kernels.cl:383-388 */
                if (update_macro && lbmo_is_store_macro(ct)) {
                    rho[id] = r;
                    u[0 * n + id] = ux;
                    u[1 * n + id] = uy;
                    u[2 * n + id] = uz;
                }

                const REAL u2 = ((ux * ux) + (uy * uy)) + (uz * uz);

                if (lbmo_is_moving(ct)) {
                    /* lid equilibrium (kernels.cl:393-398) */
                    for (int i = 0; i < LBMO_Q; ++i) f[i] = SFX(feq)(i, r, ux, uy, uz, u2, w);
                } else if (lbmo_is_bounceback(ct)) {
                    /* full-way bounce-back of the 9 opposite pairs (kernels.cl:400-408) */
                    REAL g[LBMO_Q];
                    for (int i = 0; i < LBMO_Q; ++i) g[i] = f[LBMO_OPP[i]];
                    for (int i = 0; i < LBMO_Q; ++i) f[i] = g[i];
                }

                /* BGK (kernels.cl:270-273, 412-418) */
                if (lbmo_is_collision(ct)) {
                    for (int i = 0; i < LBMO_Q; ++i) {
                        const REAL fe = SFX(feq)(i, r, ux, uy, uz, u2, w);
                        f[i] = f[i] + inv_tau * (fe - f[i]);
                    }
                }

                /* push streaming (kernels.cl:420-424) */
                for (int i = 0; i < LBMO_Q; ++i) {
                    const size_t did = (size_t)(x + LBMO_EX[i]) + (size_t)(y + LBMO_EY[i]) * dim +
                                       (size_t)(z + LBMO_EZ[i]) * dim * dim;
                    f_stream[SFX(csoa)(did, i, sd)] = f[i];
                }
            }
        }
    }
}

double SFX(lbmo_run)(const lbmo_params *p, int first_it, int nsteps, int every,
                     REAL *fa, REAL *fb, REAL *rho, REAL *u, const int *map,
                     int *which)
{
    const double t0 = lbmo_now();
    REAL *cur = fa, *nxt = fb;
    for (int k = 0; k < nsteps; ++k) {
        const int it = first_it + k;
        const int upd = (every != 0 && it != 0 && (it % every) == 0) ? 1 : 0;
        SFX(lbmo_compute)(p, nxt, cur, rho, u, map, upd, 0, p->dim);
        REAL *t = cur; cur = nxt; nxt = t;
    }
    if (which) *which = (cur == fa) ? 0 : 1;
    return lbmo_now() - t0;
}
