/*
 * droplet_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A CPU FP64 restatement, in C with OpenMP, of one time step of the
 * reference's D3Q15 two-phase (Inamuro free-energy) lattice-Boltzmann droplet
 * code. It is the parity checker for the GPU library and the timed CPU
 * baseline; nothing in the product path links or loads it.
 *
 * Statement-by-statement source (reference paths relative to its root):
 *   par / constants ............ program/lbm_drop_xy.f90:70-84, 117-129
 *   ini (f<-feq, g<-geq) ....... program/lbm_drop_xy.f90:244-251
 *   ini_op (tau_g from phi1,phi2) program/lbm_drop_xy.f90:254-285
 *   various_cal ................ program/lbm_drop_xy.f90:590-640
 *   gphi_cal ................... program/lbm_drop_xy.f90:642-666
 *   equilibrium_cal ............ program/lbm_drop_xy.f90:421-476
 *   fg_cal ..................... program/lbm_drop_xy.f90:478-515
 *   physics .................... program/lbm_drop_xy.f90:517-588
 *   spectral externalforce ..... program/lbm_drop_iht_xy.f90:722-842, 894-926
 *   Smagorinsky tau_g .......... program/LES_drop_xy.f90:481-502, 655-690
 *   moving-wall bounce-back .... prototype_program/two-phase/drop8_mpi.f90:642-674
 *
 * Fidelity rules. Every expression is evaluated in the reference's
 * left-to-right Fortran order with the same parenthesisation, x**2 as x*x,
 * divisions kept as divisions, and the i = 1..15 accumulation order; the
 * file is compiled with -ffp-contract=off so no multiply-add is fused.
 * Deliberate differences, each a property of running on one resident domain:
 *   - halo exchange (glue, glue_f) becomes periodic index wrap;
 *   - the LES strain is taken from current periodic neighbours (the
 *     reference reads halos that are one step old at rank faces,
 *     program/LES_drop_xy.f90:661);
 *   - (2 S:S)**0.5 is evaluated with sqrt;
 *   - both walls are applied (the reference's if / else-if skips the top
 *     wall when a single rank holds the whole z range, drop8_mpi.f90:651,662);
 *   - the spectral force uses an exact DFT restricted to the forced band
 *     instead of 2decomp_fft 1.5.847 over FFTW 3.3.8 (equal up to rounding),
 *     and |u_hat|^2 is re^2 + im^2 rather than abs(u_hat)**2 (the reference
 *     squares a hypot; the two differ in the last bit at most).
 * tau_g is recomputed at the start of each step from the current phi, u and
 * the stored phi min/max; this gives the same numbers the reference's physics
 * (end of the previous step) and ini_op (first step) store.
 *
 * Parity status: the reference ships no tests, golden vectors or stored
 * outputs, and it cannot be built here (Fortran + MPI + 2decomp_fft), so this
 * restatement is pinned by an independent NumPy restatement (bitwise on small
 * grids), by physical known answers (conservation, Couette, Taylor-Green
 * decay, Laplace law) and by an FFT cross-check of the forcing.
 */
#include "droplet_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* D3Q15 velocities and weights, program/lbm_drop_xy.f90:70-84 */
static const int CX[15] = {0, 1, 0, 0, -1, 0, 0, 1, -1, 1, 1, -1, 1, -1, -1};
static const int CY[15] = {0, 0, 1, 0, 0, -1, 0, 1, 1, -1, 1, -1, -1, 1, -1};
static const int CZ[15] = {0, 0, 0, 1, 0, 0, -1, 1, 1, 1, -1, -1, -1, -1, 1};
static const double EW[15] = {2.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,
                              1.0 / 9.0,  1.0 / 9.0,  1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0,
                              1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0};
static const double HW[15] = {1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
                              0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
static const double FW[15] = {-7.0 / 3.0, 1.0 / 3.0,  1.0 / 3.0,  1.0 / 3.0,  1.0 / 3.0,
                              1.0 / 3.0,  1.0 / 3.0,  1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0,
                              1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0, 1.0 / 24.0};

struct orc_state {
    dl_params P;
    int nx, ny, nz;
    size_t N;
    double *f, *g, *fnext, *gnext, *feq, *geq; /* 15*N, direction fastest */
    double *phi, *p, *u1, *u2, *u3, *taug;     /* N */
    double *p0, *lap, *grad, *gu, *gphi;       /* N, N, 3N, 9N, 9N */
    double *fx, *fy, *fz;                      /* N */
    double phi_min, phi_max; /* interpolation range for the next tau_g */
    int64_t n;               /* steps taken */
    int force_mode;
    int single;              /* the single-phase precursor step (g only) */
};

static int g_threads = 0;

int orc_abi_sizes(int* params_size, int* diag_size) {
    if (!params_size || !diag_size) return DL_ERR_ARG;
    *params_size = (int)sizeof(dl_params);
    *diag_size = (int)sizeof(dl_diag);
    return DL_OK;
}

int orc_set_threads(int nthreads) {
    g_threads = nthreads;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    return DL_OK;
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static inline size_t sidx(const orc_state* o, int x, int y, int z) {
    return (size_t)x + (size_t)o->nx * ((size_t)y + (size_t)o->ny * (size_t)z);
}

/* periodic neighbour x + d (replaces the glue halo, program/lbm_drop_xy.f90:287-358) */
static inline int wrap(int v, int n) {
    v %= n;
    return v < 0 ? v + n : v;
}

static inline size_t nbr(const orc_state* o, int x, int y, int z, int dx, int dy, int dz) {
    return sidx(o, wrap(x + dx, o->nx), wrap(y + dy, o->ny), wrap(z + dz, o->nz));
}

static double* xalloc(size_t n) {
    double* p = (double*)calloc(n ? n : 1, sizeof(double));
    return p;
}

int orc_create(const dl_params* params, int nx, int ny, int nz, orc_state** out) {
    if (!params || !out || nx < 3 || ny < 3 || nz < 3) return DL_ERR_ARG;
    orc_state* o = (orc_state*)calloc(1, sizeof(orc_state));
    if (!o) return DL_ERR_ALLOC;
    o->P = *params;
    o->nx = nx;
    o->ny = ny;
    o->nz = nz;
    o->N = (size_t)nx * ny * nz;
    size_t N = o->N;
    o->f = xalloc(15 * N);
    o->g = xalloc(15 * N);
    o->fnext = xalloc(15 * N);
    o->gnext = xalloc(15 * N);
    o->feq = xalloc(15 * N);
    o->geq = xalloc(15 * N);
    o->phi = xalloc(N);
    o->p = xalloc(N);
    o->u1 = xalloc(N);
    o->u2 = xalloc(N);
    o->u3 = xalloc(N);
    o->taug = xalloc(N);
    o->p0 = xalloc(N);
    o->lap = xalloc(N);
    o->grad = xalloc(3 * N);
    o->gu = xalloc(9 * N);
    o->gphi = xalloc(9 * N);
    o->fx = xalloc(N);
    o->fy = xalloc(N);
    o->fz = xalloc(N);
    if (!o->f || !o->g || !o->fnext || !o->gnext || !o->feq || !o->geq || !o->phi || !o->p ||
        !o->u1 || !o->u2 || !o->u3 || !o->taug || !o->p0 || !o->lap || !o->grad || !o->gu ||
        !o->gphi || !o->fx || !o->fy || !o->fz) {
        orc_destroy(o);
        return DL_ERR_ALLOC;
    }
    o->phi_min = params->phi1;
    o->phi_max = params->phi2;
    o->n = 0;
    o->force_mode = DL_FORCE_NONE;
    *out = o;
    return DL_OK;
}

int orc_destroy(orc_state* o) {
    if (!o) return DL_ERR_ARG;
    free(o->f);
    free(o->g);
    free(o->fnext);
    free(o->gnext);
    free(o->feq);
    free(o->geq);
    free(o->phi);
    free(o->p);
    free(o->u1);
    free(o->u2);
    free(o->u3);
    free(o->taug);
    free(o->p0);
    free(o->lap);
    free(o->grad);
    free(o->gu);
    free(o->gphi);
    free(o->fx);
    free(o->fy);
    free(o->fz);
    free(o);
    return DL_OK;
}

int orc_set_fields(orc_state* o, const double* phi, const double* u1, const double* u2,
                   const double* u3, const double* p) {
    if (!o || !phi || !u1 || !u2 || !u3 || !p) return DL_ERR_ARG;
    size_t bytes = o->N * sizeof(double);
    memcpy(o->phi, phi, bytes);
    memcpy(o->u1, u1, bytes);
    memcpy(o->u2, u2, bytes);
    memcpy(o->u3, u3, bytes);
    memcpy(o->p, p, bytes);
    return DL_OK;
}

int orc_get_fields(orc_state* o, double* phi, double* u1, double* u2, double* u3, double* p) {
    if (!o || !phi || !u1 || !u2 || !u3 || !p) return DL_ERR_ARG;
    size_t bytes = o->N * sizeof(double);
    memcpy(phi, o->phi, bytes);
    memcpy(u1, o->u1, bytes);
    memcpy(u2, o->u2, bytes);
    memcpy(u3, o->u3, bytes);
    memcpy(p, o->p, bytes);
    return DL_OK;
}

int orc_get_populations(orc_state* o, double* f, double* g) {
    if (!o || !f || !g) return DL_ERR_ARG;
    memcpy(f, o->f, 15 * o->N * sizeof(double));
    memcpy(g, o->g, 15 * o->N * sizeof(double));
    return DL_OK;
}

int orc_set_step(orc_state* o, int64_t step) {
    if (!o) return DL_ERR_ARG;
    o->n = step;
    return DL_OK;
}

int orc_get_step(orc_state* o, int64_t* step) {
    if (!o || !step) return DL_ERR_ARG;
    *step = o->n;
    return DL_OK;
}

int orc_get_minmax(orc_state* o, double* mn, double* mx) {
    if (!o || !mn || !mx) return DL_ERR_ARG;
    *mn = o->phi_min;
    *mx = o->phi_max;
    return DL_OK;
}

int orc_get_force(orc_state* o, double* fx, double* fy, double* fz) {
    if (!o || !fx || !fy || !fz) return DL_ERR_ARG;
    memcpy(fx, o->fx, o->N * sizeof(double));
    memcpy(fy, o->fy, o->N * sizeof(double));
    memcpy(fz, o->fz, o->N * sizeof(double));
    return DL_OK;
}

/* various_cal, program/lbm_drop_xy.f90:590-640: p0, lap(phi), grad(phi), grad(u).
 * gu[9s + a + 3*alpha] = grad_u_procs(a, alpha) = d u_a / d x_alpha. */
static void various_cal(orc_state* o) {
    const double T = o->P.T, a = o->P.a, b = o->P.b, ds = o->P.ds;
    const double lapdiv = 5.0 * (ds * ds);
    const double graddiv = 10.0 * ds;
    const int nx = o->nx, ny = o->ny, nz = o->nz;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                size_t s = sidx(o, x, y, z);
                double fun = o->phi[s];
                o->p0[s] = fun * T / (1.0 - b * fun) - a * (fun * fun);
                double lap = -(14.0 * fun);
                for (int i = 1; i < 15; ++i) lap = lap + o->phi[nbr(o, x, y, z, CX[i], CY[i], CZ[i])];
                o->lap[s] = lap / lapdiv;
                for (int al = 0; al < 3; ++al) {
                    double gf = 0.0, g1 = 0.0, g2 = 0.0, g3 = 0.0;
                    for (int i = 1; i < 15; ++i) {
                        double c = (double)(al == 0 ? CX[i] : al == 1 ? CY[i] : CZ[i]);
                        size_t nb = nbr(o, x, y, z, CX[i], CY[i], CZ[i]);
                        gf = gf + c * o->phi[nb];
                        g1 = g1 + c * o->u1[nb];
                        g2 = g2 + c * o->u2[nb];
                        g3 = g3 + c * o->u3[nb];
                    }
                    o->grad[3 * s + al] = gf / graddiv;
                    o->gu[9 * s + 0 + 3 * al] = g1 / graddiv;
                    o->gu[9 * s + 1 + 3 * al] = g2 / graddiv;
                    o->gu[9 * s + 2 + 3 * al] = g3 / graddiv;
                }
            }
}

/* gphi_cal, program/lbm_drop_xy.f90:642-666: G(al,be) = 4.5 g_al g_be - 1.5 |g|^2 delta */
static void gphi_cal(orc_state* o) {
    const size_t N = o->N;
#pragma omp parallel for schedule(static)
    for (size_t s = 0; s < N; ++s) {
        const double* gr = o->grad + 3 * s;
        for (int be = 0; be < 3; ++be)
            for (int al = 0; al < 3; ++al) {
                double kr = (al == be) ? 1.0 : 0.0;
                o->gphi[9 * s + al + 3 * be] =
                    4.5 * gr[al] * gr[be] - 1.5 * ((gr[0] * gr[0] + gr[1] * gr[1]) + gr[2] * gr[2]) * kr;
            }
    }
}

/* tau_g, program/lbm_drop_xy.f90:576-587 (and ini_op :276-280, with phi_min/max
 * = phi1/phi2 at the first step); Smagorinsky part program/LES_drop_xy.f90:481-502,
 * 663-690. */
static void taug_cal(orc_state* o) {
    const dl_params* P = &o->P;
    double mn, mx;
    if (P->visc_mode == DL_VISC_FIXED) {
        mn = P->phi1;
        mx = P->phi2;
    } else {
        mn = o->phi_min;
        mx = o->phi_max;
    }
    const double csd = P->Cs * P->Cs * P->delta * P->delta;
    const double anu23 = (2.0 / 3.0) * P->Anu;
    const size_t N = o->N;
#pragma omp parallel for schedule(static)
    for (size_t s = 0; s < N; ++s) {
        double nu = (o->phi[s] - mn) / (mx - mn) * (P->nu2 - P->nu1) + P->nu1;
        double nue = 0.0;
        if (P->les) {
            const double* gu = o->gu + 9 * s;
            double acc = 0.0;
            for (int be = 0; be < 3; ++be)
                for (int al = 0; al < 3; ++al) {
                    double st = 0.5 * (gu[al + 3 * be] + gu[be + 3 * al]);
                    acc = acc + st * st;
                }
            nue = csd * sqrt(2.0 * acc);
        }
        o->taug[s] = 0.5 + 3.0 * (nu + nue) / P->ds + anu23;
    }
}

/* equilibrium_cal, program/lbm_drop_xy.f90:421-476. Writes into fe, ge. */
static void equilibrium_cal(orc_state* o, double* fe, double* ge) {
    const dl_params* P = &o->P;
    const double kf = P->kappaf, kg = P->kappag;
    const double kf6 = kf / 6.0;
    const double anuds = P->Anu * P->ds;
    const size_t N = o->N;
#pragma omp parallel for schedule(static)
    for (size_t s = 0; s < N; ++s) {
        const double phi = o->phi[s], p = o->p[s];
        const double u1 = o->u1[s], u2 = o->u2[s], u3 = o->u3[s];
        const double* gu = o->gu + 9 * s;
        const double* gp = o->gphi + 9 * s;
        const double* gr = o->grad + 3 * s;
        for (int i = 0; i < 15; ++i) {
            const double cr[3] = {(double)CX[i], (double)CY[i], (double)CZ[i]};
            double ftemp = 0.0, gtemp = 0.0;
            for (int be = 0; be < 3; ++be)
                for (int al = 0; al < 3; ++al) {
                    ftemp = ftemp + (gu[be + 3 * al] + gu[al + 3 * be]) * cr[al] * cr[be];
                    gtemp = gtemp + gp[al + 3 * be] * cr[al] * cr[be];
                }
            fe[15 * s + i] = HW[i] * phi +
                             FW[i] * (o->p0[s] - kf * phi * o->lap[s] -
                                      kf6 * (gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2])) +
                             EW[i] * phi * 3.0 * (cr[0] * u1 + cr[1] * u2 + cr[2] * u3) +
                             EW[i] * kf * gtemp;
            double cu = u1 * cr[0] + u2 * cr[1] + u3 * cr[2];
            ge[15 * s + i] = EW[i] * (3.0 * p + 3.0 * cu + 4.5 * (cu * cu) -
                                      1.5 * (u1 * u1 + u2 * u2 + u3 * u3) + anuds * ftemp) +
                             EW[i] * kg * gtemp;
        }
    }
}

/* fg_cal, program/lbm_drop_xy.f90:478-515: pull-stream of the collided f, g
 * plus the body force, all evaluated at the source site x - c_i. */
static void fg_cal(orc_state* o) {
    const double tauf = o->P.tauf;
    const double ds3 = 3.0 * o->P.ds;
    const int nx = o->nx, ny = o->ny, nz = o->nz;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                size_t s = sidx(o, x, y, z);
                for (int i = 0; i < 15; ++i) {
                    size_t n = nbr(o, x, y, z, -CX[i], -CY[i], -CZ[i]);
                    double fs = o->f[15 * n + i], gs = o->g[15 * n + i];
                    o->fnext[15 * s + i] = fs - (fs - o->feq[15 * n + i]) / tauf;
                    o->gnext[15 * s + i] =
                        gs - (gs - o->geq[15 * n + i]) / o->taug[n] +
                        ds3 * EW[i] *
                            ((double)CX[i] * o->fx[n] + (double)CY[i] * o->fy[n] + (double)CZ[i] * o->fz[n]);
                }
            }
}

/* bounce_back_LBM on g, prototype_program/two-phase/drop8_mpi.f90:642-674.
 * Bottom plane z = 0 moves with -U, top plane z = nz-1 with +U; U is
 * wall_u from step wall_start on, zero before (drop8_mpi.f90:645-650). */
static const int BB_BOT_IN[5] = {3, 7, 8, 9, 14};   /* reference i = 4, 8, 9, 10, 15 */
static const int BB_BOT_SRC[5] = {6, 11, 12, 13, 10}; /* reference i = 7,12,13,14,11 */
static const int BB_TOP_IN[5] = {6, 10, 11, 12, 13};  /* reference i = 7,11,12,13,14 */
static const int BB_TOP_SRC[5] = {3, 14, 7, 8, 9};    /* reference i = 4,15, 8, 9,10 */

static void bounce_back(orc_state* o, int64_t n) {
    double U[3] = {0.0, 0.0, 0.0};
    if (n >= o->P.wall_start) {
        U[0] = o->P.wall_u[0];
        U[1] = o->P.wall_u[1];
        U[2] = o->P.wall_u[2];
    }
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    double* gn = o->gnext;
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            size_t s = sidx(o, x, y, 0);
            for (int k = 0; k < 5; ++k) {
                int i = BB_BOT_IN[k], j = BB_BOT_SRC[k];
                gn[15 * s + i] = gn[15 * s + j] - 6.0 * EW[j] *
                                                      ((-U[0]) * (double)CX[j] + (-U[1]) * (double)CY[j] +
                                                       (-U[2]) * (double)CZ[j]);
            }
        }
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            size_t s = sidx(o, x, y, nz - 1);
            for (int k = 0; k < 5; ++k) {
                int i = BB_TOP_IN[k], j = BB_TOP_SRC[k];
                gn[15 * s + i] = gn[15 * s + j] - 6.0 * EW[j] *
                                                      ((U[0]) * (double)CX[j] + (U[1]) * (double)CY[j] +
                                                       (U[2]) * (double)CZ[j]);
            }
        }
}

/* moments of f, g at every site: program/lbm_drop_xy.f90:541-552 */
static void moments(orc_state* o) {
    const size_t N = o->N;
#pragma omp parallel for schedule(static)
    for (size_t s = 0; s < N; ++s) {
        const double* f = o->f + 15 * s;
        const double* g = o->g + 15 * s;
        double ph = 0.0, pp = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        for (int i = 0; i < 15; ++i) {
            ph = ph + f[i];
            pp = pp + g[i] / 3.0;
            a1 = a1 + (double)CX[i] * g[i];
            a2 = a2 + (double)CY[i] * g[i];
            a3 = a3 + (double)CZ[i] * g[i];
        }
        o->phi[s] = ph;
        o->p[s] = pp;
        o->u1[s] = a1;
        o->u2[s] = a2;
        o->u3[s] = a3;
    }
}

/* physics, program/lbm_drop_xy.f90:517-574: copy next -> current, moments,
 * and the serial phi min/max scan with its if / else-if and its starting
 * values (min = phi2, max = phi1). */
static void physics(orc_state* o) {
    const size_t N = o->N;
#pragma omp parallel for schedule(static)
    for (size_t s = 0; s < N; ++s)
        for (int i = 0; i < 15; ++i) {
            o->f[15 * s + i] = o->fnext[15 * s + i];
            o->g[15 * s + i] = o->gnext[15 * s + i];
        }
    moments(o);
    double mn = o->P.phi2, mx = o->P.phi1;
    for (size_t s = 0; s < N; ++s) {
        double v = o->phi[s];
        if (v > mx)
            mx = v;
        else if (v < mn)
            mn = v;
    }
    o->phi_min = mn;
    o->phi_max = mx;
}

/* ---- spectral forcing: program/lbm_drop_iht_xy.f90:722-842 -------------
 * u_hat = DFT(u)/N on the band 1 <= |k| < kc (k_index = int(|k|)+1 with
 * 1 < k_index < kc+1); E = sum over the half spectrum (k3 >= 0) of
 * 0.5 |u_hat|^2 min(2, k3+1); f_hat = (0.5 eps / E) u_hat; F = c2r(f_hat).
 * The DFT is evaluated separably (x, then y, then z), only for the band. */
typedef struct {
    double re, im;
} cplx;

static void twiddle(int n, double* c, double* s) {
    const double pi = acos(-1.0);
    for (int m = 0; m < n; ++m) {
        double ang = 2.0 * pi * (double)m / (double)n;
        c[m] = cos(ang);
        s[m] = sin(ang);
    }
}

/* FFT-order position of wavenumber k in an axis of length n */
static inline int kpos(int k, int n) { return k >= 0 ? k : k + n; }

static void spectral_force(orc_state* o) {
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    const int K = o->P.kc - 1; /* largest |component| inside the band */
    const int kc2 = o->P.kc * o->P.kc;
    const int NK = 2 * K + 1;
    if (K < 1) {
        memset(o->fx, 0, o->N * sizeof(double));
        memset(o->fy, 0, o->N * sizeof(double));
        memset(o->fz, 0, o->N * sizeof(double));
        return;
    }
    double *cxx = xalloc(nx), *sxx = xalloc(nx), *cyy = xalloc(ny), *syy = xalloc(ny);
    double *czz = xalloc(nz), *szz = xalloc(nz);
    twiddle(nx, cxx, sxx);
    twiddle(ny, cyy, syy);
    twiddle(nz, czz, szz);
    const double* comp[3] = {o->u1, o->u2, o->u3};
    /* uh[c][kx+K][ky+K][kz], kz = 0..K */
    cplx* uh = (cplx*)calloc((size_t)3 * NK * NK * (K + 1), sizeof(cplx));
    cplx* a1 = (cplx*)calloc((size_t)NK * ny * nz, sizeof(cplx));
    cplx* a2 = (cplx*)calloc((size_t)NK * NK * nz, sizeof(cplx));
    const double Nd = (double)nx * (double)ny * (double)nz;
    for (int c = 0; c < 3; ++c) {
        const double* u = comp[c];
        /* x stage: a1[kx][y][z] = sum_x u e^{-i kx x} */
#pragma omp parallel for schedule(static)
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int kx = -K; kx <= K; ++kx) {
                    double re = 0.0, im = 0.0;
                    for (int x = 0; x < nx; ++x) {
                        int m = (int)(((long)kx * x % nx + nx) % nx);
                        double v = u[sidx(o, x, y, z)];
                        re += v * cxx[m];
                        im -= v * sxx[m];
                    }
                    cplx* d = &a1[((size_t)(kx + K) * ny + y) * nz + z];
                    d->re = re;
                    d->im = im;
                }
        /* y stage */
#pragma omp parallel for schedule(static)
        for (int z = 0; z < nz; ++z)
            for (int kx = 0; kx < NK; ++kx)
                for (int ky = -K; ky <= K; ++ky) {
                    double re = 0.0, im = 0.0;
                    for (int y = 0; y < ny; ++y) {
                        int m = (int)(((long)ky * y % ny + ny) % ny);
                        cplx v = a1[((size_t)kx * ny + y) * nz + z];
                        re += v.re * cyy[m] + v.im * syy[m];
                        im += v.im * cyy[m] - v.re * syy[m];
                    }
                    cplx* d = &a2[((size_t)kx * NK + (ky + K)) * nz + z];
                    d->re = re;
                    d->im = im;
                }
        /* z stage, normalised by N as fft_r2c does (lbm_drop_iht_xy.f90:899) */
        for (int kx = 0; kx < NK; ++kx)
            for (int ky = 0; ky < NK; ++ky)
                for (int kz = 0; kz <= K; ++kz) {
                    double re = 0.0, im = 0.0;
                    for (int z = 0; z < nz; ++z) {
                        int m = (int)(((long)kz * z) % nz);
                        cplx v = a2[((size_t)kx * NK + ky) * nz + z];
                        re += v.re * czz[m] + v.im * szz[m];
                        im += v.im * czz[m] - v.re * szz[m];
                    }
                    cplx* d = &uh[(((size_t)c * NK + kx) * NK + ky) * (K + 1) + kz];
                    d->re = re / Nd;
                    d->im = im / Nd;
                }
    }
    /* band energy in the reference's loop order: k3 outer, k2, k1 inner, each
     * in FFT index order (0, 1, .., n/2, -n/2+1, .., -1) */
    double energy = 0.0;
    for (int k3 = 0; k3 <= K; ++k3)
        for (int i2 = 0; i2 < ny; ++i2) {
            int k2 = (i2 >= ny / 2 + 1) ? i2 - ny : i2;
            if (k2 < -K || k2 > K) continue;
            for (int i1 = 0; i1 < nx; ++i1) {
                int k1 = (i1 >= nx / 2 + 1) ? i1 - nx : i1;
                if (k1 < -K || k1 > K) continue;
                int kk = k1 * k1 + k2 * k2 + k3 * k3;
                if (kk < 1 || kk >= kc2) continue;
                double e[3];
                for (int c = 0; c < 3; ++c) {
                    cplx v = uh[(((size_t)c * NK + (k1 + K)) * NK + (k2 + K)) * (K + 1) + k3];
                    e[c] = v.re * v.re + v.im * v.im;
                }
                double w = 2.0 < (double)k3 + 1.0 ? 2.0 : (double)k3 + 1.0;
                energy = energy + 0.5 * (e[0] + e[1] + e[2]) * w;
            }
        }
    const double coef = 0.5 * o->P.eps / energy;
    /* synthesis, as the c2r of the half spectrum: F = sum_kz w(kz) Re(sum f_hat e^{ik.x}) */
    double* outc[3] = {o->fx, o->fy, o->fz};
    cplx* b1 = (cplx*)calloc((size_t)NK * NK * nz, sizeof(cplx));
    cplx* b2 = (cplx*)calloc((size_t)NK * ny * nz, sizeof(cplx));
    for (int c = 0; c < 3; ++c) {
#pragma omp parallel for schedule(static)
        for (int z = 0; z < nz; ++z)
            for (int kx = -K; kx <= K; ++kx)
                for (int ky = -K; ky <= K; ++ky) {
                    double re = 0.0, im = 0.0;
                    for (int kz = 0; kz <= K; ++kz) {
                        int kk = kx * kx + ky * ky + kz * kz;
                        if (kk < 1 || kk >= kc2) continue;
                        cplx v = uh[(((size_t)c * NK + (kx + K)) * NK + (ky + K)) * (K + 1) + kz];
                        double fre = coef * v.re, fim = coef * v.im;
                        double w = kz == 0 ? 1.0 : 2.0;
                        int m = (int)(((long)kz * z) % nz);
                        re += w * (fre * czz[m] - fim * szz[m]);
                        im += w * (fre * szz[m] + fim * czz[m]);
                    }
                    cplx* d = &b1[((size_t)(kx + K) * NK + (ky + K)) * nz + z];
                    d->re = re;
                    d->im = im;
                }
#pragma omp parallel for schedule(static)
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int kx = 0; kx < NK; ++kx) {
                    double re = 0.0, im = 0.0;
                    for (int ky = -K; ky <= K; ++ky) {
                        cplx v = b1[((size_t)kx * NK + (ky + K)) * nz + z];
                        int m = (int)(((long)ky * y % ny + ny) % ny);
                        re += v.re * cyy[m] - v.im * syy[m];
                        im += v.re * syy[m] + v.im * cyy[m];
                    }
                    cplx* d = &b2[((size_t)kx * ny + y) * nz + z];
                    d->re = re;
                    d->im = im;
                }
        double* out = outc[c];
#pragma omp parallel for schedule(static)
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) {
                    double re = 0.0;
                    for (int kx = -K; kx <= K; ++kx) {
                        cplx v = b2[((size_t)(kx + K) * ny + y) * nz + z];
                        int m = (int)(((long)kx * x % nx + nx) % nx);
                        re += v.re * cxx[m] - v.im * sxx[m];
                    }
                    out[sidx(o, x, y, z)] = re;
                }
    }
    (void)kpos;
    free(b1);
    free(b2);
    free(uh);
    free(a1);
    free(a2);
    free(cxx);
    free(sxx);
    free(cyy);
    free(syy);
    free(czz);
    free(szz);
}

int orc_compute_spectral_force(orc_state* o) {
    if (!o) return DL_ERR_ARG;
    spectral_force(o);
    return DL_OK;
}

int orc_set_force(orc_state* o, int mode, const double* fx, const double* fy, const double* fz) {
    if (!o) return DL_ERR_ARG;
    size_t bytes = o->N * sizeof(double);
    if (mode == DL_FORCE_STATIC) {
        if (!fx || !fy || !fz) return DL_ERR_ARG;
        memcpy(o->fx, fx, bytes);
        memcpy(o->fy, fy, bytes);
        memcpy(o->fz, fz, bytes);
    } else if (mode == DL_FORCE_NONE || mode == DL_FORCE_SPECTRAL) {
        memset(o->fx, 0, bytes);
        memset(o->fy, 0, bytes);
        memset(o->fz, 0, bytes);
    } else {
        return DL_ERR_ARG;
    }
    o->force_mode = mode;
    return DL_OK;
}

static void equilibrium_single(orc_state* o);

/* ini, program/lbm_drop_xy.f90:244-251, and ini_op, :254-285 */
int orc_init_equilibrium(orc_state* o) {
    if (!o) return DL_ERR_ARG;
    if (o->single) {  /* ini, program/lbm_iht_xy.f90:270 */
        equilibrium_single(o);
        memcpy(o->g, o->geq, 15 * o->N * sizeof(double));
        return DL_OK;
    }
    various_cal(o);
    gphi_cal(o);
    equilibrium_cal(o, o->f, o->g);
    o->phi_min = o->P.phi1;
    o->phi_max = o->P.phi2;
    return DL_OK;
}

/* resume / precursor read: recompute phi, p, u from the given f, g */
int orc_set_populations(orc_state* o, const double* f, const double* g) {
    if (!o || !f || !g) return DL_ERR_ARG;
    memcpy(o->f, f, 15 * o->N * sizeof(double));
    memcpy(o->g, g, 15 * o->N * sizeof(double));
    moments(o);
    return DL_OK;
}

/* ---- the single-phase precursor step, program/lbm_iht_xy.f90 ------------
 * equilibrium_cal (:532-559): geq = E (3p + 3 c.u + 4.5 (c.u)^2 - 1.5 u^2) */
static void equilibrium_single(orc_state* o) {
    const size_t N = o->N;
#pragma omp parallel for schedule(static)
    for (size_t s = 0; s < N; ++s) {
        const double p = o->p[s], u1 = o->u1[s], u2 = o->u2[s], u3 = o->u3[s];
        for (int i = 0; i < 15; ++i) {
            const double cu = u1 * (double)CX[i] + u2 * (double)CY[i] + u3 * (double)CZ[i];
            o->geq[15 * s + i] = EW[i] * (3.0 * p + 3.0 * cu + 4.5 * (cu * cu) - 1.5 * (u1 * u1 + u2 * u2 + u3 * u3));
        }
    }
}

/* g_cal (:561-590) with tau_g = 1/2 + 3 (nu + nue)/ds, nue = 0 (Cs = 0, :21-22,
 * physics :649), then physics (:592-654): copy and moments p = sum g/3, u = sum c g */
static void step_single(orc_state* o) {
    const double taug = 0.5 + 3.0 * (o->P.nu1 + 0.0) / o->P.ds;
    const double ds3 = 3.0 * o->P.ds;
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    equilibrium_single(o);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                size_t s = sidx(o, x, y, z);
                for (int i = 0; i < 15; ++i) {
                    size_t n = nbr(o, x, y, z, -CX[i], -CY[i], -CZ[i]);
                    double gs = o->g[15 * n + i];
                    o->gnext[15 * s + i] =
                        gs - (gs - o->geq[15 * n + i]) / taug +
                        ds3 * EW[i] *
                            ((double)CX[i] * o->fx[n] + (double)CY[i] * o->fy[n] + (double)CZ[i] * o->fz[n]);
                }
            }
}

static void physics_single(orc_state* o) {
    const size_t N = o->N;
#pragma omp parallel for schedule(static)
    for (size_t s = 0; s < N; ++s) {
        double pp = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        for (int i = 0; i < 15; ++i) {
            const double gv = o->gnext[15 * s + i];
            o->g[15 * s + i] = gv;
            pp = pp + gv / 3.0;
            a1 = a1 + (double)CX[i] * gv;
            a2 = a2 + (double)CY[i] * gv;
            a3 = a3 + (double)CZ[i] * gv;
        }
        o->p[s] = pp;
        o->u1[s] = a1;
        o->u2[s] = a2;
        o->u3[s] = a3;
    }
}

int orc_set_single(orc_state* o, int on) {
    if (!o) return DL_ERR_ARG;
    o->single = on ? 1 : 0;
    return DL_OK;
}

/* one step = the loop body of program/lbm_drop_xy.f90:787-840, or of
 * program/lbm_iht_xy.f90:960-980 in the single-phase mode */
static void step_once(orc_state* o) {
    int64_t n = o->n + 1;
    if (o->single) {
        if (o->force_mode == DL_FORCE_SPECTRAL) spectral_force(o);
        step_single(o);
        if (o->P.walls) bounce_back(o, n);
        physics_single(o);
        o->n = n;
        return;
    }
    if (o->force_mode == DL_FORCE_SPECTRAL) spectral_force(o);
    various_cal(o);
    gphi_cal(o);
    taug_cal(o);
    equilibrium_cal(o, o->feq, o->geq);
    fg_cal(o);
    if (o->P.walls) bounce_back(o, n);
    physics(o);
    o->n = n;
}

int orc_step(orc_state* o, int nsteps) {
    if (!o || nsteps < 0) return DL_ERR_ARG;
    for (int k = 0; k < nsteps; ++k) step_once(o);
    return DL_OK;
}
