/*
 * droplet_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU FP64 restatement of the reference's D3Q15 two-phase droplet step, used
 * as the parity checker for the GPU library and as the timed CPU baseline.
 * It is never linked into, loaded by, or called from the product path.
 *
 * The entry points mirror include/droplet_gb300.h one for one (orc_* for
 * dl_*), with the same argument meaning and host layouts, so that a test can
 * drive both through the same sequence of calls.
 */
#ifndef DROPLET_ORACLE_H
#define DROPLET_ORACLE_H

#include <stdint.h>
#include "../include/droplet_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_state orc_state;

int orc_create(const dl_params* params, int nx, int ny, int nz, orc_state** out);
int orc_destroy(orc_state* o);
int orc_set_fields(orc_state* o, const double* phi, const double* u1,
                   const double* u2, const double* u3, const double* p);
int orc_init_equilibrium(orc_state* o);
int orc_set_force(orc_state* o, int mode, const double* fx, const double* fy,
                  const double* fz);
int orc_step(orc_state* o, int nsteps);
/* Nonzero: the single-phase precursor step of program/lbm_iht_xy.f90 (g only,
 * tau_g = 1/2 + 3 nu1/ds); set before orc_init_equilibrium. */
int orc_set_single(orc_state* o, int on);
int orc_get_fields(orc_state* o, double* phi, double* u1, double* u2,
                   double* u3, double* p);
int orc_get_populations(orc_state* o, double* f, double* g);
int orc_set_populations(orc_state* o, const double* f, const double* g);
int orc_set_step(orc_state* o, int64_t step);
int orc_get_step(orc_state* o, int64_t* step);
int orc_get_minmax(orc_state* o, double* phi_min, double* phi_max);
/* The body force used by the last step (for spectral mode: computed from u). */
int orc_get_force(orc_state* o, double* fx, double* fy, double* fz);
/* Compute the spectral force from the current u without stepping. */
int orc_compute_spectral_force(orc_state* o);
/* sizeof(dl_params) and sizeof(dl_diag) as this compiler lays them out
 * (lets the tests check the ctypes mirror of the header). */
int orc_abi_sizes(int* params_size, int* diag_size);
/* Number of OpenMP threads used by the loops (0 = runtime default). */
int orc_set_threads(int nthreads);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif

#endif
