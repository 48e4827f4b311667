/*
 * droplet_gb300.h -- C-ABI of the GB300 D3Q15 two-phase droplet step.
 *
 * The reference (nakano-gendai/droplet) has no library interface: its hot
 * path is the subroutine sequence inside the Fortran `program main` of
 * program/lbm_drop_xy.f90:830-840 (identical at program/lbm_drop_iht_xy.f90:1016-1026
 * and program/lbm_omp_drop.f90:827-837), with state in module-level arrays.
 * Each entry point below replaces one piece of that sequence; the comment on
 * each names the reference lines it stands in for.
 *
 * Conventions
 *  - Every function returns an int status: DL_OK (0) or a negative DL_ERR_*.
 *  - Scalar fields (phi, u1, u2, u3, p, forces) are host arrays of nx*ny*nz
 *    doubles, x fastest, then y, then z: the Fortran order of
 *    phi_procs(x,y,z) in the reference, i.e. C order [z][y][x].
 *  - Populations are host arrays of 15*nx*ny*nz doubles with the direction
 *    index fastest: the reference's f_procs(1:15,x,y,z) layout.
 *  - The library owns all device memory; the caller owns host arrays.
 *    Calls on one handle must not overlap (single-threaded per handle).
 *  - Directions i = 0..14 here are the reference's i = 1..15.
 */
#ifndef DROPLET_GB300_H
#define DROPLET_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define DL_OK               0
#define DL_ERR_ARG         -1   /* bad argument (null pointer, size, mode) */
#define DL_ERR_CUDA        -2   /* a CUDA runtime call failed */
#define DL_ERR_ALLOC       -3   /* device or host allocation failed */
#define DL_ERR_NAN         -4   /* the NaN/Inf watchdog tripped during a step */
#define DL_ERR_TIMEOUT     -5   /* a bounded device-side wait ran out */
#define DL_ERR_STATE       -6   /* call out of order (e.g. step before fields) */
#define DL_ERR_UNSUPPORTED -7   /* option not available in this form */

/* ---- storage / arithmetic forms ------------------------------------------ */
#define DL_FORM_FP64  64  /* plain form: FP64 storage and arithmetic in the
                             reference's evaluation order (no FMA contraction) */
#define DL_FORM_FP32  32  /* FP32 arithmetic; populations stored in FP32 as
                             deviations from the bulk equilibrium at phi1, p=1/3 */
#define DL_FORM_FP16  16  /* FP32 arithmetic; populations stored as scaled
                             FP16 deviations; FP64 for conservation sums */
/* OR-ed into the form: the single-phase step of the precursor turbulence
 * program (program/lbm_iht_xy.f90: equilibrium_cal :532-559, g_cal :561-590,
 * physics :592-654): g only, geq = E (3p + 3c.u + 4.5 (c.u)^2 - 1.5 u^2),
 * tau_g = 1/2 + 3 nu1/ds, the same forcing and walls. No f populations are
 * allocated; phi is not a field (dl_get_fields returns phi = phi1). Requires
 * les = 0 and Anu = 0 (the precursor's Cs = 0). */
#define DL_SINGLE_PHASE 0x100

/* ---- body-force modes ------------------------------------------------------ */
#define DL_FORCE_NONE      0
#define DL_FORCE_STATIC    1  /* caller-given Fx,Fy,Fz held fixed in time:
                                 externalforce, program/lbm_drop_xy.f90:668-693 */
#define DL_FORCE_SPECTRAL  2  /* constant-injection band forcing recomputed from
                                 u every step: externalforce,
                                 program/lbm_drop_iht_xy.f90:722-842 */

/* ---- viscosity interpolation ----------------------------------------------- */
#define DL_VISC_MINMAX 0  /* nu from the previous step's global phi min/max:
                             physics, program/lbm_drop_xy.f90:559-587 */
#define DL_VISC_FIXED  1  /* nu from the fixed phi1..phi2 range:
                             ini_op, program/lbm_drop_xy.f90:254-285 */

/* Physical and numerical parameters. Names follow the reference's
 * `module globals` (program/lbm_drop_xy.f90:10-59). */
typedef struct dl_params {
    double ds;          /* lattice spacing */
    double tauf;        /* relaxation time of f (order parameter) */
    double kappaf;      /* interface-thickness parameter */
    double kappag;      /* surface-tension parameter */
    double phi1, phi2;  /* continuous / dispersed phase order parameter */
    double a, b, T;     /* van der Waals constants of p0(phi) */
    double nu1, nu2;    /* kinematic viscosity of phase 1 / phase 2 */
    double Anu;         /* velocity-gradient correction in geq */
    double Cs, delta;   /* Smagorinsky constant and filter width (les != 0) */
    double wall_u[3];   /* top-wall velocity; the bottom wall moves with -wall_u */
    double eps;         /* energy injection rate of the spectral forcing */
    int64_t wall_start; /* first step (1-based) at which the walls move */
    int32_t visc_mode;  /* DL_VISC_* */
    int32_t les;        /* nonzero: Smagorinsky eddy viscosity in tau_g */
    int32_t walls;      /* nonzero: moving-wall bounce-back of g at z=0, z=nz-1 */
    int32_t kc;         /* spectral forcing acts on 1 <= |k| < kc */
} dl_params;

/* FP64 diagnostics over the whole domain (compensated sums). */
typedef struct dl_diag {
    double phi_sum;      /* sum of phi */
    double p_sum;        /* sum of p */
    double mom[3];       /* sum of u */
    double ke;           /* 1/2 sum |u|^2 */
    double diss;         /* sum of 2 nu(phi) S:S (stencil strain) */
    double vol_count;    /* number of sites with phi > (phi1+phi2)/2 */
    double vol_smooth;   /* sum of (phi-phi1)/(phi2-phi1) */
    double phi_min, phi_max;
    double p_in, n_in;   /* sum of p and count where (phi-phi1)/(phi2-phi1) > 0.95 */
    double p_out, n_out; /* sum of p and count where it is < 0.05 */
    double w_sum;        /* second-moment tensor of w = (phi-phi1)/(phi2-phi1) */
    double w_x[3];       /* sum w*x_a */
    double w_xx[6];      /* sum w*x_a*x_b : xx, yy, zz, xy, xz, yz */
    int64_t step;        /* steps taken since dl_create */
    int32_t nan_flag;    /* nonzero if the watchdog saw NaN/Inf */
    int32_t pad_;
} dl_diag;

/* In-situ energy diagnostics of the current fields (dl_energy). */
typedef struct dl_energy_diag {
    double psi_sum;      /* sum of phi T ln(phi/(1 - b phi)) - a phi^2: free_energy_cal,
                            program/energy_budget.f90:1012-1023 */
    double mu_sum;       /* sum of the chemical potential T ln(phi/(1 - b phi))
                            + T/(1 - b phi) - 2 a phi - kappag lap(phi):
                            chemical_potencial_cal, program/energy_budget.f90:998-1010 */
    double grad_sq_sum;  /* sum of |grad phi|^2 (14-neighbour stencil) */
    double spectrum_sum; /* sum of the returned spectrum bins */
    int64_t nbins;       /* bins returned */
    int64_t step;
} dl_energy_diag;

/* Launch accounting of the library's own kernels (for benchmarks). */
typedef struct dl_profile_stats {
    double main_ms;          /* summed device time of the fused step kernel */
    double total_ms;         /* summed device time of every timed launch */
    int64_t main_launches;   /* launches of the fused step kernel */
    int64_t timed_launches;  /* launches bracketed by events */
    int64_t launches;        /* all kernel launches issued since the last read */
} dl_profile_stats;

typedef struct dl_handle dl_handle;

/* Library version (major*10000 + minor*100 + patch). */
int dl_version(void);

/* Human-readable text of a status code. */
const char* dl_status_string(int status);

/* Allocate a whole-domain state on the current CUDA device.
 * Replaces the allocations of ini/ini_op, program/lbm_drop_xy.f90:131-285,
 * without the MPI decomposition (:143-185): the domain is resident.
 * form: DL_FORM_FP64 / FP32 / FP16, optionally | DL_SINGLE_PHASE. */
int dl_create(const dl_params* params, int nx, int ny, int nz, int form,
              dl_handle** out);

/* Free all device memory of the handle. */
int dl_destroy(dl_handle* h);

/* Run subsequent work on this cudaStream_t (NULL: the legacy default stream). */
int dl_set_stream(dl_handle* h, void* cuda_stream);

/* Upload phi, u1, u2, u3, p (x fastest). Replaces the initial-condition loop
 * of ini, program/lbm_drop_xy.f90:224-242. */
int dl_set_fields(dl_handle* h, const double* phi, const double* u1,
                  const double* u2, const double* u3, const double* p);

/* f <- feq, g <- geq from the current fields, and reset the tau_g
 * interpolation range to phi1..phi2. Replaces the tail of ini,
 * program/lbm_drop_xy.f90:244-251, and ini_op, :254-285. */
int dl_init_equilibrium(dl_handle* h);

/* Select the body force. mode DL_FORCE_STATIC uploads fx, fy, fz (x fastest);
 * the other modes take NULL. Replaces externalforce + glue(force),
 * program/lbm_drop_xy.f90:825-827 and program/lbm_drop_iht_xy.f90:1008-1014. */
int dl_set_force(dl_handle* h, int mode, const double* fx, const double* fy,
                 const double* fz);

/* Advance nsteps time steps. One step replaces the loop body
 * program/lbm_drop_xy.f90:830-840 (MPI_boundary, various_cal, gphi_cal,
 * equilibrium_cal, MPI_boundary_fg, fg_cal, physics) plus, when enabled,
 * the spectral force of program/lbm_drop_iht_xy.f90:1008-1014, the
 * Smagorinsky tau_g of program/LES_drop_xy.f90:655-690 and the moving-wall
 * bounce-back of prototype_program/two-phase/drop8_mpi.f90:642-674. */
int dl_step(dl_handle* h, int nsteps);

/* Download phi, u1, u2, u3, p (x fastest): the record content of output,
 * program/lbm_drop_xy.f90:695-719. */
int dl_get_fields(dl_handle* h, double* phi, double* u1, double* u2,
                  double* u3, double* p);

/* Download f and g, direction index fastest: the content of outputfg,
 * program/lbm_drop_xy.f90:721-743 (checkpoint). */
int dl_get_populations(dl_handle* h, double* f, double* g);

/* Upload f and g (direction fastest) and recompute phi, p, u from them:
 * resume from a checkpoint, or the precursor read of
 * program/lbm_drop_xy.f90:789-823 (which recomputes p and u from g). */
int dl_set_populations(dl_handle* h, const double* f, const double* g);

/* Set / read the step counter (used by the wall start time). */
int dl_set_step(dl_handle* h, int64_t step);
int dl_get_step(dl_handle* h, int64_t* step);

/* The phi min/max that the next step's tau_g interpolation will use:
 * phi_min/phi_max after the MPI_Allreduce, program/lbm_drop_xy.f90:559-574. */
int dl_get_minmax(dl_handle* h, double* phi_min, double* phi_max);

/* The same two values without waiting: enqueues their copy into
 * dst[0] = phi_min, dst[1] = phi_max on the handle's stream and returns. dst
 * must be page-locked host memory (cudaHostAlloc / pinned) that stays valid
 * until the copy is done; read it after the stream (or an event recorded
 * after this call) has completed. Lets a host read every step's result one
 * step behind while the GPU keeps stepping. */
int dl_get_minmax_async(dl_handle* h, double* dst);

/* Host mirror of every step's phi range (no reference counterpart: the
 * reference reduces phi's range on the host each step, program/lbm_drop_xy.f90
 * physics). With host = page-locked memory of 2 nslots doubles, dl_step
 * follows each step with a one-warp kernel that writes, for the step that
 * takes the step counter to n, host[2 (n % nslots)] = phi_min and
 * host[2 (n % nslots) + 1] = phi_max (no copy-engine transfer); the values
 * are there once an event recorded after dl_step has completed. The array
 * must stay allocated until the mirror is switched off (host = NULL) or the
 * handle is destroyed. Steps taken by dl_batch_step do not write it.
 * Returns DL_ERR_ARG if host is not page-locked memory the device can write
 * or nslots is not a power of two (1, 2, 4, ...). */
int dl_set_minmax_mirror(dl_handle* h, double* host, int64_t nslots);

/* Page-locked host memory the device can write (for dl_set_minmax_mirror and
 * the *_async host buffers) for hosts without the CUDA runtime headers, e.g.
 * a Fortran main loop: *out receives bytes of zeroed memory; release with
 * dl_host_free. Returns DL_ERR_ALLOC if the allocation fails. */
int dl_host_alloc(int64_t bytes, void** out);
int dl_host_free(void* p);

/* FP64 diagnostics of the current fields; replaces the ad-hoc sums of the
 * analysis programs (kinetic.d in program/lbm_iht_xy.f90:777-822, the
 * droplet moments of prototype_program/two-phase/drop8_mpi.f90:812-970). */
int dl_reduce(dl_handle* h, dl_diag* out);

/* In-situ turbulence and free-energy diagnostics: the sums of dl_energy_diag
 * and, when nbins > 0, the kinetic-energy spectrum of enesupe_cal
 * (program/turbulence_hit_xy.f90:588-645) in spectrum[0..nbins): bin j holds
 * the modes with int(|k|) = j (the reference's k_index = j + 1), summed over
 * k1 in [0,nx), k2 in [0,ny), k3 in [0,nz/2] of 0.5 |u_hat|^2 with weight 1 at
 * k3 = 0 and 2 elsewhere, u_hat = FFT(u)/N. The reference's array has
 * nx/2 + 1 bins; modes beyond nbins are left out. FP64 FFTs (cuFFT); the
 * first call plans the transform and allocates its buffers. */
int dl_energy(dl_handle* h, dl_energy_diag* out, double* spectrum, int64_t nbins);

/* The memory ceiling of the step's access pattern on this GPU, in GB/s: a
 * z-marching 32 x 8 column kernel pulls the 15 direction arrays of g from
 * x - c_i and writes them back with no collision, `repeats` times on the
 * handle's own g buffers (the next-step buffer is overwritten). FP32 and FP16
 * forms. No counterpart in the reference: it places the fused step's
 * achieved bandwidth between this ceiling and the copy peak. */
int dl_pull_ceiling(dl_handle* h, int repeats, double* gbytes_per_s);

/* FP64 FMA throughput of this GPU in TFLOP/s (2 flops per FMA), the bound of
 * the plain FP64 form; runs on the handle's stream. No reference counterpart. */
int dl_fp64_ceiling(dl_handle* h, double* tflops);

/* dl_reduce_static: the same diagnostics as dl_reduce, for callers that must
 * not allocate device memory once their run is set up -- a host program that
 * has reserved nearly all of the GPU's memory for its lattices, or a
 * monitoring thread that must not enter the device allocator while other
 * threads step. It allocates nothing: its working memory is one fixed array
 * of DL_REDUCE_STATIC_SCRATCH_BYTES compiled into the library, shared by
 * every handle on a device. No counterpart in the reference.
 *
 * nblocks: blocks of the one reduction launch, 1..DL_REDUCE_STATIC_MAX_BLOCKS
 * (0 = 304); larger values are rejected with DL_ERR_ARG and a message. The
 * sums are compensated and added in a fixed order, so repeated calls on the
 * same fields with the same nblocks return identical values; they agree with
 * dl_reduce to rounding (the order of the final additions differs).
 *
 * The first call on each device looks up the array's device address (once
 * per CUDA context of the device, with that device made current for the
 * call; after a cudaDeviceReset the next call looks it up again); make that
 * first call before any stream capture starts on the device. Each call clears
 * the array's 8-byte arrival counter on h's stream before its launch (a
 * memset, no allocation). Calls on one device must not
 * overlap in time (two streams, two handles or two host threads at once):
 * they share the array and would race. The call synchronises h's stream. */
#define DL_REDUCE_STATIC_MAX_BLOCKS 1216
#define DL_REDUCE_STATIC_SCRATCH_BYTES 253144
int dl_reduce_static(dl_handle* h, int nblocks, dl_diag* out);

/* Wait for all work of the handle; returns the first deferred error. */
int dl_sync(dl_handle* h);

/* Bracket kernel launches of the handle with CUDA events on its stream:
 * enable = n > 0 times every n-th launch (1: every launch; a larger n keeps the
 * events' own cost out of a timed run while still sampling it), 0 stops; resets
 * the counters (launches counts every launch either way). The reference times
 * its loop with MPI_Wtime and writes time.d (program/lbm_drop_xy.f90:785-864);
 * this is the per-kernel device-side equivalent. */
int dl_profile(dl_handle* h, int enable);

/* Synchronise, then report and reset the launch counters and event times. */
int dl_profile_read(dl_handle* h, dl_profile_stats* out);

/* Launch-shape knobs of the fused kernel (no reference counterpart: the
 * reference fixes its loop structure at compile time). key "lz": z planes
 * marched by one block (1..nz); "lz" = 0 restores the default. "prefetch" 0|1:
 * bulk L2 prefetch of the next plane's pulled rows. "pipeline" 0|1 (single
 * phase): the next plane's pulls held in registers. "projection" 0|1 (band
 * forcing, default 1): the projection of the new u on the band modes done by
 * each block of the fused step after its march, else by a launch of its own;
 * both give the same coefficients up to the FP32 summation order. "push" 0|1
 * (FP32, default 1): step in the push form where eligible (read-only keys
 * "push_eligible" and "pushed" report it). "stage" (push form) 0: the next
 * plane's populations loaded into registers (two-phase default); 1: staged in
 * shared memory by per-thread asynchronous copies (single-phase default); 2:
 * staged by two tensor (TMA) copies per plane completing on an mbarrier
 * (nx a multiple of 32 and ny of 8, else DL_ERR_UNSUPPORTED); all three give
 * the same bits. "wait_ns" (stage 2, default 2e9): the time limit of a
 * block's wait for its staged plane; when it runs out the block stops
 * waiting and dl_sync returns DL_ERR_TIMEOUT. "stage_extra_tx" (stage 2,
 * default 0; for tests of that limit): bytes the mbarrier expects beyond the
 * copies', so that no wait completes. Read back with dl_get_option. Returns
 * DL_ERR_ARG for an unknown key or value. */
int dl_set_option(dl_handle* h, const char* key, int64_t value);
int dl_get_option(dl_handle* h, const char* key, int64_t* value);

/* Copy the last error message of the handle into buf (NUL-terminated). */
int dl_last_error(dl_handle* h, char* buf, int buflen);

/* Connected components of the sites with phi >= (phi1 + phi2)/2 on the
 * periodic lattice (droplet labelling of program/percolation.f90:108-295,
 * made complete across the periodic boundaries). connectivity: 6 (faces),
 * 14 (faces + xz and yz edges, the reference's neighbour set made symmetric),
 * 18 (faces + edges) or 26. Writes the number of droplets, up to max_volumes
 * volumes (site counts, decreasing) and, if labels is not NULL, nx*ny*nz
 * labels (0 = continuous phase, k = k-th largest droplet, x fastest). */
int dl_label_droplets(dl_handle* h, int connectivity, int32_t* labels, int64_t* ndrops, double* volumes,
                      int64_t max_volumes);

/* ---- device state and the hand-written adjoint (FP32 form) ---------------------
 * No reference counterpart: the reference has no derivatives. The adjoint runs
 * the reverse of dl_step for a loss on the final phi, with the caller driving
 * checkpointing: save states with dl_save_state (device memory of
 * dl_state_floats floats), recompute segments with dl_load_state + dl_step,
 * and walk them backwards with dl_adjoint_step. It covers the shear-droplet
 * physics (walls, static force; viscosity ratio 1, or another ratio in the
 * DL_VISC_FIXED mode), the Smagorinsky eddy viscosity (LES, A_nu = 0) and the
 * band force (DL_FORCE_SPECTRAL), i.e. the forced-turbulence step of
 * program/lbm_drop_iht_xy.f90:1016-1026. */

/* Number of FP32 values of one full device state (populations and fields;
 * dl_save_state / dl_load_state / dl_adjoint_init). */
int dl_state_floats(dl_handle* h, int64_t* n);

/* Copy the current state to / from caller-owned device memory. */
int dl_save_state(dl_handle* h, void* d_dst);
int dl_load_state(dl_handle* h, const void* d_src);

/* Start the reverse pass from dLoss/dphi of the final fields (device, N floats). */
int dl_adjoint_begin(dl_handle* h, const float* d_dloss_dphi);

/* The part of a state that the reverse of one step reads (f and the fields,
 * and with LES or a viscosity ratio g as well: dl_adjoint_state_floats FP32
 * values, 20 or 35 per site): what the recomputed segment keeps per step, written by
 * dl_save_adjoint_state. */
int dl_adjoint_state_floats(dl_handle* h, int64_t* n);
int dl_save_adjoint_state(dl_handle* h, void* d_dst);

/* Reverse of time step `step` (1-based); d_state_before is the adjoint state
 * (dl_save_adjoint_state) taken before that step. */
int dl_adjoint_step(dl_handle* h, const void* d_state_before, int64_t step);

/* Reverse of dl_init_equilibrium from the initial state: writes dLoss/dphi0. */
int dl_adjoint_init(dl_handle* h, const void* d_state0, float* d_dloss_dphi0);

/* Accumulated parameter gradients: dLoss/dkappaf, dLoss/dkappag,
 * dLoss/dtauf, dLoss/dU (top-wall x velocity; bottom = -U). */
int dl_adjoint_grads(dl_handle* h, double* grads4);

/* ---- batched ensembles -------------------------------------------------------
 * The reference runs ensemble members either as Nxall*Nzall replica groups of
 * MPI ranks (MPI_Comm_Split, program/lbm_omp_drop.f90:149-166) or as a
 * sequential loop over cases (DO case_num, program/lbm_drop_iht_xy_many.f90:1211).
 * Here the members (each its own domain size and parameters, one common form
 * FP32 or FP16, one common LES setting and force mode) step together: every
 * step is one persistent launch over all members' tiles, and pairs of steps
 * are replayed from a captured CUDA graph. */
typedef struct dl_batch dl_batch;

/* params[m] and dims[3*m .. 3*m+2] = nx, ny, nz of member m. */
int dl_batch_create(const dl_params* params, const int* dims, int nmembers, int form, dl_batch** out);

/* The handle of member m, for dl_set_fields, dl_init_equilibrium,
 * dl_set_force, dl_get_fields, dl_reduce, ... (owned by the batch; do not
 * dl_destroy it; do not dl_step it on its own). */
int dl_batch_member(dl_batch* b, int m, dl_handle** member);

/* Run every member's work on this cudaStream_t. */
int dl_batch_set_stream(dl_batch* b, void* cuda_stream);

/* Advance every member by nsteps steps. Default: each member takes its own
 * one-launch steps (as dl_step) on one of up to 16 streams forked from the
 * batch stream and joined back to it before the call returns (the blocks of
 * many members fill the GPU together; launch accounting on each member's
 * handle). With "persistent" = 1: one persistent launch per step over all
 * members' tiles (members in step with each other; accounting on member 0). */
int dl_batch_step(dl_batch* b, int nsteps);

/* Knobs: "persistent" 0|1 (the mode above, default 0); "lz" z planes per
 * block or work item (default 32, at most a member's nz); "blocks_per_sm"
 * persistent blocks per SM (1 or 2); "graph" 1 = replay step pairs of the
 * persistent launch from a CUDA graph. */
int dl_batch_set_option(dl_batch* b, const char* key, int64_t value);
int dl_batch_get_option(dl_batch* b, const char* key, int64_t* value);

int dl_batch_destroy(dl_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* DROPLET_GB300_H */
