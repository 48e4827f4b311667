/* A plain C host of the library: what a Fortran or C main loop does through
 * include/droplet_gb300.h, with no Python and no CUDA headers. Builds a
 * periodic box with one droplet, steps it in the form given on the command
 * line (64, 32 or 16) and prints the diagnostics as one line of numbers:
 *   phi_sum p_sum mom_x mom_y mom_z vol_count phi_min phi_max step
 * Usage: abi_host <form> <nx> <ny> <nz> <steps> [phi_out]
 * phi_out: file to receive the initial phi (raw FP64, x fastest). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "droplet_gb300.h"

static int check(dl_handle* h, int rc, const char* what) {
    if (rc != DL_OK) {
        char msg[512] = "";
        if (h) dl_last_error(h, msg, (int)sizeof msg);
        fprintf(stderr, "%s: %s (%s)\n", what, dl_status_string(rc), msg);
        exit(1);
    }
    return rc;
}

int main(int argc, char** argv) {
    if (argc != 6 && argc != 7) {
        fprintf(stderr, "usage: %s form nx ny nz steps [phi_out]\n", argv[0]);
        return 2;
    }
    const int form = atoi(argv[1]), nx = atoi(argv[2]), ny = atoi(argv[3]), nz = atoi(argv[4]);
    const int steps = atoi(argv[5]);
    /* the parameter set of program/lbm_drop_xy.f90 (module globals) */
    dl_params p = {0};
    p.ds = 1.0;
    p.tauf = 0.8;
    p.kappaf = 0.01;
    p.kappag = 2e-3;
    p.phi1 = 2.211;
    p.phi2 = 4.895;
    p.a = 9.0 / 49.0;
    p.b = 2.0 / 21.0;
    p.T = 0.55;
    p.nu1 = 0.1;
    p.nu2 = 0.1;
    p.visc_mode = DL_VISC_MINMAX;
    p.kc = 3;
    dl_handle* h = NULL;
    check(NULL, dl_create(&p, nx, ny, nz, form, &h), "dl_create");
    const size_t n = (size_t)nx * ny * nz;
    double* f[5];
    for (int k = 0; k < 5; ++k) f[k] = (double*)calloc(n, sizeof(double));
    /* phi~ = tanh((R - r) / 1.5) around the box centre, u = 0, p = 1/3 */
    const double R = (nx < ny ? (nx < nz ? nx : nz) : (ny < nz ? ny : nz)) / 4.0;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const size_t s = (size_t)x + (size_t)nx * ((size_t)y + (size_t)ny * z);
                const double dx = x - (nx - 1) / 2.0, dy = y - (ny - 1) / 2.0, dz = z - (nz - 1) / 2.0;
                const double t = tanh((R - sqrt(dx * dx + dy * dy + dz * dz)) / 1.5);
                f[0][s] = p.phi1 + 0.5 * (t + 1.0) * (p.phi2 - p.phi1);
                f[4][s] = 1.0 / 3.0;
            }
    if (argc == 7) {
        FILE* fp = fopen(argv[6], "wb");
        if (!fp || fwrite(f[0], sizeof(double), n, fp) != n) {
            fprintf(stderr, "cannot write %s\n", argv[6]);
            return 1;
        }
        fclose(fp);
    }
    check(h, dl_set_fields(h, f[0], f[1], f[2], f[3], f[4]), "dl_set_fields");
    check(h, dl_init_equilibrium(h), "dl_init_equilibrium");
    /* every step's phi range in a page-locked mirror of 2 slots, checked
     * against dl_get_minmax: the pull form writes step k's range into slot
     * k % 2; the push form (FP32) writes the range of the state a step
     * loads, step k-1's, into slot (k-1) % 2 */
    double* mirror = NULL;
    check(h, dl_host_alloc(4 * sizeof(double), (void**)&mirror), "dl_host_alloc");
    check(h, dl_set_minmax_mirror(h, mirror, 2), "dl_set_minmax_mirror");
    int64_t push = 0;
    check(h, dl_get_option(h, "push_eligible", &push), "dl_get_option");
    int mismatches = 0;
    for (int k = 1; k <= steps; ++k) {
        double mn0, mx0;
        check(h, dl_get_minmax(h, &mn0, &mx0), "dl_get_minmax");
        check(h, dl_step(h, 1), "dl_step");
        check(h, dl_sync(h), "dl_sync");
        double mn, mx;
        check(h, dl_get_minmax(h, &mn, &mx), "dl_get_minmax");
        if (push) {
            /* before the first step the range is init's (phi1, phi2), not a computed one */
            if (k > 1 && (mirror[2 * ((k - 1) % 2)] != mn0 || mirror[2 * ((k - 1) % 2) + 1] != mx0)) ++mismatches;
        } else if (mirror[2 * (k % 2)] != mn || mirror[2 * (k % 2) + 1] != mx) {
            ++mismatches;
        }
    }
    check(h, dl_set_minmax_mirror(h, NULL, 0), "dl_set_minmax_mirror");
    check(h, dl_host_free(mirror), "dl_host_free");
    if (mismatches) {
        fprintf(stderr, "minmax mirror: %d of %d steps differ from dl_get_minmax\n", mismatches, steps);
        return 1;
    }
    dl_diag d;
    check(h, dl_reduce(h, &d), "dl_reduce");
    printf("%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %lld\n", d.phi_sum, d.p_sum, d.mom[0], d.mom[1],
           d.mom[2], d.vol_count, d.phi_min, d.phi_max, (long long)d.step);
    check(h, dl_destroy(h), "dl_destroy");
    for (int k = 0; k < 5; ++k) free(f[k]);
    return 0;
}
