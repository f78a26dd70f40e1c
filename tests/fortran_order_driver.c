/* fortran_order_driver.c -- the calling sequence of the patched 2DENSE driver
 * (source/utility/general_main.f90:23-38 with the four per-stage calls replaced by dense_stage),
 * written in C the way the Fortran module include/dense_gpu.f90 passes its arguments: the
 * configuration struct by reference, the handle by value, scalars by value or by reference as the
 * bind(C) interfaces declare them, and the block arrays as column-major host arrays
 * cons(NIp,NJp,4), prim(NIp,NJp,6), x(ni,nj), y(ni,nj) with four ghost layers.
 *
 *   fortran_order_driver <benchmark> <splitting> <recon> <ni> <nj> <nsteps> <strict> <out.bin>
 *
 * Writes cons after nsteps steps (NIp*NJp*4 doubles, column-major), then current_time and dt,
 * to out.bin. Exit status 0 on success, else the failing call's status code.
 */
#include <stdio.h>
#include <stdlib.h>

#include "dense2d.h"

static int check(int rc, const char* what, dense_handle_t* h) {
    if (rc != DENSE_OK) fprintf(stderr, "%s: %d %s\n", what, rc, dense_last_error(h));
    return rc;
}

int main(int argc, char** argv) {
    if (argc != 9) {
        fprintf(stderr, "usage: %s bench split recon ni nj nsteps strict out.bin\n", argv[0]);
        return 2;
    }
    dense_config_t cfg;
    if (check(dense_config_default(&cfg), "dense_config_default", NULL)) return 1;
    cfg.benchmark = atoi(argv[1]);
    cfg.splitting = atoi(argv[2]);
    cfg.recon = atoi(argv[3]);
    cfg.ni = atoi(argv[4]);
    cfg.nj = atoi(argv[5]);
    const int nsteps = atoi(argv[6]);
    cfg.strict = atoi(argv[7]);
    cfg.cfl = 0.5;
    cfg.var_eps = 5.0;
    cfg.var_xc = 5.0;
    cfg.var_yc = 5.0;
    const size_t nip = (size_t)cfg.ni + 8, njp = (size_t)cfg.nj + 8;
    double* cons = calloc(nip * njp * 4, sizeof(double));
    double* prim = calloc(nip * njp * 6, sizeof(double));
    double* x = calloc((size_t)cfg.ni * cfg.nj, sizeof(double));
    double* y = calloc((size_t)cfg.ni * cfg.nj, sizeof(double));
    if (!cons || !prim || !x || !y) return 3;

    /* init_general */
    int rc = check(dense_init_setup(&cfg, cons, prim, x, y), "dense_init_setup", NULL);
    if (rc) return rc;
    /* call dense_check(dense_create(cfg, h)); call dense_check(dense_upload(h, cons, prim, x, y)) */
    dense_handle_t* h = NULL;
    if ((rc = check(dense_create(&cfg, &h), "dense_create", NULL))) return rc;
    if ((rc = check(dense_upload(h, cons, prim, x, y), "dense_upload", h))) return rc;

    double current_time = 0.0, dt = cfg.dt;
    int current_step = 0;
    /* do while((current_time.lt.total_time).and.(current_step.lt.total_step)) */
    while (current_step < nsteps) {
        for (int irk = 1; irk <= cfg.stages; ++irk)
            if ((rc = check(dense_stage(h, irk, current_time, &dt), "dense_stage", h))) return rc;
        current_step = current_step + 1;
        current_time = current_time + dt;
    }
    if ((rc = check(dense_download(h, cons, prim), "dense_download", h))) return rc;
    unsigned flags = 0;
    if ((rc = check(dense_status(h, &flags), "dense_status", h))) return rc;
    dense_destroy(h);

    FILE* f = fopen(argv[8], "wb");
    if (!f) return 4;
    size_t n = fwrite(cons, sizeof(double), nip * njp * 4, f);
    n += fwrite(&current_time, sizeof(double), 1, f);
    n += fwrite(&dt, sizeof(double), 1, f);
    fclose(f);
    free(cons);
    free(prim);
    free(x);
    free(y);
    return n == nip * njp * 4 + 2 ? (flags & (DENSE_FLAG_NAN | DENSE_FLAG_NEG_RHO) ? 5 : 0) : 4;
}
