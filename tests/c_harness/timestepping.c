/*
 * A C driver of libsparc_gpu in the call order of the reference's Fortran
 * driver: Initialize_all -> solar_data -> DETERMINE_STATUS -> TIMESTEPPING
 * (driver.f90:398-476), i.e. sparc_gpu_create -> sparc_gpu_set_background ->
 * sparc_gpu_set_source -> { sparc_gpu_step(1); at mod(time, steps) == 0 the
 * surface vz at o_rad by sparc_gpu_get_field } -> sparc_gpu_destroy.
 *
 * usage: timestepping nx ny nz xlength_cm npmlbot npmltop precision nsteps
 *                     background.txt plane.bin series.bin out.bin
 *   background.txt  the six columns of the reference's background file
 *                   (r/R_sun, c, rho, p, g, Gamma_1), nz rows, bottom first
 *   plane.bin       nx*ny doubles: the forcing plane
 *   series.bin      doubles: the source time series, one per time step
 *   out.bin         written: one record of nx*ny doubles per output, the
 *                   layout of vz_cc.bin (write_binary_seq_2D)
 * Prints "records N" and exits 0, or prints the library's error and exits 1.
 */
#include <stdio.h>
#include <stdlib.h>

#include "sparc_gpu.h"

static int check(sparc_ctx* ctx, int rc, const char* what) {
    if (rc == SPARC_OK) return 0;
    fprintf(stderr, "%s: %s (%s)\n", what, sparc_gpu_errstr(rc), ctx ? sparc_gpu_last_error(ctx) : "");
    return 1;
}

static double* read_doubles(const char* path, long* n) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    *n = bytes / (long)sizeof(double);
    double* v = (double*)malloc((size_t)(*n > 0 ? *n : 1) * sizeof(double));
    if (v && fread(v, sizeof(double), (size_t)*n, f) != (size_t)*n) {
        free(v);
        v = NULL;
    }
    fclose(f);
    return v;
}

int main(int argc, char** argv) {
    if (argc != 13) {
        fprintf(stderr, "usage: %s nx ny nz xlength npmlbot npmltop precision nsteps background plane series out\n",
                argv[0]);
        return 2;
    }
    sparc_params p = {0};
    p.nx = atoi(argv[1]);
    p.ny = atoi(argv[2]);
    p.nz = atoi(argv[3]);
    p.xlength = atof(argv[4]);
    p.ylength = p.xlength;
    p.npmlbot = atoi(argv[5]);
    p.npmltop = atoi(argv[6]);
    p.precision = atoi(argv[7]);
    const int nsteps = atoi(argv[8]);
    p.option = (p.ny == 1) ? 17 : 4;
    p.compute_forward = 1;
    p.damp_waves = 1;
    p.nsrc = 1;
    p.timestep = 2.0;
    p.excitdep = -1.5e7;
    p.obsheight = 2.0e7;
    p.cadforcing = 30.0;
    p.outputcad = 30.0;
    p.nupeak = 0.0017;
    p.nuwidth = 0.0055;
    p.solartime = 1.0;

    /* solar_data: the six columns, bottom first */
    const int nz = p.nz;
    double* col = (double*)malloc((size_t)6 * nz * sizeof(double));
    FILE* fb = fopen(argv[9], "r");
    if (!col || !fb) { fprintf(stderr, "cannot read %s\n", argv[9]); return 1; }
    for (int k = 0; k < nz; ++k)
        for (int c = 0; c < 6; ++c)
            if (fscanf(fb, "%lf", &col[c * nz + k]) != 1) { fprintf(stderr, "short background file\n"); return 1; }
    fclose(fb);
    long nplane = 0, nseries = 0;
    double* plane = read_doubles(argv[10], &nplane);
    double* series = read_doubles(argv[11], &nseries);
    if (!plane || !series || nplane != (long)p.nx * p.ny) { fprintf(stderr, "bad source files\n"); return 1; }

    sparc_ctx* ctx = NULL;
    if (check(NULL, sparc_gpu_create(&p, &ctx), "sparc_gpu_create")) return 1;
    if (check(ctx, sparc_gpu_set_background(ctx, col, col + nz, col + 2 * nz, col + 3 * nz, col + 4 * nz,
                                            col + 5 * nz), "sparc_gpu_set_background")) return 1;
    if (check(ctx, sparc_gpu_set_source(ctx, 0, SPARC_SRC_SERIES, plane, 1, series, (int)nseries),
              "sparc_gpu_set_source")) return 1;
    double info[16];
    if (check(ctx, sparc_gpu_info(ctx, info, NULL, NULL), "sparc_gpu_info")) return 1;
    const int o_rad = (int)info[1], steps = (int)info[4];

    FILE* out = fopen(argv[12], "wb");
    double* rec = (double*)malloc((size_t)p.nx * p.ny * sizeof(double));
    if (!out || !rec) { fprintf(stderr, "cannot write %s\n", argv[12]); return 1; }
    int nrec = 0;
    for (int time = 0; time < nsteps; ++time) {          /* TIMESTEPPING: time = i */
        if (check(ctx, sparc_gpu_step(ctx, 1), "sparc_gpu_step")) return 1;      /* call step() */
        if (time % steps == 0) {                                                 /* driver.f90:455 */
            if (check(ctx, sparc_gpu_get_field(ctx, 0, SPARC_V_Z, o_rad, rec), "sparc_gpu_get_field")) return 1;
            fwrite(rec, sizeof(double), (size_t)p.nx * p.ny, out);
            ++nrec;
        }
    }
    fclose(out);
    if (check(ctx, sparc_gpu_sync(ctx, 1), "sparc_gpu_sync")) return 1;
    sparc_gpu_destroy(ctx);
    free(rec); free(plane); free(series); free(col);
    printf("records %d\n", nrec);
    return 0;
}
