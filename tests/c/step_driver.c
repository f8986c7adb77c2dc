/*
 * step_driver.c -- a C program that drives libnsg through include/nsg.h the way the
 * reference's main() does once its step body is replaced (the sequence of the
 * integration patch): read an initial-conditions file into the reference's
 * particles[5][N] rows, create a context, upload the rows, step, look up tracked
 * particles by id after every step, download the rows, destroy the context.
 *
 *   step_driver <init file> <out file> <nsteps> <method> <dt> <max_subdiv> <lc_rule> <lc_radius>
 *
 * The init file is the reference's format (read_initial_conditions,
 * nsphere.c:2386-2487): int32 N, then N records of five doubles
 * (r, v_r, ell, id, mu).  The out file holds int32 N, int32 nsteps, int32 ntrack,
 * uint32 status word, the rows 0..3 after the last step (N doubles each), then for
 * every step the tracked particles' r, v_r, ell (ntrack doubles each) and their
 * array index (ntrack int32).  Exit status 0 on success; on a library error the
 * message of nsg_last_error is printed and the status is 1.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "nsg.h"

#define NTRACK 10

static int fail(nsg_ctx *ctx, const char *what, int rc)
{
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, nsg_last_error(ctx));
    if (ctx) nsg_destroy(ctx);
    return 1;
}

int main(int argc, char **argv)
{
    if (argc != 9) {
        fprintf(stderr, "usage: %s init out nsteps method dt max_subdiv lc_rule lc_radius\n", argv[0]);
        return 2;
    }
    const int nsteps = atoi(argv[3]);
    FILE *f = fopen(argv[1], "rb");
    if (!f) { perror(argv[1]); return 2; }
    int32_t n32 = 0;
    if (fread(&n32, 4, 1, f) != 1 || n32 <= 0) { fprintf(stderr, "bad init file\n"); fclose(f); return 2; }
    const int64_t n = n32;
    /* the reference's state: five separately allocated rows (nsphere.c:4656-4672) */
    double *particles[5];
    for (int c = 0; c < 5; c++) {
        particles[c] = (double *)malloc((size_t)n * sizeof(double));
        if (!particles[c]) { fprintf(stderr, "out of host memory\n"); return 2; }
    }
    for (int64_t i = 0; i < n; i++) {
        double rec[5];
        if (fread(rec, 8, 5, f) != 5) { fprintf(stderr, "short init file\n"); fclose(f); return 2; }
        for (int c = 0; c < 5; c++) particles[c][i] = rec[c];
    }
    fclose(f);

    nsg_params p;
    nsg_params_default(&p);
    p.method = atoi(argv[4]);
    p.dt = atof(argv[5]);
    p.max_subdiv = atoll(argv[6]);
    p.lc_rule = atoi(argv[7]);
    p.lc_radius = atof(argv[8]);

    nsg_ctx *ctx = NULL;
    int rc = nsg_create(&ctx, &p, NULL);
    if (rc != NSG_OK) return fail(NULL, "nsg_create", rc);
    rc = nsg_upload_particles(ctx, particles, n);
    if (rc != NSG_OK) return fail(ctx, "nsg_upload_particles", rc);

    int32_t ids[NTRACK];
    const int ntrack = n < NTRACK ? (int)n : NTRACK;
    for (int t = 0; t < ntrack; t++) ids[t] = t;    /* the reference tracks ids 0..9 (nsphere.c:5845-5866) */
    double *tr = (double *)malloc((size_t)nsteps * 3 * NTRACK * sizeof(double));
    int32_t *trank = (int32_t *)malloc((size_t)nsteps * NTRACK * sizeof(int32_t));
    if (!tr || !trank) { fprintf(stderr, "out of host memory\n"); return 2; }
    for (int j = 0; j < nsteps; j++) {
        rc = nsg_step(ctx, 1);
        if (rc != NSG_OK) return fail(ctx, "nsg_step", rc);
        double *o = tr + (size_t)j * 3 * NTRACK;
        rc = nsg_gather(ctx, ids, ntrack, o, o + NTRACK, o + 2 * NTRACK, trank + (size_t)j * NTRACK);
        if (rc != NSG_OK) return fail(ctx, "nsg_gather", rc);
    }
    rc = nsg_download_particles(ctx, particles);
    if (rc != NSG_OK) return fail(ctx, "nsg_download_particles", rc);
    rc = nsg_sync(ctx, -1);
    if (rc != NSG_OK && rc != NSG_EDEVICE) return fail(ctx, "nsg_sync", rc);
    uint32_t status = 0;
    rc = nsg_status(ctx, &status);
    if (rc != NSG_OK) return fail(ctx, "nsg_status", rc);
    nsg_destroy(ctx);

    FILE *g = fopen(argv[2], "wb");
    if (!g) { perror(argv[2]); return 2; }
    const int32_t hdr[3] = {n32, nsteps, ntrack};
    fwrite(hdr, 4, 3, g);
    fwrite(&status, 4, 1, g);
    for (int c = 0; c < 4; c++) fwrite(particles[c], 8, (size_t)n, g);
    for (int j = 0; j < nsteps; j++) {
        const double *o = tr + (size_t)j * 3 * NTRACK;
        for (int q = 0; q < 3; q++) fwrite(o + q * NTRACK, 8, (size_t)ntrack, g);
        fwrite(trank + (size_t)j * NTRACK, 4, (size_t)ntrack, g);
    }
    fclose(g);
    for (int c = 0; c < 5; c++) free(particles[c]);
    free(tr);
    free(trank);
    return 0;
}
