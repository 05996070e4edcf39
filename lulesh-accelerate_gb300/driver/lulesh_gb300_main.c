/*
 * lulesh_gb300_main.c -- a C host of the GB300 step, in the shape of the
 * reference driver's main() (reference/C/LULESH-OMP.cc:2960-3227): build the
 * Sedov problem, loop TimeIncrement + LagrangeLeapFrog until stoptime, print
 * the iteration count, the final origin energy and the plane-0 symmetry test
 * in the reference's format.  It uses only include/lulesh_gb300.h.
 *
 * Usage: lulesh_gb300_main S [--init v1|v2] [--split] [--cycles N] [--calls]
 *                          [--output PATTERN] [--xyz FILE]
 *        lulesh_gb300_main -u FILE.lmesh [--split] [--cycles N] [--calls]
 *                          [--output PATTERN] [--xyz FILE]
 *   -u       an unstructured mesh file, as the reference's GPU driver takes it
 *            (reference/CUDA/lulesh-kepler-singlegpu/lulesh.cu:3321-3329);
 *            the plane-0 symmetry test is then skipped, as there
 *   --calls  drive the loop from the host, one lulesh_time_increment +
 *            lulesh_lagrange_leapfrog call per cycle, as the reference's loop
 *            does (default: one lulesh_run call)
 *   --output write the state before every cycle to PATTERN formatted with the
 *            cycle number (lulesh_dump_domain), as the Haskell host's
 *            --output does with writeDomain (src/Main.hs:85-100); implies
 *            --calls
 *   --xyz    write the final node positions to FILE in the text layout of
 *            the reference GPU driver's write_solution
 *            (reference/CUDA/lulesh-kepler-singlegpu/lulesh.cu:3451-3470):
 *            per node its index (%10d) and x, y, z (%.10f), one per line
 */
#include "lulesh_gb300.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

int main(int argc, char **argv)
{
    if (argc < 2 || (!strcmp(argv[1], "-u") && argc < 3)) {
        fprintf(stderr, "usage: %s S [--init v1|v2] [--split] [--cycles N] [--calls]\n"
                        "       %s -u FILE.lmesh [--split] [--cycles N] [--calls]\n", argv[0], argv[0]);
        return 2;
    }
    const char *lmesh = !strcmp(argv[1], "-u") ? argv[2] : NULL;
    const int s = lmesh ? 0 : atoi(argv[1]);
    int init = LULESH_INIT_V2, precision = LULESH_PRECISION_FP64, cap = 0, calls = 0;
    const char *output = NULL, *xyz = NULL;
    for (int i = lmesh ? 3 : 2; i < argc; ++i) {
        if (!strcmp(argv[i], "--init") && i + 1 < argc) init = strcmp(argv[++i], "v1") ? LULESH_INIT_V2 : LULESH_INIT_V1;
        else if (!strcmp(argv[i], "--split")) precision = LULESH_PRECISION_SPLIT;
        else if (!strcmp(argv[i], "--cycles") && i + 1 < argc) cap = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--calls")) calls = 1;
        else if (!strcmp(argv[i], "--output") && i + 1 < argc) { output = argv[++i]; calls = 1; }
        else if (!strcmp(argv[i], "--xyz") && i + 1 < argc) xyz = argv[++i];
        else {
            fprintf(stderr, "unknown argument %s\n", argv[i]);
            return 2;
        }
    }
    lulesh_ctx *ctx = NULL;
    int rc = lmesh ? lulesh_create_lmesh(lmesh, precision, NULL, &ctx)
                   : lulesh_create(s, init, precision, NULL, &ctx);
    if (rc) {
        fprintf(stderr, "lulesh_create: %d %s\n", rc, lulesh_last_error(NULL));
        return 1;
    }
    lulesh_params prm;
    lulesh_get_params(ctx, &prm);

    struct timeval t0, t1;
    gettimeofday(&t0, NULL);
    int cycles = 0;
    if (calls) {
        lulesh_scalars sc;
        lulesh_get_scalars(ctx, &sc);
        while (sc.time < prm.stoptime && (cap <= 0 || cycles < cap)) {
            if (output && (rc = lulesh_dump_domain(ctx, output, cycles))) break;
            if ((rc = lulesh_time_increment(ctx)) || (rc = lulesh_lagrange_leapfrog(ctx))) break;
            lulesh_get_scalars(ctx, &sc);
            ++cycles;
        }
    } else {
        rc = lulesh_run(ctx, cap, &cycles);
    }
    gettimeofday(&t1, NULL);
    if (rc) {
        fprintf(stderr, "step failed: %d %s\n", rc, lulesh_last_error(ctx));
        lulesh_destroy(ctx);
        return 1;
    }
    const double elapsed = (double)(t1.tv_sec - t0.tv_sec) + 1e-6 * (double)(t1.tv_usec - t0.tv_usec);
    double e0 = 0.0, ma = 0.0, ta = 0.0, mr = 0.0;
    long ne = 0;
    lulesh_origin_energy(ctx, &e0);
    lulesh_sizes(ctx, NULL, &ne, NULL);
    if (!lmesh) lulesh_symmetry(ctx, &ma, &ta, &mr);

    printf("\n\nElapsed time = %12.6e\n\n", elapsed);
    printf("Run completed:  \n");
    if (lmesh) printf("   Problem size        =  %ld \n", ne);
    else printf("   Problem size        =  %i \n", s);
    printf("   Iteration count     =  %i \n", cycles);
    printf("   Final Origin Energy = %12.6e \n", e0);
    if (!lmesh) {
        printf("   Testing Plane 0 of Energy Array:\n");
        printf("        MaxAbsDiff   = %12.6e\n", ma);
        printf("        TotalAbsDiff = %12.6e\n", ta);
        printf("        MaxRelDiff   = %12.6e\n\n", mr);
    }
    if (xyz) {
        long nn = 0;
        lulesh_sizes(ctx, NULL, NULL, &nn);
        double *p = (double *)malloc(3 * (size_t)nn * sizeof(double));
        FILE *f = p ? fopen(xyz, "w") : NULL;
        if (!f || lulesh_get_field(ctx, "x", p, nn) || lulesh_get_field(ctx, "y", p + nn, nn) ||
            lulesh_get_field(ctx, "z", p + 2 * nn, nn)) {
            fprintf(stderr, "cannot write %s\n", xyz);
            if (f) fclose(f);
            free(p);
            lulesh_destroy(ctx);
            return 1;
        }
        for (long i = 0; i < nn; ++i)
            fprintf(f, "%10ld\n%.10f\n%.10f\n%.10f\n", i, p[i], p[nn + i], p[2 * nn + i]);
        fclose(f);
        free(p);
    }
    printf("{\"cycles\": %d, \"origin_energy\": %.17e, \"max_rel_diff\": %.17e}\n", cycles, e0, mr);
    lulesh_destroy(ctx);
    return 0;
}
