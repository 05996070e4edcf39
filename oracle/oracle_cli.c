/*
 * oracle_cli.c -- command-line driver of the oracle restatement.
 *
 * TEST INFRASTRUCTURE ONLY: the "port" CPU baseline and a cross-check of the
 * oracle against the reference build.  Prints one JSON line in the same
 * format as ref_driver.cc.
 *
 * Usage: lulesh_oracle S [--init v1|v2] [--cycles N] [--warmup W]
 * (--warmup W: W cycles run before the timed --cycles N.)
 */
#include "lulesh_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s S [--init v1|v2] [--cycles N]\n", argv[0]);
        return 2;
    }
    const int s = atoi(argv[1]);
    int init = LO_INIT_V2, cycles = 0, warmup = 0;
    for (int i = 2; i < argc; ++i) {
        if (!strcmp(argv[i], "--init") && i + 1 < argc) init = strcmp(argv[++i], "v1") ? LO_INIT_V2 : LO_INIT_V1;
        else if (!strcmp(argv[i], "--cycles") && i + 1 < argc) cycles = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--warmup") && i + 1 < argc) warmup = atoi(argv[++i]);
        else { fprintf(stderr, "unknown argument %s\n", argv[i]); return 2; }
    }
    lo_domain *d = lo_create(s, init);
    if (!d) return 2;
    double elapsed = 0.0;
    int rc = 0;
    if (warmup > 0) rc = lo_run(d, warmup, &elapsed);
    const int c0 = *lo_cycle(d);
    if (rc == 0) rc = lo_run(d, cycles, &elapsed);
    const int timed = *lo_cycle(d) - c0;
    double ma, ta, mr;
    lo_symmetry(d, &ma, &ta, &mr);
    long ne = 0;
    double *e = lo_field(d, "e", &ne);
    const int cyc = *lo_cycle(d);
    printf("{\"s\": %d, \"init\": \"%s\", \"rc\": %d, \"cycles\": %d, \"origin_energy\": %.17e, "
           "\"time\": %.17e, \"deltatime\": %.17e, \"dtcourant\": %.17e, \"dthydro\": %.17e, "
           "\"max_abs_diff\": %.17e, \"total_abs_diff\": %.17e, \"max_rel_diff\": %.17e, "
           "\"elapsed_s\": %.6f, \"timed_cycles\": %d, \"threads\": %d, \"mzone_cycles_per_s\": %.6f}\n",
           s, init == LO_INIT_V1 ? "v1" : "v2", rc, cyc, e[0], *lo_scalar(d, "time"),
           *lo_scalar(d, "deltatime"), *lo_scalar(d, "dtcourant"), *lo_scalar(d, "dthydro"),
           ma, ta, mr, elapsed, timed, lo_num_threads(),
           elapsed > 0 ? (double)ne * (double)timed / elapsed * 1e-6 : 0.0);
    lo_destroy(d);
    return rc == 0 ? 0 : 1;
}
