/*
 * regions_driver.cc -- prints the element-to-region assignment of the
 * UNMODIFIED reference LULESH 2.0 (reference/C/lulesh-2.0.3), for pinning
 * the library's restatement of Domain::CreateRegionIndexSets
 * (lulesh-init.cc:377-486).
 *
 * TEST INFRASTRUCTURE ONLY.  Linked with the reference's own sources (its
 * main() renamed by the preprocessor); this file only constructs a one-rank
 * Domain and prints regNumList.
 *
 * Usage: regions_dump S NUM_REGIONS BALANCE
 * Output: one JSON line {"s", "num_regions", "balance", "runs"} where runs is
 * the run-length encoding [[region, length], ...] of regNumList.
 */
#include "lulesh.h"

#include <cstdio>
#include <cstdlib>

int main(int argc, char **argv)
{
    if (argc != 4) {
        fprintf(stderr, "usage: %s S NUM_REGIONS BALANCE\n", argv[0]);
        return 2;
    }
    const int s = atoi(argv[1]), nr = atoi(argv[2]), balance = atoi(argv[3]);
    Domain dom(1, 0, 0, 0, s, 1, nr, balance, 1);
    printf("{\"s\": %d, \"num_regions\": %d, \"balance\": %d, \"runs\": [", s, nr, balance);
    Index_t i = 0;
    bool first = true;
    while (i < dom.numElem()) {
        Index_t j = i;
        while (j < dom.numElem() && dom.regNumList(j) == dom.regNumList(i)) ++j;
        printf("%s[%d, %d]", first ? "" : ", ", (int)dom.regNumList(i), (int)(j - i));
        first = false;
        i = j;
    }
    printf("]}\n");
    return 0;
}
