/*
 * gen_main.c -- wfe.gen: write a synthetic pair file in the reference's
 * format (">pattern", "<text").
 *
 *   wfe.gen OUT N LEN_MIN [LEN_MAX [P_MIN [P_MAX [SEED [FIRST]]]]]
 */
#include <stdio.h>
#include <stdlib.h>

#include "wfe_gen.h"

int main(int argc, char** argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s OUT N LEN_MIN [LEN_MAX [P_MIN [P_MAX [SEED [FIRST]]]]]\n", argv[0]);
        return 1;
    }
    wfe_gen_config c;
    const size_t n = strtoull(argv[2], NULL, 10);
    c.len_min = (uint32_t)strtoul(argv[3], NULL, 10);
    c.len_max = argc > 4 ? (uint32_t)strtoul(argv[4], NULL, 10) : c.len_min;
    c.p_min = argc > 5 ? atof(argv[5]) : 0.05;
    c.p_max = argc > 6 ? atof(argv[6]) : c.p_min;
    c.seed = argc > 7 ? strtoull(argv[7], NULL, 10) : 1;
    const unsigned long long first = argc > 8 ? strtoull(argv[8], NULL, 10) : 0;
    if (c.len_max < c.len_min || c.len_min == 0) return 1;
    return wfe_gen_file(&c, first, n, argv[1]) == 0 ? 0 : 2;
}
