/*
 * goldnc_driver.c -- a GoldenC-style program (the structure of
 * origin/GoldenC/src/main.c:8-10,51-79: globals f, v, gDelta; data
 * g = A(phantom); MumfordShah; results written out) linked against
 * libat_engine.so, used by the drop-in tests.
 *
 *   goldnc_driver <phantom.bin> <f_out.bin> <v_out.bin> [iter_alt]
 * phantom.bin: 512*512 little-endian doubles, row-major; outputs likewise
 * (binary instead of the reference's 6-decimal text).
 */
#include <stdio.h>
#include <stdlib.h>

#include "goldnc.h"

double init_f[512][512];
double f[512][512], v[512][512];
double gDelta[180][767];

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s phantom.bin f_out.bin v_out.bin [iter_alt]\n", argv[0]);
        return 2;
    }
    FILE *fin = fopen(argv[1], "rb");
    if (!fin || fread(init_f, sizeof(double), 512 * 512, fin) != 512 * 512) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    fclose(fin);
    if (argc > 4) goldnc_set_iterations(atoi(argv[4]), 10, 10);
    A(gDelta, init_f);
    if (goldnc_status() != 0) return 1;
    MumfordShah(1000, 0.002, 0.0001);
    if (goldnc_status() != 0) return 1;
    FILE *fo = fopen(argv[2], "wb");
    FILE *vo = fopen(argv[3], "wb");
    if (!fo || !vo) return 2;
    fwrite(f, sizeof(double), 512 * 512, fo);
    fwrite(v, sizeof(double), 512 * 512, vo);
    fclose(fo);
    fclose(vo);
    return 0;
}
