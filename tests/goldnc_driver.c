/*
 * goldnc_driver.c -- a GoldenC-style program (the structure of
 * origin/GoldenC/src/main.c:8-10,51-79: globals f, v, gDelta; data
 * g = A(phantom); MumfordShah; results written out) linked against
 * libat_engine.so, used by the drop-in tests.
 *
 *   goldnc_driver <phantom.bin> <f_out.bin> <v_out.bin> [iter_alt]
 *       phantom.bin: 512*512 little-endian doubles, row-major; outputs
 *       likewise (binary, for exact comparisons)
 *   goldnc_driver --text <dir> [iter_alt]
 *       GoldenC's own files: reads <dir>/phantom.dat (512 x 512 numbers,
 *       whitespace separated, row-major, read with fscanf "%lf" as
 *       main.c:52-58) and writes <dir>/I_result.txt and <dir>/E_result.txt
 *       ("%f " per value, a newline after each row, as main.c:63-77)
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "goldnc.h"

double init_f[512][512];
double f[512][512], v[512][512];
double gDelta[180][767];

static int read_text(const char *path) {
    FILE *fp = fopen(path, "r");
    if (!fp) return 0;
    for (int i = 0; i < 512; i++)
        for (int j = 0; j < 512; j++)
            if (fscanf(fp, "%lf", &init_f[i][j]) != 1) {
                fclose(fp);
                return 0;
            }
    fclose(fp);
    return 1;
}

static int write_text(const char *path, double a[512][512]) {
    FILE *fp = fopen(path, "w");
    if (!fp) return 0;
    for (int i = 0; i < 512; i++) {
        for (int j = 0; j < 512; j++) fprintf(fp, "%f ", a[i][j]);
        fprintf(fp, "\n");
    }
    return fclose(fp) == 0;
}

static int reconstruct(void) {
    A(gDelta, init_f);
    if (goldnc_status() != 0) return 1;
    MumfordShah(1000, 0.002, 0.0001);
    return goldnc_status() != 0;
}

int main(int argc, char **argv) {
    if (argc >= 3 && strcmp(argv[1], "--text") == 0) {
        char path[4096];
        snprintf(path, sizeof(path), "%s/phantom.dat", argv[2]);
        if (!read_text(path)) {
            fprintf(stderr, "cannot read %s\n", path);
            return 2;
        }
        if (argc > 3) goldnc_set_iterations(atoi(argv[3]), 10, 10);
        if (reconstruct()) return 1;
        snprintf(path, sizeof(path), "%s/I_result.txt", argv[2]);
        if (!write_text(path, f)) return 2;
        snprintf(path, sizeof(path), "%s/E_result.txt", argv[2]);
        if (!write_text(path, v)) return 2;
        return 0;
    }
    if (argc < 4) {
        fprintf(stderr, "usage: %s phantom.bin f_out.bin v_out.bin [iter_alt]\n"
                        "       %s --text <dir> [iter_alt]\n", argv[0], argv[0]);
        return 2;
    }
    FILE *fin = fopen(argv[1], "rb");
    if (!fin || fread(init_f, sizeof(double), 512 * 512, fin) != 512 * 512) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    fclose(fin);
    if (argc > 4) goldnc_set_iterations(atoi(argv[4]), 10, 10);
    if (reconstruct()) return 1;
    FILE *fo = fopen(argv[2], "wb");
    FILE *vo = fopen(argv[3], "wb");
    if (!fo || !vo) return 2;
    fwrite(f, sizeof(double), 512 * 512, fo);
    fwrite(v, sizeof(double), 512 * 512, vo);
    fclose(fo);
    fclose(vo);
    return 0;
}
