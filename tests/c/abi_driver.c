/* abi_driver.c -- a C caller of the library through include/rrtmg_sw_gb300.h
 * only: reads a clear-sky case, calls rrtmg_sw_ini_c and rrtmg_sw_c with
 * host arrays, writes the six outputs.
 *
 * Usage: abi_driver <input file> <output file>
 * Input: ncol, nlay (int32), then play, plev, tlay, h2ovmr, o3vmr, co2vmr,
 * ch4vmr, o2vmr, asdir, asdif, aldir, aldif, coszen (FP64, Fortran order).
 * Output: sizeof(rrtmg_sw_args) (int64), status (int32), then swuflx,
 * swdflx, swhr, swuflxc, swdflxc, swhrc. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rrtmg_sw_gb300.h"

static double *rd(FILE *f, size_t n) {
    double *p = (double *)malloc(n * sizeof(double));
    if (!p || fread(p, sizeof(double), n, f) != n) {
        fprintf(stderr, "short input\n");
        exit(2);
    }
    return p;
}

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t ncol, nlay;
    if (fread(&ncol, 4, 1, f) != 1 || fread(&nlay, 4, 1, f) != 1) return 2;
    const size_t C = (size_t)ncol, L = (size_t)nlay;
    rrtmg_sw_args a;
    memset(&a, 0, sizeof a);
    a.ncol = ncol; a.nlay = nlay; a.icld = 0; a.iaer = 0;
    a.play = rd(f, C * L); a.plev = rd(f, C * (L + 1)); a.tlay = rd(f, C * L);
    a.h2ovmr = rd(f, C * L); a.o3vmr = rd(f, C * L); a.co2vmr = rd(f, C * L);
    a.ch4vmr = rd(f, C * L); a.o2vmr = rd(f, C * L);
    a.asdir = rd(f, C); a.asdif = rd(f, C); a.aldir = rd(f, C); a.aldif = rd(f, C); a.coszen = rd(f, C);
    fclose(f);
    a.adjes = 1.0; a.dyofyr = 0; a.scon = 1360.85; a.isolvar = 0;
    a.inflgsw = 2; a.iceflgsw = 3; a.liqflgsw = 1; a.idelm = 1;
    double *out[6];
    const size_t n[6] = {C * (L + 1), C * (L + 1), C * L, C * (L + 1), C * (L + 1), C * L};
    for (int i = 0; i < 6; ++i) out[i] = (double *)calloc(n[i], sizeof(double));
    a.swuflx = out[0]; a.swdflx = out[1]; a.swhr = out[2];
    a.swuflxc = out[3]; a.swdflxc = out[4]; a.swhrc = out[5];
    int32_t rc = rrtmg_sw_ini_c(1.004e3);
    if (rc == 0) rc = rrtmg_sw_c(&a);
    if (rc) fprintf(stderr, "rrtmg_sw: %s\n", rrtmg_sw_errstr_c(rc));
    FILE *g = fopen(argv[2], "wb");
    if (!g) return 2;
    const int64_t sz = (int64_t)sizeof(rrtmg_sw_args);
    fwrite(&sz, 8, 1, g);
    fwrite(&rc, 4, 1, g);
    for (int i = 0; i < 6; ++i) fwrite(out[i], sizeof(double), n[i], g);
    fclose(g);
    rrtmg_sw_finalize_c();
    return rc == 0 ? 0 : 1;
}
