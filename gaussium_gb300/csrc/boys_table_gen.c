/*
 * Writes the Boys-function grid used by the ERI kernels as a C header of hexadecimal
 * floating-point literals (exact), computed in long double:
 *
 *   row k (T_k = k / BOYS_INV_H, k = 0..BOYS_ROWS-1):
 *     col m = F_m(T_k) for m = 0..BOYS_NCOL-2,   col BOYS_NCOL-1 = exp(-T_k)
 *
 * F_top(T) comes from the series F_m(T) = exp(-T) sum_i (2T)^i / ((2m+1)(2m+3)...(2m+2i+1)),
 * whose terms are all positive, and the lower orders from the downward recursion
 * F_{m-1} = (2T F_m + exp(-T)) / (2m-1), which is stable.  The kernels evaluate
 * F_m(T) by a Taylor expansion about the nearest grid point and the downward recursion
 * (Helgaker, Jorgensen & Olsen, Molecular Electronic-Structure Theory, sec. 9.8.2).
 * The grid reaches T = 80, beyond which exp(-T) < 2e-35 changes no F_m (m <= 16) in double
 * precision, so the kernels' large-T branch needs no exponential.
 *
 * It also writes the same grid as Taylor rows per order M = 0..BOYS_TAYLOR_MMAX
 * (GS_BOYS_TAYLOR_<M>: row k = F_{M+j}(T_k) / j!, j = 0..6, and a zero) and the
 * exponential's rows (GS_BOYS_EXPT: row k = exp(-T_k) / j!, j = 0..6, and a zero): with
 * the factorials folded in, an expansion about T_k is a Horner chain of FMAs in T_k - T.
 *
 * usage: boys_table_gen OUT.h
 */
#include <math.h>
#include <stdio.h>

#define BOYS_INV_H 16
#define BOYS_TMAX 80
#define BOYS_ROWS (BOYS_TMAX * BOYS_INV_H + 1)
#define BOYS_NCOL 18 /* F_0..F_16 and exp(-T) */
#define BOYS_TAYLOR_MMAX 10 /* F_{M+6} is the highest order tabulated */

int main(int argc, char **argv)
{
    if (argc != 2) return 2;
    FILE *f = fopen(argv[1], "w");
    if (!f) return 1;
    fprintf(f, "// generated by boys_table_gen.c -- Boys function grid\n#pragma once\n");
    fprintf(f, "#define BOYS_INV_H %d\n#define BOYS_TMAX %d\n#define BOYS_ROWS %d\n#define BOYS_NCOL %d\n",
            BOYS_INV_H, BOYS_TMAX, BOYS_ROWS, BOYS_NCOL);
    const int top = BOYS_NCOL - 2;
    static long double F[BOYS_ROWS][BOYS_NCOL];
    for (int k = 0; k < BOYS_ROWS; ++k) {
        long double T = (long double)k / BOYS_INV_H;
        long double e = expl(-T);
        long double term = 1.0L / (2 * top + 1), sum = term;
        for (int i = 1; i < 100000; ++i) {
            term *= 2.0L * T / (2 * top + 2 * i + 1);
            sum += term;
            if (term < sum * 1e-24L) break;
        }
        F[k][top] = e * sum;
        for (int m = top; m >= 1; --m) F[k][m - 1] = (2.0L * T * F[k][m] + e) / (2 * m - 1);
        F[k][BOYS_NCOL - 1] = e;
    }
    fprintf(f, "#define BOYS_TAYLOR_MMAX %d\n", BOYS_TAYLOR_MMAX);
    fprintf(f, "#define GS_BOYS_TABLE_VALUES \\\n");
    for (int k = 0; k < BOYS_ROWS; ++k) {
        for (int m = 0; m < BOYS_NCOL; ++m) fprintf(f, "%a,", (double)F[k][m]);
        fprintf(f, " \\\n");
    }
    fprintf(f, "\n");
    long double fact[7] = {1, 1, 2, 6, 24, 120, 720};
    for (int M = 0; M <= BOYS_TAYLOR_MMAX; ++M) {
        fprintf(f, "#define GS_BOYS_TAYLOR_%d \\\n", M);
        for (int k = 0; k < BOYS_ROWS; ++k) {
            for (int j = 0; j <= 6; ++j) fprintf(f, "%a,", (double)(F[k][M + j] / fact[j]));
            fprintf(f, "0x0p+0, \\\n");
        }
        fprintf(f, "\n");
    }
    fprintf(f, "#define GS_BOYS_EXPT \\\n");
    for (int k = 0; k < BOYS_ROWS; ++k) {
        for (int j = 0; j <= 6; ++j) fprintf(f, "%a,", (double)(F[k][BOYS_NCOL - 1] / fact[j]));
        fprintf(f, "0x0p+0, \\\n");
    }
    fprintf(f, "\n");
    fclose(f);
    return 0;
}
