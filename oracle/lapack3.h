/* Oracle (test infrastructure only): 3x3 LU factorisation and inverse.
 *
 * The reference inverts each 3x3 diagonal block of the elasticity preconditioner
 * with LAPACK DGETRF + DGETRI (src/Fortran/elasclpr.f:39,44), linked from Intel
 * MKL, which is closed and absent here, so its exact operation order cannot be
 * known ("parity unpinned" for that step).  This file restates the published
 * reference-LAPACK algorithms for n = 3, lda = 3, lwork = 3:
 *   - DGETRF2 (recursive LU with partial pivoting, LAPACK >= 3.6): column panel
 *     found by IDAMAX (first maximum of |x|), row swap, scaling of the column by
 *     the reciprocal of the pivot when |pivot| >= DLAMCH('S') (else by division),
 *     trailing update C := C + (-u) * l in the DGEMM loop order;
 *   - DGETRI unblocked branch (NB >= N): DTRTRI/DTRTI2 upper non-unit inverse of U
 *     (DTRMV with its x(j) != 0 test, then DSCAL by -inv(u_jj)), then
 *     inv(A) * L = inv(U) column by column with the DGEMV loop order, then the
 *     column interchanges from the last pivot down.
 * Matrices are column-major (a[r + 3*c]), exactly as the Fortran caller sees the
 * C block.  The product kernel carries its own, independent statement of the
 * same steps; this one is only the checker.  It is compared against
 * scipy.linalg.lapack.dgetrf/dgetri in the tests.
 *
 * Build with -ffp-contract=off: every product and sum below is a separately
 * rounded IEEE double operation.
 */
#ifndef ORACLE_LAPACK3_H
#define ORACLE_LAPACK3_H

#include <math.h>

/* DLAMCH('S') for IEEE double: the smallest normal number, 2^-1022. */
#define ORC_SFMIN 2.2250738585072014e-308

/* IDAMAX over n entries of column-major storage starting at a[off], stride 1.
 * Returns the 0-based offset of the first entry of largest magnitude. */
static inline int orc_idamax(int n, const double *x)
{
    int best = 0;
    double dmax = fabs(x[0]);
    for (int i = 1; i < n; i++) {
        if (fabs(x[i]) > dmax) {
            best = i;
            dmax = fabs(x[i]);
        }
    }
    return best;
}

/* One-column panel of DGETRF2 on rows [r0, 3) of column c.  Returns the pivot
 * row (global, 0-based) and sets *zero when the pivot is exactly zero. */
static inline int orc_panel(double *a, int r0, int c, int *zero)
{
    double *col = a + 3 * c;
    int p = r0 + orc_idamax(3 - r0, col + r0);
    *zero = 0;
    if (col[p] != 0.0) {
        if (p != r0) {
            double t = col[r0];
            col[r0] = col[p];
            col[p] = t;
        }
        if (fabs(col[r0]) >= ORC_SFMIN) {
            double r = 1.0 / col[r0];
            for (int i = r0 + 1; i < 3; i++) col[i] = r * col[i];
        } else {
            for (int i = r0 + 1; i < 3; i++) col[i] = col[i] / col[r0];
        }
    } else {
        *zero = 1;
    }
    return p;
}

static inline void orc_swap_rows(double *a, int r1, int r2, int c0, int c1)
{
    if (r1 == r2) return;
    for (int c = c0; c < c1; c++) {
        double t = a[r1 + 3 * c];
        a[r1 + 3 * c] = a[r2 + 3 * c];
        a[r2 + 3 * c] = t;
    }
}

/* DGETRF for a 3x3 column-major matrix.  ipiv is 0-based.  Returns INFO. */
static inline int orc_dgetrf3(double a[9], int ipiv[3])
{
    int info = 0, zero;
    /* top level: N1 = 1, N2 = 2 */
    int p0 = orc_panel(a, 0, 0, &zero);
    ipiv[0] = p0;
    if (zero && info == 0) info = 1;
    orc_swap_rows(a, 0, p0, 1, 3);                 /* DLASWP on A12/A22 */
    /* DTRSM with a 1x1 unit lower triangle: no operation */
    for (int j = 1; j < 3; j++) {                  /* DGEMM: A22 -= A21 * A12 */
        double temp = -a[0 + 3 * j];
        for (int i = 1; i < 3; i++) a[i + 3 * j] = a[i + 3 * j] + temp * a[i];
    }
    /* recursion on the 2x2 trailing block: N1 = 1, N2 = 1 */
    int p1 = orc_panel(a, 1, 1, &zero);
    ipiv[1] = p1;
    if (zero && info == 0) info = 2;
    orc_swap_rows(a, 1, p1, 2, 3);
    {
        double temp = -a[1 + 3 * 2];
        a[2 + 3 * 2] = a[2 + 3 * 2] + temp * a[2 + 3 * 1];
    }
    /* 1x1 trailing block */
    ipiv[2] = 2;
    if (a[2 + 3 * 2] == 0.0 && info == 0) info = 3;
    /* interchanges of the 2x2 level applied to the left column */
    orc_swap_rows(a, 1, p1, 0, 1);
    return info;
}

/* DGETRI for a 3x3 column-major LU factorisation.  Returns INFO; when U has an
 * exact zero on its diagonal the matrix is left unchanged, as DTRTRI returns
 * before touching it. */
static inline int orc_dgetri3(double a[9], const int ipiv[3])
{
    for (int i = 0; i < 3; i++)
        if (a[i + 3 * i] == 0.0) return i + 1;
    /* DTRTI2, upper, non-unit */
    for (int j = 0; j < 3; j++) {
        a[j + 3 * j] = 1.0 / a[j + 3 * j];
        double ajj = -a[j + 3 * j];
        /* DTRMV: x := T * x, T = leading j x j block (already inverted) */
        double *x = a + 3 * j;
        for (int jj = 0; jj < j; jj++) {
            if (x[jj] != 0.0) {
                double temp = x[jj];
                for (int i = 0; i < jj; i++) x[i] = x[i] + temp * a[i + 3 * jj];
                x[jj] = x[jj] * a[jj + 3 * jj];
            }
        }
        for (int i = 0; i < j; i++) x[i] = ajj * x[i];   /* DSCAL */
    }
    /* unblocked solve of inv(A) * L = inv(U) */
    double work[3];
    for (int j = 2; j >= 0; j--) {
        for (int i = j + 1; i < 3; i++) {
            work[i] = a[i + 3 * j];
            a[i + 3 * j] = 0.0;
        }
        if (j < 2) {
            /* DGEMV: a(:,j) += -1 * A(:, j+1:3) * work(j+1:3) */
            for (int jj = j + 1; jj < 3; jj++) {
                double temp = -work[jj];
                for (int i = 0; i < 3; i++) a[i + 3 * j] = a[i + 3 * j] + temp * a[i + 3 * jj];
            }
        }
    }
    /* column interchanges */
    for (int j = 1; j >= 0; j--) {
        int jp = ipiv[j];
        if (jp != j) {
            for (int i = 0; i < 3; i++) {
                double t = a[i + 3 * j];
                a[i + 3 * j] = a[i + 3 * jp];
                a[i + 3 * jp] = t;
            }
        }
    }
    return 0;
}

#endif
