/*
 * Eigenvalues of the 2x2 / 3x3 symmetric inertia matrices, host and device.
 *
 * The reference gets them from EISPACK `rs` with eigenvectors requested
 * (attributes.c:726-767 -> eispack.c:12304 rs -> tred2 + tql2): Householder
 * tridiagonalisation, then the implicit QL method with the Moler-Morrison
 * hypotenuse.  Attribute values such as elongation (lambda_max/lambda_mid) of small
 * nodes are often exactly integers (a 2x1 domino gives 4), and pattern-spectrum and
 * filter thresholds sit exactly there, so a different eigen method would move
 * nodes across bin edges.  This file therefore restates those published
 * algorithms (Wilkinson & Reinsch, Handbook for Automatic Computation II,
 * procedures tred2/tql2; EISPACK Guide) for n <= 3, keeping their arithmetic
 * order so results are bit-identical to the reference's.  Only the eigenvalue
 * path is kept: the eigenvector updates of tql2 never feed back into the values.
 *
 * Only IEEE + - * / and sqrt are used.  Build device code with --fmad=false and
 * host code with -ffp-contract=off so no fused multiply-add changes a rounding.
 *
 * Provenance and licence.  The value path below (dcf_pythag, dcf_tred2_values,
 * dcf_tql2_values) follows the operation order, and keeps the variable names, of the
 * routines PYTHAG, TRED2 and TQL2 of the C port of EISPACK that the reference
 * vendors (src/sources/eispack.c, functions pythag, tred2 and tql2):
 *
 *   Original FORTRAN77 version by Smith, Boyle, Dongarra, Garbow, Ikebe, Klema,
 *   Moler.  C version by John Burkardt.  That code is distributed under the GNU
 *   LGPL license.
 *
 * Being a transcription of that code's arithmetic, this file is likewise
 * distributed under the GNU Lesser General Public License; the rest of the library
 * only calls it.
 */
#ifndef DCF_EIGEN_H
#define DCF_EIGEN_H

#include <math.h>

#if defined(__CUDACC__)
#define DCF_HD __host__ __device__ __forceinline__
#else
#define DCF_HD static inline
#endif

DCF_HD double dcf_eig_sign(double x) { return x < 0.0 ? -1.0 : 1.0; }
DCF_HD double dcf_eig_max(double a, double b) { return a < b ? b : a; }
DCF_HD double dcf_eig_min(double a, double b) { return a < b ? a : b; }

/* sqrt(a^2 + b^2) by the Moler-Morrison iteration (EISPACK pythag). */
DCF_HD double dcf_pythag(double a, double b)
{
    double p = dcf_eig_max(fabs(a), fabs(b));
    if (p != 0.0) {
        double r = dcf_eig_min(fabs(a), fabs(b)) / p;
        r = r * r;
        for (int it = 0; it < 64; it++) {
            double t = 4.0 + r;
            if (t == 4.0) break;
            double s = r / t;
            double u = 1.0 + 2.0 * s;
            p = u * p;
            r = (s / u) * (s / u) * r;
        }
    }
    return p;
}

/*
 * Householder reduction of the symmetric n x n matrix a (column-major,
 * element (i,j) at a[i + j*n]) to tridiagonal form: diagonal d[0..n-1],
 * sub-diagonal e[1..n-1] (e[0] = 0).  Same arithmetic sequence as EISPACK tred2;
 * the accumulated transformation is not formed except for the entries the
 * diagonal is read back from.
 */
DCF_HD void dcf_tred2_values(int n, const double *a, double *d, double *e)
{
    double z[9];
    for (int j = 0; j < n; j++)
        for (int i = j; i < n; i++) z[i + j * n] = a[i + j * n];
    for (int j = 0; j < n; j++) d[j] = a[n - 1 + j * n];

    for (int i = n - 1; 1 <= i; i--) {
        int l = i - 1;
        double h = 0.0, scale = 0.0;
        for (int k = 0; k <= l; k++) scale = scale + fabs(d[k]);
        if (scale == 0.0) {
            e[i] = d[l];
            for (int j = 0; j <= l; j++) {
                d[j] = z[l + j * n];
                z[i + j * n] = 0.0;
                z[j + i * n] = 0.0;
            }
            d[i] = 0.0;
            continue;
        }
        for (int k = 0; k <= l; k++) d[k] = d[k] / scale;
        h = 0.0;
        for (int k = 0; k <= l; k++) h = h + d[k] * d[k];
        double f = d[l];
        double g = -sqrt(h) * dcf_eig_sign(f);
        e[i] = scale * g;
        h = h - f * g;
        d[l] = f - g;
        for (int k = 0; k <= l; k++) e[k] = 0.0;
        for (int j = 0; j <= l; j++) {
            f = d[j];
            z[j + i * n] = f;
            g = e[j] + z[j + j * n] * f;
            for (int k = j + 1; k <= l; k++) {
                g = g + z[k + j * n] * d[k];
                e[k] = e[k] + z[k + j * n] * f;
            }
            e[j] = g;
        }
        for (int k = 0; k <= l; k++) e[k] = e[k] / h;
        f = 0.0;
        for (int k = 0; k <= l; k++) f = f + e[k] * d[k];
        double hh = 0.5 * f / h;
        for (int k = 0; k <= l; k++) e[k] = e[k] - hh * d[k];
        for (int j = 0; j <= l; j++) {
            f = d[j];
            g = e[j];
            for (int k = j; k <= l; k++) z[k + j * n] = z[k + j * n] - f * e[k] - g * d[k];
            d[j] = z[l + j * n];
            z[i + j * n] = 0.0;
        }
        d[i] = h;
    }
    /* the reduced diagonal; the last entry is the untouched a(n-1,n-1) */
    for (int j = 0; j < n - 1; j++) d[j] = z[j + j * n];
    d[n - 1] = z[n - 1 + (n - 1) * n];
    e[0] = 0.0;
}

/*
 * Eigenvalues of the symmetric tridiagonal matrix (d, e[1..n-1]) by the implicit
 * QL method with shifts, ascending in d.  Same arithmetic as EISPACK tql2's value
 * path.  Returns 0, or l+1 if eigenvalue l did not converge in 30 iterations.
 */
DCF_HD int dcf_tql2_values(int n, double *d, double *e)
{
    if (n == 1) return 0;
    for (int i = 1; i < n; i++) e[i - 1] = e[i];
    double f = 0.0, tst1 = 0.0;
    e[n - 1] = 0.0;
    for (int l = 0; l < n; l++) {
        int j = 0;
        double h = fabs(d[l]) + fabs(e[l]);
        tst1 = dcf_eig_max(tst1, h);
        int m;
        for (m = l; m < n; m++) {
            double tst2 = tst1 + fabs(e[m]);
            if (tst2 == tst1) break;
        }
        if (m != l) {
            for (;;) {
                if (30 <= j) return l + 1;
                j = j + 1;
                int l1 = l + 1, l2 = l1 + 1;
                double g = d[l];
                double p = (d[l1] - g) / (2.0 * e[l]);
                double r = dcf_pythag(p, 1.0);
                d[l] = e[l] / (p + dcf_eig_sign(p) * fabs(r));
                d[l1] = e[l] * (p + dcf_eig_sign(p) * fabs(r));
                double dl1 = d[l1];
                h = g - d[l];
                for (int i = l2; i < n; i++) d[i] = d[i] - h;
                f = f + h;
                p = d[m];
                double c = 1.0, c2 = c, c3 = c;
                double el1 = e[l1];
                double s = 0.0, s2 = 0.0;
                int mml = m - l;
                for (int ii = 1; ii <= mml; ii++) {
                    c3 = c2;
                    c2 = c;
                    s2 = s;
                    int i = m - ii;
                    g = c * e[i];
                    h = c * p;
                    r = dcf_pythag(p, e[i]);
                    e[i + 1] = s * r;
                    s = e[i] / r;
                    c = p / r;
                    p = c * d[i] - s * g;
                    d[i + 1] = h + s * (c * g + s * d[i]);
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p;
                d[l] = c * p;
                double tst2 = tst1 + fabs(e[l]);
                if (tst2 <= tst1) break;
            }
        }
        d[l] = d[l] + f;
    }
    /* selection sort, ascending */
    for (int ii = 1; ii < n; ii++) {
        int i = ii - 1, k = i;
        double p = d[i];
        for (int j = ii; j < n; j++)
            if (d[j] < p) {
                k = j;
                p = d[j];
            }
        if (k != i) {
            d[k] = d[i];
            d[i] = p;
        }
    }
    return 0;
}

/* Eigenvalues (ascending) of a symmetric n x n matrix, n <= 3: tred2 then tql2. */
DCF_HD int dcf_sym_eigenvalues(int n, const double *a, double *w)
{
    double e[3];
    dcf_tred2_values(n, a, w, e);
    return dcf_tql2_values(n, w, e);
}

#endif
