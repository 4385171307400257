/* Build shim (oracle pinning only): dgetrf_/dgetrs_ as the textbook unblocked
 * LU with partial pivoting (LAPACK dgetf2 semantics: first maximal pivot,
 * column scaled by the reciprocal pivot, rank-1 trailing update) and the
 * matching triangular solves. Linking the reference against this instead of
 * OpenBLAS makes its dense solves follow the same operation order as the
 * oracle's, so the oracle's IBM/FEM restatement can be checked bit for bit.
 * Column-major, one right-hand side, as the reference calls them
 * (reference src/Utils.cpp:303-304). */
#include <math.h>

void dgetrf_(int* m, int* n, double* a, int* lda, int* ipiv, int* info) {
    int M = *m, N = *n, ld = *lda;
    *info = 0;
    int mn = M < N ? M : N;
    for (int j = 0; j < mn; j++) {
        int jp = j;
        double amax = fabs(a[j + j * ld]);
        for (int i = j + 1; i < M; i++) {
            double v = fabs(a[i + j * ld]);
            if (v > amax) { amax = v; jp = i; }
        }
        ipiv[j] = jp + 1;
        if (a[jp + j * ld] != 0.0) {
            if (jp != j)
                for (int k = 0; k < N; k++) {
                    double t = a[j + k * ld];
                    a[j + k * ld] = a[jp + k * ld];
                    a[jp + k * ld] = t;
                }
            double r = 1.0 / a[j + j * ld];
            for (int i = j + 1; i < M; i++) a[i + j * ld] *= r;
        } else if (*info == 0) {
            *info = j + 1;
        }
        for (int k = j + 1; k < N; k++) {
            double t = -a[j + k * ld];
            for (int i = j + 1; i < M; i++) a[i + k * ld] += a[i + j * ld] * t;
        }
    }
}

void dgetrs_(char* trans, int* n, int* nrhs, double* a, int* lda, int* ipiv, double* b,
             int* ldb, int* info) {
    int N = *n, ld = *lda;
    (void)ldb;
    (void)nrhs;
    *info = 0;
    if (*trans == 'T' || *trans == 't') {
        for (int i = 0; i < N; i++) {
            double t = b[i];
            for (int k = 0; k < i; k++) t -= a[k + i * ld] * b[k];
            b[i] = t / a[i + i * ld];
        }
        for (int i = N - 1; i >= 0; i--) {
            double t = b[i];
            for (int k = i + 1; k < N; k++) t -= a[k + i * ld] * b[k];
            b[i] = t;
        }
        for (int i = N - 1; i >= 0; i--) {
            int p = ipiv[i] - 1;
            if (p != i) { double t = b[i]; b[i] = b[p]; b[p] = t; }
        }
    } else {
        *info = -1; /* the reference only uses the transposed solve */
    }
}
