/* Build shim: the LIFE reference calls LAPACK dgetrf_/dgetrs_
 * (reference inc/Utils.h:501-502, src/Utils.cpp:303-304). No system LAPACK is
 * installed here, so these forward to the OpenBLAS copy that scipy bundles,
 * which exports the same routines with a "scipy_" prefix. */
extern void scipy_dgetrf_(int*, int*, double*, int*, int*, int*);
extern void scipy_dgetrs_(char*, int*, int*, double*, int*, int*, double*, int*, int*, long);
void dgetrf_(int* m, int* n, double* a, int* lda, int* ipiv, int* info) {
    scipy_dgetrf_(m, n, a, lda, ipiv, info);
}
void dgetrs_(char* trans, int* n, int* nrhs, double* a, int* lda, int* ipiv,
             double* b, int* ldb, int* info) {
    scipy_dgetrs_(trans, n, nrhs, a, lda, ipiv, b, ldb, info, 1);
}
