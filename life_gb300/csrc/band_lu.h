// Dense LU with partial pivoting restricted to the band of the matrix.
//
// Utils::solveLAPACK (reference src/Utils.cpp:288-311) hands a row-major
// matrix A to column-major LAPACK, i.e. it factors M = A_sub^T (A_sub = the
// block of A without its first `bc` rows and columns) with dgetrf and solves
// with dgetrs('T'), which is A_sub x = b. This routine performs the textbook
// unblocked form of those two calls (first maximal pivot, column scaled by the
// reciprocal pivot, rank-1 trailing update, transposed triangular solves, then
// the row interchanges in reverse), in place on A's storage, but only visits
// entries inside M's band (kl below, ku above the diagonal, plus the fill-in
// pivoting creates). Entries outside the band are zero and would only add
// signed zeros, so the result is bit-identical to the dense loops while costing
// O(n*kl*(kl+ku)) instead of O(n^3). Whole rows are swapped, as LAPACK does,
// so the multipliers sit where the dense transposed solve expects them.
#pragma once

#ifndef __CUDACC__
#define LIFE_HD
#else
#define LIFE_HD __host__ __device__
#endif

namespace life {

// M(i,j) of the column-major view used by the reference's LAPACK call.
LIFE_HD inline double& lu_m(double* A, int dim, int bc, int i, int j) {
    return A[(long long)(bc + j) * dim + (bc + i)];
}

// Bandwidths of M = A_sub^T from the nonzero pattern (kl: below, ku: above).
LIFE_HD inline void lu_bandwidth(const double* A, int dim, int bc, int* kl, int* ku) {
    int lo = 0, hi = 0;
    const int n = dim - bc;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
            if (A[(long long)(bc + j) * dim + (bc + i)] != 0.0) {
                if (i - j > lo) lo = i - j;
                if (j - i > hi) hi = j - i;
            }
    *kl = lo;
    *ku = hi;
}

LIFE_HD inline void lu_band_factor(double* A, int dim, int bc, int kl, int ku, int* piv) {
    const int n = dim - bc;
    for (int j = 0; j < n; j++) {
        const int imax = j + kl < n - 1 ? j + kl : n - 1;
        int jp = j;
        double amax = lu_m(A, dim, bc, j, j);
        amax = amax < 0 ? -amax : amax;
        for (int i = j + 1; i <= imax; i++) {
            double a = lu_m(A, dim, bc, i, j);
            a = a < 0 ? -a : a;
            if (a > amax) { amax = a; jp = i; }
        }
        piv[j] = jp;
        if (lu_m(A, dim, bc, jp, j) != 0.0) {
            if (jp != j)
                for (int k = 0; k < n; k++) {
                    double t = lu_m(A, dim, bc, j, k);
                    lu_m(A, dim, bc, j, k) = lu_m(A, dim, bc, jp, k);
                    lu_m(A, dim, bc, jp, k) = t;
                }
            const double r = 1.0 / lu_m(A, dim, bc, j, j);
            for (int i = j + 1; i <= imax; i++) lu_m(A, dim, bc, i, j) *= r;
        }
        const int kmax = j + kl + ku < n - 1 ? j + kl + ku : n - 1;
        for (int k = j + 1; k <= kmax; k++) {
            const double t = -lu_m(A, dim, bc, j, k);
            for (int i = j + 1; i <= imax; i++) lu_m(A, dim, bc, i, k) += lu_m(A, dim, bc, i, j) * t;
        }
    }
}

// Transposed solve on the factors; x has dim entries, the first bc are zeroed
// (the reference zeroes the constrained DOFs, src/Utils.cpp:307).
LIFE_HD inline void lu_band_solve(const double* A, int dim, int bc, int kl, int ku, const int* piv,
                                  const double* b, double* x) {
    const int n = dim - bc;
    double* A_ = const_cast<double*>(A);
    for (int i = 0; i < bc; i++) x[i] = 0.0;
    double* y = x + bc;
    for (int i = 0; i < n; i++) y[i] = b[bc + i];
    const int w = kl + ku;
    for (int i = 0; i < n; i++) {
        double t = y[i];
        for (int k = (i - w > 0 ? i - w : 0); k < i; k++) t -= lu_m(A_, dim, bc, k, i) * y[k];
        y[i] = t / lu_m(A_, dim, bc, i, i);
    }
    for (int i = n - 1; i >= 0; i--) {
        double t = y[i];
        for (int k = i + 1; k < n; k++) t -= lu_m(A_, dim, bc, k, i) * y[k];
        y[i] = t;
    }
    for (int i = n - 1; i >= 0; i--)
        if (piv[i] != i) {
            double t = y[i];
            y[i] = y[piv[i]];
            y[piv[i]] = t;
        }
}

}  // namespace life
