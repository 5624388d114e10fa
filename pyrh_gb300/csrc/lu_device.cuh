// lu_device.cuh -- SolveLinearEq of the reference (rh/ludcmp.c:36-177) for
// one small system per thread: Crout LU with implicit partial pivoting
// (TINY 1e-20 on a zero pivot), forward and back substitution, and one
// improvement step with the residual of the original system.  A is n x n
// row-major and is overwritten by its factors; b becomes the solution.
// NMAX bounds n (the local arrays).
#pragma once

namespace pyrh {

template <int NMAX>
__device__ void lu_solve(int n, double* A, double* bvec) {
  double Ac[NMAX * NMAX], bc[NMAX];
  double vv[NMAX], res[NMAX];
  int index[NMAX];
  for (int i = 0; i < n * n; ++i) Ac[i] = A[i];
  for (int i = 0; i < n; ++i) bc[i] = bvec[i];
  for (int i = 0; i < n; ++i) {
    double big = 0.0;
    for (int j = 0; j < n; ++j) big = fmax(big, fabs(A[i * n + j]));
    vv[i] = (big == 0.0) ? 0.0 : 1.0 / big;
  }
  for (int j = 0; j < n; ++j) {
    int imax = 0;
    for (int i = 0; i < j; ++i) {
      double sum = A[i * n + j];
      for (int k = 0; k < i; ++k) sum -= A[i * n + k] * A[k * n + j];
      A[i * n + j] = sum;
    }
    double big = 0.0;
    for (int i = j; i < n; ++i) {
      double sum = A[i * n + j];
      for (int k = 0; k < j; ++k) sum -= A[i * n + k] * A[k * n + j];
      A[i * n + j] = sum;
      const double dum = vv[i] * fabs(sum);
      if (dum >= big) { big = dum; imax = i; }
    }
    if (j != imax) {
      for (int k = 0; k < n; ++k) {
        const double t = A[imax * n + k];
        A[imax * n + k] = A[j * n + k];
        A[j * n + k] = t;
      }
      vv[imax] = vv[j];
    }
    index[j] = imax;
    if (A[j * n + j] == 0.0) A[j * n + j] = 1.0e-20;
    const double dum = 1.0 / A[j * n + j];
    for (int i = j + 1; i < n; ++i) A[i * n + j] *= dum;
  }
  for (int pass = 0; pass < 2; ++pass) {
    double* x = pass ? res : bvec;
    if (pass)
      for (int i = 0; i < n; ++i) {
        res[i] = bc[i];
        for (int j = 0; j < n; ++j) res[i] -= Ac[i * n + j] * bvec[j];
      }
    int ii = -1;
    for (int i = 0; i < n; ++i) {
      const int ip = index[i];
      double sum = x[ip];
      x[ip] = x[i];
      if (ii >= 0) for (int j = ii; j < i; ++j) sum -= A[i * n + j] * x[j];
      else if (sum != 0.0) ii = i;
      x[i] = sum;
    }
    for (int i = n - 1; i >= 0; --i) {
      double sum = x[i];
      for (int j = i + 1; j < n; ++j) sum -= A[i * n + j] * x[j];
      x[i] = sum / A[i * n + i];
    }
  }
  for (int i = 0; i < n; ++i) bvec[i] += res[i];
}

}  // namespace pyrh
