// Batched FP64 Cholesky (k_chol.cu) and its log-determinant.
#pragma once

#include <cuComplex.h>
#include <cuda_runtime.h>

namespace gb {

// In-place lower Cholesky of batch row-major N x N matrices (Hermitian / symmetric, lower
// triangle read).  diag[b][i] = L_ii; bad[b] set to 1 if a pivot was not positive.
// Returns the number of kernel launches.
int chol_batched_c(cuDoubleComplex *A, int N, int batch, double *diag, int *bad, cudaStream_t st);
int chol_batched_r(double *A, int N, int batch, double *diag, int *bad, cudaStream_t st);
// logdet[b] = 2 sum_i log diag[b][i]
void chol_logdet(const double *diag, int N, int batch, double *logdet, cudaStream_t st);
// zero the strict upper triangle (turn the factored matrix into L)
void zero_upper_c(cuDoubleComplex *A, int N, int batch, cudaStream_t st);
void zero_upper_r(double *A, int N, int batch, cudaStream_t st);

} // namespace gb
