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
// The real variant with panels of OZAKI_NB whose panel solve (L21 = A21 L11^-T) and trailing
// update (A22 -= L21 L21^T) run on the tensor cores: each row is cut into OZAKI_SLICES 7-bit
// integer slices under a power-of-two row scale, the slice products accumulate exactly in FP32
// and are recombined by integer operations (k_chol_ozaki.cu).  w holds the slices of one panel
// and the inverse of its diagonal block; err gets tensor-core wait timeouts.
constexpr int OZAKI_NB = 64;
constexpr int OZAKI_SLICES = 8;
struct OzakiWork
{
    int N = 0, batch = 0;
    void *slices = nullptr;    // [batch][slice][N][OZAKI_NB] bf16: panel rows
    int *expo = nullptr;       // [batch][N]
    double *winv = nullptr;    // [batch][OZAKI_NB][OZAKI_NB]: inverse of the diagonal block
    void *wslices = nullptr;   // [batch][slice][2 OZAKI_NB][OZAKI_NB] bf16: its rows (upper half zero)
    int *wexpo = nullptr;      // [batch][2 OZAKI_NB]
    int *err = nullptr;
};
void ozaki_alloc(OzakiWork &w, int N, int batch);
void ozaki_free(OzakiWork &w);
int chol_batched_r_ozaki(double *A, int N, int batch, double *diag, int *bad, OzakiWork &w, cudaStream_t st);
// A[s0:, s0:] (lower) -= L21 L21^T with L21 = A[s0:, k0:k0+nb]; returns launches
int ozaki_trailing_update(double *A, int N, int batch, int s0, int k0, int nb, OzakiWork &w, cudaStream_t st);
// Panel L21 = A21 W^T for the full panel at k0 (rows k0 + OZAKI_NB .. N), W = L11^-1 in w.winv,
// by the same exact slice products; returns launches
int ozaki_panel_solve(double *A, int N, int batch, int k0, OzakiWork &w, cudaStream_t st);
// Random SPD matrices (X X^T / N + shift I, diagonal scale spread) through chol_batched_r and
// chol_batched_r_ozaki; returns the largest
// log-det difference, *max_rel_l the largest |L difference| / max |L|.
double chol_ozaki_selftest(int N, int batch, int seed, int spread_decades, double shift, double *max_rel_l);
// logdet[b] = 2 sum_i log diag[b][i]
void chol_logdet(const double *diag, int N, int batch, double *logdet, cudaStream_t st);
// zero the strict upper triangle (turn the factored matrix into L)
void zero_upper_c(cuDoubleComplex *A, int N, int batch, cudaStream_t st);
void zero_upper_r(double *A, int N, int batch, cudaStream_t st);

} // namespace gb
