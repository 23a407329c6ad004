// Launch wrappers of the device kernels (each .cu file implements a group).
// All matrices are row-major; "n_sup" is the supercell orbital count
// n_cells * n_ao, with supercell index (cell, unit-cell orbital).
#pragma once

#include <cuComplex.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace gb {

// Small index tables describing atoms and BvK cells (device pointers).
struct Geom
{
    int n_at = 0;      // atoms
    int n_c = 0;       // BvK cells (= number of k points)
    int n_ao = 0;      // NAOs in the unit cell
    int n_sup = 0;     // n_c * n_ao
    int max_nao = 0, max_nabf = 0;
    long long rows_c = 0;          // sum_I nabf_I * nao_I  (rows of the C matrix)
    const int *ao_off = nullptr;   // [n_at] first NAO of atom I in the unit cell
    const int *nao = nullptr;      // [n_at]
    const int *nabf = nullptr;     // [n_at]
    const long long *rowc_off = nullptr;  // [n_at] first row (I, mu=0, i=0) of the C matrix
    const int *cdiff = nullptr;    // [n_c*n_c] cdiff[a*n_c+b] = cell index of (R_a - R_b) mod period
    const int *cneg = nullptr;     // [n_c] cell index of -R mod period
};

// Upper atom pairs (I <= J) and their block offsets.
struct Pairs
{
    int n_pairs = 0;
    const int *I = nullptr, *J = nullptr;
    const long long *r_off = nullptr;  // [n_pairs] offset of chi0(R) blocks: pair p, cell c at r_off[p] + c*nI*nJ
    const long long *e_off = nullptr;  // [n_pairs] offset inside one (omega,q) slab of chi0(q,omega)
    long long e_total = 0;             // sum over pairs of nabf_I * nabf_J
};

// ---------------------------------------------------------------- k_mf.cu
// s[sign][k][n] = exp(min(0, -tau (e - ef))) * w_sign, with w+ = max(0, 1/nk - f ns/2)
// and w- = f ns / 2; bands >= nbands_g zeroed when nbands_g >= 0 (chi0.cpp:348-391).
void launch_tau_scale(const double *ekb, const double *wg, int nk, int nb, double ef, double tau,
                      int n_spins, int nbands_g, double *s_out, cudaStream_t st);
// A[sign][k] = Psi_k^T diag(s[sign][k]) conj(Psi_k), complex n_ao x n_ao per (sign, k).
void launch_gk_build(const cuDoubleComplex *psi, const double *s, int nk, int nb, int nao,
                     cuDoubleComplex *A, cudaStream_t st);
// G[sign][c][i][j] = sgn * sum_k Re(exp(-i 2pi kfrac_k.R_c) A[sign][k][i][j]); sgn = +1 (tau>0), -1 (tau<0).
void launch_phase_sum(const cuDoubleComplex *A, const double *cosph, const double *sinph, int nk,
                      int nc, int nao, double *G, cudaStream_t st);
// Gs[sign][(cK,a)][(cL,b)] = G[sign][cdiff(cL,cK)][a][b]
void launch_gsuper(const double *G, const Geom &g, double *Gs, cudaStream_t st);
// Scatter the RI blocks into C[(I,mu,i)][(c,K,k)] (zeros elsewhere must be set beforehand).
void launch_cs_scatter(const double *blob, const long long *blk_off, const int *blk_meta, int n_blocks,
                       const Geom &g, double *C, cudaStream_t st);

// ---------------------------------------------------------------- k_gemm.cu
// C = A * B (row-major, FP64), batched with strides.
void launch_dgemm(int M, int N, int K, const double *A, long long lda, long long sA, const double *B,
                  long long ldb, long long sB, double *C, long long ldc, long long sC, int batch,
                  double alpha, double beta, cudaStream_t st);
// FP32 variant (alpha = 1, beta = 0).
void launch_sgemm(int M, int N, int K, const float *A, long long lda, long long sA, const float *B,
                  long long ldb, long long sB, float *C, long long ldc, long long sC, int batch,
                  cudaStream_t st);
// out[i] = (float) in[i]
void launch_d2f(const double *in, float *out, long long n, cudaStream_t st);
// C = A * B complex (row-major), batched.
void launch_zgemm(int M, int N, int K, const cuDoubleComplex *A, long long lda, long long sA,
                  const cuDoubleComplex *B, long long ldb, long long sB, cuDoubleComplex *C, long long ldc,
                  long long sC, int batch, cudaStream_t st);

// ---------------------------------------------------------------- k_chi0_fp64.cu
// chi0(R_cJ)[I<=J] = sum over the two G+/G- passes of T1 + T2 (see engine.cu for the algebra),
// written to out at pairs.r_off[p] + cJ*nI*nJ.  Xp/Xm = C * Gs(+/-), Cm = C matrix.
void launch_chi0_fp64(const double *Xp, const double *Xm, const double *Cm, const double *Gp,
                      const double *Gm, const Geom &g, const Pairs &pr, double *out, cudaStream_t st);
// Same algebra with FP32 operands and accumulators (output still FP64).
void launch_chi0_fp32(const float *Xp, const float *Xm, const float *Cm, const float *Gp,
                      const float *Gm, const Geom &g, const Pairs &pr, double *out, cudaStream_t st);

// ---------------------------------------------------------------- k_ftct.cu
// chi0q[w][q][e] += fac * gamma[w] * sum_c exp(+i 2pi q.R_c) chi0R[p][c][e]
void launch_ftct(const double *chi0R, const Geom &g, const Pairs &pr, const double *qcos,
                 const double *qsin, int nq, const double *gamma_w, int nw, double fac,
                 cuDoubleComplex *chi0q, cudaStream_t st);
// The same transform over nslot stored chi0(R) slots (slot s at slots + s * slot_stride, each laid
// out like chi0R): chi0q += sum_s gamma[w][s] FT(chi0_s), gamma including 2/n_s.  FP64 sum over
// the slots, FP32 phase sum over R; qphase[q][c] = (cos, sin) of 2 pi q.R_c.
void launch_ftct_slots(const double *slots, long long slot_stride, int nslot, const Geom &g, const Pairs &pr,
                       const float2 *qphase, int nq, const double *gamma, int nw, cuDoubleComplex *chi0q,
                       cudaStream_t st);
// Shared memory the batched transform needs (it runs when this is at most 227 KB).
size_t ftct_slots_smem(int nc, int nq, int nw);

// ---------------------------------------------------------------- k_ec.cu
// Full N x N Hermitian (complex) or symmetric (real part) matrices from upper atom blocks.
// atom_of[N]: atom of each ABF row; pair_of[n_at*n_at]: upper pair index for I<=J.
void launch_assemble_chi0(const cuDoubleComplex *src, long long slab_stride, int n_slabs, int N,
                          const int *atom_of, const int *abf_off, const int *nabf, const int *pair_of,
                          int n_at, const long long *e_off, bool real_only, cuDoubleComplex *outc,
                          double *outr, long long out_stride, cudaStream_t st);
// Dense n_slabs x (N x N) matrices -> their upper atom-pair blocks (the inverse of assemble_chi0).
void launch_scatter_pairs(const cuDoubleComplex *dense, long long dense_stride, int n_slabs, int N, const int *pI,
                          const int *pJ, int n_pairs, const int *abf_off, const int *nabf, const long long *e_off,
                          cuDoubleComplex *out, long long slab_stride, cudaStream_t st);
void launch_assemble_v(const cuDoubleComplex *blob, const long long *blk_off, const int *blk_IJ,
                       int n_blocks, const int *abf_off, const int *nabf, int N, bool real_only,
                       cuDoubleComplex *outc, double *outr, cudaStream_t st);
// tr(P) for each batch matrix, then P <- I - P.
void launch_trace_and_negate_c(cuDoubleComplex *P, int N, int batch, cuDoubleComplex *trace, cudaStream_t st);
void launch_trace_and_negate_r(double *P, int N, int batch, double *trace, cudaStream_t st);
// In-place LU with partial pivoting (one CTA per matrix); logdet = sum log(+-u_ii).
void launch_lu_logdet_c(cuDoubleComplex *M, int N, int batch, cuDoubleComplex *logdet, cudaStream_t st);
void launch_lu_logdet_r(double *M, int N, int batch, double *logdet, cudaStream_t st);

} // namespace gb
