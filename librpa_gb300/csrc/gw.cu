// Exact exchange and the G0W0 correlation self-energy on the GPU, for k-grids and the Gamma point.
//
// The chain of LibRPA's task = g0w0 for Gamma-only inputs (molecules and Gamma-point cells); the
// k-grid chain (build_g0w0_kgrid, build_exx) runs the same steps on the Born-von Karman supercell:
//   chi0(omega)      the RPA path's chi0(q = 0, omega) (engine.cu, any chi0 precision)
//   W_c(omega)       S_c [(1 - S chi0 S)^-1 - 1] S_c with S = V^1/2, S_c = V_cut^1/2, the square
//                    roots by eigen-decomposition with eigenvalues below the threshold dropped
//                    (compute_Wc_freq_q_blacs, src/core/epsilon.cpp:1763-2322, default branch;
//                    power_hemat_blacs, src/math/utils_matrix_m_mpi.h:597-720)
//   W_c(tau)         sum_omega costrans_f2t(tau, omega) W_c(omega) (CT_FT_Wc_freq_q,
//                    epsilon.cpp:2490-2660; one k-point: no q sum)
//   Sigma(+-tau)     LibRI GW::cal_Sigmas (thirdparty/LibRI/include/RI/physics/GW.hpp:102-125)
//   Sigma(i omega)   sum_tau [cos_t2f (S+ + S-)/2 + i sin_t2f (S+ - S-)/2] (src/core/gw.cpp:627-700)
//   KS diagonal      <psi_n|Sigma(i omega)|psi_n> (gw.cpp:1100-1140)
// and the exchange of task = exx at Gamma: H_x by LibRI Exx::cal_Hs (Exx.hpp:242-283) with the
// density matrix D (MeanField::get_dmat_cplx_R, src/core/meanfield.cpp:201-244) and the truncated
// Coulomb V_cut, v_exx_n = -<psi_n|H_x|psi_n>.
//
// The four LibRI labels of cal_Hs / cal_Sigmas sum to one closed form,
//   H_pq = sum_{a,b,r,s} U[a,p,r] W[a,b] U[b,q,s] D[r,s],   U[a,p,r] = C_a[p,r] + C_a[r,p],
// which runs here as three FP64 GEMMs over dense operands: Y = U D ([(a,p), s]), Z = W U
// ([a, (q,s)]) and H = Y' Z' over (a, s).  The dense U holds N_abf n_ao^2 values, which bounds
// this formulation to cells of a few hundred orbitals; larger cells need the atom-pair-sparse
// form of the χ0 contraction.
#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <map>
#include <vector>

#include "common.h"
#include "cs_fold.h"
#include "dataset.h"
#include "dielec.h"
#include "gw.h"
#include "host_tables.h"
#include "kernels.h"
#include "minimax.h"
#include "tc_gemm.h"

namespace gb {

namespace {

// G[i][j] = sgn sum_n s_n Re(psi_ni conj(psi_nj)) (Gamma point: chi0.cpp:332-423 without the
// phase sum; with s_n the density-matrix weights it is D of meanfield.cpp:201-244)
__global__ void k_gamma_dm(const cuDoubleComplex *__restrict__ psi, const double *__restrict__ s, int nb, int nao,
                           double sgn, double *__restrict__ G)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nao * nao) return;
    const int i = t / nao, j = t % nao;
    double acc = 0.0;
    for (int n = 0; n < nb; ++n)
    {
        const cuDoubleComplex a = psi[static_cast<size_t>(n) * nao + i], b = psi[static_cast<size_t>(n) * nao + j];
        acc += s[n] * (a.x * b.x + a.y * b.y);
    }
    G[t] = sgn * acc;
}

// Yt[p][(a, s)] = Y[(a, p), s]
__global__ void k_perm_y(const double *__restrict__ Y, int N, int nao, double *__restrict__ Yt)
{
    const long long n = static_cast<long long>(N) * nao * nao;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long a = t / (static_cast<long long>(nao) * nao);
        const int p = static_cast<int>((t / nao) % nao), s = static_cast<int>(t % nao);
        Yt[(static_cast<long long>(p) * N + a) * nao + s] = Y[t];
    }
}

// Zt[(a, s)][q] = Z[a][(q, s)]
__global__ void k_perm_z(const double *__restrict__ Z, int N, int nao, double *__restrict__ Zt)
{
    const long long n = static_cast<long long>(N) * nao * nao;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long a = t / (static_cast<long long>(nao) * nao);
        const int q = static_cast<int>((t / nao) % nao), s = static_cast<int>(t % nao);
        Zt[(a * nao + s) * nao + q] = Z[t];
    }
}

// In place: A <- I - A (batch of N x N)
__global__ void k_one_minus(double *__restrict__ A, int N, int batch)
{
    const long long nn = static_cast<long long>(N) * N, n = nn * batch;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long e = t % nn;
        A[t] = ((e / N) == (e % N) ? 1.0 : 0.0) - A[t];
    }
}

// Solve A X = B in place (B <- X) by Gauss-Jordan elimination with partial pivoting, one CTA per
// batch entry: A N x N, B N x M, both row-major in global memory.  *bad is set when a pivot is 0.
__global__ void __launch_bounds__(256) k_gj_solve(double *__restrict__ Aall, double *__restrict__ Ball, int N, int M,
                                                  int *__restrict__ bad)
{
    double *A = Aall + static_cast<size_t>(blockIdx.x) * N * N;
    double *B = Ball + static_cast<size_t>(blockIdx.x) * N * M;
    extern __shared__ double col[];  // column k of A before the elimination step
    __shared__ double rv[256];
    __shared__ int ri[256];
    for (int k = 0; k < N; ++k)
    {
        // pivot: largest |A[i][k]|, i >= k
        double best = -1.0;
        int bi = k;
        for (int i = k + threadIdx.x; i < N; i += blockDim.x)
        {
            const double v = fabs(A[static_cast<size_t>(i) * N + k]);
            if (v > best)
            {
                best = v;
                bi = i;
            }
        }
        rv[threadIdx.x] = best;
        ri[threadIdx.x] = bi;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1)
        {
            if (threadIdx.x < s && (rv[threadIdx.x + s] > rv[threadIdx.x] ||
                                    (rv[threadIdx.x + s] == rv[threadIdx.x] && ri[threadIdx.x + s] < ri[threadIdx.x])))
            {
                rv[threadIdx.x] = rv[threadIdx.x + s];
                ri[threadIdx.x] = ri[threadIdx.x + s];
            }
            __syncthreads();
        }
        const int piv = ri[0];
        if (threadIdx.x == 0 && !(rv[0] > 0.0)) atomicExch(bad, 1);
        __syncthreads();
        if (piv != k)
        {
            for (int j = threadIdx.x; j < N; j += blockDim.x)
            {
                const double t = A[static_cast<size_t>(k) * N + j];
                A[static_cast<size_t>(k) * N + j] = A[static_cast<size_t>(piv) * N + j];
                A[static_cast<size_t>(piv) * N + j] = t;
            }
            for (int j = threadIdx.x; j < M; j += blockDim.x)
            {
                const double t = B[static_cast<size_t>(k) * M + j];
                B[static_cast<size_t>(k) * M + j] = B[static_cast<size_t>(piv) * M + j];
                B[static_cast<size_t>(piv) * M + j] = t;
            }
        }
        __syncthreads();
        const double pv = A[static_cast<size_t>(k) * N + k];
        const double inv = pv != 0.0 ? 1.0 / pv : 0.0;
        __syncthreads();
        for (int j = threadIdx.x; j < N; j += blockDim.x) A[static_cast<size_t>(k) * N + j] *= inv;
        for (int j = threadIdx.x; j < M; j += blockDim.x) B[static_cast<size_t>(k) * M + j] *= inv;
        for (int i = threadIdx.x; i < N; i += blockDim.x) col[i] = A[static_cast<size_t>(i) * N + k];
        __syncthreads();
        // eliminate column k from every other row
        for (long long t = threadIdx.x; t < static_cast<long long>(N) * (N + M); t += blockDim.x)
        {
            const int i = static_cast<int>(t / (N + M)), j = static_cast<int>(t % (N + M));
            if (i == k) continue;
            const double f = col[i];
            if (f == 0.0) continue;
            if (j < N)
                A[static_cast<size_t>(i) * N + j] -= f * A[static_cast<size_t>(k) * N + j];
            else
                B[static_cast<size_t>(i) * M + (j - N)] -= f * B[static_cast<size_t>(k) * M + (j - N)];
        }
        __syncthreads();
    }
}

// Sig[w][pq] += c[w] (S+ + S-)/2 + i sn[w] (S+ - S-)/2
__global__ void k_sigma_accumulate(const double *__restrict__ Sp, const double *__restrict__ Sm, int nn,
                                   const double *__restrict__ cw, const double *__restrict__ sw, int nw,
                                   cuDoubleComplex *__restrict__ Sig)
{
    const long long n = static_cast<long long>(nn) * nw;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const int w = static_cast<int>(t / nn), e = static_cast<int>(t % nn);
        const double cp = 0.5 * (Sp[e] + Sm[e]), sp = 0.5 * (Sp[e] - Sm[e]);
        cuDoubleComplex o = Sig[t];
        o.x += cw[w] * cp;
        o.y += sw[w] * sp;
        Sig[t] = o;
    }
}

// KS diagonal: out[n][w] = sum_pq conj(psi_np) Sig[w][p][q] psi_nq
__global__ void k_ks_diag(const cuDoubleComplex *__restrict__ psi, const cuDoubleComplex *__restrict__ Sig, int nb,
                          int nao, int nw, cuDoubleComplex *__restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nb * nw) return;
    const int n = t / nw, w = t % nw;
    const cuDoubleComplex *S = Sig + static_cast<size_t>(w) * nao * nao;
    const cuDoubleComplex *v = psi + static_cast<size_t>(n) * nao;
    double re = 0.0, im = 0.0;
    for (int p = 0; p < nao; ++p)
    {
        double ar = 0.0, ai = 0.0;  // (Sig psi)_p
        for (int q = 0; q < nao; ++q)
        {
            const cuDoubleComplex s = S[static_cast<size_t>(p) * nao + q], x = v[q];
            ar += s.x * x.x - s.y * x.y;
            ai += s.x * x.y + s.y * x.x;
        }
        re += v[p].x * ar + v[p].y * ai;  // conj(psi_p) (Sig psi)_p
        im += v[p].x * ai - v[p].y * ar;
    }
    out[t] = make_cuDoubleComplex(re, im);
}

// Real embedding of complex N x N matrices, batch-strided: E = [[Re A, -Im A], [Im A, Re A]]
// (2N x 2N).  Products, inverses and solves of embedded matrices are the embeddings of the complex
// ones, so the complex W_c(q) runs through the real kernels.
__global__ void k_embed(const cuDoubleComplex *__restrict__ A, long long sa, int N, int batch, double *__restrict__ E)
{
    const long long nn = static_cast<long long>(N) * N, n = nn * batch;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long b = t / nn, e = t % nn;
        const int i = static_cast<int>(e / N), j = static_cast<int>(e % N);
        const cuDoubleComplex v = A[b * sa + e];
        double *o = E + b * 4 * nn;
        const long long w = 2LL * N;
        o[i * w + j] = v.x;
        o[i * w + N + j] = -v.y;
        o[(N + i) * w + j] = v.y;
        o[(N + i) * w + N + j] = v.x;
    }
}

// The complex matrices back from their embeddings: re = E[0:N, 0:N], im = E[N:2N, 0:N].
__global__ void k_unembed(const double *__restrict__ E, int N, int batch, double *__restrict__ re, double *__restrict__ im)
{
    const long long nn = static_cast<long long>(N) * N, n = nn * batch;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long b = t / nn, e = t % nn;
        const int i = static_cast<int>(e / N), j = static_cast<int>(e % N);
        const double *o = E + b * 4 * nn;
        re[t] = o[static_cast<long long>(i) * 2 * N + j];
        im[t] = o[static_cast<long long>(N + i) * 2 * N + j];
    }
}

// Supercell matrix from cell-periodic blocks: X_s[(c a)][(d b)] = src[cell of R_d - R_c][a][b],
// src blocks cstride apart.
__global__ void k_to_super(const double *__restrict__ src, long long cstride, int n, int nc, const int *__restrict__ cdiff,
                           double *__restrict__ Xs)
{
    const long long ns = static_cast<long long>(nc) * n, tot = ns * ns;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < tot;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long r = t / ns, q = t % ns;
        const int c = static_cast<int>(r / n), a = static_cast<int>(r % n), d = static_cast<int>(q / n), b = static_cast<int>(q % n);
        Xs[t] = src[cdiff[d * nc + c] * cstride + static_cast<long long>(a) * n + b];
    }
}

// Sig[w][c][K][L] += cw[w] (S+ + S-)/2 + i sw[w] (S+ - S-)/2 with S(R_c)_KL the supercell row block
// of the cell R = 0 (row cell c0), column block c.
__global__ void k_sigma_rows(const double *__restrict__ Sp, const double *__restrict__ Sm, int c0, int nc, int n,
                             const double *__restrict__ cw, const double *__restrict__ sw, int nw,
                             cuDoubleComplex *__restrict__ Sig)
{
    const long long per = static_cast<long long>(nc) * n * n, tot = per * nw, ns = static_cast<long long>(nc) * n;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < tot;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const int w = static_cast<int>(t / per);
        const long long e = t % per;
        const int c = static_cast<int>(e / (static_cast<long long>(n) * n));
        const int K = static_cast<int>((e / n) % n), L = static_cast<int>(e % n);
        const long long src = (static_cast<long long>(c0) * n + K) * ns + static_cast<long long>(c) * n + L;
        const double cp = 0.5 * (Sp[src] + Sm[src]), sp = 0.5 * (Sp[src] - Sm[src]);
        cuDoubleComplex o = Sig[t];
        o.x += cw[w] * cp;
        o.y += sw[w] * sp;
        Sig[t] = o;
    }
}

unsigned grid_for(long long n) { return static_cast<unsigned>(std::min<long long>((n + 255) / 256, 152LL * 32)); }

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major, destroyed):
// eigenvalues w ascending, eigenvectors as the columns of Z (row-major n x n).
void sym_eig(std::vector<double> &A, int n, std::vector<double> &w, std::vector<double> &Z)
{
    Z.assign(static_cast<size_t>(n) * n, 0.0);
    for (int i = 0; i < n; ++i) Z[static_cast<size_t>(i) * n + i] = 1.0;
    auto a = [&](int i, int j) -> double & { return A[static_cast<size_t>(i) * n + j]; };
    double scale = 0.0;
    for (size_t t = 0; t < A.size(); ++t) scale = std::max(scale, std::fabs(A[t]));
    for (int sweep = 0; sweep < 100; ++sweep)
    {
        double off = 0.0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off = std::max(off, std::fabs(a(p, q)));
        if (off <= 1e-15 * scale) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q)
            {
                const double apq = a(p, q);
                if (std::fabs(apq) <= 1e-300) continue;
                const double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
                const double t = std::copysign(1.0, theta) / (std::fabs(theta) + std::sqrt(1.0 + theta * theta));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                for (int k = 0; k < n; ++k)
                {
                    const double akp = a(k, p), akq = a(k, q);
                    a(k, p) = c * akp - s * akq;
                    a(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k)
                {
                    const double apk = a(p, k), aqk = a(q, k);
                    a(p, k) = c * apk - s * aqk;
                    a(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k)
                {
                    double &zp = Z[static_cast<size_t>(k) * n + p], &zq = Z[static_cast<size_t>(k) * n + q];
                    const double x = zp, y = zq;
                    zp = c * x - s * y;
                    zq = s * x + c * y;
                }
            }
    }
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
    w.resize(n);
    std::vector<double> Zs(Z.size());
    for (int j = 0; j < n; ++j)
    {
        w[j] = a(ord[j], ord[j]);
        for (int k = 0; k < n; ++k) Zs[static_cast<size_t>(k) * n + j] = Z[static_cast<size_t>(k) * n + ord[j]];
    }
    Z.swap(Zs);
}

// A^p over the eigenvalues at or above the threshold (ascending order: the ones before the first
// eigenvalue >= threshold are dropped), as power_hemat_blacs does.
std::vector<double> power_sym(const std::vector<double> &A, int n, double power, double threshold)
{
    std::vector<double> B = A, w, Z;
    sym_eig(B, n, w, Z);
    int nf = n;
    for (int i = 0; i < n; ++i)
        if (w[i] >= threshold)
        {
            nf = i;
            break;
        }
    std::vector<double> out(static_cast<size_t>(n) * n, 0.0);
    for (int j = nf; j < n; ++j)
    {
        const double f = std::pow(w[j], power);
        for (int r = 0; r < n; ++r)
        {
            const double zr = Z[static_cast<size_t>(r) * n + j] * f;
            for (int c = 0; c < n; ++c) out[static_cast<size_t>(r) * n + c] += zr * Z[static_cast<size_t>(c) * n + j];
        }
    }
    return out;
}

// A^p of a complex Hermitian n x n matrix (row-major), over the eigenvalues at or above the
// threshold as power_sym: through its real symmetric embedding [[Re, -Im], [Im, Re]], whose
// eigenvalues are A's, each twice (power_hemat_blacs, utils_matrix_m_mpi.h:597-720).
std::vector<cplx> power_herm(const std::vector<cplx> &A, int n, double power, double threshold)
{
    const int m = 2 * n;
    std::vector<double> E(static_cast<size_t>(m) * m);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
        {
            const cplx v = A[static_cast<size_t>(i) * n + j];
            E[static_cast<size_t>(i) * m + j] = v.real();
            E[static_cast<size_t>(i) * m + n + j] = -v.imag();
            E[static_cast<size_t>(n + i) * m + j] = v.imag();
            E[static_cast<size_t>(n + i) * m + n + j] = v.real();
        }
    const std::vector<double> P = power_sym(E, m, power, threshold);
    std::vector<cplx> out(static_cast<size_t>(n) * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            out[static_cast<size_t>(i) * n + j] = cplx(P[static_cast<size_t>(i) * m + j], P[static_cast<size_t>(n + i) * m + j]);
    return out;
}

// Full Hermitian N x N matrix of the Coulomb blocks of k-point ik (upper pairs given).
std::vector<cplx> coulomb_k(const std::vector<VqBlock> &blocks, const std::vector<cplx> &blob, int ik,
                            const std::vector<int> &abf_off, int N)
{
    std::vector<cplx> V(static_cast<size_t>(N) * N, cplx(0, 0));
    for (const VqBlock &b : blocks)
    {
        if (b.ik != ik || b.I > b.J) continue;
        for (int m = 0; m < b.nmu; ++m)
            for (int n = 0; n < b.nnu; ++n)
            {
                const cplx v = blob[b.offset + static_cast<size_t>(m) * b.nnu + n];
                V[static_cast<size_t>(abf_off[b.I] + m) * N + abf_off[b.J] + n] = v;
                V[static_cast<size_t>(abf_off[b.J] + n) * N + abf_off[b.I] + m] = std::conj(v);
            }
    }
    return V;
}

// Full real symmetric N x N matrix of the Gamma-point Coulomb blocks (upper pairs, real part).
std::vector<double> coulomb_gamma(const std::vector<VqBlock> &blocks, const std::vector<cplx> &blob,
                                  const std::vector<int> &abf_off, int N)
{
    std::vector<double> V(static_cast<size_t>(N) * N, 0.0);
    for (const VqBlock &b : blocks)
    {
        if (b.ik != 0 || b.I > b.J) continue;
        for (int m = 0; m < b.nmu; ++m)
            for (int n = 0; n < b.nnu; ++n)
            {
                const double v = blob[b.offset + static_cast<size_t>(m) * b.nnu + n].real();
                V[static_cast<size_t>(abf_off[b.I] + m) * N + abf_off[b.J] + n] = v;
                V[static_cast<size_t>(abf_off[b.J] + n) * N + abf_off[b.I] + m] = v;
            }
    }
    return V;
}

// LibRI's filter of set_Ws / set_Gs / set_Vs / set_Ds (threshold_filter, RI_Tools.hpp:16-27, applied
// after the period folding of LRI-set.hpp:33-75): an atom-pair block of a cell-periodic matrix is
// dropped unless its largest |x| exceeds the threshold.  Block (I, J) of cell blockIdx.y and slice
// blockIdx.z of X, the cells cstride and the slices zstride elements apart, each cell n x n.
__global__ void k_block_filter(double *__restrict__ X, long long cstride, long long zstride, int n,
                               const int *__restrict__ off, int n_at, double thr)
{
    __shared__ double red[128];
    const int I = blockIdx.x / n_at, J = blockIdx.x % n_at;
    double *B = X + static_cast<long long>(blockIdx.y) * cstride + static_cast<long long>(blockIdx.z) * zstride;
    const int r0 = off[I], c0 = off[J], nr = off[I + 1] - r0, nc = off[J + 1] - c0;
    double m = 0.0;
    for (int t = threadIdx.x; t < nr * nc; t += blockDim.x)
        m = fmax(m, fabs(B[static_cast<long long>(r0 + t / nc) * n + c0 + t % nc]));
    red[threadIdx.x] = m;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1)
    {
        if (threadIdx.x < h) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + h]);
        __syncthreads();
    }
    if (red[0] > thr) return;
    for (int t = threadIdx.x; t < nr * nc; t += blockDim.x) B[static_cast<long long>(r0 + t / nc) * n + c0 + t % nc] = 0.0;
}

void block_filter_dev(double *X, long long cstride, int ncell, long long zstride, int nz, int n, const int *d_off,
                      int n_at, double thr, cudaStream_t st)
{
    if (thr <= 0.0) return;
    k_block_filter<<<dim3(n_at * n_at, ncell, nz), 128, 0, st>>>(X, cstride, zstride, n, d_off, n_at, thr);
    GB_LAUNCH_CHECK();
}

// The same filter on host cell-periodic blocks XR [cell][n][n] (the exchange's V(R) and D(R)).
void block_filter_host(std::vector<double> &XR, int n, const std::vector<int> &off, double thr)
{
    if (thr <= 0.0) return;
    const int n_at = static_cast<int>(off.size()) - 1;
    const size_t ncell = XR.size() / (static_cast<size_t>(n) * n);
    for (size_t c = 0; c < ncell; ++c)
        for (int I = 0; I < n_at; ++I)
            for (int J = 0; J < n_at; ++J)
            {
                double *B = XR.data() + c * n * n;
                double m = 0.0;
                for (int r = off[I]; r < off[I + 1]; ++r)
                    for (int q = off[J]; q < off[J + 1]; ++q) m = std::max(m, std::fabs(B[static_cast<size_t>(r) * n + q]));
                if (m > thr) continue;
                for (int r = off[I]; r < off[I + 1]; ++r)
                    for (int q = off[J]; q < off[J + 1]; ++q) B[static_cast<size_t>(r) * n + q] = 0.0;
            }
}

// The Born-von Karman supercell of the k-grid: atom (c, I) for cell c of the BvK list and atom
// I, cell-major.  Every k-grid quantity of the exchange and of Sigma_c is the Gamma-point
// quantity of this supercell, its matrices built from the cell-periodic blocks,
//   X_s[(c, A)][(c', B)] = X(R_c' - R_c)_AB,
// with the cell arithmetic of LibRI's periodic keys (BvK modulo, LRI_Cal_Tools.h:44-60).  With one
// k-point the supercell is the cell itself.
struct GammaSetup
{
    int n_at = 0, N = 0, nao = 0;      // supercell ABF and NAO counts (N = nc Nc, nao = nc naoc)
    int nc = 1, Nc = 0, naoc = 0, c0 = 0;  // cells, per-cell ABF and NAO counts, the cell R = 0
    std::vector<int> abf_off, ao_off;  // per atom of one cell
    std::vector<int> cdiff;            // [a][b]: cell of R_a - R_b
    std::vector<std::array<int, 3>> cells;
    DevBuf<double> U;                  // [(a, p), r] over the supercell
};

// U_s[a][p][r] += C, U_s[a][r][p] += C for the folded block (I, K, cell R) placed at every cell c:
// a = (c, I, mu), p = (c, I, i), r = (c + R, K, k).  At most the two writes of one block meet on an
// element (I = K, R = 0, i = k), so the atomic adds give the same sum in any order.
__global__ void k_super_u(const double *__restrict__ blob, const long long *__restrict__ off,
                          const int *__restrict__ meta, const int *__restrict__ nao_at, const int *__restrict__ nabf_at,
                          const int *__restrict__ ao_off, const int *__restrict__ abf_off,
                          const int *__restrict__ cadd, int nc, int Nc, int naoc, double *__restrict__ U)
{
    const int b = blockIdx.x, c = blockIdx.y;
    const int I = meta[4 * b], K = meta[4 * b + 1], R = meta[4 * b + 2];
    const int ni = nao_at[I], nk = nao_at[K], nmu = nabf_at[I];
    const int cK = cadd[c * nc + R];
    const long long naos = static_cast<long long>(nc) * naoc;
    const double *f = blob + off[b];
    const long long n = static_cast<long long>(ni) * nk * nmu;
    for (long long t = threadIdx.x; t < n; t += blockDim.x)
    {
        // block layout: (i * n_k + k) * n_mu + mu  (input.cpp:525-541)
        const int mu = static_cast<int>(t % nmu), k = static_cast<int>((t / nmu) % nk), i = static_cast<int>(t / (static_cast<long long>(nmu) * nk));
        const double v = f[t];
        const long long a = static_cast<long long>(c) * Nc + abf_off[I] + mu;
        const long long p = static_cast<long long>(c) * naoc + ao_off[I] + i;
        const long long r = static_cast<long long>(cK) * naoc + ao_off[K] + k;
        atomicAdd(U + (a * naos + p) * naos + r, v);
        atomicAdd(U + (a * naos + r) * naos + p, v);
    }
}

// The supercell of the handler's k-grid and its dense U from the RI blocks, folded onto the BvK
// cells and filtered by max |C| > thr after folding (LibRI set_tensors, RI_Tools.hpp:49-67,
// LRI-set.hpp:33-75).
// The RI coefficients the closed form contracts: the handler's (the basis of librpa_set_ao_basis_aux)
// or, for the exchange of a shrunk input, those of the small basis.
struct RiSet
{
    const std::vector<CsBlock> &blocks;
    const std::vector<double> &blob;
    const std::vector<int> &nabf;
};

void setup_gamma(const Dataset &ds, const RiSet &ri, double thr, GammaSetup &gs, cudaStream_t st)
{
    const int n_at = ds.n_atoms();
    GB_REQUIRE(n_at > 0 && static_cast<int>(ds.nao_at.size()) == n_at && static_cast<int>(ri.nabf.size()) == n_at,
               "wave-function and auxiliary bases must be set for every atom");
    gs.n_at = n_at;
    gs.abf_off.assign(n_at + 1, 0);
    gs.ao_off.assign(n_at + 1, 0);
    for (int I = 0; I < n_at; ++I)
    {
        gs.abf_off[I + 1] = gs.abf_off[I] + ri.nabf[I];
        gs.ao_off[I + 1] = gs.ao_off[I] + ds.nao_at[I];
    }
    gs.Nc = gs.abf_off[n_at];
    gs.naoc = gs.ao_off[n_at];
    GB_REQUIRE(gs.naoc == ds.n_ao, "sum of per-atom NAOs differs from the mean-field basis size");
    const PhaseTables pt = build_phase_tables(ds);
    gs.nc = pt.nc;
    gs.cells = pt.cells.R;
    gs.cdiff = pt.cdiff;
    gs.c0 = pt.cells.find(0, 0, 0);
    GB_REQUIRE(gs.c0 >= 0, "the BvK cell list lacks R = 0");
    gs.N = gs.nc * gs.Nc;
    gs.nao = gs.nc * gs.naoc;
    const int N = gs.N, nao = gs.nao, nc = gs.nc;
    GB_REQUIRE(static_cast<double>(N) * nao * nao <= 2.0e9,
               "the G0W0/exchange path holds the dense RI tensor of the BvK supercell (N_abf n_ao^2 values, "
               "times the cell count cubed on a k-grid): input too large");
    for (const CsBlock &b : ri.blocks)
        GB_REQUIRE(b.ni == ds.nao_at[b.I] && b.nj == ds.nao_at[b.J] && b.nmu == ri.nabf[b.I],
                   "RI block dimensions inconsistent with the bases");
    const Cells &cells = pt.cells;
    CsFold f = fold_cs_blocks(
        ri.blocks, ri.blob.data(), ri.blob.size(), ds.period,
        [&](const std::array<int, 3> &R) { return cells.find(R[0], R[1], R[2]); }, thr);
    // cadd[c][R]: cell of R_c + R_R
    std::vector<int> cadd(static_cast<size_t>(nc) * nc);
    for (int c = 0; c < nc; ++c)
        for (int r = 0; r < nc; ++r)
            cadd[static_cast<size_t>(c) * nc + r] = cells.find(cells.R[c][0] + cells.R[r][0], cells.R[c][1] + cells.R[r][1],
                                                               cells.R[c][2] + cells.R[r][2]);
    gs.U.alloc(static_cast<size_t>(N) * nao * nao);
    gs.U.zero(st);
    const int nblk = static_cast<int>(f.off.size());
    if (nblk > 0)
    {
        DevBuf<double> blob(ri.blob.size() + f.extra.size());
        blob.upload(ri.blob.data(), ri.blob.size(), st);
        if (!f.extra.empty())
            GB_CUDA(cudaMemcpyAsync(blob.get() + ri.blob.size(), f.extra.data(), f.extra.size() * sizeof(double),
                                    cudaMemcpyHostToDevice, st));
        auto d_off = to_dev(f.off, st);
        auto d_meta = to_dev(f.meta, st);
        auto d_nao = to_dev(ds.nao_at, st);
        auto d_nabf = to_dev(ri.nabf, st);
        auto d_aoo = to_dev(gs.ao_off, st);
        auto d_abo = to_dev(gs.abf_off, st);
        auto d_cadd = to_dev(cadd, st);
        k_super_u<<<dim3(nblk, nc), 256, 0, st>>>(blob.get(), d_off.get(), d_meta.get(), d_nao.get(), d_nabf.get(),
                                                  d_aoo.get(), d_abo.get(), d_cadd.get(), nc, gs.Nc, gs.naoc, gs.U.get());
        GB_LAUNCH_CHECK();
        GB_CUDA(cudaStreamSynchronize(st));  // the staged tables go out of scope
    }
}

void setup_gamma(const Dataset &ds, double thr, GammaSetup &gs, cudaStream_t st)
{
    setup_gamma(ds, RiSet{ds.cs_blocks, ds.cs_blob, ds.nabf_at}, thr, gs, st);
}

// X_s[(c a)][(c' b)] = XR[cell of R_c' - R_c][a][b] for the cell-periodic blocks XR [cell][n][n].
std::vector<double> to_supercell(const std::vector<double> &XR, int n, const GammaSetup &gs)
{
    const int nc = gs.nc;
    const size_t ns = static_cast<size_t>(nc) * n;
    std::vector<double> Xs(ns * ns);
    for (int c = 0; c < nc; ++c)
        for (int d = 0; d < nc; ++d)
        {
            const double *src = XR.data() + static_cast<size_t>(gs.cdiff[static_cast<size_t>(d) * nc + c]) * n * n;
            for (int a = 0; a < n; ++a)
                std::copy(src + static_cast<size_t>(a) * n, src + static_cast<size_t>(a + 1) * n,
                          Xs.data() + (static_cast<size_t>(c) * n + a) * ns + static_cast<size_t>(d) * n);
        }
    return Xs;
}

// Theta[k][c] = 2 pi kfrac_k . R_c
double k_dot_r(const Dataset &ds, int k, const std::array<int, 3> &R)
{
    return 2.0 * M_PI * (ds.kfrac[3 * k] * R[0] + ds.kfrac[3 * k + 1] * R[1] + ds.kfrac[3 * k + 2] * R[2]);
}

// V(R) [cell][N][N] = Re sum_k e^{-i 2 pi k.R} V(k) / n_k over the full k list, V(k) the full
// Hermitian matrix of the IBZ representative's upper blocks, conjugated for the other members of
// its star (FT_Vq, src/core/coulmat.cpp:7-90).
std::vector<double> coulomb_r(const Dataset &ds, const std::vector<VqBlock> &blocks, const std::vector<cplx> &blob,
                              const GammaSetup &gs)
{
    const int N = gs.Nc, nc = gs.nc, nk = ds.n_kpts;
    std::map<int, std::vector<cplx>> Vrep;
    for (const VqBlock &b : blocks)
    {
        if (b.I > b.J) continue;
        std::vector<cplx> &M = Vrep[b.ik];
        if (M.empty()) M.assign(static_cast<size_t>(N) * N, cplx(0, 0));
        for (int m = 0; m < b.nmu; ++m)
            for (int n = 0; n < b.nnu; ++n)
            {
                const cplx v = blob[b.offset + static_cast<size_t>(m) * b.nnu + n];
                M[static_cast<size_t>(gs.abf_off[b.I] + m) * N + gs.abf_off[b.J] + n] = v;
                M[static_cast<size_t>(gs.abf_off[b.J] + n) * N + gs.abf_off[b.I] + m] = std::conj(v);
            }
    }
    std::vector<double> VR(static_cast<size_t>(nc) * N * N, 0.0);
    for (int k = 0; k < nk; ++k)
    {
        const int rep = ds.ibz_map[k];
        auto it = Vrep.find(rep);
        if (it == Vrep.end()) continue;
        const bool cj = rep != k;
        for (int c = 0; c < nc; ++c)
        {
            const double th = k_dot_r(ds, k, gs.cells[c]);
            const cplx ph = std::polar(1.0 / nk, -th);
            double *dst = VR.data() + static_cast<size_t>(c) * N * N;
            for (size_t e = 0; e < static_cast<size_t>(N) * N; ++e)
                dst[e] += (ph * (cj ? std::conj(it->second[e]) : it->second[e])).real();
        }
    }
    return VR;
}

// D(R) [cell][nao][nao] = Re sum_k e^{-i 2 pi k.R} D(k), D(k)_ij = sum_n w_n psi_ni conj(psi_nj)
// with w = wg n_s / 2 (wg already divided by n_k), states up to the first below 1e-4 / n_k
// (MeanField::get_dmat_cplx_R, src/core/meanfield.cpp:201-244).
std::vector<double> dmat_r(const Dataset &ds, int s, const GammaSetup &gs)
{
    const int nao = gs.naoc, nc = gs.nc, nk = ds.n_kpts, nb = ds.n_states, ns = ds.n_spins;
    std::vector<double> DR(static_cast<size_t>(nc) * nao * nao, 0.0);
    std::vector<cplx> Dk(static_cast<size_t>(nao) * nao);
    for (int k = 0; k < nk; ++k)
    {
        std::fill(Dk.begin(), Dk.end(), cplx(0, 0));
        for (int n = 0; n < nb; ++n)
        {
            const double w = ds.wg[(static_cast<size_t>(s) * nk + k) * nb + n] * 0.5 * ns;
            if (w < 1e-4 / nk) break;
            const cplx *v = ds.wfc.data() + ((static_cast<size_t>(s) * nk + k) * nb + n) * nao;
            for (int i = 0; i < nao; ++i)
                for (int j = 0; j < nao; ++j) Dk[static_cast<size_t>(i) * nao + j] += w * v[i] * std::conj(v[j]);
        }
        for (int c = 0; c < nc; ++c)
        {
            const cplx ph = std::polar(1.0, -k_dot_r(ds, k, gs.cells[c]));
            double *dst = DR.data() + static_cast<size_t>(c) * nao * nao;
            for (size_t e = 0; e < Dk.size(); ++e) dst[e] += (ph * Dk[e]).real();
        }
    }
    return DR;
}

// H[p][q] = sum U[a,p,r] W[a,b] U[b,q,s] D[r,s] for each of nd matrices D (nd <= 2); Z = W U is
// formed once.  Work buffers: Y, Yt, Z, Zt.
struct HsWork
{
    DevBuf<double> Y, Yt, Z, Zt;
};

void hs_closed_form(const GammaSetup &gs, const double *W, const double *const *D, int nd, double *const *H,
                    HsWork &wk, cudaStream_t st)
{
    const int N = gs.N, nao = gs.nao;
    const long long nn = static_cast<long long>(nao) * nao, big = static_cast<long long>(N) * nn;
    if (wk.Y.size() < static_cast<size_t>(big))
    {
        wk.Y.alloc(big);
        wk.Yt.alloc(big);
        wk.Z.alloc(big);
        wk.Zt.alloc(big);
    }
    launch_dgemm(N, static_cast<int>(nn), N, W, N, 0, gs.U.get(), nn, 0, wk.Z.get(), nn, 0, 1, 1.0, 0.0, st);
    k_perm_z<<<grid_for(big), 256, 0, st>>>(wk.Z.get(), N, nao, wk.Zt.get());
    GB_LAUNCH_CHECK();
    for (int d = 0; d < nd; ++d)
    {
        launch_dgemm(N * nao, nao, nao, gs.U.get(), nao, 0, D[d], nao, 0, wk.Y.get(), nao, 0, 1, 1.0, 0.0, st);
        k_perm_y<<<grid_for(big), 256, 0, st>>>(wk.Y.get(), N, nao, wk.Yt.get());
        GB_LAUNCH_CHECK();
        launch_dgemm(nao, nao, static_cast<int>(static_cast<long long>(N) * nao), wk.Yt.get(), static_cast<long long>(N) * nao,
                     0, wk.Zt.get(), nao, 0, H[d], nao, 0, 1, 1.0, 0.0, st);
    }
}

// ---- the closed form on the tensor cores (3-piece BF16 splits, FP32 accumulation): the three
// products of hs_closed_form as split GEMMs.  The last one has a short output (n_ao x n_ao) and
// a long K (N n_ao), so K is cut into chunks of kChunkAbf supercell ABFs, each chunk a batch
// entry of the split GEMM, and the chunk partials are summed in FP64.
constexpr int kChunkAbf = 64;

// Zc[c][q][(al, s)] = Z[c kChunkAbf + al][(q, s)] (zero past N): the B operand of the last product
__global__ void k_chunk_z(const float *__restrict__ Z, int N, int nao, int nch, float *__restrict__ Zc)
{
    const long long kc = static_cast<long long>(kChunkAbf) * nao, n = static_cast<long long>(nch) * nao * kc;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long c = t / (static_cast<long long>(nao) * kc);
        const int q = static_cast<int>((t / kc) % nao);
        const long long k = t % kc;
        const long long a = c * kChunkAbf + k / nao;
        const int s = static_cast<int>(k % nao);
        Zc[t] = a < N ? Z[(a * nao + q) * nao + s] : 0.0f;
    }
}

// Yc[c][p][(al, s)] = Y[(c kChunkAbf + al, p)][s] (zero past N): the A operand of the last product
__global__ void k_chunk_y(const float *__restrict__ Y, int N, int nao, int nch, float *__restrict__ Yc)
{
    const long long kc = static_cast<long long>(kChunkAbf) * nao, n = static_cast<long long>(nch) * nao * kc;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long c = t / (static_cast<long long>(nao) * kc);
        const int p = static_cast<int>((t / kc) % nao);
        const long long k = t % kc;
        const long long a = c * kChunkAbf + k / nao;
        const int s = static_cast<int>(k % nao);
        Yc[t] = a < N ? Y[(a * nao + p) * nao + s] : 0.0f;
    }
}

// H[e] = sum_c Hp[c][e] in FP64
__global__ void k_sum_chunks(const float *__restrict__ Hp, long long nn, int nch, double *__restrict__ H)
{
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < nn;
         e += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        double acc = 0.0;
        for (int c = 0; c < nch; ++c) acc += static_cast<double>(Hp[static_cast<long long>(c) * nn + e]);
        H[e] = acc;
    }
}

struct HsSplitWork
{
    const GammaSetup *gs = nullptr;  // the setup whose U the cached splits hold
    SplitStore Ut, Ur, Wsp, Dsp, Zs, Ys;
    DevBuf<float> Zf, Yf, Zc, Yc, Hp;
    DevBuf<int> err;
};

int pad64(long long n) { return static_cast<int>((n + 63) / 64 * 64); }

void hs_closed_form_split(const GammaSetup &gs, const double *W, const double *const *D, int nd, double *const *H,
                          HsSplitWork &wk, cudaStream_t st)
{
    const int N = gs.N, nao = gs.nao;
    const long long nn = static_cast<long long>(nao) * nao, big = static_cast<long long>(N) * nn;
    const int kpN = pad64(N), kpA = pad64(nao);
    const int nch = (N + kChunkAbf - 1) / kChunkAbf;
    const long long kc = static_cast<long long>(kChunkAbf) * nao, chunked = static_cast<long long>(nch) * nao * kc;
    GB_REQUIRE(kc <= 0x7fffffffLL && big <= 0x7fffffffLL * 64LL, "supercell too large for the split closed form");
    if (wk.gs != &gs)
    {
        // U is fixed for the setup: its two operand layouts are split once
        wk.Ut.alloc(3, static_cast<size_t>(nn) * kpN);
        wk.Ur.alloc(3, static_cast<size_t>(N) * nao * kpA);
        split_transpose_f64(gs.U.get(), nn, N, static_cast<int>(nn), kpN, wk.Ut.bufs(), st);  // [(p, r)][a]
        split_rows_f64(gs.U.get(), nao, static_cast<long long>(N) * nao, nao, kpA, wk.Ur.bufs(), st);  // [(a, p)][r]
        wk.Wsp.alloc(3, static_cast<size_t>(N) * kpN);
        wk.Dsp.alloc(3, static_cast<size_t>(nao) * kpA);
        wk.Zf.alloc(big);
        wk.Yf.alloc(big);
        wk.Zc.alloc(chunked);
        wk.Yc.alloc(chunked);
        wk.Zs.alloc(3, chunked);
        wk.Ys.alloc(3, chunked);
        wk.Hp.alloc(static_cast<size_t>(nch) * nn);
        wk.err.alloc(1);
        wk.err.zero(st);
        wk.gs = &gs;
    }
    // Z = W U: Z[a][(q, s)]
    split_rows_f64(W, N, N, N, kpN, wk.Wsp.bufs(), st);
    tc_gemm_split(wk.Wsp.mat(N, kpN, 0), wk.Ut.mat(nn, kpN, 0), N, static_cast<int>(nn), N, 1, wk.Zf.get(), nn, 0,
                  false, wk.err.get(), st);
    k_chunk_z<<<grid_for(chunked), 256, 0, st>>>(wk.Zf.get(), N, nao, nch, wk.Zc.get());
    GB_LAUNCH_CHECK();
    split_rows_f32(wk.Zc.get(), kc, static_cast<long long>(nch) * nao, static_cast<int>(kc), static_cast<int>(kc),
                   wk.Zs.bufs(), st);
    for (int d = 0; d < nd; ++d)
    {
        // Y = U D: Y[(a, p)][s]
        split_transpose_f64(D[d], nao, nao, nao, kpA, wk.Dsp.bufs(), st);
        tc_gemm_split(wk.Ur.mat(static_cast<long long>(N) * nao, kpA, 0), wk.Dsp.mat(nao, kpA, 0), N * nao, nao, nao, 1,
                      wk.Yf.get(), nao, 0, false, wk.err.get(), st);
        k_chunk_y<<<grid_for(chunked), 256, 0, st>>>(wk.Yf.get(), N, nao, nch, wk.Yc.get());
        GB_LAUNCH_CHECK();
        split_rows_f32(wk.Yc.get(), kc, static_cast<long long>(nch) * nao, static_cast<int>(kc), static_cast<int>(kc),
                       wk.Ys.bufs(), st);
        // H = sum over chunks of Yc[c] Zc[c]^T
        tc_gemm_split(wk.Ys.mat(nao, kc, static_cast<long long>(nao) * kc), wk.Zs.mat(nao, kc, static_cast<long long>(nao) * kc),
                      nao, nao, static_cast<int>(kc), nch, wk.Hp.get(), nao, nn, false, wk.err.get(), st);
        k_sum_chunks<<<grid_for(nn), 256, 0, st>>>(wk.Hp.get(), nn, nch, H[d]);
        GB_LAUNCH_CHECK();
    }
    int herr = 0;
    wk.err.download(&herr, 1, st);
    GB_CUDA(cudaStreamSynchronize(st));
    GB_REQUIRE(herr == 0, "split GEMM of the self-energy closed form timed out");
}

// The correlation self-energy's closed form in the precision LibrpaGB300Options.sigma_precision
// asks for: FP64 GEMMs (the default), or the 3-piece split GEMMs where the split transpose of U
// fits its launch grid.  (The exchange stays FP64: through the split products its v_exx moved by
// up to 1 meV on MgO, far above the reference's print precision.)
struct SigmaClosedForm
{
    bool split = false;
    HsWork fp64;
    HsSplitWork tc;
    SigmaClosedForm(const Dataset &ds, const GammaSetup &gs)
    {
        const long long nn = static_cast<long long>(gs.nao) * gs.nao;
        split = ds.gbopt.sigma_precision == LIBRPA_GB300_SIGMA_BF16X3 && (nn + 31) / 32 <= 65535;
    }
    void run(const GammaSetup &gs, const double *W, const double *const *D, int nd, double *const *H, cudaStream_t st)
    {
        if (split)
            hs_closed_form_split(gs, W, D, nd, H, tc, st);
        else
            hs_closed_form(gs, W, D, nd, H, fp64, st);
    }
};

void require_gamma(const Dataset &ds)
{
    GB_REQUIRE(ds.n_kpts == 1 && ds.period[0] == 1 && ds.period[1] == 1 && ds.period[2] == 1,
               "the Gamma-point G0W0 chain takes one k-point (k-grids go through build_g0w0_kgrid)");
    GB_REQUIRE(ds.n_spinor == 1, "spinor (SOC) wave functions are not supported");
    GB_REQUIRE(ds.occ_set, "occupations/eigenvalues not set");
    for (size_t i = 0; i < ds.wfc_set.size(); ++i) GB_REQUIRE(ds.wfc_set[i], "wave function missing for some spin");
}

} // namespace

void build_exx(Dataset &ds, const LibrpaOptions &opts)
{
    GB_REQUIRE(ds.n_spinor == 1, "spinor (SOC) wave functions are not supported");
    GB_REQUIRE(ds.occ_set, "occupations/eigenvalues not set");
    for (size_t i = 0; i < ds.wfc_set.size(); ++i) GB_REQUIRE(ds.wfc_set[i], "wave function missing for some (spin, k)");
    GB_REQUIRE(!ds.vq_cut_blocks.empty(), "the truncated Coulomb matrix is not set (librpa_set_aux_cut_coulomb_*)");
    // with use_shrink_abfs the exchange contracts the RI coefficients of the small basis with the
    // truncated Coulomb matrix given there (Exx::build on Cs_shrinked_data, driver/task_gw_band.cpp:92-99)
    const bool shrink = opts.use_shrink_abfs == LIBRPA_SWITCH_ON;
    if (shrink)
    {
        GB_REQUIRE(static_cast<int>(ds.shrink_nabf.size()) == ds.n_atoms(),
                   "use_shrink_abfs: the small ABF basis must be set for every atom (librpa_gb300_set_shrink_basis)");
        GB_REQUIRE(!ds.shrink_cs_blocks.empty(),
                   "use_shrink_abfs: the exchange needs the RI coefficients of the small basis "
                   "(librpa_gb300_set_shrink_lri_coeff)");
    }
    GB_CUDA(cudaSetDevice(ds.gbopt.device));
    cudaStream_t st;
    GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct Guard
    {
        cudaStream_t s;
        ~Guard() { cudaStreamDestroy(s); }
    } guard{st};
    GammaSetup gs;
    if (shrink)
    {
        setup_gamma(ds, RiSet{ds.shrink_cs_blocks, ds.shrink_cs_blob, ds.shrink_nabf}, opts.libri_exx_threshold_C, gs, st);
    }
    else
        setup_gamma(ds, opts.libri_exx_threshold_C, gs, st);
    const int nao = gs.nao, naoc = gs.naoc, nc = gs.nc, ns = ds.n_spins;
    // V(R) and D(R) pass LibRI's block filters (libri_exx_threshold_V / _D; exx.cpp:365-418)
    std::vector<double> vr = coulomb_r(ds, ds.vq_cut_blocks, ds.vq_cut_blob, gs);
    block_filter_host(vr, gs.Nc, gs.abf_off, opts.libri_exx_threshold_V);
    const std::vector<double> vs = to_supercell(vr, gs.Nc, gs);
    const long long nn = static_cast<long long>(nao) * nao;
    DevBuf<double> dV(vs.size()), dD(nn), dH(nn);
    dV.upload(vs.data(), vs.size(), st);
    std::vector<double> hs(nn);
    HsWork wk;  // FP64: v_exx is held to the reference's print precision
    ds.hx.assign(ns, {});
    ds.hx_r.assign(ns, {});
    for (int s = 0; s < ns; ++s)
    {
        std::vector<double> dr = dmat_r(ds, s, gs);
        block_filter_host(dr, naoc, gs.ao_off, opts.libri_exx_threshold_D);
        const std::vector<double> dsup = to_supercell(dr, naoc, gs);
        dD.upload(dsup.data(), dsup.size(), st);
        const double *Dp[1] = {dD.get()};
        double *Hp[1] = {dH.get()};
        hs_closed_form(gs, dV.get(), Dp, 1, Hp, wk, st);
        dH.download(hs.data(), hs.size(), st);
        GB_CUDA(cudaStreamSynchronize(st));
        // H(R_c)_KL: the supercell row block of the cell R = 0, column block of cell c
        std::vector<double> &hr = ds.hx_r[s];
        hr.resize(static_cast<size_t>(nc) * naoc * naoc);
        for (int c = 0; c < nc; ++c)
            for (int K = 0; K < naoc; ++K)
                std::copy(hs.data() + (static_cast<size_t>(gs.c0) * naoc + K) * nao + static_cast<size_t>(c) * naoc,
                          hs.data() + (static_cast<size_t>(gs.c0) * naoc + K) * nao + static_cast<size_t>(c + 1) * naoc,
                          hr.data() + (static_cast<size_t>(c) * naoc + K) * naoc);
        ds.hx[s].assign(hr.begin() + static_cast<size_t>(gs.c0) * naoc * naoc,
                        hr.begin() + static_cast<size_t>(gs.c0 + 1) * naoc * naoc);
    }
    ds.hx_cells = gs.cells;
    ds.exx_generation = ds.generation;
}

double exx_state(const Dataset &ds, int s, int k, int n)
{
    const int nao = ds.n_ao, nk = ds.n_kpts;
    GB_REQUIRE(s >= 0 && s < static_cast<int>(ds.hx_r.size()) && k >= 0 && k < nk && n >= 0 && n < ds.n_states,
               "exchange state index out of range");
    const std::vector<double> &hr = ds.hx_r[s];
    const int nc = static_cast<int>(ds.hx_cells.size());
    // H(k) = sum_c e^{i 2 pi k.R_c} H(R_c) (Exx::build_KS_kgrid, src/core/exx.cpp:720-860)
    std::vector<cplx> Hk(static_cast<size_t>(nao) * nao, cplx(0, 0));
    for (int c = 0; c < nc; ++c)
    {
        const cplx ph = std::polar(1.0, k_dot_r(ds, k, ds.hx_cells[c]));
        const double *src = hr.data() + static_cast<size_t>(c) * nao * nao;
        for (size_t e = 0; e < Hk.size(); ++e) Hk[e] += ph * src[e];
    }
    const cplx *v = ds.wfc.data() + ((static_cast<size_t>(s) * nk + k) * ds.n_states + n) * nao;
    cplx acc(0, 0);
    for (int p = 0; p < nao; ++p)
    {
        cplx hv(0, 0);
        for (int q = 0; q < nao; ++q) hv += Hk[static_cast<size_t>(p) * nao + q] * v[q];
        acc += std::conj(v[p]) * hv;
    }
    return -acc.real();
}

void build_g0w0_gamma(Dataset &ds, const LibrpaOptions &opts, const TimeFreqGrids &tf)
{
    require_gamma(ds);
    GB_REQUIRE(!ds.vq_cut_blocks.empty(), "the truncated Coulomb matrix is not set (librpa_set_aux_cut_coulomb_*)");
    GB_REQUIRE(!ds.vq_blocks.empty(), "the Coulomb matrix of the dielectric function is not set");
    // chi0(q = 0, omega) from the RPA path, kept on the device
    {
        const LibrpaGB300Options saved = ds.gbopt;
        ds.gbopt.stage = LIBRPA_GB300_STAGE_CHI0;
        ds.gbopt.tau_begin = 0;
        ds.gbopt.tau_end = -1;
        try
        {
            run_rpa_gpu(ds, opts, tf, opts.n_bands_chi0);
        }
        catch (...)
        {
            ds.gbopt = saved;
            throw;
        }
        ds.gbopt = saved;
    }
    GB_REQUIRE(ds.kept_chi0 && ds.kept_nq == 1 && ds.kept_nfreq == tf.n, "chi0(omega) was not kept");
    GB_CUDA(cudaSetDevice(ds.gbopt.device));
    cudaStream_t st;
    GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct Guard
    {
        cudaStream_t s;
        ~Guard() { cudaStreamDestroy(s); }
    } guard{st};
    GammaSetup gs;
    setup_gamma(ds, opts.libri_g0w0_threshold_C, gs, st);
    const int N = gs.N, nao = gs.nao, nb = ds.n_states, ns = ds.n_spins, nw = tf.n;
    const long long NN = static_cast<long long>(N) * N, nn = static_cast<long long>(nao) * nao;

    // S = V^1/2, S_c = V_cut^1/2 on the host (one eigen-decomposition each), then on the device
    const std::vector<double> ve = coulomb_gamma(ds.vq_blocks, ds.vq_blob, gs.abf_off, N);
    const std::vector<double> vc = coulomb_gamma(ds.vq_cut_blocks, ds.vq_cut_blob, gs.abf_off, N);
    const std::vector<double> hS = power_sym(ve, N, 0.5, opts.sqrt_coulomb_threshold);
    const std::vector<double> hSc = power_sym(vc, N, 0.5, opts.sqrt_coulomb_threshold);
    DevBuf<double> S(NN), Sc(NN), ScSc(NN);
    S.upload(hS.data(), NN, st);
    Sc.upload(hSc.data(), NN, st);
    launch_dgemm(N, N, N, Sc.get(), N, 0, Sc.get(), N, 0, ScSc.get(), N, 0, 1, 1.0, 0.0, st);

    // chi0(omega) as full real matrices (real part at Gamma, lower blocks the transposes)
    DevBuf<double> X(NN * nw), T(NN * nw), Wf(NN * nw), Y(NN * nw);
    {
        std::vector<int> atom_of(N), pair_of(static_cast<size_t>(gs.n_at) * gs.n_at, -1), abf_off_n(gs.n_at),
            nabf(gs.n_at);
        std::vector<long long> eoff;
        long long e = 0;
        for (int I = 0; I < gs.n_at; ++I)
            for (int J = I; J < gs.n_at; ++J)
            {
                pair_of[static_cast<size_t>(I) * gs.n_at + J] = static_cast<int>(eoff.size());
                eoff.push_back(e);
                e += static_cast<long long>(ds.nabf_at[I]) * ds.nabf_at[J];
            }
        for (int I = 0; I < gs.n_at; ++I)
        {
            abf_off_n[I] = gs.abf_off[I];
            nabf[I] = ds.nabf_at[I];
            for (int a = gs.abf_off[I]; a < gs.abf_off[I + 1]; ++a) atom_of[a] = I;
        }
        GB_REQUIRE(static_cast<size_t>(e) == ds.kept_pair_elems, "kept chi0 layout does not match the bases");
        DevBuf<int> d_atom(N), d_pair(pair_of.size()), d_off(gs.n_at), d_nabf(gs.n_at);
        DevBuf<long long> d_eoff(eoff.size());
        d_atom.upload(atom_of.data(), N, st);
        d_pair.upload(pair_of.data(), pair_of.size(), st);
        d_off.upload(abf_off_n.data(), gs.n_at, st);
        d_nabf.upload(nabf.data(), gs.n_at, st);
        d_eoff.upload(eoff.data(), eoff.size(), st);
        launch_assemble_chi0(static_cast<const cuDoubleComplex *>(ds.kept_chi0), e, nw, N, d_atom.get(), d_off.get(),
                             d_nabf.get(), d_pair.get(), gs.n_at, d_eoff.get(), true, nullptr, X.get(), NN, st);
        GB_CUDA(cudaStreamSynchronize(st));
    }
    // eps = 1 - S chi0 S; W_c = S_c eps^-1 S_c - S_c S_c (the solve: Y = eps^-1 S_c)
    launch_dgemm(N, N, N, S.get(), N, 0, X.get(), N, NN, T.get(), N, NN, nw, 1.0, 0.0, st);
    launch_dgemm(N, N, N, T.get(), N, NN, S.get(), N, 0, X.get(), N, NN, nw, 1.0, 0.0, st);  // X <- S chi0 S
    k_one_minus<<<grid_for(NN * nw), 256, 0, st>>>(X.get(), N, nw);
    GB_LAUNCH_CHECK();
    for (int w = 0; w < nw; ++w)
        GB_CUDA(cudaMemcpyAsync(Y.get() + w * NN, Sc.get(), sizeof(double) * NN, cudaMemcpyDeviceToDevice, st));
    DevBuf<int> bad(1);
    bad.zero(st);
    const size_t gj_smem = sizeof(double) * N;
    GB_REQUIRE(gj_smem <= 48 * 1024, "auxiliary basis too large for the Gamma-point W_c solve");
    k_gj_solve<<<nw, 256, gj_smem, st>>>(X.get(), Y.get(), N, N, bad.get());
    GB_LAUNCH_CHECK();
    launch_dgemm(N, N, N, Sc.get(), N, 0, Y.get(), N, NN, Wf.get(), N, NN, nw, 1.0, 0.0, st);
    {
        // W_c(omega) -= S_c S_c for every frequency: one GEMM with a column of -1
        std::vector<double> ones(nw, -1.0);
        DevBuf<double> d_ones(nw);
        d_ones.upload(ones.data(), nw, st);
        launch_dgemm(nw, static_cast<int>(NN), 1, d_ones.get(), 1, 0, ScSc.get(), NN, 0, Wf.get(), NN, 0, 1, 1.0, 1.0, st);
        int hbad = 0;
        bad.download(&hbad, 1, st);
        GB_CUDA(cudaStreamSynchronize(st));
        GB_REQUIRE(hbad == 0, "1 - S chi0 S is singular: no W_c");
    }
    // W_c(tau) = sum_omega cos_f2t[tau][omega] W_c(omega): one GEMM over the frequency axis
    DevBuf<double> d_f2t(static_cast<size_t>(nw) * nw), Wt(NN * nw);
    d_f2t.upload(tf.cos_f2t.data(), static_cast<size_t>(nw) * nw, st);
    launch_dgemm(nw, static_cast<int>(NN), nw, d_f2t.get(), nw, 0, Wf.get(), NN, 0, Wt.get(), NN, 0, 1, 1.0, 0.0, st);
    X.release();
    T.release();
    Y.release();
    Wf.release();

    // Sigma_c(i omega) = sum_tau [cos_t2f (S+ + S-)/2 + i sin_t2f (S+ - S-)/2] per spin, then the KS diagonal
    DevBuf<cuDoubleComplex> Sig(nn * nw), dpsi(static_cast<size_t>(nb) * nao), sks(static_cast<size_t>(nb) * nw);
    DevBuf<double> sgn_s(2ull * nb), Gp(nn), Gm(nn), Sp(nn), Sm(nn), cw(nw), sw(nw);
    SigmaClosedForm cf(ds, gs);
    // LibRI's set_Ws filter on every W(tau) (libri_g0w0_threshold_Wc; gw.cpp:459-470)
    auto d_aoo_f = to_dev(gs.ao_off, st);
    auto d_abo_f = to_dev(gs.abf_off, st);
    block_filter_dev(Wt.get(), 0, 1, NN, nw, N, d_abo_f.get(), gs.n_at, opts.libri_g0w0_threshold_Wc, st);
    ds.sigc_ks.assign(ns, {});
    ds.sigc_r.assign(ns, {});
    for (int s = 0; s < ns; ++s)
    {
        Sig.zero(st);
        dpsi.upload(reinterpret_cast<const cuDoubleComplex *>(ds.wfc.data()) + static_cast<size_t>(s) * nb * nao,
                    static_cast<size_t>(nb) * nao, st);
        for (int it = 0; it < nw; ++it)
        {
            const double tau = tf.tau[it];
            // G(+-tau) weights (chi0.cpp:348-365): w+ = max(0, 1/n_k - f n_s/2) unoccupied side,
            // w- = f n_s/2 with sign -1; s = exp(min(0, -tau (e - e_F))) w
            std::vector<double> sp(nb), sm(nb);
            for (int n = 0; n < nb; ++n)
            {
                const double f = ds.wg[static_cast<size_t>(s) * nb + n];
                const double e = ds.ekb[static_cast<size_t>(s) * nb + n] - ds.efermi;
                const double wp = std::max(0.0, 1.0 / ds.n_kpts - f * 0.5 * ns), wm = f * 0.5 * ns;
                if (opts.n_bands_chi0 >= 0 && n >= opts.n_bands_chi0)
                {
                    sp[n] = sm[n] = 0.0;
                    continue;
                }
                sp[n] = std::exp(std::min(0.0, -tau * e)) * wp;
                sm[n] = std::exp(std::min(0.0, tau * e)) * wm;
            }
            sgn_s.upload(sp.data(), nb, st);
            k_gamma_dm<<<(nao * nao + 255) / 256, 256, 0, st>>>(dpsi.get(), sgn_s.get(), nb, nao, 1.0, Gp.get());
            GB_LAUNCH_CHECK();
            GB_CUDA(cudaStreamSynchronize(st));
            sgn_s.upload(sm.data(), nb, st);
            k_gamma_dm<<<(nao * nao + 255) / 256, 256, 0, st>>>(dpsi.get(), sgn_s.get(), nb, nao, -1.0, Gm.get());
            GB_LAUNCH_CHECK();
            // LibRI's set_Gs filter (libri_g0w0_threshold_G; gw.cpp:546-616)
            block_filter_dev(Gp.get(), 0, 1, 0, 1, nao, d_aoo_f.get(), gs.n_at, opts.libri_g0w0_threshold_G, st);
            block_filter_dev(Gm.get(), 0, 1, 0, 1, nao, d_aoo_f.get(), gs.n_at, opts.libri_g0w0_threshold_G, st);
            const double *Dp[2] = {Gp.get(), Gm.get()};
            double *Hp[2] = {Sp.get(), Sm.get()};
            cf.run(gs, Wt.get() + it * NN, Dp, 2, Hp, st);
            std::vector<double> c(nw), sn(nw);
            for (int w = 0; w < nw; ++w)
            {
                c[w] = tf.cos_t2f[static_cast<size_t>(w) * nw + it];
                sn[w] = tf.sin_t2f[static_cast<size_t>(w) * nw + it];
            }
            cw.upload(c.data(), nw, st);
            sw.upload(sn.data(), nw, st);
            k_sigma_accumulate<<<grid_for(nn * nw), 256, 0, st>>>(Sp.get(), Sm.get(), static_cast<int>(nn), cw.get(),
                                                                   sw.get(), nw, Sig.get());
            GB_LAUNCH_CHECK();
            GB_CUDA(cudaStreamSynchronize(st));  // the host weight vectors are reused
        }
        k_ks_diag<<<(nb * nw + 127) / 128, 128, 0, st>>>(dpsi.get(), Sig.get(), nb, nao, nw, sks.get());
        GB_LAUNCH_CHECK();
        ds.sigc_ks[s].resize(static_cast<size_t>(nb) * nw);
        sks.download(reinterpret_cast<cuDoubleComplex *>(ds.sigc_ks[s].data()), ds.sigc_ks[s].size(), st);
        ds.sigc_r[s].resize(static_cast<size_t>(nw) * nn);  // [omega][cell R = 0][p][q]
        Sig.download(reinterpret_cast<cuDoubleComplex *>(ds.sigc_r[s].data()), ds.sigc_r[s].size(), st);
        GB_CUDA(cudaStreamSynchronize(st));
    }
    ds.hx_cells = gs.cells;
    ds.gw_omega = tf.omega;
    ds.g0w0_generation = ds.generation;
    release_kept(ds);
}


// G0W0 on a k-grid (task = g0w0 with k-points; epsilon.cpp:1763-2322, :2323-2660, gw.cpp:217-876,
// :884-1240): W_c(q, omega) at every IBZ q by the real embedding of the complex matrices, with the
// head of the dielectric matrix replaced at q = 0 when replace_w_head is on (epsilon.cpp:2030-2120);
// W_c(R, omega) = Re sum_k e^{-i 2 pi k.R} W_c(k, omega) / n_k over the full k list (conjugated for
// the time-reversed members of a star); W_c(R, tau) by costrans_f2t; Sigma_c(R, +-tau) as the
// Gamma-point closed form of the BvK supercell with G(R, +-tau); Sigma_c(k, i omega) on the KS
// states of every k-point.
void build_g0w0_kgrid(Dataset &ds, const LibrpaOptions &opts, const TimeFreqGrids &tf)
{
    GB_REQUIRE(ds.n_spinor == 1, "spinor (SOC) wave functions are not supported");
    GB_REQUIRE(ds.occ_set, "occupations/eigenvalues not set");
    for (size_t i = 0; i < ds.wfc_set.size(); ++i) GB_REQUIRE(ds.wfc_set[i], "wave function missing for some (spin, k)");
    GB_REQUIRE(!ds.vq_cut_blocks.empty(), "the truncated Coulomb matrix is not set (librpa_set_aux_cut_coulomb_*)");
    GB_REQUIRE(!ds.vq_blocks.empty(), "the Coulomb matrix of the dielectric function is not set");
    const int nw = tf.n;
    const bool head = opts.replace_w_head == LIBRPA_SWITCH_ON && !ds.dielect_eps.empty();
    // eps_mac on the minimax frequencies (compute_g0w0.cpp:103-107, interpolate_dielec_func):
    // option 0 the given values, 1 a cubic spline, 2 a fitted Havriliak-Negami model; the
    // option 3 head of the reference comes from its velocity-matrix model, which its C API
    // does not feed
    std::vector<double> eps_head;
    if (head)
    {
        GB_REQUIRE(opts.option_dielect_func >= 0 && opts.option_dielect_func <= 2,
                   "replace_w_head: option_dielect_func must be 0, 1 or 2 (3 needs the head and wings of the "
                   "dielectric model, which the C API does not set)");
        eps_head = interpolate_dielec_func(opts.option_dielect_func, ds.dielect_omega, ds.dielect_eps, tf.omega);
    }
    // chi0(q, omega) of every IBZ q from the RPA path, kept on the device
    {
        const LibrpaGB300Options saved = ds.gbopt;
        ds.gbopt.stage = LIBRPA_GB300_STAGE_CHI0;
        ds.gbopt.tau_begin = 0;
        ds.gbopt.tau_end = -1;
        try
        {
            run_rpa_gpu(ds, opts, tf, opts.n_bands_chi0);
        }
        catch (...)
        {
            ds.gbopt = saved;
            throw;
        }
        ds.gbopt = saved;
    }
    GB_REQUIRE(ds.kept_chi0 && ds.kept_nfreq == nw, "chi0(q, omega) was not kept");
    GB_CUDA(cudaSetDevice(ds.gbopt.device));
    cudaStream_t st;
    GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct Guard
    {
        cudaStream_t s;
        ~Guard() { cudaStreamDestroy(s); }
    } guard{st};
    GammaSetup gs;
    setup_gamma(ds, opts.libri_g0w0_threshold_C, gs, st);
    const PhaseTables pt = build_phase_tables(ds);
    const int Nc = gs.Nc, naoc = gs.naoc, nc = gs.nc, nq = pt.nq, nk = ds.n_kpts, nb = ds.n_states, ns = ds.n_spins;
    const int n_at = gs.n_at, N2 = 2 * Nc;
    GB_REQUIRE(ds.kept_nq == nq, "kept chi0 holds another IBZ");
    const long long NN = static_cast<long long>(Nc) * Nc, M4 = 4 * NN, e_tot = static_cast<long long>(ds.kept_pair_elems);
    const double thr = opts.sqrt_coulomb_threshold;

    // layout tables of the kept chi0 (upper atom pairs of one cell)
    std::vector<int> atom_of(Nc), pair_of(static_cast<size_t>(n_at) * n_at, -1), abf_off_n(n_at), nabf(n_at);
    std::vector<long long> eoff;
    {
        long long e = 0;
        for (int I = 0; I < n_at; ++I)
            for (int J = I; J < n_at; ++J)
            {
                pair_of[static_cast<size_t>(I) * n_at + J] = static_cast<int>(eoff.size());
                eoff.push_back(e);
                e += static_cast<long long>(ds.nabf_at[I]) * ds.nabf_at[J];
            }
        GB_REQUIRE(e == e_tot, "kept chi0 layout does not match the bases");
        for (int I = 0; I < n_at; ++I)
        {
            abf_off_n[I] = gs.abf_off[I];
            nabf[I] = ds.nabf_at[I];
            for (int a = gs.abf_off[I]; a < gs.abf_off[I + 1]; ++a) atom_of[a] = I;
        }
    }
    auto d_atom = to_dev(atom_of, st);
    auto d_pair = to_dev(pair_of, st);
    auto d_off = to_dev(abf_off_n, st);
    auto d_nabf = to_dev(nabf, st);
    auto d_eoff = to_dev(eoff, st);

    // ---- W_c(q, omega), [Re | Im][q][omega][N][N]
    // With use_shrink_abfs the dielectric function and W_c live in the small ABF basis of the
    // Coulomb matrices: chi0_s = U chi0 U^H first (shrink_abfs_chi0, chi0.cpp:711-898), and W_c is
    // taken back to the basis of the RI coefficients as U^H W_c U (unfold_abfs_Wc, the two pgemm
    // calls of src/gw_old.cpp:208-225) before the q -> R transform.  Both run on the real
    // embeddings: U^H embeds as the transpose of U's embedding.
    const bool shrink = opts.use_shrink_abfs == LIBRPA_SWITCH_ON;
    std::vector<int> abf_off_w = gs.abf_off;
    if (shrink)
    {
        GB_REQUIRE(static_cast<int>(ds.shrink_nabf.size()) == n_at,
                   "use_shrink_abfs: the small ABF basis must be set for every atom (librpa_gb300_set_shrink_basis)");
        for (int I = 0; I < n_at; ++I)
        {
            GB_REQUIRE(ds.shrink_nabf[I] > 0, "use_shrink_abfs: small ABF counts must be positive");
            abf_off_w[I + 1] = abf_off_w[I] + ds.shrink_nabf[I];
        }
    }
    const int Nw = abf_off_w[n_at], N2w = 2 * Nw;
    const long long NNw = static_cast<long long>(Nw) * Nw, M4w = 4 * NNw;
    DevBuf<double> Wq(2ull * nq * nw * NN);
    {
        DevBuf<cuDoubleComplex> X(static_cast<size_t>(nw) * NN);
        DevBuf<double> Xe(nw * M4w), T(nw * M4w), Ye(nw * M4w), We(nw * M4w), Se(M4w), Sce(M4w), ScSc(M4w), d_ones(nw);
        // shrink: the embedded chi0 of the large basis, U_e (2 Nw x 2 Nc) and its transpose, and a
        // (2 Nw x 2 Nc) / (2 Nc x 2 Nw) product per frequency
        DevBuf<double> Xl, Ue, UeT, Tsl;
        if (shrink)
        {
            Xl.alloc(nw * M4);
            Ue.alloc(static_cast<size_t>(N2w) * N2);
            UeT.alloc(static_cast<size_t>(N2w) * N2);
            Tsl.alloc(static_cast<size_t>(nw) * N2w * N2);
        }
        DevBuf<int> bad(1);
        bad.zero(st);
        std::vector<double> ones(nw, -1.0);
        d_ones.upload(ones.data(), nw, st);
        auto embed_h = [&](const std::vector<cplx> &A) {
            std::vector<double> E(M4w);
            for (int i = 0; i < Nw; ++i)
                for (int j = 0; j < Nw; ++j)
                {
                    const cplx v = A[static_cast<size_t>(i) * Nw + j];
                    E[static_cast<size_t>(i) * N2w + j] = v.real();
                    E[static_cast<size_t>(i) * N2w + Nw + j] = -v.imag();
                    E[static_cast<size_t>(Nw + i) * N2w + j] = v.imag();
                    E[static_cast<size_t>(Nw + i) * N2w + Nw + j] = v.real();
                }
            return E;
        };
        const size_t gj_smem = sizeof(double) * N2w;
        GB_REQUIRE(gj_smem <= 48 * 1024, "auxiliary basis too large for the W_c solve");
        for (int q = 0; q < nq; ++q)
        {
            const int kq = pt.ibz_rep[q];
            const std::vector<cplx> ve = coulomb_k(ds.vq_blocks, ds.vq_blob, kq, abf_off_w, Nw);
            const std::vector<cplx> vc = coulomb_k(ds.vq_cut_blocks, ds.vq_cut_blob, kq, abf_off_w, Nw);
            const bool gq = std::fabs(ds.kfrac[3 * kq]) < 1e-10 && std::fabs(ds.kfrac[3 * kq + 1]) < 1e-10 &&
                            std::fabs(ds.kfrac[3 * kq + 2]) < 1e-10;
            const bool head_q = gq && head;
            std::vector<double> z0;
            double w0 = 0.0;
            std::vector<double> se_h;
            if (head_q)
            {
                // power_hemat_blacs_real on Re V (utils_matrix_m_mpi.h:886-1010): S = V^1/2 over the
                // eigenvalues at or above the threshold; z0 the eigenvector of the largest one
                std::vector<double> rv(NNw);
                for (long long e = 0; e < NNw; ++e) rv[e] = ve[e].real();
                std::vector<double> B = rv, w, Z;
                sym_eig(B, Nw, w, Z);
                w0 = w[Nw - 1];
                GB_REQUIRE(w0 >= thr, "replace_w_head: the Coulomb matrix at q = 0 has no eigenvalue above the threshold");
                z0.resize(Nw);
                for (int r = 0; r < Nw; ++r) z0[r] = Z[static_cast<size_t>(r) * Nw + Nw - 1];
                const std::vector<double> S = power_sym(rv, Nw, 0.5, thr);
                std::vector<cplx> Sc(NNw);
                for (long long e = 0; e < NNw; ++e) Sc[e] = S[e];
                se_h = embed_h(Sc);
            }
            else
                se_h = embed_h(power_herm(ve, Nw, 0.5, thr));
            const std::vector<double> sc_h = embed_h(power_herm(vc, Nw, 0.5, thr));
            Se.upload(se_h.data(), M4w, st);
            Sce.upload(sc_h.data(), M4w, st);
            launch_dgemm(N2w, N2w, N2w, Sce.get(), N2w, 0, Sce.get(), N2w, 0, ScSc.get(), N2w, 0, 1, 1.0, 0.0, st);
            launch_assemble_chi0(static_cast<const cuDoubleComplex *>(ds.kept_chi0) + static_cast<long long>(q) * e_tot,
                                 static_cast<long long>(nq) * e_tot, nw, Nc, d_atom.get(), d_off.get(), d_nabf.get(),
                                 d_pair.get(), n_at, d_eoff.get(), false, X.get(), nullptr, NN, st);
            if (shrink)
            {
                auto it = ds.shrink_u.find(kq);
                GB_REQUIRE(it != ds.shrink_u.end(), "use_shrink_abfs: no shrink transform U(q) for IBZ k index " +
                                                        std::to_string(kq) + " (librpa_gb300_set_shrink_sinvS)");
                const Dataset::ShrinkU &u = it->second;
                GB_REQUIRE(u.n_small == Nw && u.n_large == Nc,
                           "use_shrink_abfs: U(q) must be (sum of small ABFs) x (sum of ABFs) = " + std::to_string(Nw) +
                               " x " + std::to_string(Nc));
                std::vector<double> ue(static_cast<size_t>(N2w) * N2), uet(static_cast<size_t>(N2w) * N2);
                for (int i = 0; i < Nw; ++i)
                    for (int j = 0; j < Nc; ++j)
                    {
                        const cplx v = u.u[static_cast<size_t>(i) * Nc + j];
                        const size_t r0 = static_cast<size_t>(i) * N2, r1 = static_cast<size_t>(Nw + i) * N2;
                        ue[r0 + j] = v.real();
                        ue[r0 + Nc + j] = -v.imag();
                        ue[r1 + j] = v.imag();
                        ue[r1 + Nc + j] = v.real();
                    }
                for (int r = 0; r < N2w; ++r)
                    for (int c = 0; c < N2; ++c) uet[static_cast<size_t>(c) * N2w + r] = ue[static_cast<size_t>(r) * N2 + c];
                Ue.upload(ue.data(), ue.size(), st);
                UeT.upload(uet.data(), uet.size(), st);
                k_embed<<<grid_for(NN * nw), 256, 0, st>>>(X.get(), NN, Nc, nw, Xl.get());
                GB_LAUNCH_CHECK();
                // chi0_s = U chi0 U^H
                launch_dgemm(N2w, N2, N2, Ue.get(), N2, 0, Xl.get(), N2, M4, Tsl.get(), N2, static_cast<long long>(N2w) * N2,
                             nw, 1.0, 0.0, st);
                launch_dgemm(N2w, N2w, N2, Tsl.get(), N2, static_cast<long long>(N2w) * N2, UeT.get(), N2w, 0, Xe.get(),
                             N2w, M4w, nw, 1.0, 0.0, st);
            }
            else
            {
                k_embed<<<grid_for(NN * nw), 256, 0, st>>>(X.get(), NN, Nc, nw, Xe.get());
                GB_LAUNCH_CHECK();
            }
            // the head element of chi0 in V's eigenbasis, w0 z0^T chi0 z0, from the embedded chi0
            std::vector<cplx> x00(head_q ? nw : 0);
            if (head_q)
            {
                std::vector<double> hxe(nw * M4w);
                Xe.download(hxe.data(), hxe.size(), st);
                GB_CUDA(cudaStreamSynchronize(st));
                for (int w = 0; w < nw; ++w)
                {
                    const double *E = hxe.data() + static_cast<size_t>(w) * M4w;
                    cplx acc(0, 0);
                    for (int r = 0; r < Nw; ++r)
                        for (int c = 0; c < Nw; ++c)
                            acc += z0[r] * cplx(E[static_cast<size_t>(r) * N2w + c], E[static_cast<size_t>(Nw + r) * N2w + c]) * z0[c];
                    x00[w] = w0 * acc;
                }
            }
            // S chi0 S
            launch_dgemm(N2w, N2w, N2w, Se.get(), N2w, 0, Xe.get(), N2w, M4w, T.get(), N2w, M4w, nw, 1.0, 0.0, st);
            launch_dgemm(N2w, N2w, N2w, T.get(), N2w, M4w, Se.get(), N2w, 0, Xe.get(), N2w, M4w, nw, 1.0, 0.0, st);
            if (head_q)
            {
                // in V's eigenbasis the (0, 0) element of S chi0 S becomes 1 - eps_mac: add
                // ((1 - eps_mac) - X00) z0 z0^T
                std::vector<double> hxe(nw * M4w);
                Xe.download(hxe.data(), hxe.size(), st);
                GB_CUDA(cudaStreamSynchronize(st));
                for (int w = 0; w < nw; ++w)
                {
                    const cplx d = (1.0 - eps_head[w]) - x00[w];
                    double *E = hxe.data() + static_cast<size_t>(w) * M4w;
                    for (int r = 0; r < Nw; ++r)
                        for (int c = 0; c < Nw; ++c)
                        {
                            const double zz = z0[r] * z0[c];
                            E[static_cast<size_t>(r) * N2w + c] += d.real() * zz;
                            E[static_cast<size_t>(r) * N2w + Nw + c] -= d.imag() * zz;
                            E[static_cast<size_t>(Nw + r) * N2w + c] += d.imag() * zz;
                            E[static_cast<size_t>(Nw + r) * N2w + Nw + c] += d.real() * zz;
                        }
                }
                Xe.upload(hxe.data(), hxe.size(), st);
            }
            // eps = 1 - S chi0 S; W_c = S_c eps^-1 S_c - S_c S_c
            k_one_minus<<<grid_for(M4w * nw), 256, 0, st>>>(Xe.get(), N2w, nw);
            GB_LAUNCH_CHECK();
            for (int w = 0; w < nw; ++w)
                GB_CUDA(cudaMemcpyAsync(Ye.get() + w * M4w, Sce.get(), sizeof(double) * M4w, cudaMemcpyDeviceToDevice, st));
            k_gj_solve<<<nw, 256, gj_smem, st>>>(Xe.get(), Ye.get(), N2w, N2w, bad.get());
            GB_LAUNCH_CHECK();
            launch_dgemm(N2w, N2w, N2w, Sce.get(), N2w, 0, Ye.get(), N2w, M4w, We.get(), N2w, M4w, nw, 1.0, 0.0, st);
            launch_dgemm(nw, static_cast<int>(M4w), 1, d_ones.get(), 1, 0, ScSc.get(), M4w, 0, We.get(), M4w, 0, 1, 1.0, 1.0, st);
            const double *Wout = We.get();
            if (shrink)
            {
                // W_c of the large basis: U^H W_c U
                launch_dgemm(N2w, N2, N2w, We.get(), N2w, M4w, Ue.get(), N2, 0, Tsl.get(), N2,
                             static_cast<long long>(N2w) * N2, nw, 1.0, 0.0, st);
                launch_dgemm(N2, N2, N2w, UeT.get(), N2w, 0, Tsl.get(), N2, static_cast<long long>(N2w) * N2, Xl.get(), N2,
                             M4, nw, 1.0, 0.0, st);
                Wout = Xl.get();
            }
            k_unembed<<<grid_for(NN * nw), 256, 0, st>>>(Wout, Nc, nw, Wq.get() + static_cast<long long>(q) * nw * NN,
                                                         Wq.get() + (static_cast<long long>(nq) + q) * nw * NN);
            GB_LAUNCH_CHECK();
            GB_CUDA(cudaStreamSynchronize(st));  // the host matrices are rebuilt for the next q
        }
        int hbad = 0;
        bad.download(&hbad, 1, st);
        GB_CUDA(cudaStreamSynchronize(st));
        GB_REQUIRE(hbad == 0, "1 - S chi0 S is singular: no W_c");
    }
    // ---- W_c(R, omega) = sum_q [a_cq Re W_q + b_cq Im W_q], then W_c(R, tau) by costrans_f2t
    DevBuf<double> WR(static_cast<size_t>(nc) * nw * NN), Wt(static_cast<size_t>(nc) * nw * NN);
    {
        std::vector<double> coef(static_cast<size_t>(nc) * 2 * nq, 0.0);
        std::vector<int> q_of_rep(nk, -1);
        for (int q = 0; q < nq; ++q) q_of_rep[pt.ibz_rep[q]] = q;
        for (int k = 0; k < nk; ++k)
        {
            const int rep = ds.ibz_map[k], q = q_of_rep[rep];
            GB_REQUIRE(q >= 0, "k-point outside the IBZ list");
            const double sg = rep == k ? 1.0 : -1.0;
            for (int c = 0; c < nc; ++c)
            {
                const double th = k_dot_r(ds, k, gs.cells[c]);
                coef[static_cast<size_t>(c) * 2 * nq + q] += std::cos(th) / nk;
                coef[static_cast<size_t>(c) * 2 * nq + nq + q] += sg * std::sin(th) / nk;
            }
        }
        auto d_coef = to_dev(coef, st);
        launch_dgemm(nc, static_cast<int>(nw * NN), 2 * nq, d_coef.get(), 2 * nq, 0, Wq.get(), nw * NN, 0, WR.get(),
                     nw * NN, 0, 1, 1.0, 0.0, st);
        DevBuf<double> d_f2t(static_cast<size_t>(nw) * nw);
        d_f2t.upload(tf.cos_f2t.data(), static_cast<size_t>(nw) * nw, st);
        launch_dgemm(nw, static_cast<int>(NN), nw, d_f2t.get(), nw, 0, WR.get(), NN, nw * NN, Wt.get(), NN, nw * NN, nc,
                     1.0, 0.0, st);
        GB_CUDA(cudaStreamSynchronize(st));
    }
    Wq.release();
    WR.release();
    // LibRI's set_Ws filter on every W(R, tau) block (libri_g0w0_threshold_Wc; gw.cpp:459-470)
    auto d_abo_f = to_dev(gs.abf_off, st);
    auto d_aoo_f = to_dev(gs.ao_off, st);
    block_filter_dev(Wt.get(), static_cast<long long>(nw) * NN, nc, NN, nw, Nc, d_abo_f.get(), n_at,
                     opts.libri_g0w0_threshold_Wc, st);

    // ---- Sigma_c(R, i omega) per spin from the supercell closed form at every tau, then the KS
    // diagonal at every k
    const int nao = naoc;
    const long long naos = gs.nao, ns2 = naos * naos, nnc = static_cast<long long>(nao) * nao;
    auto d_ekb = to_dev(ds.ekb, st);
    auto d_wg = to_dev(ds.wg, st);
    DevBuf<cuDoubleComplex> d_psi(ds.wfc.size());
    d_psi.upload(reinterpret_cast<const cuDoubleComplex *>(ds.wfc.data()), ds.wfc.size(), st);
    auto d_gcos = to_dev(pt.gcos, st);
    auto d_gsin = to_dev(pt.gsin, st);
    auto d_cdiff = to_dev(gs.cdiff, st);
    DevBuf<double> d_s(2ull * nk * nb), d_G(2ull * nc * nnc), Ws(static_cast<size_t>(gs.N) * gs.N), Gps(ns2), Gms(ns2),
        Sp(ns2), Sm(ns2), cw(nw), sw(nw);
    DevBuf<cuDoubleComplex> d_A(2ull * nk * nnc), Sig(static_cast<size_t>(nw) * nc * nnc);
    SigmaClosedForm cf(ds, gs);
    ds.sigc_ks.assign(ns, {});
    ds.sigc_r.assign(ns, {});
    std::vector<cplx> hsig(static_cast<size_t>(nw) * nc * nnc);
    for (int sp = 0; sp < ns; ++sp)
    {
        Sig.zero(st);
        for (int it = 0; it < nw; ++it)
        {
            launch_tau_scale(d_ekb.get() + static_cast<size_t>(sp) * nk * nb, d_wg.get() + static_cast<size_t>(sp) * nk * nb,
                             nk, nb, ds.efermi, tf.tau[it], ns, opts.n_bands_chi0, d_s.get(), st);
            launch_gk_build(d_psi.get() + static_cast<size_t>(sp) * nk * nb * nao, d_s.get(), nk, nb, nao, d_A.get(), st);
            launch_phase_sum(d_A.get(), d_gcos.get(), d_gsin.get(), nk, nc, nao, d_G.get(), st);
            // LibRI's set_Gs filter on G(R, +-tau) (libri_g0w0_threshold_G; gw.cpp:546-616)
            block_filter_dev(d_G.get(), nnc, 2 * nc, 0, 1, nao, d_aoo_f.get(), n_at, opts.libri_g0w0_threshold_G, st);
            k_to_super<<<grid_for(ns2), 256, 0, st>>>(d_G.get(), nnc, nao, nc, d_cdiff.get(), Gps.get());
            k_to_super<<<grid_for(ns2), 256, 0, st>>>(d_G.get() + nc * nnc, nnc, nao, nc, d_cdiff.get(), Gms.get());
            k_to_super<<<grid_for(static_cast<long long>(gs.N) * gs.N), 256, 0, st>>>(
                Wt.get() + static_cast<long long>(it) * NN, nw * NN, Nc, nc, d_cdiff.get(), Ws.get());
            GB_LAUNCH_CHECK();
            const double *Dp[2] = {Gps.get(), Gms.get()};
            double *Hp[2] = {Sp.get(), Sm.get()};
            cf.run(gs, Ws.get(), Dp, 2, Hp, st);
            std::vector<double> c(nw), sn(nw);
            for (int w = 0; w < nw; ++w)
            {
                c[w] = tf.cos_t2f[static_cast<size_t>(w) * nw + it];
                sn[w] = tf.sin_t2f[static_cast<size_t>(w) * nw + it];
            }
            cw.upload(c.data(), nw, st);
            sw.upload(sn.data(), nw, st);
            k_sigma_rows<<<grid_for(nnc * nc * nw), 256, 0, st>>>(Sp.get(), Sm.get(), gs.c0, nc, nao, cw.get(), sw.get(),
                                                                  nw, Sig.get());
            GB_LAUNCH_CHECK();
            GB_CUDA(cudaStreamSynchronize(st));  // the host weight vectors are reused
        }
        Sig.download(reinterpret_cast<cuDoubleComplex *>(hsig.data()), hsig.size(), st);
        GB_CUDA(cudaStreamSynchronize(st));
        ds.sigc_r[sp] = hsig;
        // Sigma_c(k, i omega) = sum_c e^{i 2 pi k.R_c} Sigma_c(R_c, i omega); <psi_kn|.|psi_kn>
        std::vector<cplx> &out = ds.sigc_ks[sp];
        out.assign(static_cast<size_t>(nk) * nb * nw, cplx(0, 0));
        std::vector<cplx> Sk(nnc);
        for (int k = 0; k < nk; ++k)
            for (int w = 0; w < nw; ++w)
            {
                std::fill(Sk.begin(), Sk.end(), cplx(0, 0));
                for (int c = 0; c < nc; ++c)
                {
                    const cplx ph = std::polar(1.0, k_dot_r(ds, k, gs.cells[c]));
                    const cplx *src = hsig.data() + (static_cast<size_t>(w) * nc + c) * nnc;
                    for (long long e = 0; e < nnc; ++e) Sk[e] += ph * src[e];
                }
                for (int n = 0; n < nb; ++n)
                {
                    const cplx *v = ds.wfc.data() + ((static_cast<size_t>(sp) * nk + k) * nb + n) * nao;
                    cplx acc(0, 0);
                    for (int p = 0; p < nao; ++p)
                    {
                        cplx t(0, 0);
                        for (int q2 = 0; q2 < nao; ++q2) t += Sk[static_cast<size_t>(p) * nao + q2] * v[q2];
                        acc += std::conj(v[p]) * t;
                    }
                    out[(static_cast<size_t>(k) * nb + n) * nw + w] = acc;
                }
            }
    }
    ds.hx_cells = gs.cells;
    ds.gw_omega = tf.omega;
    ds.g0w0_generation = ds.generation;
    release_kept(ds);
}

namespace {
// The image of cell c that the block (I, J, R_c) takes at band k-points: R_c + n period with n in
// {-1, 0, 1}^3, the one nearest to x_I - x_J (Exx::build_KS_band, exx.cpp:683-725; applied when
// the atom positions are set).  table[(I n_at + J) nc + c].
std::vector<std::array<int, 3>> band_images(const Dataset &ds, int n_at, const std::vector<std::array<int, 3>> &cells)
{
    const int nc = static_cast<int>(cells.size());
    std::vector<std::array<int, 3>> img(static_cast<size_t>(n_at) * n_at * nc);
    const bool shift = static_cast<int>(ds.positions.size()) == 3 * n_at;
    // fractional positions: x_cart = frac . latvec (rows a1, a2, a3)
    std::vector<double> frac(3 * static_cast<size_t>(n_at), 0.0);
    if (shift)
    {
        const double *L = ds.latvec;
        const double det = L[0] * (L[4] * L[8] - L[5] * L[7]) - L[1] * (L[3] * L[8] - L[5] * L[6]) +
                           L[2] * (L[3] * L[7] - L[4] * L[6]);
        GB_REQUIRE(std::fabs(det) > 0.0, "singular lattice vectors");
        const double inv[9] = {(L[4] * L[8] - L[5] * L[7]) / det, (L[2] * L[7] - L[1] * L[8]) / det,
                               (L[1] * L[5] - L[2] * L[4]) / det, (L[5] * L[6] - L[3] * L[8]) / det,
                               (L[0] * L[8] - L[2] * L[6]) / det, (L[2] * L[3] - L[0] * L[5]) / det,
                               (L[3] * L[7] - L[4] * L[6]) / det, (L[1] * L[6] - L[0] * L[7]) / det,
                               (L[0] * L[4] - L[1] * L[3]) / det};
        for (int a = 0; a < n_at; ++a)
            for (int d = 0; d < 3; ++d)
                for (int e = 0; e < 3; ++e) frac[3 * a + d] += ds.positions[3 * a + e] * inv[3 * e + d];
    }
    for (int I = 0; I < n_at; ++I)
        for (int J = 0; J < n_at; ++J)
            for (int c = 0; c < nc; ++c)
            {
                std::array<int, 3> best = cells[c];
                if (shift)
                {
                    double bn = 1e300;
                    for (int i = -1; i <= 1; ++i)
                        for (int j = -1; j <= 1; ++j)
                            for (int k = -1; k <= 1; ++k)
                            {
                                const int R[3] = {cells[c][0] + i * ds.period[0], cells[c][1] + j * ds.period[1],
                                                  cells[c][2] + k * ds.period[2]};
                                double dv[3];
                                for (int e = 0; e < 3; ++e)
                                {
                                    dv[e] = 0.0;
                                    for (int d = 0; d < 3; ++d)
                                        dv[e] += (frac[3 * I + d] - frac[3 * J + d] - R[d]) * ds.latvec[3 * d + e];
                                }
                                const double n2 = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
                                if (n2 < bn)
                                {
                                    bn = n2;
                                    best = {R[0], R[1], R[2]};
                                }
                            }
                }
                img[(static_cast<size_t>(I) * n_at + J) * nc + c] = best;
            }
    return img;
}

// <psi| sum_c e^{i 2 pi k.R'} X(R_c) |psi> over the cell blocks X [cell][n_ao][n_ao], R' the band
// image of each atom-pair block
template <typename T>
cplx band_element(const Dataset &ds, const T *X, const std::vector<std::array<int, 3>> &img, const double *kb,
                  const cplx *psi)
{
    const int nao = ds.n_ao, n_at = ds.n_atoms(), nc = static_cast<int>(ds.hx_cells.size());
    std::vector<int> atom(nao);
    for (int a = 0, o = 0; a < n_at; ++a)
        for (int i = 0; i < ds.nao_at[a]; ++i) atom[o++] = a;
    cplx acc(0, 0);
    for (int c = 0; c < nc; ++c)
    {
        const T *Xc = X + static_cast<size_t>(c) * nao * nao;
        for (int p = 0; p < nao; ++p)
        {
            cplx row(0, 0);
            for (int q = 0; q < nao; ++q)
            {
                const std::array<int, 3> &R = img[(static_cast<size_t>(atom[p]) * n_at + atom[q]) * nc + c];
                const double th = 2.0 * M_PI * (kb[0] * R[0] + kb[1] * R[1] + kb[2] * R[2]);
                row += std::polar(1.0, th) * cplx(Xc[static_cast<size_t>(p) * nao + q]) * psi[q];
            }
            acc += std::conj(psi[p]) * row;
        }
    }
    return acc;
}

const cplx *band_psi(const Dataset &ds, int s, int kb, int n)
{
    GB_REQUIRE(ds.band_nk > 0 && static_cast<int>(ds.band_kfrac.size()) == 3 * ds.band_nk,
               "band data not set: librpa_set_band_kvec and librpa_set_band_occ_eigval with the same count");
    GB_REQUIRE(s >= 0 && s < ds.band_ns && kb >= 0 && kb < ds.band_nk && n >= 0 && n < ds.band_nst,
               "band state index out of range");
    return ds.band_wfc.data() + ((static_cast<size_t>(s) * ds.band_nk + kb) * ds.band_nst + n) * ds.n_ao;
}
} // namespace

double exx_band_state(const Dataset &ds, int s, int kb, int n)
{
    GB_REQUIRE(s < static_cast<int>(ds.hx_r.size()), "no exchange matrix: build the exchange first");
    const auto img = band_images(ds, ds.n_atoms(), ds.hx_cells);
    return -band_element(ds, ds.hx_r[s].data(), img, ds.band_kfrac.data() + 3 * kb, band_psi(ds, s, kb, n)).real();
}

std::vector<cplx> sigc_band_iw(const Dataset &ds, int s, int kb, int n)
{
    GB_REQUIRE(s < static_cast<int>(ds.sigc_r.size()), "no self-energy: build G0W0 first");
    const int nw = static_cast<int>(ds.gw_omega.size()), nao = ds.n_ao, nc = static_cast<int>(ds.hx_cells.size());
    const auto img = band_images(ds, ds.n_atoms(), ds.hx_cells);
    const cplx *psi = band_psi(ds, s, kb, n);
    std::vector<cplx> out(nw);
    for (int w = 0; w < nw; ++w)
        out[w] = band_element(ds, ds.sigc_r[s].data() + static_cast<size_t>(w) * nc * nao * nao, img,
                              ds.band_kfrac.data() + 3 * kb, psi);
    return out;
}

void build_g0w0(Dataset &ds, const LibrpaOptions &opts, const TimeFreqGrids &tf)
{
    // the head of the dielectric matrix is replaced at q = 0 whenever a dielectric function is
    // set (compute_g0w0.cpp:103-107, epsilon.cpp:2110-2160), Gamma-only inputs included: the
    // k-grid chain (complex W, one q-point) carries it, and the ABF shrink
    const bool head = opts.replace_w_head == LIBRPA_SWITCH_ON && !ds.dielect_eps.empty();
    if (ds.n_kpts > 1 || head || opts.use_shrink_abfs == LIBRPA_SWITCH_ON)
        build_g0w0_kgrid(ds, opts, tf);
    else
        build_g0w0_gamma(ds, opts, tf);
}

} // namespace gb
