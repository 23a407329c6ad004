// Batched blocked Cholesky factorisation in FP64 (real symmetric or complex Hermitian).
//
// Right-looking, panel width NB = 32, three launches per panel step for the whole batch:
//   k_chol_diag  : one CTA per matrix factors the NB x NB diagonal block in shared memory;
//   k_chol_panel : each CTA solves a 64-row slab of the panel below it, X L11^H = A21;
//   k_chol_update: lower-triangle trailing update A22 -= L21 L21^H in 32 x 32 tiles.
// The real variant chol_batched_r_ozaki uses panels of 64 and does the trailing update on the
// tensor cores with exact integer slices (k_chol_ozaki.cu).
// The diagonal of L is written to diag[b][i]; ln det A = 2 sum_i log L_ii (k_chol_logdet).
// On GB300 the FP64 pipe (~1 TFLOP/s) bounds these kernels; the blocking keeps them off
// the HBM roofline (each trailing element is read and written once per 32 columns).
#include <cuComplex.h>

#include "chol.h"
#include "common.h"

namespace gb {

namespace {

constexpr int NB = 32;

__device__ inline double cre(double x) { return x; }
__device__ inline double cre(cuDoubleComplex x) { return x.x; }
__device__ inline double cconjmul_acc(double acc, double a, double b) { return fma(a, b, acc); }
__device__ inline cuDoubleComplex cconjmul_acc(cuDoubleComplex acc, cuDoubleComplex a, cuDoubleComplex b)
{
    // acc + a * conj(b)
    return make_cuDoubleComplex(acc.x + a.x * b.x + a.y * b.y, acc.y + a.y * b.x - a.x * b.y);
}
__device__ inline double csub(double a, double b) { return a - b; }
__device__ inline cuDoubleComplex csub(cuDoubleComplex a, cuDoubleComplex b) { return cuCsub(a, b); }
__device__ inline double cscale(double a, double s) { return a * s; }
__device__ inline cuDoubleComplex cscale(cuDoubleComplex a, double s) { return make_cuDoubleComplex(a.x * s, a.y * s); }
template <typename T>
__device__ inline T czero();
template <>
__device__ inline double czero<double>() { return 0.0; }
template <>
__device__ inline cuDoubleComplex czero<cuDoubleComplex>() { return make_cuDoubleComplex(0.0, 0.0); }
__device__ inline double cfromreal(double x, double) { return x; }
__device__ inline cuDoubleComplex cfromreal(double x, cuDoubleComplex) { return make_cuDoubleComplex(x, 0.0); }

// Factor the nb x nb diagonal block at k0 into shared memory D (lower triangle).
template <typename T, int NBT>
__device__ void factor_diag(const T *A, int N, int k0, int nb, T (*D)[NBT + 1], int *bad)
{
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x)
    {
        const int i = t / nb, j = t % nb;
        D[i][j] = j <= i ? A[static_cast<long long>(k0 + i) * N + k0 + j] : czero<T>();
    }
    __syncthreads();
    __shared__ double sinv;  // reciprocal of the current pivot, formed once per step
    for (int p = 0; p < nb; ++p)
    {
        if (threadIdx.x == 0)
        {
            const double d2 = cre(D[p][p]);
            if (!(d2 > 0.0)) *bad = 1;
            const double l = sqrt(fmax(d2, 1e-300));
            D[p][p] = cfromreal(l, D[p][p]);
            sinv = 1.0 / l;
        }
        __syncthreads();
        const double inv = sinv;
        for (int i = p + 1 + threadIdx.x; i < nb; i += blockDim.x) D[i][p] = cscale(D[i][p], inv);
        __syncthreads();
        const int m = nb - p - 1;
        for (int t = threadIdx.x; t < m * m; t += blockDim.x)
        {
            const int i = p + 1 + t / m, j = p + 1 + t % m;
            if (j <= i) D[i][j] = csub(D[i][j], cconjmul_acc(czero<T>(), D[i][p], D[j][p]));
        }
        __syncthreads();
    }
}

// Factor the diagonal block in place (one CTA per matrix) and record the diagonal of L.
template <typename T, int NBT>
__global__ void __launch_bounds__(256) k_chol_diag(T *__restrict__ Aall, int N, int k0, double *__restrict__ diag,
                                                  int *__restrict__ bad)
{
    __shared__ T D[NBT][NBT + 1];
    const int b = blockIdx.x;
    T *A = Aall + static_cast<long long>(b) * N * N;
    const int nb = min(NBT, N - k0);
    factor_diag<T, NBT>(A, N, k0, nb, D, bad + b);
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x)
    {
        const int i = t / nb, j = t % nb;
        if (j <= i) A[static_cast<long long>(k0 + i) * N + k0 + j] = D[i][j];
    }
    for (int i = threadIdx.x; i < nb; i += blockDim.x) diag[static_cast<long long>(b) * N + k0 + i] = cre(D[i][i]);
}

// Real diagonal block for the tensor-core panel solve: factor L11 as k_chol_diag does and also
// form W = L11^-1 (lower triangular, FP64) into Wb[b][64][64], so that the panel becomes the
// product L21 = A21 W^T.  Thread c (< nb) builds column c of W by forward substitution,
// W_cc = 1 / L_cc, W_ic = -(sum_{k=c}^{i-1} L_ik W_kc) / L_ii.  Dynamic shared memory: D, W.
constexpr int DINV_SMEM = 2 * OZAKI_NB * (OZAKI_NB + 1) * static_cast<int>(sizeof(double));
__global__ void __launch_bounds__(256) k_chol_diag_inv(double *__restrict__ Aall, int N, int k0,
                                                      double *__restrict__ diag, int *__restrict__ bad,
                                                      double *__restrict__ Wb)
{
    constexpr int NBT = OZAKI_NB;
    extern __shared__ double dsm[];
    double (*D)[NBT + 1] = reinterpret_cast<double (*)[NBT + 1]>(dsm);
    double (*W)[NBT + 1] = reinterpret_cast<double (*)[NBT + 1]>(dsm + NBT * (NBT + 1));
    const int b = blockIdx.x;
    double *A = Aall + static_cast<long long>(b) * N * N;
    const int nb = min(NBT, N - k0);
    factor_diag<double, NBT>(A, N, k0, nb, D, bad + b);
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x)
    {
        const int i = t / nb, j = t % nb;
        if (j <= i) A[static_cast<long long>(k0 + i) * N + k0 + j] = D[i][j];
    }
    for (int i = threadIdx.x; i < nb; i += blockDim.x) diag[static_cast<long long>(b) * N + k0 + i] = D[i][i];
    __shared__ double invd[NBT];
    for (int i = threadIdx.x; i < nb; i += blockDim.x) invd[i] = 1.0 / D[i][i];
    __syncthreads();
    const int c = threadIdx.x;
    if (c < nb)
    {
        W[c][c] = invd[c];
        for (int i = c + 1; i < nb; ++i)
        {
            double s0 = 0.0, s1 = 0.0;  // two chains for the dependent FMA latency
            int k = c;
            for (; k + 1 < i; k += 2)
            {
                s0 = fma(D[i][k], W[k][c], s0);
                s1 = fma(D[i][k + 1], W[k + 1][c], s1);
            }
            if (k < i) s0 = fma(D[i][k], W[k][c], s0);
            W[i][c] = -(s0 + s1) * invd[i];
        }
    }
    __syncthreads();
    double *Wo = Wb + static_cast<long long>(b) * NBT * NBT;
    for (int t = threadIdx.x; t < NBT * NBT; t += blockDim.x)
    {
        const int i = t / NBT, j = t % NBT;
        Wo[t] = (i < nb && j <= i) ? W[i][j] : 0.0;
    }
}

// Panel solve X L11^H = A21 for a 64-row slab per CTA (L11 already factored in A).  Full
// panels run right-looking with the row in registers (x[p] /= L_pp, then x[q] -= x[p] conj L_qp
// for every q > p: independent updates instead of one serial sum per p) and the reciprocal
// diagonal precomputed once per CTA.
template <typename T, int NBT>
__global__ void __launch_bounds__(64) k_chol_panel(T *__restrict__ Aall, int N, int k0)
{
    __shared__ T D[NBT][NBT + 1];
    __shared__ double invd[NBT];
    const int b = blockIdx.y;
    T *A = Aall + static_cast<long long>(b) * N * N;
    const int nb = min(NBT, N - k0);
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x)
    {
        const int i = t / nb, j = t % nb;
        D[i][j] = j <= i ? A[static_cast<long long>(k0 + i) * N + k0 + j] : czero<T>();
    }
    __syncthreads();
    for (int p = threadIdx.x; p < nb; p += blockDim.x) invd[p] = 1.0 / cre(D[p][p]);
    __syncthreads();
    const int r = k0 + nb + blockIdx.x * 64 + threadIdx.x;
    if (r >= N) return;
    T *row = A + static_cast<long long>(r) * N + k0;
    if (nb == NBT)
    {
        T x[NBT];
#pragma unroll
        for (int p = 0; p < NBT; ++p) x[p] = row[p];
#pragma unroll
        for (int p = 0; p < NBT; ++p)
        {
            x[p] = cscale(x[p], invd[p]);
#pragma unroll
            for (int q = p + 1; q < NBT; ++q) x[q] = csub(x[q], cconjmul_acc(czero<T>(), x[p], D[q][p]));
        }
#pragma unroll
        for (int p = 0; p < NBT; ++p) row[p] = x[p];
        return;
    }
    T x[NBT];
    for (int p = 0; p < nb; ++p) x[p] = row[p];
    for (int p = 0; p < nb; ++p)
    {
        T s = x[p];
        for (int q = 0; q < p; ++q) s = csub(s, cconjmul_acc(czero<T>(), x[q], D[p][q]));
        x[p] = cscale(s, invd[p]);
    }
    for (int p = 0; p < nb; ++p) row[p] = x[p];
}

// Trailing update of the lower triangle, 32 x 32 tiles (ti >= tj), K = panel width.
template <typename T>
__global__ void __launch_bounds__(256) k_chol_update(T *__restrict__ Aall, int N, int k0, int ntile)
{
    __shared__ T Pi[32][NB + 1];
    __shared__ T Pj[32][NB + 1];
    const int b = blockIdx.y;
    T *A = Aall + static_cast<long long>(b) * N * N;
    const int nb = min(NB, N - k0);
    const int s0 = k0 + nb;
    // blockIdx.x enumerates lower-triangular tile pairs (ti >= tj)
    int t = blockIdx.x, ti = 0;
    while (t > ti)
    {
        t -= ti + 1;
        ++ti;
    }
    const int tj = t;
    if (ti >= ntile) return;
    const int i0 = s0 + ti * 32, j0 = s0 + tj * 32;
    for (int e = threadIdx.x; e < 32 * nb; e += blockDim.x)
    {
        const int r = e / nb, p = e % nb;
        Pi[r][p] = (i0 + r < N) ? A[static_cast<long long>(i0 + r) * N + k0 + p] : czero<T>();
        Pj[r][p] = (j0 + r < N) ? A[static_cast<long long>(j0 + r) * N + k0 + p] : czero<T>();
    }
    __syncthreads();
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 2 x 2 outputs per thread
    T acc[2][2];
    for (int u = 0; u < 2; ++u)
        for (int v = 0; v < 2; ++v) acc[u][v] = czero<T>();
    for (int p = 0; p < nb; ++p)
        for (int u = 0; u < 2; ++u)
            for (int v = 0; v < 2; ++v) acc[u][v] = cconjmul_acc(acc[u][v], Pi[ty + 16 * u][p], Pj[tx + 16 * v][p]);
    for (int u = 0; u < 2; ++u)
        for (int v = 0; v < 2; ++v)
        {
            const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
            if (i < N && j < N && j <= i)
            {
                T &a = A[static_cast<long long>(i) * N + j];
                a = csub(a, acc[u][v]);
            }
        }
}

__global__ void k_chol_logdet(const double *__restrict__ diag, int N, double *__restrict__ logdet)
{
    __shared__ double red[256];
    const double *d = diag + static_cast<long long>(blockIdx.x) * N;
    double acc = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) acc += log(d[i]);
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1)
    {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) logdet[blockIdx.x] = 2.0 * red[0];
}

// zero the strict upper triangle (L as a full matrix)
template <typename T>
__global__ void k_zero_upper(T *__restrict__ Aall, int N)
{
    T *A = Aall + static_cast<long long>(blockIdx.y) * N * N;
    const long long nn = static_cast<long long>(N) * N;
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < nn;
         e += static_cast<long long>(gridDim.x) * blockDim.x)
        if (e % N > e / N) A[e] = czero<T>();
}

template <typename T>
int chol_impl(T *A, int N, int batch, double *diag, int *bad, cudaStream_t st)
{
    int launches = 0;
    for (int k0 = 0; k0 < N; k0 += NB)
    {
        const int nb = std::min(NB, N - k0);
        const int rows_below = N - k0 - nb;
        k_chol_diag<T, NB><<<batch, 256, 0, st>>>(A, N, k0, diag, bad);
        GB_LAUNCH_CHECK();
        ++launches;
        if (rows_below > 0)
        {
            dim3 gp((rows_below + 63) / 64, batch);
            k_chol_panel<T, NB><<<gp, 64, 0, st>>>(A, N, k0);
            GB_LAUNCH_CHECK();
            const int ntile = (rows_below + 31) / 32;
            dim3 gu(ntile * (ntile + 1) / 2, batch);
            k_chol_update<T><<<gu, 256, 0, st>>>(A, N, k0, ntile);
            GB_LAUNCH_CHECK();
            launches += 2;
        }
    }
    return launches;
}

} // namespace

int chol_batched_c(cuDoubleComplex *A, int N, int batch, double *diag, int *bad, cudaStream_t st)
{
    return chol_impl(A, N, batch, diag, bad, st);
}

int chol_batched_r(double *A, int N, int batch, double *diag, int *bad, cudaStream_t st)
{
    return chol_impl(A, N, batch, diag, bad, st);
}

int chol_batched_r_ozaki(double *A, int N, int batch, double *diag, int *bad, OzakiWork &w, cudaStream_t st)
{
    constexpr int NBO = OZAKI_NB;
    static PerDeviceOnce attr;
    attr.run([] {
        GB_CUDA(cudaFuncSetAttribute(k_chol_diag_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, DINV_SMEM));
    });
    int launches = 0;
    for (int k0 = 0; k0 < N; k0 += NBO)
    {
        const int nb = std::min(NBO, N - k0);
        const int rows_below = N - k0 - nb;
        if (rows_below == 0)
        {
            k_chol_diag<double, NBO><<<batch, 256, 0, st>>>(A, N, k0, diag, bad);
            GB_LAUNCH_CHECK();
            ++launches;
            continue;
        }
        // every panel with rows below it is a full 64-wide one (panels step by 64)
        k_chol_diag_inv<<<batch, 256, DINV_SMEM, st>>>(A, N, k0, diag, bad, w.winv);
        GB_LAUNCH_CHECK();
        launches += 1 + ozaki_panel_solve(A, N, batch, k0, w, st);
        launches += ozaki_trailing_update(A, N, batch, k0 + nb, k0, nb, w, st);
    }
    return launches;
}

void chol_logdet(const double *diag, int N, int batch, double *logdet, cudaStream_t st)
{
    k_chol_logdet<<<batch, 256, 0, st>>>(diag, N, logdet);
    GB_LAUNCH_CHECK();
}

void zero_upper_c(cuDoubleComplex *A, int N, int batch, cudaStream_t st)
{
    dim3 g(std::min(1024, (N * N + 255) / 256), batch);
    k_zero_upper<cuDoubleComplex><<<g, 256, 0, st>>>(A, N);
    GB_LAUNCH_CHECK();
}

void zero_upper_r(double *A, int N, int batch, cudaStream_t st)
{
    dim3 g(std::min(1024, (N * N + 255) / 256), batch);
    k_zero_upper<double><<<g, 256, 0, st>>>(A, N);
    GB_LAUNCH_CHECK();
}

} // namespace gb
