// FP64 SIMT GEMMs (real and complex, row-major, batched by blockIdx.z).
//
// These serve the plain FP64 GPU path and the small complex products of the
// G builder and E_c; on GB300 the FP64 pipe (~1.2 TFLOP/s) is the limit, so a
// register-blocked 64x64 tile already sits on the FP64 roofline.
#include "kernels.h"
#include "common.h"

#include <algorithm>

namespace gb {

namespace {

constexpr int BM = 64, BN = 64, BK = 16;

template <typename T>
__global__ void __launch_bounds__(256) k_gemm_real(int M, int N, int K, const T *__restrict__ A, long long lda,
                                                   long long sA, const T *__restrict__ B, long long ldb,
                                                   long long sB, T *__restrict__ C, long long ldc, long long sC,
                                                   T alpha, T beta)
{
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN];
    const int bz = blockIdx.z;
    A += bz * sA;
    B += bz * sB;
    C += bz * sC;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    T acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += BK)
    {
        for (int t = threadIdx.x; t < BM * BK; t += 256)
        {
            const int r = t / BK, kk = t % BK;
            const int gm = m0 + r, gk = k0 + kk;
            As[kk][r] = (gm < M && gk < K) ? A[gm * lda + gk] : T(0);
        }
        for (int t = threadIdx.x; t < BK * BN; t += 256)
        {
            const int kk = t / BN, c = t % BN;
            const int gk = k0 + kk, gn = n0 + c;
            Bs[kk][c] = (gk < K && gn < N) ? B[gk * ldb + gn] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk)
        {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            const int gm = m0 + ty + 16 * i, gn = n0 + tx + 16 * j;
            if (gm < M && gn < N)
            {
                T v = alpha * acc[i][j];
                if (beta != T(0)) v += beta * C[gm * ldc + gn];
                C[gm * ldc + gn] = v;
            }
        }
}

constexpr int ZB = 32, ZK = 16;

__global__ void __launch_bounds__(256) k_zgemm(int M, int N, int K, const cuDoubleComplex *__restrict__ A,
                                               long long lda, long long sA, const cuDoubleComplex *__restrict__ B,
                                               long long ldb, long long sB, cuDoubleComplex *__restrict__ C,
                                               long long ldc, long long sC)
{
    __shared__ cuDoubleComplex As[ZK][ZB + 1];
    __shared__ cuDoubleComplex Bs[ZK][ZB];
    const int bz = blockIdx.z;
    A += bz * sA;
    B += bz * sB;
    C += bz * sC;
    const int m0 = blockIdx.y * ZB, n0 = blockIdx.x * ZB;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    cuDoubleComplex acc[2][2];
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) acc[i][j] = make_cuDoubleComplex(0, 0);
    for (int k0 = 0; k0 < K; k0 += ZK)
    {
        for (int t = threadIdx.x; t < ZB * ZK; t += 256)
        {
            const int r = t / ZK, kk = t % ZK;
            const int gm = m0 + r, gk = k0 + kk;
            As[kk][r] = (gm < M && gk < K) ? A[gm * lda + gk] : make_cuDoubleComplex(0, 0);
        }
        for (int t = threadIdx.x; t < ZK * ZB; t += 256)
        {
            const int kk = t / ZB, c = t % ZB;
            const int gk = k0 + kk, gn = n0 + c;
            Bs[kk][c] = (gk < K && gn < N) ? B[gk * ldb + gn] : make_cuDoubleComplex(0, 0);
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < ZK; ++kk)
        {
            const cuDoubleComplex a0 = As[kk][ty], a1 = As[kk][ty + 16];
            const cuDoubleComplex b0 = Bs[kk][tx], b1 = Bs[kk][tx + 16];
            acc[0][0] = cuCfma(a0, b0, acc[0][0]);
            acc[0][1] = cuCfma(a0, b1, acc[0][1]);
            acc[1][0] = cuCfma(a1, b0, acc[1][0]);
            acc[1][1] = cuCfma(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
        {
            const int gm = m0 + ty + 16 * i, gn = n0 + tx + 16 * j;
            if (gm < M && gn < N) C[gm * ldc + gn] = acc[i][j];
        }
}

} // namespace

void launch_dgemm(int M, int N, int K, const double *A, long long lda, long long sA, const double *B,
                  long long ldb, long long sB, double *C, long long ldc, long long sC, int batch,
                  double alpha, double beta, cudaStream_t st)
{
    if (M <= 0 || N <= 0 || batch <= 0) return;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
    k_gemm_real<double><<<grid, 256, 0, st>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC, alpha, beta);
    GB_LAUNCH_CHECK();
}

void launch_sgemm(int M, int N, int K, const float *A, long long lda, long long sA, const float *B,
                  long long ldb, long long sB, float *C, long long ldc, long long sC, int batch,
                  cudaStream_t st)
{
    if (M <= 0 || N <= 0 || batch <= 0) return;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
    k_gemm_real<float><<<grid, 256, 0, st>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC, 1.0f, 0.0f);
    GB_LAUNCH_CHECK();
}

namespace {
__global__ void k_d2f(const double *__restrict__ in, float *__restrict__ out, long long n)
{
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        out[i] = static_cast<float>(in[i]);
}
} // namespace

void launch_d2f(const double *in, float *out, long long n, cudaStream_t st)
{
    if (n <= 0) return;
    const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
    k_d2f<<<static_cast<unsigned>(blocks), 256, 0, st>>>(in, out, n);
    GB_LAUNCH_CHECK();
}

void launch_zgemm(int M, int N, int K, const cuDoubleComplex *A, long long lda, long long sA,
                  const cuDoubleComplex *B, long long ldb, long long sB, cuDoubleComplex *C, long long ldc,
                  long long sC, int batch, cudaStream_t st)
{
    if (M <= 0 || N <= 0 || batch <= 0) return;
    dim3 grid((N + ZB - 1) / ZB, (M + ZB - 1) / ZB, batch);
    k_zgemm<<<grid, 256, 0, st>>>(M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC);
    GB_LAUNCH_CHECK();
}

} // namespace gb
