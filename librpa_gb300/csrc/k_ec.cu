// E_c stage kernels: full-matrix assembly from upper atom blocks, trace and
// I - Pi, and an FP64 LU with partial pivoting returning sum log(+-u_ii).
//
// Follows LibRPA's E_c (src/core/epsilon.cpp:270-558 for k points, :43-268 for
// Gamma only): lower blocks are conj-transposes of the upper ones
// (utils_matrix_m_mpi.h:393-455), Pi = V chi0, tr Pi, M = I - Pi, LU, and
// ln det = sum_i log(u_ii) if Re u_ii > 0 else log(-u_ii) (epsilon.cpp:578-592, :640-671).
// Pivot choice follows LAPACK's i*amax: largest |Re|+|Im| (|x| for real), first index on ties.
#include <algorithm>

#include "kernels.h"
#include "common.h"

namespace gb {

namespace {

__device__ inline double mag1(double x) { return fabs(x); }
__device__ inline double mag1(cuDoubleComplex x) { return fabs(x.x) + fabs(x.y); }

// out[s][r][c]; row r in atom A (local a), col c in atom B (local b)
__global__ void k_assemble_chi0(const cuDoubleComplex *__restrict__ src, long long slab_stride, int N,
                                const int *__restrict__ atom_of, const int *__restrict__ abf_off,
                                const int *__restrict__ nabf, const int *__restrict__ pair_of, int n_at,
                                const long long *__restrict__ e_off, bool real_only,
                                cuDoubleComplex *__restrict__ outc, double *__restrict__ outr,
                                long long out_stride)
{
    const long long nn = static_cast<long long>(N) * N;
    const int s = blockIdx.y;
    for (long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; idx < nn;
         idx += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const int r = static_cast<int>(idx / N), c = static_cast<int>(idx % N);
        const int A = atom_of[r], B = atom_of[c];
        const int a = r - abf_off[A], b = c - abf_off[B];
        const cuDoubleComplex *sl = src + s * slab_stride;
        cuDoubleComplex v;
        if (A <= B)
        {
            const int p = pair_of[A * n_at + B];
            v = sl[e_off[p] + static_cast<long long>(a) * nabf[B] + b];
        }
        else
        {
            const int p = pair_of[B * n_at + A];
            v = sl[e_off[p] + static_cast<long long>(b) * nabf[A] + a];
            v.y = -v.y;
        }
        if (real_only)
            outr[s * out_stride + idx] = v.x;
        else
            outc[s * out_stride + idx] = v;
    }
}

// blk_IJ[2b] = (I, J) with I <= J; block b is nabf[I] x nabf[J] at blob[blk_off[b]]
__global__ void k_assemble_v(const cuDoubleComplex *__restrict__ blob, const long long *__restrict__ blk_off,
                             const int *__restrict__ blk_IJ, const int *__restrict__ abf_off,
                             const int *__restrict__ nabf, int N, bool real_only,
                             cuDoubleComplex *__restrict__ outc, double *__restrict__ outr)
{
    const int b = blockIdx.x;
    const int I = blk_IJ[2 * b], J = blk_IJ[2 * b + 1];
    const int nI = nabf[I], nJ = nabf[J];
    const cuDoubleComplex *src = blob + blk_off[b];
    for (int t = threadIdx.x; t < nI * nJ; t += blockDim.x)
    {
        const int mu = t / nJ, nu = t % nJ;
        const long long r = abf_off[I] + mu, c = abf_off[J] + nu;
        const cuDoubleComplex v = src[t];
        if (real_only)
        {
            outr[r * N + c] = v.x;
            if (I != J) outr[c * N + r] = v.x;
        }
        else
        {
            outc[r * N + c] = v;
            if (I != J) outc[c * N + r] = make_cuDoubleComplex(v.x, -v.y);
        }
    }
}

template <typename T>
__device__ inline T tzero();
template <>
__device__ inline double tzero<double>() { return 0.0; }
template <>
__device__ inline cuDoubleComplex tzero<cuDoubleComplex>() { return make_cuDoubleComplex(0, 0); }

__device__ inline double tadd(double a, double b) { return a + b; }
__device__ inline cuDoubleComplex tadd(cuDoubleComplex a, cuDoubleComplex b) { return cuCadd(a, b); }
__device__ inline double tneg_one_plus(double a, bool diag) { return (diag ? 1.0 : 0.0) - a; }
__device__ inline cuDoubleComplex tneg_one_plus(cuDoubleComplex a, bool diag)
{
    return make_cuDoubleComplex((diag ? 1.0 : 0.0) - a.x, -a.y);
}

template <typename T>
__global__ void k_trace_negate(T *__restrict__ P, int N, T *__restrict__ trace)
{
    T *M = P + static_cast<long long>(blockIdx.x) * N * N;
    __shared__ T red[256];
    T acc = tzero<T>();
    for (int i = threadIdx.x; i < N; i += blockDim.x) acc = tadd(acc, M[static_cast<long long>(i) * N + i]);
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1)
    {
        if (threadIdx.x < s) red[threadIdx.x] = tadd(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) trace[blockIdx.x] = red[0];
    const long long nn = static_cast<long long>(N) * N;
    for (long long idx = threadIdx.x; idx < nn; idx += blockDim.x)
    {
        const bool d = (idx / N) == (idx % N);
        M[idx] = tneg_one_plus(M[idx], d);
    }
}

__device__ inline double tdiv(double a, double b) { return a / b; }
__device__ inline cuDoubleComplex tdiv(cuDoubleComplex a, cuDoubleComplex b) { return cuCdiv(a, b); }
__device__ inline double tfms(double c, double a, double b) { return fma(-a, b, c); }
__device__ inline cuDoubleComplex tfms(cuDoubleComplex c, cuDoubleComplex a, cuDoubleComplex b)
{
    return cuCsub(c, cuCmul(a, b));
}
__device__ inline double tlogpm(double u) { return log(u > 0 ? u : -u); }
__device__ inline cuDoubleComplex tlogpm(cuDoubleComplex u)
{
    if (!(u.x > 0)) u = make_cuDoubleComplex(-u.x, -u.y);
    return make_cuDoubleComplex(log(cuCabs(u)), atan2(u.y, u.x));
}

constexpr int LU_THREADS = 1024;

template <typename T>
__global__ void __launch_bounds__(LU_THREADS) k_lu_logdet(T *__restrict__ Mall, int N, T *__restrict__ logdet)
{
    T *M = Mall + static_cast<long long>(blockIdx.x) * N * N;
    __shared__ double bval[LU_THREADS / 32];
    __shared__ int bidx[LU_THREADS / 32];
    __shared__ int piv_s;
    T ld = tzero<T>();
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    for (int k = 0; k < N; ++k)
    {
        // pivot search (largest magnitude, first index on ties)
        double best = -1.0;
        int bi = N;
        for (int r = k + threadIdx.x; r < N; r += blockDim.x)
        {
            const double m = mag1(M[static_cast<long long>(r) * N + k]);
            if (m > best) { best = m; bi = r; }
        }
        for (int off = 16; off > 0; off >>= 1)
        {
            const double ob = __shfl_down_sync(0xffffffffu, best, off);
            const int oi = __shfl_down_sync(0xffffffffu, bi, off);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) { bval[warp] = best; bidx[warp] = bi; }
        __syncthreads();
        if (warp == 0)
        {
            best = lane < LU_THREADS / 32 ? bval[lane] : -1.0;
            bi = lane < LU_THREADS / 32 ? bidx[lane] : N;
            for (int off = 16; off > 0; off >>= 1)
            {
                const double ob = __shfl_down_sync(0xffffffffu, best, off);
                const int oi = __shfl_down_sync(0xffffffffu, bi, off);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (lane == 0) piv_s = bi;
        }
        __syncthreads();
        const int p = piv_s;
        if (p != k && p < N)
            for (int c = k + threadIdx.x; c < N; c += blockDim.x)
            {
                const T t = M[static_cast<long long>(k) * N + c];
                M[static_cast<long long>(k) * N + c] = M[static_cast<long long>(p) * N + c];
                M[static_cast<long long>(p) * N + c] = t;
            }
        __syncthreads();
        const T piv = M[static_cast<long long>(k) * N + k];
        if (threadIdx.x == 0) ld = tadd(ld, tlogpm(piv));
        for (int r = k + 1 + threadIdx.x; r < N; r += blockDim.x)
            M[static_cast<long long>(r) * N + k] = tdiv(M[static_cast<long long>(r) * N + k], piv);
        __syncthreads();
        const int m = N - k - 1;
        const long long nupd = static_cast<long long>(m) * m;
        for (long long t = threadIdx.x; t < nupd; t += blockDim.x)
        {
            const int r = k + 1 + static_cast<int>(t / m), c = k + 1 + static_cast<int>(t % m);
            M[static_cast<long long>(r) * N + c] =
                tfms(M[static_cast<long long>(r) * N + c], M[static_cast<long long>(r) * N + k],
                     M[static_cast<long long>(k) * N + c]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) logdet[blockIdx.x] = ld;
}

} // namespace

void launch_assemble_chi0(const cuDoubleComplex *src, long long slab_stride, int n_slabs, int N,
                          const int *atom_of, const int *abf_off, const int *nabf, const int *pair_of,
                          int n_at, const long long *e_off, bool real_only, cuDoubleComplex *outc,
                          double *outr, long long out_stride, cudaStream_t st)
{
    const long long nn = static_cast<long long>(N) * N;
    dim3 grid(static_cast<unsigned>(std::min<long long>((nn + 255) / 256, 65535)), n_slabs);
    k_assemble_chi0<<<grid, 256, 0, st>>>(src, slab_stride, N, atom_of, abf_off, nabf, pair_of, n_at, e_off,
                                          real_only, outc, outr, out_stride);
    GB_LAUNCH_CHECK();
}

// The inverse of k_assemble_chi0 on the upper atom pairs: out[s][e_off[p] + a nabf[J] + b] =
// dense[s][(abf_off[I] + a) N + abf_off[J] + b] for pair p = (I, J), a < nabf[I], b < nabf[J].
__global__ void k_scatter_pairs(const cuDoubleComplex *__restrict__ dense, long long dense_stride, int N,
                                const int *__restrict__ pI, const int *__restrict__ pJ, int n_pairs,
                                const int *__restrict__ abf_off, const int *__restrict__ nabf,
                                const long long *__restrict__ e_off, cuDoubleComplex *__restrict__ out,
                                long long slab_stride)
{
    const int s = blockIdx.z;
    for (int p = blockIdx.y; p < n_pairs; p += gridDim.y)
    {
        const int I = pI[p], J = pJ[p], nJ = nabf[J];
        const long long nel = static_cast<long long>(nabf[I]) * nJ;
        const cuDoubleComplex *src = dense + s * dense_stride;
        cuDoubleComplex *dst = out + s * slab_stride + e_off[p];
        for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < nel;
             t += static_cast<long long>(gridDim.x) * blockDim.x)
        {
            const int a = static_cast<int>(t / nJ), b = static_cast<int>(t % nJ);
            dst[t] = src[static_cast<long long>(abf_off[I] + a) * N + abf_off[J] + b];
        }
    }
}

void launch_scatter_pairs(const cuDoubleComplex *dense, long long dense_stride, int n_slabs, int N, const int *pI,
                          const int *pJ, int n_pairs, const int *abf_off, const int *nabf, const long long *e_off,
                          cuDoubleComplex *out, long long slab_stride, cudaStream_t st)
{
    if (n_pairs == 0 || n_slabs == 0) return;
    GB_REQUIRE(n_slabs <= 65535, "too many slabs for one scatter launch");
    const dim3 grid(8, std::min(n_pairs, 65535), n_slabs);
    k_scatter_pairs<<<grid, 256, 0, st>>>(dense, dense_stride, N, pI, pJ, n_pairs, abf_off, nabf, e_off, out,
                                          slab_stride);
    GB_LAUNCH_CHECK();
}

void launch_assemble_v(const cuDoubleComplex *blob, const long long *blk_off, const int *blk_IJ,
                       int n_blocks, const int *abf_off, const int *nabf, int N, bool real_only,
                       cuDoubleComplex *outc, double *outr, cudaStream_t st)
{
    if (n_blocks == 0) return;
    k_assemble_v<<<n_blocks, 256, 0, st>>>(blob, blk_off, blk_IJ, abf_off, nabf, N, real_only, outc, outr);
    GB_LAUNCH_CHECK();
}

void launch_trace_and_negate_c(cuDoubleComplex *P, int N, int batch, cuDoubleComplex *trace, cudaStream_t st)
{
    k_trace_negate<cuDoubleComplex><<<batch, 256, 0, st>>>(P, N, trace);
    GB_LAUNCH_CHECK();
}

void launch_trace_and_negate_r(double *P, int N, int batch, double *trace, cudaStream_t st)
{
    k_trace_negate<double><<<batch, 256, 0, st>>>(P, N, trace);
    GB_LAUNCH_CHECK();
}

void launch_lu_logdet_c(cuDoubleComplex *M, int N, int batch, cuDoubleComplex *logdet, cudaStream_t st)
{
    k_lu_logdet<cuDoubleComplex><<<batch, LU_THREADS, 0, st>>>(M, N, logdet);
    GB_LAUNCH_CHECK();
}

void launch_lu_logdet_r(double *M, int N, int batch, double *logdet, cudaStream_t st)
{
    k_lu_logdet<double><<<batch, LU_THREADS, 0, st>>>(M, N, logdet);
    GB_LAUNCH_CHECK();
}

} // namespace gb
