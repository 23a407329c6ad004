// E_c stage on the tensor cores + FP64 Cholesky.
//
// LibRPA evaluates, per IBZ q and frequency w (epsilon.cpp:414-536),
//   e(q,w) = ln det(I - V chi0) + tr(V chi0)
// with an LU of I - V chi0.  With V = L L^H (V is Hermitian positive definite),
//   det(I - V chi0) = det(I - L^H chi0 L)
// and M' = I - L^H chi0 L is Hermitian positive definite (chi0 is negative semidefinite),
// so ln det comes from an FP64 Cholesky: ln det M' = 2 sum log L'_ii.  The two N^3
// products L^H chi0 L run on tcgen05 with 3-piece BF16 operands; complex matrices use
// the real embedding [[Re, -Im], [Im, Re]].  tr(V chi0) = sum_ij V_ij conj(chi0_ij) in FP64.
#include <cuComplex.h>

#include <vector>

#include "chol.h"
#include "common.h"
#include "ec_tc.h"
#include "kernels.h"
#include "tc_gemm.h"

namespace gb {

namespace {

__device__ __forceinline__ void split3(double x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l)
{
    h = __double2bfloat16(x);
    const double r1 = x - static_cast<double>(__bfloat162float(h));
    m = __double2bfloat16(r1);
    l = __double2bfloat16(r1 - static_cast<double>(__bfloat162float(m)));
}

// A operand (2M x kpad) of the embedding of X (M x K complex): rows r < M: [Re X, -Im X],
// rows M + r: [Im X, Re X].  X(r,k) = src[r][k], or conj(src[k][r]) when ctrans.
__global__ void k_embed_A(const cuDoubleComplex *__restrict__ src, long long sstride, int M, int K, int kpad,
                          bool ctrans, __nv_bfloat16 *__restrict__ p0, __nv_bfloat16 *__restrict__ p1,
                          __nv_bfloat16 *__restrict__ p2, long long ostride)
{
    const int b = blockIdx.y;
    const cuDoubleComplex *S = src + b * sstride;
    const long long n = 2LL * M * kpad;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const int row = static_cast<int>(t / kpad), col = static_cast<int>(t % kpad);
        double x = 0.0;
        if (col < 2 * K)
        {
            // rows and K both interleaved: row 2 r + (0: Re, 1: Im), column 2 k + (0: Re, 1: Im)
            const int r = row >> 1, k = col >> 1;
            cuDoubleComplex v = ctrans ? S[static_cast<long long>(k) * M + r] : S[static_cast<long long>(r) * K + k];
            if (ctrans) v.y = -v.y;
            const bool top = (row & 1) == 0, left = (col & 1) == 0;
            x = top ? (left ? v.x : -v.y) : (left ? v.y : v.x);
        }
        __nv_bfloat16 h, m, l;
        split3(x, h, m, l);
        const long long o = b * ostride + t;
        p0[o] = h;
        p1[o] = m;
        p2[o] = l;
    }
}

// B operand (N x kpad, K-major) of the embedding [Re Y; Im Y] of Y (K x N complex): row n = [Re Y(:,n), Im Y(:,n)].
__global__ void k_embed_Bt(const cuDoubleComplex *__restrict__ Y, int K, int N, int kpad,
                           __nv_bfloat16 *__restrict__ p0, __nv_bfloat16 *__restrict__ p1,
                           __nv_bfloat16 *__restrict__ p2)
{
    const long long n = static_cast<long long>(N) * kpad;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const int row = static_cast<int>(t / kpad), col = static_cast<int>(t % kpad);
        double x = 0.0;
        if (col < 2 * K)
        {
            const int k = col >> 1;  // K interleaved: 2 k + (0: Re, 1: Im)
            const cuDoubleComplex v = Y[static_cast<long long>(k) * N + row];
            x = (col & 1) == 0 ? v.x : v.y;
        }
        __nv_bfloat16 h, m, l;
        split3(x, h, m, l);
        p0[t] = h;
        p1[t] = m;
        p2[t] = l;
    }
}

// K-major B operand of a row-major FP32 matrix S (K x N): row n = S(:, n) (batched).
__global__ void k_split_T_f32(const float *__restrict__ S, long long sstride, int K, int N, int kpad,
                              __nv_bfloat16 *__restrict__ p0, __nv_bfloat16 *__restrict__ p1,
                              __nv_bfloat16 *__restrict__ p2, long long ostride)
{
    __shared__ float tile[32][33];
    const int b = blockIdx.z;
    const float *Sb = S + b * sstride;
    const int k0 = blockIdx.x * 32, n0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y)
    {
        const int k = k0 + i, n = n0 + threadIdx.x;
        tile[i][threadIdx.x] = (k < K && n < N) ? Sb[static_cast<long long>(k) * N + n] : 0.0f;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y)
    {
        const int n = n0 + i, k = k0 + threadIdx.x;
        if (n < N && k < kpad)
        {
            __nv_bfloat16 h, m, l;
            split3(static_cast<double>(tile[threadIdx.x][i]), h, m, l);
            const long long o = b * ostride + static_cast<long long>(n) * kpad + k;
            p0[o] = h;
            p1[o] = m;
            p2[o] = l;
        }
    }
}

// M'[b] = I - (Re M + i Im M), the FP32 product with interleaved rows: row 2 i = Re M(i, :),
// row 2 i + 1 = Im M(i, :) (2N x N)
__global__ void k_form_mprime_c(const float *__restrict__ Ms, int N, cuDoubleComplex *__restrict__ Mp)
{
    const int b = blockIdx.y;
    const long long nn = static_cast<long long>(N) * N;
    const float *S = Ms + b * 2 * nn;
    cuDoubleComplex *O = Mp + b * nn;
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < nn;
         e += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long i = e / N, j = e % N;
        const float *row = S + 2 * i * N + j;
        O[e] = make_cuDoubleComplex((i == j ? 1.0 : 0.0) - static_cast<double>(row[0]), -static_cast<double>(row[N]));
    }
}

// Real embedding of M' = I - M for the tensor-core Cholesky: E[2i + p][2j + q] =
// [[Re M'_ij, -Im M'_ij], [Im M'_ij, Re M'_ij]][p][q], lower triangle only (upper zero);
// Ms has interleaved rows (2 i: Re M(i, :), 2 i + 1: Im M(i, :)).  E is symmetric positive
// definite when M' is Hermitian positive definite, and ln det E = 2 ln det M'.
__global__ void k_form_mprime_emb(const float *__restrict__ Ms, int N, double *__restrict__ Ep)
{
    const int b = blockIdx.y;
    const long long nn = static_cast<long long>(N) * N, n2 = 2LL * N;
    const float *S = Ms + b * 2 * nn;
    double *O = Ep + b * n2 * n2;
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < n2 * n2;
         e += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long r = e / n2, c = e % n2;
        const long long i = r >> 1, j = c >> 1;
        const int p = static_cast<int>(r & 1), q = static_cast<int>(c & 1);
        double v = 0.0;
        if (c <= r)
        {
            const double re = (i == j ? 1.0 : 0.0) - static_cast<double>(S[2 * i * N + j]);
            const double im = -static_cast<double>(S[(2 * i + 1) * N + j]);
            v = p == q ? re : (p == 1 ? im : -im);
        }
        O[e] = v;
    }
}

__global__ void k_form_mprime_r(const float *__restrict__ Ms, int N, double *__restrict__ Mp)
{
    const int b = blockIdx.y;
    const long long nn = static_cast<long long>(N) * N;
    const float *S = Ms + b * nn;
    double *O = Mp + b * nn;
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < nn;
         e += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        // lower triangle only: the product kernel leaves the upper tiles of M unwritten
        const long long i = e / N, j = e % N;
        O[e] = j > i ? 0.0 : (i == j ? 1.0 : 0.0) - static_cast<double>(S[e]);
    }
}

// tr(V X[b]) = sum_ij V_ij X_ji (full matrices), FP64, one CTA per batch entry
unsigned blocks_for(long long n) { return static_cast<unsigned>(std::min<long long>((n + 255) / 256, 152LL * 16)); }


// tr(M) per frequency from the FP32 products M = L^H chi0 L (diagonal of the Re / Im blocks)
__global__ void k_diag_trace(const float *__restrict__ Ms, int N, int parts, double2 *__restrict__ tr)
{
    __shared__ double rr[256], ri[256];
    const long long nn = static_cast<long long>(N) * N;
    const float *S = Ms + static_cast<long long>(blockIdx.x) * parts * nn;
    double ar = 0.0, ai = 0.0;
    // rows interleaved by part: row parts * i (+ 1) holds Re (Im) of row i
    for (int i = threadIdx.x; i < N; i += blockDim.x)
    {
        ar += S[static_cast<long long>(parts) * i * N + i];
        if (parts > 1) ai += S[(static_cast<long long>(parts) * i + 1) * N + i];
    }
    rr[threadIdx.x] = ar;
    ri[threadIdx.x] = ai;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1)
    {
        if (threadIdx.x < s)
        {
            rr[threadIdx.x] += rr[threadIdx.x + s];
            ri[threadIdx.x] += ri[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) tr[blockIdx.x] = make_double2(rr[0], ri[0]);
}

// FP64 forms of the same steps (all-FP64 path): out = conj(transpose(L)) (or transpose),
// M' = I - M and tr(M)
__global__ void k_adjoint_c(const cuDoubleComplex *__restrict__ L, int N, cuDoubleComplex *__restrict__ out)
{
    const long long nn = static_cast<long long>(N) * N;
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < nn;
         e += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const cuDoubleComplex v = L[(e % N) * N + e / N];
        out[e] = make_cuDoubleComplex(v.x, -v.y);
    }
}

__global__ void k_transpose_r(const double *__restrict__ L, int N, double *__restrict__ out)
{
    const long long nn = static_cast<long long>(N) * N;
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < nn;
         e += static_cast<long long>(gridDim.x) * blockDim.x)
        out[e] = L[(e % N) * N + e / N];
}

template <typename T>
__device__ inline double2 as_d2(T v);
template <>
__device__ inline double2 as_d2<double>(double v) { return make_double2(v, 0.0); }
template <>
__device__ inline double2 as_d2<cuDoubleComplex>(cuDoubleComplex v) { return make_double2(v.x, v.y); }

template <typename T>
__global__ void k_form_mprime64(const T *__restrict__ M, int N, T *__restrict__ Mp, double2 *__restrict__ tr)
{
    __shared__ double rr[256], ri[256];
    const long long nn = static_cast<long long>(N) * N;
    const T *S = M + blockIdx.y * nn;
    T *O = Mp + blockIdx.y * nn;
    for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < nn;
         e += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const double2 v = as_d2(S[e]);
        const double d = (e / N) == (e % N) ? 1.0 : 0.0;
        if constexpr (sizeof(T) == sizeof(double))
            reinterpret_cast<double *>(O)[e] = d - v.x;
        else
            reinterpret_cast<cuDoubleComplex *>(O)[e] = make_cuDoubleComplex(d - v.x, -v.y);
    }
    if (blockIdx.x != 0) return;
    double ar = 0.0, ai = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x)
    {
        const double2 v = as_d2(S[static_cast<long long>(i) * N + i]);
        ar += v.x;
        ai += v.y;
    }
    rr[threadIdx.x] = ar;
    ri[threadIdx.x] = ai;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1)
    {
        if (threadIdx.x < s)
        {
            rr[threadIdx.x] += rr[threadIdx.x + s];
            ri[threadIdx.x] += ri[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) tr[blockIdx.y] = make_double2(rr[0], ri[0]);
}

} // namespace

struct EcChol::Impl
{
    int N = 0, nw = 0, qb = 1;
    bool cplx = true, fp64 = false;
    DevBuf<cuDoubleComplex> T64c, M64c, LHc;  // all-FP64 products
    DevBuf<double> T64r, M64r, LHr;
    long long kpad = 0;
    DevBuf<int> err, bad, badV;
    SplitStore Bl, Al;            // L as B^T and L^H (or L^T) as A, one q at a time
    DevBuf<double> diagV;
    SplitStore A1, B2;            // per-(q, w) operands, one q at a time
    DevBuf<float> Tst, Mst;
    DevBuf<double> diag, logdet;  // qb * nw matrices
    DevBuf<double2> tr;
    DevBuf<cuDoubleComplex> Mpc;
    DevBuf<double> Mpr;
    // real matrices: Cholesky trailing updates on the tensor cores (exact integer slices);
    // complex M' is factored as its real 2N x 2N embedding (emb) by the same kernels
    bool ozaki = false, emb = false;
    OzakiWork oz;
    ~Impl() { ozaki_free(oz); }
};

EcChol::EcChol(int N, int nw, bool complex_path, int qb, bool fp64_products) : impl_(std::make_unique<Impl>())
{
    Impl &m = *impl_;
    m.N = N;
    m.nw = nw;
    m.qb = qb;
    m.cplx = complex_path;
    m.fp64 = fp64_products;
    const int kdim = complex_path ? 2 * N : N;
    m.kpad = (kdim + 63) / 64 * 64;
    const long long rowsA = kdim;  // rows of the A operands
    const size_t nmat = static_cast<size_t>(qb) * nw;
    m.err.alloc(1);
    m.bad.alloc(nmat);
    m.badV.alloc(qb);
    m.diagV.alloc(static_cast<size_t>(qb) * N);
    m.emb = complex_path && !fp64_products && N > OZAKI_NB / 2;
    const size_t ndiag = m.emb ? 2 * static_cast<size_t>(N) : N;
    m.diag.alloc(nmat * ndiag);
    m.logdet.alloc(nmat);
    m.tr.alloc(nmat);
    if (m.emb)
        m.Mpr.alloc(nmat * 4 * N * N);
    else if (complex_path)
        m.Mpc.alloc(nmat * N * N);
    else
        m.Mpr.alloc(nmat * N * N);
    // V (one per q) and, for real matrices, M' go through the tensor-core Cholesky
    m.ozaki = !complex_path && !fp64_products && N > OZAKI_NB;
    if (m.ozaki) ozaki_alloc(m.oz, N, static_cast<int>(nmat));
    if (m.emb) ozaki_alloc(m.oz, 2 * N, static_cast<int>(nmat));
    if (fp64_products)
    {
        const size_t nn = static_cast<size_t>(N) * N;
        if (complex_path)
        {
            m.T64c.alloc(nw * nn);
            m.M64c.alloc(nw * nn);
            m.LHc.alloc(nn);
        }
        else
        {
            m.T64r.alloc(nw * nn);
            m.M64r.alloc(nw * nn);
            m.LHr.alloc(nn);
        }
        return;
    }
    m.Bl.alloc(3, static_cast<size_t>(N) * m.kpad);
    m.Al.alloc(3, static_cast<size_t>(rowsA) * m.kpad);
    m.A1.alloc(3, static_cast<size_t>(nw) * rowsA * m.kpad);
    m.B2.alloc(3, static_cast<size_t>(nw) * N * m.kpad);
    m.Tst.alloc(static_cast<size_t>(nw) * rowsA * N);
    m.Mst.alloc(static_cast<size_t>(nw) * rowsA * N);
}

EcChol::~EcChol() = default;

int EcChol::factor_v(void *V, int nb, std::vector<int> &bad, cudaStream_t st)
{
    Impl &m = *impl_;
    GB_REQUIRE(nb >= 1 && nb <= m.qb, "Coulomb batch larger than the E_c batch");
    m.badV.zero(st);
    int launches = 1;
    if (m.cplx)
    {
        launches += chol_batched_c(static_cast<cuDoubleComplex *>(V), m.N, nb, m.diagV.get(), m.badV.get(), st);
        zero_upper_c(static_cast<cuDoubleComplex *>(V), m.N, nb, st);
    }
    else
    {
        launches += m.ozaki ? chol_batched_r_ozaki(static_cast<double *>(V), m.N, nb, m.diagV.get(), m.badV.get(),
                                                   m.oz, st)
                            : chol_batched_r(static_cast<double *>(V), m.N, nb, m.diagV.get(), m.badV.get(), st);
        zero_upper_r(static_cast<double *>(V), m.N, nb, st);
    }
    bad.assign(nb, 0);
    int herr = 0;
    m.badV.download(bad.data(), nb, st);
    if (m.ozaki) GB_CUDA(cudaMemcpyAsync(&herr, m.oz.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    GB_REQUIRE(herr == 0, "tensor-core Cholesky update reported wait timeout code " + std::to_string(herr));
    return launches;
}

int EcChol::stage_q(const void *L, const void *X, int slot, cudaStream_t st)
{
    Impl &m = *impl_;
    const int N = m.N, nw = m.nw;
    GB_REQUIRE(slot >= 0 && slot < m.qb, "E_c batch slot out of range");
    const long long nn = static_cast<long long>(N) * N;
    int launches = 0;
    if (slot == 0)
    {
        m.err.zero(st);
        m.bad.zero(st);
    }
    if (m.fp64)
    {
        // M = L^H (chi0 L) with FP64 GEMMs, then M' = I - M and tr(M)
        const size_t off = static_cast<size_t>(slot) * nw * nn;
        dim3 gf(blocks_for(nn), nw);
        if (m.cplx)
        {
            const cuDoubleComplex *Lc = static_cast<const cuDoubleComplex *>(L);
            launch_zgemm(N, N, N, static_cast<const cuDoubleComplex *>(X), N, nn, Lc, N, 0, m.T64c.get(), N, nn, nw, st);
            k_adjoint_c<<<blocks_for(nn), 256, 0, st>>>(Lc, N, m.LHc.get());
            GB_LAUNCH_CHECK();
            launch_zgemm(N, N, N, m.LHc.get(), N, 0, m.T64c.get(), N, nn, m.M64c.get(), N, nn, nw, st);
            k_form_mprime64<cuDoubleComplex><<<gf, 256, 0, st>>>(m.M64c.get(), N, m.Mpc.get() + off,
                                                                  m.tr.get() + static_cast<size_t>(slot) * nw);
        }
        else
        {
            const double *Lr = static_cast<const double *>(L);
            launch_dgemm(N, N, N, static_cast<const double *>(X), N, nn, Lr, N, 0, m.T64r.get(), N, nn, nw, 1.0, 0.0, st);
            k_transpose_r<<<blocks_for(nn), 256, 0, st>>>(Lr, N, m.LHr.get());
            GB_LAUNCH_CHECK();
            launch_dgemm(N, N, N, m.LHr.get(), N, 0, m.T64r.get(), N, nn, m.M64r.get(), N, nn, nw, 1.0, 0.0, st);
            k_form_mprime64<double><<<gf, 256, 0, st>>>(m.M64r.get(), N, m.Mpr.get() + off,
                                                         m.tr.get() + static_cast<size_t>(slot) * nw);
        }
        GB_LAUNCH_CHECK();
        return 4;
    }
    const SplitBufs bl = m.Bl.bufs(), al = m.Al.bufs(), a1 = m.A1.bufs(), b2 = m.B2.bufs();
    const long long rowsA = m.cplx ? 2LL * N : N;
    if (m.cplx)
    {
        const cuDoubleComplex *Lc = static_cast<const cuDoubleComplex *>(L);
        const cuDoubleComplex *Xc = static_cast<const cuDoubleComplex *>(X);
        k_embed_Bt<<<blocks_for(N * m.kpad), 256, 0, st>>>(Lc, N, N, static_cast<int>(m.kpad), bl.p[0], bl.p[1], bl.p[2]);
        k_embed_A<<<dim3(blocks_for(rowsA * m.kpad), 1), 256, 0, st>>>(Lc, 0, N, N, static_cast<int>(m.kpad), true,
                                                                        al.p[0], al.p[1], al.p[2], 0);
        k_embed_A<<<dim3(blocks_for(rowsA * m.kpad), nw), 256, 0, st>>>(Xc, nn, N, N, static_cast<int>(m.kpad), false,
                                                                         a1.p[0], a1.p[1], a1.p[2], rowsA * m.kpad);
        GB_LAUNCH_CHECK();
        launches += 3;
    }
    else
    {
        const double *Lr = static_cast<const double *>(L);
        const double *Xr = static_cast<const double *>(X);
        // B^T of L and A = L^T are the same K-major matrix: row n = L(:, n)
        split_transpose_f64(Lr, N, N, N, static_cast<int>(m.kpad), bl, st);
        split_transpose_f64(Lr, N, N, N, static_cast<int>(m.kpad), al, st);
        for (int w = 0; w < nw; ++w)
        {
            SplitBufs aw{3, {a1.p[0] + w * rowsA * m.kpad, a1.p[1] + w * rowsA * m.kpad, a1.p[2] + w * rowsA * m.kpad}};
            split_rows_f64(Xr + w * nn, N, N, N, static_cast<int>(m.kpad), aw, st);
        }
        launches += 2 + nw;
    }
    // T = chi0 L  (rowsA x N per w); L is lower triangular, so the K range of an output column
    // block n starts at n (at 2n with the complex path's interleaved K)
    TcGemmOpts o1, o2;
    o1.tri = 1;
    o2.tri = 2;  // A = L^H: row m is zero before column m (interleaved: row 2m + p before K 2m)
    if (m.cplx)
        o1.tri_mul = 2;  // K interleaved: L(:, n) is zero before K index 2n
    else
        o2.lower_tiles = true;  // M is symmetric: its lower triangle is all that is read
    tc_gemm_split(m.A1.mat(rowsA, m.kpad, rowsA * m.kpad), m.Bl.mat(N, m.kpad, 0), static_cast<int>(rowsA), N,
                  static_cast<int>(m.cplx ? 2 * N : N), nw, m.Tst.get(), N, rowsA * N, false, m.err.get(), st, o1);
    // B2 = K-major form of T (row n = T(:, n))
    {
        dim3 g(static_cast<unsigned>((m.kpad + 31) / 32), static_cast<unsigned>((N + 31) / 32), nw);
        k_split_T_f32<<<g, dim3(32, 8), 0, st>>>(m.Tst.get(), rowsA * N, static_cast<int>(rowsA), N,
                                                 static_cast<int>(m.kpad), b2.p[0], b2.p[1], b2.p[2], N * m.kpad);
        GB_LAUNCH_CHECK();
    }
    // M = L^H T
    tc_gemm_split(m.Al.mat(rowsA, m.kpad, 0), m.B2.mat(N, m.kpad, N * m.kpad), static_cast<int>(rowsA), N,
                  static_cast<int>(m.cplx ? 2 * N : N), nw, m.Mst.get(), N, rowsA * N, false, m.err.get(), st, o2);
    // tr(V chi0) = tr(L^H chi0 L) from the same products as M': to first order the FP32
    // rounding of M cancels between ln det(I - M) and tr(M)
    k_diag_trace<<<nw, 256, 0, st>>>(m.Mst.get(), N, m.cplx ? 2 : 1, m.tr.get() + static_cast<size_t>(slot) * nw);
    GB_LAUNCH_CHECK();
    const size_t off = static_cast<size_t>(slot) * nw * nn;
    if (m.emb)
        k_form_mprime_emb<<<dim3(blocks_for(4 * nn), nw), 256, 0, st>>>(m.Mst.get(), N, m.Mpr.get() + 4 * off);
    else if (m.cplx)
        k_form_mprime_c<<<dim3(blocks_for(nn), nw), 256, 0, st>>>(m.Mst.get(), N, m.Mpc.get() + off);
    else
        k_form_mprime_r<<<dim3(blocks_for(nn), nw), 256, 0, st>>>(m.Mst.get(), N, m.Mpr.get() + off);
    GB_LAUNCH_CHECK();
    return launches + 5;
}

int EcChol::finish(int nslots, std::vector<std::complex<double>> &trace_out,
                   std::vector<std::complex<double>> &logdet_out, cudaStream_t st)
{
    Impl &m = *impl_;
    const int N = m.N;
    GB_REQUIRE(nslots >= 1 && nslots <= m.qb, "E_c batch slot count out of range");
    const int nmat = nslots * m.nw;
    int launches = 1;
    if (m.emb)
        launches += chol_batched_r_ozaki(m.Mpr.get(), 2 * N, nmat, m.diag.get(), m.bad.get(), m.oz, st);
    else if (m.cplx)
        launches += chol_batched_c(m.Mpc.get(), N, nmat, m.diag.get(), m.bad.get(), st);
    else
        launches += m.ozaki ? chol_batched_r_ozaki(m.Mpr.get(), N, nmat, m.diag.get(), m.bad.get(), m.oz, st)
                            : chol_batched_r(m.Mpr.get(), N, nmat, m.diag.get(), m.bad.get(), st);
    chol_logdet(m.diag.get(), m.emb ? 2 * N : N, nmat, m.logdet.get(), st);
    std::vector<double> ld(nmat);
    std::vector<int> bad(nmat);
    std::vector<double2> tr(nmat);
    int herr = 0;
    m.logdet.download(ld.data(), nmat, st);
    m.bad.download(bad.data(), nmat, st);
    m.tr.download(tr.data(), nmat, st);
    int herr_oz = 0;
    m.err.download(&herr, 1, st);
    if (m.ozaki || m.emb) GB_CUDA(cudaMemcpyAsync(&herr_oz, m.oz.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    GB_REQUIRE(herr == 0, "tensor-core E_c GEMM reported wait timeout code " + std::to_string(herr));
    GB_REQUIRE(herr_oz == 0, "tensor-core Cholesky update reported wait timeout code " + std::to_string(herr_oz));
    for (int b = 0; b < nmat; ++b)
        GB_REQUIRE(!bad[b], "I - L^H chi0 L is not positive definite (chi0 not negative semidefinite?)");
    trace_out.assign(nmat, {0.0, 0.0});
    logdet_out.assign(nmat, {0.0, 0.0});
    for (int b = 0; b < nmat; ++b)
    {
        trace_out[b] = {tr[b].x, m.cplx ? tr[b].y : 0.0};
        logdet_out[b] = {m.emb ? 0.5 * ld[b] : ld[b], 0.0};  // ln det E = 2 ln det M'
    }
    return launches;
}

} // namespace gb
