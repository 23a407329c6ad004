// Split-precision GEMM on the 5th-generation tensor cores.
//
//   D[b][m][n] (+)= sum_k A[b][m][k] * B[b][n][k]
// with A = A_hi + A_lo and B = B_hi + B_lo held as BF16 pairs and the product
// formed from three tcgen05.mma terms (hi*hi + hi*lo + lo*hi) into one FP32
// TMEM accumulator; the dropped lo*lo term and the split residuals leave a
// relative error of about 2^-16 per product.
//
// One CTA computes a 128 x 128 output tile.  Warp 0 (one lane) streams the
// four operand tiles of each 64-wide K step into a 3-stage shared-memory ring
// with TMA (128-byte swizzle); warp 1 (one lane) issues the MMAs and releases
// each stage with tcgen05.commit; after the last step all four warps drain
// TMEM with tcgen05.ld and write FP32 results.  Every mbarrier wait is bounded
// and reports a timeout through the device error flag instead of hanging.
#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>

#include "common.h"
#include "tc_common.cuh"
#include "work_schedule.h"
#include "tc_gemm.h"

namespace gb {

namespace {

using namespace tc;

constexpr int BM = 128, BN = 128, BK = 64;
constexpr int TILE_A = BM * BK * 2;  // bytes per bf16 tile
constexpr int TILE_B = BN * BK * 2;

template <int NS>
struct Cfg
{
    static constexpr int STAGES = NS == 2 ? 3 : 2;
    static constexpr int STAGE_BYTES = NS * TILE_A + NS * TILE_B;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
    static_assert(SMEM_BYTES <= 227 * 1024, "shared memory budget");
};

struct TmapSet
{
    CUtensorMap a[3], b[3];  // hi, lo (NS = 2) or hi, mid, lo (NS = 3)
};

// Split terms, smallest first.  NS = 2: lo*hi, hi*lo, hi*hi.
// NS = 3 (hi, mid, lo = pieces 0, 1, 2): the six terms with piece-order sum <= 2.
__host__ __device__ constexpr int n_terms(int ns) { return ns == 2 ? 3 : 6; }
__host__ __device__ constexpr int term_a(int ns, int t)
{
    return ns == 2 ? (t == 0 ? 1 : 0) : (t == 0 ? 2 : (t == 1 ? 0 : (t == 2 ? 1 : (t == 3 ? 1 : 0))));
}
__host__ __device__ constexpr int term_b(int ns, int t)
{
    return ns == 2 ? (t == 1 ? 1 : 0) : (t == 0 ? 0 : (t == 1 ? 2 : (t == 2 ? 1 : (t == 3 ? 0 : (t == 4 ? 1 : 0)))));
}

// The tensor core's FP32 accumulation truncates, so its error grows linearly with the
// number of accumulating MMAs.  The mainloop therefore restarts two TMEM accumulators every
// K stage -- one for hi*hi, one for the smaller cross terms -- in a double buffer, and four
// drain warps add each stage's pair into round-to-nearest FP32 registers while the next
// stage's MMAs run.
constexpr int GEMM_THREADS = 256;  // warp 0: TMA, warp 1: MMA, warps 4-7: drain + epilogue
using sched::tile_coords;  // grouped raster / lower-tile order of the output tiles (work_schedule.h)

template <int NS>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    k_tc_gemm(const __grid_constant__ TmapSet maps, int M, int N, int K, float *__restrict__ D, long long ldd,
              long long sD, int accumulate_out, int a_bcast, int b_bcast, int tri, int tri_mul, int lower,
              int *__restrict__ err)
{
    constexpr int STAGES = Cfg<NS>::STAGES, STAGE_BYTES = Cfg<NS>::STAGE_BYTES;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *accf = empty + STAGES;   // [2] accumulator pair b ready for draining
    uint64_t *acce = accf + 2;         // [2] accumulator pair b drained
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acce + 2);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    int mt, nt;
    tile_coords(blockIdx.x, (M + BM - 1) / BM, (N + BN - 1) / BN, lower, mt, nt);
    const int n0 = nt * BN, m0 = mt * BM, b = blockIdx.z;
    const int nk = (K + BK - 1) / BK;
    // K blocks that can be nonzero: B[n][k] = 0 for k < tri_mul n (tri 1), A[m][k] = 0 for k < m
    // (tri 2)
    const int kb0 = tri == 1 ? tri_mul * n0 / BK : (tri == 2 ? m0 / BK : 0);
    const int nsteps = nk - kb0;

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < STAGES; ++s)
        {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int i = 0; i < 2; ++i)
        {
            mbar_init(&accf[i], 1);
            mbar_init(&acce[i], 128);
        }
        fence_barrier_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, 4 * BN);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    bool ok = true;

    if (warp == 0 && lane == 0)
    {
        const int za = a_bcast ? 0 : b, zb = b_bcast ? 0 : b;
        for (int it = 0; it < nsteps; ++it)
        {
            const int kb = kb0 + it, s = it % STAGES, r = it / STAGES;
            if (!mbar_wait(&empty[s], (r & 1) ^ 1))
            {
                atomicExch(err, 101);
                break;
            }
            unsigned char *st = smem + s * STAGE_BYTES;
            mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
#pragma unroll
            for (int p = 0; p < NS; ++p)
            {
                tma_load_3d(st + p * TILE_A, &maps.a[p], kb * BK, m0, za, &full[s]);
                tma_load_3d(st + NS * TILE_A + p * TILE_B, &maps.b[p], kb * BK, n0, zb, &full[s]);
            }
        }
    }
    else if (warp == 1 && lane == 0)
    {
        constexpr uint32_t idesc = idesc_bf16_f32(BM, BN);
        for (int it = 0; it < nsteps; ++it)
        {
            const int s = it % STAGES, r = it / STAGES;
            const int ab = it & 1;
            if (!mbar_wait(&full[s], r & 1) || !mbar_wait(&acce[ab], ((it >> 1) & 1) ^ 1))
            {
                atomicExch(err, 102);
                break;
            }
            tc_fence_after();
            const uint32_t t_hh = tmem + ab * 2 * BN, t_x = t_hh + BN;
            unsigned char *st = smem + s * STAGE_BYTES;
            uint64_t da[NS], db[NS];
#pragma unroll
            for (int p = 0; p < NS; ++p)
            {
                da[p] = smem_desc_sw128(st + p * TILE_A);
                db[p] = smem_desc_sw128(st + NS * TILE_A + p * TILE_B);
            }
#pragma unroll
            for (int k = 0; k < BK / 16; ++k)
            {
                const uint64_t dk = static_cast<uint64_t>(k * 32 >> 4);
#pragma unroll
                for (int t = 0; t < n_terms(NS) - 1; ++t)  // cross terms, smallest first
                    mma_bf16(t_x, da[term_a(NS, t)] + dk, db[term_b(NS, t)] + dk, idesc, (k | t) != 0);
                mma_bf16(t_hh, da[0] + dk, db[0] + dk, idesc, k != 0);
            }
            mma_commit(&empty[s]);
            mma_commit(&accf[ab]);
        }
    }
    else if (warp >= 4)
    {
        const int w = warp - 4;
        const uint32_t lane_base = static_cast<uint32_t>(w * 32) << 16;
        float acc[BN];
#pragma unroll
        for (int c = 0; c < BN; ++c) acc[c] = 0.0f;
        for (int it = 0; it < nsteps; ++it)
        {
            const int ab = it & 1;
            if (!mbar_wait(&accf[ab], (it >> 1) & 1))
            {
                atomicExch(err, 103);
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t t_hh = tmem + ab * 2 * BN, t_x = t_hh + BN;
#pragma unroll
            for (int c0 = 0; c0 < BN; c0 += 16)
            {
                float vh[16], vx[16];
                tmem_ld16(t_hh + lane_base + c0, vh);
                tmem_ld16(t_x + lane_base + c0, vx);
#pragma unroll
                for (int i = 0; i < 16; ++i) acc[c0 + i] += vh[i] + vx[i];
            }
            tc_fence_before();
            mbar_arrive(&acce[ab]);
        }
        const int m = m0 + w * 32 + lane;
        if (ok && m < M)
        {
            float *drow = D + b * sD + static_cast<long long>(m) * ldd;
#pragma unroll
            for (int c = 0; c < BN; ++c)
            {
                const int n = n0 + c;
                if (n < N) drow[n] = accumulate_out ? drow[n] + acc[c] : acc[c];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 4 * BN);
}

// x = hi + mid (+ lo) as BF16 pieces (round to nearest each); zero padding of columns [cols, kpad)
template <typename T>
__device__ __forceinline__ void split_value(T x, int ns, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l)
{
    const double xd = static_cast<double>(x);
    h = __double2bfloat16(xd);
    const double r1 = xd - static_cast<double>(__bfloat162float(h));
    m = __double2bfloat16(r1);
    const double r2 = r1 - static_cast<double>(__bfloat162float(m));
    l = __double2bfloat16(r2);
    (void)ns;
}

template <typename T>
__global__ void k_split_rows(const T *__restrict__ src, long long lds, long long rows, int cols, int kpad, int ns,
                             __nv_bfloat16 *__restrict__ p0, __nv_bfloat16 *__restrict__ p1,
                             __nv_bfloat16 *__restrict__ p2)
{
    const long long n = rows * kpad;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long r = t / kpad;
        const int c = static_cast<int>(t % kpad);
        const T x = c < cols ? src[r * lds + c] : T(0);
        __nv_bfloat16 h, m, l;
        split_value(x, ns, h, m, l);
        p0[t] = h;
        if (ns == 2)
            p1[t] = m;
        else
        {
            p1[t] = m;
            p2[t] = l;
        }
    }
}

// dst[n][k] from src[k][n] (B operand of a row-major K x N matrix)
template <typename T>
__global__ void k_split_transpose(const T *__restrict__ src, long long lds, int K, int N, int kpad, int ns,
                                  __nv_bfloat16 *__restrict__ p0, __nv_bfloat16 *__restrict__ p1,
                                  __nv_bfloat16 *__restrict__ p2)
{
    __shared__ T tile[32][33];
    const int k0 = blockIdx.x * 32, nb0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y)
    {
        const int k = k0 + i, n = nb0 + threadIdx.x;
        tile[i][threadIdx.x] = (k < K && n < N) ? src[static_cast<long long>(k) * lds + n] : T(0);
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y)
    {
        const int n = nb0 + i, k = k0 + threadIdx.x;
        if (n < N && k < kpad)
        {
            __nv_bfloat16 h, m, l;
            split_value(tile[threadIdx.x][i], ns, h, m, l);
            const long long o = static_cast<long long>(n) * kpad + k;
            p0[o] = h;
            p1[o] = m;
            if (ns == 3) p2[o] = l;
        }
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    GB_REQUIRE(fn, "cuTensorMapEncodeTiled not available from the driver");
    return fn;
}

} // namespace

void make_tmap_bf16(CUtensorMap *map, const void *base, long long inner, long long rows, long long batch,
                    long long row_stride_elems, long long batch_stride_elems, int box_inner, int box_rows)
{
    GB_REQUIRE((reinterpret_cast<uintptr_t>(base) & 15) == 0, "TMA base address must be 16-byte aligned");
    GB_REQUIRE((row_stride_elems * 2) % 16 == 0 && (batch_stride_elems * 2) % 16 == 0,
               "TMA strides must be multiples of 16 bytes");
    cuuint64_t dims[3] = {static_cast<cuuint64_t>(inner), static_cast<cuuint64_t>(rows),
                          static_cast<cuuint64_t>(batch)};
    cuuint64_t strides[2] = {static_cast<cuuint64_t>(row_stride_elems * 2),
                             static_cast<cuuint64_t>((batch > 1 ? batch_stride_elems : row_stride_elems * rows) * 2)};
    cuuint32_t box[3] = {static_cast<cuuint32_t>(box_inner), static_cast<cuuint32_t>(box_rows), 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(base), dims, strides, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    GB_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed: " + std::to_string(static_cast<int>(r)));
}

void split_rows_f64(const double *src, long long lds, long long rows, int cols, int kpad, const SplitBufs &o,
                    cudaStream_t st)
{
    const long long n = rows * kpad;
    const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 32);
    k_split_rows<double><<<static_cast<unsigned>(blocks), 256, 0, st>>>(src, lds, rows, cols, kpad, o.ns, o.p[0],
                                                                         o.p[1], o.p[2]);
    GB_LAUNCH_CHECK();
}

void split_rows_f32(const float *src, long long lds, long long rows, int cols, int kpad, const SplitBufs &o,
                    cudaStream_t st)
{
    const long long n = rows * kpad;
    const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 32);
    k_split_rows<float><<<static_cast<unsigned>(blocks), 256, 0, st>>>(src, lds, rows, cols, kpad, o.ns, o.p[0],
                                                                       o.p[1], o.p[2]);
    GB_LAUNCH_CHECK();
}

void split_transpose_f64(const double *src, long long lds, int K, int N, int kpad, const SplitBufs &o,
                         cudaStream_t st)
{
    dim3 grid((kpad + 31) / 32, (N + 31) / 32);
    k_split_transpose<double><<<grid, dim3(32, 8), 0, st>>>(src, lds, K, N, kpad, o.ns, o.p[0], o.p[1], o.p[2]);
    GB_LAUNCH_CHECK();
}

template <int NS>
static void launch_tc(const SplitMat &A, const SplitMat &B, int M, int N, int K, int batch, float *D, long long ldd,
                      long long sD, bool accumulate, int *err, cudaStream_t st, const TcGemmOpts &o)
{
    TmapSet maps;
    const int ba = A.batch_stride == 0 ? 1 : batch, bb = B.batch_stride == 0 ? 1 : batch;
    for (int p = 0; p < NS; ++p)
    {
        make_tmap_bf16(&maps.a[p], A.p[p], A.kpad, A.rows, ba, A.kpad, A.batch_stride, BK, BM);
        make_tmap_bf16(&maps.b[p], B.p[p], B.kpad, B.rows, bb, B.kpad, B.batch_stride, BK, BN);
    }
    static PerDeviceOnce attr;
    attr.run([] {
        GB_CUDA(cudaFuncSetAttribute(k_tc_gemm<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg<NS>::SMEM_BYTES));
    });
    const long long ntm = (M + BM - 1) / BM, ntn = (N + BN - 1) / BN;
    GB_REQUIRE(!o.lower_tiles || ntm == ntn, "lower-tile GEMM needs a square tile grid");
    GB_REQUIRE(o.tri >= 0 && o.tri <= 2, "triangular operand mode must be 0, 1 or 2");
    GB_REQUIRE(o.tri_mul == 1 || o.tri_mul == 2, "triangular K multiplier must be 1 or 2");
    GB_REQUIRE(o.tri == 0 || K >= (o.tri == 1 ? o.tri_mul * N : M), "triangular operand shorter than its K range");
    const long long tiles = o.lower_tiles ? ntm * (ntm + 1) / 2 : ntm * ntn;
    dim3 grid(static_cast<unsigned>(tiles), 1, batch);
    k_tc_gemm<NS><<<grid, GEMM_THREADS, Cfg<NS>::SMEM_BYTES, st>>>(maps, M, N, K, D, ldd, sD, accumulate ? 1 : 0,
                                                          A.batch_stride == 0, B.batch_stride == 0, o.tri,
                                                          o.tri_mul, o.lower_tiles ? 1 : 0, err);
    GB_LAUNCH_CHECK();
}

void tc_gemm_set_attributes()
{
    GB_CUDA(cudaFuncSetAttribute(k_tc_gemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg<2>::SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_tc_gemm<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg<3>::SMEM_BYTES));
}

void tc_gemm_split(const SplitMat &A, const SplitMat &B, int M, int N, int K, int batch, float *D, long long ldd,
                   long long sD, bool accumulate, int *err, cudaStream_t st, const TcGemmOpts &o)
{
    GB_REQUIRE(A.ns == B.ns && (A.ns == 2 || A.ns == 3), "split operands must have the same piece count (2 or 3)");
    GB_REQUIRE(K <= A.kpad && K <= B.kpad && A.kpad % BK == 0 && B.kpad % BK == 0, "split operand padding");
    if (A.ns == 2)
        launch_tc<2>(A, B, M, N, K, batch, D, ldd, sD, accumulate, err, st, o);
    else
        launch_tc<3>(A, B, M, N, K, batch, D, ldd, sD, accumulate, err, st, o);
}

// ------------------------------------------------------------------ self-test
double tc_gemm_selftest(int M, int N, int K, int seed, int ns)
{
    cudaStream_t st;
    GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const int kpad = (K + BK - 1) / BK * BK;
    std::vector<double> ha(static_cast<size_t>(M) * K), hb(static_cast<size_t>(K) * N);
    uint64_t x = 0x9E3779B97F4A7C15ull * (seed + 1);
    auto rnd = [&] {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        return (static_cast<double>(x >> 11) / 9007199254740992.0) * 2.0 - 1.0;
    };
    for (auto &v : ha) v = rnd();
    for (auto &v : hb) v = rnd();
    DevBuf<double> a(ha.size()), bm(hb.size()), ref(static_cast<size_t>(M) * N);
    a.upload(ha.data(), ha.size(), st);
    bm.upload(hb.data(), hb.size(), st);
    SplitStore sa(ns, static_cast<size_t>(M) * kpad), sb(ns, static_cast<size_t>(N) * kpad);
    split_rows_f64(a.get(), K, M, K, kpad, sa.bufs(), st);
    split_transpose_f64(bm.get(), N, K, N, kpad, sb.bufs(), st);
    DevBuf<float> d(static_cast<size_t>(M) * N);
    DevBuf<int> err(1);
    err.zero(st);
    tc_gemm_split(sa.mat(M, kpad, 0), sb.mat(N, kpad, 0), M, N, K, 1, d.get(), N, 0, false, err.get(), st);
    launch_dgemm(M, N, K, a.get(), K, 0, bm.get(), N, 0, ref.get(), N, 0, 1, 1.0, 0.0, st);
    std::vector<float> hd(static_cast<size_t>(M) * N);
    std::vector<double> hr(hd.size());
    int herr = 0;
    d.download(hd.data(), hd.size(), st);
    ref.download(hr.data(), hr.size(), st);
    err.download(&herr, 1, st);
    GB_CUDA(cudaStreamSynchronize(st));
    cudaStreamDestroy(st);
    GB_REQUIRE(herr == 0, "tcgen05 GEMM reported wait timeout code " + std::to_string(herr));
    double num = 0.0, den = 0.0;
    for (size_t i = 0; i < hd.size(); ++i)
    {
        num = std::fmax(num, std::fabs(hd[i] - hr[i]));
        den = std::fmax(den, std::fabs(hr[i]));
    }
    return num / den;
}

} // namespace gb
