// Trailing update of the real batched Cholesky on the tensor cores, to FP64 accuracy.
//
// After a panel step the lower trailing matrix needs A22 -= L21 L21^T, with L21 the panel rows
// below the diagonal block (OZAKI_NB = 64 columns).  Each row r of L21 is scaled by 2^-e_r (e_r
// from frexp of the row's largest magnitude, so every scaled value v lies in (-1, 1)) and cut
// into OZAKI_SLICES = 8 integer slices of 7 bits,
//     v = sum_p s_p 2^{-7(p+1)},   s_p in [-127, 127]   (exact in BF16),
// so that
//     (L21 L21^T)[i][j] = 2^{e_i + e_j} sum_{p,q} 2^{-7(p+q+2)} (S_p S_q^T)[i][j].
// One slice product sums 64 terms below 2^14 in magnitude (below 2^20), and the group of
// products with the same d = p + q has at most 8 members (below 2^23): integers below 2^24,
// which the tensor core's FP32 accumulation holds exactly whatever its rounding.  The groups
// d = 0..7 (36 products) are kept; a dropped product is below 2^-63 |x_i| |x_j| per term, so
// the update matches FP64 arithmetic.  The epilogue recombines the groups in FP64 and
// subtracts from A22.
//
// One CTA per 128 x 64 tile of the lower trailing matrix: one lane loads the 8 + 8 slice tiles
// with TMA, one lane issues the MMAs into 8 TMEM accumulators (one per group d), four warps
// run the epilogue.  Every wait is bounded and reports a timeout through the error flag.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "chol.h"
#include "common.h"
#include "tc_common.cuh"
#include "kernels.h"
#include "tc_gemm.h"

#include <vector>

namespace gb {

namespace {

using namespace tc;

constexpr int OM = 128, ON = 64, OK = OZAKI_NB;  // tile rows, tile columns, K
constexpr int SL = OZAKI_SLICES;
constexpr int TILE_A = OM * OK * 2;   // 16 KB per slice
constexpr int TILE_B = ON * OK * 2;   // 8 KB per slice
constexpr int OZ_SMEM = SL * (TILE_A + TILE_B) + 1024 + 256;
static_assert(OK == 64, "one 128-byte swizzle row per slice row");
static_assert(OZ_SMEM <= 227 * 1024, "shared memory budget");
constexpr int OZ_THREADS = 192;  // warp 0: TMA, warp 1: MMA, warps 2-5: epilogue

struct OzMaps
{
    CUtensorMap a, b;  // the same slice buffer with 128-row and 64-row boxes
};

// One warp per panel row: row scale and the 8 integer slices.
__global__ void k_ozaki_slice(const double *__restrict__ A, int N, int s0, int k0, int nb,
                              __nv_bfloat16 *__restrict__ S, int *__restrict__ E)
{
    const int b = blockIdx.y;
    const int rl = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;  // row inside the panel
    const int lane = threadIdx.x % 32;
    const int R = N - s0;
    if (rl >= R) return;
    const double *row = A + static_cast<long long>(b) * N * N + static_cast<long long>(s0 + rl) * N + k0;
    double v[2];
    double m = 0.0;
#pragma unroll
    for (int h = 0; h < 2; ++h)
    {
        const int c = lane + 32 * h;
        v[h] = c < nb ? row[c] : 0.0;
        m = fmax(m, fabs(v[h]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    int e = 0;
    if (m > 0.0) frexp(m, &e);  // m = f 2^e, f in [0.5, 1): |v 2^-e| < 1
    const size_t plane = static_cast<size_t>(N) * OK;
    __nv_bfloat16 *Sb = S + static_cast<size_t>(b) * SL * plane + static_cast<size_t>(rl) * OK;
#pragma unroll
    for (int h = 0; h < 2; ++h)
    {
        const int c = lane + 32 * h;
        double t = ldexp(v[h], -e);
#pragma unroll
        for (int p = 0; p < SL; ++p)
        {
            t *= 128.0;
            const double s = trunc(t);
            t -= s;
            Sb[p * plane + c] = __double2bfloat16(s);
        }
    }
    if (lane == 0) E[static_cast<size_t>(b) * N + rl] = e;
}

__device__ __forceinline__ void tile_of(int t, int nrt, int nct, int &ti, int &tj)
{
    // lower tiles: row tile ti (128 rows) meets column tiles tj <= 2 ti + 1 (64 columns)
    for (ti = 0; ti < nrt; ++ti)
    {
        const int cnt = min(2 * ti + 2, nct);
        if (t < cnt)
        {
            tj = t;
            return;
        }
        t -= cnt;
    }
    ti = nrt;  // out of range
    tj = 0;
}

__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_ozaki_syrk(const __grid_constant__ OzMaps maps, double *__restrict__ Aall, int N, int s0,
                 const int *__restrict__ Eall, int *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    unsigned char *sA = smem, *sB = smem + SL * TILE_A;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + SL * (TILE_A + TILE_B));
    uint64_t *done = full + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int b = blockIdx.y;
    const int R = N - s0;
    const int nrt = (R + OM - 1) / OM, nct = (R + ON - 1) / ON;
    int ti, tj;
    tile_of(blockIdx.x, nrt, nct, ti, tj);
    if (ti >= nrt) return;  // uniform over the CTA

    if (threadIdx.x == 0)
    {
        mbar_init(full, 1);
        mbar_init(done, 1);
        fence_barrier_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, SL * ON);  // 8 groups x 64 columns = 512
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    bool ok = true;

    if (warp == 0 && lane == 0)
    {
        mbar_arrive_expect_tx(full, SL * (TILE_A + TILE_B));
#pragma unroll
        for (int p = 0; p < SL; ++p)
        {
            tma_load_3d(sA + p * TILE_A, &maps.a, 0, ti * OM, b * SL + p, full);
            tma_load_3d(sB + p * TILE_B, &maps.b, 0, tj * ON, b * SL + p, full);
        }
        // the copies must land before the CTA may exit, also when the MMA lane gave up
        if (!mbar_wait(full, 0)) atomicExch(err, 303);
    }
    else if (warp == 1 && lane == 0)
    {
        if (!mbar_wait(full, 0))
        {
            atomicExch(err, 301);
        }
        else
        {
            tc_fence_after();
            constexpr uint32_t idesc = idesc_bf16_f32(OM, ON);
            for (int d = 0; d < SL; ++d)
            {
                bool first = true;
                for (int p = 0; p <= d; ++p)
                {
                    const int q = d - p;
                    const uint64_t da = smem_desc_sw128(sA + p * TILE_A), db = smem_desc_sw128(sB + q * TILE_B);
#pragma unroll
                    for (int k = 0; k < OK / 16; ++k)
                    {
                        const uint64_t dk = static_cast<uint64_t>(k * 32 >> 4);
                        mma_bf16(tmem + d * ON, da + dk, db + dk, idesc, first && k == 0 ? 0 : 1);
                    }
                    first = false;
                }
            }
        }
        mma_commit(done);  // arrives once the issued MMAs (if any) are complete
    }
    else if (warp >= 2)
    {
        const int quad = warp % 4;  // TMEM lane quadrant this warp may read
        const uint32_t lane_base = static_cast<uint32_t>(quad * 32) << 16;
        if (!__all_sync(0xffffffffu, mbar_wait(done, 0)))
        {
            if (lane == 0) atomicExch(err, 302);
            ok = false;
        }
        if (ok)
        {
            tc_fence_after();
            const int il = quad * 32 + lane;
            const int i = s0 + ti * OM + il;
            const int *E = Eall + static_cast<size_t>(b) * N;
            const int ei = i < N ? E[i - s0] : 0;
            double *Arow = Aall + static_cast<long long>(b) * N * N + static_cast<long long>(i) * N;
#pragma unroll 1
            for (int c0 = 0; c0 < ON; c0 += 16)
            {
                double acc[16];
#pragma unroll
                for (int c = 0; c < 16; ++c) acc[c] = 0.0;
#pragma unroll 1
                for (int d = 0; d < SL; ++d)
                {
                    uint32_t v[16];
                    tmem_ld16_nowait(tmem + d * ON + c0 + lane_base, v);
                    tmem_wait_ld();
                    const double sc = ldexp(1.0, -7 * (d + 2));
#pragma unroll
                    for (int c = 0; c < 16; ++c) acc[c] += static_cast<double>(__uint_as_float(v[c])) * sc;
                }
                if (i < N)
                {
#pragma unroll
                    for (int c = 0; c < 16; ++c)
                    {
                        const int j = s0 + tj * ON + c0 + c;
                        if (j < N && j <= i) Arow[j] -= ldexp(acc[c], ei + __ldg(E + (j - s0)));
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, SL * ON);
}

} // namespace

void ozaki_alloc(OzakiWork &w, int N, int batch)
{
    ozaki_free(w);
    GB_CUDA(cudaMalloc(&w.slices, sizeof(__nv_bfloat16) * static_cast<size_t>(batch) * SL * N * OK));
    GB_CUDA(cudaMalloc(&w.expo, sizeof(int) * static_cast<size_t>(batch) * N));
    GB_CUDA(cudaMalloc(&w.err, sizeof(int)));
    GB_CUDA(cudaMemset(w.err, 0, sizeof(int)));
    w.N = N;
    w.batch = batch;
}

void ozaki_free(OzakiWork &w)
{
    if (w.slices) cudaFree(w.slices);
    if (w.expo) cudaFree(w.expo);
    if (w.err) cudaFree(w.err);
    w = OzakiWork{};
}

int ozaki_trailing_update(double *A, int N, int batch, int s0, int k0, int nb, OzakiWork &w, cudaStream_t st)
{
    GB_REQUIRE(w.slices && w.N == N && batch <= w.batch, "Ozaki work space does not match the factorisation");
    GB_REQUIRE(nb <= OK, "panel wider than the Ozaki slices");
    const int R = N - s0;
    __nv_bfloat16 *S = static_cast<__nv_bfloat16 *>(w.slices);
    dim3 gs(static_cast<unsigned>((R + 7) / 8), batch);
    k_ozaki_slice<<<gs, 256, 0, st>>>(A, N, s0, k0, nb, S, w.expo);
    GB_LAUNCH_CHECK();
    OzMaps maps;
    // dims {K = 64, rows R, planes batch * 8}; plane stride N * 64 elements
    make_tmap_bf16(&maps.a, S, OK, R, static_cast<long long>(batch) * SL, OK, static_cast<long long>(N) * OK, OK, OM);
    make_tmap_bf16(&maps.b, S, OK, R, static_cast<long long>(batch) * SL, OK, static_cast<long long>(N) * OK, OK, ON);
    static bool attr = false;
    if (!attr)
    {
        GB_CUDA(cudaFuncSetAttribute(k_ozaki_syrk, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM));
        attr = true;
    }
    const int nrt = (R + OM - 1) / OM, nct = (R + ON - 1) / ON;
    long long tiles = 0;
    for (int ti = 0; ti < nrt; ++ti) tiles += std::min(2 * ti + 2, nct);
    dim3 grid(static_cast<unsigned>(tiles), batch);
    k_ozaki_syrk<<<grid, OZ_THREADS, OZ_SMEM, st>>>(maps, A, N, s0, w.expo, w.err);
    GB_LAUNCH_CHECK();
    return 2;
}

double chol_ozaki_selftest(int N, int batch, int seed, int spread_decades, double *max_rel_l)
{
    // SPD test matrices A = D (X X^T / N + 0.05 I) D with D = diag(10^u), u uniform in
    // [-spread/2, spread/2]; factored by the FP64 CUDA-core Cholesky and by the tensor-core
    // variant.  Returns max_b |logdet difference|; *max_rel_l = max |L difference| / max |L|.
    cudaStream_t st;
    GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const size_t nn = static_cast<size_t>(N) * N;
    uint64_t x = 0x9E3779B97F4A7C15ull * (seed + 1);
    auto rnd = [&] {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        return (static_cast<double>(x >> 11) / 9007199254740992.0) * 2.0 - 1.0;
    };
    std::vector<double> hx(nn * batch), hxt(nn * batch), ha(nn * batch);
    for (int b = 0; b < batch; ++b)
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
            {
                const double v = rnd();
                hx[b * nn + static_cast<size_t>(i) * N + j] = v;
                hxt[b * nn + static_cast<size_t>(j) * N + i] = v;
            }
    DevBuf<double> dx(nn * batch), dxt(nn * batch), a1(nn * batch), a2(nn * batch);
    dx.upload(hx.data(), hx.size(), st);
    dxt.upload(hxt.data(), hxt.size(), st);
    launch_dgemm(N, N, N, dx.get(), N, nn, dxt.get(), N, nn, a1.get(), N, nn, batch, 1.0 / N, 0.0, st);
    a1.download(ha.data(), ha.size(), st);
    GB_CUDA(cudaStreamSynchronize(st));
    std::vector<double> dsc(N);
    for (int b = 0; b < batch; ++b)
    {
        for (int i = 0; i < N; ++i) dsc[i] = std::pow(10.0, 0.5 * spread_decades * rnd());
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
            {
                double &v = ha[b * nn + static_cast<size_t>(i) * N + j];
                v = (v + (i == j ? 0.05 : 0.0)) * dsc[i] * dsc[j];
            }
    }
    a1.upload(ha.data(), ha.size(), st);
    a2.upload(ha.data(), ha.size(), st);
    DevBuf<double> d1(static_cast<size_t>(N) * batch), d2(static_cast<size_t>(N) * batch), l1(batch), l2(batch);
    DevBuf<int> bad(batch);
    bad.zero(st);
    OzakiWork w;
    ozaki_alloc(w, N, batch);
    chol_batched_r(a1.get(), N, batch, d1.get(), bad.get(), st);
    chol_batched_r_ozaki(a2.get(), N, batch, d2.get(), bad.get(), w, st);
    chol_logdet(d1.get(), N, batch, l1.get(), st);
    chol_logdet(d2.get(), N, batch, l2.get(), st);
    std::vector<double> h1(nn * batch), h2(nn * batch), g1(batch), g2(batch);
    std::vector<int> hbad(batch);
    int herr = 0;
    a1.download(h1.data(), h1.size(), st);
    a2.download(h2.data(), h2.size(), st);
    l1.download(g1.data(), batch, st);
    l2.download(g2.data(), batch, st);
    bad.download(hbad.data(), batch, st);
    GB_CUDA(cudaMemcpyAsync(&herr, w.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    ozaki_free(w);
    cudaStreamDestroy(st);
    GB_REQUIRE(herr == 0, "Ozaki update reported wait timeout code " + std::to_string(herr));
    for (int b = 0; b < batch; ++b) GB_REQUIRE(hbad[b] == 0, "test matrix not positive definite");
    double num = 0.0, den = 0.0, dl = 0.0;
    for (int b = 0; b < batch; ++b)
    {
        dl = std::fmax(dl, std::fabs(g1[b] - g2[b]));
        for (int i = 0; i < N; ++i)
            for (int j = 0; j <= i; ++j)
            {
                const size_t t = b * nn + static_cast<size_t>(i) * N + j;
                num = std::fmax(num, std::fabs(h1[t] - h2[t]));
                den = std::fmax(den, std::fabs(h1[t]));
            }
    }
    if (max_rel_l) *max_rel_l = num / den;
    return dl;
}

} // namespace gb
