// Panel solve and trailing update of the real batched Cholesky on the tensor cores, to FP64
// accuracy.  The panel L21 = A21 W^T (W = L11^-1 from k_chol_diag_inv) and the update below are
// the same exact slice products; they differ only in the operands and in the epilogue, which
// writes the panel and subtracts from the trailing matrix (k_ozaki_syrk<TRSM>).
//
// After a panel step the lower trailing matrix needs A22 -= L21 L21^T, with L21 the panel rows
// below the diagonal block (OZAKI_NB = 64 columns).  Each row r of L21 is scaled by 2^-e_r (e_r
// the exponent of the row's largest magnitude, so every scaled value v lies in (-1, 1)) and cut
// into OZAKI_SLICES = 8 integer slices of 7 bits (sign and magnitude digits of |v| 2^56),
//     v = sum_p s_p 2^{-7(p+1)},   s_p in [-127, 127]   (exact in BF16),
// so that
//     (L21 L21^T)[i][j] = 2^{e_i + e_j} sum_{p,q} 2^{-7(p+q+2)} (S_p S_q^T)[i][j].
// One slice product sums 64 terms below 2^14 in magnitude (below 2^20), and the group of
// products with the same d = p + q has at most 8 members (below 2^23): integers below 2^24,
// which the tensor core's FP32 accumulation holds exactly whatever its rounding.  The groups
// d = 0..7 (36 products) are kept; a dropped product is below 2^-56 |v_i| |v_j| per term, so
// the update matches FP64 arithmetic.
//
// The epilogue is integer work: GB300's FP64 pipe issues about two operations per clock per
// SM, so the 8 groups are converted to int32 and combined into the fixed-point value
//     U = sum_d T_d 2^{7(7-d)}   (value = U 2^{e_i + e_j - 63}, |U| < 2^69),
// rounded to W = U / 2^7 in 64 bits (resolution 2^-56 of 2^{e_i + e_j}, below the FP64
// rounding of the entries it updates), turned into a double by integer operations, and one
// FP64 subtraction per element applies it.
//
// Work item of a CTA: a block of 128 trailing columns j (the MMA's M, TMEM lanes) against up
// to OZ_CHUNK blocks of 32 trailing rows i (the MMA's N) with i >= j; per 16-wide K step,
// 8 MMAs (one per column-side slice p, N = 32 (8 - p)) cover the 36 slice products.  The 8 column-side
// slices stay in shared memory; the row-side slices stream through a 2-stage ring, and two
// TMEM accumulators (8 groups x 32 columns each) let the epilogue of one row block overlap
// the MMAs of the next.  Lanes of a warp hold consecutive columns j, so every read-modify-write
// of A[i][j] is a coalesced 256-byte row segment.  Warp 0 issues TMA, warp 1 the MMAs, warps
// 2-17 run the epilogue (each lane reads its A entries before it waits for the MMAs).  Every wait is bounded; a timeout sets the error flag and the CTA
// winds down (later CTAs return at once).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "chol.h"
#include "common.h"
#include "kernels.h"
#include "ozaki_fixed.h"
#include "work_schedule.h"
#include "tc_common.cuh"
#include "tc_gemm.h"

namespace gb {

namespace {

using namespace tc;

constexpr int OM = 128, ON = 32, OK = OZAKI_NB;  // columns j per item, rows i per tile, K
constexpr int SL = OZAKI_SLICES;
static_assert(SL == ozaki::OZ_SLICES, "slice count of the integer arithmetic");
constexpr int OZ_CHUNK = 32;          // row tiles per CTA
constexpr int TILE_A = OM * OK * 2;   // 16 KB per slice
constexpr int TILE_B = ON * OK * 2;   // 4 KB per slice
constexpr int STAGE_B = SL * TILE_B;  // 32 KB per ring stage
constexpr int OZ_SMEM = SL * TILE_A + 2 * STAGE_B + 1024 + 256;
static_assert(OK == 64, "one 128-byte swizzle row per slice row");
static_assert(OZ_SMEM <= 227 * 1024, "shared memory budget");
constexpr int OZ_EPI_WARPS = 16;  // 4 per TMEM lane quadrant, 8 tile columns each
constexpr int EC = ON / (OZ_EPI_WARPS / 4);
static_assert(EC == 8, "the epilogue loads 8 TMEM columns at a time");

constexpr int OZ_THREADS = 32 * (2 + OZ_EPI_WARPS);
constexpr int ACC_COLS = SL * ON;  // 256 TMEM columns per accumulator

struct OzMaps
{
    CUtensorMap a, b;  // the same slice buffer with 128-row and 32-row boxes
};

// One warp per row: row exponent and the 8 integer slices, by integer operations on the FP64 bit
// patterns (the digits of |v| 2^56, v = x 2^-e; subnormal entries count as zero).  Row rl of the
// slab is A[b][row0 + rl][col0 .. col0 + nb) (matrices bstride elements apart, row stride lda);
// its slices go to S[b][p][rl][0..64) with dst_rows rows per slice plane, its exponent to
// E[b * dst_rows + rl].
__global__ void k_ozaki_slice(const double *__restrict__ A, long long bstride, int lda, int row0, int col0, int nb,
                              int R, __nv_bfloat16 *__restrict__ S, int *__restrict__ E, int dst_rows)
{
    const int b = blockIdx.y;
    const int rl = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;  // row inside the slab
    const int lane = threadIdx.x % 32;
    if (rl >= R) return;
    const double *row = A + static_cast<long long>(b) * bstride + static_cast<long long>(row0 + rl) * lda + col0;
    unsigned long long u[2];
    unsigned long long m = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h)
    {
        const int c = lane + 32 * h;
        u[h] = c < nb ? static_cast<unsigned long long>(__double_as_longlong(row[c])) : 0ull;
        m = max(m, u[h] & 0x7FFFFFFFFFFFFFFFull);  // magnitudes order like their bit patterns
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int e = ozaki::row_exponent(m);  // max < 2^e
    const bool nonzero = (m >> 52) != 0;
    const size_t plane = static_cast<size_t>(dst_rows) * OK;
    __nv_bfloat16 *Sb = S + static_cast<size_t>(b) * SL * plane + static_cast<size_t>(rl) * OK;
#pragma unroll
    for (int h = 0; h < 2; ++h)
    {
        const int c = lane + 32 * h;
        int dig[SL];
        ozaki::slice_digits(u[h], e, nonzero, dig);
#pragma unroll
        for (int p = 0; p < SL; ++p) Sb[p * plane + c] = __float2bfloat16_rn(static_cast<float>(dig[p]));
    }
    if (lane == 0) E[static_cast<size_t>(b) * dst_rows + rl] = e;
}

// Work item t -> (column block jm, first row tile, row tile count)
__device__ __forceinline__ bool item_of(int t, int njm, int nti, int &jm, int &ti0, int &cnt)
{
    return sched::ozaki_item(t, njm, nti, OZ_CHUNK, jm, ti0, cnt);
}

// Bounded wait that gives up at once after any earlier timeout of the CTA.
__device__ __forceinline__ bool oz_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int *err, int code)
{
    if (*abort_flag) return false;
    if (mbar_wait(bar, parity)) return true;
    *abort_flag = 1;
    atomicExch(err, code);
    return false;
}

// TRSM = false: trailing update, A[i][j] -= (L21 L21^T)[i][j] for s0 <= j <= i (column side
// = row side = the panel rows, exponents Erow).  TRSM = true: panel product, A[i][k0 + c] =
// (A21 W^T)[i][c] for the OZAKI_NB rows c of W = L11^-1 (column side = W's slices, exponents
// Ecol[b][c], 2 OZAKI_NB per matrix), all rows i >= s0 = k0 + OZAKI_NB.
template <bool TRSM>
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_ozaki_syrk(const __grid_constant__ OzMaps maps, double *__restrict__ Aall, int N, int s0,
                 const int *__restrict__ Erow, const int *__restrict__ Ecol, int k0, int *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    unsigned char *sA = smem, *sB = smem + SL * TILE_A;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sB + 2 * STAGE_B);
    uint64_t *fullA = bars, *fullB = bars + 1, *emptyB = bars + 3, *tfull = bars + 5, *tempty = bars + 7,
             *fin = bars + 9;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 10);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 11);
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int b = blockIdx.y;
    const int R = N - s0;
    const int nti = (R + ON - 1) / ON, njm = TRSM ? 1 : (R + OM - 1) / OM;
    int jm, ti0, cnt;
    if (!item_of(blockIdx.x, njm, nti, jm, ti0, cnt)) return;  // uniform over the CTA
    volatile int *skip_flag = abort_flag + 1;

    if (threadIdx.x == 0)
    {
        mbar_init(fullA, 1);
        for (int s = 0; s < 2; ++s)
        {
            mbar_init(fullB + s, 1);
            mbar_init(emptyB + s, 1);
            mbar_init(tfull + s, 1);
            mbar_init(tempty + s, OZ_EPI_WARPS);
        }
        mbar_init(fin, 1);
        *abort_flag = 0;
        *skip_flag = *reinterpret_cast<volatile int *>(err);  // an earlier CTA timed out: no work
        fence_barrier_init();
    }
    if (warp == 1) tmem_alloc(tmem_slot, 2 * ACC_COLS);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (*skip_flag)
    {
    }
    else if (warp == 0)
    {
        if (lane == 0)
        {
            mbar_arrive_expect_tx(fullA, SL * TILE_A);
            for (int p = 0; p < SL; ++p) tma_load_3d(sA + p * TILE_A, &maps.a, 0, jm * OM, b * SL + p, fullA);
            int issued = 0;
            for (int t = 0; t < cnt; ++t)
            {
                const int s = t & 1;
                if (t >= 2 && !oz_wait(emptyB + s, ((t >> 1) - 1) & 1, abort_flag, err, 311)) break;
                mbar_arrive_expect_tx(fullB + s, STAGE_B);
                for (int q = 0; q < SL; ++q)
                    tma_load_3d(sB + s * STAGE_B + q * TILE_B, &maps.b, 0, (ti0 + t) * ON, b * SL + q, fullB + s);
                issued = t + 1;
            }
            // the copies must land before the CTA exits, also after a timeout
            mbar_wait(fullA, 0);
            for (int t = issued > 2 ? issued - 2 : 0; t < issued; ++t) mbar_wait(fullB + (t & 1), (t >> 1) & 1);
        }
    }
    else if (warp == 1)
    {
        if (lane == 0)
        {
            bool ok = oz_wait(fullA, 0, abort_flag, err, 312);
            tc_fence_after();
            for (int t = 0; ok && t < cnt; ++t)
            {
                const int s = t & 1;
                if (!oz_wait(fullB + s, (t >> 1) & 1, abort_flag, err, 313)) break;
                if (t >= 2 && !oz_wait(tempty + s, ((t >> 1) - 1) & 1, abort_flag, err, 314)) break;
                tc_fence_after();
                // The row-side slices of a stage are stacked (slice q at rows 32 q), so one MMA
                // with N = 32 (8 - p) forms A_p B_q^T for every q <= 7 - p, and writing it at
                // TMEM column 32 p puts each block into its group d = p + q.  The first MMA
                // (p = 0, k = 0) spans all 8 groups and starts them from zero.
                const uint32_t acc = tmem + s * ACC_COLS;
                const uint64_t db = smem_desc_sw128(sB + s * STAGE_B);
#pragma unroll
                for (int k = 0; k < OK / 16; ++k)
                {
                    const uint64_t dk = static_cast<uint64_t>(k * 32 >> 4);
#pragma unroll
                    for (int p = 0; p < SL; ++p)
                        mma_bf16(acc + p * ON, smem_desc_sw128(sA + p * TILE_A) + dk, db + dk,
                                 idesc_bf16_f32(OM, ON * (SL - p)), (p == 0 && k == 0) ? 0u : 1u);
                }
                mma_commit(emptyB + s);
                mma_commit(tfull + s);
            }
            // every issued MMA completes before TMEM is released
            mma_commit(fin);
            mbar_wait(fin, 0);
        }
    }
    else
    {
        const int ew = warp - 2;
        const int quad = warp % 4;  // TMEM lane quadrant this warp may read
        const int part = ew / 4;    // which EC of the 32 tile columns
        const uint32_t lane_base = static_cast<uint32_t>(quad * 32) << 16;
        const int jl = jm * OM + quad * 32 + lane;  // column-side index (trailing column or row c of W)
        // output column and its validity
        const int j = TRSM ? k0 + jl : s0 + jl;
        const bool jok = TRSM ? jl < OZAKI_NB : j < N;
        const int *E = Erow + static_cast<size_t>(b) * N;
        const int ej = jok ? (TRSM ? Ecol[static_cast<size_t>(b) * 2 * OZAKI_NB + jl] : E[jl]) : 0;
        double *Ab = Aall + static_cast<long long>(b) * N * N;
        // the EC entries of A this lane updates in tile t, read one tile ahead
        auto load_a = [&](int t, double (&a)[EC]) {
            const int ib = s0 + (ti0 + t) * ON + part * EC;
#pragma unroll
            for (int c = 0; c < EC; ++c)
            {
                const int i = ib + c;
                a[c] = (!TRSM && i < N && jok && j <= i) ? Ab[static_cast<long long>(i) * N + j] : 0.0;
            }
        };
        double av[EC], an[EC];
        load_a(0, av);
        for (int t = 0; t < cnt; ++t)
        {
            const int s = t & 1;
            const int ib = s0 + (ti0 + t) * ON + part * EC;
            if (t + 1 < cnt) load_a(t + 1, an);
            const bool ok = __all_sync(0xffffffffu, oz_wait(tfull + s, (t >> 1) & 1, abort_flag, err, 315));
            if (!ok) break;
            tc_fence_after();
            const uint32_t acc = tmem + s * ACC_COLS + part * EC + lane_base;
            int U[4][EC];
#pragma unroll
            for (int g = 0; g < 4; ++g)
            {
                uint32_t v0[EC], v1[EC];
                tmem_ld8_nowait(acc + (2 * g) * ON, v0);
                tmem_ld8_nowait(acc + (2 * g + 1) * ON, v1);
                tmem_wait_ld();
#pragma unroll
                for (int c = 0; c < EC; ++c)
                    U[g][c] = __float2int_rn(__uint_as_float(v0[c])) * 128 + __float2int_rn(__uint_as_float(v1[c]));
            }
            // TMEM of this accumulator is free again
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty + s);
            const int ei_own = (ib - s0 + (lane % EC)) < R ? E[ib - s0 + (lane % EC)] : 0;
#pragma unroll
            for (int c = 0; c < EC; ++c)
            {
                const int i = ib + c;
                const int ei = __shfl_sync(0xffffffffu, ei_own, c);
                if (i < N && jok && (TRSM || j <= i))
                {
                    // U = hi 2^28 + lo (value U 2^(e_i + e_j - 63), |U| < 2^69), kept as
                    // W = U / 2^7 rounded: an absolute resolution of 2^-56 of the row scales
                    const long long w = ozaki::combine_groups(U[0][c], U[1][c], U[2][c], U[3][c]);
                    const double v = ozaki::fixed_to_double(w, ei + ej - 56);
                    Ab[static_cast<long long>(i) * N + j] = TRSM ? v : av[c] - v;
                }
            }
#pragma unroll
            for (int c = 0; c < EC; ++c) av[c] = an[c];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, 2 * ACC_COLS);
}

} // namespace

void ozaki_alloc(OzakiWork &w, int N, int batch)
{
    ozaki_free(w);
    GB_CUDA(cudaMalloc(&w.slices, sizeof(__nv_bfloat16) * static_cast<size_t>(batch) * SL * N * OK));
    GB_CUDA(cudaMalloc(&w.expo, sizeof(int) * static_cast<size_t>(batch) * N));
    GB_CUDA(cudaMalloc(&w.err, sizeof(int)));
    GB_CUDA(cudaMemset(w.err, 0, sizeof(int)));
    GB_CUDA(cudaMalloc(&w.winv, sizeof(double) * static_cast<size_t>(batch) * OK * OK));
    const size_t wsl = static_cast<size_t>(batch) * SL * 2 * OK * OK;
    GB_CUDA(cudaMalloc(&w.wslices, sizeof(__nv_bfloat16) * wsl));
    GB_CUDA(cudaMemset(w.wslices, 0, sizeof(__nv_bfloat16) * wsl));  // rows OK..2 OK stay zero
    GB_CUDA(cudaMalloc(&w.wexpo, sizeof(int) * static_cast<size_t>(batch) * 2 * OK));
    GB_CUDA(cudaMemset(w.wexpo, 0, sizeof(int) * static_cast<size_t>(batch) * 2 * OK));
    w.N = N;
    w.batch = batch;
}

void ozaki_free(OzakiWork &w)
{
    if (w.slices) cudaFree(w.slices);
    if (w.expo) cudaFree(w.expo);
    if (w.err) cudaFree(w.err);
    if (w.winv) cudaFree(w.winv);
    if (w.wslices) cudaFree(w.wslices);
    if (w.wexpo) cudaFree(w.wexpo);
    w = OzakiWork{};
}

namespace {
void set_syrk_attributes()
{
    static PerDeviceOnce attr;
    attr.run([] {
        GB_CUDA(cudaFuncSetAttribute(k_ozaki_syrk<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM));
        GB_CUDA(cudaFuncSetAttribute(k_ozaki_syrk<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM));
    });
}
} // namespace

int ozaki_trailing_update(double *A, int N, int batch, int s0, int k0, int nb, OzakiWork &w, cudaStream_t st)
{
    GB_REQUIRE(w.slices && w.N == N && batch <= w.batch, "Ozaki work space does not match the factorisation");
    GB_REQUIRE(nb <= OK, "panel wider than the Ozaki slices");
    const int R = N - s0;
    __nv_bfloat16 *S = static_cast<__nv_bfloat16 *>(w.slices);
    dim3 gs(static_cast<unsigned>((R + 7) / 8), batch);
    k_ozaki_slice<<<gs, 256, 0, st>>>(A, static_cast<long long>(N) * N, N, s0, k0, nb, R, S, w.expo, N);
    GB_LAUNCH_CHECK();
    OzMaps maps;
    // dims {K = 64, rows R, planes batch * 8}; plane stride N * 64 elements
    make_tmap_bf16(&maps.a, S, OK, R, static_cast<long long>(batch) * SL, OK, static_cast<long long>(N) * OK, OK, OM);
    make_tmap_bf16(&maps.b, S, OK, R, static_cast<long long>(batch) * SL, OK, static_cast<long long>(N) * OK, OK, ON);
    set_syrk_attributes();
    const int nti = (R + ON - 1) / ON, njm = (R + OM - 1) / OM;
    const long long items = sched::ozaki_items(njm, nti, OZ_CHUNK);
    dim3 grid(static_cast<unsigned>(items), batch);
    k_ozaki_syrk<false><<<grid, OZ_THREADS, OZ_SMEM, st>>>(maps, A, N, s0, w.expo, w.expo, k0, w.err);
    GB_LAUNCH_CHECK();
    return 2;
}

int ozaki_panel_solve(double *A, int N, int batch, int k0, OzakiWork &w, cudaStream_t st)
{
    GB_REQUIRE(w.slices && w.winv && w.N == N && batch <= w.batch, "Ozaki work space does not match the factorisation");
    const int s0 = k0 + OK;
    const int R = N - s0;
    GB_REQUIRE(R > 0, "panel solve without rows below the diagonal block");
    __nv_bfloat16 *S = static_cast<__nv_bfloat16 *>(w.slices), *SW = static_cast<__nv_bfloat16 *>(w.wslices);
    // rows of W = L11^-1 (64 per matrix, planes of 128 rows whose upper half stays zero)
    k_ozaki_slice<<<dim3(OK / 8, batch), 256, 0, st>>>(w.winv, static_cast<long long>(OK) * OK, OK, 0, 0, OK, OK, SW,
                                                       w.wexpo, 2 * OK);
    GB_LAUNCH_CHECK();
    // rows of A21
    k_ozaki_slice<<<dim3(static_cast<unsigned>((R + 7) / 8), batch), 256, 0, st>>>(
        A, static_cast<long long>(N) * N, N, s0, k0, OK, R, S, w.expo, N);
    GB_LAUNCH_CHECK();
    OzMaps maps;
    make_tmap_bf16(&maps.a, SW, OK, 2 * OK, static_cast<long long>(batch) * SL, OK, 2LL * OK * OK, OK, OM);
    make_tmap_bf16(&maps.b, S, OK, R, static_cast<long long>(batch) * SL, OK, static_cast<long long>(N) * OK, OK, ON);
    set_syrk_attributes();
    const int nti = (R + ON - 1) / ON;
    dim3 grid(static_cast<unsigned>((nti + OZ_CHUNK - 1) / OZ_CHUNK), batch);
    k_ozaki_syrk<true><<<grid, OZ_THREADS, OZ_SMEM, st>>>(maps, A, N, s0, w.expo, w.wexpo, k0, w.err);
    GB_LAUNCH_CHECK();
    return 3;
}

double chol_ozaki_selftest(int N, int batch, int seed, int spread_decades, double shift, double *max_rel_l)
{
    // SPD test matrices A = D (X X^T / N + shift I) D with D = diag(10^u), u uniform in
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
                v = (v + (i == j ? shift : 0.0)) * dsc[i] * dsc[j];
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
