// Tensor-core chi0 path (BF16 split products on tcgen05, FP32 accumulation).
//
// Per (tau, spin), with the algebra of k_chi0_simt.cu:
//  1. X(+-) = C * G_super(+-): one batched split-precision GEMM (k_tc_gemm.cu); the B operand
//     G_super^T is built and split directly from G(R).
//  2. T1 (fused, this file): for each upper atom pair (I, J) and a tile of 128 rows
//     (cell cJ, mu), accumulate in TMEM
//        D[(cJ,mu)][nu] = sum_{pass} sum_{j, K'} E[(cJ,mu)][j, K'] * C^J[nu][j, K']
//        E[(cJ,mu)][j, K'] = sum_i Ga[cJ]_{ij} X_b^I[mu i][shift_cJ(K')]
//     where K' runs over the supercell orbitals (cell R', atom L, orbital l) of C^J's own
//     frame and shift_cJ maps R' -> R' + R_cJ (the T1 term with R_L = R' + R_J).
//     Eight producer warps form E in FP32 on the CUDA cores (packed FP32x2 FMAs, 4 columns a
//     thread), split it into BF16 pieces and
//     write the 128 x 64 A tile of each pipeline stage into swizzled shared memory; one lane
//     streams the matching C^J tile (64 K-elements per row, pre-arranged in HBM) with TMA and
//     one lane issues the tcgen05.mma terms.  K order: pass, 8-column chunk, group of 8 j.
//  3. T2 (small, CUDA cores): D += sum_{i,j} X_b^I[mu i; (cJ,J) j] X_a^J[nu j; (-cJ,I) i].
// Every wait is bounded (tc_common.cuh) and failures surface through a device error flag.
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <cstdlib>
#include <vector>

#include "../../include/librpa_gb300.h"
#include "work_schedule.h"
#include "tc_common.cuh"
#include "tc_gemm.h"

namespace gb {

namespace {

using namespace tc;

constexpr int NS = 3;            // BF16 pieces per operand (hi, mid, lo): 6 MMA terms
constexpr int T1_BM = 128;       // rows (cJ, mu) per CTA
constexpr int CW = 8;            // supercell columns per chunk
constexpr int JG = 8;            // j per pipeline stage (JG * CW = 64 = K per stage)
constexpr int T1_STAGES = 2;     // A (E tile) ring: producers fill one while the MMAs read the other
constexpr int T1_MAXB = 8;       // C^J (B tile) ring: up to 8 stages of TMA look-ahead
constexpr int T1_NMAX = 128;     // max N tile (ABFs of one atom, padded to 16)
// Two producer layouts.  Wide (P2 = false): warps 0-7 build E, 2 threads per row with 4
// columns each; 12 warps, up to 168 registers a thread.  Narrow (P2 = true, the streamed
// 4-column-aligned case): warps 0-15 build E, 4 threads per row with 2 columns each, so twice
// the warps hide the X gather latency; 20 warps, up to 102 registers a thread.  In both, the
// 4 warps after the producers drain the accumulators, and lane 0 of the first of them also
// issues the C^J TMA copies and the MMAs.
template <bool P2>
struct T1Layout
{
    static constexpr int producers = P2 ? 512 : 256;
    static constexpr int drain_warp0 = producers / 32;
    static constexpr int threads = producers + 128;
};
constexpr int A_TILE = T1_BM * 64 * 2;       // bytes per A piece
constexpr int T1_MAXA = 32;                  // max NAOs per atom (G buffer row stride)
constexpr int T1_SMEM_MAX = 227 * 1024;
// Shared memory: T1_STAGES x NS A pieces | nbs x NS B pieces of b_tile bytes | G blocks | barriers.
// b_tile = NT_max * 128 rounded up to 1024; G blocks hold, per pass and cell, rap(RA) rows i
// of gj FP32 entries j.

// A row group: the n_abf(I) rows mu of one chi0 block (pair (I, J), cell cJ).
struct T1Group
{
    int pair, cell;
};

// A tile: up to 128 consecutive rows of the row groups of one atom J (groups ordered by the NAO
// count of I, then by I, then cell), all contracted with the same C^J operand.
struct T1Work
{
    int J;         // atom of the B operand
    int g0;        // first row group
    int r0;        // first row inside that group
    int nrows;     // valid rows (<= 128)
    int nslot;     // row groups the tile touches
    int kc0, kc1;  // chunks [kc0, kc1) of the supercell axis this CTA contracts
    int split;     // 1: one of several K parts of the tile, added atomically to the output
    int ra;        // most NAOs of an I atom among the tile's row groups (the producers' i range)
};

constexpr int T1_MAXSPEC = 8;    // distinct (NAO, ABF) species with their own B maps
constexpr int T1_KPARTS = 4;     // default K parts per tile (each part a CTA, added into chi0(R) atomically)
constexpr int T1_KPARTS_MAX = 8; // largest K-part count the tuner tries

// C^J B-operand maps, one rank-3 map per (species, piece): dims {ktot, nabf, atoms of the species}.
struct T1Maps
{
    CUtensorMap m[T1_MAXSPEC][3];
    long long ktot[T1_MAXSPEC];
};

struct T1Args
{
    Geom g;
    Pairs pr;
    const float *X;          // [2][rows_c][n_sup]: sign 0 = X(+), sign 1 = X(-)
    long long xsign;         // rows_c * n_sup
    const double *G;         // [2][n_c][n_ao][n_ao]
    const int *cadd;         // [n_c*n_c] cadd[a*n_c+b] = cell of R_a + R_b
    const T1Work *work;
    const T1Group *groups;
    const int *spec;           // [n_at] species of each atom
    const int *spec_idx;       // [n_at] index of the atom inside its species
    const int *aJpad;          // NAOs of each atom rounded up to JG
    int nkc;                   // number of CW-wide chunks of the supercell axis
    int b_tile;                // bytes per B piece (1024-aligned)
    int nbs;                   // stages of the B ring (2..T1_MAXB)
    int gj;                    // j entries per i row of the G blocks (largest aJpad)
    int maxcj;                 // most row groups a 128-row tile can touch
    int vec4;                  // n_ao % 4 == 0: 4-column X gathers are one aligned float4
    double *out;               // chi0R
    int *err;
};

__device__ __forceinline__ void named_bar_sync(int id, int n)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

__host__ __device__ constexpr int rap(int ra) { return (ra + 1) & ~1; }

__device__ __forceinline__ uint32_t bf2_bits(__nv_bfloat162 h)
{
    return *reinterpret_cast<const uint32_t *>(&h);
}

// Three-piece BF16 split of a pair of FP32 values (hi, mid, lo), each piece packed as bf16x2
// (element 0 in the low half): hi = rn(e), mid = rn(e - hi), lo = rn(e - hi - mid).
__device__ __forceinline__ void split3_pair(float2 e, uint32_t &h, uint32_t &m, uint32_t &l)
{
    const float2 neg1 = make_float2(-1.0f, -1.0f);
    const __nv_bfloat162 hh = __floats2bfloat162_rn(e.x, e.y);
    const float2 r1 = __ffma2_rn(__bfloat1622float2(hh), neg1, e);
    const __nv_bfloat162 mm = __floats2bfloat162_rn(r1.x, r1.y);
    const float2 r2 = __ffma2_rn(__bfloat1622float2(mm), neg1, r1);
    h = bf2_bits(hh);
    m = bf2_bits(mm);
    l = bf2_bits(__floats2bfloat162_rn(r2.x, r2.y));
}

// RA: register blocking over the NAOs i of atom I (13, 16 or 32: at least the largest NAO
// count); NTC: accumulator columns held by the drain warps (64 or 128).
//
// Both LibRI passes share the B operand C^J, so one A tile carries E(+) + E(-) (pass 0:
// G(+) with X(-), pass 1: G(-) with X(+)) and each K step is contracted once.  With NTC = 64
// the three C^J pieces sit on top of each other along N and each K16 step is three MMAs,
// hi x [Ch;Cm;Cl] (N = 3 NT), mid x [Ch;Cm] (N = 2 NT) and lo x Ch (N = NT), landing in three
// accumulator blocks of orders 1, 2^-8 and 2^-16; with NTC = 128 the six products are issued
// one by one into a hi*hi block and a cross-term block.
template <int RA, int NTC, bool SV, bool P2>
__global__ void __launch_bounds__(T1Layout<P2>::threads, 1) k_t1_tc(const __grid_constant__ T1Args a,
                                                                   const __grid_constant__ T1Maps maps)
{
    constexpr int PRODUCERS = T1Layout<P2>::producers;
    constexpr int DRAIN_WARP0 = T1Layout<P2>::drain_warp0;
    constexpr bool STACKN = NTC == 64;
    constexpr int NBLK = STACKN ? 3 : 2;           // accumulator blocks per buffer
    constexpr uint32_t TMEM_COLS = 512;
    static_assert(2 * NBLK * NTC <= static_cast<int>(TMEM_COLS), "TMEM budget");
    constexpr int RP = rap(RA);
    constexpr bool BOTHX = RA <= 13;  // keep both passes' X values of a chunk in registers
    // SV: 4-column X gathers are aligned (n_ao % 4 == 0), so the producers stream X through a
    // register ring, one chunk (both stages, up to 16 j) per pass; otherwise the gathers go one
    // column at a time below
    constexpr bool STREAM = SV && RA <= 16 && JG == 8;
    static_assert(!P2 || STREAM, "the narrow producer layout streams 4-column-aligned X");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int stage_bytes = NS * A_TILE;      // A ring stage
    const int bstage_bytes = NS * a.b_tile;   // B ring stage
    const int nbs = a.nbs;
    const int gst = a.gj;                     // j entries per i row of a G block
    const int g_floats = 2 * a.maxcj * RP * gst;
    unsigned char *bring = smem + T1_STAGES * stage_bytes;
    float *gsm = reinterpret_cast<float *>(bring + nbs * bstage_bytes);
    uint64_t *full = reinterpret_cast<uint64_t *>(gsm + g_floats);  // A ring: producers filled
    uint64_t *empty = full + T1_STAGES;                              // A ring: MMAs done
    uint64_t *bfull = empty + T1_STAGES;                             // B ring: TMA landed
    uint64_t *bempty = bfull + T1_MAXB;                              // B ring: MMAs done
    uint64_t *accf = bempty + T1_MAXB;
    uint64_t *acce = accf + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acce + 2);

    const Geom &g = a.g;
    const T1Work w = a.work[blockIdx.x];
    const int J = w.J;
    const int aJ = g.nao[J], bJ = g.nabf[J];
    const int njg = a.aJpad[J] / JG;
    const int NT = (bJ + 15) / 16 * 16;
    const int nc = g.n_c, nao = g.n_ao;
    const long long nsup = g.n_sup;
    // row r of the tile -> (row group, mu); false beyond the tile's valid rows
    auto row_of = [&](int r, int &grp, int &mu) -> bool {
        if (r >= w.nrows) return false;
        int off = w.r0 + r, gi = w.g0;
        for (int k = 0; k < w.nslot; ++k, ++gi)
        {
            const int b = g.nabf[a.pr.I[a.groups[gi].pair]];
            if (off < b)
            {
                grp = gi;
                mu = off;
                return true;
            }
            off -= b;
        }
        return false;
    };
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int kc0 = w.kc0, kc1 = w.kc1;
    const int total_stages = (kc1 - kc0) * njg;

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < T1_STAGES; ++s)
        {
            mbar_init(&full[s], PRODUCERS / 32);  // one arrival per producer warp
            mbar_init(&empty[s], 1);
        }
        for (int s = 0; s < nbs; ++s)
        {
            mbar_init(&bfull[s], 1);
            mbar_init(&bempty[s], 1);
        }
        for (int i = 0; i < 2; ++i)
        {
            mbar_init(&accf[i], 1);
            mbar_init(&acce[i], 4);               // one arrival per drain warp
        }
        fence_barrier_init();
    }
    if (warp == 0) tmem_alloc(tmem_slot, TMEM_COLS);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (threadIdx.x < PRODUCERS)
    {
        // ---------------- producers: E tiles
        const int t = threadIdx.x;
        const int r = P2 ? t >> 2 : t >> 1;  // row in tile
        const int cq = P2 ? t & 3 : t & 1;   // 2- (narrow) or 4-column (wide) group inside the 8-column chunk
        int grp = 0, mu = 0;
        const bool valid = row_of(r, grp, mu);
        const int slot = valid ? grp - w.g0 : 0;
        const int I = a.pr.I[a.groups[valid ? grp : w.g0].pair];
        const int cJ = valid ? a.groups[grp].cell : 0;
        const int aI = g.nao[I];
        const long long xrow = g.rowc_off[I] + static_cast<long long>(mu) * aI;
        // G blocks of both passes for the tile's row groups, [pass][slot][i][j] in FP32
        const int per_pass = w.nslot * RP * gst;
        for (int e = t; e < 2 * per_pass; e += PRODUCERS)
        {
            const int pass = e / per_pass, rem = e % per_pass;
            const int sl = rem / (RP * gst), ij = rem % (RP * gst);
            const int i = ij / gst, j = ij % gst;
            const T1Group gr = a.groups[w.g0 + sl];
            const int Ig = a.pr.I[gr.pair];
            float v = 0.0f;
            if (i < g.nao[Ig] && j < aJ)
                v = static_cast<float>(a.G[((static_cast<size_t>(pass) * nc + gr.cell) * nao + g.ao_off[Ig] + i) * nao +
                                           g.ao_off[J] + j]);
            gsm[(static_cast<size_t>(pass) * a.maxcj + sl) * RP * gst + ij] = v;
        }
        named_bar_sync(1, PRODUCERS);
        const float4 *gp[2];
#pragma unroll
        for (int pass = 0; pass < 2; ++pass)
            gp[pass] = reinterpret_cast<const float4 *>(gsm) + (static_cast<size_t>(pass) * a.maxcj + slot) * RP * gst / 4;
        const float *Xp[2] = {a.X + a.xsign, a.X};  // pass 0 contracts G(+) with X(-), pass 1 G(-) with X(+)
        // X_b^I[mu i][shift_cJ(col)] for the thread's 4 columns of chunk kc (np passes from pass p0)
        // The tile's i range: row groups of one NAO count share tiles, so on a tile of small
        // atoms the loops over i stop at its own count (a CTA-uniform branch), not at RA.
        const int ira = w.ra;
        auto load_x = [&](int kc, int p0, int np, float4 (&x0)[RA], float4 (&x1)[BOTHX ? RA : 1]) {
            const long long col0 = static_cast<long long>(kc) * CW + cq * 4;
            if (a.vec4)
            {
                long long src = -1;
                if (col0 < nsup && valid)
                {
                    const int cp = static_cast<int>(col0 / nao), ao = static_cast<int>(col0 % nao);
                    src = static_cast<long long>(a.cadd[cp * nc + cJ]) * nao + ao;
                }
                const float *b0 = Xp[p0] + xrow * nsup + src;
#pragma unroll
                for (int i = 0; i < RA; ++i)
                    if (i < ira) x0[i] = (i < aI && src >= 0) ? __ldg(reinterpret_cast<const float4 *>(b0 + i * nsup))
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
                if constexpr (BOTHX)
                    if (np == 2)
                    {
                        const float *b1 = Xp[p0 + 1] + xrow * nsup + src;
#pragma unroll
                        for (int i = 0; i < RA; ++i)
                            if (i < ira) x1[i] = (i < aI && src >= 0) ? __ldg(reinterpret_cast<const float4 *>(b1 + i * nsup))
                                                         : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
            }
            else
            {
                long long src[4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                {
                    const long long col = col0 + q;
                    src[q] = -1;
                    if (col < nsup && valid)
                    {
                        const int cp = static_cast<int>(col / nao), ao = static_cast<int>(col % nao);
                        src[q] = static_cast<long long>(a.cadd[cp * nc + cJ]) * nao + ao;
                    }
                }
                auto gather = [&](const float *Xb, float4(&x)[RA]) {
#pragma unroll
                    for (int i = 0; i < RA; ++i)
                    {
                        if (i >= ira) continue;
                        const float *xr = Xb + (xrow + i) * nsup;
                        const bool ri = i < aI;
                        x[i] = make_float4(ri && src[0] >= 0 ? xr[src[0]] : 0.f, ri && src[1] >= 0 ? xr[src[1]] : 0.f,
                                           ri && src[2] >= 0 ? xr[src[2]] : 0.f, ri && src[3] >= 0 ? xr[src[3]] : 0.f);
                    }
                };
                gather(Xp[p0], x0);
                if constexpr (BOTHX)
                    if (np == 2) gather(Xp[p0 + 1], x1);
            }
        };
        // E[j][col pair] += sum_i g_ij x_i for JH consecutive j from j0
        constexpr int JH = JG / 2;
        auto contract = [&](const float4 *gb, int j0, const float4 (&x)[RA], float2 (&e)[JH][2]) {
#pragma unroll
            for (int i = 0; i < RA; ++i)
            {
                if (i >= ira) continue;
                // one 16-byte load gives g_ij for the JH = 4 values of j; each is paired {g, g}
                // in registers as the broadcast operand of the packed FMAs
                static_assert(JH == 4, "one float4 of G per (i, half stage)");
                const float4 gg = gb[(i * gst + j0) / 4];
                const float2 xa = make_float2(x[i].x, x[i].y), xb = make_float2(x[i].z, x[i].w);
                const float gv[4] = {gg.x, gg.y, gg.z, gg.w};
#pragma unroll
                for (int q = 0; q < 4; ++q)
                {
                    const float2 gq = make_float2(gv[q], gv[q]);
                    e[q][0] = __ffma2_rn(gq, xa, e[q][0]);
                    e[q][1] = __ffma2_rn(gq, xb, e[q][1]);
                }
            }
        };
        bool ok = true;
        int st_count = 0;
        // split E into 3 BF16 pieces and store the 4 x 8 values (jl, column) of j group jh
        auto store_e = [&](unsigned char *stg, int jh, const float2 (&e)[JH][2]) {
#pragma unroll
            for (int jl = 0; jl < JH; ++jl)
            {
                uint32_t h01, m01, l01, h23, m23, l23;
                split3_pair(e[jl][0], h01, m01, l01);
                split3_pair(e[jl][1], h23, m23, l23);
                const uint32_t off = sw128_offset(r, (jh * JH + jl) * CW + cq * 4);
                *reinterpret_cast<uint2 *>(stg + off) = make_uint2(h01, h23);
                *reinterpret_cast<uint2 *>(stg + A_TILE + off) = make_uint2(m01, m23);
                *reinterpret_cast<uint2 *>(stg + 2 * A_TILE + off) = make_uint2(l01, l23);
            }
        };
        if constexpr (P2)
        {
            // Narrow layout: 2 columns a thread (float2 gathers, one packed FMA per (i, j)).  The
            // chunk's 2 RA rows (pass, i) are read in the flat order q = pass RA + i, each XD steps
            // before its use from an XD-entry register ring; the last XD reads of a chunk fetch the
            // first rows of the next one.  The order is padded to QP, a multiple of XD, so that
            // row q of every chunk sits in ring slot q mod XD.
            constexpr int XD = 8;
            constexpr int QP = (2 * RA + XD - 1) / XD * XD;
            static_assert(XD <= 2 * RA, "ring deeper than a chunk");
            const float2 zero2 = make_float2(0.f, 0.f);
            auto chunk_base = [&](int kc, const float *&b0, const float *&b1) -> bool {
                const long long col0 = static_cast<long long>(kc) * CW + cq * 2;
                if (kc >= kc1 || col0 >= nsup || !valid) return false;
                const int cp = static_cast<int>(col0 / nao), ao = static_cast<int>(col0 % nao);
                const long long src = static_cast<long long>(a.cadd[cp * nc + cJ]) * nao + ao;
                b0 = Xp[0] + xrow * nsup + src;
                b1 = Xp[1] + xrow * nsup + src;
                return true;
            };
            auto ld = [&](const float *b0, const float *b1, int q, bool live) -> float2 {
                const int i = q % RA;
                const float *b = q < RA ? b0 : b1;
                return (live && q < 2 * RA && i < aI) ? __ldg(reinterpret_cast<const float2 *>(b + i * nsup)) : zero2;
            };
            const float *c0 = Xp[0], *c1 = Xp[0], *n0 = Xp[0], *n1 = Xp[0];
            bool clive = chunk_base(kc0, c0, c1);
            bool nlive = chunk_base(kc0 + 1, n0, n1);
            float2 xb[XD];
#pragma unroll
            for (int q = 0; q < XD; ++q) xb[q] = ld(c0, c1, q, clive);
            for (int kc = kc0; kc < kc1 && ok; ++kc)
            {
                float2 e[4][JH];  // [group of 4 j][jl]: j 0..15, the thread's 2 columns
#pragma unroll
                for (int jh = 0; jh < 4; ++jh)
#pragma unroll
                    for (int jl = 0; jl < JH; ++jl) e[jh][jl] = zero2;
#pragma unroll
                for (int q = 0; q < QP; ++q)
                {
                    const int pass = q / RA, i = q % RA;
                    const float2 x = xb[q % XD];
                    xb[q % XD] = q + XD < QP ? ld(c0, c1, q + XD, clive) : ld(n0, n1, q + XD - QP, nlive);
                    if (q >= 2 * RA) continue;  // padding of the read order
#pragma unroll
                    for (int jh = 0; jh < 4; ++jh)
                    {
                        const float4 gg = gp[pass][(i * gst + jh * JH) / 4];
                        const float gv[4] = {gg.x, gg.y, gg.z, gg.w};
#pragma unroll
                        for (int qq = 0; qq < 4; ++qq)
                        {
                            if (RA == 13 && 4 * jh + qq >= 13) continue;
                            e[jh][qq] = __ffma2_rn(make_float2(gv[qq], gv[qq]), x, e[jh][qq]);
                        }
                    }
                }
                c0 = n0;
                c1 = n1;
                clive = nlive;
                nlive = chunk_base(kc + 2, n0, n1);
#pragma unroll
                for (int jg = 0; jg < 2; ++jg)
                {
                    if (jg >= njg || !ok) break;
                    const int s = st_count % T1_STAGES, rr = st_count / T1_STAGES;
                    ++st_count;
                    unsigned char *stg = smem + s * stage_bytes;
                    if (!__all_sync(0xffffffffu, mbar_wait(&empty[s], (rr & 1) ^ 1)))
                    {
                        if (lane == 0) atomicExch(a.err, 201);
                        ok = false;
                        break;
                    }
#pragma unroll
                    for (int jh = 0; jh < 2; ++jh)
#pragma unroll
                        for (int jl = 0; jl < JH; ++jl)
                        {
                            uint32_t h, m, l;
                            split3_pair(e[2 * jg + jh][jl], h, m, l);
                            const uint32_t off = sw128_offset(r, (jh * JH + jl) * CW + cq * 2);
                            *reinterpret_cast<uint32_t *>(stg + off) = h;
                            *reinterpret_cast<uint32_t *>(stg + A_TILE + off) = m;
                            *reinterpret_cast<uint32_t *>(stg + 2 * A_TILE + off) = l;
                        }
                    fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&full[s]);
                }
            }
        }
        else if constexpr (STREAM)
        {
            // One chunk (both stages, all 16 j) per pass over its 2 RA rows (pass, i) of X.
            // Row (pass, i) of chunk kc sits in xb[i] from RA steps before its use: reading
            // pass 0 row i refills xb[i] with pass 1 row i, reading pass 1 row i refills it
            // with pass 0 row i of chunk kc + 1, so the gathers stay half a chunk ahead.
            const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
            auto chunk_base = [&](int kc, const float *&b0, const float *&b1) -> bool {
                const long long col0 = static_cast<long long>(kc) * CW + cq * 4;
                if (kc >= kc1 || col0 >= nsup || !valid) return false;
                const int cp = static_cast<int>(col0 / nao), ao = static_cast<int>(col0 % nao);
                const long long src = static_cast<long long>(a.cadd[cp * nc + cJ]) * nao + ao;
                b0 = Xp[0] + xrow * nsup + src;
                b1 = Xp[1] + xrow * nsup + src;
                return true;
            };
            auto ld = [&](const float *b, int i, bool live) -> float4 {
                return (live && i < aI) ? __ldg(reinterpret_cast<const float4 *>(b + i * nsup)) : zero4;
            };
            const float *c0 = Xp[0], *c1 = Xp[0], *n0 = Xp[0], *n1 = Xp[0];
            bool clive = chunk_base(kc0, c0, c1);
            bool nlive = chunk_base(kc0 + 1, n0, n1);
            float4 xb[RA];
#pragma unroll
            for (int i = 0; i < RA; ++i) xb[i] = ld(c0, i, clive);
            for (int kc = kc0; kc < kc1 && ok; ++kc)
            {
                float2 e[4][JH][2];  // [group of 4 j][jl][column pair]: j 0..15
#pragma unroll
                for (int jh = 0; jh < 4; ++jh)
#pragma unroll
                    for (int jl = 0; jl < JH; ++jl) e[jh][jl][0] = e[jh][jl][1] = make_float2(0.f, 0.f);
#pragma unroll
                for (int pass = 0; pass < 2; ++pass)
                {
#pragma unroll
                    for (int i = 0; i < RA; ++i)
                    {
                        const float4 x = xb[i];
                        xb[i] = pass == 0 ? ld(c1, i, clive) : ld(n0, i, nlive);
                        const float2 xa = make_float2(x.x, x.y), xc = make_float2(x.z, x.w);
#pragma unroll
                        for (int jh = 0; jh < 4; ++jh)
                        {
                            const float4 gg = gp[pass][(i * gst + jh * JH) / 4];
                            const float gv[4] = {gg.x, gg.y, gg.z, gg.w};
#pragma unroll
                            for (int q = 0; q < 4; ++q)
                            {
                                // RA = 13: no atom has more than 13 NAOs, j = 13..15 stay zero
                                if (RA == 13 && 4 * jh + q >= 13) continue;
                                const float2 gq = make_float2(gv[q], gv[q]);
                                e[jh][q][0] = __ffma2_rn(gq, xa, e[jh][q][0]);
                                e[jh][q][1] = __ffma2_rn(gq, xc, e[jh][q][1]);
                            }
                        }
                    }
                }
                c0 = n0;
                c1 = n1;
                clive = nlive;
                nlive = chunk_base(kc + 2, n0, n1);
                // stage (kc, jg) holds j [8 jg, 8 jg + 8): the groups of 4 j are 2 jg and 2 jg + 1
#pragma unroll
                for (int jg = 0; jg < 2; ++jg)
                {
                    if (jg >= njg || !ok) break;
                    const int s = st_count % T1_STAGES, rr = st_count / T1_STAGES;
                    ++st_count;
                    unsigned char *stg = smem + s * stage_bytes;
                    if (!__all_sync(0xffffffffu, mbar_wait(&empty[s], (rr & 1) ^ 1)))
                    {
                        if (lane == 0) atomicExch(a.err, 201);
                        ok = false;
                        break;
                    }
                    store_e(stg, 0, e[2 * jg]);
                    store_e(stg, 1, e[2 * jg + 1]);
                    fence_proxy_async_smem();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&full[s]);
                }
            }
        }
        else
        {
        float4 x0[RA], x1[BOTHX ? RA : 1];
        for (int kc = kc0; kc < kc1 && ok; ++kc)
        {
            if constexpr (BOTHX) load_x(kc, 0, 2, x0, x1);
            for (int jg = 0; jg < njg; ++jg, ++st_count)
            {
                const int s = st_count % T1_STAGES, rr = st_count / T1_STAGES;
                unsigned char *stg = smem + s * stage_bytes;
#pragma unroll 1
                for (int h = 0; h < 2; ++h)
                {
                    const int j0 = jg * JG + h * JH;
                    float2 e[JH][2];
#pragma unroll
                    for (int jl = 0; jl < JH; ++jl) e[jl][0] = e[jl][1] = make_float2(0.f, 0.f);
                    if constexpr (BOTHX)
                    {
                        contract(gp[0], j0, x0, e);
                        contract(gp[1], j0, x1, e);
                    }
                    else
                    {
                        load_x(kc, 0, 1, x0, x1);
                        contract(gp[0], j0, x0, e);
                        load_x(kc, 1, 1, x0, x1);
                        contract(gp[1], j0, x0, e);
                    }
                    if (h == 0)
                    {
                        // warp-uniform outcome: the warp arrives on full[s] as one
                        if (!__all_sync(0xffffffffu, mbar_wait(&empty[s], (rr & 1) ^ 1)))
                        {
                            if (lane == 0) atomicExch(a.err, 201);
                            ok = false;
                            break;
                        }
                    }
#pragma unroll
                    for (int jl = 0; jl < JH; ++jl)
                    {
                        uint32_t h01, m01, l01, h23, m23, l23;
                        split3_pair(e[jl][0], h01, m01, l01);
                        split3_pair(e[jl][1], h23, m23, l23);
                        const uint32_t off = sw128_offset(r, (h * JH + jl) * CW + cq * 4);
                        *reinterpret_cast<uint2 *>(stg + off) = make_uint2(h01, h23);
                        *reinterpret_cast<uint2 *>(stg + A_TILE + off) = make_uint2(m01, m23);
                        *reinterpret_cast<uint2 *>(stg + 2 * A_TILE + off) = make_uint2(l01, l23);
                    }
                }
                if (!ok) break;
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[s]);
            }
        }
    }
        }
    else
    {
        // ---------------- drain warps: per-stage accumulator blocks -> FP32 registers -> chi0R.
        // Lane 0 of warp 8 issues, per stage st, the MMAs of st and then the C^J TMA copy of
        // st + nbs - 1 (nbs - 1 stages of look-ahead hide the HBM latency of the B tiles),
        // before its warp drains st - 1: the tensor pipe always holds the next stage.
        const int wq = warp - DRAIN_WARP0;
        const bool ctrl = wq == 0 && lane == 0;
        const uint32_t lane_base = static_cast<uint32_t>(wq * 32) << 16;
        const uint32_t bbytes = static_cast<uint32_t>(NT) * 64 * 2;  // one piece of a B tile
        const int sp = a.spec[J], zj = a.spec_idx[J];
        const long long ktot = maps.ktot[sp];
        // C^J tiles stream through L2 once per tile: evict them first, keep the X^I rows
        const uint64_t pol_b = l2_policy_evict_first();
        auto issue_tma = [&](int st) -> bool {
            const int s = st % nbs, rr = st / nbs;
            if (!mbar_wait(&bempty[s], (rr & 1) ^ 1))
            {
                atomicExch(a.err, 202);
                return false;
            }
            const int x = (kc0 * njg + st) * 64;  // K offset (kc * njg + jg) * 64
            if (x < 0 || static_cast<long long>(x) + 64 > ktot || (x & 7) != 0)
            {
                atomicExch(a.err, 205);  // coordinate outside the C^J operand: skip the copy
                return false;
            }
            unsigned char *bst = bring + s * bstage_bytes;
            mbar_arrive_expect_tx(&bfull[s], NS * bbytes);
#pragma unroll
            for (int p = 0; p < NS; ++p)  // pieces stacked along N: rows [p NT, (p + 1) NT)
                tma_load_3d_hint(bst + p * bbytes, &maps.m[sp][p], x, 0, zj, &bfull[s], pol_b);
            return true;
        };
        auto issue_mma = [&](int st) -> bool {
            const int s = st % T1_STAGES, rr = st / T1_STAGES;
            const int sb = st % nbs, rb = st / nbs;
            const int ab = st & 1;
            if (!mbar_wait(&full[s], rr & 1) || !mbar_wait(&bfull[sb], rb & 1) ||
                !mbar_wait(&acce[ab], ((st >> 1) & 1) ^ 1))
            {
                atomicExch(a.err, 203);
                return false;
            }
            tc_fence_after();
            unsigned char *stg = smem + s * stage_bytes;
            unsigned char *bst = bring + sb * bstage_bytes;
            const uint32_t tb = tmem + static_cast<uint32_t>(ab * NBLK * NTC);
            uint64_t da[NS], db[NS];
#pragma unroll
            for (int p = 0; p < NS; ++p)
            {
                da[p] = smem_desc_sw128(stg + p * A_TILE);
                db[p] = smem_desc_sw128(bst + p * bbytes);
            }
            if constexpr (STACKN)
            {
                const uint32_t i3 = idesc_bf16_f32(T1_BM, 3 * NT), i2 = idesc_bf16_f32(T1_BM, 2 * NT),
                               i1 = idesc_bf16_f32(T1_BM, NT);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                {
                    const uint64_t dk = static_cast<uint64_t>(k * 32 >> 4);
                    mma_bf16(tb, da[0] + dk, db[0] + dk, i3, k != 0);                       // hi x [Ch;Cm;Cl]
                    mma_bf16(tb + NT, da[1] + dk, db[0] + dk, i2, 1);                       // mid x [Ch;Cm]
                    mma_bf16(tb + 2 * NT, da[2] + dk, db[0] + dk, i1, 1);                   // lo x Ch
                }
            }
            else
            {
                const uint32_t idesc = idesc_bf16_f32(T1_BM, NT);
                const uint32_t t_hh = tb, t_x = tb + NTC;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                {
                    const uint64_t dk = static_cast<uint64_t>(k * 32 >> 4);
                    // cross terms (smallest first) into t_x, hi*hi into t_hh; both restart each stage
                    mma_bf16(t_x, da[2] + dk, db[0] + dk, idesc, k != 0);
                    mma_bf16(t_x, da[0] + dk, db[2] + dk, idesc, 1);
                    mma_bf16(t_x, da[1] + dk, db[1] + dk, idesc, 1);
                    mma_bf16(t_x, da[1] + dk, db[0] + dk, idesc, 1);
                    mma_bf16(t_x, da[0] + dk, db[1] + dk, idesc, 1);
                    mma_bf16(t_hh, da[0] + dk, db[0] + dk, idesc, k != 0);
                }
            }
            mma_commit(&empty[s]);
            mma_commit(&bempty[sb]);
            mma_commit(&accf[ab]);
            return true;
        };
        float acc[NTC];
#pragma unroll
        for (int c = 0; c < NTC; ++c) acc[c] = 0.0f;
        bool ok = true;
        int issued = 0, copied = 0;  // MMA stages and B-tile copies issued (control lane)
        if (ctrl)
            for (int st = 0; st < nbs - 1 && st < total_stages && ok; ++st)
                if ((ok = issue_tma(st))) ++copied;
        for (int st = 0; st <= total_stages; ++st)
        {
            if (wq == 0)
            {
                if (ctrl && ok && st < total_stages)
                {
                    ok = issue_mma(st);
                    if (ok) ++issued;
                    if (ok && st + nbs - 1 < total_stages)
                        if ((ok = issue_tma(st + nbs - 1))) ++copied;
                }
                ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            }
            if (!ok) break;
            if (st == 0) continue;
            const int sd = st - 1, ab = sd & 1;
            if (!__all_sync(0xffffffffu, mbar_wait(&accf[ab], (sd >> 1) & 1)))
            {
                if (lane == 0) atomicExch(a.err, 204);
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t tb = tmem + static_cast<uint32_t>(ab * NBLK * NTC) + lane_base;
#pragma unroll
            for (int c0 = 0; c0 < NTC; c0 += 16)
            {
                if (c0 < NT)
                {
                    if constexpr (STACKN && P2)
                    {
                        // narrow layout (96 registers a thread): one block of 16 loaded values live
                        // at a time, added into the running sums from the leading block down
#pragma unroll
                        for (int b = 0; b < 3; ++b)
                        {
                            uint32_t v[16];
                            tmem_ld16_nowait(tb + b * NT + c0, v);
                            tmem_wait_ld();
#pragma unroll
                            for (int i = 0; i < 16; ++i) acc[c0 + i] += __uint_as_float(v[i]);
                        }
                    }
                    else if constexpr (STACKN)
                    {
                        uint32_t v0[16], v1[16], v2[16];
                        tmem_ld16_nowait(tb + c0, v0);
                        tmem_ld16_nowait(tb + NT + c0, v1);
                        tmem_ld16_nowait(tb + 2 * NT + c0, v2);
                        tmem_wait_ld();
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            acc[c0 + i] += __uint_as_float(v0[i]) + (__uint_as_float(v1[i]) + __uint_as_float(v2[i]));
                    }
                    else
                    {
                        uint32_t vx[16], vh[16];
                        tmem_ld16_nowait(tb + NTC + c0, vx);
                        tmem_ld16_nowait(tb + c0, vh);
                        tmem_wait_ld();
#pragma unroll
                        for (int i = 0; i < 16; ++i) acc[c0 + i] += __uint_as_float(vx[i]);
#pragma unroll
                        for (int i = 0; i < 16; ++i) acc[c0 + i] += __uint_as_float(vh[i]);
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[ab]);
        }
        if (ctrl && !ok && issued > 0)
        {
            // error path: let this CTA's issued MMAs finish before its TMEM is released
            const int last = issued - 1;
            mbar_wait(&empty[last % T1_STAGES], (last / T1_STAGES) & 1);
        }
        if (ctrl && !ok)
            for (int st = issued; st < copied; ++st)  // and its B copies land before the CTA exits
                mbar_wait(&bfull[st % nbs], (st / nbs) & 1);
        int grp = 0, mu = 0;
        if (ok && row_of(wq * 32 + lane, grp, mu))
        {
            const T1Group gr = a.groups[grp];
            const int bI = g.nabf[a.pr.I[gr.pair]];
            double *orow = a.out + a.pr.r_off[gr.pair] + (static_cast<long long>(gr.cell) * bI + mu) * bJ;
#pragma unroll
            for (int c = 0; c < NTC; ++c)
                if (c < bJ)
                {
                    if (w.split)
                        atomicAdd(orow + c, static_cast<double>(acc[c]));
                    else
                        orow[c] = static_cast<double>(acc[c]);
                }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TMEM_COLS);
}

// T2 for one (pair, cJ) and one 64 x 64 tile of its (mu, nu) block:
//   out[mu][nu] += sum_pass sum_{i,j} Xb^I[mu i; (cJ,J) j] * Xa^J[nu j; (-cJ,I) i].
// Grid: x = (pair, cJ) group, y = output tile (T2_TILES x T2_TILES of them; CTAs beyond the
// pair's own block return at once), so that a Gamma-only cell, with one group per pair, still
// spreads over the SMs.  Per pass and chunk of i, the two operands are staged K-major in
// shared memory (K = (i, j)): S1[k][mu] and S2[k][nu]; each of the 256 threads accumulates a
// 4 x 4 block of (mu, nu) with two 16-byte shared loads per 16 FMAs.  Tiles are disjoint and the
// CTA sums both passes before its one add, so the result does not depend on CTA order.
constexpr int T2_THREADS = 256;
constexpr int T2_TILE = 64;
constexpr int T2_TILES = T1_NMAX / T2_TILE;  // per dimension: up to 128 ABFs per atom
constexpr int T2_SMEM_FLOATS = 12288;        // 48 KB

__global__ void __launch_bounds__(T2_THREADS) k_t2(const float *__restrict__ X, long long xsign, Geom g, Pairs pr,
                                                  const T1Group *__restrict__ groups, double *__restrict__ out)
{
    __shared__ __align__(16) float sm[T2_SMEM_FLOATS];
    const int p = groups[blockIdx.x].pair, cJ = groups[blockIdx.x].cell;
    const int I = pr.I[p], J = pr.J[p];
    const int aI = g.nao[I], aJ = g.nao[J], bI = g.nabf[I], bJ = g.nabf[J];
    const int mt0 = static_cast<int>(blockIdx.y / T2_TILES) * T2_TILE, nt0 = static_cast<int>(blockIdx.y % T2_TILES) * T2_TILE;
    if (mt0 >= bI || nt0 >= bJ) return;  // whole CTA: no barrier skipped by part of it
    const int mn = min(T2_TILE, bI - mt0), nn = min(T2_TILE, bJ - nt0);
    const long long nsup = g.n_sup;
    const long long colJ = static_cast<long long>(cJ) * g.n_ao + g.ao_off[J];
    const long long colI = static_cast<long long>(g.cneg[cJ]) * g.n_ao + g.ao_off[I];
    double *o = out + pr.r_off[p] + static_cast<long long>(cJ) * bI * bJ;
    // i per chunk so that both operands fit: 2 * T2_TILE * ic * aJ floats
    const int ic = max(1, min(aI, T2_SMEM_FLOATS / (2 * T2_TILE * aJ)));
    float *S1 = sm;                                                // [k][T2_TILE]
    float *S2 = sm + static_cast<size_t>(ic) * aJ * T2_TILE;       // [k][T2_TILE]
    const int m0 = (static_cast<int>(threadIdx.x) / (T2_TILE / 4)) * 4;
    const int n0 = (static_cast<int>(threadIdx.x) % (T2_TILE / 4)) * 4;
    float acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
    for (int pass = 0; pass < 2; ++pass)
    {
        const float *Xb = X + (pass == 0 ? xsign : 0);
        const float *Xa = X + (pass == 0 ? 0 : xsign);
        for (int i0 = 0; i0 < aI; i0 += ic)
        {
            const int ni = min(ic, aI - i0), nk = ni * aJ;
            __syncthreads();
            // S1[(i - i0) aJ + j][mu] = Xb[(I, mt0 + mu, i)][(cJ, J, j)]  (j fastest: contiguous reads)
            for (int t = threadIdx.x; t < T2_TILE * nk; t += T2_THREADS)
            {
                const int mu = t / nk, k = t % nk, il = k / aJ, jj = k % aJ;
                S1[k * T2_TILE + mu] =
                    mu < mn ? Xb[(g.rowc_off[I] + static_cast<long long>(mt0 + mu) * aI + i0 + il) * nsup + colJ + jj]
                            : 0.f;
            }
            // S2[(i - i0) aJ + j][nu] = Xa[(J, nt0 + nu, j)][(-cJ, I, i)]  (i fastest)
            for (int t = threadIdx.x; t < T2_TILE * nk; t += T2_THREADS)
            {
                const int nu = t / nk, r = t % nk, jj = r / ni, il = r % ni;
                S2[(il * aJ + jj) * T2_TILE + nu] =
                    nu < nn ? Xa[(g.rowc_off[J] + static_cast<long long>(nt0 + nu) * aJ + jj) * nsup + colI + i0 + il]
                            : 0.f;
            }
            __syncthreads();
            for (int k = 0; k < nk; ++k)
            {
                const float4 av = *reinterpret_cast<const float4 *>(S1 + k * T2_TILE + m0);
                const float4 bv = *reinterpret_cast<const float4 *>(S2 + k * T2_TILE + n0);
                const float a4[4] = {av.x, av.y, av.z, av.w}, b4[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(a4[a], b4[b], acc[a][b]);
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
            if (m0 + a < mn && n0 + b < nn)
                o[static_cast<long long>(mt0 + m0 + a) * bJ + nt0 + n0 + b] += static_cast<double>(acc[a][b]);
}

// B operand of X = C * Gs: row n = (cL, l), column k = (cK, k'):  Gs^T[n][k] = G[cdiff(cL,cK)][k'][l]
__global__ void k_gsT_split(const double *__restrict__ G, Geom g, long long kpad, __nv_bfloat16 *__restrict__ p0,
                            __nv_bfloat16 *__restrict__ p1, __nv_bfloat16 *__restrict__ p2)
{
    const long long nsup = g.n_sup;
    const int sign = blockIdx.y;
    const long long n_el = nsup * kpad;
    const int nao = g.n_ao, nc = g.n_c;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n_el;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long n = t / kpad, k = t % kpad;
        double x = 0.0;
        if (k < nsup)
        {
            const int cL = static_cast<int>(n / nao), l = static_cast<int>(n % nao);
            const int cK = static_cast<int>(k / nao), kk = static_cast<int>(k % nao);
            const int c = g.cdiff[cL * nc + cK];
            x = G[((static_cast<size_t>(sign) * nc + c) * nao + kk) * nao + l];
        }
        const __nv_bfloat16 h = __double2bfloat16(x);
        const double r1 = x - static_cast<double>(__bfloat162float(h));
        const __nv_bfloat16 m = __double2bfloat16(r1);
        const __nv_bfloat16 l = __double2bfloat16(r1 - static_cast<double>(__bfloat162float(m)));
        p0[sign * n_el + t] = h;
        p1[sign * n_el + t] = m;
        p2[sign * n_el + t] = l;
    }
}

// T1 B-operand layout of atom J: row nu, K index ((kc * aJpad + j) * CW + col) for
// C^J[nu][j][kc*CW + col] (zero beyond the atom's NAOs and the supercell width).
__global__ void k_cb_layout(const double *__restrict__ C, Geom g, int J, int ajp, int nkc, long long ktot,
                            __nv_bfloat16 *__restrict__ p0, __nv_bfloat16 *__restrict__ p1,
                            __nv_bfloat16 *__restrict__ p2)
{
    const int aJ = g.nao[J], bJ = g.nabf[J];
    const long long n = static_cast<long long>(bJ) * ktot;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const int nu = static_cast<int>(t / ktot);
        const long long k = t % ktot;
        const long long kc = k / (static_cast<long long>(ajp) * CW);
        const int rem = static_cast<int>(k % (static_cast<long long>(ajp) * CW));
        const int j = rem / CW, col = rem % CW;
        const long long c = kc * CW + col;
        double x = 0.0;
        if (j < aJ && c < g.n_sup) x = C[(g.rowc_off[J] + static_cast<long long>(nu) * aJ + j) * g.n_sup + c];
        const __nv_bfloat16 h = __double2bfloat16(x);
        const double r1 = x - static_cast<double>(__bfloat162float(h));
        const __nv_bfloat16 m = __double2bfloat16(r1);
        const __nv_bfloat16 l = __double2bfloat16(r1 - static_cast<double>(__bfloat162float(m)));
        p0[t] = h;
        p1[t] = m;
        p2[t] = l;
    }
}

} // namespace

struct TcChi0::Impl
{
    Geom g;
    Pairs pr;
    long long kpad = 0;
    int nkc = 0;
    bool t1_simt = false;
    SplitStore csplit, gs;
    DevBuf<float> X, Gf, Cf;
    DevBuf<int> err, cadd, ajpad;
    DevBuf<T1Work> work;
    DevBuf<T1Group> groups;
    int n_work = 0, n_groups = 0;
    std::vector<int> hI, hJ, nabf_h, nao_h;
    bool all_active = false;  // the uploaded work list covers every (pair, cell)
    bool has_split = false;   // some tiles are K parts that add into chi0(R) atomically
    int n_sm = 0;
    // Row groups of the active (pair, cell) blocks, ordered by J, then I, then cell, and the
    // 128-row tiles over each J's rows; active == nullptr: every block.
    void build_work(const unsigned char *active, cudaStream_t st);
    std::vector<SplitStore> cb;  // per species: C^J of its atoms, stacked
    T1Maps maps{};
    DevBuf<int> spec, spec_idx;
    int b_tile = 0, maxcj = 0, smem = 0, ra = 16, ntc = 64, nbs = 2, gj = JG;
    // Launch choices of the contraction: producer layout and K parts per tile.  The tuner
    // times the candidates on the first unscreened contraction of a shape and keeps the
    // fastest for every later call on that shape (tuned_choice).
    bool narrow_ok = false, narrow = false;
    int kparts = T1_KPARTS;
    bool kparts_forced = false, tuned = false;
    std::string shape_key;
    void autotune(const double *G, double *chi0R, cudaStream_t st);
    void launch_t1(const T1Args &a, cudaStream_t st);
};

namespace {
struct T1Choice
{
    bool narrow;
    int kparts;
    double ms;
};
std::mutex g_tune_mu;
std::map<std::string, T1Choice> g_tuned;  // shape key -> choice (process-wide)
} // namespace

namespace {
using T1Fn = void (*)(T1Args, T1Maps);
// The narrow producer layout serves the streamed (4-column-aligned, RA <= 16) cases with up
// to 64 ABFs on atom J (its 96 registers a thread hold 64 accumulator columns, not 128).
bool t1_narrow_ok(int ra, int ntc, bool sv) { return ra <= 16 && sv && ntc == 64; }

int t1_threads(bool narrow) { return narrow ? T1Layout<true>::threads : T1Layout<false>::threads; }

T1Fn t1_kernel(int ra, int ntc, bool sv, bool narrow)
{
    if (narrow) return ra == 13 ? k_t1_tc<13, 64, true, true> : k_t1_tc<16, 64, true, true>;
    if (ra == 13 && sv) return ntc == 64 ? k_t1_tc<13, 64, true, false> : k_t1_tc<13, 128, true, false>;
    if (ra == 13) return ntc == 64 ? k_t1_tc<13, 64, false, false> : k_t1_tc<13, 128, false, false>;
    if (ra == 16 && sv) return ntc == 64 ? k_t1_tc<16, 64, true, false> : k_t1_tc<16, 128, true, false>;
    if (ra == 16) return ntc == 64 ? k_t1_tc<16, 64, false, false> : k_t1_tc<16, 128, false, false>;
    return ntc == 64 ? k_t1_tc<32, 64, false, false> : k_t1_tc<32, 128, false, false>;
}
} // namespace

TcChi0::TcChi0(const Geom &g, const Pairs &pr, const double *C, cudaStream_t st) : impl_(std::make_unique<Impl>())
{
    Impl &m = *impl_;
    m.g = g;
    m.pr = pr;
    const long long nsup = g.n_sup;
    m.kpad = (nsup + 63) / 64 * 64;
    m.nkc = static_cast<int>((nsup + CW - 1) / CW);
    const char *env = std::getenv("LIBRPA_GB300_T1");
    m.t1_simt = env && std::string(env) == "simt";
    GB_REQUIRE(g.max_nao <= T1_MAXA, "the tensor-core chi0 kernel supports up to 32 NAOs per atom");
    GB_REQUIRE(g.max_nabf <= T1_NMAX, "the tensor-core chi0 kernel supports up to 128 ABFs per atom");
    m.csplit.alloc(NS, static_cast<size_t>(g.rows_c) * m.kpad);
    split_rows_f64(C, nsup, g.rows_c, static_cast<int>(nsup), static_cast<int>(m.kpad), m.csplit.bufs(), st);
    m.gs.alloc(NS, 2ull * nsup * m.kpad);
    m.X.alloc(2ull * g.rows_c * nsup);
    m.err.alloc(1);
    m.err.zero(st);
    // host copies of the small tables (Geom holds device pointers)
    std::vector<int> nao(g.n_at), nabf(g.n_at), cdiff(static_cast<size_t>(g.n_c) * g.n_c);
    GB_CUDA(cudaMemcpyAsync(nao.data(), g.nao, sizeof(int) * g.n_at, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(nabf.data(), g.nabf, sizeof(int) * g.n_at, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(cdiff.data(), g.cdiff, sizeof(int) * cdiff.size(), cudaMemcpyDeviceToHost, st));
    std::vector<int> hI(pr.n_pairs), hJ(pr.n_pairs);
    GB_CUDA(cudaMemcpyAsync(hI.data(), pr.I, sizeof(int) * pr.n_pairs, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(hJ.data(), pr.J, sizeof(int) * pr.n_pairs, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    // cadd[a][b] = cell of R_a + R_b: the unique c with cdiff[c][b] == a
    std::vector<int> cadd(cdiff.size(), -1);
    for (int c = 0; c < g.n_c; ++c)
        for (int b = 0; b < g.n_c; ++b) cadd[cdiff[c * g.n_c + b] * g.n_c + b] = c;
    m.cadd.alloc(cadd.size());
    m.cadd.upload(cadd.data(), cadd.size(), st);
    if (m.t1_simt)
    {
        m.Cf.alloc(static_cast<size_t>(g.rows_c) * nsup);
        launch_d2f(C, m.Cf.get(), g.rows_c * nsup, st);
        m.Gf.alloc(2ull * g.n_c * g.n_ao * g.n_ao);
        return;
    }
    // T1 B operands grouped by species (same NAO and ABF counts) and their TMA maps
    std::vector<int> ajp(g.n_at), spec(g.n_at), spec_idx(g.n_at);
    std::vector<std::pair<int, int>> species;
    std::vector<int> spec_count;
    for (int J = 0; J < g.n_at; ++J)
    {
        ajp[J] = (nao[J] + JG - 1) / JG * JG;
        const std::pair<int, int> key{nao[J], nabf[J]};
        int sp = -1;
        for (size_t k = 0; k < species.size(); ++k)
            if (species[k] == key) sp = static_cast<int>(k);
        if (sp < 0)
        {
            sp = static_cast<int>(species.size());
            species.push_back(key);
            spec_count.push_back(0);
        }
        GB_REQUIRE(sp < T1_MAXSPEC, "the tensor-core chi0 kernel supports up to 8 atom species");
        spec[J] = sp;
        spec_idx[J] = spec_count[sp]++;
    }
    m.cb.resize(species.size());
    for (size_t sp = 0; sp < species.size(); ++sp)
    {
        const int na = species[sp].first, nb = species[sp].second;
        const int ap = (na + JG - 1) / JG * JG;
        const long long ktot = static_cast<long long>(m.nkc) * ap * CW;
        const long long per_atom = static_cast<long long>(nb) * ktot;
        m.cb[sp].alloc(NS, static_cast<size_t>(per_atom) * spec_count[sp]);
        const SplitBufs b = m.cb[sp].bufs();
        for (int J = 0; J < g.n_at; ++J)
        {
            if (spec[J] != static_cast<int>(sp)) continue;
            const long long o = per_atom * spec_idx[J];
            k_cb_layout<<<static_cast<unsigned>(std::min<long long>((per_atom + 255) / 256, 152LL * 16)), 256, 0, st>>>(
                C, g, J, ap, m.nkc, ktot, b.p[0] + o, b.p[1] + o, b.p[2] + o);
            GB_LAUNCH_CHECK();
        }
        const int NT = (nb + 15) / 16 * 16;
        for (int p = 0; p < NS; ++p)
            make_tmap_bf16(&m.maps.m[sp][p], b.p[p], ktot, nb, spec_count[sp], ktot, per_atom, 64, NT);
        m.maps.ktot[sp] = ktot;
    }
    m.ajpad.alloc(ajp.size());
    m.ajpad.upload(ajp.data(), ajp.size(), st);
    m.spec.alloc(spec.size());
    m.spec.upload(spec.data(), spec.size(), st);
    m.spec_idx.alloc(spec_idx.size());
    m.spec_idx.upload(spec_idx.data(), spec_idx.size(), st);
    m.hI = hI;
    m.hJ = hJ;
    m.nabf_h = nabf;
    m.nao_h = nao;
    {
        int dev = 0;
        GB_CUDA(cudaGetDevice(&dev));
        GB_CUDA(cudaDeviceGetAttribute(&m.n_sm, cudaDevAttrMultiProcessorCount, dev));
    }
    m.work.alloc(static_cast<size_t>(pr.n_pairs) * g.n_c * ((g.max_nabf + T1_BM - 1) / T1_BM + 1) * T1_KPARTS_MAX +
                 8 * static_cast<size_t>(m.n_sm));
    m.groups.alloc(static_cast<size_t>(pr.n_pairs) * g.n_c);
    int ntmax = 16, minb = 1 << 30;
    for (int J = 0; J < g.n_at; ++J)
    {
        ntmax = std::max(ntmax, (nabf[J] + 15) / 16 * 16);
        minb = std::min(minb, nabf[J]);
    }
    m.b_tile = (ntmax * 128 + 1023) / 1024 * 1024;
    m.maxcj = (T1_BM + minb - 1) / minb + 1;
    m.ra = g.max_nao == 13 ? 13 : g.max_nao <= 16 ? 16 : 32;
    m.ntc = ntmax <= 64 ? 64 : 128;
    m.gj = 2 * JG;  // the streaming producers read 16 values of j per row i
    for (int J = 0; J < g.n_at; ++J) m.gj = std::max(m.gj, ajp[J]);
    // shared memory: A ring + at least two B stages + the G slots; fewer G slots than a tile of
    // small row groups could touch only shortens such tiles
    const int slot_bytes = 2 * rap(m.ra) * m.gj * 4;
    const int base = T1_STAGES * NS * A_TILE + 1024 + 512;
    const int fit = (T1_SMEM_MAX - base - 2 * NS * m.b_tile) / slot_bytes;
    GB_REQUIRE(fit >= 1, "chi0 tile does not fit shared memory (too many ABFs or NAOs per atom)");
    m.maxcj = std::min(m.maxcj, fit);
    const int fixed = base + m.maxcj * slot_bytes;
    m.nbs = std::min(T1_MAXB, (T1_SMEM_MAX - fixed) / (NS * m.b_tile));
    m.smem = fixed + m.nbs * NS * m.b_tile;
    const bool sv = g.n_ao % 4 == 0;
    m.narrow_ok = t1_narrow_ok(m.ra, m.ntc, sv);
    m.narrow = m.narrow_ok;
    // the cap, not this shape's own size: contractions of other shapes on other host threads share
    // the kernel, and a smaller value set by one of them would fail this one's launch
    GB_CUDA(cudaFuncSetAttribute(t1_kernel(m.ra, m.ntc, sv, false), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 T1_SMEM_MAX));
    if (m.narrow_ok)
        GB_CUDA(cudaFuncSetAttribute(t1_kernel(m.ra, m.ntc, sv, true), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     T1_SMEM_MAX));
    // the shape the tuner's choice is kept for: per-atom sizes, cells, pairs, SM count
    {
        std::string key = std::to_string(g.n_c) + ":" + std::to_string(g.n_ao) + ":" + std::to_string(pr.n_pairs) +
                          ":" + std::to_string(m.n_sm) + ":";
        for (int J = 0; J < g.n_at; ++J) key += std::to_string(nao[J]) + "/" + std::to_string(nabf[J]) + ",";
        m.shape_key = key;
        // LIBRPA_GB300_T1_LAUNCH = "narrow:<kparts>" or "wide:<kparts>" fixes the choice (no tuning)
        if (const char *fx = std::getenv("LIBRPA_GB300_T1_LAUNCH"))
        {
            const std::string v(fx);
            const size_t c = v.find(':');
            GB_REQUIRE(c != std::string::npos, "LIBRPA_GB300_T1_LAUNCH must read narrow:<kparts> or wide:<kparts>");
            const std::string lay = v.substr(0, c);
            const int kp = std::atoi(v.c_str() + c + 1);
            GB_REQUIRE((lay == "narrow" || lay == "wide") && kp >= 1 && kp <= T1_KPARTS_MAX,
                       "LIBRPA_GB300_T1_LAUNCH must read narrow:<kparts> or wide:<kparts>, kparts 1-8");
            m.narrow = lay == "narrow" && m.narrow_ok;
            m.kparts = kp;
            m.kparts_forced = true;
            m.tuned = true;
        }
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = m.tuned ? g_tuned.end() : g_tuned.find(key);
        if (it != g_tuned.end())
        {
            m.narrow = it->second.narrow;
            m.kparts = it->second.kparts;
            m.kparts_forced = true;
            m.tuned = true;
        }
    }
    m.build_work(nullptr, st);
    GB_CUDA(cudaStreamSynchronize(st));
}

void TcChi0::Impl::launch_t1(const T1Args &a, cudaStream_t st)
{
    t1_kernel(ra, ntc, a.vec4 != 0, narrow)<<<n_work, t1_threads(narrow), smem, st>>>(a, maps);
    GB_LAUNCH_CHECK();
}

// Times every candidate (producer layout x K parts per tile) on this contraction's own inputs,
// one warm and one timed launch each, and keeps the fastest.  The candidates write chi0R; the
// caller's own launch after the tuning overwrites it (zeroing it first when tiles are split).
void TcChi0::Impl::autotune(const double *G, double *chi0R, cudaStream_t st)
{
    T1Args a{};
    a.g = g;
    a.pr = pr;
    a.X = X.get();
    a.xsign = g.rows_c * g.n_sup;
    a.G = G;
    a.cadd = cadd.get();
    a.work = work.get();
    a.groups = groups.get();
    a.spec = spec.get();
    a.spec_idx = spec_idx.get();
    a.aJpad = ajpad.get();
    a.nkc = nkc;
    a.b_tile = b_tile;
    a.nbs = nbs;
    a.gj = gj;
    a.maxcj = maxcj;
    a.vec4 = g.n_ao % 4 == 0 ? 1 : 0;
    a.out = chi0R;
    a.err = err.get();
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    T1Choice best{narrow, kparts, 1e30};
    const int kp_cand[] = {1, 2, 4, 8};
    for (int lay = 0; lay < (narrow_ok ? 2 : 1); ++lay)
        for (int kp : kp_cand)
        {
            if (kp > T1_KPARTS_MAX || (kp > 1 && nkc < 2 * kp)) continue;
            narrow = lay == 0 && narrow_ok;
            kparts = kp;
            kparts_forced = true;
            all_active = false;
            build_work(nullptr, st);
            if (n_work == 0) continue;
            launch_t1(a, st);
            GB_CUDA(cudaEventRecord(e0, st));
            launch_t1(a, st);
            GB_CUDA(cudaEventRecord(e1, st));
            GB_CUDA(cudaEventSynchronize(e1));
            float ms = 0.0f;
            GB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best.ms) best = T1Choice{narrow, kp, ms};
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    narrow = best.narrow;
    kparts = best.kparts;
    kparts_forced = true;
    all_active = false;
    tuned = true;
    build_work(nullptr, st);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[shape_key] = best;
}

void TcChi0::Impl::build_work(const unsigned char *active, cudaStream_t st)
{
    if (!active && all_active) return;
    std::vector<T1Group> grp;
    std::vector<T1Work> tiles;
    std::vector<std::vector<int>> pairs_of(g.n_at);
    for (int p = 0; p < pr.n_pairs; ++p) pairs_of[hJ[p]].push_back(p);
    for (int J = 0; J < g.n_at; ++J)
    {
        // I atoms of one NAO count next to each other, so that most tiles hold row groups of one
        // NAO count and their producers loop over that many orbitals i, not over the largest
        std::sort(pairs_of[J].begin(), pairs_of[J].end(), [&](int x, int y) {
            return nao_h[hI[x]] != nao_h[hI[y]] ? nao_h[hI[x]] < nao_h[hI[y]] : hI[x] < hI[y];
        });
        const int gbeg = static_cast<int>(grp.size());
        for (int p : pairs_of[J])
            for (int c = 0; c < g.n_c; ++c)
                if (!active || active[static_cast<size_t>(p) * g.n_c + c]) grp.push_back({p, c});
        // tiles of 128 rows over the concatenated rows of this J's groups; a tile closes at 128
        // rows or when it touches maxcj row groups (its G slots)
        const int gend = static_cast<int>(grp.size());
        std::vector<int> grows(gend - gbeg);
        for (int gi = gbeg; gi < gend; ++gi) grows[gi - gbeg] = nabf_h[hI[grp[gi].pair]];
        std::vector<sched::RowTile> rt;
        sched::pack_row_tiles(grows.data(), gend - gbeg, gbeg, T1_BM, maxcj, rt);
        for (const sched::RowTile &r : rt)
        {
            GB_REQUIRE(r.nslot <= maxcj, "chi0 tile touches more row groups than its shared-memory G slots");
            int ra_t = 0;
            for (int k = 0; k < r.nslot; ++k) ra_t = std::max(ra_t, nao_h[hI[grp[r.g0 + k].pair]]);
            tiles.push_back(T1Work{J, r.g0, r.r0, r.nrows, r.nslot, 0, nkc, 0, ra_t});
        }
    }
    // launch order: by the I atom of a tile's first row group, so the CTAs resident at one time
    // stream the same X^I rows (the largest operand) through L2
    std::stable_sort(tiles.begin(), tiles.end(), [&](const T1Work &x, const T1Work &y) {
        return hI[grp[x.g0].pair] < hI[grp[y.g0].pair];
    });
    // Every tile contracts the same K range, so the last, partial wave of CTAs leaves SMs idle:
    // its tiles are cut into K parts (added atomically into chi0(R)) when that shortens the
    // makespan.  Launches of under 16 waves run every tile in T1_KPARTS K parts, finer units
    // for the scheduler (measured: the 16-atom workload's 1155 tiles ran 6% faster as 4 parts,
    // 8 parts no better; the 256-atom workload's 10k tiles gained nothing).
    has_split = false;
    {
        const std::vector<sched::KPart> plan =
            sched::plan_kparts(static_cast<int>(tiles.size()), n_sm, nkc, kparts, kparts_forced);
        std::vector<T1Work> cut;
        cut.reserve(plan.size());
        for (const sched::KPart &k : plan)
        {
            T1Work u = tiles[k.tile];
            u.kc0 = k.kc0;
            u.kc1 = k.kc1;
            u.split = k.split;
            has_split = has_split || k.split != 0;
            cut.push_back(u);
        }
        tiles.swap(cut);
    }
    n_groups = static_cast<int>(grp.size());
    n_work = static_cast<int>(tiles.size());
    GB_REQUIRE(tiles.size() <= work.size() && grp.size() <= groups.size(), "chi0 work list overflow");
    if (n_groups > 0)
    {
        groups.upload(grp.data(), grp.size(), st);
        work.upload(tiles.data(), tiles.size(), st);
    }
    all_active = active == nullptr;
}

TcChi0::~TcChi0() = default;

void TcChi0::launch_choice(int &narrow, int &kparts) const
{
    narrow = impl_->narrow ? 1 : 0;
    kparts = impl_->kparts;
}

int TcChi0::run(const double *Gs, const double *G, double *chi0R, cudaStream_t st)
{
    (void)Gs;
    return prepare(G, st) + contract(G, chi0R, nullptr, false, st);
}

int TcChi0::prepare(const double *G, cudaStream_t st)
{
    Impl &m = *impl_;
    const Geom &g = m.g;
    const long long nsup = g.n_sup;
    dim3 grid(static_cast<unsigned>(std::min<long long>((nsup * m.kpad + 255) / 256, 152LL * 32)), 2);
    const SplitBufs gb = m.gs.bufs();
    k_gsT_split<<<grid, 256, 0, st>>>(G, g, m.kpad, gb.p[0], gb.p[1], gb.p[2]);
    GB_LAUNCH_CHECK();
    tc_gemm_split(m.csplit.mat(g.rows_c, m.kpad, 0), m.gs.mat(nsup, m.kpad, nsup * m.kpad), static_cast<int>(g.rows_c),
                  static_cast<int>(nsup), static_cast<int>(nsup), 2, m.X.get(), nsup, g.rows_c * nsup, false,
                  m.err.get(), st);
    return 2;
}

int TcChi0::contract(const double *G, double *chi0R, const unsigned char *active, bool zero_first, cudaStream_t st)
{
    Impl &m = *impl_;
    const Geom &g = m.g;
    const long long nsup = g.n_sup;
    int launches = 0;
    if (!m.t1_simt && !active && !m.tuned) m.autotune(G, chi0R, st);
    if (!m.t1_simt) m.build_work(active, st);
    // K-part tiles add into chi0(R), so their rows start from zero
    if (zero_first || (!m.t1_simt && m.has_split))
        GB_CUDA(cudaMemsetAsync(chi0R, 0, sizeof(double) * static_cast<size_t>(m.pr.e_total) * g.n_c, st));
    if (m.t1_simt)
    {
        GB_REQUIRE(!active, "block screening needs the tensor-core chi0 kernel");
        const long long ng = static_cast<long long>(g.n_c) * g.n_ao * g.n_ao;
        launch_d2f(G, m.Gf.get(), 2 * ng, st);
        launch_chi0_fp32(m.X.get(), m.X.get() + g.rows_c * nsup, m.Cf.get(), m.Gf.get(), m.Gf.get() + ng, g, m.pr,
                         chi0R, st);
        launches += 2;
    }
    else
    {
        T1Args a;
        a.g = g;
        a.pr = m.pr;
        a.X = m.X.get();
        a.xsign = g.rows_c * nsup;
        a.G = G;
        a.cadd = m.cadd.get();
        a.work = m.work.get();
        a.groups = m.groups.get();
        a.spec = m.spec.get();
        a.spec_idx = m.spec_idx.get();
        a.aJpad = m.ajpad.get();
        a.nkc = m.nkc;
        a.b_tile = m.b_tile;
        a.nbs = m.nbs;
        a.gj = m.gj;
        a.maxcj = m.maxcj;
        a.vec4 = g.n_ao % 4 == 0 ? 1 : 0;
        a.out = chi0R;
        a.err = m.err.get();
        if (m.n_work > 0)
        {
            m.launch_t1(a, st);
            k_t2<<<dim3(m.n_groups, T2_TILES * T2_TILES), T2_THREADS, 0, st>>>(m.X.get(), g.rows_c * nsup, g, m.pr,
                                                                             m.groups.get(), chi0R);
            GB_LAUNCH_CHECK();
            launches += 2;
        }
    }
    int herr = 0;
    m.err.download(&herr, 1, st);
    GB_CUDA(cudaStreamSynchronize(st));
    GB_REQUIRE(herr == 0, "tensor-core chi0 kernel reported wait timeout code " + std::to_string(herr));
    return launches;
}

} // namespace gb
