// tcgen05 (5th-generation tensor core) building blocks: BF16 hi/lo split
// operands, TMA descriptors, the split-precision GEMM, and the chi0 path built
// on them.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include <memory>

#include "common.h"
#include "kernels.h"

namespace gb {

// A K-major operand held as ns = 2 (hi, lo) or ns = 3 (hi, mid, lo) BF16 pieces:
// rows x kpad (kpad a multiple of 64), batch_stride elements between batch entries
// (0: the same matrix for every batch entry).
struct SplitMat
{
    int ns;
    const __nv_bfloat16 *p[3];
    long long rows;
    long long kpad;
    long long batch_stride;
};

struct SplitBufs
{
    int ns;
    __nv_bfloat16 *p[3];
};

// Owning storage for the pieces of one split operand.
struct SplitStore
{
    int ns = 0;
    DevBuf<__nv_bfloat16> piece[3];
    SplitStore() = default;
    SplitStore(int n, size_t elems) { alloc(n, elems); }
    void alloc(int n, size_t elems)
    {
        ns = n;
        for (int i = 0; i < 3; ++i)
            if (i < n) piece[i].alloc(elems);
            else piece[i].release();
    }
    SplitBufs bufs() const { return {ns, {piece[0].get(), piece[1].get(), ns == 3 ? piece[2].get() : nullptr}}; }
    SplitMat mat(long long rows, long long kpad, long long batch_stride) const
    {
        return {ns, {piece[0].get(), piece[1].get(), ns == 3 ? piece[2].get() : nullptr}, rows, kpad, batch_stride};
    }
};

void make_tmap_bf16(CUtensorMap *map, const void *base, long long inner, long long rows, long long batch,
                    long long row_stride_elems, long long batch_stride_elems, int box_inner, int box_rows);
// split of row-major [rows][cols] into [rows][kpad] pieces (zero padded)
void split_rows_f64(const double *src, long long lds, long long rows, int cols, int kpad, const SplitBufs &o,
                    cudaStream_t st);
void split_rows_f32(const float *src, long long lds, long long rows, int cols, int kpad, const SplitBufs &o,
                    cudaStream_t st);
// split of the transpose: src [K][N] row-major -> dst [N][kpad]
void split_transpose_f64(const double *src, long long lds, int K, int N, int kpad, const SplitBufs &o,
                         cudaStream_t st);
// Structure the split GEMM may skip.  tri = 1: B[n][k] = 0 for k < n (B^T lower triangular),
// tri = 2: A[m][k] = 0 for k < m; the K loop of an output tile then starts at its first
// nonzero 64-wide block (the skipped products are exact zeros).  lower_tiles: only output tiles
// on or below the diagonal are computed (symmetric results); the others are left untouched.
struct TcGemmOpts
{
    int tri = 0;
    int tri_mul = 1;  // tri = 1: B[n][k] = 0 for k < tri_mul * n (2 for interleaved complex K)
    bool lower_tiles = false;
};
// D[b] (+)= A[b] * B[b]^T from BF16 split pieces (ns = 2: 3 products, ns = 3: 6 products),
// FP32 TMEM accumulation.
void tc_gemm_split(const SplitMat &A, const SplitMat &B, int M, int N, int K, int batch, float *D, long long ldd,
                   long long sD, bool accumulate, int *err, cudaStream_t st, const TcGemmOpts &o = TcGemmOpts{});
// Set the split GEMM kernels' shared-memory attribute on the current device.
void tc_gemm_set_attributes();
// D = A * B through the split GEMM with all scratch in a fixed static device array
// (tc_gemm_noalloc.cu); synchronises `st` before returning.
void tc_gemm_noalloc(int M, int N, int K, const double *A, const double *B, float *D, int ns, cudaStream_t st);
// Random M x N x K product vs the FP64 SIMT GEMM on the device; returns max |diff| / max |ref|.
double tc_gemm_selftest(int M, int N, int K, int seed, int ns);

class TcChi0
{
public:
    TcChi0(const Geom &g, const Pairs &pr, const double *C, cudaStream_t st);
    ~TcChi0();
    // G (both signs, [sign][cell][i][j]) and the supercell G -> chi0(R) upper-pair blocks.
    int run(const double *Gs, const double *G, double *chi0R, cudaStream_t st);
    // The two halves of run(): X(+-) = C * G_super(+-) ...
    int prepare(const double *G, cudaStream_t st);
    // ... and the block contraction of the active (pair, cell) blocks (active: host mask
    // [pair * n_cells + cell], nullptr = all).  zero_first clears chi0R first, so blocks left
    // out read zero; a later call with zero_first = false adds further blocks.
    int contract(const double *G, double *chi0R, const unsigned char *active, bool zero_first, cudaStream_t st);
    // The contraction's launch choice: narrow producer layout (1) or wide (0), K parts per tile.
    void launch_choice(int &narrow, int &kparts) const;

    struct Impl;

private:
    std::unique_ptr<Impl> impl_;
};

} // namespace gb
