// Split-precision tcgen05 GEMM that allocates no device memory.
//
// Some callers cannot let a library allocate: a host DFT code that sizes its own device
// pool to the whole of HBM before it calls in (any cudaMalloc would then fail or evict its
// arrays), or a caller that must not block on the allocator's implicit device-wide
// synchronisation in the middle of its own asynchronous work. For them this variant of
// tc_gemm_split keeps its scratch -- the BF16 pieces of both operands and the kernel's
// error flag -- in one file-scope device array of fixed size, kScratchBytes.
//
// Set-up: the first call on a device (with that device current) looks up the array's
// device address with cudaGetSymbolAddress and sets the GEMM kernels' shared-memory
// attribute there; make that first call before any stream capture. Every call, the first
// and the later ones, launches its kernels, then synchronises the stream and copies the
// 4-byte error flag to the host before it returns.
//
// There is one scratch array per device, so calls whose GPU work overlaps (two host
// threads, or two streams on the same device) race on it: serialise them.
#include <mutex>
#include <string>

#include "common.h"
#include "tc_gemm.h"

namespace gb {

namespace {

constexpr size_t kScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr size_t kAlign = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mu;
unsigned char *g_scratch_ptr[kMaxDevices] = {};

size_t round_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

unsigned char *scratch_on_current_device()
{
    int dev = -1;
    GB_CUDA(cudaGetDevice(&dev));
    GB_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal out of range for the allocation-free GEMM");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev])
    {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        GB_REQUIRE(e == cudaSuccess && p, std::string("cudaGetSymbolAddress of the GEMM scratch failed: ") +
                                               cudaGetErrorString(e));
        tc_gemm_set_attributes();
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    return g_scratch_ptr[dev];
}

} // namespace

void tc_gemm_noalloc(int M, int N, int K, const double *A, const double *B, float *D, int ns, cudaStream_t st)
{
    GB_REQUIRE(M > 0 && N > 0 && K > 0, "M, N and K must be positive");
    GB_REQUIRE(ns == 2 || ns == 3, "pieces must be 2 or 3");
    GB_REQUIRE(A && B && D, "A, B and D must be device pointers");
    const long long kpad = (static_cast<long long>(K) + 63) / 64 * 64;
    const size_t a_piece = round_up(static_cast<size_t>(M) * kpad * sizeof(__nv_bfloat16));
    const size_t b_piece = round_up(static_cast<size_t>(N) * kpad * sizeof(__nv_bfloat16));
    const size_t need = static_cast<size_t>(ns) * (a_piece + b_piece) + kAlign;
    GB_REQUIRE(need <= kScratchBytes,
               "allocation-free GEMM: needs " + std::to_string(need) + " bytes of scratch (pieces * (M + N) * kpad * 2"
               " + alignment), more than its fixed " + std::to_string(kScratchBytes) + "-byte array");
    unsigned char *base = scratch_on_current_device();
    SplitBufs sa{ns, {nullptr, nullptr, nullptr}}, sb{ns, {nullptr, nullptr, nullptr}};
    size_t off = 0;
    for (int p = 0; p < ns; ++p, off += a_piece) sa.p[p] = reinterpret_cast<__nv_bfloat16 *>(base + off);
    for (int p = 0; p < ns; ++p, off += b_piece) sb.p[p] = reinterpret_cast<__nv_bfloat16 *>(base + off);
    int *err = reinterpret_cast<int *>(base + off);
    // the only scratch that must start at zero is the error flag: the split kernels write every
    // element of the pieces, padding columns included
    GB_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    split_rows_f64(A, K, M, K, static_cast<int>(kpad), sa, st);
    split_transpose_f64(B, N, K, N, static_cast<int>(kpad), sb, st);
    const SplitMat ma{ns, {sa.p[0], sa.p[1], sa.p[2]}, M, kpad, 0};
    const SplitMat mb{ns, {sb.p[0], sb.p[1], sb.p[2]}, N, kpad, 0};
    tc_gemm_split(ma, mb, M, N, K, 1, D, N, 0, false, err, st);
    int herr = 0;
    GB_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    GB_REQUIRE(herr == 0, "tcgen05 GEMM reported wait timeout code " + std::to_string(herr));
}

} // namespace gb
