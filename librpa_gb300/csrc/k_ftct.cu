// R -> q Fourier transform and tau -> omega cosine transform of chi0, fused.
//
// Restates chi_libri_ft_ct (LibRPA src/core/chi0.cpp:507-596):
//   chi0(q, w)[I<=J] += (2/n_s) * gamma(w, tau) * exp(+i 2pi q.R) * chi0(R, tau)[I,J]
// One CTA per upper atom pair; each thread owns block elements, gathers the
// n_c cell values once, and streams the (w, q) read-modify-writes coalesced
// along the element axis.  HBM-bound: per element and tau it moves
// 8 n_c bytes in and 2 * 16 n_w n_q bytes of chi0(q, w).
#include "kernels.h"
#include "common.h"

namespace gb {

namespace {

__global__ void __launch_bounds__(256) k_ftct(const double *__restrict__ chi0R, Geom g, Pairs pr,
                                              const double *__restrict__ qcos, const double *__restrict__ qsin,
                                              int nq, const double *__restrict__ gw, int nw, double fac,
                                              cuDoubleComplex *__restrict__ chi0q)
{
    const int p = blockIdx.x;
    const int I = pr.I[p], J = pr.J[p];
    const long long nel = static_cast<long long>(g.nabf[I]) * g.nabf[J];
    const int nc = g.n_c;
    const double *src = chi0R + pr.r_off[p];
    const long long eoff = pr.e_off[p];
    for (long long e = static_cast<long long>(blockIdx.y) * blockDim.x + threadIdx.x; e < nel;
         e += static_cast<long long>(gridDim.y) * blockDim.x)
    {
        for (int q = 0; q < nq; ++q)
        {
            double re = 0.0, im = 0.0;
            for (int c = 0; c < nc; ++c)
            {
                const double v = src[static_cast<long long>(c) * nel + e];
                re = fma(qcos[q * nc + c], v, re);
                im = fma(qsin[q * nc + c], v, im);
            }
            for (int w = 0; w < nw; ++w)
            {
                const double f = fac * gw[w];
                cuDoubleComplex *d = chi0q + (static_cast<long long>(w) * nq + q) * pr.e_total + eoff + e;
                cuDoubleComplex o = *d;
                o.x = fma(f, re, o.x);
                o.y = fma(f, im, o.y);
                *d = o;
            }
        }
    }
}

} // namespace

void launch_ftct(const double *chi0R, const Geom &g, const Pairs &pr, const double *qcos,
                 const double *qsin, int nq, const double *gamma_w, int nw, double fac,
                 cuDoubleComplex *chi0q, cudaStream_t st)
{
    int maxel = g.max_nabf * g.max_nabf;
    dim3 grid(pr.n_pairs, (maxel + 255) / 256);
    k_ftct<<<grid, 256, 0, st>>>(chi0R, g, pr, qcos, qsin, nq, gamma_w, nw, fac, chi0q);
    GB_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------------------------
// The same transform over a batch of stored chi0(R, tau) slots, applied once per batch instead
// of once per slot (slot = one (tau, spin) contraction output; the reduced-precision chi0 paths):
//   chi0(q, w) += sum_slot fac gamma(w, slot) sum_R e^{+i 2pi q.R} chi0_slot(R)
// The cosine transform over the slots (a minimax quadrature sum) runs in FP64; the R -> q
// phase sum of its result in FP32 (the precision of the chi0 blocks these paths produce).
// One CTA per (pair, FT_E block elements): the CTA stages C(R, w, e) = sum_slot gamma chi0 in
// shared memory, then each output (q, w, e) is an n_c-term sum read from there, and chi0(q, w)
// is read and written once per batch.  FT_E is 32 with many cells and up to 256 with few, so
// that the 256 threads of a CTA have n_c FT_E >= 256 items in the first phase.
namespace {

constexpr int FT_MAXW = 34;   // largest minimax grid

int ft_elems(int nc) { return nc >= 8 ? 32 : nc >= 2 ? 128 : 256; }

__global__ void __launch_bounds__(256) k_ftct_slots(const double *__restrict__ slots, long long slot_stride, int nslot,
                                                   Geom g, Pairs pr, const float2 *__restrict__ qph, int nq,
                                                   const double *__restrict__ gam, int nw, int FT_E,
                                                   cuDoubleComplex *__restrict__ chi0q)
{
    extern __shared__ __align__(16) unsigned char ft_smem[];
    const int nc = g.n_c;
    float *Cw = reinterpret_cast<float *>(ft_smem);                                       // [nc][nw][FT_E]
    float2 *ph = reinterpret_cast<float2 *>(Cw + static_cast<size_t>(nc) * nw * FT_E);    // [nq][nc]
    const int p = blockIdx.x;
    const int I = pr.I[p], J = pr.J[p];
    const int nel = g.nabf[I] * g.nabf[J];
    const int e0 = blockIdx.y * FT_E;
    if (e0 >= nel) return;  // uniform over the CTA
    for (int t = threadIdx.x; t < nq * nc; t += blockDim.x) ph[t] = qph[t];
    // cosine transform over the slots, FP64: item (R, e)
    for (int it = threadIdx.x; it < nc * FT_E; it += blockDim.x)
    {
        const int R = it / FT_E, e = it % FT_E;
        double c[FT_MAXW];
#pragma unroll
        for (int w = 0; w < FT_MAXW; ++w) c[w] = 0.0;
        if (e0 + e < nel)
        {
            const double *src = slots + pr.r_off[p] + static_cast<long long>(R) * nel + e0 + e;
            for (int s = 0; s < nslot; ++s)
            {
                const double v = src[static_cast<long long>(s) * slot_stride];
#pragma unroll
                for (int w = 0; w < FT_MAXW; ++w)
                    if (w < nw) c[w] = fma(gam[static_cast<size_t>(w) * nslot + s], v, c[w]);
            }
        }
#pragma unroll
        for (int w = 0; w < FT_MAXW; ++w)
            if (w < nw) Cw[(static_cast<size_t>(R) * nw + w) * FT_E + e] = static_cast<float>(c[w]);
    }
    __syncthreads();
    // R -> q: output (q, w, e), e fastest across the lanes of a warp
    const int e = threadIdx.x % FT_E;
    if (e0 + e >= nel) return;
    const long long eoff = pr.e_off[p] + e0 + e;
    for (int qw = threadIdx.x / FT_E; qw < nq * nw; qw += blockDim.x / FT_E)
    {
        const int q = qw / nw, w = qw % nw;
        float re = 0.0f, im = 0.0f;
        for (int R = 0; R < nc; ++R)
        {
            const float v = Cw[(static_cast<size_t>(R) * nw + w) * FT_E + e];
            const float2 f = ph[q * nc + R];
            re = fmaf(f.x, v, re);
            im = fmaf(f.y, v, im);
        }
        cuDoubleComplex *d = chi0q + (static_cast<long long>(w) * nq + q) * pr.e_total + eoff;
        cuDoubleComplex o = *d;
        o.x += static_cast<double>(re);
        o.y += static_cast<double>(im);
        *d = o;
    }
}

} // namespace

size_t ftct_slots_smem(int nc, int nq, int nw)
{
    return sizeof(float) * static_cast<size_t>(nc) * nw * ft_elems(nc) + sizeof(float2) * static_cast<size_t>(nq) * nc;
}

void launch_ftct_slots(const double *slots, long long slot_stride, int nslot, const Geom &g, const Pairs &pr,
                       const float2 *qphase, int nq, const double *gamma, int nw, cuDoubleComplex *chi0q,
                       cudaStream_t st)
{
    GB_REQUIRE(nw >= 1 && nw <= FT_MAXW, "minimax grid larger than the FT/CT kernel supports");
    const size_t smem = ftct_slots_smem(g.n_c, nq, nw);
    GB_REQUIRE(smem <= 227 * 1024, "FT/CT staging does not fit shared memory (too many cells x frequencies)");
    static PerDeviceOnce attr;
    attr.run([] { GB_CUDA(cudaFuncSetAttribute(k_ftct_slots, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024)); });
    const int maxel = g.max_nabf * g.max_nabf, fe = ft_elems(g.n_c);
    dim3 grid(pr.n_pairs, (maxel + fe - 1) / fe);
    k_ftct_slots<<<grid, 256, smem, st>>>(slots, slot_stride, nslot, g, pr, qphase, nq, gamma, nw, fe, chi0q);
    GB_LAUNCH_CHECK();
}

} // namespace gb
