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

} // namespace gb
