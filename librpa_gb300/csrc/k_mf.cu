// Mean-field side kernels: occupation/energy weights, G_k(tau) products,
// the k -> R phase sum, the supercell G matrix, and the RI scatter.
//
// G(R, +-tau) follows LibRPA's LibRI-routing builder (src/core/chi0.cpp:303-426):
//   G_ij(R, tau) = sgn * Re sum_k exp(-i 2pi kfrac_k.R) sum_n psi_ni(k) s_n(k) conj(psi_nj(k))
// with s_n = exp(min(0, -tau (e_n - e_F))) * w_n, w+ = max(0, 1/nk - f ns/2), w- = f ns/2,
// sgn = -1 for tau < 0, and Re taken after the k sum.
#include "kernels.h"
#include "common.h"

namespace gb {

namespace {

__global__ void k_tau_scale(const double *__restrict__ ekb, const double *__restrict__ wg, int nk, int nb,
                            double ef, double tau, int n_spins, int nbands_g, double *__restrict__ s)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int nkb = nk * nb;
    if (idx >= nkb) return;
    const int n = idx % nb;
    const double w = wg[idx];  // already scaled by 1/nk
    double wp = 1.0 / nk - w / 2.0 * n_spins;
    if (wp < 0) wp = 0;
    const double wm = w * 0.5 * n_spins;
    double ph_p = -tau * (ekb[idx] - ef);
    if (ph_p > 0) ph_p = 0;
    double ph_m = tau * (ekb[idx] - ef);
    if (ph_m > 0) ph_m = 0;
    double sp = exp(ph_p) * wp;
    double sm = exp(ph_m) * wm;
    if (nbands_g >= 0 && n >= nbands_g) sp = sm = 0.0;
    s[idx] = sp;
    s[nkb + idx] = sm;
}

// A[b][i][j] = sum_n psi[k][n][i] * s[b][n] * conj(psi[k][n][j]);  b = sign*nk + k
constexpr int GK_T = 32;
constexpr int GK_BN = 16;

__global__ void __launch_bounds__(256) k_gk_build(const cuDoubleComplex *__restrict__ psi,
                                                  const double *__restrict__ s, int nk, int nb, int nao,
                                                  cuDoubleComplex *__restrict__ A)
{
    __shared__ cuDoubleComplex Pi[GK_BN][GK_T];
    __shared__ cuDoubleComplex Pj[GK_BN][GK_T];
    const int b = blockIdx.z;
    const int k = b % nk;
    const int i0 = blockIdx.y * GK_T, j0 = blockIdx.x * GK_T;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const cuDoubleComplex *P = psi + static_cast<size_t>(k) * nb * nao;
    const double *sb = s + static_cast<size_t>(b) * nb;
    cuDoubleComplex acc[2][2];
    for (int a = 0; a < 2; ++a)
        for (int c = 0; c < 2; ++c) acc[a][c] = make_cuDoubleComplex(0, 0);
    for (int n0 = 0; n0 < nb; n0 += GK_BN)
    {
        for (int t = threadIdx.x; t < GK_BN * GK_T; t += blockDim.x)
        {
            const int nn = t / GK_T, cc = t % GK_T;
            const int n = n0 + nn;
            cuDoubleComplex vi = make_cuDoubleComplex(0, 0), vj = make_cuDoubleComplex(0, 0);
            if (n < nb)
            {
                if (i0 + cc < nao) vi = P[static_cast<size_t>(n) * nao + i0 + cc];
                if (j0 + cc < nao)
                {
                    const cuDoubleComplex p = P[static_cast<size_t>(n) * nao + j0 + cc];
                    vj = make_cuDoubleComplex(p.x * sb[n], -p.y * sb[n]);
                }
            }
            Pi[nn][cc] = vi;
            Pj[nn][cc] = vj;
        }
        __syncthreads();
#pragma unroll 4
        for (int nn = 0; nn < GK_BN; ++nn)
        {
            const cuDoubleComplex a0 = Pi[nn][ty * 2], a1 = Pi[nn][ty * 2 + 1];
            const cuDoubleComplex b0 = Pj[nn][tx * 2], b1 = Pj[nn][tx * 2 + 1];
            acc[0][0] = cuCfma(a0, b0, acc[0][0]);
            acc[0][1] = cuCfma(a0, b1, acc[0][1]);
            acc[1][0] = cuCfma(a1, b0, acc[1][0]);
            acc[1][1] = cuCfma(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
    cuDoubleComplex *Ab = A + static_cast<size_t>(b) * nao * nao;
    for (int a = 0; a < 2; ++a)
        for (int c = 0; c < 2; ++c)
        {
            const int i = i0 + ty * 2 + a, j = j0 + tx * 2 + c;
            if (i < nao && j < nao) Ab[static_cast<size_t>(i) * nao + j] = acc[a][c];
        }
}

// G[sign][c][i][j] = sgn * sum_k (cos th_kc Re A + sin th_kc Im A),  th = 2pi kfrac_k.R_c
constexpr int PS_CB = 8;

__global__ void k_phase_sum(const cuDoubleComplex *__restrict__ A, const double *__restrict__ cosph,
                            const double *__restrict__ sinph, int nk, int nc, int nao,
                            double *__restrict__ G)
{
    const size_t nn = static_cast<size_t>(nao) * nao;
    const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int sign = blockIdx.y;
    if (idx >= nn) return;
    const double sg = sign == 0 ? 1.0 : -1.0;
    const cuDoubleComplex *As = A + static_cast<size_t>(sign) * nk * nn + idx;
    for (int c0 = 0; c0 < nc; c0 += PS_CB)
    {
        double acc[PS_CB];
#pragma unroll
        for (int t = 0; t < PS_CB; ++t) acc[t] = 0.0;
        for (int k = 0; k < nk; ++k)
        {
            const cuDoubleComplex a = As[static_cast<size_t>(k) * nn];
#pragma unroll
            for (int t = 0; t < PS_CB; ++t)
            {
                const int c = c0 + t;
                if (c < nc) acc[t] += cosph[k * nc + c] * a.x + sinph[k * nc + c] * a.y;
            }
        }
#pragma unroll
        for (int t = 0; t < PS_CB; ++t)
        {
            const int c = c0 + t;
            if (c < nc) G[(static_cast<size_t>(sign) * nc + c) * nn + idx] = sg * acc[t];
        }
    }
}

__global__ void k_gsuper(const double *__restrict__ G, int nc, int nao, const int *__restrict__ cdiff,
                         double *__restrict__ Gs)
{
    const long long nsup = static_cast<long long>(nc) * nao;
    const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int sign = blockIdx.y;
    if (idx >= nsup * nsup) return;
    const long long r = idx / nsup, col = idx % nsup;
    const int cK = static_cast<int>(r / nao), a = static_cast<int>(r % nao);
    const int cL = static_cast<int>(col / nao), b = static_cast<int>(col % nao);
    const int c = cdiff[cL * nc + cK];
    Gs[static_cast<size_t>(sign) * nsup * nsup + idx] =
        G[((static_cast<size_t>(sign) * nc + c) * nao + a) * nao + b];
}

// blk_meta[4*b] = (I, J, cell, unused); element (i, j, mu) of block b at blob[off + (i*nj + j)*nmu + mu]
__global__ void k_cs_scatter(const double *__restrict__ blob, const long long *__restrict__ blk_off,
                             const int *__restrict__ meta, Geom g, double *__restrict__ C)
{
    const int b = blockIdx.x;
    const int I = meta[4 * b], J = meta[4 * b + 1], c = meta[4 * b + 2];
    const int ni = g.nao[I], nj = g.nao[J], nmu = g.nabf[I];
    const long long n = static_cast<long long>(ni) * nj * nmu;
    const double *src = blob + blk_off[b];
    for (long long t = threadIdx.x; t < n; t += blockDim.x)
    {
        const int mu = static_cast<int>(t % nmu);
        const long long ij = t / nmu;
        const int j = static_cast<int>(ij % nj), i = static_cast<int>(ij / nj);
        const long long row = g.rowc_off[I] + static_cast<long long>(mu) * ni + i;
        const long long col = static_cast<long long>(c) * g.n_ao + g.ao_off[J] + j;
        C[row * g.n_sup + col] = src[t];
    }
}

} // namespace

void launch_tau_scale(const double *ekb, const double *wg, int nk, int nb, double ef, double tau,
                      int n_spins, int nbands_g, double *s_out, cudaStream_t st)
{
    const int n = nk * nb;
    k_tau_scale<<<(n + 255) / 256, 256, 0, st>>>(ekb, wg, nk, nb, ef, tau, n_spins, nbands_g, s_out);
    GB_LAUNCH_CHECK();
}

void launch_gk_build(const cuDoubleComplex *psi, const double *s, int nk, int nb, int nao,
                     cuDoubleComplex *A, cudaStream_t st)
{
    dim3 grid((nao + GK_T - 1) / GK_T, (nao + GK_T - 1) / GK_T, 2 * nk);
    // psi index for batch b uses k = b % nk; s is laid out [sign][k][n] = [b][n]
    k_gk_build<<<grid, 256, 0, st>>>(psi, s, nk, nb, nao, A);
    GB_LAUNCH_CHECK();
}

void launch_phase_sum(const cuDoubleComplex *A, const double *cosph, const double *sinph, int nk,
                      int nc, int nao, double *G, cudaStream_t st)
{
    const size_t nn = static_cast<size_t>(nao) * nao;
    dim3 grid(static_cast<unsigned>((nn + 255) / 256), 2);
    k_phase_sum<<<grid, 256, 0, st>>>(A, cosph, sinph, nk, nc, nao, G);
    GB_LAUNCH_CHECK();
}

void launch_gsuper(const double *G, const Geom &g, double *Gs, cudaStream_t st)
{
    const long long n = static_cast<long long>(g.n_sup) * g.n_sup;
    dim3 grid(static_cast<unsigned>((n + 255) / 256), 2);
    k_gsuper<<<grid, 256, 0, st>>>(G, g.n_c, g.n_ao, g.cdiff, Gs);
    GB_LAUNCH_CHECK();
}

void launch_cs_scatter(const double *blob, const long long *blk_off, const int *blk_meta, int n_blocks,
                       const Geom &g, double *C, cudaStream_t st)
{
    if (n_blocks == 0) return;
    k_cs_scatter<<<n_blocks, 256, 0, st>>>(blob, blk_off, blk_meta, g, C);
    GB_LAUNCH_CHECK();
}

} // namespace gb
