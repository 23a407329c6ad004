// chi0(R, tau) atom-pair blocks on CUDA cores (FP64 plain path, FP32 variant).
//
// LibRI computes chi0s as two cal_loop3 passes (RPA.hpp:104-137) with labels
// a1b1_a2b2 and a1b2_a2b1 (LRI-cal_loop3.hpp:902-1032).  With the
// supercell products  X_b^I[mu i; (cL,L) l] = sum_{(cK,K) k} C^I[mu i; (cK,K) k] G_b[K;L,RL-RK]_{kl}
// (computed by a GEMM before this kernel) the two labels of one pass (Ga, Gb) are
//   T1[mu,nu] = sum_{i,j} Ga[I;J,RJ]_{ij} sum_{(cL,L) l} X_b^I[mu i;(cL,L) l] C^J[nu j;(L, RL-RJ) l]
//   T2[mu,nu] = sum_{i,j} X_b^I[mu i;(cJ,J) j] X_a^J[nu j;(c(-RJ),I) i]
// T2 uses Re G[I;L,R]_{il} = Re G[L;I,-R]_{li}, which the G builder satisfies exactly up to rounding.
// The passes are (Ga,Gb) = (G+,G-) and (G-,G+).  Only upper pairs I<=J are formed:
// they are the only blocks the R->q transform reads (chi0.cpp:521-534).
//
// One CTA owns a 48 x 48 (mu, nu) tile of one (pair, cell) block; the K loop walks
// the supercell orbital axis in chunks of LC columns, forming E = Ga^T X_b on the fly.
#include "kernels.h"
#include "common.h"

namespace gb {

namespace {

constexpr int TT = 48;   // mu / nu tile
constexpr int LC = 4;    // supercell columns per K step

template <typename T>
__global__ void __launch_bounds__(256) k_chi0_simt(const T *__restrict__ Xp, const T *__restrict__ Xm,
                                                   const T *__restrict__ Cm, const T *__restrict__ Gp,
                                                   const T *__restrict__ Gm, Geom g, Pairs pr,
                                                   double *__restrict__ out)
{
    extern __shared__ unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    const int MA = g.max_nao;
    T *gs = sm;                               // [MA][MA]
    T *Xs = gs + MA * MA;                     // [TT][MA][LC]
    T *Cs = Xs + TT * MA * LC;                // [TT][MA][LC]
    T *Es = Cs + TT * MA * LC;                // [TT][MA][LC]

    const int p = blockIdx.x / g.n_c;
    const int cJ = blockIdx.x % g.n_c;
    const int I = pr.I[p], J = pr.J[p];
    const int aI = g.nao[I], aJ = g.nao[J];
    const int bI = g.nabf[I], bJ = g.nabf[J];
    const int mu0 = blockIdx.y * TT, nu0 = blockIdx.z * TT;
    if (mu0 >= bI || nu0 >= bJ) return;
    const int mt = min(TT, bI - mu0), nt = min(TT, bJ - nu0);
    const long long nsup = g.n_sup;
    const long long rI = g.rowc_off[I], rJ = g.rowc_off[J];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int *cd = g.cdiff;
    const int nc = g.n_c, nao = g.n_ao;

    T acc[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) acc[a][b] = T(0);

    for (int pass = 0; pass < 2; ++pass)
    {
        const T *Ga = pass == 0 ? Gp : Gm;
        const T *Xb = pass == 0 ? Xm : Xp;
        const T *Xa = pass == 0 ? Xp : Xm;
        for (int t = threadIdx.x; t < aI * aJ; t += blockDim.x)
        {
            const int i = t / aJ, j = t % aJ;
            gs[i * MA + j] = Ga[(static_cast<size_t>(cJ) * nao + g.ao_off[I] + i) * nao + g.ao_off[J] + j];
        }
        __syncthreads();
        // ---- T1
        for (long long l0 = 0; l0 < nsup; l0 += LC)
        {
            for (int t = threadIdx.x; t < TT * MA * LC; t += blockDim.x)
            {
                const int lc = t % LC;
                const int q = t / LC;
                const int ii = q % MA, m = q / MA;
                const long long col = l0 + lc;
                T vx = T(0), vc = T(0);
                if (col < nsup)
                {
                    if (m < mt && ii < aI) vx = Xb[(rI + static_cast<long long>(mu0 + m) * aI + ii) * nsup + col];
                    if (m < nt && ii < aJ)
                    {
                        const int cL = static_cast<int>(col / nao);
                        const long long colp = static_cast<long long>(cd[cL * nc + cJ]) * nao + (col % nao);
                        vc = Cm[(rJ + static_cast<long long>(nu0 + m) * aJ + ii) * nsup + colp];
                    }
                }
                Xs[t] = vx;
                Cs[t] = vc;
            }
            __syncthreads();
            // E[m][j][lc] = sum_i g[i][j] X[m][i][lc]
            for (int t = threadIdx.x; t < TT * MA * LC; t += blockDim.x)
            {
                const int lc = t % LC;
                const int q = t / LC;
                const int j = q % MA, m = q / MA;
                T e = T(0);
                if (j < aJ && m < mt)
                    for (int i = 0; i < aI; ++i) e += gs[i * MA + j] * Xs[(m * MA + i) * LC + lc];
                Es[t] = e;
            }
            __syncthreads();
            for (int j = 0; j < aJ; ++j)
#pragma unroll
                for (int lc = 0; lc < LC; ++lc)
                {
                    T ev[3], cv[3];
#pragma unroll
                    for (int a = 0; a < 3; ++a) ev[a] = Es[((ty + 16 * a) * MA + j) * LC + lc];
#pragma unroll
                    for (int b = 0; b < 3; ++b) cv[b] = Cs[((tx + 16 * b) * MA + j) * LC + lc];
#pragma unroll
                    for (int a = 0; a < 3; ++a)
#pragma unroll
                        for (int b = 0; b < 3; ++b) acc[a][b] += ev[a] * cv[b];
                }
            __syncthreads();
        }
        // ---- T2: sum_{i,j} Xb^I[mu i; (cJ,J) j] * Xa^J[nu j; (c(-RJ), I) i]
        const long long colJ = static_cast<long long>(cJ) * nao + g.ao_off[J];
        const long long colI = static_cast<long long>(g.cneg[cJ]) * nao + g.ao_off[I];
        for (int i = 0; i < aI; ++i)
        {
            for (int t = threadIdx.x; t < TT * MA; t += blockDim.x)
            {
                const int j = t % MA, m = t / MA;
                T v1 = T(0), v2 = T(0);
                if (j < aJ)
                {
                    if (m < mt) v1 = Xb[(rI + static_cast<long long>(mu0 + m) * aI + i) * nsup + colJ + j];
                    if (m < nt) v2 = Xa[(rJ + static_cast<long long>(nu0 + m) * aJ + j) * nsup + colI + i];
                }
                Xs[t] = v1;
                Cs[t] = v2;
            }
            __syncthreads();
            for (int j = 0; j < aJ; ++j)
            {
                T ev[3], cv[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) ev[a] = Xs[(ty + 16 * a) * MA + j];
#pragma unroll
                for (int b = 0; b < 3; ++b) cv[b] = Cs[(tx + 16 * b) * MA + j];
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = 0; b < 3; ++b) acc[a][b] += ev[a] * cv[b];
            }
            __syncthreads();
        }
    }
    double *o = out + pr.r_off[p] + static_cast<long long>(cJ) * bI * bJ;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
        {
            const int m = ty + 16 * a, n = tx + 16 * b;
            if (m < mt && n < nt) o[static_cast<long long>(mu0 + m) * bJ + nu0 + n] = static_cast<double>(acc[a][b]);
        }
}

template <typename T>
void launch_chi0_simt(const T *Xp, const T *Xm, const T *Cm, const T *Gp, const T *Gm, const Geom &g,
                      const Pairs &pr, double *out, cudaStream_t st)
{
    const int MA = g.max_nao;
    const size_t smem = sizeof(T) * (static_cast<size_t>(MA) * MA + 3ull * TT * MA * LC);
    GB_REQUIRE(smem <= 227 * 1024, "atom NAO count too large for the SIMT chi0 kernel");
    // the cap once per device (calls of other shapes may run on other host threads)
    static PerDeviceOnce attr;
    attr.run([] { GB_CUDA(cudaFuncSetAttribute(k_chi0_simt<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024)); });
    const int tiles_mu = (g.max_nabf + TT - 1) / TT;
    dim3 grid(pr.n_pairs * g.n_c, tiles_mu, tiles_mu);
    k_chi0_simt<T><<<grid, 256, smem, st>>>(Xp, Xm, Cm, Gp, Gm, g, pr, out);
    GB_LAUNCH_CHECK();
}

} // namespace

void launch_chi0_fp64(const double *Xp, const double *Xm, const double *Cm, const double *Gp,
                      const double *Gm, const Geom &g, const Pairs &pr, double *out, cudaStream_t st)
{
    launch_chi0_simt<double>(Xp, Xm, Cm, Gp, Gm, g, pr, out, st);
}

void launch_chi0_fp32(const float *Xp, const float *Xm, const float *Cm, const float *Gp,
                      const float *Gm, const Geom &g, const Pairs &pr, double *out, cudaStream_t st)
{
    launch_chi0_simt<float>(Xp, Xm, Cm, Gp, Gm, g, pr, out, st);
}

} // namespace gb
