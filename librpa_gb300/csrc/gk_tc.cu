// G_k(tau) = Psi^T diag(s) conj(Psi) as a split-precision tcgen05 GEMM, then the k -> R sum.
//
// With psi = a + i b and s_n >= 0 (occupation weight times a decaying exponential),
//   Re A_ij = sum_n (sqrt(s_n) a_ni)(sqrt(s_n) a_nj) + (sqrt(s_n) b_ni)(sqrt(s_n) b_nj)
//   Im A_ij = sum_n (sqrt(s_n) b_ni)(sqrt(s_n) a_nj) - (sqrt(s_n) a_ni)(sqrt(s_n) b_nj)
// so one operand P[b][(part, i)][K] (K = n for the a half, nb + n for the b half) serves as
// both A (all rows) and B (the part-0 rows): D[b][(part, i)][j] = sum_K P[(part,i)][K] P[(0,j)][K].
// One k point (Gamma) needs only the real part.
#include <cmath>

#include "gk_tc.h"

namespace gb {

namespace {

__global__ void k_psi_split(const cuDoubleComplex *__restrict__ psi, const double *__restrict__ s, int nk, int nb,
                            int nao, int parts, int kw, long long kpad, __nv_bfloat16 *__restrict__ p0,
                            __nv_bfloat16 *__restrict__ p1, __nv_bfloat16 *__restrict__ p2)
{
    const int b = blockIdx.y;  // sign * nk + k
    const int k = b % nk;
    const long long n_el = static_cast<long long>(parts) * nao * kpad;
    const size_t base = static_cast<size_t>(b) * n_el;
    for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n_el;
         t += static_cast<long long>(gridDim.x) * blockDim.x)
    {
        const long long row = t / kpad;
        const int K = static_cast<int>(t % kpad);
        const int part = static_cast<int>(row / nao), i = static_cast<int>(row % nao);
        double x = 0.0;
        if (K < kw * nb)
        {
            const int half = K / nb, n = K % nb;
            const cuDoubleComplex z = psi[(static_cast<size_t>(k) * nb + n) * nao + i];
            const double sq = sqrt(s[static_cast<size_t>(b) * nb + n]);
            if (part == 0)
                x = sq * (half == 0 ? z.x : z.y);
            else
                x = sq * (half == 0 ? z.y : -z.x);
        }
        const __nv_bfloat16 h = __double2bfloat16(x);
        const double r1 = x - static_cast<double>(__bfloat162float(h));
        const __nv_bfloat16 m = __double2bfloat16(r1);
        const __nv_bfloat16 l = __double2bfloat16(r1 - static_cast<double>(__bfloat162float(m)));
        p0[base + t] = h;
        p1[base + t] = m;
        p2[base + t] = l;
    }
}

// G[sign][c][i][j] = sgn * sum_k (cos th_kc Re A + sin th_kc Im A), A from D[b][(part,i)][j]
constexpr int PS_CB = 8;

__global__ void k_phase_sum_f32(const float *__restrict__ D, int parts, const double *__restrict__ cosph,
                                const double *__restrict__ sinph, int nk, int nc, int nao, double *__restrict__ G)
{
    const size_t nn = static_cast<size_t>(nao) * nao;
    const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int sign = blockIdx.y;
    if (idx >= nn) return;
    const double sg = sign == 0 ? 1.0 : -1.0;
    const size_t slab = static_cast<size_t>(parts) * nn;
    for (int c0 = 0; c0 < nc; c0 += PS_CB)
    {
        double acc[PS_CB];
#pragma unroll
        for (int t = 0; t < PS_CB; ++t) acc[t] = 0.0;
        for (int k = 0; k < nk; ++k)
        {
            const float *Db = D + (static_cast<size_t>(sign) * nk + k) * slab;
            const double re = Db[idx], im = parts > 1 ? Db[nn + idx] : 0.0;
#pragma unroll
            for (int t = 0; t < PS_CB; ++t)
            {
                const int c = c0 + t;
                if (c < nc) acc[t] += cosph[k * nc + c] * re + sinph[k * nc + c] * im;
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

} // namespace

GkTc::GkTc(int nk, int nb, int nao, bool psi_real)
    : nk_(nk), nb_(nb), nao_(nao), parts_(nk > 1 ? 2 : 1), kw_(psi_real ? 1 : 2)
{
    kpad_ = (static_cast<long long>(kw_) * nb + 63) / 64 * 64;
    a_.alloc(3, 2ull * nk * parts_ * nao * kpad_);
    d_.alloc(2ull * nk * parts_ * nao * nao);
}

int GkTc::run(const cuDoubleComplex *psi, const double *s, const double *cosph, const double *sinph, int nc,
              double *G, int *err, cudaStream_t st)
{
    const long long n_el = static_cast<long long>(parts_) * nao_ * kpad_;
    const SplitBufs p = a_.bufs();
    dim3 grid(static_cast<unsigned>(std::min<long long>((n_el + 255) / 256, 152LL * 16)), 2 * nk_);
    k_psi_split<<<grid, 256, 0, st>>>(psi, s, nk_, nb_, nao_, parts_, kw_, kpad_, p.p[0], p.p[1], p.p[2]);
    GB_LAUNCH_CHECK();
    // A: all (part, i) rows; B: the part-0 rows of the same batch entry
    const SplitMat A = a_.mat(static_cast<long long>(parts_) * nao_, kpad_, n_el);
    const SplitMat B = a_.mat(nao_, kpad_, n_el);
    tc_gemm_split(A, B, parts_ * nao_, nao_, kw_ * nb_, 2 * nk_, d_.get(), nao_,
                  static_cast<long long>(parts_) * nao_ * nao_, false, err, st);
    const size_t nn = static_cast<size_t>(nao_) * nao_;
    dim3 gp(static_cast<unsigned>((nn + 255) / 256), 2);
    k_phase_sum_f32<<<gp, 256, 0, st>>>(d_.get(), parts_, cosph, sinph, nk_, nc, nao_, G);
    GB_LAUNCH_CHECK();
    return 3;
}

} // namespace gb
