// chi0(R, tau) contraction of one tau slice on the host cores, FP64, OpenMP.
//
// Test and measurement infrastructure only (the fused part of oracle/cpu_path.py, which the
// reference CPU arm of bench.py times).  It evaluates the LibRI two-pass chi0 algebra
// (RPA.hpp:104-137 with LRI-cal_loop3.hpp:902-1032) in the supercell form of
// rpa_oracle.cal_chi0s_dense, for every upper atom pair (I <= J) and BvK cell R:
//
//   T1[mu, nu] = sum_{K} sum_j E[mu, K, j] C^J[nu, j, K - R]
//   E[mu, K, j] = sum_i G+(R)_{ij} X-^I[mu i, K] + G-(R)_{ij} X+^I[mu i, K]
//   T2[mu, nu] = sum_{pass} sum_{i,j} X_b^I[mu i, (R, J) j] X_a^J[nu j, (-R, I) i]
//
// E is formed block by block (a few supercell columns at a time) and contracted at once, so
// that it never leaves the cache; one OpenMP work item is one (J, R, I) output block.
#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

constexpr int KB = 8;  // supercell columns per E block (never crossing a cell boundary)

// XX^I[mu][K][q]: q < a_I from X(-) (pass 0, paired with G(+)), q >= a_I from X(+) (pass 1)
void build_xx(int aI, int bI, long long nsup, const double *Xp, const double *Xm, long long row0, double *XX)
{
    const int Q = 2 * aI;
#pragma omp parallel for schedule(static)
    for (int mu = 0; mu < bI; ++mu)
        for (int i = 0; i < aI; ++i)
        {
            const double *xm = Xm + (row0 + static_cast<long long>(mu) * aI + i) * nsup;
            const double *xp = Xp + (row0 + static_cast<long long>(mu) * aI + i) * nsup;
            double *o = XX + static_cast<long long>(mu) * nsup * Q;
            for (long long K = 0; K < nsup; ++K)
            {
                o[K * Q + i] = xm[K];
                o[K * Q + aI + i] = xp[K];
            }
        }
}

// acc[bI][bJ] += E[bI][L] * Cb[bJ][L]^T, the rows of Cb `cstride` doubles apart
void gemm_nt(int bI, int bJ, int L, const double *E, const double *Cb, long long cstride, double *acc)
{
    int mu = 0;
    for (; mu + 4 <= bI; mu += 4)
    {
        const double *e0 = E + static_cast<long long>(mu) * L, *e1 = e0 + L, *e2 = e1 + L, *e3 = e2 + L;
        int nu = 0;
        for (; nu + 2 <= bJ; nu += 2)
        {
            const double *c0 = Cb + nu * cstride, *c1 = c0 + cstride;
            double a00 = 0, a01 = 0, a10 = 0, a11 = 0, a20 = 0, a21 = 0, a30 = 0, a31 = 0;
#pragma omp simd reduction(+ : a00, a01, a10, a11, a20, a21, a30, a31)
            for (int t = 0; t < L; ++t)
            {
                a00 += e0[t] * c0[t];
                a01 += e0[t] * c1[t];
                a10 += e1[t] * c0[t];
                a11 += e1[t] * c1[t];
                a20 += e2[t] * c0[t];
                a21 += e2[t] * c1[t];
                a30 += e3[t] * c0[t];
                a31 += e3[t] * c1[t];
            }
            double *r = acc + static_cast<long long>(mu) * bJ + nu;
            r[0] += a00;
            r[1] += a01;
            r[bJ] += a10;
            r[bJ + 1] += a11;
            r[2 * bJ] += a20;
            r[2 * bJ + 1] += a21;
            r[3 * bJ] += a30;
            r[3 * bJ + 1] += a31;
        }
        for (; nu < bJ; ++nu)
        {
            const double *c0 = Cb + nu * cstride;
            double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
#pragma omp simd reduction(+ : a0, a1, a2, a3)
            for (int t = 0; t < L; ++t)
            {
                a0 += e0[t] * c0[t];
                a1 += e1[t] * c0[t];
                a2 += e2[t] * c0[t];
                a3 += e3[t] * c0[t];
            }
            double *r = acc + static_cast<long long>(mu) * bJ + nu;
            r[0] += a0;
            r[bJ] += a1;
            r[2 * bJ] += a2;
            r[3 * bJ] += a3;
        }
    }
    for (; mu < bI; ++mu)
    {
        const double *e0 = E + static_cast<long long>(mu) * L;
        for (int nu = 0; nu < bJ; ++nu)
        {
            const double *c0 = Cb + nu * cstride;
            double a0 = 0;
#pragma omp simd reduction(+ : a0)
            for (int t = 0; t < L; ++t) a0 += e0[t] * c0[t];
            acc[static_cast<long long>(mu) * bJ + nu] += a0;
        }
    }
}

} // namespace

extern "C" {

// Adds chi0(R, tau) of one tau slice (one spin) to chi0R[nc][e_tot].
//   nao, nabf [n_at]; aoff [n_at + 1] orbital offsets; rowoff [n_at + 1] row offsets of the
//   RI rows (I, mu, i) in X(+-) [rows_c][nsup], nsup = nc * n_ao;
//   G(+-) [nc][n_ao][n_ao]; CT[J] = C^J as [nu][cell][ao][ajp(J)] with j padded to
//   ajp(J) = a_J rounded up to even (zeros); dshift[c][cL] = cell of R_L - R_c;
//   cneg[c] = cell of -R_c; eoff[p] the offset of upper pair p (I <= J, row-major) in a cell's
//   e_tot elements, each block b_I x b_J row-major.
// Returns 0.
int cpu_chi0_tau(int n_at, const int *nao, const int *nabf, const int *aoff, const long long *rowoff, int nc,
                 int n_ao, const double *Xp, const double *Xm, const double *Gp, const double *Gm,
                 const double *const *CT, const int *dshift, const int *cneg, const long long *eoff,
                 long long e_tot, double *chi0R)
{
    const long long nsup = static_cast<long long>(nc) * n_ao;
    std::vector<std::vector<double>> XX(n_at);
    for (int I = 0; I < n_at; ++I)
    {
        XX[I].resize(static_cast<size_t>(nabf[I]) * nsup * 2 * nao[I]);
        build_xx(nao[I], nabf[I], nsup, Xp, Xm, rowoff[I], XX[I].data());
    }
    std::vector<int> pidx(static_cast<size_t>(n_at) * n_at, -1);
    {
        int p = 0;
        for (int I = 0; I < n_at; ++I)
            for (int J = I; J < n_at; ++J) pidx[static_cast<size_t>(I) * n_at + J] = p++;
    }
    // work items (J, c, I <= J)
    std::vector<int> items;
    for (int J = 0; J < n_at; ++J)
        for (int c = 0; c < nc; ++c)
            for (int I = 0; I <= J; ++I)
            {
                items.push_back(J);
                items.push_back(c);
                items.push_back(I);
            }
    const long long n_items = static_cast<long long>(items.size() / 3);
#pragma omp parallel
    {
        std::vector<double> E, GG, acc;
#pragma omp for schedule(dynamic, 1)
        for (long long w = 0; w < n_items; ++w)
        {
            const int J = items[3 * w], c = items[3 * w + 1], I = items[3 * w + 2];
            const int aI = nao[I], aJ = nao[J], bI = nabf[I], bJ = nabf[J];
            const int Q = 2 * aI, ajp = (aJ + 1) & ~1;
            GG.assign(static_cast<size_t>(Q) * ajp, 0.0);
            for (int i = 0; i < aI; ++i)
                for (int j = 0; j < aJ; ++j)
                {
                    const long long g = (static_cast<long long>(c) * n_ao + aoff[I] + i) * n_ao + aoff[J] + j;
                    GG[static_cast<size_t>(i) * ajp + j] = Gp[g];
                    GG[static_cast<size_t>(aI + i) * ajp + j] = Gm[g];
                }
            acc.assign(static_cast<size_t>(bI) * bJ, 0.0);
            E.resize(static_cast<size_t>(bI) * KB * ajp);
            const double *xx = XX[I].data();
            const double *ct = CT[J];
            const long long crow = static_cast<long long>(nc) * n_ao * ajp;  // C^J row stride (nu)
            for (int cL = 0; cL < nc; ++cL)
            {
                const int csh = dshift[static_cast<size_t>(c) * nc + cL];
                for (int l0 = 0; l0 < n_ao; l0 += KB)
                {
                    const int kb = std::min(KB, n_ao - l0);
                    const int L = kb * ajp;
                    const long long K0 = static_cast<long long>(cL) * n_ao + l0;
                    // E[mu][kk][j] = sum_q XX[mu][K0 + kk][q] GG[q][j]
                    for (int mu = 0; mu < bI; ++mu)
                    {
                        const double *xr = xx + (static_cast<long long>(mu) * nsup + K0) * Q;
                        double *er = E.data() + static_cast<size_t>(mu) * L;
                        for (int kk = 0; kk < kb; ++kk)
                        {
                            double *e = er + kk * ajp;
                            for (int j = 0; j < ajp; ++j) e[j] = 0.0;
                            for (int q = 0; q < Q; ++q)
                            {
                                const double x = xr[kk * Q + q];
                                const double *g = GG.data() + static_cast<size_t>(q) * ajp;
#pragma omp simd
                                for (int j = 0; j < ajp; ++j) e[j] += x * g[j];
                            }
                        }
                    }
                    const double *cb = ct + (static_cast<long long>(csh) * n_ao + l0) * ajp;
                    gemm_nt(bI, bJ, L, E.data(), cb, crow, acc.data());
                }
            }
            // T2: pass (b, a) = (-, +) and (+, -)
            const int cm = cneg[c];
            for (int pass = 0; pass < 2; ++pass)
            {
                const double *Xb = pass == 0 ? Xm : Xp, *Xa = pass == 0 ? Xp : Xm;
                for (int mu = 0; mu < bI; ++mu)
                    for (int nu = 0; nu < bJ; ++nu)
                    {
                        double s = 0.0;
                        for (int i = 0; i < aI; ++i)
                        {
                            const double *x1 = Xb + (rowoff[I] + static_cast<long long>(mu) * aI + i) * nsup +
                                               static_cast<long long>(c) * n_ao + aoff[J];
                            for (int j = 0; j < aJ; ++j)
                                s += x1[j] * Xa[(rowoff[J] + static_cast<long long>(nu) * aJ + j) * nsup +
                                                static_cast<long long>(cm) * n_ao + aoff[I] + i];
                        }
                        acc[static_cast<size_t>(mu) * bJ + nu] += s;
                    }
            }
            double *out = chi0R + static_cast<long long>(c) * e_tot + eoff[pidx[static_cast<size_t>(I) * n_at + J]];
            for (int t = 0; t < bI * bJ; ++t) out[t] += acc[t];
        }
    }
    return 0;
}

} // extern "C"

// ---------------------------------------------------------------------------------------------
// ln det(M) of a batch of matrices by LU with partial pivoting, the E_c determinant of
// epsilon.cpp:489-536 (ScaLAPACK pzgetrf, then sum_i log(+-u_ii) with the sign taken so that
// the real part is positive).  One matrix per OpenMP thread, each factored by a blocked
// right-looking LU; pivots by the largest |Re| + |Im| (LAPACK's izamax rule).
namespace {

constexpr int LU_NB = 32;

// Complex matrices as interleaved (re, im) doubles, row-major n x n.
void lu_logdet_c(int n, double *A, double *out_re, double *out_im)
{
    auto re = [&](int i, int j) -> double & { return A[2 * (static_cast<long long>(i) * n + j)]; };
    auto im = [&](int i, int j) -> double & { return A[2 * (static_cast<long long>(i) * n + j) + 1]; };
    for (int k0 = 0; k0 < n; k0 += LU_NB)
    {
        const int nb = std::min(LU_NB, n - k0), k1 = k0 + nb;
        // panel: columns [k0, k1), rows [k0, n)
        for (int k = k0; k < k1; ++k)
        {
            int p = k;
            double best = -1.0;
            for (int i = k; i < n; ++i)
            {
                const double a = std::fabs(re(i, k)) + std::fabs(im(i, k));
                if (a > best)
                {
                    best = a;
                    p = i;
                }
            }
            if (p != k)
                for (int j = 0; j < 2 * n; ++j) std::swap(A[2LL * p * n + j], A[2LL * k * n + j]);
            const double pr = re(k, k), pi = im(k, k);
            const double den = pr * pr + pi * pi;
            const double ir = den > 0 ? pr / den : 0.0, ii = den > 0 ? -pi / den : 0.0;
            for (int i = k + 1; i < n; ++i)
            {
                const double xr = re(i, k), xi = im(i, k);
                const double lr = xr * ir - xi * ii, li = xr * ii + xi * ir;
                re(i, k) = lr;
                im(i, k) = li;
                double *a = &re(i, k + 1);
                const double *u = &re(k, k + 1);
                const int m = k1 - k - 1;
                for (int j = 0; j < m; ++j)
                {
                    const double ur = u[2 * j], ui = u[2 * j + 1];
                    a[2 * j] -= lr * ur - li * ui;
                    a[2 * j + 1] -= lr * ui + li * ur;
                }
            }
        }
        if (k1 >= n) break;
        // U12 = L11^-1 A12 (unit lower triangular solve), rows [k0, k1), columns [k1, n)
        for (int k = k0; k < k1; ++k)
            for (int i = k + 1; i < k1; ++i)
            {
                const double lr = re(i, k), li = im(i, k);
                double *a = &re(i, k1);
                const double *u = &re(k, k1);
                const int m = n - k1;
                for (int j = 0; j < m; ++j)
                {
                    const double ur = u[2 * j], ui = u[2 * j + 1];
                    a[2 * j] -= lr * ur - li * ui;
                    a[2 * j + 1] -= lr * ui + li * ur;
                }
            }
        // A22 -= L21 U12
        for (int i = k1; i < n; ++i)
            for (int k = k0; k < k1; ++k)
            {
                const double lr = re(i, k), li = im(i, k);
                double *a = &re(i, k1);
                const double *u = &re(k, k1);
                const int m = n - k1;
                for (int j = 0; j < m; ++j)
                {
                    const double ur = u[2 * j], ui = u[2 * j + 1];
                    a[2 * j] -= lr * ur - li * ui;
                    a[2 * j + 1] -= lr * ui + li * ur;
                }
            }
    }
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < n; ++i)
    {
        double dr = re(i, i), di = im(i, i);
        if (!(dr > 0.0))
        {
            dr = -dr;
            di = -di;
        }
        sr += 0.5 * std::log(dr * dr + di * di);
        si += std::atan2(di, dr);
    }
    *out_re = sr;
    *out_im = si;
}

void lu_logdet_r(int n, double *A, double *out)
{
    auto a = [&](int i, int j) -> double & { return A[static_cast<long long>(i) * n + j]; };
    for (int k0 = 0; k0 < n; k0 += LU_NB)
    {
        const int nb = std::min(LU_NB, n - k0), k1 = k0 + nb;
        for (int k = k0; k < k1; ++k)
        {
            int p = k;
            double best = -1.0;
            for (int i = k; i < n; ++i)
                if (std::fabs(a(i, k)) > best)
                {
                    best = std::fabs(a(i, k));
                    p = i;
                }
            if (p != k)
                for (int j = 0; j < n; ++j) std::swap(a(p, j), a(k, j));
            const double inv = a(k, k) != 0.0 ? 1.0 / a(k, k) : 0.0;
            for (int i = k + 1; i < n; ++i)
            {
                const double l = a(i, k) * inv;
                a(i, k) = l;
                for (int j = k + 1; j < k1; ++j) a(i, j) -= l * a(k, j);
            }
        }
        if (k1 >= n) break;
        for (int k = k0; k < k1; ++k)
            for (int i = k + 1; i < k1; ++i)
            {
                const double l = a(i, k);
                for (int j = k1; j < n; ++j) a(i, j) -= l * a(k, j);
            }
        for (int i = k1; i < n; ++i)
            for (int k = k0; k < k1; ++k)
            {
                const double l = a(i, k);
                double *r = &a(i, 0);
                const double *u = &a(k, 0);
#pragma omp simd
                for (int j = k1; j < n; ++j) r[j] -= l * u[j];
            }
    }
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += std::log(std::fabs(a(i, i)));
    *out = s;
}

} // namespace

extern "C" {

// ln det of `batch` n x n matrices stored one after another (complex: interleaved (re, im)),
// overwritten by their LU factors.  out[2 b] = Re, out[2 b + 1] = Im of matrix b's
// sum_i log(+-u_ii).  Returns 0.
int cpu_lu_logdet(int n, int batch, int is_complex, double *A, double *out)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (int b = 0; b < batch; ++b)
    {
        if (is_complex)
            lu_logdet_c(n, A + 2LL * b * n * n, &out[2 * b], &out[2 * b + 1]);
        else
        {
            lu_logdet_r(n, A + static_cast<long long>(b) * n * n, &out[2 * b]);
            out[2 * b + 1] = 0.0;
        }
    }
    return 0;
}

} // extern "C"
