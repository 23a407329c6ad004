// Block screening kernels and the learned block-norm predictor (forward, backward, Adam).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>

#include "screen.h"

namespace gb {

namespace {

constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + MLP_H * MLP_IN;
constexpr int OFF_W2 = OFF_B1 + MLP_H;
constexpr int OFF_B2 = OFF_W2 + MLP_H * MLP_H;
constexpr int OFF_W3 = OFF_B2 + MLP_H;
constexpr int OFF_B3 = OFF_W3 + MLP_H;
static_assert(OFF_B3 + 1 == MLP_NPARAM, "parameter layout");
constexpr float LOG_FLOOR = -40.0f;  // log10 of an all-zero block

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z)
{
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__device__ __forceinline__ float block_max_warp(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// ---------------------------------------------------------------- block kernels
__global__ void k_g_block_filter(double *__restrict__ G, Geom g, double thr)
{
    const int I = blockIdx.x / g.n_at, J = blockIdx.x % g.n_at;
    const int c = blockIdx.y, sign = blockIdx.z;
    const int ni = g.nao[I], nj = g.nao[J];
    double *B = G + ((static_cast<size_t>(sign) * g.n_c + c) * g.n_ao + g.ao_off[I]) * g.n_ao + g.ao_off[J];
    __shared__ double red[4];
    double m = 0.0;
    for (int t = threadIdx.x; t < ni * nj; t += blockDim.x) m = fmax(m, fabs(B[static_cast<size_t>(t / nj) * g.n_ao + t % nj]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = m;
    __syncthreads();
    m = fmax(fmax(red[0], red[1]), fmax(red[2], red[3]));
    if (m > thr) return;  // kept: max-norm above the threshold
    for (int t = threadIdx.x; t < ni * nj; t += blockDim.x) B[static_cast<size_t>(t / nj) * g.n_ao + t % nj] = 0.0;
}

__global__ void k_block_maxnorm(const double *__restrict__ chi0R, Geom g, Pairs pr, double *__restrict__ norm)
{
    const int p = blockIdx.x / g.n_c, c = blockIdx.x % g.n_c;
    const int bI = g.nabf[pr.I[p]], bJ = g.nabf[pr.J[p]];
    const double *B = chi0R + pr.r_off[p] + static_cast<long long>(c) * bI * bJ;
    __shared__ double red[4];
    double m = 0.0;
    for (int t = threadIdx.x; t < bI * bJ; t += blockDim.x) m = fmax(m, fabs(B[t]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = m;
    __syncthreads();
    if (threadIdx.x == 0) norm[blockIdx.x] = fmax(fmax(red[0], red[1]), fmax(red[2], red[3]));
}

__global__ void k_block_drop(double *__restrict__ chi0R, Geom g, Pairs pr, const double *__restrict__ norm, double thr)
{
    if (norm[blockIdx.x] > thr) return;
    const int p = blockIdx.x / g.n_c, c = blockIdx.x % g.n_c;
    const int bI = g.nabf[pr.I[p]], bJ = g.nabf[pr.J[p]];
    double *B = chi0R + pr.r_off[p] + static_cast<long long>(c) * bI * bJ;
    for (int t = threadIdx.x; t < bI * bJ; t += blockDim.x) B[t] = 0.0;
}

// one warp per (pair, cell) block
__global__ void k_block_features(const double *__restrict__ G, Geom g, Pairs pr, const float *__restrict__ dist,
                                 const float *__restrict__ cmax, const float *__restrict__ kind, float ltau,
                                 float *__restrict__ feat, int n_blk)
{
    const int b = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    if (b >= n_blk) return;
    const int p = b / g.n_c, c = b % g.n_c;
    const int I = pr.I[p], J = pr.J[p];
    const int ni = g.nao[I], nj = g.nao[J];
    float gm[2];
    for (int sign = 0; sign < 2; ++sign)
    {
        const double *B = G + ((static_cast<size_t>(sign) * g.n_c + c) * g.n_ao + g.ao_off[I]) * g.n_ao + g.ao_off[J];
        float m = 0.0f;
        for (int t = lane; t < ni * nj; t += 32) m = fmaxf(m, static_cast<float>(fabs(B[static_cast<size_t>(t / nj) * g.n_ao + t % nj])));
        gm[sign] = block_max_warp(m);
    }
    if (lane == 0)
    {
        float *f = feat + static_cast<size_t>(b) * MLP_IN;
        const float cc = cmax[I] * cmax[J];
        f[0] = dist[b];
        f[1] = ltau;
        f[2] = cc > 0.0f ? log10f(cc) : LOG_FLOOR;
        f[3] = gm[0] > 0.0f ? log10f(gm[0]) : LOG_FLOOR;
        f[4] = gm[1] > 0.0f ? log10f(gm[1]) : LOG_FLOOR;
        f[5] = log10f(static_cast<float>(g.nabf[I]) * static_cast<float>(g.nabf[J]));
        f[6] = log10f(static_cast<float>(ni) * static_cast<float>(nj));
        f[7] = kind[I];
        f[8] = kind[J];
    }
}

// ---------------------------------------------------------------- MLP
// norm: mean[IN], scale[IN], target mean, target scale, margin
__global__ void __launch_bounds__(128) k_mlp_fwd(const __half *__restrict__ W, const float *__restrict__ norm,
                                                 const float *__restrict__ x, int n, float *__restrict__ y)
{
    __shared__ float sW[MLP_NPARAM];
    for (int t = threadIdx.x; t < MLP_NPARAM; t += blockDim.x) sW[t] = __half2float(W[t]);
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float xn[MLP_IN];
#pragma unroll
    for (int f = 0; f < MLP_IN; ++f) xn[f] = (x[static_cast<size_t>(s) * MLP_IN + f] - norm[f]) / norm[MLP_IN + f];
    float h1[MLP_H];
#pragma unroll
    for (int k = 0; k < MLP_H; ++k)
    {
        float z = sW[OFF_B1 + k];
#pragma unroll
        for (int f = 0; f < MLP_IN; ++f) z = fmaf(sW[OFF_W1 + k * MLP_IN + f], xn[f], z);
        h1[k] = gelu(z);
    }
    float out = sW[OFF_B3];
    for (int o = 0; o < MLP_H; ++o)
    {
        float z = sW[OFF_B2 + o];
#pragma unroll
        for (int k = 0; k < MLP_H; ++k) z = fmaf(sW[OFF_W2 + o * MLP_H + k], h1[k], z);
        out = fmaf(sW[OFF_W3 + o], gelu(z), out);
    }
    y[s] = out * norm[2 * MLP_IN + 1] + norm[2 * MLP_IN];
}

// Mean-squared-error gradient over samples [off, off + cnt) of (x, y), scaled by inv_n; one
// thread per sample, 64 samples per block; per-block sums go to grad / loss with atomics.
constexpr int GB = 64;

__global__ void __launch_bounds__(GB) k_mlp_grad(const __half *__restrict__ W, const float *__restrict__ norm,
                                                 const float *__restrict__ x, const float *__restrict__ y, int off,
                                                 int cnt, float inv_n, float *__restrict__ grad,
                                                 float *__restrict__ loss)
{
    __shared__ __half sW[MLP_NPARAM];
    __shared__ float sH1[GB][MLP_H + 1];  // h1, later dz1
    __shared__ float sZ[GB][MLP_H + 1];   // z2, later dz2
    __shared__ float sX[GB][MLP_IN];
    __shared__ float sDY[GB];
    for (int t = threadIdx.x; t < MLP_NPARAM; t += blockDim.x) sW[t] = W[t];
    __syncthreads();
    const int t = threadIdx.x;
    const int s = blockIdx.x * GB + t;
    const bool valid = s < cnt;
    const size_t gs = static_cast<size_t>(off) + (valid ? s : 0);
    float xn[MLP_IN];
#pragma unroll
    for (int f = 0; f < MLP_IN; ++f)
    {
        xn[f] = valid ? (x[gs * MLP_IN + f] - norm[f]) / norm[MLP_IN + f] : 0.0f;
        sX[t][f] = xn[f];
    }
    float z1[MLP_H];
#pragma unroll
    for (int k = 0; k < MLP_H; ++k)
    {
        float z = __half2float(sW[OFF_B1 + k]);
#pragma unroll
        for (int f = 0; f < MLP_IN; ++f) z = fmaf(__half2float(sW[OFF_W1 + k * MLP_IN + f]), xn[f], z);
        z1[k] = z;
        sH1[t][k] = gelu(z);
    }
    float out = __half2float(sW[OFF_B3]);
    for (int o = 0; o < MLP_H; ++o)
    {
        float z = __half2float(sW[OFF_B2 + o]);
#pragma unroll
        for (int k = 0; k < MLP_H; ++k) z = fmaf(__half2float(sW[OFF_W2 + o * MLP_H + k]), sH1[t][k], z);
        sZ[t][o] = z;
        out = fmaf(__half2float(sW[OFF_W3 + o]), gelu(z), out);
    }
    const float tn = valid ? (y[gs] - norm[2 * MLP_IN]) / norm[2 * MLP_IN + 1] : 0.0f;
    const float r = valid ? out - tn : 0.0f;
    const float dy = 2.0f * r * inv_n;
    sDY[t] = dy;
    // loss: block sum of r^2 * inv_n
    {
        float l = r * r * inv_n;
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if (t % 32 == 0) atomicAdd(loss, l);
    }
    __syncthreads();
    // dW3[o] = sum_t dy_t gelu(z2_t[o]), db3 = sum_t dy_t
    {
        const int o = t;
        float a = 0.0f;
        for (int u = 0; u < GB; ++u) a = fmaf(sDY[u], gelu(sZ[u][o]), a);
        atomicAdd(&grad[OFF_W3 + o], a);
        if (t == 0)
        {
            float b = 0.0f;
            for (int u = 0; u < GB; ++u) b += sDY[u];
            atomicAdd(&grad[OFF_B3], b);
        }
    }
    __syncthreads();
    // dz2 (own row)
    for (int o = 0; o < MLP_H; ++o) sZ[t][o] = dy * __half2float(sW[OFF_W3 + o]) * gelu_d(sZ[t][o]);
    __syncthreads();
    // dW2[o][k] = sum_t dz2_t[o] h1_t[k]; db2[o] = sum_t dz2_t[o]
    for (int e = t; e < MLP_H * MLP_H; e += GB)
    {
        const int o = e / MLP_H, k = e % MLP_H;
        float a = 0.0f;
        for (int u = 0; u < GB; ++u) a = fmaf(sZ[u][o], sH1[u][k], a);
        atomicAdd(&grad[OFF_W2 + e], a);
    }
    {
        const int o = t;
        float a = 0.0f;
        for (int u = 0; u < GB; ++u) a += sZ[u][o];
        atomicAdd(&grad[OFF_B2 + o], a);
    }
    __syncthreads();
    // dz1[k] = gelu'(z1[k]) sum_o W2[o][k] dz2[o]  (own row, into sH1)
#pragma unroll
    for (int k = 0; k < MLP_H; ++k)
    {
        float a = 0.0f;
        for (int o = 0; o < MLP_H; ++o) a = fmaf(__half2float(sW[OFF_W2 + o * MLP_H + k]), sZ[t][o], a);
        sH1[t][k] = a * gelu_d(z1[k]);
    }
    __syncthreads();
    // dW1[k][f] = sum_t dz1_t[k] xn_t[f]; db1[k] = sum_t dz1_t[k]
    {
        const int k = t;
        float a[MLP_IN] = {};
        float b = 0.0f;
        for (int u = 0; u < GB; ++u)
        {
            const float d = sH1[u][k];
            b += d;
#pragma unroll
            for (int f = 0; f < MLP_IN; ++f) a[f] = fmaf(d, sX[u][f], a[f]);
        }
#pragma unroll
        for (int f = 0; f < MLP_IN; ++f) atomicAdd(&grad[OFF_W1 + k * MLP_IN + f], a[f]);
        atomicAdd(&grad[OFF_B1 + k], b);
    }
}

__global__ void k_adam(float *__restrict__ p, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ g, float lr, float c1, float c2, __half *__restrict__ W16)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_NPARAM) return;
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
    p[i] = pi;
    W16[i] = __float2half_rn(pi);
}

__global__ void k_to_half(const float *__restrict__ p, __half *__restrict__ W16, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) W16[i] = __float2half_rn(p[i]);
}

} // namespace

// ---------------------------------------------------------------- launches
void launch_g_block_filter(double *G, const Geom &g, double thr, cudaStream_t st)
{
    dim3 grid(static_cast<unsigned>(g.n_at * g.n_at), static_cast<unsigned>(g.n_c), 2);
    k_g_block_filter<<<grid, 128, 0, st>>>(G, g, thr);
    GB_LAUNCH_CHECK();
}

void launch_block_maxnorm(const double *chi0R, const Geom &g, const Pairs &pr, double *norm, cudaStream_t st)
{
    k_block_maxnorm<<<pr.n_pairs * g.n_c, 128, 0, st>>>(chi0R, g, pr, norm);
    GB_LAUNCH_CHECK();
}

void launch_block_drop(double *chi0R, const Geom &g, const Pairs &pr, const double *norm, double thr, cudaStream_t st)
{
    k_block_drop<<<pr.n_pairs * g.n_c, 128, 0, st>>>(chi0R, g, pr, norm, thr);
    GB_LAUNCH_CHECK();
}

void launch_block_features(const double *G, const Geom &g, const Pairs &pr, const float *dist, const float *cmax,
                           const float *kind, double tau, float *feat, cudaStream_t st)
{
    const int n_blk = pr.n_pairs * g.n_c;
    k_block_features<<<(n_blk + 3) / 4, 128, 0, st>>>(G, g, pr, dist, cmax, kind, static_cast<float>(std::log10(tau)),
                                                      feat, n_blk);
    GB_LAUNCH_CHECK();
}

void mlp_predict(const ScreenModel &m, const float *d_x, int n, float *d_y, cudaStream_t st)
{
    GB_REQUIRE(m.trained && static_cast<int>(m.params.size()) == MLP_NPARAM &&
                   static_cast<int>(m.norm.size()) == MLP_NNORM,
               "the screening model is not trained");
    if (n == 0) return;
    DevBuf<float> p(MLP_NPARAM), nrm(MLP_NNORM);
    DevBuf<__half> w(MLP_NPARAM);
    p.upload(m.params.data(), MLP_NPARAM, st);
    nrm.upload(m.norm.data(), MLP_NNORM, st);
    k_to_half<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(p.get(), w.get(), MLP_NPARAM);
    GB_LAUNCH_CHECK();
    k_mlp_fwd<<<(n + 127) / 128, 128, 0, st>>>(w.get(), nrm.get(), d_x, n, d_y);
    GB_LAUNCH_CHECK();
    GB_CUDA(cudaStreamSynchronize(st));
}

double mlp_loss_grad(const float *params, const float *norm, const float *x, const float *y, int n, float *grad,
                     cudaStream_t st)
{
    GB_REQUIRE(n > 0, "empty batch");
    DevBuf<float> p(MLP_NPARAM), nrm(MLP_NNORM), dx(static_cast<size_t>(n) * MLP_IN), dy(n), g(MLP_NPARAM), l(1);
    DevBuf<__half> w(MLP_NPARAM);
    p.upload(params, MLP_NPARAM, st);
    nrm.upload(norm, MLP_NNORM, st);
    dx.upload(x, static_cast<size_t>(n) * MLP_IN, st);
    dy.upload(y, n, st);
    g.zero(st);
    l.zero(st);
    k_to_half<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(p.get(), w.get(), MLP_NPARAM);
    GB_LAUNCH_CHECK();
    k_mlp_grad<<<(n + GB - 1) / GB, GB, 0, st>>>(w.get(), nrm.get(), dx.get(), dy.get(), 0, n, 1.0f / n, g.get(), l.get());
    GB_LAUNCH_CHECK();
    float hl = 0.0f;
    g.download(grad, MLP_NPARAM, st);
    l.download(&hl, 1, st);
    GB_CUDA(cudaStreamSynchronize(st));
    return hl;
}

void mlp_train(ScreenModel &m, const std::vector<float> &x, const std::vector<float> &y, int iterations, double lr,
               unsigned long long seed, cudaStream_t st)
{
    const size_t n = y.size();
    GB_REQUIRE(n >= 16 && x.size() == n * MLP_IN, "too few logged samples to train the screening model");
    // normalisation
    std::vector<float> norm(MLP_NNORM, 0.0f);
    for (int f = 0; f < MLP_IN; ++f)
    {
        double s = 0, s2 = 0;
        for (size_t i = 0; i < n; ++i)
        {
            s += x[i * MLP_IN + f];
            s2 += static_cast<double>(x[i * MLP_IN + f]) * x[i * MLP_IN + f];
        }
        const double mu = s / n, var = std::max(0.0, s2 / n - mu * mu);
        norm[f] = static_cast<float>(mu);
        norm[MLP_IN + f] = static_cast<float>(std::max(std::sqrt(var), 1e-3));
    }
    {
        double s = 0, s2 = 0;
        for (size_t i = 0; i < n; ++i)
        {
            s += y[i];
            s2 += static_cast<double>(y[i]) * y[i];
        }
        const double mu = s / n, var = std::max(0.0, s2 / n - mu * mu);
        norm[2 * MLP_IN] = static_cast<float>(mu);
        norm[2 * MLP_IN + 1] = static_cast<float>(std::max(std::sqrt(var), 1e-3));
    }
    // shuffled copy of the samples
    std::mt19937_64 rng(seed);
    std::vector<size_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    std::shuffle(perm.begin(), perm.end(), rng);
    std::vector<float> xs(n * MLP_IN), ys(n);
    for (size_t i = 0; i < n; ++i)
    {
        ys[i] = y[perm[i]];
        for (int f = 0; f < MLP_IN; ++f) xs[i * MLP_IN + f] = x[perm[i] * MLP_IN + f];
    }
    // He-style initialisation
    std::vector<float> params(MLP_NPARAM, 0.0f);
    std::normal_distribution<double> nd(0.0, 1.0);
    for (int i = 0; i < MLP_H * MLP_IN; ++i) params[OFF_W1 + i] = static_cast<float>(nd(rng) * std::sqrt(2.0 / MLP_IN));
    for (int i = 0; i < MLP_H * MLP_H; ++i) params[OFF_W2 + i] = static_cast<float>(nd(rng) * std::sqrt(2.0 / MLP_H));
    for (int i = 0; i < MLP_H; ++i) params[OFF_W3 + i] = static_cast<float>(nd(rng) * std::sqrt(1.0 / MLP_H));
    DevBuf<float> dx(xs.size()), dyv(n), p(MLP_NPARAM), mm(MLP_NPARAM), vv(MLP_NPARAM), g(MLP_NPARAM), nrm(MLP_NNORM),
        l(1), pred(n);
    DevBuf<__half> w(MLP_NPARAM);
    dx.upload(xs.data(), xs.size(), st);
    dyv.upload(ys.data(), n, st);
    p.upload(params.data(), MLP_NPARAM, st);
    nrm.upload(norm.data(), MLP_NNORM, st);
    mm.zero(st);
    vv.zero(st);
    k_to_half<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(p.get(), w.get(), MLP_NPARAM);
    GB_LAUNCH_CHECK();
    const int batch = static_cast<int>(std::min<size_t>(n, 16384));
    size_t off = 0;
    double b1t = 1.0, b2t = 1.0;
    for (int it = 0; it < iterations; ++it)
    {
        if (off + batch > n) off = 0;
        g.zero(st);
        l.zero(st);
        k_mlp_grad<<<(batch + GB - 1) / GB, GB, 0, st>>>(w.get(), nrm.get(), dx.get(), dyv.get(), static_cast<int>(off),
                                                          batch, 1.0f / batch, g.get(), l.get());
        GB_LAUNCH_CHECK();
        b1t *= 0.9;
        b2t *= 0.999;
        const double lr_t = lr * (it < iterations / 2 ? 1.0 : 0.1);  // one step decay
        k_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(p.get(), mm.get(), vv.get(), g.get(), static_cast<float>(lr_t),
                                                          static_cast<float>(1.0 - b1t), static_cast<float>(1.0 - b2t),
                                                          w.get());
        GB_LAUNCH_CHECK();
        off += batch;
    }
    // residuals over every sample set the decision margin
    k_mlp_fwd<<<static_cast<unsigned>((n + 127) / 128), 128, 0, st>>>(w.get(), nrm.get(), dx.get(), static_cast<int>(n),
                                                                      pred.get());
    GB_LAUNCH_CHECK();
    std::vector<float> hp(n);
    pred.download(hp.data(), n, st);
    p.download(params.data(), MLP_NPARAM, st);
    GB_CUDA(cudaStreamSynchronize(st));
    double se = 0.0;
    for (size_t i = 0; i < n; ++i) se += (hp[i] - ys[i]) * static_cast<double>(hp[i] - ys[i]);
    const double rmse = std::sqrt(se / n);
    norm[2 * MLP_IN + 2] = static_cast<float>(std::max(0.5, 3.0 * rmse));
    m.params = params;
    m.norm = norm;
    m.trained = true;
    m.train_rmse = rmse;
}

} // namespace gb
