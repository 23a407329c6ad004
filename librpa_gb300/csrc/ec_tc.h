// Tensor-core + FP64-Cholesky E_c stage (ec_tc.cu).
#pragma once

#include <complex>
#include <memory>
#include <vector>

#include <cuda_runtime.h>

namespace gb {

class EcChol
{
public:
    // N: auxiliary-basis size; nw: frequencies per q; complex_path: k-point (complex) matrices,
    // otherwise Gamma-only real parts; qb: q points whose M' = I - L^H chi0 L are factorised
    // in one batch; fp64_products: M = L^H chi0 L by FP64 CUDA-core GEMMs instead of the
    // split-precision tensor-core GEMMs.
    EcChol(int N, int nw, bool complex_path, int qb, bool fp64_products = false);
    ~EcChol();
    // V = L L^H in place for nb (<= qb) Coulomb matrices stored one after another (N x N each).
    // bad[b] != 0 where V has no Cholesky factor (not positive definite: the Gamma-point bare
    // Coulomb matrix of a real crystal can be indefinite); the caller evaluates those q by
    // the LU form, which needs no definiteness.
    int factor_v(void *V, int nb, std::vector<int> &bad, cudaStream_t st);
    // For batch slot `slot`: M = L^H chi0 L for the nw chi0 matrices X (tensor-core GEMMs),
    // M' = I - M kept for finish(), and tr(V chi0) = tr(M) per frequency.
    int stage_q(const void *L, const void *X, int slot, cudaStream_t st);
    // Batched FP64 Cholesky of the nslots * nw matrices M'; trace[s * nw + w] = tr(V chi0) and
    // logdet[s * nw + w] = ln det(I - V chi0) = 2 sum_i ln L'_ii.
    int finish(int nslots, std::vector<std::complex<double>> &trace, std::vector<std::complex<double>> &logdet,
               cudaStream_t st);

    struct Impl;

private:
    std::unique_ptr<Impl> impl_;
};

} // namespace gb
