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
    // N: auxiliary-basis size; nw: frequencies handled per call; complex_path: k-point (complex)
    // matrices, otherwise Gamma-only real parts.
    EcChol(int N, int nw, bool complex_path);
    ~EcChol();
    // V: full N x N Coulomb matrix of one q (overwritten by its Cholesky factor); X: nw full
    // chi0(q, w) matrices.  Returns tr(V chi0) and ln det(I - V chi0) per frequency.
    int run_q(void *V, void *X, std::vector<std::complex<double>> &trace, std::vector<std::complex<double>> &logdet,
              cudaStream_t st);

    struct Impl;

private:
    std::unique_ptr<Impl> impl_;
};

} // namespace gb
