// G_k(tau) products on the tensor cores (reduced-precision chi0 paths only).
#pragma once

#include <cuComplex.h>

#include "common.h"
#include "tc_gemm.h"

namespace gb {

// G[sign][cell][i][j] = sgn Re sum_k exp(-i th_kc) sum_n psi_ni(k) s_n conj(psi_nj(k)) with the
// band sum as one split-precision (3 BF16 pieces, 6 products) tcgen05 GEMM per (sign, k):
// rows (Re | Im part, i) against columns j over K = (Re, Im) x band, each scaled by sqrt(s_n).
class GkTc
{
public:
    // psi_real: every wave-function coefficient is real (the Im half of K is dropped).
    GkTc(int nk, int nb, int nao, bool psi_real);
    // psi: this spin's [k][n][i]; s: [sign][k][n] from launch_tau_scale; cos/sin: [k][cell]
    // phase tables.  Returns kernels launched.
    int run(const cuDoubleComplex *psi, const double *s, const double *cosph, const double *sinph, int nc,
            double *G, int *err, cudaStream_t st);

private:
    int nk_, nb_, nao_, parts_, kw_;
    long long kpad_;
    SplitStore a_;
    DevBuf<float> d_;
};

} // namespace gb
