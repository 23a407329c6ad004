// Reduced-precision chi0 contraction paths (selected by LibrpaGB300Options.chi0_precision).
#pragma once

#include <memory>

#include "common.h"
#include "kernels.h"

namespace gb {

class Chi0Fast
{
public:
    // C is the FP64 RI matrix [(I,mu,i)][(cell,K,k)] already scattered on the device.
    Chi0Fast(int precision, const Geom &g, const Pairs &pr, const double *C, cudaStream_t st);
    ~Chi0Fast();
    // One (tau, spin): from the supercell G (both signs) and the unit-cell G blocks,
    // write chi0(R, tau) upper-pair blocks (FP64) to chi0R.  Returns kernels launched.
    int run(const double *Gs, const double *Gp, const double *Gm, double *chi0R, cudaStream_t st);
    // The tensor-core path (nullptr for the FP32 CUDA-core path), for block screening.
    class TcChi0 *tensor_path();

    struct Impl;

private:
    std::unique_ptr<Impl> impl_;
};

} // namespace gb
