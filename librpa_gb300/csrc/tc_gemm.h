// tcgen05 (5th-generation tensor core) chi0 path: BF16 3-term split products,
// FP32 accumulation in TMEM, operands staged to shared memory by TMA.
#pragma once

#include <memory>

#include "common.h"
#include "kernels.h"

namespace gb {

class TcChi0
{
public:
    TcChi0(const Geom &g, const Pairs &pr, const double *C, cudaStream_t st);
    ~TcChi0();
    // G (both signs, [sign][cell][i][j]) and the supercell G -> chi0(R) upper-pair blocks.
    int run(const double *Gs, const double *G, double *chi0R, cudaStream_t st);

    struct Impl;

private:
    std::unique_ptr<Impl> impl_;
};

} // namespace gb
