// Placeholder translation unit for the tcgen05 chi0 path.
#include "tc_gemm.h"

namespace gb {

struct TcChi0::Impl
{
};

TcChi0::TcChi0(const Geom &, const Pairs &, const double *, cudaStream_t)
{
    GB_FAIL("BF16x3 tensor-core chi0 path not available in this build");
}
TcChi0::~TcChi0() = default;
int TcChi0::run(const double *, const double *, double *, cudaStream_t) { return 0; }

} // namespace gb
