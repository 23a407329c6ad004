// Reduced-precision chi0 paths.
//
// FP32: the FP64 algebra of k_chi0_simt.cu with FP32 operands (SIMT).
// BF16X3: the two GEMM-shaped stages on the 5th-generation tensor cores
// (tcgen05.mma with TMEM accumulators, operands staged by TMA), each FP64
// operand split as hi + lo BF16 and the product formed from three terms
// (hi*hi + hi*lo + lo*hi) with FP32 accumulation; see k_tc_gemm.cu.
#include "chi0_fast.h"

#include "tc_gemm.h"
#include "../../include/librpa_gb300.h"

namespace gb {

struct Chi0Fast::Impl
{
    int prec;
    Geom g;
    Pairs pr;
    // FP32 path
    DevBuf<float> Cf, Gsf, Xf, Gf;
    // BF16x3 path
    std::unique_ptr<TcChi0> tc;
};

Chi0Fast::Chi0Fast(int precision, const Geom &g, const Pairs &pr, const double *C, cudaStream_t st)
    : impl_(std::make_unique<Impl>())
{
    Impl &m = *impl_;
    m.prec = precision;
    m.g = g;
    m.pr = pr;
    const long long nsup = g.n_sup;
    if (precision == LIBRPA_GB300_CHI0_FP32)
    {
        m.Cf.alloc(static_cast<size_t>(g.rows_c) * nsup);
        launch_d2f(C, m.Cf.get(), g.rows_c * nsup, st);
        m.Gsf.alloc(2ull * nsup * nsup);
        m.Xf.alloc(2ull * g.rows_c * nsup);
        m.Gf.alloc(2ull * g.n_c * g.n_ao * g.n_ao);
    }
    else if (precision == LIBRPA_GB300_CHI0_BF16X3)
    {
        m.tc = std::make_unique<TcChi0>(g, pr, C, st);
    }
    else
        GB_FAIL("unknown chi0 precision mode " + std::to_string(precision));
}

Chi0Fast::~Chi0Fast() = default;

TcChi0 *Chi0Fast::tensor_path() { return impl_->tc.get(); }

int Chi0Fast::run(const double *Gs, const double *Gp, const double *Gm, double *chi0R, cudaStream_t st)
{
    Impl &m = *impl_;
    const Geom &g = m.g;
    const long long nsup = g.n_sup;
    if (m.prec == LIBRPA_GB300_CHI0_FP32)
    {
        launch_d2f(Gs, m.Gsf.get(), 2 * nsup * nsup, st);
        launch_sgemm(static_cast<int>(g.rows_c), static_cast<int>(nsup), static_cast<int>(nsup), m.Cf.get(), nsup, 0,
                     m.Gsf.get(), nsup, nsup * nsup, m.Xf.get(), nsup, g.rows_c * nsup, 2, st);
        const long long ng = static_cast<long long>(g.n_c) * g.n_ao * g.n_ao;
        (void)Gm;
        launch_d2f(Gp, m.Gf.get(), 2 * ng, st);  // Gp and Gm are contiguous: [sign][cell][i][j]
        launch_chi0_fp32(m.Xf.get(), m.Xf.get() + g.rows_c * nsup, m.Cf.get(), m.Gf.get(), m.Gf.get() + ng, g, m.pr,
                         chi0R, st);
        return 4;
    }
    return m.tc->run(Gs, Gp, chi0R, st);
}

} // namespace gb
