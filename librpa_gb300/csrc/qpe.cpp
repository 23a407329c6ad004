#include "qpe.h"

#include <cmath>

#include "common.h"

namespace gb {

PadeContinuation::PadeContinuation(int n_pars, const std::vector<std::complex<double>> &x,
                                   const std::vector<std::complex<double>> &data)
{
    const int n_data = static_cast<int>(data.size());
    GB_REQUIRE(n_data > 0 && x.size() == data.size(), "Pade continuation needs matching, non-empty points and data");
    std::vector<std::complex<double>> d;
    if (n_pars < 0 || n_data <= n_pars)
    {
        par_x_ = x;
        d = data;
    }
    else
    {
        GB_REQUIRE(n_pars >= 2, "Pade continuation needs at least two parameters");
        par_x_.assign(n_pars, std::complex<double>(0.0, 0.0));
        d.assign(n_pars, std::complex<double>(0.0, 0.0));
        const int step = n_data / (n_pars - 1);
        for (int p = 0; p < n_pars - 1; ++p)
        {
            par_x_[p] = x[static_cast<size_t>(p) * step];
            d[p] = data[static_cast<size_t>(p) * step];
        }
        // the last data point; its abscissa is left at zero, as the reference leaves it
        d[n_pars - 1] = data[n_data - 1];
    }
    const int n = static_cast<int>(par_x_.size());
    // Thiele's reciprocal differences: g[i][0] = f_i,
    // g[i][p] = (g[p-1][p-1] - g[i][p-1]) / ((x_i - x_{p-1}) g[i][p-1]); coefficients g[p][p]
    std::vector<std::complex<double>> g(static_cast<size_t>(n) * n);
    for (int i = 0; i < n; ++i) g[static_cast<size_t>(i) * n] = d[i];
    for (int p = 1; p < n; ++p)
        for (int i = p; i < n; ++i)
            g[static_cast<size_t>(i) * n + p] =
                (g[static_cast<size_t>(p - 1) * n + p - 1] - g[static_cast<size_t>(i) * n + p - 1]) /
                ((par_x_[i] - par_x_[p - 1]) * g[static_cast<size_t>(i) * n + p - 1]);
    par_y_.resize(n);
    for (int p = 0; p < n; ++p) par_y_[p] = g[static_cast<size_t>(p) * n + p];
}

std::complex<double> PadeContinuation::operator()(std::complex<double> z) const
{
    std::complex<double> t(1.0, 0.0);
    for (int p = n_pars() - 1; p > 0; --p) t = 1.0 + par_y_[p] * (z - par_x_[p - 1]) / t;
    return par_y_[0] / t;
}

QpeResult solve_qpe(const PadeContinuation &pade, double e_mf, double e_fermi, double vxc, double vexx,
                    double diff_init, double thres, int n_iter_max)
{
    const double escale = 0.1;  // mixing of the residual into the next iterate
    int n_iter = 0;
    double e_last = e_mf, diff = diff_init;
    std::complex<double> sig_last(0.0, 0.0);
    while (n_iter++ < n_iter_max)
    {
        const double e_this = e_last + escale * diff;
        const std::complex<double> sig = pade(std::complex<double>(e_this - e_fermi, 0.0));
        diff = e_mf - vxc + vexx + sig.real() - e_this;
        e_last = e_mf - vxc + vexx + sig.real();
        sig_last = sig;
        if (std::fabs(diff) < thres || n_iter == n_iter_max - 1) break;
    }
    return {n_iter > n_iter_max - 1 ? 1 : 0, e_last, sig_last};
}

} // namespace gb
