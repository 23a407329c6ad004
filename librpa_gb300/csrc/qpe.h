// Quasi-particle equation of G0W0 on the host: Thiele-Pade continuation of the correlation
// self-energy from the imaginary axis and the damped fixed-point solve, as LibRPA does them
// (AnalyContPade, src/core/analycont.cpp:12-70; qpe_solver_pade_self_consistent,
// src/core/qpe_solver.cpp).  Scalar work per state; it stays on the CPU as in the reference.
#pragma once

#include <complex>
#include <vector>

namespace gb {

class PadeContinuation
{
public:
    // n_pars < 0 or >= the number of points: all points; otherwise n_pars points picked at a
    // stride of n/(n_pars - 1), the last one the last data point.
    PadeContinuation(int n_pars, const std::vector<std::complex<double>> &x,
                     const std::vector<std::complex<double>> &data);
    std::complex<double> operator()(std::complex<double> z) const;
    int n_pars() const { return static_cast<int>(par_x_.size()); }

private:
    std::vector<std::complex<double>> par_x_, par_y_;
};

struct QpeResult
{
    int info;                    // 0: converged, 1: iteration limit
    double e_qp;                 // e_mf - vxc + vexx + Re Sigma_c(e_qp - e_fermi)
    std::complex<double> sigc;   // Sigma_c at the last iterate
};

QpeResult solve_qpe(const PadeContinuation &pade, double e_mf, double e_fermi, double vxc, double vexx,
                    double diff_init = 1.0e-3, double thres = 1.0e-5, int n_iter_max = 200);

} // namespace gb
