#include "dielec.h"

#include <algorithm>
#include <cmath>

#include "common.h"

namespace gb {
namespace {

// The cubic spline of src/math/interpolate.cpp:9-67, with the steps in the order the reference
// takes them: the elimination and the back substitution of the tridiagonal system share one loop,
// so a back-substitution step that comes before the elimination has reached its row reads that
// row's z as zero.  Pieces a_i + b_i t + c_i t^2 + d_i t^3, t = x - x_i.
struct Spline
{
    std::vector<double> x, a, b, c, d;

    Spline(const std::vector<double> &xs, const std::vector<double> &ys) : x(xs), a(ys)
    {
        const int n = static_cast<int>(xs.size());
        GB_REQUIRE(n >= 2 && ys.size() == xs.size(),
                   "cubic spline: at least 2 points, with one value per point");
        std::vector<double> h(n - 1), slope3(n - 1), l(n, 1.0), mu(n - 1, 0.0), z(n, 0.0);
        for (int i = 0; i + 1 < n; ++i)
        {
            h[i] = xs[i + 1] - xs[i];
            slope3[i] = 3.0 * (ys[i + 1] - ys[i]) / h[i];
        }
        for (int i = 1; i + 1 < n; ++i)
        {
            l[i] = 2.0 * (xs[i + 1] - xs[i - 1]) - h[i - 1] * mu[i - 1];
            mu[i] = h[i] / l[i];
        }
        c.assign(n, 0.0);
        for (int i = 1; i < n; ++i)
        {
            z[i] = (slope3[i - 1] - h[i - 1] * z[i - 1]) / l[i];
            const int r = n - 1 - i;
            c[r] = z[r + 1] - mu[r] * c[r + 1];
        }
        b.assign(n, 0.0);
        d.assign(n, 0.0);
        for (int i = 0; i + 1 < n; ++i)
        {
            b[i] = (ys[i + 1] - ys[i]) / h[i] - h[i] * (c[i + 1] + 2.0 * c[i]) / 3.0;
            d[i] = (c[i + 1] - c[i]) / (3.0 * h[i]);
        }
    }

    // interpolate.cpp:70-139: inside [x_0, x_{n-1}] the first piece whose interval holds u;
    // outside, the cubic in t = u - x_0 built from the values and slopes of the two end points
    // of the nearer end interval.
    double operator()(double u) const
    {
        const int n = static_cast<int>(x.size());
        if (u < x[0] || u > x[n - 1])
        {
            const int i0 = u < x[0] ? 0 : n - 2;
            const double h = x[i0 + 1] - x[i0], t = u - x[i0];
            const double dy = a[i0 + 1] - a[i0], m0 = b[i0], dm = b[i0 + 1] - b[i0];
            const double h2 = h * h, h3 = h2 * h;
            return a[i0] + m0 * t + (3.0 * dy / h2 - 2.0 * m0 / h - dm / h) * t * t +
                   (-2.0 * dy / h3 + m0 / h2 + dm / h2) * t * t * t;
        }
        for (int i = 0; i + 1 < n; ++i)
            if (u >= x[i] && u <= x[i + 1])
            {
                const double t = u - x[i];
                return a[i] + b[i] * t + c[i] * t * t + d[i] * t * t * t;
            }
        return 0.0;
    }
};

// The two-term Havriliak-Negami model on the imaginary axis and its parameter gradient
// (dielecmodel.cpp:34-63): p = (e1, a1, b1, t1, e2, a2, b2, t2).
constexpr int kHnPars = 8;

double hn_value(double u, const double *p)
{
    return 1.0 + (p[0] - 1.0) / std::pow(1.0 + std::pow(u * p[3], p[1]), p[2]) +
           (p[4] - 1.0) / std::pow(1.0 + std::pow(u * p[7], p[5]), p[6]);
}

void hn_gradient(double u, const double *p, double *g)
{
    for (int t = 0; t < 2; ++t)
    {
        const double *q = p + 4 * t;   // e, a, b, tau of this term
        double *gq = g + 4 * t;
        const double s = u * q[3], sa = std::pow(s, q[1]), base = 1.0 + sa;
        gq[0] = 1.0 / std::pow(base, q[2]);
        // d/da and d/dtau of (e - 1) base^-b
        const double dbase = (q[0] - 1.0) * (-q[2]) / std::pow(base, q[2] + 1.0);
        gq[1] = dbase * std::log(s) * sa;
        gq[2] = (1.0 - q[0]) * std::log(base) / std::pow(base, q[2]);
        gq[3] = dbase * q[1] / q[3] * sa;
    }
}

double sq_error(const std::vector<double> &p, const std::vector<double> &xs, const std::vector<double> &ys)
{
    double e = 0.0;
    for (size_t i = 0; i < ys.size(); ++i)
    {
        const double r = hn_value(xs[i], p.data()) - ys[i];
        e += r * r;
    }
    return e;
}

// Lower Cholesky factor of the symmetric matrix whose lower triangle is a (n x n, row-major);
// false when a pivot falls below 1e-30 (fitting.cpp:36-60).
bool cholesky_lower(int n, const std::vector<double> &a, std::vector<double> &l)
{
    for (int i = 0; i < n; ++i)
    {
        for (int j = 0; j < i; ++j)
        {
            double s = 0.0;
            for (int k = 0; k < j; ++k) s += l[i * n + k] * l[j * n + k];
            l[i * n + j] = (a[i * n + j] - s) / l[j * n + j];
        }
        double s = 0.0;
        for (int k = 0; k < i; ++k) s += l[i * n + k] * l[i * n + k];
        s = a[i * n + i] - s;
        if (s < 1e-30) return false;
        l[i * n + i] = std::sqrt(s);
    }
    return true;
}

void cholesky_solve(int n, const std::vector<double> &l, const std::vector<double> &rhs, std::vector<double> &x)
{
    for (int i = 0; i < n; ++i)
    {
        double s = 0.0;
        for (int j = 0; j < i; ++j) s += l[i * n + j] * x[j];
        x[i] = (rhs[i] - s) / l[i * n + i];
    }
    for (int i = n - 1; i >= 0; --i)
    {
        double s = 0.0;
        for (int j = i + 1; j < n; ++j) s += l[j * n + i] * x[j];
        x[i] = (x[i] - s) / l[i * n + i];
    }
}

// Levenberg-Marquardt as src/math/fitting.cpp:90-199 runs it: at most 10000 iterations, damping
// lambda from 0.1, times 10 after a rejected step (a rejection also counts as an iteration) and
// divided by 10 after an accepted one; the damped normal matrix is J^T J with its diagonal scaled
// by (1 + lambda); the fit stops after an accepted step that lowers the squared error by less
// than 1e-8.
void fit_hn(std::vector<double> &p, const std::vector<double> &xs, const std::vector<double> &ys)
{
    const int np = kHnPars, max_iter = 10000;
    const double up = 10.0, down = 0.1, target = 1e-8;
    double lambda = 0.1;
    double err = sq_error(p, xs, ys), new_err = 0.0, derr = 0.0;
    std::vector<double> jtj(np * np), chol(np * np, 0.0), jtr(np), g(np), step(np), trial(np, 0.0);
    for (int it = 0; it < max_iter; ++it)
    {
        std::fill(jtj.begin(), jtj.end(), 0.0);
        std::fill(jtr.begin(), jtr.end(), 0.0);
        for (size_t k = 0; k < xs.size(); ++k)
        {
            hn_gradient(xs[k], p.data(), g.data());
            const double r = ys[k] - hn_value(xs[k], p.data());
            for (int i = 0; i < np; ++i)
            {
                jtr[i] += r * g[i];
                for (int j = 0; j <= i; ++j) jtj[i * np + j] += g[i] * g[j];
            }
        }
        // the diagonal is scaled in place, by (1 + lambda) first and by the ratio of the new and
        // old factors after each rejection
        double mult = 1.0 + lambda;
        bool rejected = true;
        while (rejected && it < max_iter)
        {
            for (int i = 0; i < np; ++i) jtj[i * np + i] *= mult;
            rejected = !cholesky_lower(np, jtj, chol);
            if (!rejected)
            {
                cholesky_solve(np, chol, jtr, step);
                for (int i = 0; i < np; ++i) trial[i] = p[i] + step[i];
                new_err = sq_error(trial, xs, ys);
                derr = new_err - err;
                rejected = derr > 0.0;
            }
            if (rejected)
            {
                mult = (1.0 + lambda * up) / (1.0 + lambda);
                lambda *= up;
                ++it;
            }
        }
        p = trial;
        err = new_err;
        lambda *= down;
        if (!rejected && -derr < target) break;
    }
}

} // namespace

std::vector<double> interpolate_dielec_func(int option, const std::vector<double> &omega_in,
                                            const std::vector<double> &eps_in,
                                            const std::vector<double> &omega_target)
{
    GB_REQUIRE(omega_in.size() == eps_in.size(), "dielectric function: one value per frequency");
    std::vector<double> out(omega_target.size());
    switch (option)
    {
    case 0:
        GB_REQUIRE(eps_in.size() == omega_target.size(),
                   "option_dielect_func = 0: the dielectric function must be given at the nfreq minimax frequencies");
        return eps_in;
    case 1:
    {
        const Spline s(omega_in, eps_in);
        for (size_t i = 0; i < out.size(); ++i) out[i] = s(omega_target[i]);
        return out;
    }
    case 2:
    {
        GB_REQUIRE(!eps_in.empty(), "option_dielect_func = 2: no dielectric function to fit");
        std::vector<double> p(kHnPars, 1.0);
        p[0] = p[4] = eps_in[0];
        fit_hn(p, omega_in, eps_in);
        for (size_t i = 0; i < out.size(); ++i) out[i] = hn_value(omega_target[i], p.data());
        return out;
    }
    default:
        GB_FAIL("option_dielect_func: 0 (given values), 1 (spline) or 2 (model fit) on this path");
    }
}

} // namespace gb
