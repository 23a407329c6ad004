// Minimax grids: table lookup + least-squares fit of the cosine/sine
// transformation weights.  The fit solves, for every grid point, the
// over-determined system A w = psi on log-spaced transition energies x in
// [e_min, e_max] with the pseudo-inverse V diag(S/(reg^2+S^2)) U^T, the same
// regularised formula as minimax_grids.F90:366-388.  The SVD is a one-sided
// (Hestenes) Jacobi SVD written here, which keeps high relative accuracy on
// the small singular values of these badly scaled exponential bases.
#include "minimax.h"

#include <dlfcn.h>

#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>
#include <atomic>
#include <mutex>
#include <thread>
#include <sstream>
#include <tuple>

#include "common.h"

namespace gb {

namespace {

struct Table
{
    std::vector<double> erange;
    std::vector<std::vector<double>> cols;  // index 0 .. n_ranges
};

struct Tables
{
    std::map<int, Table> omega, tau;
};

std::mutex g_tab_mu;
std::map<std::string, Tables> g_tab_cache;

const Tables &load_tables(const std::string &path)
{
    std::lock_guard<std::mutex> lk(g_tab_mu);
    auto it = g_tab_cache.find(path);
    if (it != g_tab_cache.end()) return it->second;
    std::ifstream f(path);
    if (!f.good()) GB_FAIL("cannot open minimax table file " + path);
    Tables t;
    Table *cur = nullptr;
    std::string line;
    while (std::getline(f, line))
    {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream ss(line);
        std::string tag;
        ss >> tag;
        if (tag == "table")
        {
            std::string kind;
            int n, nr;
            ss >> kind >> n >> nr;
            auto &m = (kind == "omega") ? t.omega : t.tau;
            cur = &m[n];
            cur->cols.assign(nr + 1, {});
        }
        else if (tag == "erange")
        {
            double v;
            while (ss >> v) cur->erange.push_back(v);
        }
        else if (tag == "col")
        {
            int k;
            ss >> k;
            double v;
            auto &c = cur->cols.at(k - 1);
            while (ss >> v) c.push_back(v);
        }
    }
    return g_tab_cache.emplace(path, std::move(t)).first->second;
}

// get_points_weights_{omega,tau}: choose the energy-range column, rescale.
std::vector<double> coeffs(const std::map<int, Table> &m, bool is_omega, int n, double e_range)
{
    auto it = m.find(n);
    if (it == m.end()) GB_FAIL("unsupported minimax grids size: " + std::to_string(n));
    const Table &t = it->second;
    const int len = static_cast<int>(t.erange.size());
    int idx = len + 1;
    double best = HUGE_VAL;
    for (int j = 1; j <= len; ++j)
    {
        const double v = t.erange[j - 1];
        if (e_range < v && v < best)
        {
            idx = j;
            best = v;
        }
    }
    double e_ratio = 1.0;
    if (idx == 1 && n > 20)
    {
        e_ratio = t.erange[0] / e_range;
        if (e_ratio > 1.5) e_ratio = e_ratio / 1.5;
    }
    std::vector<double> ac = t.cols.at(idx - 1);
    GB_REQUIRE(static_cast<int>(ac.size()) == 2 * n, "corrupt minimax table");
    for (double &v : ac) v = is_omega ? v / e_ratio : v * e_ratio;
    return ac;
}

// One-sided Jacobi SVD of a column-major m x n matrix (m >= n).
// On return A holds U*S (columns), S the column norms, V the right vectors.
void jacobi_svd(std::vector<double> &A, int m, int n, std::vector<double> &S, std::vector<double> &V)
{
    V.assign(static_cast<size_t>(n) * n, 0.0);
    for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
    const double eps = 1e-15;
    for (int sweep = 0; sweep < 80; ++sweep)
    {
        double off = 0.0;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q)
            {
                double *ap = &A[static_cast<size_t>(p) * m];
                double *aq = &A[static_cast<size_t>(q) * m];
                double alpha = 0, beta = 0, gamma = 0;
                for (int i = 0; i < m; ++i)
                {
                    alpha += ap[i] * ap[i];
                    beta += aq[i] * aq[i];
                    gamma += ap[i] * aq[i];
                }
                if (gamma == 0.0) continue;
                const double c0 = std::fabs(gamma) / std::sqrt(alpha * beta);
                if (!(c0 > eps)) continue;
                off = std::fmax(off, c0);
                const double zeta = (beta - alpha) / (2.0 * gamma);
                const double t = std::copysign(1.0, zeta) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / std::sqrt(1.0 + t * t);
                const double s = c * t;
                for (int i = 0; i < m; ++i)
                {
                    const double x = ap[i], y = aq[i];
                    ap[i] = c * x - s * y;
                    aq[i] = s * x + c * y;
                }
                double *vp = &V[static_cast<size_t>(p) * n];
                double *vq = &V[static_cast<size_t>(q) * n];
                for (int i = 0; i < n; ++i)
                {
                    const double x = vp[i], y = vq[i];
                    vp[i] = c * x - s * y;
                    vq[i] = s * x + c * y;
                }
            }
        if (off <= eps) break;
    }
    S.assign(n, 0.0);
    for (int j = 0; j < n; ++j)
    {
        double s2 = 0.0;
        const double *a = &A[static_cast<size_t>(j) * m];
        for (int i = 0; i < m; ++i) s2 += a[i] * a[i];
        S[j] = std::sqrt(s2);
    }
}

// get_transformation_weights for one transform type (1: cos t->w, 2: cos w->t, 3: sin t->w).
// Returns row-major W[i_point * n + j] and the maximal fit error.
std::vector<double> fit_weights(int n, const std::vector<double> &tau, const std::vector<double> &omega,
                                double emin, double emax, int ttype, double reg, double &max_err)
{
    int num_x = (static_cast<int>(std::log10(emax / emin)) + 1) * 200;
    if (num_x < n) num_x = n;
    const double x_factor = std::pow(emax / emin, 1.0 / (static_cast<double>(num_x) - 1.0));
    std::vector<double> x(num_x);
    for (int i = 0; i < num_x; ++i) x[i] = emin * std::pow(x_factor, i);
    std::vector<double> W(static_cast<size_t>(n) * n, 0.0);
    std::vector<double> errs(n, 0.0);
    // the x-dependent factor of the basis functions is the same for every point: exp(-x tau_j)
    // (types 1, 3) or 2 x / (x^2 + omega_j^2) (type 2), [j][i]
    std::vector<double> base(static_cast<size_t>(num_x) * n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < num_x; ++i)
            base[static_cast<size_t>(j) * num_x + i] =
                ttype == 2 ? 2.0 * x[i] / (x[i] * x[i] + omega[j] * omega[j]) : std::exp(-x[i] * tau[j]);
    // one least-squares fit per point ip, independent of the others: spread over host threads
    auto fit_point = [&](int ip) {
        std::vector<double> A(static_cast<size_t>(num_x) * n), psi(num_x), S, V;
        for (int j = 0; j < n; ++j)
        {
            const double f = ttype == 1 ? std::cos(omega[ip] * tau[j])
                                        : ttype == 2 ? std::cos(tau[ip] * omega[j]) : std::sin(omega[ip] * tau[j]);
            for (int i = 0; i < num_x; ++i)
                A[static_cast<size_t>(j) * num_x + i] = f * base[static_cast<size_t>(j) * num_x + i];
        }
        for (int i = 0; i < num_x; ++i)
        {
            if (ttype == 1)
                psi[i] = 2.0 * x[i] / (x[i] * x[i] + omega[ip] * omega[ip]);
            else if (ttype == 2)
                psi[i] = std::exp(-x[i] * tau[ip]);
            else
                psi[i] = 2.0 * omega[ip] / (x[i] * x[i] + omega[ip] * omega[ip]);
        }
        std::vector<double> Ain = A;
        // Householder QR first (A = Q R, psi <- Q^T psi), then the one-sided Jacobi SVD of the
        // n x n factor R = U_r S V^T: the same singular triplets as A's (U = Q U_r) at a sweep cost
        // of n^3 instead of n^2 num_x.
        for (int k = 0; k < n; ++k)
        {
            double *ak = &A[static_cast<size_t>(k) * num_x];
            double nrm = 0.0;
            for (int i = k; i < num_x; ++i) nrm += ak[i] * ak[i];
            nrm = std::sqrt(nrm);
            if (nrm == 0.0) continue;
            const double alpha = ak[k] > 0 ? -nrm : nrm;
            // v = a_k(k:) - alpha e_k, H = I - 2 v v^T / (v^T v)
            const double v0 = ak[k] - alpha;
            const double vtv = nrm * nrm - ak[k] * ak[k] + v0 * v0;
            ak[k] = v0;
            if (vtv > 0.0)
            {
                auto reflect = [&](double *y) {
                    double d = 0.0;
                    for (int i = k; i < num_x; ++i) d += ak[i] * y[i];
                    const double f = 2.0 * d / vtv;
                    for (int i = k; i < num_x; ++i) y[i] -= f * ak[i];
                };
                for (int j = k + 1; j < n; ++j) reflect(&A[static_cast<size_t>(j) * num_x]);
                reflect(psi.data());
            }
            ak[k] = alpha;
        }
        std::vector<double> R(static_cast<size_t>(n) * n, 0.0);
        for (int j = 0; j < n; ++j)
            for (int i = 0; i <= j; ++i) R[static_cast<size_t>(j) * n + i] = A[static_cast<size_t>(j) * num_x + i];
        jacobi_svd(R, n, n, S, V);
        // w = sum_j V[:, j] * S_j/(reg^2+S_j^2) * (u_j . psi),  u_j = A_j / S_j, over the
        // numerical rank: singular values below num_x * eps * S_max are dropped, the rank rule
        // of a least-squares solver.  GreenX keeps them all, which only matters for fits that are
        // singular to double precision (many points over a small energy range, e.g. 32 points
        // at E_max/E_min = 80, where the exp(-x tau) columns are graded down to 1e-150): there its
        // weights are set by LAPACK's rounding, while 1/S of the exact tiny singular values the
        // Jacobi SVD resolves gives weights of 1e30 and beyond.
        double smax = 0.0;
        for (int j = 0; j < n; ++j) smax = std::fmax(smax, S[j]);
        const double s_floor = static_cast<double>(num_x) * 2.220446049250313e-16 * smax;
        std::vector<double> w(n, 0.0);
        for (int j = 0; j < n; ++j)
        {
            if (!(S[j] > s_floor)) continue;
            // u_j . psi = (U_r)_j . (Q^T psi)(0:n)
            double ut = 0.0;
            const double *a = &R[static_cast<size_t>(j) * n];
            for (int i = 0; i < n; ++i) ut += a[i] * psi[i];
            ut /= S[j];
            const double f = S[j] / (reg * reg + S[j] * S[j]) * ut;
            for (int k = 0; k < n; ++k) w[k] += V[static_cast<size_t>(j) * n + k] * f;
        }
        for (int k = 0; k < n; ++k) W[static_cast<size_t>(ip) * n + k] = w[k];
        double e = 0.0;
        for (int i = 0; i < num_x; ++i)
        {
            double fv = 0.0;
            for (int k = 0; k < n; ++k) fv += w[k] * Ain[static_cast<size_t>(k) * num_x + i];
            e = std::fmax(e, std::fabs(psi[i] - fv));
        }
        errs[ip] = e;
    };
    const int nthr = std::max(1, std::min(n, static_cast<int>(std::thread::hardware_concurrency())));
    if (nthr <= 1)
        for (int ip = 0; ip < n; ++ip) fit_point(ip);
    else
    {
        std::atomic<int> next{0};
        std::vector<std::thread> pool;
        for (int t = 0; t < nthr; ++t)
            pool.emplace_back([&] {
                for (int ip = next++; ip < n; ip = next++) fit_point(ip);
            });
        for (std::thread &th : pool) th.join();
    }
    max_err = 0.0;
    for (double e : errs) max_err = std::fmax(max_err, e);
    return W;
}

} // namespace

std::string minimax_table_path()
{
    if (const char *env = std::getenv("LIBRPA_GB300_MINIMAX_TABLES")) return env;
    Dl_info info;
    if (dladdr(reinterpret_cast<void *>(&minimax_table_path), &info) && info.dli_fname)
    {
        std::string so(info.dli_fname);
        auto pos = so.find_last_of('/');
        std::string dir = pos == std::string::npos ? "." : so.substr(0, pos);
        return dir + "/data/greenx_minimax_tables.txt";
    }
    return "data/greenx_minimax_tables.txt";
}

static TimeFreqGrids minimax_grids_uncached(int n, double emin, double emax, double reg);

// The grids are a pure function of (n, e_min, e_max, regularisation): repeated E_c calls on the
// same systems reuse the results of up to 256 windows (a few MB) instead of refitting (the fit
// costs milliseconds to tens of ms); the cache is emptied when it is full.
namespace {
using GridKey = std::tuple<int, double, double, double>;
std::mutex g_grid_mu;
std::map<GridKey, TimeFreqGrids> g_grid_cache;
} // namespace

void clear_grid_cache()
{
    std::lock_guard<std::mutex> lk(g_grid_mu);
    g_grid_cache.clear();
}

TimeFreqGrids minimax_grids(int n, double emin, double emax, double reg)
{
    std::mutex &mu = g_grid_mu;
    std::map<GridKey, TimeFreqGrids> &cache = g_grid_cache;
    const GridKey key{n, emin, emax, reg};
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    TimeFreqGrids g = minimax_grids_uncached(n, emin, emax, reg);
    std::lock_guard<std::mutex> lk(mu);
    if (cache.size() >= 256) cache.clear();
    cache.emplace(key, g);
    return g;
}

static TimeFreqGrids minimax_grids_uncached(int n, double emin, double emax, double reg)
{
    GB_REQUIRE(emin > 0 && emax > emin, "minimax grid needs 0 < e_min < e_max");
    const Tables &t = load_tables(minimax_table_path());
    const double e_range = emax / emin;
    TimeFreqGrids g;
    g.n = n;
    auto ac = coeffs(t.omega, true, n, e_range);
    g.omega.resize(n);
    g.omega_w.resize(n);
    for (int i = 0; i < n; ++i)
    {
        g.omega[i] = ac[i] * emin;
        g.omega_w[i] = ac[n + i] * emin;
    }
    ac = coeffs(t.tau, false, n, e_range);
    g.tau.resize(n);
    g.tau_w.resize(n);
    for (int i = 0; i < n; ++i)
    {
        g.tau[i] = ac[i] / (2.0 * emin);
        g.tau_w[i] = ac[n + i] / (2.0 * emin);
    }
    auto cw = fit_weights(n, g.tau, g.omega, emin, emax, 1, reg, g.max_errors[0]);
    auto ctw = fit_weights(n, g.tau, g.omega, emin, emax, 2, reg, g.max_errors[1]);
    auto sw = fit_weights(n, g.tau, g.omega, emin, emax, 3, reg, g.max_errors[2]);
    g.cos_t2f.resize(static_cast<size_t>(n) * n);
    g.cos_f2t.resize(static_cast<size_t>(n) * n);
    g.sin_t2f.resize(static_cast<size_t>(n) * n);
    for (int iw = 0; iw < n; ++iw)
        for (int it = 0; it < n; ++it)
        {
            const double c = std::cos(g.tau[it] * g.omega[iw]);
            const double s = std::sin(g.tau[it] * g.omega[iw]);
            g.cos_t2f[iw * n + it] = cw[iw * n + it] * c;   // cosft_wt(j=w, i=t)
            g.cos_f2t[it * n + iw] = ctw[it * n + iw] * c;  // cosft_tw(i=t, j=w)
            g.sin_t2f[iw * n + it] = sw[iw * n + it] * s;
        }
    double dual = 0.0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
        {
            double acc = 0.0;
            for (int k = 0; k < n; ++k) acc += g.cos_t2f[i * n + k] * g.cos_f2t[k * n + j];
            if (i == j) acc -= 1.0;
            dual = std::fmax(dual, std::fabs(acc));
        }
    g.cosft_duality_error = dual;
    return g;
}

} // namespace gb
