// Exercises include/librpa.hpp (the C++ interface) against the C API it wraps: option defaults,
// an input error turned into an exception, and (argument "gpu") one E_c of a tiny Gamma-point
// system through the wrapper and through the C API on a second handler, which must agree.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "librpa.hpp"

namespace {

int fail(const char *what)
{
    std::fprintf(stderr, "FAIL: %s\n", what);
    return 1;
}

// One atom, 3 NAOs, 4 ABFs, 3 states (1 occupied), Gamma only: fixed numbers, no randomness.
struct Tiny
{
    int nao = 3, nabf = 4, nb = 3;
    std::vector<double> wg{2.0, 0.0, 0.0}, ekb{-0.5, 0.3, 0.9};
    std::vector<double> wr{0.8, 0.5, 0.33, -0.5, 0.8, 0.33, 0.33, 0.0, -0.94}, wi = std::vector<double>(9, 0.0);
    std::vector<double> cs, vr, vi;
    Tiny()
    {
        for (int t = 0; t < nao * nao * nabf; ++t) cs.push_back(0.1 * std::cos(0.7 * t) + (t % 5 == 0 ? 0.2 : 0.0));
        for (int a = 0; a < nabf; ++a)
            for (int b = 0; b < nabf; ++b)
            {
                vr.push_back(a == b ? 2.0 + a : 0.1 / (1 + a + b));
                vi.push_back(0.0);
            }
    }
};

void load_cpp(librpa::Handler &h, const Tiny &t)
{
    h.set_scf_dimension(1, 1, t.nb, t.nao);
    h.set_wg_ekb_efermi(1, 1, t.nb, t.wg.data(), t.ekb.data(), 0.0);
    h.set_wfc(0, 0, t.nb, t.nao, t.wr.data(), t.wi.data());
    h.set_ao_basis_wfc({static_cast<size_t>(t.nao)});
    h.set_ao_basis_aux({static_cast<size_t>(t.nabf)});
    const int R[3] = {0, 0, 0};
    h.set_lri_coeff(LIBRI, 0, 0, t.nao, t.nao, t.nabf, R, t.cs.data());
    h.set_aux_bare_coulomb_k_atom_pair(0, 0, 0, t.nabf, t.nabf, t.vr.data(), t.vi.data(), 0.0);
}

void load_c(LibrpaHandler *h, const Tiny &t)
{
    const size_t nw = t.nao, na = t.nabf;
    librpa_set_scf_dimension(h, 1, 1, t.nb, t.nao, 1);
    librpa_set_wg_ekb_efermi(h, 1, 1, t.nb, t.wg.data(), t.ekb.data(), 0.0);
    librpa_set_wfc(h, 0, 0, t.nb, t.nao, t.wr.data(), t.wi.data());
    librpa_set_ao_basis_wfc(h, 1, &nw);
    librpa_set_ao_basis_aux(h, 1, &na);
    const int R[3] = {0, 0, 0};
    librpa_set_lri_coeff(h, LIBRI, 0, 0, t.nao, t.nao, t.nabf, R, t.cs.data());
    librpa_set_aux_bare_coulomb_k_atom_pair(h, 0, 0, 0, t.nabf, t.nabf, t.vr.data(), t.vi.data(), 0.0);
}

} // namespace

int main(int argc, char **argv)
{
    const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
    librpa::Options o;
    LibrpaOptions c;
    librpa_init_options(&c);
    if (std::memcmp(static_cast<LibrpaOptions *>(&o), &c, sizeof(c)) != 0) return fail("Options defaults");
    if (librpa::get_major_version() != librpa_get_major_version()) return fail("version");

    librpa::Handler h(MPI_COMM_WORLD);
    bool threw = false;
    try
    {
        // RI block before the bases: the C API records an error, the wrapper throws it
        const int R[3] = {0, 0, 0};
        std::vector<double> cs(12, 0.0);
        h.set_lri_coeff(LIBRI, 0, 0, 2, 2, 3, R, cs.data());
    }
    catch (const std::runtime_error &e)
    {
        threw = std::strstr(e.what(), "basis") != nullptr;
    }
    if (!threw) return fail("input error not thrown");

    const Tiny t;
    load_cpp(h, t);
    o.nfreq = 6;
    o.tfgrids_type = Minimax;
    std::vector<std::complex<double>> per_q(1);
    double ec = 0.0;
    try
    {
        ec = h.get_rpa_correlation_energy(o, per_q);
    }
    catch (const std::runtime_error &e)
    {
        if (gpu) return fail(e.what());
        if (!std::strstr(e.what(), "CUDA")) return fail("no-GPU error message");
        std::printf("OK no-gpu: %s\n", e.what());
        return 0;
    }
    if (!gpu) return fail("E_c without a GPU");
    LibrpaHandler *hc = librpa_create_handler(MPI_COMM_WORLD);
    load_c(hc, t);
    double re = 0, im = 0;
    const double ec_c = librpa_get_rpa_correlation_energy(hc, &o, 1, &re, &im);
    librpa_destroy_handler(hc);
    if (!(std::isfinite(ec) && ec == ec_c && per_q[0].real() == re && per_q[0].imag() == im))
        return fail("wrapper E_c differs from the C API's");
    if (!(ec < 0.0)) return fail("E_c not negative");
    std::printf("OK gpu: E_c = %.12f\n", ec);
    return 0;
}
