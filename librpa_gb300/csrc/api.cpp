// C ABI of the GB300 RPA library: the LibRPA entry points of librpa.h with
// the same names, arguments and copy semantics, plus the additive GB300
// extensions of librpa_gb300.h.  No C++ exception crosses this boundary:
// every entry catches, records the message on the handler (and process-wide),
// and returns NaN / a nonzero status / nothing, as its signature allows.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <limits>
#include <atomic>
#include <thread>
#include <algorithm>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/librpa.h"
#include "chol.h"
#include "common.h"
#include "dataset.h"
#include "dielec.h"
#include "screen.h"
#include "host_tables.h"
#include "minimax.h"
#include "gw.h"
#include "qpe.h"
#include "tc_gemm.h"

namespace {

using gb::cplx;
using gb::Dataset;

std::mutex g_mu;
std::vector<std::unique_ptr<Dataset>> g_instances(1);  // slot 0 is a sentinel (instance_manager.cpp:15-57)
std::string g_last_error;
int g_last_code = 0;

Dataset *get_ds(LibrpaHandler *h)
{
    if (!h) GB_FAIL("null handler");
    const int id = h->instance_id_;
    std::lock_guard<std::mutex> lk(g_mu);
    if (id <= 0 || id >= static_cast<int>(g_instances.size()) || !g_instances[id]) GB_FAIL("invalid handler");
    return g_instances[id].get();
}

void record_error(LibrpaHandler *h, const std::string &msg)
{
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_last_error = msg;
        g_last_code = 1;
    }
    if (h)
    {
        const int id = h->instance_id_;
        std::lock_guard<std::mutex> lk(g_mu);
        if (id > 0 && id < static_cast<int>(g_instances.size()) && g_instances[id])
        {
            g_instances[id]->last_error = msg;
            g_instances[id]->last_error_code = 1;
        }
    }
    std::fprintf(stderr, "librpa_gb300 error: %s\n", msg.c_str());
}

void clear_error(Dataset *ds)
{
    ds->last_error.clear();
    ds->last_error_code = 0;
}

// Runs one API call: the handler's error state then reflects this call alone (the last-error
// contract: code 0 when the last call on h succeeded).
template <typename F>
void guarded(LibrpaHandler *h, F &&f)
{
    if (h)
    {
        const int id = h->instance_id_;
        std::lock_guard<std::mutex> lk(g_mu);
        if (id > 0 && id < static_cast<int>(g_instances.size()) && g_instances[id])
        {
            g_instances[id]->last_error.clear();
            g_instances[id]->last_error_code = 0;
        }
    }
    try
    {
        f();
    }
    catch (const std::exception &e)
    {
        record_error(h, e.what());
    }
    catch (...)
    {
        record_error(h, "unknown error");
    }
}

// MeanField::get_E_min_max / get_band_gap (meanfield.cpp:151-197) on the stored data.
void e_min_max(const Dataset &ds, double &emin, double &emax)
{
    double lb = std::numeric_limits<double>::max(), ub = std::numeric_limits<double>::min();
    double homo = -1e6, lumo = 1e6;
    const int nk = ds.n_kpts, nb = ds.n_states;
    for (int s = 0; s < ds.n_spins; ++s)
    {
        for (int k = 0; k < nk; ++k)
        {
            lb = std::min(lb, ds.ekb[(static_cast<size_t>(s) * nk + k) * nb]);
            ub = std::max(ub, ds.ekb[(static_cast<size_t>(s) * nk + k) * nb + nb - 1]);
        }
        const double midpoint = 1.0 / (ds.n_spins * nk * ds.n_spinor);
        for (int k = 0; k < nk; ++k)
        {
            int hl = -1;
            for (int n = 0; n < nb; ++n)
                if (ds.wg[(static_cast<size_t>(s) * nk + k) * nb + n] >= midpoint) hl = n;
            GB_REQUIRE(hl + 1 < nb, "no unoccupied state: cannot define the band gap");
            lumo = std::min(lumo, ds.ekb[(static_cast<size_t>(s) * nk + k) * nb + hl + 1]);
            if (hl != -1) homo = std::max(homo, ds.ekb[(static_cast<size_t>(s) * nk + k) * nb + hl]);
        }
    }
    emin = lumo - homo;
    emax = ub - lb;
}

gb::TimeFreqGrids make_grids(const Dataset &ds, const LibrpaOptions &o)
{
    // TFGrids::generate (timefreq.cpp:117-154): the Gauss-Legendre / Chebyshev cases
    // fall through to the minimax branch in LibRPA, so they produce minimax grids too.
    switch (o.tfgrids_type)
    {
    case GaussLegendre:
    case GaussChebyshevI:
    case GaussChebyshevII:
    case Minimax:
    {
        double emin_mf = 0, emax_mf = 0;
        if (o.minimax_emin <= 0 || o.minimax_emax <= 0)
        {
            GB_REQUIRE(ds.occ_set, "occupations/eigenvalues needed for the minimax energy window");
            e_min_max(ds, emin_mf, emax_mf);
        }
        const double emax = o.minimax_emax > 0 ? o.minimax_emax : emax_mf;
        const double emin = o.minimax_emin > 0 ? o.minimax_emin : emin_mf;
        return gb::minimax_grids(o.nfreq, emin, emax, o.minimax_regulation);
    }
    case EvenSpaced_TF:
    {
        // generate_evenspaced_tf (timefreq.cpp:173-191): uniform nodes, diagonal "transform"
        GB_REQUIRE(o.tfgrids_freq_min > 0 && o.tfgrids_time_min > 0, "emin/tmin must be positive");
        gb::TimeFreqGrids g;
        const int n = o.nfreq;
        g.n = n;
        g.tau.resize(n);
        g.tau_w.resize(n);
        g.omega.resize(n);
        g.omega_w.resize(n);
        g.cos_t2f.assign(static_cast<size_t>(n) * n, 0.0);
        g.cos_f2t.assign(static_cast<size_t>(n) * n, 0.0);
        g.sin_t2f.assign(static_cast<size_t>(n) * n, 0.0);
        const double w = 1.0 / n;
        for (int i = 0; i < n; ++i)
        {
            g.omega[i] = o.tfgrids_freq_min + o.tfgrids_freq_interval * i;
            g.omega_w[i] = w;
            g.tau[i] = o.tfgrids_time_min + o.tfgrids_time_interval * i;
            g.tau_w[i] = w;
            g.cos_t2f[i * n + i] = w;
            g.sin_t2f[i * n + i] = w;
            g.cos_f2t[i * n + i] = 1.0 / w;
        }
        return g;
    }
    case EvenSpaced:
        GB_FAIL("even-spaced frequency grids have no time grid: the conventional chi0 method is not part of this build");
    default:
        GB_FAIL("requested time-frequency grid is not implemented");
    }
}

const char *kBuildInfo =
    "librpa-gb300 1.0.0: space-time RPA correlation energy on NVIDIA GB300 (sm_103a), "
    "C++17 host + hand-written CUDA kernels; built " __DATE__ " " __TIME__;

void set_wfc_impl(Dataset *ds, int ispin, int isoc, int ik, int nstates_local, int nbasis_local,
                  const double *re, const double *im, const double *ri)
{
    GB_REQUIRE(ds->n_spins > 0, "call librpa_set_scf_dimension first");
    GB_REQUIRE(ispin >= 0 && ispin < ds->n_spins && ik >= 0 && ik < ds->n_kpts, "spin or k index out of range");
    GB_REQUIRE(nstates_local == ds->n_states && nbasis_local == ds->n_ao,
               "distributed (local) eigenvector blocks are not supported: pass all states and basis functions");
    const size_t n = static_cast<size_t>(ds->n_states) * ds->n_ao;
    const size_t base = ((static_cast<size_t>(ispin) * ds->n_spinor + isoc) * ds->n_kpts + ik) * n;
    for (size_t i = 0; i < n; ++i)
        ds->wfc[base + i] = ri ? cplx(ri[2 * i], ri[2 * i + 1]) : cplx(re[i], im[i]);
    ds->wfc_set[(static_cast<size_t>(ispin) * ds->n_spinor + isoc) * ds->n_kpts + ik] = 1;
}

// One Coulomb store: the bare matrix (V of chi0 and of the dielectric function) or the truncated
// one (exchange and W); both are kept as (ik, I, J) blocks.
struct VqStore
{
    std::vector<cplx> &blob;
    std::vector<gb::VqBlock> &blocks;
    std::map<std::array<int, 3>, size_t> &index;
    std::vector<gb::Vq2DBlock> &blocks_2d;
};
VqStore bare_store(Dataset *ds) { return {ds->vq_blob, ds->vq_blocks, ds->vq_index, ds->vq_2d}; }
VqStore cut_store(Dataset *ds) { return {ds->vq_cut_blob, ds->vq_cut_blocks, ds->vq_cut_index, ds->vq_cut_2d}; }

void add_vq_block(VqStore st, int ik, int I, int J, int nmu, int nnu, const double *re, const double *im, double thr)
{
    // input.cpp:556-581: keep the block if max |Re V| >= threshold
    double mx = 0.0;
    const size_t n = static_cast<size_t>(nmu) * nnu;
    for (size_t t = 0; t < n; ++t) mx = std::max(mx, std::fabs(re[t]));
    if (!(mx >= thr)) return;
    std::array<int, 3> key{ik, I, J};
    auto it = st.index.find(key);
    if (it != st.index.end() && st.blocks[it->second].nmu == nmu && st.blocks[it->second].nnu == nnu)
    {
        const size_t off = st.blocks[it->second].offset;
        for (size_t t = 0; t < n; ++t) st.blob[off + t] = cplx(re[t], im[t]);
        return;
    }
    gb::VqBlock b{ik, I, J, nmu, nnu, st.blob.size()};
    for (size_t t = 0; t < n; ++t) st.blob.emplace_back(re[t], im[t]);
    st.index[key] = st.blocks.size();
    st.blocks.push_back(b);
}

void add_vq_block(Dataset *ds, int ik, int I, int J, int nmu, int nnu, const double *re, const double *im,
                  double thr)
{
    add_vq_block(bare_store(ds), ik, I, J, nmu, nnu, re, im, thr);
}

// Redistribute 2D-block Coulomb input into atom-pair blocks (Dataset::redistribute_coulomb_blacs2ap).
void merge_vq_2d(Dataset *ds, VqStore st, const std::vector<int> &nabf);
void merge_vq_2d(Dataset *ds, bool shrink = false)
{
    merge_vq_2d(ds, bare_store(ds), shrink ? ds->shrink_nabf : ds->nabf_at);
    merge_vq_2d(ds, cut_store(ds), ds->nabf_at);
}

// nabf: the ABF basis the 2D matrices are given in (the small one of the ABF shrink for the bare
// Coulomb matrix with use_shrink_abfs)
void merge_vq_2d(Dataset *ds, VqStore st, const std::vector<int> &nabf)
{
    if (st.blocks_2d.empty()) return;
    const int nat = static_cast<int>(nabf.size());
    GB_REQUIRE(nat > 0, "auxiliary basis needed to use 2D-block Coulomb input");
    std::vector<int> off(nat + 1, 0);
    for (int I = 0; I < nat; ++I) off[I + 1] = off[I] + nabf[I];
    const int N = off[nat];
    std::map<int, std::vector<cplx>> full;
    for (const auto &b : st.blocks_2d)
    {
        GB_REQUIRE(b.mu_begin >= 0 && b.mu_end <= N && b.nu_begin >= 0 && b.nu_end <= N,
                   "2D Coulomb block outside the auxiliary basis");
        auto &M = full[b.ik];
        if (M.empty()) M.assign(static_cast<size_t>(N) * N, cplx(0, 0));
        const int nr = b.mu_end - b.mu_begin, ncl = b.nu_end - b.nu_begin;
        for (int r = 0; r < nr; ++r)
            for (int c = 0; c < ncl; ++c)
                M[static_cast<size_t>(b.mu_begin + r) * N + b.nu_begin + c] = b.data[static_cast<size_t>(r) * ncl + c];
    }
    for (auto &kv : full)
        for (int I = 0; I < nat; ++I)
            for (int J = I; J < nat; ++J)
            {
                const int nmu = nabf[I], nnu = nabf[J];
                std::vector<double> re(static_cast<size_t>(nmu) * nnu), im(re.size());
                for (int a = 0; a < nmu; ++a)
                    for (int b = 0; b < nnu; ++b)
                    {
                        const cplx v = kv.second[static_cast<size_t>(off[I] + a) * N + off[J] + b];
                        re[static_cast<size_t>(a) * nnu + b] = v.real();
                        im[static_cast<size_t>(a) * nnu + b] = v.imag();
                    }
                add_vq_block(st, kv.first, I, J, nmu, nnu, re.data(), im.data(), -1.0);
            }
    st.blocks_2d.clear();
}

} // namespace

extern "C" {

// ------------------------------------------------------------------ global
const char *librpa_get_build_info(void) { return kBuildInfo; }
int librpa_get_major_version(void) { return 1; }
int librpa_get_minor_version(void) { return 0; }
int librpa_get_patch_version(void) { return 0; }
void librpa_init_global(LibrpaSwitch, const char *, LibrpaSwitch) {}
void librpa_finalize_global(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto &p : g_instances)
        if (p) gb::release_kept(*p);
}

void librpa_print_profile(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (size_t i = 1; i < g_instances.size(); ++i)
    {
        if (!g_instances[i]) continue;
        const auto &s = g_instances[i]->stats;
        std::printf("librpa_gb300 profile (handler %zu)\n", i);
        std::printf("  total %.6f s | grids %.6f | upload %.6f | G %.6f | chi0 %.6f | FT+CT %.6f | E_c %.6f\n",
                    s.t_total, s.t_grids, s.t_upload, s.t_gf, s.t_chi0, s.t_ftct, s.t_ec);
        std::printf("  chi0 FLOP %.4e (LibRI order %.4e) | E_c FLOP %.4e | launches %lld\n", s.chi0_flops,
                    s.chi0_flops_libri, s.ec_flops, s.n_launches);
    }
}

void librpa_test(void)
{
    guarded(nullptr, [&] {
        const auto g = gb::minimax_grids(16, 0.25, 25.0, 0.0);
        std::printf("librpa_gb300 self-test: minimax(16) duality error %.3e, CUDA devices %d\n",
                    g.cosft_duality_error, gb::device_count());
    });
}

// ------------------------------------------------------------------ options
void librpa_init_options(LibrpaOptions *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    librpa_set_output_dir(o, ".");
    o->parallel_routing = AUTO;
    o->output_level = LIBRPA_VERBOSE_INFO;
    o->vq_threshold = 0.0;
    o->use_kpara_scf_eigvec = LIBRPA_SWITCH_OFF;
    o->tfgrids_type = TFGRID_UNSET;
    o->nfreq = 6;
    o->tfgrids_freq_min = 0.005;
    o->tfgrids_freq_interval = 0.0;
    o->tfgrids_freq_max = 1000.0;
    o->tfgrids_time_min = 0.005;
    o->tfgrids_time_interval = 0.0;
    o->minimax_emin = -1.0;
    o->minimax_emax = -1.0;
    o->minimax_regulation = 0.0;
    o->use_fullcoul_eps = LIBRPA_SWITCH_ON;
    o->use_fullcoul_exx = LIBRPA_SWITCH_OFF;
    o->use_fullcoul_wc = LIBRPA_SWITCH_OFF;
    o->n_bands_chi0 = -1;
    o->n_bands_sigc = -1;
    o->gf_threshold = 0.0;
    o->use_scalapack_ecrpa = LIBRPA_SWITCH_ON;
    o->use_shrink_abfs = LIBRPA_SWITCH_OFF;
    o->use_shrink_chi = LIBRPA_SWITCH_OFF;
    o->n_params_anacon = -1;
    o->use_scalapack_gw_wc = LIBRPA_SWITCH_ON;
    o->use_cholesky_gw_wc = LIBRPA_SWITCH_OFF;
    o->replace_w_head = LIBRPA_SWITCH_OFF;
    o->option_dielect_func = 0;
    o->use_2d_dielectric = LIBRPA_SWITCH_OFF;
    o->sqrt_coulomb_threshold = 0.0;
    o->load_sigc_from_file = LIBRPA_SWITCH_OFF;
    o->libri_chi0_threshold_C = 0.0;
    o->libri_chi0_threshold_G = 0.0;
    o->libri_exx_threshold_C = 0.0;
    o->libri_exx_threshold_D = 0.0;
    o->libri_exx_threshold_V = 0.0;
    o->libri_g0w0_threshold_C = 0.0;
    o->libri_g0w0_threshold_G = 0.0;
    o->libri_g0w0_threshold_Wc = 0.0;
    o->output_gw_sigc_mat = LIBRPA_SWITCH_OFF;
    o->output_gw_sigc_mat_rt = LIBRPA_SWITCH_OFF;
    o->output_gw_sigc_mat_rf = LIBRPA_SWITCH_OFF;
    o->option_output_Wc_Rf_mat = 0;
}

void librpa_set_output_dir(LibrpaOptions *o, const char *dir)
{
    if (!o || !dir) return;
    std::string s(dir);
    if (s.empty() || s.back() != '/') s += '/';
    std::strncpy(o->output_dir, s.c_str(), LIBRPA_MAX_STRLEN - 1);
    o->output_dir[LIBRPA_MAX_STRLEN - 1] = '\0';
}

// ------------------------------------------------------------------ handler
LibrpaHandler *librpa_create_handler(MPI_Comm)
{
    try
    {
        std::lock_guard<std::mutex> lk(g_mu);
        g_instances.push_back(std::make_unique<Dataset>());
        const int id = static_cast<int>(g_instances.size()) - 1;
        librpa_gb300_init_options(&g_instances[id]->gbopt);
        return new LibrpaHandler{id};
    }
    catch (const std::exception &e)
    {
        record_error(nullptr, e.what());
        return nullptr;
    }
}

void librpa_destroy_handler(LibrpaHandler *h)
{
    if (!h) return;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        const int id = h->instance_id_;
        if (id > 0 && id < static_cast<int>(g_instances.size()) && g_instances[id])
        {
            gb::release_kept(*g_instances[id]);
            g_instances[id].reset();
        }
    }
    delete h;
}

// ------------------------------------------------------------------ input
void librpa_set_scf_dimension(LibrpaHandler *h, int nspins, int nkpts, int nstates, int nbasis, int nspinor)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(nspins > 0 && nkpts > 0 && nstates > 0 && nbasis > 0 && (nspinor == 1 || nspinor == 2),
                   "invalid mean-field dimensions");
        ds->n_spins = nspins;
        ds->n_kpts = nkpts;
        ds->n_states = nstates;
        ds->n_ao = nbasis;
        ds->n_spinor = nspinor;
        ds->wg.assign(static_cast<size_t>(nspins) * nkpts * nstates, 0.0);
        ds->ekb.assign(ds->wg.size(), 0.0);
        ds->wfc.assign(static_cast<size_t>(nspins) * nspinor * nkpts * nstates * nbasis, cplx(0, 0));
        ds->wfc_set.assign(static_cast<size_t>(nspins) * nspinor * nkpts, 0);
        ds->occ_set = false;
        clear_error(ds);
    });
}

void librpa_set_wg_ekb_efermi(LibrpaHandler *h, int nspins, int nkpts, int nstates, const double *wg,
                              const double *ekb, double efermi)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(nspins == ds->n_spins && nkpts == ds->n_kpts && nstates == ds->n_states,
                   "dimensions differ from librpa_set_scf_dimension");
        const size_t n = static_cast<size_t>(nspins) * nkpts * nstates;
        for (size_t i = 0; i < n; ++i)
        {
            ds->wg[i] = wg[i] / nkpts;  // input.cpp:82
            ds->ekb[i] = ekb[i];
        }
        ds->efermi = efermi;
        ds->occ_set = true;
    });
}

void librpa_set_wfc(LibrpaHandler *h, int ispin, int ik, int ns_loc, int nb_loc, const double *re, const double *im)
{
    guarded(h, [&] { Dataset *ds = get_ds(h); ds->generation++; set_wfc_impl(ds, ispin, 0, ik, ns_loc, nb_loc, re, im, nullptr); });
}

void librpa_set_wfc_spinor(LibrpaHandler *h, int ik, int ns_loc, int nb_loc, const double *ur, const double *ui,
                           const double *dr, const double *di)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(ds->n_spinor == 2, "spinor wfc set requires n_spinor initialized to 2");
        set_wfc_impl(ds, 0, 0, ik, ns_loc, nb_loc, ur, ui, nullptr);
        set_wfc_impl(ds, 0, 1, ik, ns_loc, nb_loc, dr, di, nullptr);
    });
}

void librpa_set_wfc_packed(LibrpaHandler *h, int ispin, int ik, int ns_loc, int nb_loc, const double *ri)
{
    guarded(h, [&] { Dataset *ds = get_ds(h); ds->generation++; set_wfc_impl(ds, ispin, 0, ik, ns_loc, nb_loc, nullptr, nullptr, ri); });
}

void librpa_set_wfc_spinor_packed(LibrpaHandler *h, int ik, int ns_loc, int nb_loc, const double *u, const double *d)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(ds->n_spinor == 2, "spinor wfc set requires n_spinor initialized to 2");
        set_wfc_impl(ds, 0, 0, ik, ns_loc, nb_loc, nullptr, nullptr, u);
        set_wfc_impl(ds, 0, 1, ik, ns_loc, nb_loc, nullptr, nullptr, d);
    });
}

void librpa_set_ao_basis_wfc(LibrpaHandler *h, int natoms, const size_t *nbs)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(natoms > 0, "natoms must be positive");
        ds->nao_at.assign(nbs, nbs + natoms);
    });
}

void librpa_set_ao_basis_aux(LibrpaHandler *h, int natoms, const size_t *nbs)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(natoms > 0, "natoms must be positive");
        ds->nabf_at.assign(nbs, nbs + natoms);
    });
}

// ABF shrink inputs.  The reference keeps them in Dataset::basis_aux_shrink and Dataset::sinvS
// (src/api/dataset.h:67-88); its driver reads them from Cs_shrinked_data_* and shrink_sinvS_*
// (driver/read_data.cpp:2455-2622).  They are read per call, so no staged input is invalidated.
void librpa_gb300_set_shrink_basis(LibrpaHandler *h, int natoms, const size_t *nbs_aux_small)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(natoms > 0 && nbs_aux_small, "natoms must be positive and the counts given");
        ds->shrink_nabf.assign(nbs_aux_small, nbs_aux_small + natoms);
    });
}

void librpa_gb300_set_shrink_sinvS(LibrpaHandler *h, int ik, int n_small, int n_large, const double *re,
                                   const double *im)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(ik >= 0 && n_small > 0 && n_large > 0 && re, "invalid shrink transform arguments");
        Dataset::ShrinkU &u = ds->shrink_u[ik];
        u.n_small = n_small;
        u.n_large = n_large;
        const size_t n = static_cast<size_t>(n_small) * n_large;
        u.u.resize(n);
        for (size_t t = 0; t < n; ++t) u.u[t] = cplx(re[t], im ? im[t] : 0.0);
    });
}

void librpa_set_latvec_and_G(LibrpaHandler *h, const double lat[9], const double G[9])
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        for (int i = 0; i < 9; ++i)
        {
            ds->latvec[i] = lat[i];
            ds->recvec[i] = G[i] / (2.0 * M_PI);  // pbc.cpp:76
        }
        ds->latt_set = true;
    });
}

void librpa_set_atoms(LibrpaHandler *h, int natoms, const int *types, const double *pos)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        ds->types.assign(types, types + natoms);
        ds->positions.assign(pos, pos + 3 * natoms);
    });
}

void librpa_set_kgrids_kvec(LibrpaHandler *h, int nk1, int nk2, int nk3, const double *kvecs)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(nk1 > 0 && nk2 > 0 && nk3 > 0, "k grid must be positive");
        ds->period[0] = nk1;
        ds->period[1] = nk2;
        ds->period[2] = nk3;
        const int nk = nk1 * nk2 * nk3;
        ds->klist.resize(3ull * nk);
        ds->kfrac.resize(3ull * nk);
        for (int k = 0; k < nk; ++k)
        {
            double kv[3];
            for (int d = 0; d < 3; ++d) kv[d] = kvecs[3 * k + d] / (2.0 * M_PI);
            for (int d = 0; d < 3; ++d) ds->klist[3 * k + d] = kv[d];
            // kfrac = latvec * kvec with -0 cleanup (pbc.cpp:96-100)
            for (int a = 0; a < 3; ++a)
            {
                double f = ds->latvec[3 * a] * kv[0] + ds->latvec[3 * a + 1] * kv[1] + ds->latvec[3 * a + 2] * kv[2];
                if (std::fabs(f) < 1e-8) f = 0.0;
                ds->kfrac[3 * k + a] = f;
            }
        }
        ds->ibz_map.resize(nk);
        for (int k = 0; k < nk; ++k) ds->ibz_map[k] = k;
    });
}

void librpa_set_ibz_mapping(LibrpaHandler *h, int nkpts, const int *map)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(nkpts == ds->period[0] * ds->period[1] * ds->period[2],
                   "irk_point_id_mapping size not equal to n_k_points");
        for (int k = 0; k < nkpts; ++k) GB_REQUIRE(map[k] >= 0 && map[k] < nkpts, "IBZ mapping index out of range");
        ds->ibz_map.assign(map, map + nkpts);
    });
}

namespace {
// One RI block (I, J, R) copied into a block store, replacing an earlier block of the same key.
void store_cs_block(std::vector<double> &blob, std::vector<gb::CsBlock> &blocks,
                    std::map<std::array<int, 5>, size_t> &index, int I, int J, int ni, int nj, int nmu,
                    const int R[3], const double *Cs)
{
    const size_t n = static_cast<size_t>(ni) * nj * nmu;
    std::array<int, 5> key{I, J, R[0], R[1], R[2]};
    auto it = index.find(key);
    if (it != index.end())
    {
        std::memcpy(&blob[blocks[it->second].offset], Cs, n * sizeof(double));
        return;
    }
    gb::CsBlock b{I, J, {R[0], R[1], R[2]}, ni, nj, nmu, blob.size()};
    blob.insert(blob.end(), Cs, Cs + n);
    index[key] = blocks.size();
    blocks.push_back(b);
}
} // namespace

void librpa_set_lri_coeff(LibrpaHandler *h, LibrpaParallelRouting, int I, int J, int ni, int nj, int nmu,
                          const int R[3], const double *Cs)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        // input.cpp:497-500
        GB_REQUIRE(!ds->nao_at.empty(), "wave function basis not set, call (librpa_)set_ao_basis_wfc first");
        GB_REQUIRE(!ds->nabf_at.empty(), "auxiliary basis not set, call (librpa_)set_ao_basis_aux first");
        GB_REQUIRE(I >= 0 && J >= 0 && I < static_cast<int>(ds->nao_at.size()) && J < static_cast<int>(ds->nao_at.size()),
                   "atom index out of range");
        GB_REQUIRE(ds->nabf_at[I] == nmu && ds->nao_at[I] == ni && ds->nao_at[J] == nj, "RI block dimensions inconsistent");
        store_cs_block(ds->cs_blob, ds->cs_blocks, ds->cs_index, I, J, ni, nj, nmu, R, Cs);
    });
}

void librpa_gb300_set_shrink_lri_coeff(LibrpaHandler *h, int I, int J, int ni, int nj, int nmu, const int R[3],
                                       const double *Cs)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(!ds->nao_at.empty(), "wave function basis not set, call (librpa_)set_ao_basis_wfc first");
        GB_REQUIRE(!ds->shrink_nabf.empty(), "small auxiliary basis not set, call librpa_gb300_set_shrink_basis first");
        GB_REQUIRE(R && Cs, "null argument");
        GB_REQUIRE(I >= 0 && J >= 0 && I < static_cast<int>(ds->nao_at.size()) && J < static_cast<int>(ds->nao_at.size()) &&
                       I < static_cast<int>(ds->shrink_nabf.size()),
                   "atom index out of range");
        GB_REQUIRE(ds->shrink_nabf[I] == nmu && ds->nao_at[I] == ni && ds->nao_at[J] == nj,
                   "RI block dimensions inconsistent with the small basis");
        store_cs_block(ds->shrink_cs_blob, ds->shrink_cs_blocks, ds->shrink_cs_index, I, J, ni, nj, nmu, R, Cs);
    });
}

void librpa_set_aux_bare_coulomb_k_atom_pair(LibrpaHandler *h, int ik, int I, int J, int nmu, int nnu,
                                             const double *re, const double *im, double thr)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(ik >= 0 && ik < static_cast<int>(ds->ibz_map.size()) || ds->klist.empty(), "k index out of range");
        add_vq_block(ds, ik, I, J, nmu, nnu, re, im, thr);
    });
}

void librpa_set_aux_cut_coulomb_k_atom_pair(LibrpaHandler *h, int ik, int I, int J, int nmu, int nnu,
                                            const double *re, const double *im, double thr)
{
    // input.cpp:584-610: the truncated Coulomb blocks, stored like the bare ones
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        GB_REQUIRE(ik >= 0 && ik < static_cast<int>(ds->ibz_map.size()) || ds->klist.empty(), "k index out of range");
        add_vq_block(cut_store(ds), ik, I, J, nmu, nnu, re, im, thr);
    });
}

void librpa_set_aux_bare_coulomb_k_2d_block(LibrpaHandler *h, int ik, int mb, int me, int nb_, int ne,
                                            const double *re, const double *im)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        const int nr = me - mb, ncl = ne - nb_;
        if (nr < 1 || ncl < 1) return;
        gb::Vq2DBlock b{ik, mb, me, nb_, ne, {}};
        b.data.resize(static_cast<size_t>(nr) * ncl);
        for (size_t t = 0; t < b.data.size(); ++t) b.data[t] = cplx(re[t], im[t]);
        ds->vq_2d.push_back(std::move(b));
    });
}

void librpa_set_aux_cut_coulomb_k_2d_block(LibrpaHandler *h, int ik, int mb, int me, int nb_, int ne,
                                           const double *re, const double *im)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        const int nr = me - mb, ncl = ne - nb_;
        if (nr < 1 || ncl < 1) return;
        gb::Vq2DBlock b{ik, mb, me, nb_, ne, {}};
        b.data.resize(static_cast<size_t>(nr) * ncl);
        for (size_t t = 0; t < b.data.size(); ++t) b.data[t] = cplx(re[t], im[t]);
        ds->vq_cut_2d.push_back(std::move(b));
    });
}

void librpa_set_dielect_func_imagfreq(LibrpaHandler *h, int nfreq, const double *om, const double *eps)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h); ds->generation++;
        ds->dielect_omega.assign(om, om + nfreq);
        ds->dielect_eps.assign(eps, eps + nfreq);
    });
}

// Band-point inputs (input.cpp:710-820).  They do not enter the k-grid results (H_x(R),
// Sigma_c(R)), so they leave those valid: no generation change.
void librpa_set_band_kvec(LibrpaHandler *h, int n, const double *kf)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(n > 0 && kf, "band k-points: count and coordinates required");
        ds->band_kfrac.assign(kf, kf + 3 * n);
    });
}

void librpa_set_band_occ_eigval(LibrpaHandler *h, int ns, int nk, int nst, const double *occ, const double *eig)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(ns > 0 && nk > 0 && nst > 0 && occ && eig, "band occupations: dimensions and data required");
        const size_t n = static_cast<size_t>(ns) * nk * nst;
        ds->band_occ.assign(occ, occ + n);
        ds->band_eig.assign(eig, eig + n);
        // occupations scaled by 1 / n_kpts_band as the SCF ones (input.cpp:755)
        for (double &o : ds->band_occ) o /= nk;
        ds->band_ns = ns;
        ds->band_nk = nk;
        ds->band_nst = nst;
        ds->band_wfc.assign(n * static_cast<size_t>(ds->n_ao), cplx(0, 0));
    });
}

void librpa_set_wfc_band(LibrpaHandler *h, int ispin, int ik, int nst, int nbas, const double *re, const double *im)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(ds->band_nk > 0, "band eigenvectors: call librpa_set_band_occ_eigval first");
        GB_REQUIRE(ispin >= 0 && ispin < ds->band_ns && ik >= 0 && ik < ds->band_nk && nst == ds->band_nst &&
                       nbas == ds->n_ao && re && im,
                   "band eigenvectors: indices or dimensions differ from librpa_set_band_occ_eigval / the SCF basis");
        const size_t n = static_cast<size_t>(nst) * nbas;
        cplx *dst = ds->band_wfc.data() + (static_cast<size_t>(ispin) * ds->band_nk + ik) * n;
        for (size_t t = 0; t < n; ++t) dst[t] = cplx(re[t], im[t]);
    });
}

void librpa_set_wfc_band_spinor(LibrpaHandler *h, int, int, int, const double *, const double *, const double *,
                                const double *)
{
    guarded(h, [&] { GB_FAIL("spinor (SOC) wave functions are not supported by the GPU G0W0 and exchange path"); });
}

void librpa_set_wfc_band_packed(LibrpaHandler *h, int ispin, int ik, int nst, int nbas, const double *ri)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(ds->band_nk > 0, "band eigenvectors: call librpa_set_band_occ_eigval first");
        GB_REQUIRE(ispin >= 0 && ispin < ds->band_ns && ik >= 0 && ik < ds->band_nk && nst == ds->band_nst &&
                       nbas == ds->n_ao && ri,
                   "band eigenvectors: indices or dimensions differ from librpa_set_band_occ_eigval / the SCF basis");
        const size_t n = static_cast<size_t>(nst) * nbas;
        cplx *dst = ds->band_wfc.data() + (static_cast<size_t>(ispin) * ds->band_nk + ik) * n;
        for (size_t t = 0; t < n; ++t) dst[t] = cplx(ri[2 * t], ri[2 * t + 1]);
    });
}

void librpa_set_wfc_band_spinor_packed(LibrpaHandler *h, int, int, int, const double *, const double *)
{
    guarded(h, [&] { GB_FAIL("spinor (SOC) wave functions are not supported by the GPU G0W0 and exchange path"); });
}

void librpa_reset_band_data(LibrpaHandler *h)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        ds->band_kfrac.clear();
        ds->band_occ.clear();
        ds->band_eig.clear();
        ds->band_wfc.clear();
        ds->band_ns = ds->band_nk = ds->band_nst = 0;
    });
}

// ------------------------------------------------------------------ compute
void librpa_get_imaginary_frequency_grids(LibrpaHandler *h, const LibrpaOptions *p_opts, double *omegas,
                                          double *weights)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(p_opts, "null options");
        const auto g = make_grids(*ds, *p_opts);
        std::memcpy(omegas, g.omega.data(), sizeof(double) * g.n);
        std::memcpy(weights, g.omega_w.data(), sizeof(double) * g.n);
    });
}

double librpa_get_rpa_correlation_energy(LibrpaHandler *h, const LibrpaOptions *p_opts, int n_ibz_kpoints,
                                         double *re, double *im)
{
    double out = std::numeric_limits<double>::quiet_NaN();
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        clear_error(ds);
        GB_REQUIRE(p_opts, "null options");
        const LibrpaOptions &o = *p_opts;
        // compute_rpa.cpp:50-64: distributed eigenvectors need the k-parallel switch
        for (unsigned char f : ds->wfc_set)
            if (!f && o.use_kpara_scf_eigvec != LIBRPA_SWITCH_ON)
                GB_FAIL("inconsistent input: eigenvectors missing for some k while use_kpara_scf_eigvec is off");
        switch (o.parallel_routing)
        {
        case AUTO: case RTAU: case ATOMPAIR: case LIBRI: break;
        default: GB_FAIL("invalid parallel routing");
        }
        if (ds->klist.empty())
        {
            // Gamma-only default lattice (PeriodicBoundaryData constructor, pbc.cpp:16-32)
            ds->klist.assign(3, 0.0);
            ds->kfrac.assign(3, 0.0);
            ds->ibz_map.assign(1, 0);
        }
        // with use_shrink_abfs the Coulomb matrix is given in the small ABF basis
        merge_vq_2d(ds, o.use_shrink_abfs == LIBRPA_SWITCH_ON);
        std::memset(&ds->stats, 0, sizeof(ds->stats));
        const double t0 = gb::wall_seconds();
        const auto g = make_grids(*ds, o);
        ds->stats.t_grids = gb::wall_seconds() - t0;
        GB_REQUIRE(!g.tau.empty(), "time grids required for the space-time method");
        const auto res = gb::run_rpa_gpu(*ds, o, g, o.n_bands_chi0);
        ds->stats.t_total += ds->stats.t_grids;
        if (static_cast<int>(res.per_q.size()) != n_ibz_kpoints)
            std::fprintf(stderr, "WARNING: parsed n_ibz_kpoints is not consistent with generated CorrEne object: %d != %zu\n",
                         n_ibz_kpoints, res.per_q.size());
        const int ncopy = std::min<int>(n_ibz_kpoints, static_cast<int>(res.per_q.size()));
        for (int q = 0; q < ncopy; ++q)
        {
            if (re) re[q] = res.per_q[q].real();
            if (im) im[q] = res.per_q[q].imag();
        }
        out = res.ec.real();
    });
    return out;
}

// No counterpart in the reference: the E_c call of n independent handlers, run concurrently on
// host threads (each call stages its inputs and launches on its own CUDA stream, so the GPU
// overlaps the calls' kernels, transfers and host set-up).
int librpa_gb300_get_rpa_correlation_energy_batch(LibrpaHandler **hs, int n, const LibrpaOptions *opts, int n_threads,
                                                  double *ec)
{
    int failed = -1;
    guarded(nullptr, [&] {
        GB_REQUIRE(n >= 0 && (n == 0 || (hs && opts && ec)), "null argument");
        {
            // one thread per handler at a time: a handler listed twice would race with itself
            std::vector<LibrpaHandler *> seen(hs, hs + n);
            std::sort(seen.begin(), seen.end());
            GB_REQUIRE(std::adjacent_find(seen.begin(), seen.end()) == seen.end(),
                       "librpa_gb300_get_rpa_correlation_energy_batch: a handler is listed twice");
        }
        std::vector<int> nq(n, 1);
        for (int i = 0; i < n; ++i)
        {
            const Dataset *ds = get_ds(hs[i]);
            std::vector<int> reps(ds->ibz_map.begin(), ds->ibz_map.end());
            std::sort(reps.begin(), reps.end());
            nq[i] = std::max<int>(1, static_cast<int>(std::unique(reps.begin(), reps.end()) - reps.begin()));
        }
        const int hw = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
        const int nt = std::max(1, std::min(n, n_threads > 0 ? n_threads : std::min(4, hw)));
        std::atomic<int> next{0}, bad{0};
        auto work = [&] {
            std::vector<double> re, im;
            for (int i = next++; i < n; i = next++)
            {
                re.assign(nq[i], 0.0);
                im.assign(nq[i], 0.0);
                ec[i] = librpa_get_rpa_correlation_energy(hs[i], &opts[i], nq[i], re.data(), im.data());
                if (std::isnan(ec[i])) ++bad;
            }
        };
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) pool.emplace_back(work);
        for (std::thread &th : pool) th.join();
        failed = bad.load();
    });
    return failed;
}


namespace {
// Set-up shared by the exchange and G0W0 calls: Gamma-only default lattice, 2D Coulomb input
// redistributed to atom pairs.
void prepare_gw(Dataset *ds)
{
    if (ds->klist.empty())
    {
        ds->klist.assign(3, 0.0);
        ds->kfrac.assign(3, 0.0);
        ds->ibz_map.assign(1, 0);
    }
    merge_vq_2d(ds);
}

} // namespace

// compute_exx.cpp: librpa_build_exx (H_x(R) on the GPU, k-grids and the Gamma point; gw.cu)
void librpa_build_exx(LibrpaHandler *h, const LibrpaOptions *p_opts)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        clear_error(ds);
        GB_REQUIRE(p_opts, "null options");
        prepare_gw(ds);
        gb::build_exx(*ds, *p_opts);
    });
}

// compute_exx.cpp:56-112: v_exx of states [i_state_low, i_state_high) at the given k-points,
// vexx[(isp * n_kpts_this + ik_this) * n_states_calc + i]
void librpa_get_exx_pot_kgrid(LibrpaHandler *h, const LibrpaOptions *p_opts, const int n_spins, const int n_kpts_this,
                              const int *iks_this, int i_state_low, int i_state_high, double *vexx)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        clear_error(ds);
        GB_REQUIRE(p_opts && iks_this && vexx, "null argument");
        i_state_low = std::max(0, i_state_low);
        i_state_high = std::min(ds->n_states, i_state_high);
        GB_REQUIRE(n_spins == ds->n_spins, "parsed nspins is not consistent with the SCF starting point");
        if (i_state_high <= i_state_low) return;
        if (ds->hx_r.empty() || ds->exx_generation != ds->generation)
        {
            prepare_gw(ds);
            gb::build_exx(*ds, *p_opts);
        }
        const int nc = i_state_high - i_state_low;
        for (int k = 0; k < n_kpts_this; ++k)
            GB_REQUIRE(iks_this[k] >= 0 && iks_this[k] < ds->n_kpts, "k-point index out of range");
        for (int isp = 0; isp < n_spins; ++isp)
            for (int k = 0; k < n_kpts_this; ++k)
                for (int i = 0; i < nc; ++i)
                    vexx[(static_cast<size_t>(isp) * n_kpts_this + k) * nc + i] =
                        gb::exx_state(*ds, isp, iks_this[k], i_state_low + i);
    });
}

// compute_exx.cpp:115-180: v_exx at band k-points (librpa_set_band_*), from the k-grid H_x(R)
void librpa_get_exx_pot_band_k(LibrpaHandler *h, const LibrpaOptions *p_opts, const int n_spins,
                               const int n_kpts_band_this, const int *iks_band_this, int i_state_low, int i_state_high,
                               double *vexx_band)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        clear_error(ds);
        GB_REQUIRE(p_opts && iks_band_this && vexx_band, "null argument");
        GB_REQUIRE(ds->band_nk > 0, "Meanfield data for band calculation is not set");
        i_state_low = std::max(0, i_state_low);
        i_state_high = std::min(ds->band_nst, i_state_high);
        GB_REQUIRE(n_spins == ds->n_spins, "parsed nspins is not consistent with the SCF starting point");
        if (i_state_high <= i_state_low) return;
        if (ds->hx_r.empty() || ds->exx_generation != ds->generation)
        {
            prepare_gw(ds);
            gb::build_exx(*ds, *p_opts);
        }
        const int nc = i_state_high - i_state_low;
        for (int isp = 0; isp < n_spins; ++isp)
            for (int k = 0; k < n_kpts_band_this; ++k)
                for (int i = 0; i < nc; ++i)
                    vexx_band[(static_cast<size_t>(isp) * n_kpts_band_this + k) * nc + i] =
                        gb::exx_band_state(*ds, isp, iks_band_this[k], i_state_low + i);
    });
}

// compute_g0w0.cpp:22-166: chi0, W_c and Sigma_c on the GPU (k-grids and the Gamma point; gw.cu)
void librpa_build_g0w0_sigma(LibrpaHandler *h, const LibrpaOptions *p_opts)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        clear_error(ds);
        GB_REQUIRE(p_opts, "null options");
        prepare_gw(ds);
        const auto g = make_grids(*ds, *p_opts);
        GB_REQUIRE(!g.tau.empty(), "time grids required for the space-time method");
        gb::build_g0w0(*ds, *p_opts, g);
    });
}

// No counterpart in the reference: the KS-diagonal Sigma_c(i omega) that the quasi-particle step
// continues, after librpa_build_g0w0_sigma; [state][omega] for states [lo, hi) of one spin at
// k-point ik of the SCF grid (k-point 0 without the _k suffix).
int librpa_gb300_get_g0w0_sigc_iw_k(LibrpaHandler *h, int ispin, int ik, int i_state_low, int i_state_high, double *re,
                                    double *im)
{
    int rc = 1;
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(!ds->sigc_ks.empty() && ds->g0w0_generation == ds->generation,
                   "no self-energy: call librpa_build_g0w0_sigma first");
        GB_REQUIRE(ispin >= 0 && ispin < static_cast<int>(ds->sigc_ks.size()), "spin index out of range");
        const int nw = static_cast<int>(ds->gw_omega.size()), nb = ds->n_states;
        const int nk = static_cast<int>(ds->sigc_ks[ispin].size() / (static_cast<size_t>(nb) * nw));
        GB_REQUIRE(ik >= 0 && ik < nk, "k-point index out of range");
        GB_REQUIRE(0 <= i_state_low && i_state_low <= i_state_high && i_state_high <= nb, "state range out of range");
        GB_REQUIRE(re && im, "null array");
        const cplx *src = ds->sigc_ks[ispin].data() + static_cast<size_t>(ik) * nb * nw;
        for (int n = i_state_low; n < i_state_high; ++n)
            for (int w = 0; w < nw; ++w)
            {
                const cplx v = src[static_cast<size_t>(n) * nw + w];
                re[static_cast<size_t>(n - i_state_low) * nw + w] = v.real();
                im[static_cast<size_t>(n - i_state_low) * nw + w] = v.imag();
            }
        rc = 0;
    });
    return rc;
}

int librpa_gb300_get_g0w0_sigc_iw(LibrpaHandler *h, int ispin, int i_state_low, int i_state_high, double *re,
                                  double *im)
{
    return librpa_gb300_get_g0w0_sigc_iw_k(h, ispin, 0, i_state_low, i_state_high, re, im);
}

// compute_g0w0.cpp:168-260: Sigma_c of states [i_state_low, i_state_high) at the quasi-particle
// energy (Pade continuation with n_params_anacon, damped fixed point); NaN where the solver failed
void librpa_get_g0w0_sigc_kgrid(LibrpaHandler *h, const LibrpaOptions *p_opts, const int n_spins, const int n_kpts_this,
                                const int *iks_this, int i_state_low, int i_state_high, const double *vxc,
                                const double *vexx, double *sigc_re, double *sigc_im)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        clear_error(ds);
        GB_REQUIRE(p_opts && iks_this && vxc && vexx && sigc_re && sigc_im, "null argument");
        i_state_low = std::max(0, i_state_low);
        i_state_high = std::min(ds->n_states, i_state_high);
        GB_REQUIRE(n_spins == ds->n_spins, "parsed nspins is not consistent with the SCF starting point");
        if (i_state_high <= i_state_low) return;
        if (ds->sigc_ks.empty() || ds->g0w0_generation != ds->generation)
        {
            prepare_gw(ds);
            const auto g = make_grids(*ds, *p_opts);
            gb::build_g0w0(*ds, *p_opts, g);
        }
        const int nc = i_state_high - i_state_low, nw = static_cast<int>(ds->gw_omega.size());
        const int nb = ds->n_states, nk = ds->n_kpts;
        std::vector<std::complex<double>> x(nw), f(nw);
        for (int w = 0; w < nw; ++w) x[w] = {0.0, ds->gw_omega[w]};
        for (int k = 0; k < n_kpts_this; ++k)
            GB_REQUIRE(iks_this[k] >= 0 && iks_this[k] < nk, "k-point index out of range");
        for (int isp = 0; isp < n_spins; ++isp)
            for (int k = 0; k < n_kpts_this; ++k)
            {
                const int ik = iks_this[k];
                for (int i = 0; i < nc; ++i)
                {
                    const int n = i_state_low + i;
                    const size_t o = (static_cast<size_t>(isp) * n_kpts_this + k) * nc + i;
                    for (int w = 0; w < nw; ++w)
                        f[w] = ds->sigc_ks[isp][(static_cast<size_t>(ik) * nb + n) * nw + w];
                    const gb::PadeContinuation pade(p_opts->n_params_anacon, x, f);
                    const gb::QpeResult r = gb::solve_qpe(pade, ds->ekb[(static_cast<size_t>(isp) * nk + ik) * nb + n],
                                                          ds->efermi, vxc[o], vexx[o]);
                    sigc_re[o] = r.info == 0 ? r.sigc.real() : std::numeric_limits<double>::quiet_NaN();
                    sigc_im[o] = r.info == 0 ? r.sigc.imag() : std::numeric_limits<double>::quiet_NaN();
                }
            }
    });
}

// compute_g0w0.cpp:263-366: Sigma_c at band k-points from the k-grid Sigma_c(R, i omega), the
// quasi-particle equation with the band eigenvalues and the SCF Fermi level
void librpa_get_g0w0_sigc_band_k(LibrpaHandler *h, const LibrpaOptions *p_opts, const int n_spins,
                                 const int n_kpts_band_this, const int *iks_band_this, int i_state_low,
                                 int i_state_high, const double *vxc_band, const double *vexx_band, double *sigc_re,
                                 double *sigc_im)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        clear_error(ds);
        GB_REQUIRE(p_opts && iks_band_this && vxc_band && vexx_band && sigc_re && sigc_im, "null argument");
        GB_REQUIRE(ds->band_nk > 0, "Meanfield data for band calculation is not set");
        i_state_low = std::max(0, i_state_low);
        i_state_high = std::min(ds->band_nst, i_state_high);
        GB_REQUIRE(n_spins == ds->n_spins, "parsed nspins is not consistent with the SCF starting point");
        if (i_state_high <= i_state_low) return;
        if (ds->sigc_r.empty() || ds->g0w0_generation != ds->generation)
        {
            prepare_gw(ds);
            const auto g = make_grids(*ds, *p_opts);
            gb::build_g0w0(*ds, *p_opts, g);
        }
        const int nc = i_state_high - i_state_low, nw = static_cast<int>(ds->gw_omega.size());
        std::vector<std::complex<double>> x(nw);
        for (int w = 0; w < nw; ++w) x[w] = {0.0, ds->gw_omega[w]};
        for (int isp = 0; isp < n_spins; ++isp)
            for (int k = 0; k < n_kpts_band_this; ++k)
            {
                const int kb = iks_band_this[k];
                for (int i = 0; i < nc; ++i)
                {
                    const int n = i_state_low + i;
                    const size_t o = (static_cast<size_t>(isp) * n_kpts_band_this + k) * nc + i;
                    const std::vector<std::complex<double>> f = gb::sigc_band_iw(*ds, isp, kb, n);
                    const gb::PadeContinuation pade(p_opts->n_params_anacon, x, f);
                    const gb::QpeResult r = gb::solve_qpe(
                        pade, ds->band_eig[(static_cast<size_t>(isp) * ds->band_nk + kb) * ds->band_nst + n], ds->efermi,
                        vxc_band[o], vexx_band[o]);
                    sigc_re[o] = r.info == 0 ? r.sigc.real() : std::numeric_limits<double>::quiet_NaN();
                    sigc_im[o] = r.info == 0 ? r.sigc.imag() : std::numeric_limits<double>::quiet_NaN();
                }
            }
    });
}

// ------------------------------------------------------------------ GB300 extensions
void librpa_gb300_init_options(LibrpaGB300Options *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->chi0_precision = LIBRPA_GB300_CHI0_BF16X3;
    o->ec_path = LIBRPA_GB300_EC_CHOL;
    o->screen_mode = LIBRPA_GB300_SCREEN_OFF;
    o->screen_threshold = 1e-6;
    o->audit_fraction = 0.02;
    o->seed = 12345ULL;
    o->use_cuda_graph = 1;
    o->keep_chi0 = 0;
    o->tau_begin = 0;
    o->tau_end = -1;
    o->q_begin = 0;
    o->q_end = -1;
    o->sigma_precision = LIBRPA_GB300_SIGMA_FP64;
    o->stage = LIBRPA_GB300_STAGE_FULL;
    o->device = 0;
    o->reuse_device_inputs = 1;
}

void librpa_gb300_set_options(LibrpaHandler *h, const LibrpaGB300Options *o)
{
    guarded(h, [&] {
        GB_REQUIRE(o, "null options");
        Dataset *ds = get_ds(h);
        // the kept self-energy depends on the precisions it was built with
        if (o->chi0_precision != ds->gbopt.chi0_precision || o->sigma_precision != ds->gbopt.sigma_precision)
            ds->g0w0_generation = 0;
        ds->gbopt = *o;
    });
}

void librpa_gb300_get_stats(LibrpaHandler *h, LibrpaGB300Stats *s)
{
    guarded(h, [&] {
        GB_REQUIRE(s, "null stats");
        *s = get_ds(h)->stats;
    });
}

const char *librpa_get_last_error(LibrpaHandler *h)
{
    if (!h) return g_last_error.c_str();
    try
    {
        return get_ds(h)->last_error.c_str();
    }
    catch (...)
    {
        return g_last_error.c_str();
    }
}

int librpa_get_last_error_code(LibrpaHandler *h)
{
    if (!h) return g_last_code;
    try
    {
        return get_ds(h)->last_error_code;
    }
    catch (...)
    {
        return 1;
    }
}

int librpa_gb300_minimax_grid(int n, double emin, double emax, double reg, double *tau, double *tau_w,
                              double *omega, double *omega_w, double *cos_t2f, double *cos_f2t, double *sin_t2f,
                              double *dual)
{
    int rc = 1;
    guarded(nullptr, [&] {
        const auto g = gb::minimax_grids(n, emin, emax, reg);
        auto cp = [](double *dst, const std::vector<double> &v) {
            if (dst) std::memcpy(dst, v.data(), v.size() * sizeof(double));
        };
        cp(tau, g.tau);
        cp(tau_w, g.tau_w);
        cp(omega, g.omega);
        cp(omega_w, g.omega_w);
        cp(cos_t2f, g.cos_t2f);
        cp(cos_f2t, g.cos_f2t);
        cp(sin_t2f, g.sin_t2f);
        if (dual) *dual = g.cosft_duality_error;
        rc = 0;
    });
    return rc;
}

int librpa_gb300_phase_tables(LibrpaHandler *h, int *n_cells, int *n_q, int *cells, int *ibz_rep, double *ibz_w,
                              double *g_phase, double *q_phase)
{
    int rc = 1;
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        const gb::PhaseTables t = gb::build_phase_tables(*ds);
        if (n_cells) *n_cells = t.nc;
        if (n_q) *n_q = t.nq;
        if (cells)
            for (int c = 0; c < t.nc; ++c)
                for (int d = 0; d < 3; ++d) cells[3 * c + d] = t.cells.R[c][d];
        for (int q = 0; q < t.nq; ++q)
        {
            if (ibz_rep) ibz_rep[q] = t.ibz_rep[q];
            if (ibz_w) ibz_w[q] = t.ibz_w[q];
        }
        if (g_phase)
            for (size_t i = 0; i < t.gcos.size(); ++i)
            {
                g_phase[2 * i] = t.gcos[i];
                g_phase[2 * i + 1] = t.gsin[i];
            }
        if (q_phase)
            for (size_t i = 0; i < t.qcos.size(); ++i)
            {
                q_phase[2 * i] = t.qcos[i];
                q_phase[2 * i + 1] = t.qsin[i];
            }
        rc = 0;
    });
    return rc;
}

int librpa_gb300_solve_qpe(int n_states, int n_freq, const double *omegas, const double *sigc_re,
                           const double *sigc_im, int n_params, const double *e_mf, double e_fermi,
                           const double *vxc, const double *vexx, double *e_qp, double *sigc_qp_re,
                           double *sigc_qp_im)
{
    int rc = -1;
    guarded(nullptr, [&] {
        GB_REQUIRE(n_states >= 0 && n_freq > 0, "need n_states >= 0 and n_freq > 0");
        GB_REQUIRE(omegas && sigc_re && sigc_im && e_mf && vxc && vexx && e_qp && sigc_qp_re && sigc_qp_im,
                   "null array");
        std::vector<std::complex<double>> x(n_freq), f(n_freq);
        for (int k = 0; k < n_freq; ++k) x[k] = {0.0, omegas[k]};
        int failed = 0;
        for (int s = 0; s < n_states; ++s)
        {
            for (int k = 0; k < n_freq; ++k)
                f[k] = {sigc_re[static_cast<size_t>(s) * n_freq + k], sigc_im[static_cast<size_t>(s) * n_freq + k]};
            const gb::PadeContinuation pade(n_params, x, f);
            const gb::QpeResult r = gb::solve_qpe(pade, e_mf[s], e_fermi, vxc[s], vexx[s]);
            if (r.info == 0)
            {
                e_qp[s] = r.e_qp;
                sigc_qp_re[s] = r.sigc.real();
                sigc_qp_im[s] = r.sigc.imag();
            }
            else
            {
                e_qp[s] = sigc_qp_re[s] = sigc_qp_im[s] = std::numeric_limits<double>::quiet_NaN();
                ++failed;
            }
        }
        rc = failed;
    });
    return rc;
}

int librpa_gb300_get_chi0_block(LibrpaHandler *h, int ifreq, int iq, int I, int J, double *re, double *im)
{
    int rc = 1;
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(ds->kept_chi0, "no chi0 kept: run with LibrpaGB300Options.keep_chi0 = 1");
        const int nat = static_cast<int>(ds->nabf_at.size());
        GB_REQUIRE(I >= 0 && I <= J && J < nat, "need 0 <= I <= J < n_atoms");
        GB_REQUIRE(ifreq >= 0 && ifreq < ds->kept_nfreq && iq >= 0 && iq < ds->kept_nq, "frequency or q index out of range");
        int p = 0;
        for (int a = 0; a < I; ++a) p += nat - a;
        p += J - I;
        const size_t nel = static_cast<size_t>(ds->nabf_at[I]) * ds->nabf_at[J];
        std::vector<cplx> buf(nel);
        const size_t off = (static_cast<size_t>(ifreq) * ds->kept_nq + iq) * ds->kept_pair_elems + ds->kept_pair_offset[p];
        GB_CUDA(cudaMemcpy(buf.data(), static_cast<cplx *>(ds->kept_chi0) + off, nel * sizeof(cplx), cudaMemcpyDeviceToHost));
        for (size_t t = 0; t < nel; ++t)
        {
            re[t] = buf[t].real();
            im[t] = buf[t].imag();
        }
        rc = 0;
    });
    return rc;
}

int librpa_gb300_device_count(void) { return gb::device_count(); }

double librpa_gb300_selftest_tc_gemm(int M, int N, int K, int seed, int pieces)
{
    double r = std::numeric_limits<double>::quiet_NaN();
    guarded(nullptr, [&] {
        GB_REQUIRE(gb::device_count() > 0, "no CUDA device visible");
        r = gb::tc_gemm_selftest(M, N, K, seed, pieces);
    });
    return r;
}

double librpa_gb300_selftest_chol_ozaki(int N, int batch, int seed, int spread_decades, double shift, double *max_rel_l)
{
    double r = std::numeric_limits<double>::quiet_NaN();
    guarded(nullptr, [&] {
        GB_REQUIRE(gb::device_count() > 0, "no CUDA device visible");
        GB_REQUIRE(N > 0 && batch > 0, "N and batch must be positive");
        GB_REQUIRE(shift > 0.0, "the diagonal shift must be positive");
        r = gb::chol_ozaki_selftest(N, batch, seed, spread_decades, shift, max_rel_l);
    });
    return r;
}

// ---- kept chi0(q, omega) for tau-shard reductions; no counterpart in the reference
long long librpa_gb300_chi0_qw_elems(LibrpaHandler *h)
{
    long long n = -1;
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        n = ds->kept_chi0 ? static_cast<long long>(ds->kept_chi0_bytes / sizeof(cplx)) : 0;
    });
    return n;
}

int librpa_gb300_copy_chi0_qw(LibrpaHandler *h, double *dst, int on_device)
{
    int rc = 1;
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(ds->kept_chi0, "no chi0(q, omega) kept: run with keep_chi0 = 1 or stage = STAGE_CHI0");
        GB_REQUIRE(dst, "null destination");
        GB_CUDA(cudaMemcpy(dst, ds->kept_chi0, ds->kept_chi0_bytes,
                           on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
        rc = 0;
    });
    return rc;
}

int librpa_gb300_load_chi0_qw(LibrpaHandler *h, const double *src, long long n_elems, int on_device)
{
    int rc = 1;
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(ds->kept_chi0, "no chi0(q, omega) layout kept: run a STAGE_CHI0 call first");
        GB_REQUIRE(src && n_elems == static_cast<long long>(ds->kept_chi0_bytes / sizeof(cplx)),
                   "chi0(q, omega) size differs from the kept layout");
        GB_CUDA(cudaMemcpy(ds->kept_chi0, src, ds->kept_chi0_bytes,
                           on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
        rc = 0;
    });
    return rc;
}

// ---- learned screening (screen.cu); no counterpart in the reference
int librpa_gb300_train_screening(LibrpaHandler *h, int iterations, double learning_rate, double *rmse)
{
    int rc = 1;
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        GB_REQUIRE(gb::device_count() > 0, "no CUDA device visible");
        GB_REQUIRE(iterations > 0 && learning_rate > 0, "iterations and learning_rate must be positive");
        GB_CUDA(cudaSetDevice(ds->gbopt.device));
        cudaStream_t st;
        GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        try
        {
            gb::mlp_train(ds->screen_model, ds->screen_log.x, ds->screen_log.y, iterations, learning_rate,
                          ds->gbopt.seed, st);
        }
        catch (...)
        {
            cudaStreamDestroy(st);
            throw;
        }
        cudaStreamDestroy(st);
        if (rmse) *rmse = ds->screen_model.train_rmse;
        rc = 0;
    });
    return rc;
}

long long librpa_gb300_screening_samples(LibrpaHandler *h)
{
    long long n = -1;
    guarded(h, [&] { n = static_cast<long long>(get_ds(h)->screen_log.size()); });
    return n;
}

int librpa_gb300_get_screening_samples(LibrpaHandler *h, float *x, float *y, long long n)
{
    int rc = 1;
    guarded(h, [&] {
        const gb::ScreenLog &lg = get_ds(h)->screen_log;
        GB_REQUIRE(n >= 0 && static_cast<size_t>(n) <= lg.size(), "more samples requested than logged");
        std::copy(lg.x.begin(), lg.x.begin() + n * gb::MLP_IN, x);
        std::copy(lg.y.begin(), lg.y.begin() + n, y);
        rc = 0;
    });
    return rc;
}

// No counterpart in the reference: append block samples logged elsewhere (another handler's
// plain-screening runs, other systems), so one model trains on the logs of several systems.
int librpa_gb300_add_screening_samples(LibrpaHandler *h, const float *x, const float *y, long long n)
{
    int rc = 1;
    guarded(h, [&] {
        GB_REQUIRE(n >= 0, "negative sample count");
        GB_REQUIRE(n == 0 || (x && y), "null sample arrays");
        for (long long t = 0; t < n; ++t) GB_REQUIRE(std::isfinite(y[t]), "non-finite sample target");
        for (long long t = 0; t < n * gb::MLP_IN; ++t) GB_REQUIRE(std::isfinite(x[t]), "non-finite sample feature");
        gb::ScreenLog &lg = get_ds(h)->screen_log;
        lg.x.insert(lg.x.end(), x, x + n * gb::MLP_IN);
        lg.y.insert(lg.y.end(), y, y + n);
        rc = 0;
    });
    return rc;
}

void librpa_gb300_clear_grid_cache(void)
{
    guarded(nullptr, [&] { gb::clear_grid_cache(); });
}

int librpa_gb300_get_screening_model(LibrpaHandler *h, float *params, float *norm)
{
    int rc = 1;
    guarded(h, [&] {
        const gb::ScreenModel &m = get_ds(h)->screen_model;
        GB_REQUIRE(m.trained, "no screening model: train one first");
        std::copy(m.params.begin(), m.params.end(), params);
        std::copy(m.norm.begin(), m.norm.end(), norm);
        rc = 0;
    });
    return rc;
}

int librpa_gb300_set_screening_model(LibrpaHandler *h, const float *params, const float *norm)
{
    int rc = 1;
    guarded(h, [&] {
        gb::ScreenModel &m = get_ds(h)->screen_model;
        GB_REQUIRE(params && norm, "null model arrays");
        for (int f = 0; f < gb::MLP_IN; ++f)
            GB_REQUIRE(norm[gb::MLP_IN + f] > 0.0f, "feature scales must be positive");
        GB_REQUIRE(norm[2 * gb::MLP_IN + 1] > 0.0f, "target scale must be positive");
        m.params.assign(params, params + gb::MLP_NPARAM);
        m.norm.assign(norm, norm + gb::MLP_NNORM);
        m.trained = true;
        rc = 0;
    });
    return rc;
}

void librpa_gb300_clear_screening(LibrpaHandler *h)
{
    guarded(h, [&] {
        Dataset *ds = get_ds(h);
        ds->screen_log = gb::ScreenLog{};
        ds->screen_model = gb::ScreenModel{};
    });
}

int librpa_gb300_mlp_loss_grad(const float *params, const float *norm, const float *x, const float *y, int n,
                               float *grad, double *loss)
{
    int rc = 1;
    guarded(nullptr, [&] {
        GB_REQUIRE(gb::device_count() > 0, "no CUDA device visible");
        GB_REQUIRE(params && norm && x && y && grad && n > 0, "bad arguments");
        cudaStream_t st;
        GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        double l = 0.0;
        try
        {
            l = gb::mlp_loss_grad(params, norm, x, y, n, grad, st);
        }
        catch (...)
        {
            cudaStreamDestroy(st);
            throw;
        }
        cudaStreamDestroy(st);
        if (loss) *loss = l;
        rc = 0;
    });
    return rc;
}

// interpolate_dielec_func (dielecmodel.cpp:65-104) on caller arrays; host work (dielec.cpp)
int librpa_gb300_interpolate_dielec_func(int option, int n_in, const double *omega_in, const double *eps_in,
                                         int n_out, const double *omega_out, double *eps_out)
{
    int rc = 1;
    guarded(nullptr, [&] {
        GB_REQUIRE(n_in > 0 && n_out >= 0, "need n_in > 0 and n_out >= 0");
        GB_REQUIRE(omega_in && eps_in && (n_out == 0 || (omega_out && eps_out)), "null array");
        const std::vector<double> out =
            gb::interpolate_dielec_func(option, std::vector<double>(omega_in, omega_in + n_in),
                                        std::vector<double>(eps_in, eps_in + n_in),
                                        std::vector<double>(omega_out, omega_out + n_out));
        std::copy(out.begin(), out.end(), eps_out);
        rc = 0;
    });
    return rc;
}

// No counterpart in the reference: the allocation-free split GEMM (tc_gemm_noalloc.cu).
int librpa_gb300_tc_gemm_noalloc(int M, int N, int K, const double *A, const double *B, float *D, int pieces,
                                 void *stream)
{
    int rc = 1;
    guarded(nullptr, [&] {
        gb::tc_gemm_noalloc(M, N, K, A, B, D, pieces, static_cast<cudaStream_t>(stream));
        rc = 0;
    });
    return rc;
}

} // extern "C"
