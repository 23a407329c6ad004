#pragma once
/*
 * C++ interface (replaces LibRPA include/librpa.hpp:1-381 and its definitions in
 * src/api/librpa.cpp).  Header-only: every method forwards to the C API of this library.
 *
 * The C API records errors on the handler instead of throwing (librpa_get_last_error); the
 * methods here turn a recorded error into a std::runtime_error carrying that message, which is
 * how the reference's C++ interface reports failures (its internals throw).
 */
#include "librpa.h"

#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

namespace librpa
{

typedef LibrpaParallelRouting ParallelRouting;
typedef LibrpaTimeFreqGrid TimeFreqGrid;
typedef LibrpaSwitch Switch;
typedef LibrpaKind Kind;
typedef LibrpaVerbose Verbose;

/* librpa.hpp:57-69: LibrpaOptions initialised with the defaults. */
class Options : public ::LibrpaOptions
{
public:
    Options() { ::librpa_init_options(this); }
    void set_output_dir(const char *output_dir) { ::librpa_set_output_dir(this, output_dir); }
};

inline const char *get_build_info(void) { return ::librpa_get_build_info(); }
inline int get_major_version(void) { return ::librpa_get_major_version(); }
inline int get_minor_version(void) { return ::librpa_get_minor_version(); }
inline int get_patch_version(void) { return ::librpa_get_patch_version(); }
inline void init_global(Switch switch_redirect_stdout = LIBRPA_SWITCH_OFF, const char *redirect_path = "stdout",
                        Switch switch_process_output = LIBRPA_SWITCH_ON)
{
    ::librpa_init_global(switch_redirect_stdout, redirect_path, switch_process_output);
}
inline void finalize_global(void) { ::librpa_finalize_global(); }
inline void test(void) { ::librpa_test(); }
inline void print_profile(void) { ::librpa_print_profile(); }

/* librpa.hpp:158-378: RAII owner of one LibrpaHandler. */
class Handler
{
private:
    LibrpaHandler *h_ = nullptr;

    void check() const
    {
        if (h_ && ::librpa_get_last_error_code(h_)) throw std::runtime_error(::librpa_get_last_error(h_));
    }

public:
    Handler() : h_(nullptr) {}
    explicit Handler(MPI_Comm comm) : h_(nullptr) { init(comm); }
    Handler(const Handler &) = delete;
    Handler &operator=(const Handler &) = delete;
    ~Handler() { free(); }

    const LibrpaHandler *get_c_handler() const { return h_; }

    void init(MPI_Comm comm)
    {
        if (h_) throw std::runtime_error("double creating handler");
        h_ = ::librpa_create_handler(comm);
        if (!h_) throw std::runtime_error(::librpa_get_last_error(nullptr));
    }

    void free()
    {
        if (h_) ::librpa_destroy_handler(h_);
        h_ = nullptr;
    }

    /* Input (set) functions */
    void set_scf_dimension(int nspins, int nkpts, int nstates, int nbasis, int nspinor = 1)
    {
        ::librpa_set_scf_dimension(h_, nspins, nkpts, nstates, nbasis, nspinor);
        check();
    }
    void set_wg_ekb_efermi(int nspins, int nkpts, int nstates, const double *wg, const double *ekb, double efermi)
    {
        ::librpa_set_wg_ekb_efermi(h_, nspins, nkpts, nstates, wg, ekb, efermi);
        check();
    }
    void set_wfc(int ispin, int ik, int nstates_local, int nbasis_local, const double *wfc_real,
                 const double *wfc_imag)
    {
        ::librpa_set_wfc(h_, ispin, ik, nstates_local, nbasis_local, wfc_real, wfc_imag);
        check();
    }
    void set_wfc_spinor(int ik, int nstates_local, int nbasis_local, const double *wfc_up_real,
                        const double *wfc_up_imag, const double *wfc_dn_real, const double *wfc_dn_imag)
    {
        ::librpa_set_wfc_spinor(h_, ik, nstates_local, nbasis_local, wfc_up_real, wfc_up_imag, wfc_dn_real,
                                wfc_dn_imag);
        check();
    }
    void set_wfc_packed(int ispin, int ik, int nstates_local, int nbasis_local, const std::complex<double> *wfc)
    {
        ::librpa_set_wfc_packed(h_, ispin, ik, nstates_local, nbasis_local, reinterpret_cast<const double *>(wfc));
        check();
    }
    void set_wfc_spinor_packed(int ik, int nstates_local, int nbasis_local, const std::complex<double> *wfc_up,
                               const std::complex<double> *wfc_dn)
    {
        ::librpa_set_wfc_spinor_packed(h_, ik, nstates_local, nbasis_local, reinterpret_cast<const double *>(wfc_up),
                                       reinterpret_cast<const double *>(wfc_dn));
        check();
    }
    void set_ao_basis_wfc(const std::vector<size_t> &nbs_wfc)
    {
        ::librpa_set_ao_basis_wfc(h_, static_cast<int>(nbs_wfc.size()), nbs_wfc.data());
        check();
    }
    void set_ao_basis_aux(const std::vector<size_t> &nbs_aux)
    {
        ::librpa_set_ao_basis_aux(h_, static_cast<int>(nbs_aux.size()), nbs_aux.data());
        check();
    }
    void set_latvec_and_G(const double lat_mat[9], const double G_mat[9])
    {
        ::librpa_set_latvec_and_G(h_, lat_mat, G_mat);
        check();
    }
    void set_atoms(const std::vector<int> &types, const std::vector<double> &pos_cart)
    {
        ::librpa_set_atoms(h_, static_cast<int>(types.size()), types.data(), pos_cart.data());
        check();
    }
    void set_kgrids_kvec(int nk1, int nk2, int nk3, const double *kvecs)
    {
        ::librpa_set_kgrids_kvec(h_, nk1, nk2, nk3, kvecs);
        check();
    }
    void set_ibz_mapping(const std::vector<int> &map_ibzk)
    {
        ::librpa_set_ibz_mapping(h_, static_cast<int>(map_ibzk.size()), map_ibzk.data());
        check();
    }
    void set_lri_coeff(ParallelRouting routing, int I, int J, int nbasis_i, int nbasis_j, int naux_mu,
                       const int R[3], const double *Cs_in)
    {
        ::librpa_set_lri_coeff(h_, routing, I, J, nbasis_i, nbasis_j, naux_mu, R, Cs_in);
        check();
    }
    void set_aux_bare_coulomb_k_atom_pair(int ik, int I, int J, int naux_mu, int naux_nu, const double *Vq_real_in,
                                          const double *Vq_imag_in, double vq_threshold)
    {
        ::librpa_set_aux_bare_coulomb_k_atom_pair(h_, ik, I, J, naux_mu, naux_nu, Vq_real_in, Vq_imag_in,
                                                  vq_threshold);
        check();
    }
    void set_aux_cut_coulomb_k_atom_pair(int ik, int I, int J, int naux_mu, int naux_nu, const double *Vq_real_in,
                                         const double *Vq_imag_in, double vq_threshold)
    {
        ::librpa_set_aux_cut_coulomb_k_atom_pair(h_, ik, I, J, naux_mu, naux_nu, Vq_real_in, Vq_imag_in,
                                                 vq_threshold);
        check();
    }
    void set_aux_bare_coulomb_k_2d_block(int ik, int mu_begin, int mu_end, int nu_begin, int nu_end,
                                         const double *Vq_real_in, const double *Vq_imag_in)
    {
        ::librpa_set_aux_bare_coulomb_k_2d_block(h_, ik, mu_begin, mu_end, nu_begin, nu_end, Vq_real_in, Vq_imag_in);
        check();
    }
    void set_aux_cut_coulomb_k_2d_block(int ik, int mu_begin, int mu_end, int nu_begin, int nu_end,
                                        const double *Vq_real_in, const double *Vq_imag_in)
    {
        ::librpa_set_aux_cut_coulomb_k_2d_block(h_, ik, mu_begin, mu_end, nu_begin, nu_end, Vq_real_in, Vq_imag_in);
        check();
    }
    void set_dielect_func_imagfreq(const std::vector<double> &omegas_imag, const std::vector<double> &dielect_func)
    {
        ::librpa_set_dielect_func_imagfreq(h_, static_cast<int>(omegas_imag.size()), omegas_imag.data(),
                                           dielect_func.data());
        check();
    }
    void set_band_kvec(int n_kpts_band, const double *kfrac_band)
    {
        ::librpa_set_band_kvec(h_, n_kpts_band, kfrac_band);
        check();
    }
    void set_band_occ_eigval(int n_spins, int n_kpts_band, int n_states, const double *occ, const double *eig)
    {
        ::librpa_set_band_occ_eigval(h_, n_spins, n_kpts_band, n_states, occ, eig);
        check();
    }
    void set_wfc_band(int ispin, int ik_band, int nstates_local, int nbasis_local, const double *wfc_real,
                      const double *wfc_imag)
    {
        ::librpa_set_wfc_band(h_, ispin, ik_band, nstates_local, nbasis_local, wfc_real, wfc_imag);
        check();
    }
    void set_wfc_band_spinor(int ik_band, int nstates_local, int nbasis_local, const double *wfc_up_real,
                             const double *wfc_up_imag, const double *wfc_dn_real, const double *wfc_dn_imag)
    {
        ::librpa_set_wfc_band_spinor(h_, ik_band, nstates_local, nbasis_local, wfc_up_real, wfc_up_imag, wfc_dn_real,
                                     wfc_dn_imag);
        check();
    }
    void set_wfc_band_packed(int ispin, int ik_band, int nstates_local, int nbasis_local,
                             const std::complex<double> *wfc)
    {
        ::librpa_set_wfc_band_packed(h_, ispin, ik_band, nstates_local, nbasis_local,
                                     reinterpret_cast<const double *>(wfc));
        check();
    }
    void set_wfc_band_spinor_packed(int ik_band, int nstates_local, int nbasis_local,
                                    const std::complex<double> *wfc_up, const std::complex<double> *wfc_dn)
    {
        ::librpa_set_wfc_band_spinor_packed(h_, ik_band, nstates_local, nbasis_local,
                                            reinterpret_cast<const double *>(wfc_up),
                                            reinterpret_cast<const double *>(wfc_dn));
        check();
    }
    void reset_band_data()
    {
        ::librpa_reset_band_data(h_);
        check();
    }

    /* Compute (build/get) functions */
    void get_imaginary_frequency_grids(const Options &opts, std::vector<double> &omegas, std::vector<double> &weights)
    {
        omegas.resize(opts.nfreq);
        weights.resize(opts.nfreq);
        ::librpa_get_imaginary_frequency_grids(h_, &opts, omegas.data(), weights.data());
        check();
    }
    /* rpa_corr_ibzk_contrib: sized by the caller to the number of IBZ k-points, as in the reference */
    double get_rpa_correlation_energy(const Options &opts, std::vector<std::complex<double>> &rpa_corr_ibzk_contrib)
    {
        const int nq = static_cast<int>(rpa_corr_ibzk_contrib.size());
        std::vector<double> re(nq), im(nq);
        const double ec = ::librpa_get_rpa_correlation_energy(h_, &opts, nq, re.data(), im.data());
        check();
        for (int iq = 0; iq < nq; ++iq) rpa_corr_ibzk_contrib[iq] = std::complex<double>(re[iq], im[iq]);
        return ec;
    }
    void build_exx(const Options &opts)
    {
        ::librpa_build_exx(h_, &opts);
        check();
    }
    std::vector<double> get_exx_pot_kgrid(const Options &opts, const int n_spins, const std::vector<int> &iks_this,
                                          int i_state_low, int i_state_high)
    {
        const int nk = static_cast<int>(iks_this.size());
        std::vector<double> vexx(static_cast<size_t>(n_spins) * nk * (i_state_high - i_state_low));
        ::librpa_get_exx_pot_kgrid(h_, &opts, n_spins, nk, iks_this.data(), i_state_low, i_state_high, vexx.data());
        check();
        return vexx;
    }
    std::vector<double> get_exx_pot_band_k(const Options &opts, const int n_spins,
                                           const std::vector<int> &iks_band_this, int i_state_low, int i_state_high)
    {
        const int nk = static_cast<int>(iks_band_this.size());
        std::vector<double> vexx(static_cast<size_t>(n_spins) * nk * (i_state_high - i_state_low));
        ::librpa_get_exx_pot_band_k(h_, &opts, n_spins, nk, iks_band_this.data(), i_state_low, i_state_high,
                                    vexx.data());
        check();
        return vexx;
    }
    void build_g0w0_sigma(const Options &opts)
    {
        ::librpa_build_g0w0_sigma(h_, &opts);
        check();
    }
    std::vector<std::complex<double>> get_g0w0_sigc_kgrid(const Options &opts, const int n_spins,
                                                          const std::vector<int> &iks_this, int i_state_low,
                                                          int i_state_high, const std::vector<double> &vxc,
                                                          const std::vector<double> &vexx)
    {
        const int nk = static_cast<int>(iks_this.size());
        const size_t n = static_cast<size_t>(n_spins) * nk * (i_state_high - i_state_low);
        std::vector<double> re(n), im(n);
        ::librpa_get_g0w0_sigc_kgrid(h_, &opts, n_spins, nk, iks_this.data(), i_state_low, i_state_high, vxc.data(),
                                     vexx.data(), re.data(), im.data());
        check();
        std::vector<std::complex<double>> sigc(n);
        for (size_t i = 0; i < n; ++i) sigc[i] = std::complex<double>(re[i], im[i]);
        return sigc;
    }
    std::vector<std::complex<double>> get_g0w0_sigc_band_k(const Options &opts, const int n_spins,
                                                           const std::vector<int> &iks_band_this, int i_state_low,
                                                           int i_state_high, const std::vector<double> &vxc_band,
                                                           const std::vector<double> &vexx_band)
    {
        const int nk = static_cast<int>(iks_band_this.size());
        const size_t n = static_cast<size_t>(n_spins) * nk * (i_state_high - i_state_low);
        std::vector<double> re(n), im(n);
        ::librpa_get_g0w0_sigc_band_k(h_, &opts, n_spins, nk, iks_band_this.data(), i_state_low, i_state_high,
                                      vxc_band.data(), vexx_band.data(), re.data(), im.data());
        check();
        std::vector<std::complex<double>> sigc(n);
        for (size_t i = 0; i < n; ++i) sigc[i] = std::complex<double>(re[i], im[i]);
        return sigc;
    }
};

} // namespace librpa
