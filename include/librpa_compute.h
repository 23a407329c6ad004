#pragma once
/*
 * Compute entry points (replaces LibRPA include/librpa_compute.h:26-142).
 * The RPA calls run on one GB300 GPU.  The exchange and G0W0 calls run on the GPU for k-grid
 * and Gamma-point inputs; the band-k-point variants project their k-grid results.
 */
#include "librpa_handler.h"
#include "librpa_options.h"

#ifdef __cplusplus
extern "C" {
#endif

/* librpa_compute.h:26-27 -- minimax frequency nodes and weights (opts->nfreq each). */
void librpa_get_imaginary_frequency_grids(LibrpaHandler *h, const LibrpaOptions *p_opts,
                                          double *omegas, double *weights);

/* librpa_compute.h:42-44 -- RPA correlation energy (real part returned); per-IBZ-k
 * contributions written to the caller's arrays of length n_ibz_kpoints.
 * Returns NaN on error (see librpa_get_last_error in librpa_gb300.h). */
double librpa_get_rpa_correlation_energy(LibrpaHandler *h, const LibrpaOptions *p_opts,
                                         int n_ibz_kpoints, double *rpa_corr_ibzk_contrib_re,
                                         double *rpa_corr_ibzk_contrib_im);

/* librpa_compute.h:51-70 -- exchange on the k-grid (or at the Gamma point): H_x(R) from the
 * density matrix and the truncated Coulomb matrix (librpa_set_aux_cut_coulomb_*); v_exx of states
 * [i_state_low, i_state_high) at the k-points iks_this,
 * vexx[(isp * n_kpts_this + ik_this) * n_states + i].  Errors are recorded on the handler. */
void librpa_build_exx(LibrpaHandler *h, const LibrpaOptions *p_opts);
void librpa_get_exx_pot_kgrid(LibrpaHandler *h, const LibrpaOptions *p_opts,
                              const int n_spins, const int n_kpts_this, const int *iks_this,
                              int i_state_low, int i_state_high, double *vexx);
/* librpa_compute.h:72-88 -- v_exx at band k-points (librpa_set_band_*): the k-grid H_x(R)
 * projected on the band states, in the layout of vexx. */
void librpa_get_exx_pot_band_k(LibrpaHandler *h, const LibrpaOptions *p_opts,
                               const int n_spins, const int n_kpts_band_this, const int *iks_band_this,
                               int i_state_low, int i_state_high, double *vexx_band);
/* librpa_compute.h:90-125 -- G0W0 on the k-grid (or at the Gamma point): chi0, W_c (bare Coulomb
 * for the dielectric function, truncated Coulomb for W) and Sigma_c on the GPU; Sigma_c at the quasi-particle
 * energy of states [i_state_low, i_state_high) after the Pade continuation (n_params_anacon)
 * and the quasi-particle equation, in the layout of vexx; NaN where the solver failed. */
void librpa_build_g0w0_sigma(LibrpaHandler *h, const LibrpaOptions *p_opts);
void librpa_get_g0w0_sigc_kgrid(LibrpaHandler *h, const LibrpaOptions *p_opts,
                                const int n_spins, const int n_kpts_this,
                                const int *iks_this, int i_state_low, int i_state_high,
                                const double *vxc, const double *vexx, double *sigc_re, double *sigc_im);
/* librpa_compute.h:127-142 -- Sigma_c at band k-points from the k-grid Sigma_c(R, i omega), the
 * band eigenvalues and the SCF Fermi level, in the layout of sigc_re; NaN where the solver failed. */
void librpa_get_g0w0_sigc_band_k(LibrpaHandler *h, const LibrpaOptions *p_opts,
                                 const int n_spins, const int n_kpts_band_this,
                                 const int *iks_band_this, int i_state_low, int i_state_high,
                                 const double *vxc_band, const double *vexx_band, double *sigc_band_re, double *sigc_band_im);

#ifdef __cplusplus
}
#endif
