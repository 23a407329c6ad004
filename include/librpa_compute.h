#pragma once
/*
 * Compute entry points (replaces LibRPA include/librpa_compute.h:26-142).
 * The RPA calls run on one GB300 GPU; the EXX and G0W0 entries are exported
 * for ABI compatibility and record an "unsupported" error.
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

/* librpa_compute.h:51-142 -- not part of the RPA path; each records an error. */
void librpa_build_exx(LibrpaHandler *h, const LibrpaOptions *p_opts);
void librpa_get_exx_pot_kgrid(LibrpaHandler *h, const LibrpaOptions *p_opts,
                              const int n_spins, const int n_kpts_this, const int *iks_this,
                              int i_state_low, int i_state_high, double *vexx);
void librpa_get_exx_pot_band_k(LibrpaHandler *h, const LibrpaOptions *p_opts,
                               const int n_spins, const int n_kpts_band_this, const int *iks_band_this,
                               int i_state_low, int i_state_high, double *vexx_band);
void librpa_build_g0w0_sigma(LibrpaHandler *h, const LibrpaOptions *p_opts);
void librpa_get_g0w0_sigc_kgrid(LibrpaHandler *h, const LibrpaOptions *p_opts,
                                const int n_spins, const int n_kpts_this,
                                const int *iks_this, int i_state_low, int i_state_high,
                                const double *vxc, const double *vexx, double *sigc_re, double *sigc_im);
void librpa_get_g0w0_sigc_band_k(LibrpaHandler *h, const LibrpaOptions *p_opts,
                                 const int n_spins, const int n_kpts_band_this,
                                 const int *iks_band_this, int i_state_low, int i_state_high,
                                 const double *vxc_band, const double *vexx_band, double *sigc_band_re, double *sigc_band_im);

#ifdef __cplusplus
}
#endif
