#pragma once
/*
 * Input setters (replaces LibRPA include/librpa_input.h:25-325).
 * Every setter copies the caller's data; the caller keeps ownership.
 */
#include <stddef.h>
#include "librpa_enums.h"
#include "librpa_handler.h"

#ifdef __cplusplus
extern "C" {
#endif

/* librpa_input.h:25 (nspinor defaults to 1 in C++) */
#ifdef __cplusplus
void librpa_set_scf_dimension(LibrpaHandler* h, int nspins, int nkpts, int nstates, int nbasis, int nspinor = 1);
#else
void librpa_set_scf_dimension(LibrpaHandler* h, int nspins, int nkpts, int nstates, int nbasis, int nspinor);
#endif
/* librpa_input.h:37 -- wg are raw occupations; they are scaled by 1/nkpts as LibRPA does (input.cpp:82). */
void librpa_set_wg_ekb_efermi(LibrpaHandler* h, int nspins, int nkpts, int nstates,
                              const double* wg, const double* ekb, double efermi);
/* librpa_input.h:50 -- band-major (nstates x nbasis) real and imaginary parts. */
void librpa_set_wfc(LibrpaHandler* h, int ispin, int ik, int nstates_local, int nbasis_local,
                    const double* wfc_real, const double* wfc_imag);
/* librpa_input.h:66 -- spinor input is accepted; the RPA call rejects nspinor > 1. */
void librpa_set_wfc_spinor(LibrpaHandler* h, int ik, int nstates_local, int nbasis_local,
                           const double* wfc_up_real, const double* wfc_up_imag,
                           const double* wfc_dn_real, const double* wfc_dn_imag);
/* librpa_input.h:80 -- interleaved (re, im) pairs. */
void librpa_set_wfc_packed(LibrpaHandler* h, int ispin, int ik, int nstates_local, int nbasis_local,
                           const double* wfc_ri);
/* librpa_input.h:93 */
void librpa_set_wfc_spinor_packed(LibrpaHandler* h, int ik, int nstates_local,
                                  int nbasis_local, const double* wfc_up_ri,
                                  const double* wfc_dn_ri);
/* librpa_input.h:104 */
void librpa_set_ao_basis_wfc(LibrpaHandler* h, int natoms, const size_t* nbs_wfc);
/* librpa_input.h:112 */
void librpa_set_ao_basis_aux(LibrpaHandler* h, int natoms, const size_t* nbs_aux);
/* librpa_input.h:120 -- lat_mat holds a1, a2, a3 consecutively (Bohr); G_mat likewise (Bohr^-1, with 2 pi). */
void librpa_set_latvec_and_G(LibrpaHandler* h, const double lat_mat[9], const double G_mat[9]);
/* librpa_input.h:129 */
void librpa_set_atoms(LibrpaHandler* h, int natoms, const int* types, const double* posi_cart);
/* librpa_input.h:140 -- Cartesian k vectors in Bohr^-1 (with 2 pi). */
void librpa_set_kgrids_kvec(LibrpaHandler* h, int nk1, int nk2, int nk3, const double* kvecs);
/* librpa_input.h:152 */
void librpa_set_ibz_mapping(LibrpaHandler* h, int nkpts, const int* map_ibzk);
/* librpa_input.h:167 -- one (I, J, R) block, (nbasis_i*nbasis_j) x naux_mu row-major. */
void librpa_set_lri_coeff(LibrpaHandler* h, LibrpaParallelRouting routing, int I, int J,
                          int nbasis_i, int nbasis_j, int naux_mu, const int R[3],
                          const double* Cs_in);
/* librpa_input.h:184 -- block kept only if max|Re V| >= vq_threshold (input.cpp:577). */
void librpa_set_aux_bare_coulomb_k_atom_pair(LibrpaHandler* h, int ik, int I, int J, int naux_mu,
                                             int naux_nu, const double* Vq_real_in,
                                             const double* Vq_imag_in, double vq_threshold);
/* librpa_input.h:201 -- stored, not used by the RPA energy. */
void librpa_set_aux_cut_coulomb_k_atom_pair(LibrpaHandler* h, int ik, int I, int J, int naux_mu,
                                            int naux_nu, const double* Vq_real_in,
                                            const double* Vq_imag_in, double vq_threshold);
/* librpa_input.h:218 -- row-major local block [mu_begin, mu_end) x [nu_begin, nu_end). */
void librpa_set_aux_bare_coulomb_k_2d_block(LibrpaHandler* h, int ik, int mu_begin, int mu_end,
                                            int nu_begin, int nu_end, const double* Vq_real_in,
                                            const double* Vq_imag_in);
/* librpa_input.h:234 -- stored, not used by the RPA energy. */
void librpa_set_aux_cut_coulomb_k_2d_block(LibrpaHandler* h, int ik, int mu_begin, int mu_end,
                                           int nu_begin, int nu_end, const double* Vq_real_in,
                                           const double* Vq_imag_in);
/* librpa_input.h:247 -- GW input, stored only. */
void librpa_set_dielect_func_imagfreq(LibrpaHandler* h, int nfreq, const double* omegas_imag,
                                      const double* dielect_func);
/* librpa_input.h:256-321 -- band-structure inputs of the GW path, stored only. */
void librpa_set_band_kvec(LibrpaHandler* h, int n_kpts_band, const double* kfrac_band);
void librpa_set_band_occ_eigval(LibrpaHandler* h, int n_spins, int n_kpts_band, int n_states,
                                const double* occ, const double* eig);
void librpa_set_wfc_band(LibrpaHandler* h, int ispin, int ik_band, int nstates_local,
                         int nbasis_local, const double* wfc_real, const double* wfc_imag);
void librpa_set_wfc_band_spinor(LibrpaHandler* h, int ik_band, int nstates_local,
                                int nbasis_local, const double* wfc_up_real, const double* wfc_up_imag,
                                const double* wfc_dn_real, const double* wfc_dn_imag);
void librpa_set_wfc_band_packed(LibrpaHandler* h, int ispin, int ik_band, int nstates_local,
                                int nbasis_local, const double* wfc_ri);
void librpa_set_wfc_band_spinor_packed(LibrpaHandler* h, int ik_band, int nstates_local,
                                       int nbasis_local, const double* wfc_up_ri, const double* wfc_dn_ri);
void librpa_reset_band_data(LibrpaHandler* h);

#ifdef __cplusplus
}
#endif
