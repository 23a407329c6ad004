#pragma once
/*
 * Runtime options (replaces LibRPA include/librpa_options.h:33-232).
 * The struct layout is byte-identical to LibRPA's so that the Fortran binding
 * and existing callers keep working; GB300-specific knobs live in
 * librpa_gb300.h, not here.
 */
#include "librpa_enums.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LIBRPA_MAX_STRLEN 200

typedef struct
{
    char output_dir[LIBRPA_MAX_STRLEN];
    LibrpaParallelRouting parallel_routing;
    LibrpaVerbose output_level;
    double vq_threshold;
    LibrpaSwitch use_kpara_scf_eigvec;
    LibrpaTimeFreqGrid tfgrids_type;
    int nfreq;
    double tfgrids_freq_min;
    double tfgrids_freq_interval;
    double tfgrids_freq_max;
    double tfgrids_time_min;
    double tfgrids_time_interval;
    double minimax_emin;
    double minimax_emax;
    double minimax_regulation;
    LibrpaSwitch use_fullcoul_exx;
    LibrpaSwitch use_fullcoul_eps;
    LibrpaSwitch use_fullcoul_wc;
    int n_bands_chi0;
    int n_bands_sigc;
    double gf_threshold;
    LibrpaSwitch use_scalapack_ecrpa;
    LibrpaSwitch use_shrink_abfs;
    LibrpaSwitch use_shrink_chi;
    int n_params_anacon;
    LibrpaSwitch use_scalapack_gw_wc;
    LibrpaSwitch use_cholesky_gw_wc;
    LibrpaSwitch replace_w_head;
    int option_dielect_func;
    LibrpaSwitch use_2d_dielectric;
    LibrpaSwitch load_sigc_from_file;
    double sqrt_coulomb_threshold;
    double libri_chi0_threshold_C;
    double libri_chi0_threshold_G;
    double libri_exx_threshold_C;
    double libri_exx_threshold_D;
    double libri_exx_threshold_V;
    double libri_g0w0_threshold_C;
    double libri_g0w0_threshold_G;
    double libri_g0w0_threshold_Wc;
    LibrpaSwitch output_gw_sigc_mat;
    LibrpaSwitch output_gw_sigc_mat_rt;
    LibrpaSwitch output_gw_sigc_mat_rf;
    int option_output_Wc_Rf_mat;
} LibrpaOptions;

/* librpa_options.h:222 -- defaults of src/api/options.cpp:11-67. */
void librpa_init_options(LibrpaOptions *opts);
/* librpa_options.h:230 */
void librpa_set_output_dir(LibrpaOptions *opts, const char *output_dir);

#ifdef __cplusplus
}
#endif
