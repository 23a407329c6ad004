// Minimax imaginary time/frequency grids (host, FP64).
//
// Port of the grid set-up LibRPA obtains from the GreenX library:
//   TFGrids::generate_minimax           src/core/timefreq.cpp:193-236
//   gx_minimax_grid                     thirdparty/greenX/GX-TimeFrequency/src/minimax_grids.F90:53-237
//   get_transformation_weights          minimax_grids.F90:299-406
//   er_aw_aux%get_coeff_weight          minimax_utils.F90 (energy-range bin selection)
// The tabulated coefficients are read from data/greenx_minimax_tables.txt.
#pragma once

#include <string>
#include <vector>

namespace gb {

struct TimeFreqGrids
{
    int n = 0;
    std::vector<double> tau, tau_w, omega, omega_w;
    // Row-major n x n matrices with the cos/sin factor included, oriented like
    // LibRPA's TFGrids members: cos_t2f[iw*n + it], cos_f2t[it*n + iw], sin_t2f[iw*n + it].
    std::vector<double> cos_t2f, cos_f2t, sin_t2f;
    double cosft_duality_error = 0.0;
    double max_errors[3] = {0, 0, 0};
};

// Directory-independent table location: $LIBRPA_GB300_MINIMAX_TABLES, else
// <directory of the shared library>/data/greenx_minimax_tables.txt.
std::string minimax_table_path();

// Throws gb::Error for unsupported n (GreenX supports 6, 8, ..., 34) or bad energies.
// Results are kept per (n, e_min, e_max, regularization) for later calls in the process.
TimeFreqGrids minimax_grids(int n, double emin, double emax, double regularization);
// Forget the kept grids: the next call fits them again.
void clear_grid_cache();

} // namespace gb
