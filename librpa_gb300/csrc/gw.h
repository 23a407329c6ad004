// Exact exchange and G0W0 self-energy at the Gamma point on the GPU (gw.cu).
#pragma once

#include "../../include/librpa_options.h"

namespace gb {

struct Dataset;
struct TimeFreqGrids;

// H_x per spin (n_ao x n_ao, Hartree) into ds.hx: LibRI Exx::cal_Hs at Gamma with the density
// matrix and the truncated Coulomb matrix.
void build_exx_gamma(Dataset &ds, const LibrpaOptions &opts);
// Sigma_c(i omega) on the KS states per spin into ds.sigc_ks ([state][omega]) and the imaginary
// frequencies into ds.gw_omega.
void build_g0w0_gamma(Dataset &ds, const LibrpaOptions &opts, const TimeFreqGrids &tf);

} // namespace gb
