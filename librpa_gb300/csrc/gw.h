// Exact exchange (k-grids) and the G0W0 self-energy (Gamma point) on the GPU (gw.cu).
#pragma once

#include <complex>
#include <vector>

#include "../../include/librpa_options.h"

namespace gb {

struct Dataset;
struct TimeFreqGrids;

// H_x(R) per spin into ds.hx_r ([cell][n_ao][n_ao], Hartree; the cells in ds.hx_cells) and
// H_x(R = 0) into ds.hx: LibRI Exx::cal_Hs with the density matrix D(R) and the truncated Coulomb
// matrix V(R) of the k-grid (one cell at the Gamma point), as the Gamma-point closed form of the
// Born-von Karman supercell.
void build_exx(Dataset &ds, const LibrpaOptions &opts);
// v_exx of state n of spin s at k-point k (SCF grid), after build_exx: -<psi|H_x(k)|psi>.
double exx_state(const Dataset &ds, int s, int k, int n);
// Sigma_c(i omega) on the KS states of every k-point per spin into ds.sigc_ks ([k][state][omega])
// and the imaginary frequencies into ds.gw_omega: the Gamma-point chain for one k-point, the
// k-grid chain (W_c(q) at every IBZ q, the BvK supercell closed form for Sigma_c(R)) otherwise.
void build_g0w0(Dataset &ds, const LibrpaOptions &opts, const TimeFreqGrids &tf);
void build_g0w0_gamma(Dataset &ds, const LibrpaOptions &opts, const TimeFreqGrids &tf);
void build_g0w0_kgrid(Dataset &ds, const LibrpaOptions &opts, const TimeFreqGrids &tf);
// At band k-point kb (librpa_set_band_*), after build_exx / build_g0w0: v_exx of band state n,
// and the KS-diagonal Sigma_c(i omega) of band state n, each from the R blocks moved to the image
// nearest to the atom pair (exx.cpp:683-725) and summed with e^{i 2 pi k.R}.
double exx_band_state(const Dataset &ds, int s, int kb, int n);
std::vector<std::complex<double>> sigc_band_iw(const Dataset &ds, int s, int kb, int n);

} // namespace gb
