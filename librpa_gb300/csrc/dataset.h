// Host-side dataset held by one handler: a copy of everything the librpa_set_*
// calls pass in (the caller keeps ownership of its buffers, as in LibRPA's
// src/api/input.cpp).  The GPU engine stages it to the device per call.
#pragma once

#include <array>
#include <complex>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/librpa_gb300.h"
#include "../../include/librpa_options.h"
#include "screen_model.h"

namespace gb {

using cplx = std::complex<double>;

struct CsBlock
{
    int I, J, R[3], ni, nj, nmu;
    size_t offset;  // into Dataset::cs_blob, (ni*nj) x nmu row-major
};

struct VqBlock
{
    int ik, I, J, nmu, nnu;
    size_t offset;  // into Dataset::vq_blob, nmu x nnu row-major complex
};

struct Vq2DBlock
{
    int ik, mu_begin, mu_end, nu_begin, nu_end;
    std::vector<cplx> data;  // row-major
};

struct Dataset
{
    // mean field (MeanField, src/core/meanfield.h)
    int n_spins = 0, n_kpts = 0, n_states = 0, n_ao = 0, n_spinor = 1;
    std::vector<double> wg;    // [s][k][n], already scaled by 1/n_kpts (input.cpp:82)
    std::vector<double> ekb;   // [s][k][n]
    double efermi = 0.0;
    bool occ_set = false;
    std::vector<cplx> wfc;     // [s][spinor][k][n][ao]
    std::vector<unsigned char> wfc_set;  // [s][spinor][k]

    // bases (AtomicBasis)
    std::vector<int> nao_at, nabf_at;

    // lattice / k mesh (PeriodicBoundaryData, src/core/pbc.cpp)
    bool latt_set = false;
    double latvec[9] = {1e5, 0, 0, 0, 1e5, 0, 0, 0, 1e5};  // rows a1, a2, a3 (Bohr)
    double recvec[9] = {1e-5, 0, 0, 0, 1e-5, 0, 0, 0, 1e-5};
    int period[3] = {1, 1, 1};
    std::vector<double> klist;  // [k][3] Cartesian / 2pi
    std::vector<double> kfrac;  // [k][3]
    std::vector<int> ibz_map{0};
    std::vector<int> types;
    std::vector<double> positions;

    // RI coefficients (Cs_LRI) and Coulomb matrices
    std::vector<double> cs_blob;
    std::vector<CsBlock> cs_blocks;
    std::map<std::array<int, 5>, size_t> cs_index;  // (I,J,R) -> index into cs_blocks
    std::vector<cplx> vq_blob;
    std::vector<VqBlock> vq_blocks;
    std::map<std::array<int, 3>, size_t> vq_index;   // (ik,I,J) -> index
    std::vector<Vq2DBlock> vq_2d;
    // truncated Coulomb matrix (exchange and W of G0W0), stored like the bare one
    std::vector<cplx> vq_cut_blob;
    std::vector<VqBlock> vq_cut_blocks;
    std::map<std::array<int, 3>, size_t> vq_cut_index;
    std::vector<Vq2DBlock> vq_cut_2d;

    // ABF shrink (use_shrink_abfs, chi0.cpp:711-898): the small ABF count per atom (the basis of
    // the Coulomb matrix and of E_c then) and U(q) = sinvS(q), n_small x n_large row-major, keyed
    // like the Coulomb blocks by the k index of the IBZ representative
    struct ShrinkU
    {
        int n_small = 0, n_large = 0;
        std::vector<cplx> u;
    };
    std::vector<int> shrink_nabf;
    std::map<int, ShrinkU> shrink_u;
    // the RI coefficients in the small basis (the Cs_shrinked_data files of the reference's driver):
    // the exchange of a shrunk input contracts them with the truncated Coulomb matrix of that basis
    std::vector<double> shrink_cs_blob;
    std::vector<CsBlock> shrink_cs_blocks;
    std::map<std::array<int, 5>, size_t> shrink_cs_index;

    // Gamma-point exchange and G0W0 results (gw.cu), valid while generation is unchanged
    std::vector<std::vector<double>> hx;       // per spin: H_x(R = 0), n_ao x n_ao
    std::vector<std::vector<double>> hx_r;     // per spin: H_x(R) [cell][n_ao][n_ao]
    std::vector<std::array<int, 3>> hx_cells;  // the cells R of hx_r and sigc_r
    std::vector<std::vector<cplx>> sigc_r;     // per spin: Sigma_c(R, i omega) [omega][cell][n_ao][n_ao]
    std::vector<std::vector<cplx>> sigc_ks;    // per spin: Sigma_c(i omega) on the KS states, [n][omega]
    std::vector<double> gw_omega;              // the imaginary frequencies of sigc_ks
    unsigned long long exx_generation = 0, g0w0_generation = 0;

    // GW-side inputs that the RPA path does not use (kept so the setters behave)
    std::vector<double> dielect_omega, dielect_eps;
    // band k-points off the SCF grid (task = exx_band / g0w0_band): k fractions, and per
    // [spin][band k][state] occupations / eigenvalues and [spin][band k][state][ao] eigenvectors
    // (dimensions from librpa_set_band_occ_eigval)
    std::vector<double> band_kfrac, band_occ, band_eig;
    std::vector<cplx> band_wfc;
    int band_ns = 0, band_nk = 0, band_nst = 0;

    // GB300 extensions
    LibrpaGB300Options gbopt{};
    ScreenLog screen_log;      // block features and norms logged by plain-screening calls
    ScreenModel screen_model;  // learned block-norm predictor
    LibrpaGB300Stats stats{};
    int last_error_code = 0;
    std::string last_error;

    // Device copies of the inputs, reused by later calls while no setter ran
    // (generation unchanged) and LibrpaGB300Options.reuse_device_inputs is set.
    unsigned long long generation = 1;
    std::shared_ptr<void> dev_cache;

    // chi0(q, omega) kept on the device after a call (keep_chi0)
    void *kept_chi0 = nullptr;  // device buffer owned via engine helpers
    size_t kept_chi0_bytes = 0;
    std::vector<size_t> kept_pair_offset;  // per upper pair (I<=J) element offset
    size_t kept_pair_elems = 0;
    int kept_nfreq = 0, kept_nq = 0;

    int n_atoms() const
    {
        int n = static_cast<int>(nabf_at.size());
        if (static_cast<int>(nao_at.size()) > n) n = static_cast<int>(nao_at.size());
        if (static_cast<int>(types.size()) > n) n = static_cast<int>(types.size());
        return n;
    }
};

struct RpaResult
{
    cplx ec{0.0, 0.0};
    std::vector<cplx> per_q;  // per IBZ k-point, order of first appearance
};

struct TimeFreqGrids;

// GPU pipeline (engine.cu).  Throws gb::Error on failure.
RpaResult run_rpa_gpu(Dataset &ds, const LibrpaOptions &opts, const TimeFreqGrids &grids,
                      int nbands_g);
void release_kept(Dataset &ds);
int device_count();

} // namespace gb
