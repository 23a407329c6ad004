// Host-side index and phase tables of the RPA path, built from the handler's data before any
// device work: the BvK cell list, cell differences and negations, the G(R) Bloch phases, the IBZ
// q list with weights and the R -> q Fourier phases.  Shared by the GPU engine and a diagnostic
// C entry point that lets the tables be checked without a GPU.
#pragma once

#include <array>
#include <map>
#include <vector>

#include "cs_fold.h"

namespace gb {

struct Dataset;

struct Cells
{
    std::vector<std::array<int, 3>> R;
    std::map<std::array<int, 3>, int> index;
    int period[3];
    int find(int x, int y, int z) const
    {
        std::array<int, 3> k{centred_mod(x, period[0]), centred_mod(y, period[1]), centred_mod(z, period[2])};
        auto it = index.find(k);
        return it == index.end() ? -1 : it->second;
    }
};

// construct_R_grid (src/core/pbc.cpp:178-190): x outer, z inner, centred range
Cells make_cells(const int period[3]);

struct PhaseTables
{
    Cells cells;
    int nc = 0, nk = 0, nq = 0;
    std::vector<int> cdiff, cneg;        // cell of R_a - R_b, of -R_a
    std::vector<double> gcos, gsin;      // [k][c]: theta = 2 pi kfrac_k . R_c (G kphase e^{-i theta})
    std::vector<int> ibz_rep;            // IBZ representatives (full k index), first-seen order
    std::vector<double> ibz_w;           // count / n_k
    std::vector<double> qcos, qsin;      // [q][c]: 2 pi q . (R_c latvec), q = k_cart / 2 pi
};

// chi0.cpp:379-380 (G phases), pbc.cpp:110-153 (IBZ list), chi0.cpp:582 (FT phases)
PhaseTables build_phase_tables(const Dataset &ds);

} // namespace gb
