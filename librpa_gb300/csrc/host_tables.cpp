#include "host_tables.h"

#include <cmath>

#include "common.h"
#include "dataset.h"

namespace gb {

Cells make_cells(const int period[3])
{
    Cells c;
    for (int d = 0; d < 3; ++d) c.period[d] = period[d];
    for (int x = -(period[0]) / 2; x <= (period[0] - 1) / 2; ++x)
        for (int y = -(period[1]) / 2; y <= (period[1] - 1) / 2; ++y)
            for (int z = -(period[2]) / 2; z <= (period[2] - 1) / 2; ++z)
            {
                c.index[{x, y, z}] = static_cast<int>(c.R.size());
                c.R.push_back({x, y, z});
            }
    return c;
}

PhaseTables build_phase_tables(const Dataset &ds)
{
    PhaseTables t;
    t.cells = make_cells(ds.period);
    const Cells &cells = t.cells;
    const int nc = static_cast<int>(cells.R.size()), nk = ds.n_kpts;
    t.nc = nc;
    t.nk = nk;
    GB_REQUIRE(nk > 0 && static_cast<int>(ds.kfrac.size()) >= 3 * nk && static_cast<int>(ds.klist.size()) >= 3 * nk &&
                   static_cast<int>(ds.ibz_map.size()) >= nk,
               "k points not set");
    t.cdiff.resize(static_cast<size_t>(nc) * nc);
    t.cneg.resize(nc);
    for (int a = 0; a < nc; ++a)
    {
        for (int b = 0; b < nc; ++b)
            t.cdiff[a * nc + b] = cells.find(cells.R[a][0] - cells.R[b][0], cells.R[a][1] - cells.R[b][1],
                                             cells.R[a][2] - cells.R[b][2]);
        t.cneg[a] = cells.find(-cells.R[a][0], -cells.R[a][1], -cells.R[a][2]);
    }
    t.gcos.resize(static_cast<size_t>(nk) * nc);
    t.gsin.resize(static_cast<size_t>(nk) * nc);
    for (int k = 0; k < nk; ++k)
        for (int c = 0; c < nc; ++c)
        {
            const double th = 2.0 * M_PI *
                              (ds.kfrac[3 * k] * cells.R[c][0] + ds.kfrac[3 * k + 1] * cells.R[c][1] +
                               ds.kfrac[3 * k + 2] * cells.R[c][2]);
            t.gcos[k * nc + c] = std::cos(th);
            t.gsin[k * nc + c] = std::sin(th);
        }
    {
        std::map<int, int> seen;
        for (int k = 0; k < nk; ++k)
        {
            const int r = ds.ibz_map[k];
            auto it = seen.find(r);
            if (it == seen.end())
            {
                seen[r] = static_cast<int>(t.ibz_rep.size());
                t.ibz_rep.push_back(r);
                t.ibz_w.push_back(1.0 / nk);
            }
            else
                t.ibz_w[it->second] += 1.0 / nk;
        }
    }
    t.nq = static_cast<int>(t.ibz_rep.size());
    t.qcos.resize(static_cast<size_t>(t.nq) * nc);
    t.qsin.resize(static_cast<size_t>(t.nq) * nc);
    for (int q = 0; q < t.nq; ++q)
        for (int c = 0; c < nc; ++c)
        {
            double Rc[3] = {0, 0, 0};
            for (int d = 0; d < 3; ++d)
                for (int a = 0; a < 3; ++a) Rc[d] += cells.R[c][a] * ds.latvec[a * 3 + d];
            const double *qv = &ds.klist[3 * t.ibz_rep[q]];
            const double arg = (qv[0] * Rc[0] + qv[1] * Rc[1] + qv[2] * Rc[2]) * 2.0 * M_PI;
            t.qcos[q * nc + c] = std::cos(arg);
            t.qsin[q * nc + c] = std::sin(arg);
        }
    return t;
}

} // namespace gb
