// RI coefficient blocks C(I, J, R) -> the (I, J, cell) table the chi0 path stages, with LibRI's
// periodic folding.  LibRI's set_tensors takes every cell vector modulo the Born-von Karman
// period into the centred range, sums blocks that land on the same key and only then applies
// the threshold filter (RI_Tools::cal_period, thirdparty/LibRI/include/RI/ri/RI_Tools.hpp:49-67;
// LRI::set_tensors_map2, LRI-set.hpp:33-75).  Host code, shared with a host-compiled unit test.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <map>
#include <vector>

namespace gb {

// LibRI's Array_Operator operator%: (i % n + 3n/2) % n - n/2 with C integer semantics.
inline int centred_mod(int i, int n)
{
    int r = i % n;
    r = (r + 3 * n / 2) % n;
    return r - n / 2;
}

struct CsFold
{
    std::vector<long long> off;  // per staged block: offset into blob ++ extra
    std::vector<int> meta;       // per staged block: I, J, cell, 0
    std::vector<double> extra;   // sums of blocks that folded onto one key
};

// blocks: objects with I, J, R[3], ni, nj, nmu, offset (into blob).  cell_of(Rfolded) -> cell
// index or -1.  Staged blocks keep the order of their keys' first appearance.  A key held by
// one block points into blob; blocks sharing a key are summed into `extra`, whose offsets count
// from blob_size (the caller stages blob ++ extra).
template <typename Block, typename CellOf>
CsFold fold_cs_blocks(const std::vector<Block> &blocks, const double *blob, std::size_t blob_size,
                      const int period[3], CellOf cell_of, double threshold)
{
    struct Group
    {
        int I, J, c;
        std::size_t n;
        std::vector<std::size_t> members;
    };
    std::vector<Group> groups;
    std::map<std::array<int, 3>, std::size_t> index;  // (I, J, cell) -> group
    for (std::size_t bi = 0; bi < blocks.size(); ++bi)
    {
        const Block &b = blocks[bi];
        const std::array<int, 3> Rf{centred_mod(b.R[0], period[0]), centred_mod(b.R[1], period[1]),
                                    centred_mod(b.R[2], period[2])};
        const int c = cell_of(Rf);
        if (c < 0) continue;
        const std::array<int, 3> key{b.I, b.J, c};
        auto it = index.find(key);
        if (it == index.end())
        {
            index.emplace(key, groups.size());
            groups.push_back({b.I, b.J, c, static_cast<std::size_t>(b.ni) * b.nj * b.nmu, {bi}});
        }
        else
            groups[it->second].members.push_back(bi);
    }
    CsFold out;
    for (const Group &g : groups)
    {
        const double *src;
        long long off;
        if (g.members.size() == 1)
        {
            off = static_cast<long long>(blocks[g.members[0]].offset);
            src = blob + blocks[g.members[0]].offset;
        }
        else
        {
            const std::size_t e0 = out.extra.size();
            out.extra.resize(e0 + g.n, 0.0);
            for (std::size_t m : g.members)
                for (std::size_t t = 0; t < g.n; ++t) out.extra[e0 + t] += blob[blocks[m].offset + t];
            off = static_cast<long long>(blob_size + e0);
            src = nullptr;
        }
        if (threshold > 0)
        {
            const double *v = src ? src : out.extra.data() + (off - static_cast<long long>(blob_size));
            double mx = 0.0;
            for (std::size_t t = 0; t < g.n; ++t) mx = std::max(mx, std::fabs(v[t]));
            if (mx <= threshold)  // LibRI keeps a block whose max-norm exceeds the threshold
            {
                if (!src) out.extra.resize(out.extra.size() - g.n);
                continue;
            }
        }
        out.off.push_back(off);
        out.meta.insert(out.meta.end(), {g.I, g.J, g.c, 0});
    }
    return out;
}

} // namespace gb
