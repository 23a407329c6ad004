// Host driver for librpa_gb300/csrc/cs_fold.h: reads "p0 p1 p2 threshold n_blocks" and then per
// block "I J R0 R1 R2 ni nj nmu v_0 .. v_{ni nj nmu - 1}"; prints the staged table, one line
// "I J cell values..." per staged block (cells numbered x outer, z inner over the centred range).
#include <array>
#include <iomanip>
#include <iostream>
#include <vector>

#include "cs_fold.h"

struct Block
{
    int I, J, R[3], ni, nj, nmu;
    std::size_t offset;
};

int main()
{
    int period[3];
    double thr;
    int nb;
    std::cin >> period[0] >> period[1] >> period[2] >> thr >> nb;
    std::vector<Block> blocks(nb);
    std::vector<double> blob;
    for (Block &b : blocks)
    {
        std::cin >> b.I >> b.J >> b.R[0] >> b.R[1] >> b.R[2] >> b.ni >> b.nj >> b.nmu;
        b.offset = blob.size();
        for (int t = 0; t < b.ni * b.nj * b.nmu; ++t)
        {
            double v;
            std::cin >> v;
            blob.push_back(v);
        }
    }
    auto cell_of = [&](const std::array<int, 3> &R) {
        const int x = R[0] + period[0] / 2, y = R[1] + period[1] / 2, z = R[2] + period[2] / 2;
        return (x * period[1] + y) * period[2] + z;
    };
    const gb::CsFold f = gb::fold_cs_blocks(blocks, blob.data(), blob.size(), period, cell_of, thr);
    std::cout << f.off.size() << '\n' << std::setprecision(17);
    for (std::size_t k = 0; k < f.off.size(); ++k)
    {
        const int I = f.meta[4 * k], J = f.meta[4 * k + 1], c = f.meta[4 * k + 2];
        std::cout << I << ' ' << J << ' ' << c;
        // the block's size from the first input block with the same atoms
        int n = 0;
        for (const Block &b : blocks)
            if (b.I == I && b.J == J)
            {
                n = b.ni * b.nj * b.nmu;
                break;
            }
        const long long o = f.off[k];
        for (int t = 0; t < n; ++t)
            std::cout << ' ' << (o < static_cast<long long>(blob.size()) ? blob[o + t] : f.extra[o - blob.size() + t]);
        std::cout << '\n';
    }
    return 0;
}
