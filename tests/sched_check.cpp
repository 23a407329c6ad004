// Host driver for the scheduling helpers of librpa_gb300/csrc/work_schedule.h: reads one request per
// line on stdin and prints the schedule it gives.
//   T ntm ntn lower        -> one line per CTA: "mt nt" (ntm ntn or ntm (ntm + 1) / 2 lines)
//   O njm nti chunk        -> "items", one line "jm ti0 cnt" per item, then "end <ok>" where ok
//                             says whether the item after the last is rejected
//   K n_tiles n_sm nkc kmax -> "units", then one line "tile kc0 kc1 split" per CTA
//   P bm slots n r_0 .. r_{n-1} -> "tiles", then one line "g0 r0 nrows nslot" per row tile
#include <iostream>
#include <string>

#include "work_schedule.h"

int main()
{
    using namespace gb::sched;
    std::string op;
    while (std::cin >> op)
    {
        if (op == "T")
        {
            int ntm, ntn, lower;
            std::cin >> ntm >> ntn >> lower;
            const int n = lower ? ntm * (ntm + 1) / 2 : ntm * ntn;
            for (int t = 0; t < n; ++t)
            {
                int mt, nt;
                tile_coords(t, ntm, ntn, lower, mt, nt);
                std::cout << mt << ' ' << nt << '\n';
            }
        }
        else if (op == "O")
        {
            int njm, nti, chunk;
            std::cin >> njm >> nti >> chunk;
            const long long n = ozaki_items(njm, nti, chunk);
            std::cout << n << '\n';
            int jm, ti0, cnt;
            for (long long t = 0; t < n; ++t)
            {
                const bool ok = ozaki_item(static_cast<int>(t), njm, nti, chunk, jm, ti0, cnt);
                std::cout << (ok ? jm : -1) << ' ' << ti0 << ' ' << cnt << '\n';
            }
            std::cout << "end " << (ozaki_item(static_cast<int>(n), njm, nti, chunk, jm, ti0, cnt) ? 0 : 1) << '\n';
        }
        else if (op == "K")
        {
            int n_tiles, n_sm, nkc, kmax;
            std::cin >> n_tiles >> n_sm >> nkc >> kmax;
            const std::vector<KPart> plan = plan_kparts(n_tiles, n_sm, nkc, kmax);
            std::cout << plan.size() << '\n';
            for (const KPart &k : plan) std::cout << k.tile << ' ' << k.kc0 << ' ' << k.kc1 << ' ' << k.split << '\n';
        }
        else if (op == "P")
        {
            int bm, slots, n;
            std::cin >> bm >> slots >> n;
            std::vector<int> rows(n);
            for (int &r : rows) std::cin >> r;
            std::vector<RowTile> tiles;
            pack_row_tiles(rows.data(), n, 0, bm, slots, tiles);
            std::cout << tiles.size() << '\n';
            for (const RowTile &t : tiles) std::cout << t.g0 << ' ' << t.r0 << ' ' << t.nrows << ' ' << t.nslot << '\n';
        }
        else
        {
            std::cerr << "unknown request " << op << '\n';
            return 1;
        }
    }
    return 0;
}
