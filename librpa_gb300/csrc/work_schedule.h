// Work scheduling shared by the kernels and host-compiled unit tests: the tile order of the
// split GEMM, the work items of the tensor-core Cholesky update, and the row tiles and K parts
// of the chi0 contraction.
#pragma once

#include <cmath>
#include <vector>

#if defined(__CUDACC__)
#define SCHED_HD __host__ __device__ __forceinline__
#else
#define SCHED_HD inline
#endif

namespace gb {
namespace sched {

SCHED_HD int imin(int a, int b) { return a < b ? a : b; }

constexpr int RASTER_GROUP = 8;  // output-tile rows per raster group of the split GEMM

// Split GEMM: linear CTA index t -> output tile (mt, nt).  Tiles run column by column inside
// groups of RASTER_GROUP tile rows, so the CTAs resident at one time share a few A row panels
// and B column panels in L2.  lower != 0: only tiles with nt <= mt (square tile grid), in the
// same grouped order; t ranges over ntm (ntm + 1) / 2 tiles.
SCHED_HD void tile_coords(int t, int ntm, int ntn, int lower, int &mt, int &nt)
{
    constexpr int G = RASTER_GROUP;
    if (!lower)
    {
        const int g = t / (G * ntn);
        const int gm = imin(G, ntm - g * G);
        const int l = t - g * G * ntn;
        mt = g * G + l % gm;
        nt = l / gm;
        return;
    }
    int g = 0, rem = t;
    for (;; ++g)
    {
        const int gm = imin(G, ntm - g * G);
        const int cnt = gm * (g * G + 1) + gm * (gm - 1) / 2;
        if (rem < cnt || gm <= 0) break;
        rem -= cnt;
    }
    const int gm = imin(G, ntm - g * G), r0 = g * G;
    for (nt = 0; nt < ntn; ++nt)
    {
        const int rows = nt <= r0 ? gm : r0 + gm - nt;
        if (rem < rows)
        {
            mt = (nt <= r0 ? r0 : nt) + rem;
            return;
        }
        rem -= rows;
    }
    mt = 0;  // not reached for t below the lower-tile count
}

// Tensor-core Cholesky update: work item t -> (block jm of 128 trailing columns, first row tile
// ti0 of 32 rows, row tile count cnt <= chunk) over the row tiles that meet the lower triangle
// (32 ti + 31 >= 128 jm); njm column blocks, nti row tiles.
SCHED_HD bool ozaki_item(int t, int njm, int nti, int chunk, int &jm, int &ti0, int &cnt)
{
    for (jm = 0; jm < njm; ++jm)
    {
        const int first = 4 * jm;
        const int nch = (nti - first + chunk - 1) / chunk;
        if (t < nch)
        {
            ti0 = first + t * chunk;
            cnt = imin(chunk, nti - ti0);
            return true;
        }
        t -= nch;
    }
    return false;
}

// Number of work items of ozaki_item (the grid size).
inline long long ozaki_items(int njm, int nti, int chunk)
{
    long long items = 0;
    for (int jm = 0; jm < njm; ++jm) items += (nti - 4 * jm + chunk - 1) / chunk;
    return items;
}

// chi0 contraction: the rows of n row groups (group g has rows[g] rows), taken in order,
// packed into tiles of at most bm rows that touch at most max_slots >= 1 groups (the G slots of
// a CTA).  A tile closes when it is full, when it has used its slots or after the last group.
// Group indices in the tiles are offset by g_base.
struct RowTile
{
    int g0, r0, nrows, nslot;  // first group, first row inside it, rows, groups touched
};

inline void pack_row_tiles(const int *rows, int n, int g_base, int bm, int max_slots, std::vector<RowTile> &out)
{
    int gi = 0, off = 0;  // current group and row inside it
    while (gi < n)
    {
        RowTile t{g_base + gi, off, 0, 0};
        int g2 = gi, o2 = off;
        while (t.nrows < bm && g2 < n && t.nslot < max_slots)
        {
            const int b = rows[g2];
            const int take = imin(b - o2, bm - t.nrows);
            t.nrows += take;
            ++t.nslot;
            o2 += take;
            if (o2 == b)
            {
                ++g2;
                o2 = 0;
            }
        }
        out.push_back(t);
        gi = g2;
        off = o2;
    }
}

// chi0 contraction: how the n_tiles equal tiles (each nkc chunks of K) become CTAs.
//  - A launch of fewer than 16 waves runs every tile as kparts K parts (finer units for the
//    scheduler).
//  - The units of the last, partial wave are then cut into up to 8 K parts each, the count
//    that minimises the length of the final waves (plus 1% per part for the extra atomics).
//    E.g. 91 tiles of 40 chunks over 152 SMs: 364 quarter-tiles, whose last 60 become 300
//    parts of 2 chunks, two fifth-length waves in place of one full one.
// Returns (tile, kc0, kc1, split) per CTA in launch order; split = 1 marks K parts, whose sums
// are added into the output.
struct KPart
{
    int tile, kc0, kc1, split;
};

// force: cut every tile into kparts_max parts whatever the wave count (a tuner's candidate);
// otherwise only launches of under 16 waves are cut.
inline std::vector<KPart> plan_kparts(int n_tiles, int n_sm, int nkc, int kparts_max, bool force = false)
{
    std::vector<KPart> out;
    const int kparts =
        force || static_cast<long long>(n_tiles) < 16LL * (n_sm > 0 ? n_sm : 1) ? kparts_max : 1;
    const bool cut = kparts > 1 && nkc >= 2 * kparts;
    for (int t = 0; t < n_tiles; ++t)
    {
        if (!cut)
        {
            out.push_back({t, 0, nkc, 0});
            continue;
        }
        for (int q = 0; q < kparts; ++q)
            out.push_back({t, static_cast<int>(static_cast<long long>(nkc) * q / kparts),
                           static_cast<int>(static_cast<long long>(nkc) * (q + 1) / kparts), 1});
    }
    const int nt = static_cast<int>(out.size()), rem = n_sm > 0 ? nt % n_sm : 0;
    if (n_sm > 0 && nt >= n_sm && rem > 0 && nkc >= 2)
    {
        int parts = 1;
        double best = 1.0;
        for (int sp = 2; sp <= 8 && sp <= nkc; ++sp)
        {
            const double c = std::ceil(static_cast<double>(sp) * rem / n_sm) / sp + 0.01 * sp;
            if (c < best)
            {
                best = c;
                parts = sp;
            }
        }
        if (parts > 1)
        {
            std::vector<KPart> tail(out.end() - rem, out.end());
            out.resize(nt - rem);
            for (const KPart &u : tail)
                for (int q = 0; q < parts; ++q)
                {
                    const int a = u.kc0 + static_cast<int>(static_cast<long long>(u.kc1 - u.kc0) * q / parts);
                    const int b = u.kc0 + static_cast<int>(static_cast<long long>(u.kc1 - u.kc0) * (q + 1) / parts);
                    if (b > a) out.push_back({u.tile, a, b, 1});
                }
        }
    }
    return out;
}

} // namespace sched
} // namespace gb
