"""The work scheduling of the kernels (librpa_gb300/csrc/work_schedule.h), compiled for the host:

- tile_coords (split GEMM, k_tc_gemm.cu): every output tile exactly once, in groups of
  RASTER_GROUP tile rows walked column by column; in lower-tile mode exactly the tiles with
  nt <= mt, in the same group order;
- ozaki_item (tensor-core Cholesky update, k_chol_ozaki.cu): the row tiles that meet the lower
  triangle of each 128-column block exactly once, in chunks of at most OZ_CHUNK row tiles, and
  nothing past the grid size ozaki_items reports;
- pack_row_tiles (chi0 contraction, tc_chi0.cu): every row of every row group exactly once, in
  order, in tiles of at most 128 rows over at most max_slots groups, each tile closed only when
  full, out of slots or at the last group;
- plan_kparts (chi0 contraction, tc_chi0.cu): the K chunks of every tile exactly once, K parts
  flagged for atomic accumulation, the plan within the work list the contraction allocates
  (n_tiles T1_KPARTS + 8 n_sm entries) and a greedy makespan within one part of the uncut
  tiles' (no longer at all on the tabulated shapes).
"""
import heapq
import random
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
G = 8          # RASTER_GROUP
OZ_CHUNK = 32  # row tiles per CTA of the Cholesky update
T1_KPARTS = 4


@pytest.fixture(scope="module")
def sched(tmp_path_factory):
    exe = tmp_path_factory.mktemp("sched") / "sched_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "librpa_gb300" / "csrc"),
                    str(ROOT / "tests" / "sched_check.cpp"), "-o", str(exe)], check=True)

    def run(line):
        out = subprocess.run([str(exe)], input=line + "\n", capture_output=True, text=True, check=True)
        return out.stdout.split("\n")[:-1]
    return run


@pytest.mark.parametrize("ntm,ntn", [(1, 1), (1, 7), (7, 1), (8, 8), (9, 5), (17, 3), (20, 20), (33, 40), (80, 6)])
def test_gemm_tiles_cover_the_grid_in_raster_groups(sched, ntm, ntn):
    tiles = [tuple(map(int, l.split())) for l in sched(f"T {ntm} {ntn} 0")]
    assert sorted(tiles) == [(m, n) for m in range(ntm) for n in range(ntn)]
    # group g holds tile rows [8g, 8g + 8), column by column, rows ascending inside a column
    t = 0
    for g0 in range(0, ntm, G):
        gm = min(G, ntm - g0)
        for n in range(ntn):
            for m in range(g0, g0 + gm):
                assert tiles[t] == (m, n), (t, tiles[t])
                t += 1


@pytest.mark.parametrize("nt", [1, 2, 7, 8, 9, 16, 17, 23, 40, 81])
def test_gemm_lower_tiles_cover_the_triangle_in_raster_groups(sched, nt):
    tiles = [tuple(map(int, l.split())) for l in sched(f"T {nt} {nt} 1")]
    assert sorted(tiles) == [(m, n) for m in range(nt) for n in range(m + 1)]
    want = []
    for g0 in range(0, nt, G):
        gm = min(G, nt - g0)
        for n in range(g0 + gm):
            want += [(m, n) for m in range(max(g0, n), g0 + gm)]
    assert tiles == want


@pytest.mark.parametrize("R", [1, 31, 32, 33, 127, 128, 129, 500, 1024, 1025, 4000, 8128])
@pytest.mark.parametrize("trsm", [False, True])
def test_cholesky_update_items_cover_the_lower_triangle(sched, R, trsm):
    nti = (R + 31) // 32
    njm = 1 if trsm else (R + 127) // 128
    out = sched(f"O {njm} {nti} {OZ_CHUNK}")
    n = int(out[0])
    items = [tuple(map(int, l.split())) for l in out[1:1 + n]]
    assert out[1 + n] == "end 1"
    seen = set()
    for jm, ti0, cnt in items:
        assert 0 <= jm < njm and 1 <= cnt <= OZ_CHUNK and ti0 + cnt <= nti
        for ti in range(ti0, ti0 + cnt):
            assert (jm, ti) not in seen
            seen.add((jm, ti))
    # row tile ti (rows 32 ti .. 32 ti + 31) meets column block jm (columns 128 jm ..) iff
    # 32 ti + 31 >= 128 jm
    want = {(jm, ti) for jm in range(njm) for ti in range(nti) if 32 * ti + 31 >= 128 * jm}
    assert seen == want


def _pack(sched, rows, bm, slots):
    out = sched(f"P {bm} {slots} {len(rows)} " + " ".join(map(str, rows)))
    n = int(out[0])
    return [tuple(map(int, l.split())) for l in out[1:1 + n]]


def _check_pack(tiles, rows, bm, slots):
    covered = []  # (group, row) in tile order
    for g0, r0, nrows, nslot in tiles:
        assert 1 <= nslot <= slots and 0 <= nrows <= bm
        g, r, left, touched = g0, r0, nrows, 0
        while left > 0 or (touched < nslot and g < len(rows)):
            take = min(rows[g] - r, left)
            covered += [(g, r + k) for k in range(take)]
            left -= take
            touched += 1
            r += take
            if r == rows[g]:
                g, r = g + 1, 0
            if touched == nslot:
                break
        assert left == 0 and touched == nslot
        # closed because full, out of slots or past the last group
        assert nrows == bm or nslot == slots or g == len(rows)
    assert covered == [(g, r) for g in range(len(rows)) for r in range(rows[g])]


@pytest.mark.parametrize("rows,slots", [
    ([40] * 7, 5), ([40] * 30, 5), ([13, 200, 7, 128, 128, 1], 4), ([128] * 5, 2), ([129, 127, 2], 3),
    ([300], 2), ([1] * 300, 4), ([40, 0, 40, 40, 40], 5), ([], 3)])
def test_row_tiles_cover_each_row_once(sched, rows, slots):
    tiles = _pack(sched, rows, 128, slots)
    _check_pack(tiles, rows, 128, slots)


def test_row_tiles_random_groups(sched):
    rng = random.Random(13)
    for _ in range(200):
        rows = [rng.choice([rng.randint(1, 300), 40, 80, 128]) for _ in range(rng.randint(1, 60))]
        slots = max(2, (128 + min(rows) - 1) // min(rows) + 1) if rng.random() < 0.7 else rng.randint(1, 6)
        _check_pack(_pack(sched, rows, 128, slots), rows, 128, slots)


def test_row_tiles_slot_count_never_binds_at_the_default(sched):
    # the contraction gives every tile ceil(128 / min rows) + 1 slots; with that many no tile
    # closes for lack of slots before it is full (except the last)
    rng = random.Random(17)
    for _ in range(200):
        rows = [rng.randint(8, 260) for _ in range(rng.randint(1, 40))]
        slots = (128 + min(rows) - 1) // min(rows) + 1
        tiles = _pack(sched, rows, 128, slots)
        assert all(t[2] == 128 for t in tiles[:-1]), (rows, tiles)


def _makespan(units, n_sm, nkc):
    """Greedy list schedule in launch order, each unit costing its share of K."""
    free = [0.0] * n_sm
    for _, a, b, _ in units:
        t = heapq.heappop(free)
        heapq.heappush(free, t + (b - a) / nkc)
    return max(free)


def _plan(sched, n_tiles, n_sm, nkc, kmax=T1_KPARTS):
    out = sched(f"K {n_tiles} {n_sm} {nkc} {kmax}")
    n = int(out[0])
    return [tuple(map(int, l.split())) for l in out[1:1 + n]]


def _check_plan(units, n_tiles, n_sm, nkc):
    parts = {}
    for tile, a, b, split in units:
        assert 0 <= tile < n_tiles and 0 <= a < b <= nkc and split in (0, 1)
        parts.setdefault(tile, []).append((a, b, split))
    assert sorted(parts) == list(range(n_tiles))
    for tile, ps in parts.items():
        ps.sort()
        assert ps[0][0] == 0 and ps[-1][1] == nkc
        assert all(ps[i][1] == ps[i + 1][0] for i in range(len(ps) - 1)), (tile, ps)
        # a tile in one piece writes its output, a tile in parts adds into it
        assert all(s == (0 if len(ps) == 1 else 1) for _, _, s in ps), (tile, ps)
    assert len(units) <= n_tiles * T1_KPARTS + 8 * n_sm


@pytest.mark.parametrize("n_tiles,n_sm,nkc", [
    (1, 152, 40), (91, 152, 40), (152, 152, 40), (153, 152, 40), (1155, 152, 31), (1155, 152, 7),
    (2431, 152, 40), (2432, 152, 40), (2433, 152, 40), (10240, 152, 20), (10300, 152, 1),
    (300, 148, 3), (37, 1, 5), (5, 0, 9)])
def test_kpart_plan_covers_k_exactly_once(sched, n_tiles, n_sm, nkc):
    units = _plan(sched, n_tiles, n_sm, nkc)
    _check_plan(units, n_tiles, n_sm, nkc)
    if n_sm > 0:
        whole = [(t, 0, nkc, 0) for t in range(n_tiles)]
        assert _makespan(units, n_sm, nkc) <= _makespan(whole, n_sm, nkc) + 1e-12


def test_kpart_plan_random_shapes(sched):
    # K parts of unequal length (nkc not a multiple of the part count) can leave a greedy
    # schedule up to one part longer than the whole tiles' (list scheduling: at most the mean
    # load plus one unit); the cases of the table above, on GB300's SM count, come out no longer
    rng = random.Random(3)
    for _ in range(60):
        n_sm = rng.choice([1, 2, 13, 148, 152])
        n_tiles = rng.randint(1, 40 * n_sm)
        nkc = rng.randint(1, 64)
        units = _plan(sched, n_tiles, n_sm, nkc)
        _check_plan(units, n_tiles, n_sm, nkc)
        whole = [(t, 0, nkc, 0) for t in range(n_tiles)]
        longest = max(b - a for _, a, b, _ in units) / nkc
        assert _makespan(units, n_sm, nkc) <= _makespan(whole, n_sm, nkc) + longest + 1e-12, (n_tiles, n_sm, nkc)


def test_kpart_plan_worked_example(sched):
    # 91 tiles of 40 chunks on 152 SMs: under 16 waves, so 364 quarter-tiles of 10 chunks; the
    # last wave's 60 quarter-tiles become 5 parts of 2 chunks each
    units = _plan(sched, 91, 152, 40)
    assert len(units) == 304 + 300
    assert all(b - a == 10 for _, a, b, _ in units[:304])
    assert all(b - a == 2 for _, a, b, _ in units[304:])
    # 16 waves or more: tiles stay whole, only the partial last wave is cut
    units = _plan(sched, 2433, 152, 40)
    assert all((a, b, s) == (0, 40, 0) for _, a, b, s in units[:2432])
    assert len(units) > 2433 and all(s == 1 for *_, s in units[2432:])
