"""LibRI's periodic folding of the RI coefficient blocks (librpa_gb300/csrc/cs_fold.h), compiled
for the host: cell vectors taken modulo the BvK period into the centred range, blocks that land
on one (I, J, cell) key summed, the threshold filter applied to the sums, first-seen order kept.
The oracle's cs_tensors follows the same rule (thirdparty/LibRI/include/RI/ri/RI_Tools.hpp:49-67)."""
import random
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle.rpa_oracle import centred_mod

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def fold(tmp_path_factory):
    exe = tmp_path_factory.mktemp("csf") / "cs_fold_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "librpa_gb300" / "csrc"),
                    str(ROOT / "tests" / "cs_fold_check.cpp"), "-o", str(exe)], check=True)

    def run(period, thr, blocks):
        lines = [f"{period[0]} {period[1]} {period[2]} {thr!r} {len(blocks)}"]
        for (I, J, R, sizes, vals) in blocks:
            lines.append(f"{I} {J} {R[0]} {R[1]} {R[2]} {sizes[0]} {sizes[1]} {sizes[2]} "
                         + " ".join(repr(float(v)) for v in vals))
        out = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True,
                             check=True).stdout.split("\n")
        n = int(out[0])
        res = []
        for l in out[1:1 + n]:
            t = l.split()
            res.append((int(t[0]), int(t[1]), int(t[2]), np.array([float(x) for x in t[3:]])))
        return res
    return run


def _model(period, thr, blocks):
    cells = [(x, y, z) for x in range(-(period[0] // 2), (period[0] - 1) // 2 + 1)
             for y in range(-(period[1] // 2), (period[1] - 1) // 2 + 1)
             for z in range(-(period[2] // 2), (period[2] - 1) // 2 + 1)]
    order, acc = [], {}
    for (I, J, R, _s, vals) in blocks:
        key = (I, J, cells.index(centred_mod(R, period)))
        if key not in acc:
            order.append(key)
            acc[key] = np.array(vals, float)
        else:
            acc[key] = acc[key] + vals
    return [(k[0], k[1], k[2], acc[k]) for k in order if not (thr > 0 and np.abs(acc[k]).max() <= thr)]


def _check(got, want):
    assert [g[:3] for g in got] == [w[:3] for w in want]
    for g, w in zip(got, want):
        np.testing.assert_allclose(g[3], w[3], rtol=0, atol=1e-15)


def test_centred_blocks_pass_through_unchanged(fold):
    period = (3, 2, 1)
    rng = np.random.default_rng(0)
    blocks = [(0, 1, (x, y, 0), (2, 1, 3), rng.standard_normal(6)) for x in (-1, 0, 1) for y in (-1, 0)]
    got = fold(period, 0.0, blocks)
    assert len(got) == 6
    _check(got, _model(period, 0.0, blocks))


def test_out_of_range_cells_fold_and_collisions_sum(fold):
    period = (2, 2, 2)
    rng = np.random.default_rng(1)
    # the Born-von Karman range [0, n) of FHI-aims output, plus an image one period away
    blocks = [(0, 0, (x, y, z), (1, 2, 2), rng.standard_normal(4)) for x in (0, 1) for y in (0, 1) for z in (0, 1)]
    blocks.append((0, 0, (2, 0, 0), (1, 2, 2), rng.standard_normal(4)))   # folds onto (0, 0, 0)
    blocks.append((0, 0, (-1, 0, 1), (1, 2, 2), rng.standard_normal(4)))  # folds onto (1, 0, 1)
    got = fold(period, 0.0, blocks)
    assert len(got) == 8
    _check(got, _model(period, 0.0, blocks))


def test_threshold_applies_to_the_sum(fold):
    period = (2, 1, 1)
    v = np.array([1e-3, -2e-3])
    blocks = [(0, 1, (0, 0, 0), (1, 1, 2), v), (0, 1, (2, 0, 0), (1, 1, 2), -v + 1e-9),  # sum ~1e-9: dropped
              (0, 1, (1, 0, 0), (1, 1, 2), 1e-9 * np.ones(2)), (0, 1, (-1, 0, 0), (1, 1, 2), v)]  # sum above
    got = fold(period, 1e-6, blocks)
    want = _model(period, 1e-6, blocks)
    assert len(got) == 1
    _check(got, want)


def test_random_block_sets(fold):
    rng = random.Random(4)
    for _ in range(40):
        period = tuple(rng.choice([1, 2, 3, 4]) for _ in range(3))
        blocks = []
        for _b in range(rng.randint(1, 30)):
            I, J = rng.randrange(3), rng.randrange(3)
            R = tuple(rng.randint(-5, 5) for _ in range(3))
            sizes = (1 + I, 1 + J, 2)
            blocks.append((I, J, R, sizes, np.array([rng.uniform(-1, 1) * 10 ** rng.randint(-8, 0)
                                                     for _ in range(sizes[0] * sizes[1] * 2)])))
        thr = rng.choice([0.0, 1e-6, 1e-3])
        _check(fold(period, thr, blocks), _model(period, thr, blocks))
