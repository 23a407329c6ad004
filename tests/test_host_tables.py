"""The GPU path's host index and phase tables (librpa_gb300_phase_tables, no GPU needed) against
the oracle's conventions, on real periodic FHI-aims input (BCC He, 2x2x2 k-points) and on a
synthetic cell with an IBZ reduction: the BvK cell list, the IBZ list and weights, the G(R)
Bloch phases and the R -> q Fourier phases."""
import math

import numpy as np
import pytest

import librpa_gb300 as L
from conftest import load_he_exx, load_mgo, oracle_input
from librpa_gb300 import synthetic as sy
from oracle.rpa_oracle import TWO_PI, k_lists, r_grid


def _check(s):
    h = L.Handler()
    L.load_system(h, s)
    t = L.phase_tables(h, s.n_kpts)
    inp = oracle_input(s)
    rl = r_grid(inp.period)
    assert [tuple(r) for r in t["cells"]] == rl
    klist, kfrac, ibz_order, ibz_w = k_lists(inp)
    assert list(t["ibz_rep"]) == ibz_order
    np.testing.assert_allclose(t["ibz_w"], ibz_w, rtol=0, atol=1e-15)
    # build_gf: G(R) += e^{i ang} G(k), ang = -2 pi kfrac . R
    for k in range(inp.n_kpts):
        for c, R in enumerate(rl):
            ang = -float(np.dot(kfrac[k], R)) * TWO_PI
            np.testing.assert_allclose(t["g_phase"][k, c], [math.cos(-ang), math.sin(-ang)], atol=1e-13)
    # ft_ct_accumulate: arg = 2 pi q . (R latvec), q = k_cart / 2 pi of the IBZ point
    for q, kq in enumerate(ibz_order):
        for c, R in enumerate(rl):
            arg = float(np.dot(klist[kq], np.asarray(R, float) @ inp.latvec)) * TWO_PI
            np.testing.assert_allclose(t["q_phase"][q, c], [math.cos(arg), math.sin(arg)], atol=1e-13)
    return t


def test_he_bcc_fhi_aims_tables(lib):
    t = _check(load_he_exx())
    assert len(t["cells"]) == 8 and len(t["ibz_rep"]) == 8


@pytest.mark.parametrize("period", [(2, 1, 1), (3, 2, 1), (3, 3, 3)])
def test_synthetic_tables(lib, period):
    s = sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[6, 8], period=period, nocc=2, seed=5)
    t = _check(s)
    assert len(t["ibz_rep"]) <= s.n_kpts


def test_mgo_ibz_reduced_tables(lib):
    """The only real input with an IBZ reduction (MgO: 27 k-points, 14 irreducible)."""
    t = _check(load_mgo())
    assert len(t["cells"]) == 27 and len(t["ibz_rep"]) == 14
    assert abs(t["ibz_w"].sum() - 1.0) < 1e-14
