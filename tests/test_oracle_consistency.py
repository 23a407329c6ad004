"""Oracle self-consistency: literal LibRI loops vs the supercell reformulation (no GPU)."""
import numpy as np
import pytest

from conftest import oracle_input
from librpa_gb300 import synthetic as sy
from oracle.rpa_oracle import (Options, blocks_of, build_gf, cal_chi0s_dense, cal_chi0s_loops, centred_mod,
                               cs_tensors, k_lists, r_grid, rpa_correlation_energy)


@pytest.mark.parametrize("period,nao,nabf", [((2, 1, 1), [3, 5], [7, 10]), ((3, 1, 1), [4, 2], [6, 9]),
                                             ((2, 2, 1), [3, 3], [5, 5]), ((1, 1, 1), [2, 4, 3], [4, 6, 5])])
def test_chi0_loops_equal_dense(period, nao, nabf):
    s = sy.small_periodic(n_atoms=len(nao), nao=nao, nabf=nabf, period=period, nocc=2, seed=11)
    inp = oracle_input(s)
    _, kfrac, _, _ = k_lists(inp)
    rl = r_grid(inp.period)
    tau = 0.37
    Gp = blocks_of(build_gf(inp, 0, tau, kfrac, rl), inp.nao)
    Gn = blocks_of(build_gf(inp, 0, -tau, kfrac, rl), inp.nao)
    C = cs_tensors(inp)
    a = cal_chi0s_loops(C, Gp, Gn, inp.n_atoms, inp.period)
    b = cal_chi0s_dense(C, Gp, Gn, inp.nao, inp.nabf, inp.period)
    for key, v in b.items():
        assert np.allclose(a[key], v, rtol=1e-11, atol=1e-13 * np.abs(v).max())


def test_centred_mod_matches_libri():
    # LibRI Array_Operator: (i % n + 3n/2) % n - n/2 with C remainder semantics
    for n in (1, 2, 3, 4, 5):
        for i in range(-9, 10):
            r = centred_mod((i, 0, 0), (n, 1, 1))[0]
            assert -(n // 2) <= r <= (n - 1) // 2
            assert (r - i) % n == 0


def test_gf_real_symmetry():
    """Re G[I;J,R]_{ij} = Re G[J;I,-R]_{ji}, which the reformulated T2 term relies on."""
    s = sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[5, 6], period=(3, 1, 1), seed=5)
    inp = oracle_input(s)
    _, kfrac, _, _ = k_lists(inp)
    rl = r_grid(inp.period)
    G = build_gf(inp, 0, 0.5, kfrac, rl)
    for R in rl:
        mR = centred_mod((-R[0], -R[1], -R[2]), inp.period)
        assert np.allclose(G[R], G[mR].T, atol=1e-13)


def test_ec_negative_and_real_parts_consistent():
    s = sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[5, 6], period=(2, 1, 1), seed=3)
    r = rpa_correlation_energy(oracle_input(s), Options(nfreq=16, minimax_emin=s.minimax_emin,
                                                        minimax_emax=s.minimax_emax))
    assert r["ec"].real < 0
    assert abs(r["ec"].imag) < 1e-10 * abs(r["ec"].real)


@pytest.mark.parametrize("split", [False, True])
def test_cell_vectors_fold_like_libri(split):
    """C blocks given on cells [0, n), or split over two images a period apart, give the E_c of
    the centred input: cs_tensors folds them as LibRI's cal_period does."""
    from oracle.rpa_oracle import rpa_correlation_energy
    s = sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[6, 8], period=(3, 2, 1), nocc=2, seed=5)
    t = sy.with_cells_relabelled(s, split=split)
    assert set(t.Cs) != set(s.Cs)
    o = Options(nfreq=s.nfreq, minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)
    a = rpa_correlation_energy(oracle_input(s), o)["ec"]
    b = rpa_correlation_energy(oracle_input(t), o)["ec"]
    assert abs(a - b) <= 1e-13 * abs(a)
