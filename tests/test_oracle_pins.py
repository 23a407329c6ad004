"""The oracle pinned against the reference's own golden data (no GPU)."""
import numpy as np
import pytest

from conftest import he_ref, load_h2o, load_he_exx, load_li_g0w0, load_mgo, minimax_ref, oracle_input
from oracle.minimax import minimax_grid
from oracle.rpa_oracle import Options, build_gf, e_min_max, k_lists, r_grid, rpa_correlation_energy


def test_h2o_regression_ec_loops():
    """LibRI-loop restatement reproduces the H2O regression E_c (reference log: -0.306258510 Ha)."""
    s = load_h2o()
    r = rpa_correlation_energy(oracle_input(s), Options(nfreq=16), chi0_impl="loops")
    assert abs(r["ec"].real - s.ec_reference) < 5e-9  # log prints 9 decimals
    assert abs(r["ec"].imag) < 1e-12


def test_h2o_regression_ec_dense():
    s = load_h2o()
    r = rpa_correlation_energy(oracle_input(s), Options(nfreq=16), chi0_impl="dense")
    assert abs(r["ec"].real - s.ec_reference) < 5e-9


def test_minimax_h2o16_matches_reference_log():
    """16-point grids of the H2O run: nodes/weights to the 16 printed digits, matrices to 6 digits."""
    s = load_h2o()
    emin, emax = e_min_max(oracle_input(s))
    g = minimax_grid(16, emin, emax)
    ref = minimax_ref()["h2o16"]
    for k in ("omega", "omega_w", "tau", "tau_w"):
        np.testing.assert_allclose(g[k], ref[k], rtol=2e-15, atol=1e-16)
    for k in ("cos_t2f", "sin_t2f", "cos_f2t"):
        np.testing.assert_allclose(g[k], np.array(ref[k]), rtol=6e-6, atol=1e-10)


def test_minimax_h2_32_matches_reference_log():
    """32-point grids of the H2 G0W0 run: nodes/weights to the printed 16 digits, cosine and sine
    t->f matrices to their 6 digits (the f->t fit is singular at 32 points and not compared)."""
    ref = minimax_ref()["h2_32"]
    g = minimax_grid(32, ref["emin"], ref["emax"])
    for k in ("omega", "omega_w", "tau", "tau_w"):
        np.testing.assert_allclose(g[k], ref[k], rtol=1e-13, atol=1e-16)
    for k in ("cos_t2f", "sin_t2f"):
        m = np.array(ref[k])
        np.testing.assert_allclose(g[k], m, rtol=0, atol=6e-6 * np.abs(m).max())


def test_minimax_ng6_reference_unit_test():
    """check_minimax_ng6_HF_123 of the reference unit tests (omega nodes/weights to 1e-5)."""
    ref = minimax_ref()["ng6_HF_123"]
    g = minimax_grid(6, ref["emin"], ref["emax"])
    assert np.abs(g["omega"] - ref["omega"]).max() < ref["tol"]
    assert np.abs(g["omega_w"] - ref["omega_w"]).max() < ref["tol"]


def test_he_bcc_gf_minus_density_matrix():
    """Known-answer test of the G builder: G(tau -> 0-) = -D for BCC He at Gamma (test_meanfield.cpp)."""
    d = he_ref()
    nb = nao = 8
    wk = np.array(d["wkc_gamma_T"]).reshape(nao, nb)   # [iw][ib]
    wfc = wk.T.astype(complex)[None, None]              # [s][k][ib][iw]
    wg = np.zeros((1, 1, nb))
    wg[0, 0, :d["n_occ_bands"]] = d["occupation"]
    from oracle.rpa_oracle import RPAInput
    inp = RPAInput(n_spins=1, n_kpts=1, n_bands=nb, n_ao=nao, wg=wg, ekb=np.array(d["eig"])[None, None],
                   efermi=d["efermi"], wfc=wfc, latvec=np.eye(3) * 10, period=(1, 1, 1), kvecs=np.zeros((1, 3)),
                   ibz_map=np.zeros(1, int), nao=[nao], nabf=[1], Cs={}, Vq={})
    _, kfrac, _, _ = k_lists(inp)
    G = build_gf(inp, 0, d["tau"], kfrac, r_grid((1, 1, 1)))[(0, 0, 0)]
    D = (wfc[0, 0, :2].T @ wfc[0, 0, :2].conj()).real
    for c in d["checks"]:
        val = D[c["i"], c["j"]] if c["what"] == "dmat_gamma" else G[c["i"], c["j"]]
        assert abs(val - c["value"]) < d["thres"]


def test_he_bcc_periodic_rpa_loops_equal_dense():
    """Real periodic FHI-aims data (BCC He, 2x2x2 k-points, C cells in [0, 2) that LibRI folds):
    the literal LibRI-loop chi0 and the dense restatement give one E_c.  The loop conventions
    they share are pinned by the periodic exchange of the same dataset (test_gw_oracle.py)."""
    s = load_he_exx()
    inp = oracle_input(s)
    a = rpa_correlation_energy(inp, Options(nfreq=16), chi0_impl="dense")["ec"]
    b = rpa_correlation_energy(inp, Options(nfreq=16), chi0_impl="loops")["ec"]
    assert a.real < 0 and abs(a.imag) < 1e-12
    assert abs(a - b) <= 1e-11 * abs(a)


def test_li_spin_polarised_rpa_loops_equal_dense():
    """Two spin channels (the Li atom): the LibRI-loop and dense chi0 give one E_c."""
    inp = oracle_input(load_li_g0w0())
    assert inp.n_spins == 2
    a = rpa_correlation_energy(inp, Options(nfreq=16), chi0_impl="dense")["ec"]
    b = rpa_correlation_energy(inp, Options(nfreq=16), chi0_impl="loops")["ec"]
    assert a.real < 0 and abs(a - b) <= 1e-12 * abs(a)


def unfold_ibz(s):
    """The same system with every k-point irreducible: V at the time-reversed partners as the
    conjugate of the representative's, weights 1/n_k each."""
    import copy
    t = copy.copy(s)
    vq = {}
    for k in range(s.n_kpts):
        rep = int(s.ibz_map[k])
        for (ik, I, J), v in s.Vq.items():
            if ik == rep:
                vq[(k, I, J)] = v if k == rep else v.conj()
    t.Vq = vq
    t.ibz_map = np.arange(s.n_kpts)
    return t


def test_mgo_ibz_reduction_gives_the_full_bz_ec():
    """MgO: E_c over the 14 irreducible q-points with weights count/n_k equals E_c over all 27
    with V(-q) = V(q)^*, i.e. the IBZ weighting of the E_c sum (compute_rpa.cpp) is exact."""
    s = load_mgo()
    a = rpa_correlation_energy(oracle_input(s), Options(nfreq=s.nfreq))
    b = rpa_correlation_energy(oracle_input(unfold_ibz(s)), Options(nfreq=s.nfreq))
    assert len(a["per_q"]) == 14 and len(b["per_q"]) == 27
    assert abs(a["ec"] - b["ec"]) <= 1e-10 * abs(a["ec"])  # rounding: 2.5e-12 measured


def test_mgo_gamma_coulomb_is_indefinite():
    """The bare Coulomb matrix V(q = Gamma) of the real MgO input is indefinite (its smallest
    eigenvalue is about -0.2, the largest about 42), so V = L L^H does not exist there and a
    Cholesky-form E_c must take that q by the LU form (epsilon.cpp:489-536), which needs no
    definiteness.  The other irreducible q have positive definite V(q).  This keeps the GPU
    path's LU fallback exercised by the MgO parity test."""
    from oracle.rpa_oracle import assemble_full, k_lists
    s = load_mgo()
    inp = oracle_input(s)
    _, _, ibz_order, _ = k_lists(inp)
    lows = []
    for ikf in ibz_order:
        blocks = {(I, J): v for (ik, I, J), v in inp.Vq.items() if ik == ikf}
        lows.append(np.linalg.eigvalsh(assemble_full(blocks, inp.nabf)).min())
    assert lows[0] < -0.1  # Gamma
    assert all(v > 0 for v in lows[1:])
