"""The G0W0 oracle (oracle/gw_oracle.py) pinned against the reference's H2O G0W0 regression run,
and its pieces checked on their own (no GPU)."""
import numpy as np
import pytest

from conftest import load_h2o_g0w0, load_he_exx, load_li_g0w0, load_mgo, oracle_input
from oracle.gw_oracle import (HA2EV, BandPoints, Pade, cal_hs_batched, cal_hs_cells, cal_hs_loops, coulomb_r, dmat_r, exx_kgrid,
                              full_from_blocks, g0w0_gamma, g0w0_kgrid, ordered_blocks, power_hemat,
                              qpe_solve, wc_freq)
from oracle.rpa_oracle import Options, cs_tensors


@pytest.fixture(scope="module")
def h2o():
    s = load_h2o_g0w0()
    inp = oracle_input(s)
    r = g0w0_gamma(inp, s.v_cut, s.vxc, Options(nfreq=s.nfreq), n_params=s.n_params_anacon)
    return s, inp, r


def test_h2o_quasiparticle_table(h2o):
    """Every column of the reference's table (refs/g0w0_aims_mole_H2O_libri/librpa/librpa.out,
    printed to 5 decimals in eV; the regression suite allows 5e-4 eV) to its print precision."""
    s, inp, r = h2o
    t = s.qp_table
    assert t.shape == (24, 8) and all(f == 0 for f in r["info"][0])
    got = {
        "e_mf": inp.ekb[0, 0] * HA2EV,
        "v_xc": s.vxc[0, 0] * HA2EV,
        "v_exx": r["vexx"][0] * HA2EV,
        "ReSigc": r["sigc"][0].real * HA2EV,
        "ImSigc": r["sigc"][0].imag * HA2EV,
        "e_qp": r["e_qp"][0] * HA2EV,
    }
    for col, name in enumerate(["e_mf", "v_xc", "v_exx", "ReSigc", "ImSigc", "e_qp"], start=2):
        np.testing.assert_allclose(got[name], t[:, col], rtol=0, atol=6e-6, err_msg=name)
    # the printed e_qp is e_mf - v_xc + v_exx + Re Sigma_c (driver/task/g0w0.cpp:274)
    np.testing.assert_allclose(t[:, 2] - t[:, 3] + t[:, 4] + t[:, 5], t[:, 7], atol=2.5e-5)


def test_li_atom_both_spin_channels():
    """The spin-polarised Li atom (refs/g0w0_aims_Li_atom_libri/librpa/librpa.out, 16 points,
    all of them in the Pade fit): every column of both spin channels to print precision."""
    s = load_li_g0w0()
    inp = oracle_input(s)
    assert inp.n_spins == 2
    r = g0w0_gamma(inp, s.v_cut, s.vxc, Options(nfreq=s.nfreq), n_params=s.n_params_anacon)
    for sp in range(2):
        t = s.qp_tables[sp]
        got = np.c_[inp.ekb[sp, 0] * HA2EV, s.vxc[sp, 0] * HA2EV, r["vexx"][sp] * HA2EV,
                    r["sigc"][sp].real * HA2EV, r["sigc"][sp].imag * HA2EV, r["e_qp"][sp] * HA2EV]
        np.testing.assert_allclose(got, t[:, 2:], rtol=0, atol=6e-6, err_msg=f"spin {sp}")


def test_periodic_exchange_bcc_he_every_k_point():
    """Periodic exchange (2-atom cell, 2x2x2 k-points, C blocks given on cells [0, 2) that LibRI
    folds into the centred BvK range): v_exx of all 8 bands at all 8 k-points against
    refs/exx_aims_bccHe_k_parallel_libri/librpa/librpa.out (5 decimals in Hartree; the suite
    checks the first k-point to 1e-4)."""
    s = load_he_exx()
    inp = oracle_input(s)
    assert inp.n_kpts == 8 and any(max(R) > 0 for (_I, _J, R) in inp.Cs)
    e = exx_kgrid(inp, s.v_cut)
    t = s.exx_tables
    assert t.shape == (8, 8, 3)
    np.testing.assert_allclose(e[0], t[:, :, 1], rtol=0, atol=6e-6)


def test_periodic_exchange_mgo_ibz_reduced():
    """MgO, 3x3x3 k-points of which 14 are irreducible by time reversal: the truncated Coulomb is
    given at the IBZ points only, so V(R) takes the conjugated partners (FT_Vq, coulmat.cpp:7-90).
    v_exx of all 17 states at all 27 k-points against refs/g0w0_aims_MgO_libri/librpa/librpa.out
    (5 decimals in eV)."""
    s = load_mgo()
    inp = oracle_input(s)
    assert inp.n_kpts == 27 and len(set(int(x) for x in inp.ibz_map)) == 14
    e = exx_kgrid(inp, s.v_cut)
    np.testing.assert_allclose(e[0] * HA2EV, s.qp_tables[:, :, 4], rtol=0, atol=6e-6)


def test_kgrid_chain_reduces_to_the_gamma_chain(h2o):
    """g0w0_kgrid on the H2O molecule (one k-point, no head correction) gives g0w0_gamma's
    quasi-particle energies: the IBZ unfolding, BvK shift and Bloch sums reduce to the identity."""
    s, inp, r = h2o
    k = g0w0_kgrid(inp, s.v_cut, s.vxc, Options(nfreq=s.nfreq), n_params=s.n_params_anacon)
    np.testing.assert_allclose(k["vexx"][0, 0], r["vexx"][0], rtol=0, atol=1e-12)
    np.testing.assert_allclose(k["e_qp"][0][0], r["e_qp"][0], rtol=0, atol=1e-10)
    np.testing.assert_allclose(k["sigc"][0][0], r["sigc"][0], rtol=0, atol=1e-10)


def test_band_points_on_the_scf_grid_reproduce_the_kgrid_results(mgo):
    """Band k-points (task = g0w0_band) placed on SCF k-points, with the SCF eigenpairs, give the
    k-grid quasi-particle energies: Sigma_c(R) and H_x(R) summed at arbitrary k are the same
    Bloch sums.  Three MgO k-points, one of them off the IBZ representatives."""
    from oracle.rpa_oracle import k_lists
    s, inp, full = mgo
    _, kfrac, _, _ = k_lists(inp)
    pick = [0, 5, 17]
    band = BandPoints(kfrac=kfrac[pick], wfc=inp.wfc[:, pick], ekb=inp.ekb[:, pick], efermi=inp.efermi,
                      vxc=s.vxc[:, pick])
    part = g0w0_kgrid(inp, s.v_cut, s.vxc, Options(nfreq=s.nfreq), n_params=s.n_params_anacon, epsmac=s.epsmac,
                      band=band)
    np.testing.assert_allclose(part["vexx"][0], full["vexx"][0][pick], rtol=0, atol=1e-12)
    np.testing.assert_allclose(part["e_qp"][0], full["e_qp"][0][pick], rtol=0, atol=1e-10)


def test_batched_label_sum_equals_literal_loops():
    """cal_hs_batched (the site loop over L batched by cells) and cal_hs_cells (every cell sum
    vectorised) against the literal loops, on the periodic BCC He exchange (8 cells)."""
    from oracle.rpa_oracle import r_grid
    s = load_he_exx()
    inp = oracle_input(s)
    rl = r_grid(inp.period)
    C = cs_tensors(inp)
    VR, D = coulomb_r(inp, s.v_cut, rl), dmat_r(inp, 0, rl)
    a = cal_hs_loops(C, VR, D, inp.n_atoms, inp.period)
    b = cal_hs_batched(C, VR, D, inp.n_atoms, inp.period)
    c = cal_hs_cells(C, VR, D, inp.nao, inp.nabf, inp.period)
    assert sorted(a) == sorted(b) and set(a) <= set(c)
    scale = max(np.abs(v).max() for v in a.values())
    for k in a:
        np.testing.assert_allclose(b[k], a[k], rtol=0, atol=1e-13 * scale)
        np.testing.assert_allclose(c[k], a[k], rtol=0, atol=1e-13 * scale)
    assert all(np.abs(c[k]).max() == 0.0 for k in c if k not in a)


@pytest.fixture(scope="module")
def mgo():
    s = load_mgo()
    inp = oracle_input(s)
    r = g0w0_kgrid(inp, s.v_cut, s.vxc, Options(nfreq=s.nfreq), n_params=s.n_params_anacon, epsmac=s.epsmac)
    return s, inp, r


def test_mgo_kgrid_g0w0_tables(mgo):
    """Periodic G0W0 (MgO, 3x3x3 k-points from 14 IBZ points, head of the dielectric matrix
    replaced by eps_mac, 6 minimax points, all 6 in the Pade fit): every column of all 27 tables
    of refs/g0w0_aims_MgO_libri/librpa/librpa.out to print precision (459 states)."""
    s, inp, r = mgo
    t = s.qp_tables
    got = np.stack([r["vexx"][0] * HA2EV, r["sigc"][0].real * HA2EV, r["sigc"][0].imag * HA2EV,
                    r["e_qp"][0] * HA2EV], axis=-1)
    np.testing.assert_allclose(got, t[:, :, 4:8], rtol=0, atol=6e-6)


def test_sigma_on_the_imaginary_axis_has_negative_imaginary_part(h2o):
    """Sigma_c(i omega) = sum_s |M_s|^2 / (i omega - E_s) with positive weights, so every KS
    diagonal element has Im Sigma_c(i omega) < 0 at omega > 0, and |Sigma_c| -> 0 as omega grows."""
    s, inp, r = h2o
    sig = r["sigc_iw"][0]
    assert np.all(sig.imag < 0)
    assert np.all(np.abs(sig[:, -1]) < np.abs(sig).max(axis=1))


def _dense_hs(C, W, D, nao, nabf):
    """H_{pq} = sum U[a, p, r] W[a, b] U[b, q, s] D[r, s] with U[a, p, r] = C_a[p, r] + C_a[r, p]
    the orbital-symmetrised coefficient: the four LibRI labels summed in closed form."""
    oa = np.concatenate([[0], np.cumsum(nao)]).astype(int)
    ob = np.concatenate([[0], np.cumsum(nabf)]).astype(int)
    T = np.zeros((ob[-1], oa[-1], oa[-1]))
    for (I, K, _R), c in C.items():
        T[ob[I]:ob[I + 1], oa[I]:oa[I + 1], oa[K]:oa[K + 1]] += c
    U = T + T.transpose(0, 2, 1)
    return np.einsum("apr,ab,bqs,rs->pq", U, W, U, D, optimize=True)


def test_label_sum_equals_symmetrised_dense_form(h2o):
    s, inp, r = h2o
    rng = np.random.default_rng(3)
    C = cs_tensors(inp, 0.0)
    nb, na = sum(inp.nabf), inp.n_ao
    W = rng.standard_normal((nb, nb))
    W = W + W.T
    D = rng.standard_normal((na, na))
    D = D + D.T
    H = full_from_blocks(cal_hs_loops(C, ordered_blocks(W, inp.nabf), ordered_blocks(D, inp.nao),
                                      inp.n_atoms, (1, 1, 1)), inp.nao)
    Hd = _dense_hs(C, W, D, inp.nao, inp.nabf)
    np.testing.assert_allclose(H, Hd, rtol=0, atol=1e-12 * np.abs(Hd).max())


def test_pade_reproduces_a_rational_function():
    rng = np.random.default_rng(0)
    poles = rng.uniform(-2, 2, 3) + 1j * rng.uniform(0.1, 1, 3)
    res = rng.uniform(0.2, 1, 3)

    def f(z):
        return sum(a / (z - p) for a, p in zip(res, poles))

    xs = [1j * w for w in np.linspace(0.05, 8, 16)]
    pade = Pade(16, xs, [f(x) for x in xs])
    for z in [0.3, -1.1 + 0.2j, 2.5j, -0.7]:
        assert abs(pade(z) - f(z)) < 1e-8 * max(1.0, abs(f(z)))
    # more points than parameters: evenly spaced selection, the last point kept
    p2 = Pade(6, xs, [f(x) for x in xs])
    assert p2.n == 6 and p2.y[0] == f(xs[0])


def test_qpe_solver_fixed_point():
    # Sigma(x) = A / (x - P): a two-point Thiele fraction represents a single pole exactly
    A, P = 0.1, -2.0
    xs = [0.5j, 1.5j]
    pade = Pade(2, xs, [A / (x - P) for x in xs])
    assert abs(pade(0.7) - A / (0.7 - P)) < 1e-14
    e_mf, ef, vxc, sx = -0.4, -0.1, -0.3, -0.6
    info, e, sig = qpe_solve(pade, e_mf=e_mf, e_fermi=ef, vxc=vxc, sigma_x=sx)
    assert info == 0
    assert abs(sig - A / (e - ef - P)) < 1e-6          # Sigma at the last iterate
    assert abs(e - (e_mf - vxc + sx + A / (e - ef - P))) < 1e-5   # the QP equation


def test_power_hemat_filters_below_threshold():
    rng = np.random.default_rng(1)
    Q, _ = np.linalg.qr(rng.standard_normal((6, 6)))
    w = np.array([-1e-3, 1e-9, 0.5, 1.0, 2.0, 4.0])
    A = (Q * w) @ Q.T
    S = power_hemat(A, 0.5, 0.0)       # negative eigenvalue dropped
    np.testing.assert_allclose(S @ S, (Q * np.where(w >= 0, w, 0)) @ Q.T, atol=1e-12)
    S = power_hemat(A, 0.5, 1e-6)      # everything below 1e-6 dropped
    np.testing.assert_allclose(S @ S, (Q * np.where(w >= 1e-6, w, 0)) @ Q.T, atol=1e-12)


def test_wc_is_vcut_half_epsinv_minus_one_vcut_half():
    """Without truncation (V_cut = V) and a small chi0, Wc = (1 - V chi0)^-1 V - V."""
    rng = np.random.default_rng(2)
    A = rng.standard_normal((8, 8))
    V = A @ A.T + 8 * np.eye(8)
    B = rng.standard_normal((8, 8))
    chi = -0.01 * (B @ B.T)
    W = wc_freq(chi, V, V)
    np.testing.assert_allclose(W, np.linalg.solve(np.eye(8) - V @ chi, V) - V, atol=1e-10)


def test_block_filters_are_identity_at_zero_and_empty_above_every_block():
    """LibRI's block filter restated (drop_small): threshold 0 keeps every block; a threshold above
    every block's max-norm drops them all, and the exchange built from no density matrix blocks is
    zero."""
    import numpy as np
    from conftest import load_he_exx, oracle_input
    from oracle.gw_oracle import drop_small, exx_kgrid
    blocks = {(0, 0, (0, 0, 0)): np.array([[1.0, -2.0]]), (0, 1, (0, 0, 0)): np.array([[0.5]])}
    assert drop_small(blocks, 0.0) is blocks
    assert list(drop_small(blocks, 1.0)) == [(0, 0, (0, 0, 0))]
    assert drop_small(blocks, 2.0) == {}
    s = load_he_exx()
    assert np.abs(exx_kgrid(oracle_input(s), s.v_cut, thr_d=1e9)).max() == 0.0
