"""Exchange and G0W0 (k-grids and the Gamma point) on the GPU through the C ABI
(librpa_get_exx_pot_kgrid, librpa_get_g0w0_sigc_kgrid), against the reference's own tables and
the CPU oracle (needs a GB300)."""
import numpy as np
import pytest

import librpa_gb300 as L
from conftest import load_bn_shrink_g0w0, load_h2o_g0w0, load_he_exx, load_li_g0w0, load_mgo, oracle_input
from oracle.dielec import interpolate_dielec_func
from oracle.gw_oracle import HA2EV, BandPoints, exx_kgrid, g0w0_gamma, g0w0_kgrid
from oracle.rpa_oracle import Options as OOpts

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib):
    if lib.librpa_gb300_device_count() == 0:
        pytest.fail("no CUDA device visible for a gpu-marked test")


def _opts(s):
    return L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                     n_params_anacon=s.n_params_anacon)


def _run(s, prec, keep=None, sigma=L.SIGMA_FP64):
    """v_exx and Sigma_c(e_qp) of every state, per spin, through the library; e_qp from them.
    keep (a list) receives the handler."""
    h = L.Handler()
    if keep is not None:
        keep.append(h)
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=prec, ec_path=L.EC_LU_FP64, sigma_precision=sigma))
    o = _opts(s)
    nb = s.n_bands
    vexx = h.get_exx_pot_kgrid(o, s.n_spins, [0], 0, nb)
    vxc = s.vxc.reshape(s.n_spins, 1, nb)
    sig = h.get_g0w0_sigc_kgrid(o, s.n_spins, [0], 0, nb, vxc, vexx)
    e_qp = s.ekb[:, :1, :] - vxc + vexx + sig.real
    return vexx[:, 0], sig[:, 0], e_qp[:, 0]


@pytest.fixture(scope="module")
def h2o():
    s = load_h2o_g0w0()
    return s, g0w0_gamma(oracle_input(s), s.v_cut, s.vxc, OOpts(nfreq=s.nfreq), n_params=s.n_params_anacon)


def test_h2o_table_fp64(h2o):
    """H2O (24 states, 16 minimax points, 16 Pade parameters), FP64 chi0: v_exx, Re/Im Sigma_c and
    e_qp of every state against the reference's table (refs/g0w0_aims_mole_H2O_libri, printed
    to 5 decimals in eV) and against the oracle."""
    s, r = h2o
    vexx, sig, e_qp = _run(s, L.CHI0_FP64)
    t = s.qp_table
    np.testing.assert_allclose(vexx[0] * HA2EV, t[:, 4], rtol=0, atol=6e-6)
    np.testing.assert_allclose(sig[0].real * HA2EV, t[:, 5], rtol=0, atol=6e-6)
    np.testing.assert_allclose(sig[0].imag * HA2EV, t[:, 6], rtol=0, atol=6e-6)
    np.testing.assert_allclose(e_qp[0] * HA2EV, t[:, 7], rtol=0, atol=3e-5)
    np.testing.assert_allclose(vexx[0], r["vexx"][0], rtol=0, atol=1e-10)
    np.testing.assert_allclose(sig[0], r["sigc"][0], rtol=0, atol=1e-7)
    # the GPU's imaginary-axis self-energy itself
    h = []
    _run(s, L.CHI0_FP64, h)
    np.testing.assert_allclose(h[0].g0w0_sigc_iw(0, 0, s.n_bands, s.nfreq), r["sigc_iw"][0], rtol=0, atol=1e-10)


@pytest.mark.parametrize("sigma", [L.SIGMA_FP64, L.SIGMA_BF16X3])
def test_h2o_tensor_core_chi0_within_1mev(h2o, sigma):
    """The default 3-piece BF16 tensor-core chi0 feeding the same chain, with the self-energy's
    contraction in FP64 and as 3-piece BF16 split GEMMs: the KS-diagonal
    Sigma_c(i omega) of every state and frequency within 1 meV of the FP64 oracle (the G0W0 bar).
    The analytic continuation to the real axis with 16 Pade parameters is ill-conditioned for the
    high virtual states (measured: up to 0.15 eV at the quasi-particle energy for the highest
    states from the tensor-core chi0), so at the quasi-particle energy the bar is applied to the
    states around the gap: the top three occupied and the first three empty ones."""
    s, r = h2o
    hs = []
    _, sig, _ = _run(s, L.CHI0_BF16X3, hs, sigma)
    iw = hs[0].g0w0_sigc_iw(0, 0, s.n_bands, s.nfreq)
    assert np.abs(iw - r["sigc_iw"][0]).max() * HA2EV < 1e-3, np.abs(iw - r["sigc_iw"][0]).max() * HA2EV
    homo = int(np.sum(s.wg[0, 0] > 0)) - 1
    frontier = slice(homo - 2, homo + 4)
    assert np.abs(sig[0][frontier] - r["sigc"][0][frontier]).max() * HA2EV < 1e-3


def test_gamma_point_head_correction_from_a_spline(h2o):
    """A Gamma-only input with replace_w_head and a dielectric function given on its own 20-point
    grid (option_dielect_func = 1): the reference replaces the head at q = 0 for any input once a
    dielectric function is set, so the chain runs with eps_mac spline-mapped onto the 16 minimax
    frequencies.  FP64 chi0 against the oracle's k-grid chain (one q-point) fed the oracle's
    spline of the same data; the head moves Sigma_c well beyond that tolerance."""
    s, r0 = h2o
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64))
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  n_params_anacon=s.n_params_anacon, replace_w_head=1, option_dielect_func=1)
    om, _ = h.get_imaginary_frequency_grids(o)
    grid = np.geomspace(om[0] * 0.7, om[-1] * 1.3, 20)
    eps = 1.0 + 1.5 / (1.0 + (grid / 0.4) ** 2)
    h.set_dielect_func_imagfreq(grid, eps)
    nb = s.n_bands
    vexx = h.get_exx_pot_kgrid(o, s.n_spins, [0], 0, nb)
    vxc = s.vxc.reshape(s.n_spins, 1, nb)
    sig = h.get_g0w0_sigc_kgrid(o, s.n_spins, [0], 0, nb, vxc, vexx)
    iw = h.g0w0_sigc_iw(0, 0, nb, s.nfreq)
    epsmac = interpolate_dielec_func(1, grid, eps, om)
    r = g0w0_kgrid(oracle_input(s), s.v_cut, s.vxc, OOpts(nfreq=s.nfreq), n_params=s.n_params_anacon,
                   epsmac=epsmac)
    np.testing.assert_allclose(iw, np.asarray(r["sigc_iw"][0]).reshape(iw.shape), rtol=0, atol=1e-10)
    np.testing.assert_allclose(sig[0, 0], np.asarray(r["sigc"][0]).ravel(), rtol=0, atol=1e-7)
    assert np.abs(iw - r0["sigc_iw"][0]).max() > 1e-4


def test_li_spin_polarised_table():
    """Spin-polarised Li atom (refs/g0w0_aims_Li_atom_libri): both spin channels, every column."""
    s = load_li_g0w0()
    vexx, sig, e_qp = _run(s, L.CHI0_FP64)
    for sp in range(2):
        t = s.qp_tables[sp]
        got = np.c_[vexx[sp] * HA2EV, sig[sp].real * HA2EV, sig[sp].imag * HA2EV]
        np.testing.assert_allclose(got, t[:, 4:7], rtol=0, atol=6e-6, err_msg=f"spin {sp}")
        np.testing.assert_allclose(e_qp[sp] * HA2EV, t[:, 7], rtol=0, atol=3e-5)


def _vexx_kgrid(s):
    h = L.Handler()
    L.load_system(h, s)
    return h.get_exx_pot_kgrid(L.Options(nfreq=16, tfgrids_type=L.Minimax), s.n_spins, list(range(s.n_kpts)), 0,
                               s.n_bands)


def test_periodic_exchange_bcc_he_every_k_point():
    """BCC He (2-atom cell, 2x2x2 k-points, C blocks given on cells [0, 2) that LibRI folds): v_exx
    of all 8 bands at all 8 k-points against the reference's table
    (refs/exx_aims_bccHe_k_parallel_libri, 5 decimals in Hartree) and the oracle (1e-10)."""
    s = load_he_exx()
    got = _vexx_kgrid(s)
    np.testing.assert_allclose(got[0], s.exx_tables[:, :, 1], rtol=0, atol=6e-6)
    np.testing.assert_allclose(got, exx_kgrid(oracle_input(s), s.v_cut), rtol=0, atol=1e-10)


def test_periodic_exchange_mgo_ibz_reduced():
    """MgO (3x3x3 k-points, 14 irreducible by time reversal, the truncated Coulomb given at those
    only): v_exx of all 17 states at all 27 k-points against the reference's G0W0 table
    (refs/g0w0_aims_MgO_libri, 5 decimals in eV)."""
    s = load_mgo()
    got = _vexx_kgrid(s)
    np.testing.assert_allclose(got[0] * HA2EV, s.qp_tables[:, :, 4], rtol=0, atol=6e-6)


def _mgo_run(s, prec, sigma=L.SIGMA_FP64):
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=prec, ec_path=L.EC_LU_FP64, sigma_precision=sigma))
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  n_params_anacon=s.n_params_anacon, replace_w_head=1, option_dielect_func=0)
    om, _ = h.get_imaginary_frequency_grids(o)
    h.set_dielect_func_imagfreq(om, s.epsmac)
    nb, nk = s.n_bands, s.n_kpts
    ks = list(range(nk))
    vexx = h.get_exx_pot_kgrid(o, s.n_spins, ks, 0, nb)
    vxc = s.vxc.reshape(s.n_spins, nk, nb)
    sig = h.get_g0w0_sigc_kgrid(o, s.n_spins, ks, 0, nb, vxc, vexx)
    return h, o, vexx, vxc, sig


@pytest.fixture(scope="module")
def mgo_fp64():
    s = load_mgo()
    return (s,) + _mgo_run(s, L.CHI0_FP64)


def test_mgo_kgrid_g0w0_tables(mgo_fp64):
    """Periodic G0W0 (MgO, 3x3x3 k-points from 14 IBZ points, head of the dielectric matrix
    replaced by the given eps_mac, 6 minimax points, all 6 in the Pade fit), FP64 chi0 and FP64
    self-energy products: v_exx, Re/Im Sigma_c and e_qp of all 17 states at all 27 k-points
    against the reference's tables (refs/g0w0_aims_MgO_libri, 5 decimals in eV)."""
    s, h, o, vexx, vxc, sig = mgo_fp64
    nb = s.n_bands
    e_qp = s.ekb - vxc + vexx + sig.real
    got = np.stack([vexx[0] * HA2EV, sig[0].real * HA2EV, sig[0].imag * HA2EV, e_qp[0] * HA2EV], axis=-1)
    np.testing.assert_allclose(got, s.qp_tables[:, :, 4:8], rtol=0, atol=6e-6)
    # band k-points placed on three SCF points reproduce those points' results (task = g0w0_band)
    kb = [0, 5, 13]
    h.set_band_points(h_kfrac(s)[kb], s.wg[:, kb], s.ekb[:, kb], s.wfc[:, kb])
    # (the k fractions of the input carry about 1e-11 of rounding, which the images shifted by a
    # period turn into phase differences of about 1e-10: far below the tables' print precision)
    vb = h.get_exx_pot_band_k(o, s.n_spins, [0, 1, 2], 0, nb)
    np.testing.assert_allclose(vb, vexx[:, kb], rtol=0, atol=1e-9)
    sb = h.get_g0w0_sigc_band_k(o, s.n_spins, [0, 1, 2], 0, nb, vxc[:, kb], vb)
    np.testing.assert_allclose(sb, sig[:, kb], rtol=0, atol=1e-8)


def test_mgo_tensor_core_self_energy_within_1mev(mgo_fp64):
    """Tensor-core chi0 and the self-energies' closed form as 3-piece BF16 split GEMMs
    (sigma_precision = BF16X3: FP32 accumulation, the long contraction cut into ABF chunks summed
    in FP64) on MgO.
    Sigma_c(i omega) of every state at k-point 0 within 1 meV of the all-FP64 run, and Sigma_c at
    the quasi-particle energy of the states around the gap at every k-point within 1 meV."""
    s, h64, _, vexx64, _, sig64 = mgo_fp64
    h, _, vexx, _, sig = _mgo_run(s, L.CHI0_BF16X3, L.SIGMA_BF16X3)
    nb = s.n_bands
    # the exchange stays FP64 whatever sigma_precision says
    np.testing.assert_allclose(vexx, vexx64, rtol=0, atol=1e-10)
    d_iw = np.abs(h.g0w0_sigc_iw(0, 0, nb, s.nfreq) - h64.g0w0_sigc_iw(0, 0, nb, s.nfreq)).max() * HA2EV
    assert d_iw < 1e-3, d_iw
    homo = int(np.sum(s.wg[0, 0] > 0)) - 1
    frontier = slice(homo - 2, homo + 4)
    d_qp = np.abs(sig[0][:, frontier] - sig64[0][:, frontier]).max() * HA2EV
    assert d_qp < 1e-3, d_qp


def h_kfrac(s):
    """Fractional coordinates of the SCF k-points (k_cart / 2 pi times the lattice vectors)."""
    return (np.asarray(s.kvecs) / (2 * np.pi)) @ np.asarray(s.latvec).T


def test_periodic_exchange_at_band_points_off_the_grid():
    """v_exx at k-points off the SCF grid (task = exx_band) for BCC He: the R blocks moved to the
    image nearest to each atom pair (exx.cpp:683-725) and summed at k, against the oracle's
    restatement; arbitrary orthonormal band vectors, so every matrix element counts."""
    s = load_he_exx()
    rng = np.random.default_rng(3)
    kf = np.array([[0.1, 0.2, 0.3], [0.5, 0.25, 0.0], [0.37, 0.0, 0.61]])
    nkb, nb, nao = len(kf), s.n_bands, s.n_ao
    wfc = np.zeros((s.n_spins, nkb, nb, nao), complex)
    for k in range(nkb):
        q, _ = np.linalg.qr(rng.standard_normal((nao, nao)) + 1j * rng.standard_normal((nao, nao)))
        wfc[0, k] = q[:nb]
    ekb = np.sort(rng.uniform(-1, 1, (s.n_spins, nkb, nb)), axis=-1)
    h = L.Handler()
    L.load_system(h, s)
    h.set_band_points(kf, np.zeros_like(ekb), ekb, wfc)
    got = h.get_exx_pot_band_k(L.Options(nfreq=16, tfgrids_type=L.Minimax), s.n_spins, list(range(nkb)), 0, nb)
    ref = exx_kgrid(oracle_input(s), s.v_cut, BandPoints(kf, wfc, ekb, s.efermi))
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10)


@pytest.fixture(scope="module")
def bn_shrink():
    s = load_bn_shrink_g0w0()
    r = g0w0_kgrid(oracle_input(s), s.v_cut, s.vxc, OOpts(nfreq=s.nfreq), n_params=s.n_params_anacon,
                   sqrt_threshold=s.sqrt_coulomb_threshold)
    return s, r


def _bn_run(s, prec):
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=prec, ec_path=L.EC_LU_FP64))
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  n_params_anacon=s.n_params_anacon, use_shrink_abfs=1,
                  sqrt_coulomb_threshold=s.sqrt_coulomb_threshold)
    nb, nk = s.n_bands, s.n_kpts
    ks = list(range(nk))
    vexx = h.get_exx_pot_kgrid(o, s.n_spins, ks, 0, nb)
    vxc = s.vxc.reshape(s.n_spins, nk, nb)
    sig = h.get_g0w0_sigc_kgrid(o, s.n_spins, ks, 0, nb, vxc, vexx)
    return h, vexx, vxc, sig


def test_bn_shrink_g0w0_tables(bn_shrink):
    """G0W0 with the ABF shrink (the reference's ABACUS BN case, 2x2x2 k-points, 60 + 59 ABFs
    shrunk to 17 + 17), FP64 chi0: chi0 shrunk by U chi0 U^H and W_c unfolded by U^H W_c U on the
    GPU, the exchange on the RI coefficients of the small basis.  Against the oracle (v_exx 1e-10,
    Sigma_c(i omega) 1e-9, Sigma_c(e_qp) 1e-7 Ha) and the reference's 8 tables: v_exx at print
    precision, Sigma_c to 2e-4 eV and e_qp to 4e-4 eV (the bounds of the oracle's own agreement:
    an ill-conditioned 16-point cosine fit and the solver's 1e-5 Ha stopping threshold)."""
    s, r = bn_shrink
    h, vexx, vxc, sig = _bn_run(s, L.CHI0_FP64)
    np.testing.assert_allclose(vexx[0], r["vexx"][0], rtol=0, atol=1e-10)
    for ik in range(s.n_kpts):  # librpa_gb300_get_g0w0_sigc_iw_k at every SCF k-point
        np.testing.assert_allclose(h.g0w0_sigc_iw(0, 0, s.n_bands, s.nfreq, ik), r["sigc_iw"][0][ik], rtol=0, atol=1e-9)
    with pytest.raises(L.LibrpaError, match="k-point index out of range"):
        h.g0w0_sigc_iw(0, 0, s.n_bands, s.nfreq, s.n_kpts)
    # band k-points on three SCF points (task = g0w0_band with the shrink) reproduce their results
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  n_params_anacon=s.n_params_anacon, use_shrink_abfs=1,
                  sqrt_coulomb_threshold=s.sqrt_coulomb_threshold)
    kb = [0, 3, 7]
    h.set_band_points(h_kfrac(s)[kb], s.wg[:, kb], s.ekb[:, kb], s.wfc[:, kb])
    vb = h.get_exx_pot_band_k(o, s.n_spins, [0, 1, 2], 0, s.n_bands)
    np.testing.assert_allclose(vb, vexx[:, kb], rtol=0, atol=1e-9)
    sb = h.get_g0w0_sigc_band_k(o, s.n_spins, [0, 1, 2], 0, s.n_bands, vxc[:, kb], vb)
    np.testing.assert_allclose(sb, sig[:, kb], rtol=0, atol=1e-8)
    np.testing.assert_allclose(sig[0], r["sigc"][0], rtol=0, atol=1e-7)
    t = s.qp_tables
    e_qp = s.ekb - vxc + vexx + sig.real
    np.testing.assert_allclose(vexx[0] * HA2EV, t[:, :, 4], rtol=0, atol=6e-6)
    np.testing.assert_allclose(sig[0].real * HA2EV, t[:, :, 5], rtol=0, atol=2e-4)
    np.testing.assert_allclose(sig[0].imag * HA2EV, t[:, :, 6], rtol=0, atol=2e-4)
    np.testing.assert_allclose(e_qp[0] * HA2EV, t[:, :, 7], rtol=0, atol=4e-4)


def test_bn_shrink_g0w0_tensor_core_chi0_within_1mev(bn_shrink):
    """The default tensor-core chi0 through the same shrunk chain: Sigma_c(i omega) of every
    state at k-point 0 within 1 meV of the FP64 oracle."""
    s, r = bn_shrink
    h, _, _, _ = _bn_run(s, L.CHI0_BF16X3)
    iw = h.g0w0_sigc_iw(0, 0, s.n_bands, s.nfreq)
    assert np.abs(iw - r["sigc_iw"][0][0]).max() * HA2EV < 1e-3


def _threshold_between(blocks):
    """A threshold halfway (geometrically) between two distinct middle block max-norms: about half
    of the blocks fall under it and none is near it (blocks related by symmetry share a max-norm)."""
    m = np.sort([np.abs(v).max() for v in blocks.values() if np.abs(v).max() > 0])
    u = [m[0]]
    for x in m[1:]:
        if x > u[-1] * (1 + 1e-6):
            u.append(x)
    i = max(1, len(u) // 2)
    return float(np.sqrt(u[i - 1] * u[i]))


def test_exchange_block_filters_match_the_oracle():
    """libri_exx_threshold_V / _D drop the V(R) and D(R) blocks LibRI's set_Vs / set_Ds filters drop
    (exx.cpp:365-418): BCC He with thresholds that remove about half of each, against the oracle
    with the same filters (1e-10 Ha), and visibly different from the unfiltered exchange."""
    from oracle.gw_oracle import coulomb_r, dmat_r
    from oracle.rpa_oracle import r_grid
    s = load_he_exx()
    inp = oracle_input(s)
    rl = r_grid(inp.period)
    tv = _threshold_between(coulomb_r(inp, s.v_cut, rl))
    td = _threshold_between(dmat_r(inp, 0, rl))
    h = L.Handler()
    L.load_system(h, s)
    o = L.Options(nfreq=16, tfgrids_type=L.Minimax, libri_exx_threshold_V=tv, libri_exx_threshold_D=td)
    got = h.get_exx_pot_kgrid(o, s.n_spins, list(range(s.n_kpts)), 0, s.n_bands)
    ref = exx_kgrid(inp, s.v_cut, thr_v=tv, thr_d=td)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-10)
    assert np.abs(ref - exx_kgrid(inp, s.v_cut)).max() > 1e-4


def test_self_energy_block_filters_match_the_oracle(h2o, bn_shrink):
    """libri_g0w0_threshold_G / _Wc drop the G(R, +-tau) and W(R, tau) blocks LibRI's set_Gs /
    set_Ws filters drop (gw.cpp:459-616), on the Gamma-point chain (H2O) and the k-grid chain (BN
    with the shrink): FP64, against the oracle with the same filters (Sigma_c(i omega) to 1e-9),
    and different from the unfiltered result."""
    s, r0 = h2o
    thr = dict(libri_g0w0_threshold_G=2e-3, libri_g0w0_threshold_Wc=2e-3)
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64))
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  n_params_anacon=s.n_params_anacon, **thr)
    h.get_g0w0_sigc_kgrid(o, s.n_spins, [0], 0, s.n_bands, s.vxc.reshape(s.n_spins, 1, -1),
                          h.get_exx_pot_kgrid(o, s.n_spins, [0], 0, s.n_bands))
    r = g0w0_gamma(oracle_input(s), s.v_cut, s.vxc, OOpts(nfreq=s.nfreq), n_params=s.n_params_anacon,
                   thr_w=2e-3, thr_g=2e-3)
    iw = h.g0w0_sigc_iw(0, 0, s.n_bands, s.nfreq)
    np.testing.assert_allclose(iw, r["sigc_iw"][0], rtol=0, atol=1e-9)
    assert np.abs(iw - r0["sigc_iw"][0]).max() > 1e-6

    b, _ = bn_shrink
    h = L.Handler()
    L.load_system(h, b)
    h.set_gb300_options(L.gb300_options(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64))
    o = L.Options(nfreq=b.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  n_params_anacon=b.n_params_anacon, use_shrink_abfs=1,
                  sqrt_coulomb_threshold=b.sqrt_coulomb_threshold, **thr)
    ks = list(range(b.n_kpts))
    h.get_g0w0_sigc_kgrid(o, b.n_spins, ks, 0, b.n_bands, b.vxc.reshape(b.n_spins, b.n_kpts, -1),
                          h.get_exx_pot_kgrid(o, b.n_spins, ks, 0, b.n_bands))
    rb = g0w0_kgrid(oracle_input(b), b.v_cut, b.vxc, OOpts(nfreq=b.nfreq), n_params=b.n_params_anacon,
                    sqrt_threshold=b.sqrt_coulomb_threshold, thr_w=2e-3, thr_g=2e-3)
    np.testing.assert_allclose(h.g0w0_sigc_iw(0, 0, b.n_bands, b.nfreq), rb["sigc_iw"][0][0], rtol=0, atol=1e-9)


def test_precision_change_rebuilds_the_self_energy(h2o):
    """The kept self-energy belongs to the precisions it was built with: switching
    sigma_precision on the handler rebuilds it (and gives what a fresh handler gives)."""
    s, _ = h2o
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64))
    o = _opts(s)
    nb = s.n_bands
    vexx = h.get_exx_pot_kgrid(o, s.n_spins, [0], 0, nb)
    vxc = s.vxc.reshape(s.n_spins, 1, nb)
    h.get_g0w0_sigc_kgrid(o, s.n_spins, [0], 0, nb, vxc, vexx)
    iw64 = h.g0w0_sigc_iw(0, 0, nb, s.nfreq)
    h.set_gb300_options(L.gb300_options(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64,
                                        sigma_precision=L.SIGMA_BF16X3))
    h.get_g0w0_sigc_kgrid(o, s.n_spins, [0], 0, nb, vxc, vexx)
    iw_split = h.g0w0_sigc_iw(0, 0, nb, s.nfreq)
    assert 0 < np.abs(iw_split - iw64).max() * HA2EV < 1e-3
    h2 = L.Handler()
    L.load_system(h2, s)
    h2.set_gb300_options(L.gb300_options(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64,
                                         sigma_precision=L.SIGMA_BF16X3))
    h2.get_g0w0_sigc_kgrid(o, s.n_spins, [0], 0, nb, vxc, h2.get_exx_pot_kgrid(o, s.n_spins, [0], 0, nb))
    np.testing.assert_allclose(h2.g0w0_sigc_iw(0, 0, nb, s.nfreq), iw_split, rtol=0, atol=1e-12)
