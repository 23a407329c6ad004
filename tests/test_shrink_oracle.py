"""The ABF shrink of chi0 (use_shrink_abfs; shrink_abfs_chi0, src/core/chi0.cpp:711-898) in the
oracle, and the BN shrink fixture read like the reference's driver reads it.  The reference prints
no E_c for a shrunk dataset, so the E_c restatement is held by exact properties: the identity and
any unitary U with V taken along leave E_c unchanged.  Its G0W0 run on the same data prints
quasi-particle tables, which pin the shrink in G0W0 (W_c unfolded as U^H W_c U, the exchange on
the RI coefficients of the small basis)."""
import numpy as np
import pytest

from conftest import load_bn_shrink, load_bn_shrink_g0w0, oracle_input, shrunk_copy
from librpa_gb300 import synthetic as sy
from oracle.rpa_oracle import Options, rpa_correlation_energy


def _ec(s, shrink):
    return rpa_correlation_energy(oracle_input(s), Options(nfreq=s.nfreq, minimax_emin=s.minimax_emin,
                                                           minimax_emax=s.minimax_emax, use_shrink_abfs=shrink))


def test_bn_shrink_fixture():
    """Cs in the 60 + 59 ABF basis, Coulomb and U(q) in the 17 + 17 one, every IBZ point present
    (read_ri_shrink / handle_sinvS_file, driver/read_data.cpp:2455-2622)."""
    s = load_bn_shrink()
    assert s.nabf == [60, 59] and s.nabf_small == [17, 17] and s.n_kpts == 8
    assert sorted(s.sinvS) == list(range(8))
    for U in s.sinvS.values():
        assert U.shape == (34, 119) and np.linalg.matrix_rank(U) == 34
    assert all(v.shape == (17, 17) for v in s.Vq.values())
    for iq in range(8):
        V = np.block([[s.Vq[(iq, 0, 0)], s.Vq[(iq, 0, 1)]], [s.Vq[(iq, 0, 1)].conj().T, s.Vq[(iq, 1, 1)]]])
        assert np.linalg.eigvalsh(V).min() > 0.3


@pytest.mark.parametrize("period", [(1, 1, 1), (2, 1, 1)])
def test_identity_and_unitary_shrink_leave_ec_unchanged(period):
    """U = I gives the unshrunk E_c; so does any unitary U(q) with V(q) -> U V U^H, since
    U chi0 U^H U V U^H = U chi0 V U^H keeps trace and determinant."""
    s = sy.small_periodic(n_atoms=2, nao=[4, 5], nabf=[9, 7], period=period, nfreq=8)
    ref = _ec(s, False)["ec"]
    ident = shrunk_copy(s, s.nabf, unitary=True)
    n = sum(s.nabf)
    ident.sinvS = {q: np.eye(n) for q in ident.sinvS}
    ident.Vq = s.Vq
    assert abs(_ec(ident, True)["ec"] - ref) <= 1e-13 * abs(ref)
    u = shrunk_copy(s, s.nabf, unitary=True)
    assert abs(_ec(u, True)["ec"] - ref) <= 1e-11 * abs(ref)


def test_projection_changes_ec_and_bn_value():
    """A real projection to fewer ABFs changes E_c (the shrink is applied at all), and the BN
    case's shrunk E_c stays what this restatement gives (-0.32482 Ha: 8 IBZ points, the 3 classes
    of equivalent q equal to 1e-12)."""
    s = sy.small_periodic(n_atoms=2, nao=[4, 5], nabf=[9, 7], period=(2, 1, 1), nfreq=8)
    ref = _ec(s, False)["ec"]
    p = shrunk_copy(s, [6, 5])
    assert abs(_ec(p, True)["ec"] - ref) > 1e-6 * abs(ref)
    r = _ec(load_bn_shrink(), True)
    assert abs(r["ec"].real - (-0.3248215193081771)) < 1e-9
    pq = np.array(r["per_q"]).real
    assert abs(pq[1] - pq[2]) < 1e-12 and abs(pq[3] - pq[5]) < 1e-12


def test_bn_shrink_g0w0_against_the_reference_tables():
    """G0W0 of the BN shrink case on its 2x2x2 k-grid (refs/g0w0_band_abacus_BN_shrink_libri):
    chi0 of the 60 + 59 ABF basis shrunk to 17 + 17, W_c there with the given Coulomb matrices,
    unfolded as U^H W_c U for Sigma_c on the large basis; the exchange from Cs_shrinked_data and
    the truncated Coulomb matrix of the small basis (driver/task_gw_band.cpp:92-250,
    src/gw_old.cpp:55-280).  v_exx matches all 208 states at print precision.  Sigma_c matches to
    2e-4 eV: this 16-point grid's cosine f->t fit is ill-conditioned (the run prints a duality
    error of 0.34; relative noise of 1e-8 in those weights moves Sigma_c by 3e-5 eV here), so the
    last digits follow the LAPACK build.  e_qp matches to 4e-4 eV, the quasi-particle solver's
    stopping threshold (1e-5 Ha): the reference's own e_qp differs from
    e_mf - v_xc + v_exx + Re Sigma_c by up to 2.8e-4 eV."""
    from oracle.gw_oracle import HA2EV, g0w0_kgrid
    s = load_bn_shrink_g0w0()
    t = s.qp_tables
    # the table's own inconsistency bounds what e_qp can be held to
    assert np.abs(t[:, :, 2] - t[:, :, 3] + t[:, :, 4] + t[:, :, 5] - t[:, :, 7]).max() < 3e-4
    r = g0w0_kgrid(oracle_input(s), s.v_cut, s.vxc, Options(nfreq=s.nfreq), n_params=s.n_params_anacon,
                   sqrt_threshold=s.sqrt_coulomb_threshold)
    np.testing.assert_allclose(s.vxc[0] * HA2EV, t[:, :, 3], rtol=0, atol=6e-6)
    np.testing.assert_allclose(r["vexx"][0] * HA2EV, t[:, :, 4], rtol=0, atol=6e-6)
    np.testing.assert_allclose(r["sigc"][0].real * HA2EV, t[:, :, 5], rtol=0, atol=2e-4)
    np.testing.assert_allclose(r["sigc"][0].imag * HA2EV, t[:, :, 6], rtol=0, atol=2e-4)
    np.testing.assert_allclose(r["e_qp"][0] * HA2EV, t[:, :, 7], rtol=0, atol=4e-4)
