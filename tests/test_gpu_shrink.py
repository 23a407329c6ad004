"""ABF shrink on the GPU (use_shrink_abfs: chi0 taken to the small ABF basis by U chi0 U^H,
src/core/chi0.cpp:711-898, E_c there) through the C ABI, against the oracle (needs a GB300)."""
import numpy as np
import pytest

import librpa_gb300 as L
from conftest import load_bn_shrink, oracle_input, shrunk_copy
from librpa_gb300 import synthetic as sy
from oracle.rpa_oracle import Options as OOpts, rpa_correlation_energy

pytestmark = pytest.mark.gpu

MEV_PER_ATOM = 3.674932e-6  # 0.1 meV in Hartree


@pytest.fixture(scope="module", autouse=True)
def _built(lib):
    if lib.librpa_gb300_device_count() == 0:
        pytest.fail("no CUDA device visible for a gpu-marked test")


def _gpu(s, prec, ec_path, shrink=True):
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=prec, ec_path=ec_path))
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI, minimax_emin=s.minimax_emin,
                  minimax_emax=s.minimax_emax, use_shrink_abfs=int(shrink))
    ec, perq = h.get_rpa_correlation_energy(o, L.n_ibz(s))
    return h, ec, perq


def _oracle(s, shrink=True):
    return rpa_correlation_energy(oracle_input(s), OOpts(nfreq=s.nfreq, minimax_emin=s.minimax_emin,
                                                         minimax_emax=s.minimax_emax, use_shrink_abfs=shrink))


def test_bn_shrink_vs_oracle():
    """The ABACUS BN case (2x2x2 k, 60 + 59 ABFs shrunk to 17 + 17 by its own sinvS): FP64 chi0
    with the LU form to 1e-10 of the oracle, and the default tensor-core chi0 with the Cholesky
    form within 0.1 meV/atom."""
    s = load_bn_shrink()
    o = _oracle(s)
    _, ec, perq = _gpu(s, L.CHI0_FP64, L.EC_LU_FP64)
    assert abs(ec - o["ec"].real) <= 1e-10 * abs(o["ec"].real), (ec, o["ec"])
    np.testing.assert_allclose(perq, o["per_q"], rtol=1e-9, atol=1e-13)
    h, ec2, perq2 = _gpu(s, L.CHI0_BF16X3, L.EC_CHOL)
    assert h.stats()["ec_lu_fallback_q"] == 0
    assert abs(ec2 - o["ec"].real) <= MEV_PER_ATOM * len(s.nao)
    np.testing.assert_allclose(perq2, o["per_q"], rtol=0, atol=MEV_PER_ATOM * len(s.nao))


@pytest.mark.parametrize("period", [(1, 1, 1), (2, 1, 1)])
def test_unitary_shrink_keeps_ec_and_projection_matches_oracle(period):
    """A unitary U(q) with V -> U V U^H leaves the GPU E_c at the unshrunk one; a projection to
    fewer ABFs gives the oracle's shrunk E_c (Gamma: real U, real E_c path; k grid: complex)."""
    s = sy.small_periodic(n_atoms=3, nao=[4, 5, 6], nabf=[9, 7, 11], period=period, nfreq=8)
    _, ref, _ = _gpu(s, L.CHI0_FP64, L.EC_LU_FP64, shrink=False)
    _, ecu, _ = _gpu(shrunk_copy(s, s.nabf, unitary=True), L.CHI0_FP64, L.EC_LU_FP64)
    assert abs(ecu - ref) <= 1e-10 * abs(ref)
    p = shrunk_copy(s, [6, 5, 8])
    o = _oracle(p)
    for ec_path in (L.EC_LU_FP64, L.EC_CHOL_FP64):
        _, ec, perq = _gpu(p, L.CHI0_FP64, ec_path)
        assert abs(ec - o["ec"].real) <= 1e-10 * abs(o["ec"].real), (ec_path, ec, o["ec"])
        np.testing.assert_allclose(perq, o["per_q"], rtol=1e-9, atol=1e-13)


def test_shrink_inputs_are_checked():
    """use_shrink_abfs without the small basis, without U(q), with a U of the wrong size, or with
    a complex U at the Gamma point is an error with a message, not a wrong number."""
    s = sy.small_periodic(n_atoms=2, nao=[4, 5], nabf=[9, 7], period=(1, 1, 1), nfreq=8)
    p = shrunk_copy(s, [6, 5])
    bare = sy.small_periodic(n_atoms=2, nao=[4, 5], nabf=[9, 7], period=(1, 1, 1), nfreq=8)
    bare.Vq, bare.nabf_small = p.Vq, p.nabf_small  # Coulomb in the small basis, no shrink inputs set
    with pytest.raises(L.LibrpaError, match="small ABF basis"):
        _gpu(bare, L.CHI0_FP64, L.EC_LU_FP64)
    h = L.Handler()
    L.load_system(h, bare)
    h.set_shrink_basis([6, 5])
    o = L.Options(nfreq=8, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI, use_shrink_abfs=1)
    with pytest.raises(L.LibrpaError, match="no shrink transform"):
        h.get_rpa_correlation_energy(o, 1)
    h.set_shrink_sinvS(0, np.ones((11, 15)))
    with pytest.raises(L.LibrpaError, match="must be"):
        h.get_rpa_correlation_energy(o, 1)
    h.set_shrink_sinvS(0, p.sinvS[0] * (1 + 1e-3j))
    with pytest.raises(L.LibrpaError, match="real at the Gamma point"):
        h.get_rpa_correlation_energy(o, 1)
