"""Options of the RPA path against the oracle (needs a GB300): spin-polarised input (the 2/n_s
factor and per-spin G), LibRI's input filters libri_chi0_threshold_C / _G (keep a block when its
max-norm exceeds the threshold), and the n_bands_chi0 band cut of the Green's function."""
import dataclasses

import numpy as np
import pytest

import librpa_gb300 as L
from conftest import oracle_input
from librpa_gb300 import synthetic as sy
from oracle.rpa_oracle import Options as OOpts, rpa_correlation_energy

pytestmark = pytest.mark.gpu

MEV_PER_ATOM = 3.674932e-6


@pytest.fixture(scope="module", autouse=True)
def _built(lib):
    if lib.librpa_gb300_device_count() == 0:
        pytest.fail("no CUDA device visible for a gpu-marked test")


def _base():
    return sy.small_periodic(n_atoms=2, nao=[4, 5], nabf=[9, 12], period=(2, 1, 1), nocc=3, seed=17)


def _spin_polarised(s):
    """Two spin channels: occupations 1 per spin, the second channel's virtual states shifted."""
    wg = np.concatenate([s.wg / 2, s.wg / 2])
    ekb = np.concatenate([s.ekb, s.ekb + np.where(s.wg > 0, 0.0, 0.05)])
    wfc = np.concatenate([s.wfc, s.wfc])
    return dataclasses.replace(s, name=s.name + "_spin2", n_spins=2, wg=wg, ekb=ekb, wfc=wfc)


def _gpu(s, prec, ec_path=L.EC_LU_FP64, **kw):
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=prec, ec_path=ec_path))
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax, **kw)
    ec, perq = h.get_rpa_correlation_energy(o, L.n_ibz(s))
    return ec, perq


def _oracle(s, **kw):
    return rpa_correlation_energy(oracle_input(s), OOpts(nfreq=s.nfreq, minimax_emin=s.minimax_emin,
                                                         minimax_emax=s.minimax_emax, **kw))


def _check(s, **kw):
    ref = _oracle(s, **kw)
    ec64, q64 = _gpu(s, L.CHI0_FP64, **kw)
    assert abs(ec64 - ref["ec"].real) <= 1e-10 * abs(ref["ec"].real), (ec64, ref["ec"].real)
    np.testing.assert_allclose(q64, ref["per_q"], rtol=1e-9, atol=1e-13)
    ecf, _ = _gpu(s, L.CHI0_BF16X3, ec_path=L.EC_CHOL, **kw)
    assert abs(ecf - ref["ec"].real) <= MEV_PER_ATOM * len(s.nao), (ecf, ref["ec"].real)
    return ref["ec"].real


def test_spin_polarised():
    s = _spin_polarised(_base())
    e2 = _check(s)
    e1 = _oracle(_base())["ec"].real
    assert abs(e2 - e1) > 1e-6  # the second channel differs


def test_libri_threshold_C_and_G():
    s = _base()
    cmax = sorted(np.abs(m).max() for m in s.Cs.values())
    thr_c = float(cmax[len(cmax) // 2])  # drops about half of the RI blocks
    full = _oracle(s)["ec"].real
    e_c = _check(s, libri_chi0_threshold_C=thr_c)
    assert abs(e_c - full) > 1e-8
    e_g = _check(s, libri_chi0_threshold_G=3e-2)
    assert abs(e_g - full) > 1e-8


def test_n_bands_chi0_cut():
    s = _base()
    full = _oracle(s)["ec"].real
    e = _check(s, n_bands_chi0=s.n_bands - 3)
    assert abs(e - full) > 1e-8
