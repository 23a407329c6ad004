"""Tau-shard stages through the C ABI on one GPU: the partial chi0(q, omega) of two tau slices,
summed on the host and loaded back, give the unsharded E_c (needs a GB300)."""
import numpy as np
import pytest

import librpa_gb300 as L
from librpa_gb300 import synthetic as sy
from librpa_gb300.tau_shard import tau_slices

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built(lib):
    if lib.librpa_gb300_device_count() == 0:
        pytest.fail("no CUDA device visible for a gpu-marked test")


@pytest.mark.parametrize("prec,ec_path", [(L.CHI0_FP64, L.EC_LU_FP64), (L.CHI0_BF16X3, L.EC_CHOL)])
@pytest.mark.parametrize("world", [2, 3])
def test_sequential_shards_match_full(prec, ec_path, world):
    s = sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[6, 8], period=(2, 1, 1), nocc=2, seed=9)
    h = L.Handler()
    L.load_system(h, s)
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)
    h.set_gb300_options(L.gb300_options(chi0_precision=prec, ec_path=ec_path))
    full, full_q = h.get_rpa_correlation_energy(o, L.n_ibz(s))
    total = None
    for b, e in tau_slices(s.nfreq, world):
        h.set_gb300_options(L.gb300_options(chi0_precision=prec, ec_path=ec_path, tau_begin=b, tau_end=e,
                                            stage=L.STAGE_CHI0))
        ec_part, _ = h.get_rpa_correlation_energy(o, L.n_ibz(s))
        assert ec_part == 0.0
        part = h.chi0_qw()
        total = part if total is None else total + part
    h.load_chi0_qw(total)
    h.set_gb300_options(L.gb300_options(chi0_precision=prec, ec_path=ec_path, stage=L.STAGE_EC))
    ec, perq = h.get_rpa_correlation_energy(o, L.n_ibz(s))
    assert abs(ec - full) <= 1e-12 * abs(full), (ec, full)
    np.testing.assert_allclose(perq, full_q, rtol=1e-11, atol=1e-14)
