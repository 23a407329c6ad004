"""Tau- and q-shard stages through the C ABI on one GPU, one emulated rank after the other: the
partial chi0(q, omega) of the tau slices, summed on the host and loaded back, give the
unsharded E_c, and the E_c stages restricted to disjoint q slices add up to it (needs a GB300)."""
import numpy as np
import pytest

import librpa_gb300 as L
from librpa_gb300 import synthetic as sy
from librpa_gb300.tau_shard import q_slices, tau_slices

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
    # FP64 path: every slot is transformed in FP64, so the shards add up to rounding.  Tensor-core
    # path: each call's slots are transformed together with an FP32 phase sum over R, so a
    # different grouping of the tau slots changes E_c at the FP32 level (measured 4e-9 relative),
    # far below the 0.1 meV/atom bar
    rtol = 1e-12 if prec == L.CHI0_FP64 else 1e-7
    assert abs(ec - full) <= rtol * abs(full), (ec, full)
    np.testing.assert_allclose(perq, full_q, rtol=10 * rtol, atol=1e-14 if prec == L.CHI0_FP64 else 1e-12)


@pytest.mark.parametrize("world", [2, 3])
def test_q_sliced_ec_stages_add_up(world):
    s = sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[6, 8], period=(3, 1, 1), nocc=2, seed=9)
    h = L.Handler()
    L.load_system(h, s)
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)
    nq = L.n_ibz(s)
    h.set_gb300_options(L.gb300_options(keep_chi0=0))
    full, full_q = h.get_rpa_correlation_energy(o, nq)
    h.set_gb300_options(L.gb300_options(stage=L.STAGE_CHI0))
    h.get_rpa_correlation_energy(o, nq)
    chi0 = h.chi0_qw()
    per_q = np.zeros(nq, complex)
    for qa, qe in q_slices(nq, world):
        # the rank's share after the reduce-scatter: its own q columns, the others zero
        mine = chi0.reshape(s.nfreq, nq, -1).copy()
        mine[:, :qa, :] = 0
        mine[:, qe:, :] = 0
        h.load_chi0_qw(mine.reshape(-1))
        h.set_gb300_options(L.gb300_options(stage=L.STAGE_EC, q_begin=qa, q_end=qe))
        ec, pq = h.get_rpa_correlation_energy(o, nq)
        assert np.all(pq[:qa] == 0) and np.all(pq[qe:] == 0)
        assert abs(ec - pq.sum().real) <= 1e-13 * max(1.0, abs(ec))
        per_q += pq
    np.testing.assert_allclose(per_q, full_q, rtol=1e-11, atol=1e-14)
    assert abs(per_q.sum().real - full) <= 1e-12 * abs(full)



def test_tensor_copies_of_chi0_qw():
    """The device-resident exchange's copies: chi0(q, omega) copied device to device into a torch
    tensor equals the host copy bit for bit, and loading a tensor back (here the sum of two tau
    slices' partials, added on the GPU) gives the unsharded E_c, as the host-array path does."""
    import torch
    s = sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[6, 8], period=(2, 1, 1), nocc=2, seed=9)
    h = L.Handler()
    L.load_system(h, s)
    o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                  minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)
    prec = dict(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64)
    h.set_gb300_options(L.gb300_options(**prec))
    full, _ = h.get_rpa_correlation_energy(o, L.n_ibz(s))
    dev = torch.device("cuda", 0)
    total = None
    for b, e in tau_slices(s.nfreq, 2):
        h.set_gb300_options(L.gb300_options(**prec, tau_begin=b, tau_end=e, stage=L.STAGE_CHI0))
        h.get_rpa_correlation_energy(o, L.n_ibz(s))
        t = h.chi0_qw_tensor(dev)
        assert t.is_cuda and np.array_equal(t.cpu().numpy().view(np.complex128), h.chi0_qw())
        total = t if total is None else total + t
    h.load_chi0_qw_tensor(total)
    h.set_gb300_options(L.gb300_options(**prec, stage=L.STAGE_EC))
    ec, _ = h.get_rpa_correlation_energy(o, L.n_ibz(s))
    assert abs(ec - full) <= 1e-12 * abs(full), (ec, full)
