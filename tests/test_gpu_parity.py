"""GPU path vs the oracle through the C ABI (needs a GB300)."""
import copy

import numpy as np
import pytest

import librpa_gb300 as L
from conftest import load_h2o, load_he_exx, load_li_g0w0, load_mgo, oracle_input
from librpa_gb300 import synthetic as sy
from oracle.rpa_oracle import Options as OOpts, rpa_correlation_energy

pytestmark = pytest.mark.gpu

MEV_PER_ATOM = 3.674932e-6  # 0.1 meV in Hartree


def _opts(s):
    return L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                     minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)


def run_gpu(s, prec, keep=False, ec_path=L.EC_LU_FP64):
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=prec, keep_chi0=int(keep), ec_path=ec_path))
    ec, perq = h.get_rpa_correlation_energy(_opts(s), L.n_ibz(s))
    return h, ec, perq


def run_oracle(s):
    return rpa_correlation_energy(oracle_input(s), OOpts(nfreq=s.nfreq, minimax_emin=s.minimax_emin,
                                                         minimax_emax=s.minimax_emax))


@pytest.fixture(scope="module", autouse=True)
def _built(lib):
    if lib.librpa_gb300_device_count() == 0:
        pytest.fail("no CUDA device visible for a gpu-marked test")


def test_h2o_regression_fp64():
    """H2O regression dataset: GPU FP64 path vs the reference's printed E_c and the oracle."""
    s = load_h2o()
    h, ec, perq = run_gpu(s, L.CHI0_FP64)
    o = run_oracle(s)
    assert abs(ec - s.ec_reference) < 5e-9
    assert abs(ec - o["ec"].real) < 1e-11
    assert abs(perq[0] - o["per_q"][0]) < 1e-11
    st = h.stats()
    assert st["n_launches"] > 0 and st["chi0_flops"] > 0


@pytest.mark.parametrize("period,nao,nabf,nocc", [((2, 1, 1), [3, 5], [7, 10], 2), ((3, 1, 1), [4, 2], [6, 9], 2),
                                                  ((2, 2, 1), [3, 3], [5, 5], 1), ((1, 1, 1), [2, 4, 3], [4, 6, 5], 3),
                                                  ((3, 2, 1), [5, 4], [12, 9], 3)])
def test_small_periodic_fp64_vs_oracle(period, nao, nabf, nocc):
    s = sy.small_periodic(n_atoms=len(nao), nao=nao, nabf=nabf, period=period, nocc=nocc, seed=21)
    h, ec, perq = run_gpu(s, L.CHI0_FP64, keep=True)
    o = run_oracle(s)
    assert abs(ec - o["ec"].real) <= 1e-10 * abs(o["ec"].real)
    np.testing.assert_allclose(perq, o["per_q"], rtol=1e-9, atol=1e-12)
    # chi0(q, w) blocks
    for iw in (0, s.nfreq // 2, s.nfreq - 1):
        for iq in range(L.n_ibz(s)):
            for (I, J), ref in o["chi0q"][iw][iq].items():
                got = h.get_chi0_block(iw, iq, I, J, s.nabf[I], s.nabf[J])
                np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("split", [False, True])
def test_cell_vectors_outside_the_centred_range(split):
    """C blocks given on cells [0, n) (as FHI-aims writes them), or split over two images a
    period apart, are folded into the centred BvK range and summed as LibRI does: the same
    E_c as the centred input, on the FP64 and the tensor-core paths."""
    s = sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[6, 8], period=(3, 2, 1), nocc=2, seed=5)
    t = sy.with_cells_relabelled(s, split=split)
    for prec in (L.CHI0_FP64, L.CHI0_BF16X3):
        _, a, pa = run_gpu(s, prec)
        _, b, pb = run_gpu(t, prec)
        assert abs(a - b) <= 1e-12 * abs(a), (prec, a, b)
        np.testing.assert_allclose(pb, pa, rtol=1e-11, atol=1e-15)


def test_he_bcc_fhi_aims_periodic_vs_oracle():
    """Real periodic FHI-aims input (BCC He, 2x2x2 k-points, C cells written in [0, 2)): FP64 path
    vs the oracle, and the default tensor-core path within 0.1 meV/atom."""
    s = load_he_exx()
    o = run_oracle(s)
    _, ec, perq = run_gpu(s, L.CHI0_FP64)
    assert abs(ec - o["ec"].real) <= 1e-10 * abs(o["ec"].real)
    np.testing.assert_allclose(perq, o["per_q"], rtol=1e-9, atol=1e-12)
    # default path: every V(q) of He is positive definite, so no q needs the LU form
    h2, ec2, perq2 = run_gpu(s, L.CHI0_BF16X3, ec_path=L.EC_CHOL)
    assert h2.stats()["ec_lu_fallback_q"] == 0
    assert abs(ec2 - o["ec"].real) <= MEV_PER_ATOM * len(s.nao)
    np.testing.assert_allclose(perq2, o["per_q"], rtol=0, atol=MEV_PER_ATOM * len(s.nao))
    # the all-FP64 Cholesky form keeps FP64 accuracy
    h3, ec3, _ = run_gpu(s, L.CHI0_FP64, ec_path=L.EC_CHOL_FP64)
    assert h3.stats()["ec_lu_fallback_q"] == 0
    assert abs(ec3 - o["ec"].real) <= 1e-9 * abs(o["ec"].real)


def test_coulomb_given_as_2d_blocks():
    """V(q) handed over as 2D blocks of the full matrix (librpa_set_aux_bare_coulomb_k_2d_block,
    the BLACS-distributed form of the FHI-aims interface) gives the E_c of the atom-pair form."""
    s = sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[6, 8], period=(3, 1, 1), nocc=2, seed=5)
    _, ref, pref = run_gpu(s, L.CHI0_FP64)
    nb = s.nabf
    off = np.concatenate([[0], np.cumsum(nb)]).astype(int)
    N = int(off[-1])
    h = L.Handler()
    t = copy.copy(s)
    t.Vq = {}
    L.load_system(h, t)
    for ik in sorted({k[0] for k in s.Vq}):
        M = np.zeros((N, N), complex)
        for (kk, I, J), v in s.Vq.items():
            if kk != ik:
                continue
            M[off[I]:off[I + 1], off[J]:off[J + 1]] = v
            M[off[J]:off[J + 1], off[I]:off[I + 1]] = v.conj().T
        # two row blocks, as two BLACS processes would hand them over
        for r0, r1 in ((0, N // 2), (N // 2, N)):
            blk = np.ascontiguousarray(M[r0:r1, :])
            h.set_aux_bare_coulomb_k_2d_block(ik, r0, r1, 0, N, np.ascontiguousarray(blk.real),
                                              np.ascontiguousarray(blk.imag))
    h.set_gb300_options(L.gb300_options(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64))
    ec, perq = h.get_rpa_correlation_energy(_opts(s), L.n_ibz(s))
    assert abs(ec - ref) <= 1e-12 * abs(ref)
    np.testing.assert_allclose(perq, pref, rtol=1e-11, atol=1e-15)


def test_li_spin_polarised_vs_oracle():
    """Two spin channels (the Li atom of the reference's G0W0 suite): FP64 path vs the oracle."""
    s = load_li_g0w0()
    o = run_oracle(s)
    _, ec, perq = run_gpu(s, L.CHI0_FP64)
    assert abs(ec - o["ec"].real) <= 1e-10 * abs(o["ec"].real)


def test_mgo_ibz_reduced_vs_oracle():
    """MgO (FHI-aims, 3x3x3 k-points of which 14 are irreducible, V(q) given at those only): the
    IBZ path of the library (chi0 and E_c at the irreducible q, weights count/n_k) against the
    oracle, FP64 and tensor-core paths.  The synthetic inputs have no IBZ reduction."""
    s = load_mgo()
    s.nfreq = 6
    o = run_oracle(s)
    _, ec, perq = run_gpu(s, L.CHI0_FP64)
    assert len(perq) == 14
    assert abs(ec - o["ec"].real) <= 1e-10 * abs(o["ec"].real)
    np.testing.assert_allclose(perq, o["per_q"], rtol=1e-9, atol=1e-12)
    # default path: V(Gamma) of MgO is indefinite, so that q goes through the LU form
    h2, ec2, perq2 = run_gpu(s, L.CHI0_BF16X3, ec_path=L.EC_CHOL)
    assert h2.stats()["ec_lu_fallback_q"] == 1
    assert abs(ec2 - o["ec"].real) <= MEV_PER_ATOM * len(s.nao)
    np.testing.assert_allclose(perq2, o["per_q"], rtol=0, atol=MEV_PER_ATOM * len(s.nao))
    # the all-FP64 Cholesky form takes the same fallback and keeps FP64 accuracy
    h3, ec3, _ = run_gpu(s, L.CHI0_FP64, ec_path=L.EC_CHOL_FP64)
    assert h3.stats()["ec_lu_fallback_q"] == 1
    assert abs(ec3 - o["ec"].real) <= 1e-9 * abs(o["ec"].real)


def test_mgo_ibz_reduced_equals_full_bz():
    """The library's E_c of MgO over the 14 irreducible q-points equals its E_c with all 27
    k-points irreducible (V(-q) = V(q)^*)."""
    from test_oracle_pins import unfold_ibz
    s = load_mgo()
    _, a, _ = run_gpu(s, L.CHI0_FP64)
    _, b, pb = run_gpu(unfold_ibz(s), L.CHI0_FP64)
    assert len(pb) == 27
    assert abs(a - b) <= 1e-10 * abs(a)


def test_fcc2_k222_fp64_vs_oracle():
    s = sy.fcc2_k222()
    h, ec, perq = run_gpu(s, L.CHI0_FP64)
    o = run_oracle(s)
    assert abs(ec - o["ec"].real) <= 1e-10 * abs(o["ec"].real)
    np.testing.assert_allclose(perq, o["per_q"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("prec", [L.CHI0_FP32, L.CHI0_BF16X3])
def test_reduced_precision_within_tolerance(prec):
    """Reduced-precision chi0 paths stay within 0.1 meV/atom of the FP64 GPU path."""
    s = sy.fcc2_k222()
    _, e64, _ = run_gpu(s, L.CHI0_FP64)
    _, e, _ = run_gpu(s, prec)
    assert abs(e - e64) <= MEV_PER_ATOM * len(s.nao)


def test_h2o_cholesky_ec_path():
    """Gamma-only (real) E_c through V = L L^T, tensor-core L^T chi0 L and FP64 Cholesky."""
    s = load_h2o()
    _, e_lu, _ = run_gpu(s, L.CHI0_FP64, ec_path=L.EC_LU_FP64)
    _, e_ch, _ = run_gpu(s, L.CHI0_FP64, ec_path=L.EC_CHOL)
    # the tensor-core products carry ~1e-7 relative error; bar: a tenth of 0.1 meV/atom
    tol = 0.1 * MEV_PER_ATOM * len(s.nao)
    assert abs(e_ch - e_lu) < tol
    assert abs(e_ch - s.ec_reference) < tol


@pytest.mark.parametrize("period", [(2, 1, 1), (3, 2, 1)])
def test_complex_cholesky_ec_path(period):
    s = sy.small_periodic(n_atoms=2, nao=[4, 5], nabf=[9, 12], period=period, nocc=2, seed=5)
    _, e_lu, q_lu = run_gpu(s, L.CHI0_FP64, ec_path=L.EC_LU_FP64)
    _, e_ch, q_ch = run_gpu(s, L.CHI0_FP64, ec_path=L.EC_CHOL)
    tol = 0.1 * MEV_PER_ATOM * len(s.nao)
    assert abs(e_ch - e_lu) <= tol
    np.testing.assert_allclose(q_ch.real, q_lu.real, atol=tol / L.n_ibz(s))


def test_default_fast_path_fcc2():
    """Default options (3-piece BF16 tcgen05 chi0 + Cholesky E_c) within 0.1 meV/atom of FP64 + LU."""
    s = sy.fcc2_k222()
    _, e64, _ = run_gpu(s, L.CHI0_FP64, ec_path=L.EC_LU_FP64)
    _, e, _ = run_gpu(s, L.CHI0_BF16X3, ec_path=L.EC_CHOL)
    assert abs(e - e64) <= MEV_PER_ATOM * len(s.nao)


@pytest.mark.parametrize("case", ["h2o", "k2x1x1", "k3x2x1"])
def test_all_fp64_cholesky_ec_matches_lu(case):
    """The all-FP64 Cholesky form of E_c (the FP64 GPU baseline) equals the reference-form LU."""
    if case == "h2o":
        s = load_h2o()
    else:
        period = (2, 1, 1) if case == "k2x1x1" else (3, 2, 1)
        s = sy.small_periodic(n_atoms=2, nao=[4, 5], nabf=[9, 12], period=period, nocc=2, seed=5)
    _, e_lu, q_lu = run_gpu(s, L.CHI0_FP64, ec_path=L.EC_LU_FP64)
    _, e_ch, q_ch = run_gpu(s, L.CHI0_FP64, ec_path=L.EC_CHOL_FP64)
    assert abs(e_ch - e_lu) <= 1e-10 * abs(e_lu), (e_ch, e_lu)
    np.testing.assert_allclose(q_ch.real, q_lu.real, rtol=1e-9, atol=1e-13)


@pytest.mark.parametrize("case", ["fcc2_k222", "h2o"])
def test_every_routing_gives_the_libri_ec(case):
    """parallel_routing = RTAU, ATOMPAIR and AUTO return the LibRI routing's E_c through the C ABI:
    this build runs one block schedule (the LibRI algebra) for every routing value.  On the 2-atom
    fcc cell the reference's AUTO would pick RTAU (3 atom pairs < 8 cells; decide_auto_routing,
    src/mpi/base_mpi.cpp:149-153); its RTAU and ATOMPAIR chi0 builders are not used as an oracle
    because the reference marks them broken, so the LibRI E_c (itself checked against the oracle
    above) is the target for all four."""
    s = sy.fcc2_k222() if case == "fcc2_k222" else load_h2o()
    out = {}
    for routing in (L.LIBRI, L.RTAU, L.ATOMPAIR, L.AUTO):
        h = L.Handler()
        L.load_system(h, s)
        h.set_gb300_options(L.gb300_options(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64))
        o = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=routing,
                      minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)
        out[routing], _ = h.get_rpa_correlation_energy(o, L.n_ibz(s))
    for routing in (L.RTAU, L.ATOMPAIR, L.AUTO):
        assert out[routing] == out[L.LIBRI]


def test_batch_call_equals_single_calls():
    """librpa_gb300_get_rpa_correlation_energy_batch: several independent small cells of mixed
    species evaluated concurrently give each cell's own E_c, as its single call does."""
    cells = sy.batch32_small()[:8]
    single, hs, opts = [], [], []
    for s in cells:
        h, ec, _ = run_gpu(s, L.CHI0_BF16X3, ec_path=L.EC_CHOL)
        single.append(ec)
        hs.append(h)
        opts.append(L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                              minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax))
    got = L.rpa_correlation_energy_batch(hs, opts, n_threads=4)
    # the K parts of the contraction add into chi0 atomically, in varying order
    np.testing.assert_allclose(got, single, rtol=1e-9, atol=0)


def test_atoms_beyond_the_tensor_core_tiles():
    """An atom with more than 32 NAOs and 128 ABFs (36 and 140 here) is outside the tensor-core
    contraction's tiles: the default options run the FP32 path instead (reported in the stats)
    and stay within 0.1 meV/atom of the oracle; the FP64 path matches it to 1e-10."""
    s = sy.small_periodic(n_atoms=2, nao=[36, 6], nabf=[140, 20], period=(2, 1, 1), nocc=3, seed=11, nfreq=8)
    o = run_oracle(s)
    h, ec, _ = run_gpu(s, L.CHI0_BF16X3, ec_path=L.EC_CHOL)
    assert h.stats()["chi0_precision_used"] == L.CHI0_FP32
    assert abs(ec - o["ec"].real) <= MEV_PER_ATOM * len(s.nao), (ec, o["ec"])
    h64, ec64, _ = run_gpu(s, L.CHI0_FP64)
    assert h64.stats()["chi0_precision_used"] == L.CHI0_FP64
    assert abs(ec64 - o["ec"].real) <= 1e-10 * abs(o["ec"].real)
