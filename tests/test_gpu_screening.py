"""Block screening on the GPU through the C ABI: the plain threshold rule against the oracle,
the MLP kernels' gradients against the CPU restatement, and what the learned screening saves
over the plain rule at the same result (needs a GB300)."""
import ctypes as C

import numpy as np
import pytest

import librpa_gb300 as L
from conftest import oracle_input
from librpa_gb300 import synthetic as sy
from oracle import mlp
from oracle.rpa_oracle import Options as OOpts, rpa_correlation_energy

pytestmark = pytest.mark.gpu

MEV_PER_ATOM = 3.674932e-6
THR = 1e-4  # splits the blocks of the test cluster: the large-tau blocks fall below it


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.fixture(scope="module")
def cluster():
    return sy.cluster_gamma("scr8", 8, [(13, 40)], 808, decay_ang=1.5)


@pytest.fixture(scope="module", autouse=True)
def _built(lib):
    if lib.librpa_gb300_device_count() == 0:
        pytest.fail("no CUDA device visible for a gpu-marked test")


def _opts(s):
    return L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                     minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)


def _handler(s, **kw):
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(**kw))
    return h


def test_mlp_gradients_match_cpu_oracle(lib):
    rng = np.random.default_rng(11)
    n = 300
    params = rng.normal(0.0, 0.25, mlp.NPARAM).astype(np.float32)
    norm = np.concatenate([[5.0, 0.0, -2.0, -3.0, -3.0, 3.2, 2.2, 0.5, 0.5], [3.0, 1.0, 1.0, 2.0, 2.0, 0.4, 0.3, 0.5, 0.5],
                           [-5.0, 2.0, 0.5]]).astype(np.float32)
    assert norm.size == mlp.NNORM
    x = (rng.normal(0.0, 1.0, (n, mlp.IN)) * norm[mlp.IN:2 * mlp.IN] + norm[:mlp.IN]).astype(np.float32)
    y = rng.normal(-5.0, 2.0, n).astype(np.float32)
    grad = np.zeros(mlp.NPARAM, np.float32)
    loss = C.c_double()
    rc = lib.librpa_gb300_mlp_loss_grad(_ptr(params), _ptr(norm), _ptr(x), _ptr(y), n, _ptr(grad), C.byref(loss))
    assert rc == 0, lib.librpa_get_last_error(None).decode()
    ref_loss, ref_grad = mlp.loss_grad(params, norm, x, y)
    # FP32 kernels vs the FP64 restatement on the same FP16 weights
    assert abs(loss.value - ref_loss) <= 1e-5 * abs(ref_loss)
    scale = np.abs(ref_grad).max()
    assert np.abs(grad - ref_grad).max() <= 1e-4 * scale, np.abs(grad - ref_grad).max() / scale


def test_plain_screening_matches_oracle(cluster):
    s = cluster
    h = _handler(s, chi0_precision=0, ec_path=L.EC_LU_FP64, screen_mode=L.SCREEN_THRESHOLD, screen_threshold=THR)
    ec, _ = h.get_rpa_correlation_energy(_opts(s), 1)
    st = h.stats()
    ref = rpa_correlation_energy(oracle_input(s), OOpts(nfreq=s.nfreq, minimax_emin=s.minimax_emin,
                                                        minimax_emax=s.minimax_emax), block_threshold=THR)
    unscreened = rpa_correlation_energy(oracle_input(s), OOpts(nfreq=s.nfreq, minimax_emin=s.minimax_emin,
                                                               minimax_emax=s.minimax_emax))
    assert abs(ec - ref["ec"].real) < 1e-9, (ec, ref["ec"].real)
    assert abs(ref["ec"].real - unscreened["ec"].real) > 1e-9  # the rule drops blocks here
    assert st["blocks_computed"] == st["blocks_total"] == 36 * s.nfreq
    assert L.load_library().librpa_gb300_screening_samples(h.h) == 36 * s.nfreq


def test_learned_screening_skips_blocks_at_the_plain_result(cluster, lib):
    """Train on the plain run's logged blocks, then screen with the MLP: fewer blocks are
    contracted and E_c equals the plain threshold-screened E_c."""
    s = cluster
    h = _handler(s, chi0_precision=1, screen_mode=L.SCREEN_THRESHOLD, screen_threshold=THR)
    ec_plain, _ = h.get_rpa_correlation_energy(_opts(s), 1)
    plain = h.stats()
    rmse = C.c_double()
    assert lib.librpa_gb300_train_screening(h.h, 800, 3e-3, C.byref(rmse)) == 0, lib.librpa_get_last_error(None).decode()
    assert rmse.value < 0.5  # log10 units
    # the trained model against the CPU restatement on the logged samples
    n = lib.librpa_gb300_screening_samples(h.h)
    x = np.zeros((n, mlp.IN), np.float32)
    y = np.zeros(n, np.float32)
    assert lib.librpa_gb300_get_screening_samples(h.h, _ptr(x), _ptr(y), n) == 0
    params = np.zeros(mlp.NPARAM, np.float32)
    norm = np.zeros(mlp.NNORM, np.float32)
    assert lib.librpa_gb300_get_screening_model(h.h, _ptr(params), _ptr(norm)) == 0
    pred = mlp.forward(params, norm, x)
    assert np.sqrt(np.mean((pred - y) ** 2)) < 0.5
    h.set_gb300_options(L.gb300_options(chi0_precision=1, screen_mode=L.SCREEN_MLP, screen_threshold=THR,
                                        audit_fraction=0.05, seed=5))
    ec_mlp, _ = h.get_rpa_correlation_energy(_opts(s), 1)
    st = h.stats()
    assert st["blocks_total"] == plain["blocks_total"]
    assert st["blocks_computed"] < 0.9 * st["blocks_total"], (st["blocks_computed"], st["blocks_total"])
    assert st["screen_fallbacks"] == 0
    assert st["audit_max_dropped"] <= THR
    assert abs(ec_mlp - ec_plain) < 1e-10, (ec_mlp, ec_plain)


def test_learned_screening_transfers_across_mixed_species_cells(lib, capsys):
    """Mixed species (NAO/ABF 5/20, 13/60, 26/110, the shapes of the mixed-species workload): the
    MLP trains on block norms logged by the plain runs of three other small cells, pooled with
    librpa_gb300_add_screening_samples, and screens a 12-atom cell it has never seen.  Against
    the plain threshold rule on that cell it contracts fewer blocks at an E_c within 0.1 meV/atom;
    the species and block-dimension features tell the three species apart."""
    spec = [(5, 20), (13, 60), (26, 110)]
    xs, ys = [], []
    for n, seed in [(6, 911), (7, 912), (8, 913)]:
        s = sy.cluster_gamma(f"train{n}", n, spec, seed, decay_ang=1.5)
        h = _handler(s, chi0_precision=1, screen_mode=L.SCREEN_THRESHOLD, screen_threshold=THR)
        h.get_rpa_correlation_energy(_opts(s), 1)
        m = lib.librpa_gb300_screening_samples(h.h)
        x = np.zeros((m, mlp.IN), np.float32)
        y = np.zeros(m, np.float32)
        assert lib.librpa_gb300_get_screening_samples(h.h, _ptr(x), _ptr(y), m) == 0
        assert set(np.unique(x[:, 7])) <= {0.0, 1.0, 2.0}  # species feature
        xs.append(x)
        ys.append(y)
    x = np.concatenate(xs)
    y = np.concatenate(ys)
    t = sy.cluster_gamma("target12", 12, spec, 901, decay_ang=1.5)
    hp = _handler(t, chi0_precision=1, screen_mode=L.SCREEN_THRESHOLD, screen_threshold=THR)
    ec_plain, _ = hp.get_rpa_correlation_energy(_opts(t), 1)
    h = _handler(t, chi0_precision=1, screen_mode=L.SCREEN_MLP, screen_threshold=THR, audit_fraction=0.02, seed=3)
    assert lib.librpa_gb300_add_screening_samples(h.h, _ptr(x), _ptr(y), len(y)) == 0
    assert lib.librpa_gb300_screening_samples(h.h) == len(y)
    rmse = C.c_double()
    assert lib.librpa_gb300_train_screening(h.h, 1500, 3e-3, C.byref(rmse)) == 0, lib.librpa_get_last_error(None).decode()
    ec_mlp, _ = h.get_rpa_correlation_energy(_opts(t), 1)
    st = h.stats()
    skipped = 1.0 - st["blocks_computed"] / st["blocks_total"]
    with capsys.disabled():
        print(f"\nmixed-species transfer: train rmse {rmse.value:.3f} dec, skipped {skipped:.1%} of "
              f"{st['blocks_total']} blocks, audited {st['blocks_audited']}, fallbacks {st['screen_fallbacks']}, "
              f"dEc vs plain {abs(ec_mlp - ec_plain) / len(t.nao) * 27211.386:.2e} meV/atom")
    assert skipped >= 0.10
    assert abs(ec_mlp - ec_plain) <= MEV_PER_ATOM * len(t.nao)
