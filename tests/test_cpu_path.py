"""The host-core RPA path of the oracle (oracle/cpu_path.py with its OpenMP kernels), which
bench.py times as the reference CPU arm, against the oracle's restatement on small inputs."""
import numpy as np
import pytest

from conftest import load_h2o, load_li_g0w0, oracle_input
from librpa_gb300 import synthetic as sy
from oracle.cpu_path import CpuPath
from oracle.rpa_oracle import Options, rpa_correlation_energy


def _cases():
    return [
        ("fcc2_k222", sy.fcc2_k222()),
        ("uneven_k2", sy.small_periodic(n_atoms=2, nao=[3, 5], nabf=[7, 10], period=(2, 1, 1), nocc=2, seed=21)),
        ("three_atoms_gamma", sy.small_periodic(n_atoms=3, nao=[2, 4, 3], nabf=[4, 6, 5], period=(1, 1, 1),
                                                nocc=3, seed=21)),
        ("odd_nao_k6", sy.small_periodic(n_atoms=2, nao=[5, 4], nabf=[12, 9], period=(3, 2, 1), nocc=3, seed=21)),
        ("mixed_species", sy.cluster_gamma("m", 4, [(5, 20), (13, 60), (26, 110)], 77)),
    ]


@pytest.mark.parametrize("name,s", _cases(), ids=[c[0] for c in _cases()])
def test_cpu_path_matches_oracle(name, s):
    inp = sy.to_oracle_input(s)
    o = Options(nfreq=s.nfreq, minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)
    ref = rpa_correlation_energy(inp, o)
    cp = CpuPath(inp, o)
    ec, per_q = cp.run()
    assert abs(ec - ref["ec"]) <= 1e-10 * abs(ref["ec"])
    np.testing.assert_allclose(per_q, ref["per_q"], rtol=1e-9, atol=1e-14)
    # the OpenMP kernels against the same algebra in numpy calls
    cn = CpuPath(inp, o, kernel="numpy")
    ecn, _ = cn.run()
    assert np.abs(cp.chi0q_tau - cn.chi0q_tau).max() <= 1e-12 * np.abs(cn.chi0q_tau).max()
    assert abs(ec - ecn) <= 1e-10 * abs(ecn)


def test_cpu_path_real_inputs():
    """The reference's H2O regression E_c and the spin-polarised Li atom through the CPU path."""
    s = load_h2o()
    o = Options(nfreq=16)
    ec, _ = CpuPath(oracle_input(s), o).run()
    assert abs(ec.real - s.ec_reference) < 5e-9
    li = load_li_g0w0()
    ol = Options(nfreq=li.nfreq)
    ref = rpa_correlation_energy(oracle_input(li), ol)
    ec, _ = CpuPath(oracle_input(li), ol).run()
    assert abs(ec - ref["ec"]) <= 1e-10 * abs(ref["ec"])
