"""The library's host quasi-particle solver (librpa_gb300_solve_qpe: Thiele-Pade continuation +
damped fixed point) against the oracle's restatement and the reference's H2O and Li tables,
fed with the oracle's Sigma_c(i omega) (no GPU needed)."""
import numpy as np
import pytest

import librpa_gb300 as L
from conftest import load_h2o_g0w0, load_li_g0w0, oracle_input
from oracle.gw_oracle import HA2EV, Pade, g0w0_gamma, qpe_solve
from oracle.rpa_oracle import Options


@pytest.mark.parametrize("case", ["h2o", "li"])
def test_qpe_matches_oracle_and_reference(lib, case):
    s = load_h2o_g0w0() if case == "h2o" else load_li_g0w0()
    inp = oracle_input(s)
    r = g0w0_gamma(inp, s.v_cut, s.vxc, Options(nfreq=s.nfreq), n_params=s.n_params_anacon)
    om = r["grid"]["omega"]
    for sp in range(inp.n_spins):
        e_qp, sig, bad = L.solve_qpe(om, r["sigc_iw"][sp], inp.ekb[sp, 0], inp.efermi, s.vxc[sp, 0],
                                     r["vexx"][sp], n_params=s.n_params_anacon)
        assert bad == 0
        np.testing.assert_allclose(e_qp, r["e_qp"][sp], rtol=0, atol=1e-12)
        np.testing.assert_allclose(sig, r["sigc"][sp], rtol=0, atol=1e-12)
        table = s.qp_table if case == "h2o" else s.qp_tables[sp]
        np.testing.assert_allclose(e_qp * HA2EV, table[:, 7], rtol=0, atol=6e-6)
        np.testing.assert_allclose(sig.real * HA2EV, table[:, 5], rtol=0, atol=6e-6)


def test_pade_subsampling_and_breakdown(lib):
    """Fewer parameters than points (strided selection, last point kept) agrees with the oracle
    where the continued fraction is well conditioned (a three-pole function, 4 or 5 parameters;
    with more parameters than the function has degrees of freedom the reciprocal differences
    approach 0/0 and both restatements are rounding-bound).  Constant data make the fraction
    break down: the state comes back as NaN, as the reference prints it."""
    om = np.linspace(0.05, 12.0, 16)
    poles = np.array([-0.6 + 0.1j, 0.3 + 0.2j, 0.9 + 0.05j])
    sig = np.array([[sum(0.1 / (1j * w - p) for p in poles) for w in om]])
    e_mf, vxc, vexx = np.array([-0.3]), np.array([-0.4]), np.array([-0.6])
    for npar in (4, 5):
        e_qp, sg, bad = L.solve_qpe(om, sig, e_mf, -0.1, vxc, vexx, n_params=npar)
        pade = Pade(npar, [1j * w for w in om], list(sig[0]))
        info, e_ref, s_ref = qpe_solve(pade, e_mf[0], -0.1, vxc[0], vexx[0])
        assert bad == 0 and abs(e_qp[0] - e_ref) < 1e-10 and abs(sg[0] - s_ref) < 1e-10, npar
    e_qp, sg, bad = L.solve_qpe(om, np.ones((1, 16), complex), e_mf, -0.1, vxc, vexx)
    assert np.isnan(e_qp[0]) and np.isnan(sg[0])
