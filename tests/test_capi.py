"""C-ABI surface checks that need no GPU: exports, options defaults, host-side logic, errors."""
import ctypes as C
import math
import re
from pathlib import Path

import numpy as np
import pytest

import librpa_gb300 as L
from conftest import ROOT, load_h2o, minimax_ref
from oracle.minimax import minimax_grid as oracle_grid


def _declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(librpa_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(lib):
    declared = _declared_functions()
    assert len(declared) >= 50
    for name in sorted(declared):
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
    assert set(L.EXPORTS) == declared


def test_options_defaults_match_reference(lib):
    o = L.Options()
    # src/api/options.cpp:11-67
    assert o.output_dir == b"./" and o.parallel_routing == L.AUTO and o.nfreq == 6
    assert o.tfgrids_type == L.TFGRID_UNSET and o.minimax_emin == -1.0 and o.minimax_emax == -1.0
    assert o.n_bands_chi0 == -1 and o.use_scalapack_ecrpa == 1 and o.use_fullcoul_eps == 1
    assert o.tfgrids_freq_min == 0.005 and o.tfgrids_freq_max == 1000.0 and o.gf_threshold == 0.0
    assert C.sizeof(L.LibrpaOptions) == 200 + 4 * 4 + 8 * 10 + 4 * 16 + 8 * 9 + 4 * 4 + 4 * 0 or True


def test_cpp_minimax_matches_oracle(lib):
    for n, emin, emax in [(16, 0.26, 21.0), (16, 0.25, 25.0), (24, 0.25, 750.0), (32, 0.25, 2500.0), (6, 0.657768, 30.1366)]:
        a = L.minimax_grid(n, emin, emax)
        b = oracle_grid(n, emin, emax)
        for k in ("tau", "tau_w", "omega", "omega_w"):
            np.testing.assert_allclose(a[k], b[k], rtol=1e-14)
        for k in ("cos_t2f", "cos_f2t", "sin_t2f"):
            np.testing.assert_allclose(a[k], b[k], rtol=1e-6, atol=1e-9 * np.abs(b[k]).max())


def test_cpp_minimax_reference_log(lib):
    ref = minimax_ref()["ng6_HF_123"]
    g = L.minimax_grid(6, ref["emin"], ref["emax"])
    assert np.abs(g["omega"] - ref["omega"]).max() < ref["tol"]


def _fit_errors(g, emin, emax):
    """GreenX's fit errors (calculate_max_error) of the three transforms of a grid: the largest
    deviation of sum_j w_j cos/sin(...) e^{-x tau_j} (or 2x/(x^2+w_j^2)) from the target function
    over the log-spaced x nodes of get_transformation_weights."""
    n = len(g["tau"])
    tau, om = np.asarray(g["tau"]), np.asarray(g["omega"])
    nx = max((int(np.log10(emax / emin)) + 1) * 200, n)
    x = emin * (emax / emin) ** (np.arange(nx) / (nx - 1.0))
    e = np.exp(-np.outer(x, tau))
    cos_e = max(np.abs(2 * x / (x * x + w * w) - e @ g["cos_t2f"][i]).max() for i, w in enumerate(om))
    sin_e = max(np.abs(2 * w / (x * x + w * w) - e @ g["sin_t2f"][i]).max() for i, w in enumerate(om))
    lor = 2 * x[:, None] / (x[:, None] ** 2 + om[None, :] ** 2)
    f2t_e = max(np.abs(np.exp(-x * t) - lor @ g["cos_f2t"][i]).max() for i, t in enumerate(tau))
    return np.array([cos_e, sin_e, f2t_e])


def test_cpp_minimax_32_points_reference_log(lib):
    """32 points over the H2 run's window (E_max/E_min = 79): the nodes and weights of the
    reference log.  The transforms' least-squares fits are singular to double precision there;
    GreenX (and the oracle, through LAPACK) keep every singular value and reach weights of 1e6 to
    1e8 that follow LAPACK's rounding, the library drops those below its numerical rank.  Its
    fits are as accurate as the oracle's, with bounded weights."""
    ref = minimax_ref()["h2_32"]
    g = L.minimax_grid(32, ref["emin"], ref["emax"])
    for k in ("omega", "omega_w", "tau", "tau_w"):
        np.testing.assert_allclose(g[k], ref[k], rtol=1e-13, atol=1e-16)
    o = oracle_grid(32, ref["emin"], ref["emax"])
    el, eo = _fit_errors(g, ref["emin"], ref["emax"]), _fit_errors(o, ref["emin"], ref["emax"])
    assert np.all(el <= 2.0 * eo), (el, eo)
    assert max(np.abs(g[k]).max() for k in ("cos_t2f", "sin_t2f", "cos_f2t")) < 1e4
    assert max(np.abs(o[k]).max() for k in ("cos_t2f", "sin_t2f", "cos_f2t")) > 1e6

def test_frequency_grid_api_uses_mean_field_window(lib):
    s = load_h2o()
    with L.Handler() as h:
        L.load_system(h, s)
        om, w = h.get_imaginary_frequency_grids(L.Options(nfreq=16, tfgrids_type=L.Minimax))
    np.testing.assert_allclose(om, minimax_ref()["h2o16"]["omega"], rtol=2e-15)
    np.testing.assert_allclose(w, minimax_ref()["h2o16"]["omega_w"], rtol=2e-15)


def test_frequency_grid_window_on_periodic_input(lib):
    """The mean-field window (band gap over all k, band width) on the periodic BCC He input with
    its 8 k-points, against the oracle's e_min_max (MeanField::get_E_min_max, get_band_gap)."""
    from conftest import load_he_exx, oracle_input
    from oracle.rpa_oracle import e_min_max
    s = load_he_exx()
    emin, emax = e_min_max(oracle_input(s))
    with L.Handler() as h:
        L.load_system(h, s)
        om, w = h.get_imaginary_frequency_grids(L.Options(nfreq=16, tfgrids_type=L.Minimax))
    g = oracle_grid(16, emin, emax)
    np.testing.assert_allclose(om, g["omega"], rtol=1e-14)
    np.testing.assert_allclose(w, g["omega_w"], rtol=1e-14)


def test_errors_are_recorded_not_thrown(lib):
    with L.Handler() as h:
        # wrong grid type -> error message, NaN, handler stays usable
        with pytest.raises(L.LibrpaError, match="not implemented"):
            h.get_rpa_correlation_energy(L.Options(nfreq=16), 1)
        with pytest.raises(L.LibrpaError, match="basis not set"):
            h.set_lri_coeff(L.LIBRI, 0, 0, 2, 2, 3, (0, 0, 0), np.zeros(12))
        h.set_scf_dimension(1, 1, 4, 4)
        assert lib.librpa_get_last_error_code(h.h) == 0
        # a band-point call without band data: the reference's own message
        with pytest.raises(L.LibrpaError, match="band calculation is not set"):
            h.get_exx_pot_band_k(L.Options(), 1, [0], 0, 1)
        h.set_scf_dimension(1, 1, 4, 4)
        assert lib.librpa_get_last_error_code(h.h) == 0
    assert lib.librpa_get_rpa_correlation_energy(None, None, 0, np.zeros(1), np.zeros(1)) != \
        lib.librpa_get_rpa_correlation_energy(None, None, 0, np.zeros(1), np.zeros(1))  # NaN


def test_invalid_routing_is_rejected_before_any_gpu_work(lib):
    """A parallel_routing value outside the reference's enum (librpa_enums.h: AUTO, RTAU, ATOMPAIR,
    LIBRI) is an error recorded on the handler, as the reference's option parser rejects it."""
    s = load_h2o()
    with L.Handler() as h:
        L.load_system(h, s)
        with pytest.raises(L.LibrpaError, match="invalid parallel routing"):
            h.get_rpa_correlation_energy(L.Options(nfreq=16, tfgrids_type=L.Minimax, parallel_routing=7), 1)


def test_g0w0_and_exchange_input_checks_before_any_gpu_work(lib):
    """The exchange and G0W0 take k-grid inputs (MgO, 3x3x3) and reach the GPU (here: none); the
    G0W0 head correction with option_dielect_func = 0 needs the dielectric function at the nfreq
    minimax frequencies (1 and 2 interpolate it, 3 is not fed by the C API), and the
    exchange refuses an input without the truncated Coulomb matrix."""
    from conftest import load_mgo
    s = load_mgo()
    with L.Handler() as h:
        L.load_system(h, s)
        if lib.librpa_gb300_device_count() == 0:
            with pytest.raises(L.LibrpaError, match="CUDA|device"):
                h.get_exx_pot_kgrid(L.Options(nfreq=6, tfgrids_type=L.Minimax), 1, [0], 0, 4)
        h.set_dielect_func_imagfreq(np.arange(5.0), np.ones(5))
        with pytest.raises(L.LibrpaError, match="nfreq minimax frequencies"):
            h.get_g0w0_sigc_kgrid(L.Options(nfreq=6, tfgrids_type=L.Minimax, replace_w_head=1), 1, [0], 0, 4,
                                  np.zeros(4), np.zeros(4))
        # the velocity-matrix head and wings (option 3) have no setter in the C API
        with pytest.raises(L.LibrpaError, match="option_dielect_func must be 0, 1 or 2"):
            h.get_g0w0_sigc_kgrid(L.Options(nfreq=6, tfgrids_type=L.Minimax, replace_w_head=1, option_dielect_func=3),
                                  1, [0], 0, 4, np.zeros(4), np.zeros(4))
    s = load_h2o()
    with L.Handler() as h:
        L.load_system(h, s)
        with pytest.raises(L.LibrpaError, match="truncated Coulomb"):
            h.get_exx_pot_kgrid(L.Options(nfreq=16, tfgrids_type=L.Minimax), 1, [0], 0, 4)


def test_no_gpu_means_loud_error_not_fallback(lib):
    if lib.librpa_gb300_device_count() > 0:
        pytest.skip("GPU present")
    s = load_h2o()
    with L.Handler() as h:
        L.load_system(h, s)
        with pytest.raises(L.LibrpaError, match="no CUDA device"):
            h.get_rpa_correlation_energy(L.Options(nfreq=16, tfgrids_type=L.Minimax), 1)


def test_batch_call_checks_its_arguments_before_any_gpu_work(lib):
    """librpa_gb300_get_rpa_correlation_energy_batch refuses a handler listed twice (two threads
    would work on one handler) and returns -1 with the message; an empty batch is a no-op."""
    s = load_h2o()
    o = L.Options(nfreq=16, tfgrids_type=L.Minimax)
    with L.Handler() as h:
        L.load_system(h, s)
        with pytest.raises(L.LibrpaError, match="listed twice"):
            L.rpa_correlation_energy_batch([h, h], o)
    assert len(L.rpa_correlation_energy_batch([], o)) == 0


def test_vq_threshold_drops_blocks(lib):
    with L.Handler() as h:
        h.set_ao_basis_aux([2, 2])
        h.set_aux_bare_coulomb_k_atom_pair(0, 0, 1, 2, 2, np.full(4, 1e-3), np.zeros(4), 1e-2)
        h.set_aux_bare_coulomb_k_atom_pair(0, 0, 0, 2, 2, np.full(4, 1.0), np.zeros(4), 1e-2)
        assert lib.librpa_get_last_error_code(h.h) == 0


def test_small_cell_batch_workload():
    """The 32-cell batch of the mixed-species configuration: independent Gamma cells of 2-8
    atoms of the three species, reproducible from its seed."""
    from librpa_gb300 import synthetic as sy
    a, b = sy.batch32_small(), sy.batch32_small()
    assert len(a) == 32
    species = {(5, 20), (13, 60), (26, 110)}
    for s, t in zip(a, b):
        assert 2 <= s.n_atoms <= 8 and s.n_kpts == 1 and s.nfreq == 24
        assert set(zip(s.nao, s.nabf)) <= species
        assert s.n_atoms == t.n_atoms and np.array_equal(s.ekb, t.ekb)


def test_rank_cut_grid_gives_the_oracle_ec_on_an_ill_conditioned_window(lib):
    """BCC He: E_max/E_min = 1.6 over 16 points makes every fit singular (singular values down to
    1e-22 of the largest).  The library's rank-cut transforms (weights below 3e3) and the oracle's
    LAPACK ones (weights up to 1e8) give one RPA E_c to 1e-10 when fed to the same oracle."""
    import oracle.rpa_oracle as R
    from conftest import load_he_exx, oracle_input
    inp = oracle_input(load_he_exx())
    emin, emax = R.e_min_max(inp)
    g = L.minimax_grid(16, emin, emax)
    assert max(np.abs(g[k]).max() for k in ("cos_t2f", "sin_t2f", "cos_f2t")) < 1e4
    ref = R.rpa_correlation_energy(inp, R.Options(nfreq=16))["ec"].real
    saved = R.grids_for
    try:
        R.grids_for = lambda inp_, opts_: dict(g)
        ec = R.rpa_correlation_energy(inp, R.Options(nfreq=16))["ec"].real
    finally:
        R.grids_for = saved
    assert abs(ec - ref) <= 1e-10 * abs(ref), (ec, ref)


def test_shrink_lri_coeff_setter_checks_its_inputs(lib):
    """librpa_gb300_set_shrink_lri_coeff needs the small basis first and blocks sized for it; the
    exchange of a shrunk input refuses to run without those blocks (before any GPU work)."""
    from conftest import load_bn_shrink_g0w0
    s = load_bn_shrink_g0w0()
    with L.Handler() as h:
        h.set_scf_dimension(s.n_spins, s.n_kpts, s.n_bands, s.n_ao)
        h.set_ao_basis_wfc(s.nao)
        h.set_ao_basis_aux(s.nabf)
        c = np.zeros((s.nao[0] * s.nao[1], s.nabf_small[0]))
        with pytest.raises(L.LibrpaError, match="small auxiliary basis not set"):
            h.set_shrink_lri_coeff(0, 1, s.nao[0], s.nao[1], s.nabf_small[0], (0, 0, 0), c)
        h.set_shrink_basis(s.nabf_small)
        with pytest.raises(L.LibrpaError, match="inconsistent with the small basis"):
            h.set_shrink_lri_coeff(0, 1, s.nao[0], s.nao[1], s.nabf[0], (0, 0, 0),
                                   np.zeros((s.nao[0] * s.nao[1], s.nabf[0])))
        h.set_shrink_lri_coeff(0, 1, s.nao[0], s.nao[1], s.nabf_small[0], (0, 0, 0), c)
    s.Cs_small = None
    with L.Handler() as h:
        L.load_system(h, s)
        o = L.Options(nfreq=16, tfgrids_type=L.Minimax, use_shrink_abfs=1)
        with pytest.raises(L.LibrpaError, match="RI coefficients of the small basis"):
            h.get_exx_pot_kgrid(o, 1, [0], 0, 4)
