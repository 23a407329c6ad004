"""The dielectric function of the G0W0 head correction mapped onto the minimax frequencies
(interpolate_dielec_func, src/core/dielecmodel.cpp:65-104): the library's host entry
librpa_gb300_interpolate_dielec_func against the oracle restatement, for the spline and the
Havriliak-Negami fit, inside and outside the data range.  Host work: runs without a GPU."""
import numpy as np
import pytest

import librpa_gb300 as L
from conftest import load_mgo
from oracle import dielec as O


def _model(u, p):
    return np.array([O.hn_value(x, p) for x in u])


# a two-pole eps(i omega) of an insulator (eps(0) ~ 3.4) on a log grid, and minimax-like targets
# from below the grid's first point to beyond its last
P_TRUE = [3.4, 0.9, 1.1, 2.0, 1.6, 1.0, 0.7, 0.3]
OMEGA_IN = np.geomspace(0.02, 40.0, 24)
EPS_IN = _model(OMEGA_IN, P_TRUE)
TARGETS = np.geomspace(0.005, 120.0, 16)


def test_spline_matches_the_oracle_in_and_out_of_range(lib):
    got = L.interpolate_dielec_func(1, OMEGA_IN, EPS_IN, TARGETS)
    want = O.interpolate_dielec_func(1, OMEGA_IN, EPS_IN, TARGETS)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=0)
    # inside the range it follows the smooth model closely
    inside = (TARGETS >= OMEGA_IN[0]) & (TARGETS <= OMEGA_IN[-1])
    np.testing.assert_allclose(got[inside], _model(TARGETS[inside], P_TRUE), rtol=2e-2)


def test_spline_passes_through_its_points(lib):
    """Every piece ends on the next data point, whatever its curvature coefficients, so at the
    data frequencies the spline returns the data (here: the same grid in and out, option 1 equal
    to option 0 up to rounding)."""
    got = L.interpolate_dielec_func(1, OMEGA_IN, EPS_IN, OMEGA_IN)
    np.testing.assert_allclose(got, EPS_IN, rtol=1e-13, atol=0)
    np.testing.assert_array_equal(L.interpolate_dielec_func(0, OMEGA_IN, EPS_IN, OMEGA_IN), EPS_IN)


def test_spline_of_few_points_and_the_reference_step_order(lib):
    """With 2 and 3 points the shared elimination / back-substitution loop of the reference
    (back substitution reading z = 0 ahead of the elimination) gives coefficients that differ from
    the textbook natural spline; both implementations follow the reference."""
    for n in (2, 3, 5):
        x = np.linspace(0.1, 2.0, n)
        y = 1.0 + 2.0 / (1.0 + x ** 2)
        t = np.array([0.0, 0.05, 0.3, 1.1, 1.999, 2.5, 4.0])
        np.testing.assert_allclose(L.interpolate_dielec_func(1, x, y, t), O.interpolate_dielec_func(1, x, y, t),
                                   rtol=1e-13, atol=0)


def test_havriliak_negami_fit_matches_the_oracle_and_recovers_the_model(lib):
    got = L.interpolate_dielec_func(2, OMEGA_IN, EPS_IN, TARGETS)
    want = O.interpolate_dielec_func(2, OMEGA_IN, EPS_IN, TARGETS)
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=0)
    # the reference stops after an accepted step that lowers the squared error by less than 1e-8,
    # well before the 8 parameters settle: the fitted curve follows the model to about 1%
    inside = (TARGETS >= OMEGA_IN[0]) & (TARGETS <= OMEGA_IN[-1])
    np.testing.assert_allclose(got[inside], _model(TARGETS[inside], P_TRUE), rtol=1e-2)


def test_mgo_dielectric_function_all_options(lib):
    """The MgO eps_mac of the reference's G0W0 case at its 6 minimax frequencies, mapped onto a
    16-point grid by the spline and by the model fit."""
    s = load_mgo()
    h = L.Handler()
    L.load_system(h, s)
    om, _ = h.get_imaginary_frequency_grids(L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax))
    tg = np.geomspace(om[0] * 0.5, om[-1] * 2.0, 16)
    for opt in (1, 2):
        np.testing.assert_allclose(L.interpolate_dielec_func(opt, om, s.epsmac, tg),
                                   O.interpolate_dielec_func(opt, om, s.epsmac, tg), rtol=1e-9, atol=0,
                                   err_msg=f"option {opt}")
    np.testing.assert_array_equal(L.interpolate_dielec_func(0, om, s.epsmac, om), s.epsmac)


def test_errors(lib):
    with pytest.raises(L.LibrpaError, match="minimax frequencies"):
        L.interpolate_dielec_func(0, OMEGA_IN, EPS_IN, TARGETS)
    with pytest.raises(L.LibrpaError, match="option_dielect_func"):
        L.interpolate_dielec_func(3, OMEGA_IN, EPS_IN, TARGETS)
    with pytest.raises(L.LibrpaError, match="at least 2 points"):
        L.interpolate_dielec_func(1, OMEGA_IN[:1], EPS_IN[:1], TARGETS)
