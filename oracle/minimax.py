"""Oracle (test infrastructure only): minimax time/frequency grids in numpy.

CPU restatement of LibRPA's minimax grid set-up, used only by tests/, the
smoke check and bench.py's CPU-baseline leg to check the product's C++ grid
generator.  It follows:

* ``TFGrids::generate_minimax``            src/core/timefreq.cpp:193-236
* ``gx_minimax_grid``                      thirdparty/greenX/GX-TimeFrequency/src/minimax_grids.F90:53-237
* ``get_transformation_weights``           minimax_grids.F90:299-406 (SVD least squares,
                                            Tikhonov term S/(reg^2+S^2))
* ``calculate_psi_and_mat_A``              minimax_grids.F90:423-516
* ``er_aw_aux%get_coeff_weight``           minimax_utils.F90 (energy-range bin, e_ratio rescale)
* the C-side transpose of the weight matrices in src/interface/gx_minimax_wrp.f90:170-176,
  so ``cos_t2f[i_omega, i_tau]`` is ``TFGrids::costrans_t2f(ifreq, it)``.

The tabulated coefficients are read from the product's data file
(librpa_gb300/data/greenx_minimax_tables.txt), which holds GreenX's numbers verbatim.
"""
from __future__ import annotations

import math
from functools import lru_cache
from pathlib import Path

import numpy as np

TABLES = Path(__file__).resolve().parent.parent / "librpa_gb300" / "data" / "greenx_minimax_tables.txt"


@lru_cache(maxsize=None)
def load_tables(path: str = str(TABLES)):
    tables = {"omega": {}, "tau": {}}
    cur = None
    for line in Path(path).read_text().splitlines():
        if not line or line.startswith("#"):
            continue
        tok = line.split()
        if tok[0] == "table":
            kind, n = tok[1], int(tok[2])
            cur = {"erange": None, "cols": {}}
            tables[kind][n] = cur
        elif tok[0] == "erange":
            cur["erange"] = np.array([float(x) for x in tok[1:]])
        elif tok[0] == "col":
            cur["cols"][int(tok[1])] = np.array([float(x) for x in tok[2:]])
    return tables


def _coeffs(kind: str, n: int, e_range: float) -> np.ndarray:
    """get_points_weights_{omega,tau} (minimax_omega.F90:2186-2223, minimax_tau.F90:2902-2939)."""
    tables = load_tables()
    if n not in tables[kind]:
        raise ValueError(f"unsupported minimax grids size: {n}")
    t = tables[kind][n]
    er = t["erange"]
    # find_erange: first range value strictly greater than e_range (else len+1)
    idx = len(er) + 1
    best = math.inf
    for j, v in enumerate(er, start=1):
        if e_range < v and v < best:
            idx, best = j, v
    e_ratio = 1.0
    if idx == 1 and n > 20:
        e_ratio = er[0] / e_range
        if e_ratio > 1.5:
            e_ratio = e_ratio / 1.5
    ac = t["cols"][idx].copy()
    if kind == "omega":
        return ac / e_ratio
    return ac * e_ratio


def _fit_weights(n, tau, omega, emin, emax, ttype, reg):
    """get_transformation_weights for one transform type; returns (n, n) weights[i_point, :]."""
    num_x = (int(math.log10(emax / emin)) + 1) * 200
    num_x = max(num_x, n)
    x_factor = (emax / emin) ** (1.0 / (num_x - 1.0))
    x = emin * x_factor ** np.arange(num_x)
    W = np.zeros((n, n))
    for ip in range(n):
        if ttype == 1:  # cos t->w
            om = omega[ip]
            psi = 2.0 * x / (x * x + om * om)
            A = np.cos(om * tau)[None, :] * np.exp(-np.outer(x, tau))
        elif ttype == 2:  # cos w->t
            t = tau[ip]
            psi = np.exp(-x * t)
            A = np.cos(t * omega)[None, :] * 2.0 * x[:, None] / (x[:, None] ** 2 + omega[None, :] ** 2)
        elif ttype == 3:  # sin t->w
            om = omega[ip]
            psi = 2.0 * om / (x * x + om * om)
            A = np.sin(om * tau)[None, :] * np.exp(-np.outer(x, tau))
        else:
            raise ValueError(ttype)
        U, S, VT = np.linalg.svd(A, full_matrices=False)
        s_inv = S / (reg * reg + S * S)
        W[ip] = VT.T @ (s_inv * (U.T @ psi))
    return W


def minimax_grid(n: int, emin: float, emax: float, regularization: float = 0.0):
    """Returns dict with tau, tau_w, omega, omega_w, cos_t2f[w,t], cos_f2t[t,w], sin_t2f[w,t]."""
    e_range = emax / emin
    ac = _coeffs("omega", n, e_range)
    omega = ac[:n] * emin
    omega_w = ac[n:] * emin
    ac = _coeffs("tau", n, e_range)
    tau = ac[:n] / (2.0 * emin)
    tau_w = ac[n:] / (2.0 * emin)
    cw = _fit_weights(n, tau, omega, emin, emax, 1, regularization)  # cosft_wt(j=omega, i=tau)
    ctw = _fit_weights(n, tau, omega, emin, emax, 2, regularization)  # cosft_tw(i=tau, j=omega)
    sw = _fit_weights(n, tau, omega, emin, emax, 3, regularization)
    ct = np.cos(np.outer(omega, tau))  # [j=omega, i=tau]
    cos_t2f = cw * ct
    cos_f2t = ctw * ct.T
    sin_t2f = sw * np.sin(np.outer(omega, tau))
    dual = np.abs(cos_t2f @ cos_f2t - np.eye(n)).max()
    return {
        "tau": tau, "tau_w": tau_w, "omega": omega, "omega_w": omega_w,
        "cos_t2f": cos_t2f, "cos_f2t": cos_f2t, "sin_t2f": sin_t2f,
        "cosft_duality_error": dual,
    }
