"""Oracle (test infrastructure only): the macroscopic dielectric function eps(i omega) mapped
onto the minimax frequencies for the G0W0 head correction, as LibRPA's interpolate_dielec_func
does it (src/core/dielecmodel.cpp:65-104).

  option 0  the given values (the input grid is the target grid)
  option 1  CubicSpline (src/math/interpolate.cpp:9-150), in the reference's own step order:
            the elimination and the back substitution of its tridiagonal system run in one loop
            (:44-53), so back-substitution steps ahead of the elimination read z = 0; outside the
            data range the cubic of :75-117 built from the end interval's values and slopes
  option 2  LevMarqFitting (src/math/fitting.cpp:90-199; Levenberg-Marquardt after R. Babich's
            published C code) of the two-term Havriliak-Negami model DoubleHavriliakNegami
            (dielecmodel.cpp:34-63), all 8 parameters started at 1 but e1 = e2 = eps(omega_0)

Pure Python floats (a few dozen points). Pinned by the reference's structure (the spline
reproduces its data points; the fit recovers data drawn from the model) and by the library's C
entry librpa_gb300_interpolate_dielec_func, which restates the same steps.
"""
from __future__ import annotations

import math


def cubic_spline(xs, ys):
    """Coefficients (a, b, c, d) of interpolate.cpp:9-67."""
    n = len(xs)
    if n < 2 or len(ys) != n:
        raise ValueError("cubic spline: at least 2 points, with one value per point")
    h = [xs[i + 1] - xs[i] for i in range(n - 1)]
    alpha = [3 * (ys[i + 1] - ys[i]) / h[i] for i in range(n - 1)]
    l = [0.0] * n
    mu = [0.0] * (n - 1)
    l[0] = 1.0
    for i in range(1, n - 1):
        l[i] = 2 * (xs[i + 1] - xs[i - 1]) - h[i - 1] * mu[i - 1]
        mu[i] = h[i] / l[i]
    l[n - 1] = 1.0
    z = [0.0] * n
    c = [0.0] * n
    for i in range(1, n):
        z[i] = (alpha[i - 1] - h[i - 1] * z[i - 1]) / l[i]
        c[n - i - 1] = z[n - i] - mu[n - i - 1] * c[n - i]
    a = list(ys)
    b = [0.0] * n
    d = [0.0] * n
    for i in range(n - 1):
        b[i] = (ys[i + 1] - ys[i]) / h[i] - h[i] * (c[i + 1] + 2 * c[i]) / 3
        d[i] = (c[i + 1] - c[i]) / (3 * h[i])
    return a, b, c, d


def spline_eval(xs, coef, x):
    """interpolate.cpp:70-139."""
    a, b, c, d = coef
    n = len(xs)
    if x < xs[0] or x > xs[n - 1]:
        i = 0 if x < xs[0] else n - 2
        x0, x1 = xs[i], xs[i + 1]
        y0, y1, m0, m1 = a[i], a[i + 1], b[i], b[i + 1]
        h = x1 - x0
        t = x - x0
        dy = y1 - y0
        dm = m1 - m0
        return (y0 + m0 * t + (3 * dy / h ** 2 - 2 * m0 / h - dm / h) * t ** 2
                + (-2 * dy / h ** 3 + m0 / h ** 2 + dm / h ** 2) * t ** 3)
    for i in range(n - 1):
        if xs[i] <= x <= xs[i + 1]:
            t = x - xs[i]
            return a[i] + b[i] * t + c[i] * t ** 2 + d[i] * t ** 3
    return 0.0


def hn_value(u, p):
    """DoubleHavriliakNegami::func_imfreq."""
    return (1.0 + (p[0] - 1.0) / math.pow(1.0 + math.pow(u * p[3], p[1]), p[2])
            + (p[4] - 1.0) / math.pow(1.0 + math.pow(u * p[7], p[5]), p[6]))


def hn_grad(u, p):
    """DoubleHavriliakNegami::grad_imfreq: d hn_value / d p."""
    g = [0.0] * 8
    for t in range(2):
        e, al, be, ta = p[4 * t:4 * t + 4]
        s = u * ta
        base = 1.0 + math.pow(s, al)
        g[4 * t] = 1.0 / math.pow(base, be)
        g[4 * t + 1] = (e - 1.0) * (-be) / math.pow(base, be + 1) * math.log(s) * math.pow(s, al)
        g[4 * t + 2] = (1.0 - e) * math.log(base) / math.pow(base, be)
        g[4 * t + 3] = (e - 1.0) * (-be) / math.pow(base, be + 1) * al / ta * math.pow(s, al)
    return g


def _err(p, xs, ys):
    e = 0.0
    for x, y in zip(xs, ys):
        r = hn_value(x, p) - y
        e += r * r
    return e


def _dot(pairs):
    # left-to-right accumulation (the built-in sum() of floats compensates, which the reference's
    # loops do not)
    acc = 0.0
    for a, b in pairs:
        acc += a * b
    return acc


def _chol(n, a):
    l = [[0.0] * n for _ in range(n)]
    for i in range(n):
        for j in range(i):
            s = _dot((l[i][k], l[j][k]) for k in range(j))
            l[i][j] = (a[i][j] - s) / l[j][j]
        s = a[i][i] - _dot((l[i][k], l[i][k]) for k in range(i))
        if s < 1e-30:
            return None
        l[i][i] = math.sqrt(s)
    return l


def _chol_solve(n, l, b):
    x = [0.0] * n
    for i in range(n):
        x[i] = (b[i] - _dot((l[i][j], x[j]) for j in range(i))) / l[i][i]
    for i in range(n - 1, -1, -1):
        x[i] = (x[i] - _dot((l[j][i], x[j]) for j in range(i + 1, n))) / l[i][i]
    return x


def levmarq_fit(p, xs, ys, max_iter=10000, lam=0.1, up=10.0, down=10.0, target=1e-8):
    """LevMarqFitting::fit (fitting.cpp:99-199): returns the fitted parameters."""
    p = list(p)
    n = len(p)
    err = _err(p, xs, ys)
    newp = [0.0] * n
    newerr = 0.0
    derr = 0.0
    it = 0
    while it < max_iter:
        h = [[0.0] * n for _ in range(n)]
        d = [0.0] * n
        for x, y in zip(xs, ys):
            g = hn_grad(x, p)
            r = y - hn_value(x, p)
            for i in range(n):
                d[i] += r * g[i]
                for j in range(i + 1):
                    h[i][j] += g[i] * g[j]
        mult = 1 + lam
        ill = True
        while ill and it < max_iter:
            for i in range(n):
                h[i][i] *= mult
            ch = _chol(n, h)
            ill = ch is None
            if not ill:
                delta = _chol_solve(n, ch, d)
                newp = [p[i] + delta[i] for i in range(n)]
                newerr = _err(newp, xs, ys)
                derr = newerr - err
                ill = derr > 0
            if ill:
                mult = (1 + lam * up) / (1 + lam)
                lam *= up
                it += 1
        p = list(newp)
        err = newerr
        lam *= 1 / down
        if not ill and -derr < target:
            break
        it += 1
    return p


def interpolate_dielec_func(option, omega_in, eps_in, omega_target):
    """dielecmodel.cpp:65-104."""
    omega_in = [float(v) for v in omega_in]
    eps_in = [float(v) for v in eps_in]
    omega_target = [float(v) for v in omega_target]
    if option == 0:
        if len(eps_in) != len(omega_target):
            raise ValueError("option 0: the dielectric function must be given at the target frequencies")
        return list(eps_in)
    if option == 1:
        coef = cubic_spline(omega_in, eps_in)
        return [spline_eval(omega_in, coef, x) for x in omega_target]
    if option == 2:
        p = [1.0] * 8
        p[0] = p[4] = eps_in[0]
        p = levmarq_fit(p, omega_in, eps_in)
        return [hn_value(x, p) for x in omega_target]
    raise ValueError("Unsupported value for option")
