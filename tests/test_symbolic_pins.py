"""Symbolic pins of the oracle's right-hand sides (the formulas every kernel
restates), after the reference's SymPy checks:

* verification/test_kerr_ham_analytic.py:94-111 — the grouped analytic
  partials of the Kerr Hamiltonian against SymPy's derivative of 2H on the
  432-point grid (r, theta, a, L_z), 1e-9 relative in float64; here all five
  components of the right-hand side (dr, dtheta, dphi from the momenta,
  dp_r, dp_theta from the partials) are pinned;
* verification/test_christoffel_sympy.py — the Schwarzschild geodesic
  equation rebuilt from the metric (Christoffel symbols by the
  metric-compatibility formula) against the oracle's right-hand side.
"""

from __future__ import annotations

import ctypes as C
import itertools

import numpy as np
import pytest

sp = pytest.importorskip("sympy")


def _kerr_rhs_f64(oracle, y6, c5):
    y = np.ascontiguousarray(y6, dtype=np.float64)
    c = np.ascontiguousarray(c5, dtype=np.float64)
    d = np.zeros(6, dtype=np.float64)
    oracle.lib().oracle_kerr_rhs_f64(oracle._p(y), oracle._p(c), oracle._p(d))
    return d


def _schw_rhs_f64(oracle, y8, rs):
    y = np.ascontiguousarray(y8, dtype=np.float64)
    d = np.zeros(8, dtype=np.float64)
    oracle.lib().oracle_schw_rhs_f64(oracle._p(y), C.c_double(rs), oracle._p(d))
    return d


def test_kerr_rhs_matches_symbolic_hamiltonian(oracle):
    r, th, pr, pth, E, L, a, M = sp.symbols("r theta p_r p_theta E L a M", real=True)
    s2, c2 = sp.sin(th) ** 2, sp.cos(th) ** 2
    Sigma = r**2 + a**2 * c2
    Delta = r**2 - 2 * M * r + a**2
    A = (r**2 + a**2) ** 2 - a**2 * Delta * s2
    # 2H = g^{mu nu} p_mu p_nu for p_t = -E, p_phi = L (Boyer-Lindquist inverse metric)
    twoH = (-A * E**2 + 4 * M * r * a * E * L) / (Sigma * Delta) \
        + (Delta - a**2 * s2) * L**2 / (Sigma * Delta * s2) + (Delta * pr**2 + pth**2) / Sigma
    args = (r, th, pr, pth, E, L, a, M)
    f = {k: sp.lambdify(args, e, "math") for k, e in {
        "dr": sp.diff(twoH, pr) / 2, "dth": sp.diff(twoH, pth) / 2, "dph": sp.diff(twoH, L) / 2,
        "dpr": -sp.diff(twoH, r) / 2, "dpth": -sp.diff(twoH, th) / 2}.items()}
    grid = itertools.product([2.6, 3.1, 6.0, 12.0, 40.0, 150.0], [0.05, 0.4, 1.0, np.pi / 2, 2.4, np.pi - 0.05],
                             [0.0, 0.5, 0.94, 0.998], [-7.5, 0.0, 3.7])
    n = 0
    for rv, thv, av, Lv in grid:
        Ev, Mv, prv, pthv = 1.0, 1.0, 0.6, 2.3
        d = _kerr_rhs_f64(oracle, [0.0, rv, thv, 0.0, prv, pthv], [Ev, Lv, 0.0, av, Mv])
        got = {"dr": d[1], "dth": d[2], "dph": d[3], "dpr": d[4], "dpth": d[5]}
        for k, fn in f.items():
            ref = fn(rv, thv, prv, pthv, Ev, Lv, av, Mv)
            assert got[k] == pytest.approx(ref, rel=1e-9, abs=1e-9), (k, rv, thv, av, Lv)
        n += 1
    assert n == 432


def test_schwarzschild_rhs_matches_christoffel_symbols(oracle):
    t, r, th, ph = sp.symbols("t r theta phi", real=True)
    rs = sp.symbols("rs", positive=True)
    f = 1 - rs / r
    g = sp.diag(-f, 1 / f, r**2, r**2 * sp.sin(th) ** 2)
    x = (t, r, th, ph)
    gi = g.inv()
    u = sp.symbols("ut ur uth uph", real=True)
    rhs = []
    for mu in range(4):
        acc = 0
        for nu in range(4):
            for sg in range(4):
                gam = sum(gi[mu, lam] * (sp.diff(g[lam, sg], x[nu]) + sp.diff(g[lam, nu], x[sg])
                                         - sp.diff(g[nu, sg], x[lam])) for lam in range(4)) / 2
                acc -= gam * u[nu] * u[sg]
        rhs.append(sp.lambdify((r, th, rs, *u), acc, "math"))
    rng = np.random.default_rng(5)
    for _ in range(200):
        rv, thv = rng.uniform(2.2, 80.0), rng.uniform(0.05, np.pi - 0.05)
        uv = rng.uniform(-1.0, 1.0, 4)
        d = _schw_rhs_f64(oracle, [0.0, rv, thv, 0.3, *uv], 2.0)
        assert d[1] == pytest.approx(uv[1], rel=1e-15) and d[0] == pytest.approx(uv[0], rel=1e-15)
        for mu in range(4):
            ref = rhs[mu](rv, thv, 2.0, *uv)
            assert d[4 + mu] == pytest.approx(ref, rel=1e-10, abs=1e-12), (mu, rv, thv)
