"""The reference's physics known-answer tests (its Catch2 suite), restated on
the oracle — the FP32 formulas the kernels share — with the reference's own
thresholds:

* radius-adaptive step, tests/test_adaptive_step.cpp:65-150 (deflection within
  0.5 % of a fine fixed step, E and L to 3e-4, >= 5x fewer steps);
* Schwarzschild RK4, tests/test_schwarzschild.cpp:21-125 and
  tests/test_conserved.cpp:45-95 (radial fall stays radial, circular orbit at
  6 M, photon sphere closes to 0.5 %, photon E / L / null condition to 3e-4);
* Kerr Hamiltonian RK4, tests/test_kerr_hamilton.cpp:31-353 (2H = 0 on a null
  orbit, equatorial symmetry, photon sphere, bounded non-equatorial orbit,
  20000-step stress, 2H along a long geodesic, analytic partials vs finite
  differences at 5e-3, repulsive polar barrier);
* equatorial crossing, tests/test_disc_intersection.cpp:20-95;
* Kerr geometry on the path, verification/test_kerr_geometry.py:95-228 (the
  prograde ISCO as the circular-orbit energy minimum, the equatorial photon
  orbits, the mixed form's spherical photon orbit radius).
"""

from __future__ import annotations

import math

import pytest

import numpy as np


def _tangential_photon(r0, rs):
    # state (t, r, theta, phi, u^t, u^r, u^theta, u^phi) at periapsis r0 in the
    # equatorial plane; null condition with u^r = u^theta = 0
    ut = 1.0 / (1.0 - rs / r0)
    uphi = math.sqrt(1.0 - rs / r0) * ut / r0
    return np.array([0.0, r0, 0.5 * math.pi, 0.0, ut, 0.0, 0.0, uphi], dtype=np.float32)


def _motion_angle(y):
    cp, sp = math.cos(y[3]), math.sin(y[3])
    vx = y[5] * cp - y[1] * y[7] * sp
    vy = y[5] * sp + y[1] * y[7] * cp
    return math.atan2(vy, vx)


def test_adaptive_step_preserves_deflection(oracle):
    rs, r0, r_out = 2.0, 8.0, 400.0
    ref, n_ref, _, _ = oracle.schw_integrate(_tangential_photon(r0, rs), 0.01, rs, r_out, False)
    ad, n_ad, _, _ = oracle.schw_integrate(_tangential_photon(r0, rs), 0.12, rs, r_out, True)
    assert n_ref > 0 and n_ad > 0
    psi_ref, psi_ad = _motion_angle(ref), _motion_angle(ad)
    deflection = abs(psi_ref - 0.5 * math.pi)
    assert deflection > 0.1
    assert abs(psi_ad - psi_ref) < 0.005 * max(deflection, 1.0)


def test_adaptive_step_conserves_e_and_l(oracle):
    _, n, max_e, max_l = oracle.schw_integrate(_tangential_photon(8.0, 2.0), 0.12, 2.0, 400.0, True, budget=100000)
    assert n > 0
    assert max_e < 3e-4 and max_l < 3e-4


def test_adaptive_step_takes_5x_fewer_steps(oracle):
    _, n_fixed, _, _ = oracle.schw_integrate(_tangential_photon(8.0, 2.0), 0.12, 2.0, 200.0, False)
    _, n_ad, _, _ = oracle.schw_integrate(_tangential_photon(8.0, 2.0), 0.12, 2.0, 200.0, True)
    assert n_fixed > 0 and n_ad > 0
    assert n_ad * 5 <= n_fixed


# --- Schwarzschild geodesic RK4 (tests/test_schwarzschild.cpp:21-125,
#     tests/test_conserved.cpp:45-95) ---------------------------------------

F = np.float32
PI = F(math.pi)


def test_radial_free_fall_stays_radial(oracle):
    rs = F(2.0)
    y = np.array([0, 50, PI / 2, 0, 1 / math.sqrt(1 - 2 / 50), 0, 0, 0], dtype=np.float32)
    for _ in range(500):
        y = oracle.schw_rk4_n(y, 0.1, rs)
        assert abs(y[6]) < 1e-5 and abs(y[7]) < 1e-5
        assert abs(y[2] - PI / 2) < 1e-5 and abs(y[3]) < 1e-5
    assert rs < y[1] < 50


def test_circular_timelike_orbit_at_isco_stays_circular(oracle):
    r0 = F(6.0)
    ut = F(1.0) / np.sqrt(F(1.0) - F(3.0) / r0)
    uphi = np.sqrt(F(1.0) / (r0 * r0 * r0)) * ut
    y = np.array([0, r0, PI / 2, 0, ut, 0, 0, uphi], dtype=np.float32)
    n = int(F(2.0) * PI / uphi / F(0.05))
    r_min = r_max = float(r0)
    for _ in range(n):
        y = oracle.schw_rk4_n(y, 0.05, 2.0)
        r_min, r_max = min(r_min, y[1]), max(r_max, y[1])
        assert abs(y[2] - PI / 2) < 1e-4
    assert abs(r_max - r0) < 0.005 * r0 and abs(r_min - r0) < 0.005 * r0


def test_photon_sphere_orbit_closes(oracle):
    r0 = F(3.0)
    y = np.array([0, r0, PI / 2, 0, r0 / np.sqrt(F(1) - F(2) / r0), 0, 0, 1.0], dtype=np.float32)
    y = oracle.schw_rk4_n(y, 0.01, 2.0, int(F(2) * PI / F(0.01)))
    assert abs(y[1] - r0) < 0.005 * r0


def test_photon_conserves_energy_momentum_and_null_condition(oracle):
    rs, r0, b = 2.0, 50.0, 20.0
    y = np.array([0, r0, PI / 2, 0, 1 / (1 - rs / r0), 0, 0, b / (r0 * r0)], dtype=np.float32)

    def inv(s):
        f = 1 - rs / s[1]
        st = math.sin(s[2])
        E = f * s[4]
        L = s[1] ** 2 * st * st * s[7]
        N = -f * s[4] ** 2 + s[5] ** 2 / f + s[1] ** 2 * (s[6] ** 2 + st * st * s[7] ** 2)
        return E, L, N

    E0, L0, N0 = inv(y)
    worst = [0.0, 0.0, 0.0]
    for _ in range(10000):
        y = oracle.schw_rk4_n(y, 0.1, rs)
        if y[1] < rs * 1.01:
            break
        E, L, N = inv(y)
        worst = [max(worst[0], abs(E - E0) / abs(E0)), max(worst[1], abs(L - L0) / abs(L0)),
                 max(worst[2], abs(N - N0) / (E0 * E0))]
    assert max(worst) < 3e-4, worst


# --- Kerr Hamiltonian integrator (tests/test_kerr_hamilton.cpp:31-353) -----

def _momenta(r, th, ur, uth, a, M=1.0):
    r, th, ur, uth, a = (F(x) for x in (r, th, ur, uth, a))
    sigma = r * r + a * a * np.cos(th) ** 2
    delta = r * r - F(2 * M) * r + a * a
    return sigma / delta * ur, sigma * uth


def _photon_sphere_consts():
    r = F(3.0)
    f = F(1) - F(2) / r
    uphi = np.sqrt(f) / r
    return r, uphi, (f * F(1.0), r * r * uphi, 0.0, 0.0, 1.0)


def test_two_H_zero_on_null_orbit(oracle):
    r, _, c = _photon_sphere_consts()
    pr, pth = _momenta(r, PI / 2, 0, 0, 0)
    assert abs(oracle.kerr_two_H(r, PI / 2, pr, pth, c)) < 1e-4


def test_equatorial_rhs_has_no_polar_motion(oracle):
    for a in (0.0, 0.5, 0.94):
        d = oracle.kerr_rhs([0, 10, PI / 2, 0, 0, 0], (1.0, 4.0, 0.0, a, 1.0))
        assert abs(d[2]) < 1e-6 and abs(d[5]) < 1e-4


def test_kerr_photon_sphere_closes_at_zero_spin(oracle):
    r, uphi, c = _photon_sphere_consts()
    pr, pth = _momenta(r, PI / 2, 0, 0, 0)
    n = int(F(2) * PI / uphi / F(0.01))
    y = oracle.kerr_rk4_n([0, r, PI / 2, 0, pr, pth], 0.01, c, n)
    assert abs(y[1] - r) < 0.005 * r and abs(y[2] - PI / 2) < 1e-4


def test_non_equatorial_geodesic_stays_bounded(oracle):
    E, L, Q, a = F(1), F(3), F(2), F(0.5)
    r, th = F(10), PI / F(3)
    R = ((r * r + a * a) * E - a * L) ** 2 - (r * r - F(2) * r + a * a) * (Q + (L - a * E) ** 2)
    assert R > 0
    delta = r * r - F(2) * r + a * a
    y = np.array([0, r, th, 0, np.sqrt(R) / delta, 0], dtype=np.float32)
    c = (E, L, Q, a, 1.0)
    assert abs(oracle.kerr_two_H(y[1], y[2], y[4], y[5], c)) < 2e-2
    ths, rs = [th], [r]
    for _ in range(1500):
        y = oracle.kerr_rk4_n(y, 0.1, c)
        if not (np.isfinite(y[1]) and np.isfinite(y[2])):
            break
        ths.append(y[2])
        rs.append(y[1])
    assert max(ths) - min(ths) > 0.01 and min(ths) > 0.1 and max(ths) < math.pi - 0.1
    assert abs(oracle.kerr_two_H(y[1], y[2], y[4], y[5], c)) < 1e-1
    assert np.all(np.isfinite(rs))


def test_long_escape_stays_finite(oracle):
    a, r = F(0.3), F(50)
    delta = r * r - F(2) * r + a * a
    sigma = r * r
    y = np.array([0, r, PI / 2, 0, sigma / delta, 0], dtype=np.float32)
    c = (1.0, 2.0, 0.0, a, 1.0)
    for _ in range(200):
        y = oracle.kerr_rk4_n(y, 0.1, c, 100)
        if y[1] > 1e6:
            break
    assert np.all(np.isfinite(y))
    H2 = oracle.kerr_two_H(y[1], y[2], y[4], y[5], c)
    assert math.isfinite(H2) and abs(H2) < 1.0


def test_two_H_preserved_along_long_geodesic(oracle):
    a, r0, ur, uphi = F(0.5), F(30), F(1), F(0.01)
    delta = r0 * r0 - F(2) * r0 + a * a
    g_tt = -(F(1) - F(2) / r0)
    g_tp = -F(2) * a / r0
    g_rr = r0 * r0 / delta
    g_pp = ((r0 * r0 + a * a) ** 2 - a * a * delta) / (r0 * r0)
    B = F(2) * g_tp * uphi
    Cq = g_rr * ur * ur + g_pp * uphi * uphi
    ut = (-B - np.sqrt(B * B - F(4) * g_tt * Cq)) / (F(2) * g_tt)
    c = (-(g_tt * ut + g_tp * uphi), g_tp * ut + g_pp * uphi, 0.0, a, 1.0)
    pr, pth = _momenta(r0, PI / 2, ur, 0, a)
    y = np.array([0, r0, PI / 2, 0, pr, pth], dtype=np.float32)
    assert abs(oracle.kerr_two_H(y[1], y[2], y[4], y[5], c)) < 1e-3
    y = oracle.kerr_rk4_n(y, 0.1, c, 2000)
    H2 = oracle.kerr_two_H(y[1], y[2], y[4], y[5], c)
    assert math.isfinite(H2) and abs(H2) < 1e-2


def test_analytic_partials_match_finite_differences(oracle):
    h = 1e-4
    for r in (3.1, 6.0, 12.0, 40.0):
        for th in (0.4, 1.0, float(PI / 2), 2.4):
            for a in (0.0, 0.5, 0.94):
                c = (1.0, 3.7, 0.0, a, 1.0)
                d = oracle.kerr_rhs([0, r, th, 0, 0.6, 2.3], c)
                H = lambda rr, tt: float(oracle.kerr_two_H(rr, tt, 0.6, 2.3, c))
                fd_r = -0.5 * (H(F(r) + F(h), th) - H(F(r) - F(h), th)) / (2 * h)
                fd_t = -0.5 * (H(r, F(th) + F(h)) - H(r, F(th) - F(h))) / (2 * h)
                assert abs(d[4] - fd_r) / max(1.0, abs(fd_r)) < 5e-3, (r, th, a)
                assert abs(d[5] - fd_t) / max(1.0, abs(fd_t)) < 5e-3, (r, th, a)


def test_polar_barrier_is_repulsive(oracle):
    y = [0, 8.0, float(PI - F(0.01)), 0, 0.0, 1.0]
    d = oracle.kerr_rhs(y, (1.0, 0.05, 0.0, 0.9, 1.0))
    assert d[5] < 0
    d0 = oracle.kerr_rhs(y, (1.0, 0.0, 0.0, 0.9, 1.0))
    assert np.isfinite(d0[5]) and abs(d0[5]) < abs(d[5])


# --- Equatorial crossing (tests/test_disc_intersection.cpp:20-95) ----------

def test_crossing_detection_and_fraction(oracle):
    hp = PI / 2
    assert not oracle.crossing(hp - F(0.3), hp - F(0.05))[0]
    assert not oracle.crossing(hp + F(0.2), hp + F(0.4))[0]
    x, f = oracle.crossing(hp - F(0.1), hp + F(0.1))
    assert x and abs(f - 0.5) <= 1e-6
    x, f = oracle.crossing(hp - F(0.04), hp + F(0.12))
    assert x and abs(f - 0.25) <= 1e-6
    (x1, f1), (x2, f2) = oracle.crossing(hp - F(0.2), hp + F(0.3)), oracle.crossing(hp + F(0.3), hp - F(0.2))
    assert x1 and x2 and abs(f1 + f2 - 1.0) <= 1e-6
    x, f = oracle.crossing(hp - F(0.15), hp + F(0.05))
    r_cross = F(12.4) + F(f) * (F(11.9) - F(12.4))
    assert x and 11.9 <= r_cross <= 12.4 and abs(r_cross - 12.025) <= 1e-5


# --- Kerr geometry used on the path (verification/test_kerr_geometry.py:95-228):
#     the prograde ISCO (disc inner edge), the equatorial photon orbits (the
#     mixed form's band, the differentiable form's capture radius) ----------

def _circular_energy(r, a, M=1.0):
    # specific energy of a prograde circular equatorial orbit (Bardeen, Press & Teukolsky 1972)
    v = math.sqrt(M / r)
    return (1 - 2 * v * v + a * v ** 3) / math.sqrt(1 - 3 * v * v + 2 * a * v ** 3)


def test_isco_is_the_circular_orbit_energy_minimum():
    from scipy.optimize import brentq
    import singularity_gb300 as S
    for a in (0.0, 0.5, 0.94, 0.998):
        dE = lambda r: (_circular_energy(r + 1e-6, a) - _circular_energy(r - 1e-6, a)) / 2e-6
        r_pro = 2 * (1 + math.cos(2 / 3 * math.acos(-a)))  # circular orbits exist outside it
        r_min = brentq(dE, r_pro + 1e-3, 9.0)
        got = S.kerr_isco_prograde(1.0, a)
        assert got == pytest.approx(r_min, rel=3e-4), (a, got, r_min)
    assert S.kerr_isco_prograde(1.0, 0.0) == pytest.approx(6.0, rel=3e-4)


def test_equatorial_photon_orbits_close():
    """The prograde / retrograde circular photon orbit radii 2M(1 + cos(2/3 acos(-+a/M)))
    satisfy r^(3/2) - 3M r^(1/2) +- 2 a M^(1/2) = 0; a = 0 gives 3M."""
    for a in (0.0, 0.5, 0.94, 0.998):
        r_pro = 2 * (1 + math.cos(2 / 3 * math.acos(-a)))
        r_ret = 2 * (1 + math.cos(2 / 3 * math.acos(a)))
        assert abs(r_pro ** 1.5 - 3 * r_pro ** 0.5 + 2 * a) < 1e-9
        assert abs(r_ret ** 1.5 - 3 * r_ret ** 0.5 - 2 * a) < 1e-9
    assert 2 * (1 + math.cos(2 / 3 * math.acos(0.0))) == pytest.approx(3.0)


def test_photon_orbit_radius_spans_the_photon_region(oracle):
    """The mixed form's r_c(xi): across the photon region it returns the
    spherical orbit of that xi (the equatorial orbits bound the region)."""
    import ctypes as C
    L = oracle.lib()
    L.oracle_photon_orbit_radius.restype = C.c_double
    L.oracle_photon_orbit_radius.argtypes = [C.c_double, C.c_double, C.c_double]
    a = 0.5
    xi = lambda r: (r * r * (3 - r) - a * a * (r + 1)) / (a * (r - 1))
    r_pro = 2 * (1 + math.cos(2 / 3 * math.acos(-a)))
    r_ret = 2 * (1 + math.cos(2 / 3 * math.acos(a)))
    for r in np.linspace(r_pro, r_ret, 9)[1:-1]:
        assert L.oracle_photon_orbit_radius(a, 1.0, xi(r)) == pytest.approx(r, abs=4e-4)
