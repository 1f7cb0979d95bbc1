"""Properties of the error-controlled integrator's CPU specification (no GPU).

The reference has no adaptive driver, so these pins are physical and
numerical: convergence to the fine fixed-step solution, precision forms that
agree at the stated tolerance, Carter-constant drift, and the photon-orbit
radius used by the mixed form's FP64 zone.
"""

from __future__ import annotations

import numpy as np
import pytest


def _scene(sgx, w=48, h=27, spp=1, spin=0.94, dist=40.0, incl_deg=75.0, fov=30.0, max_steps=20000):
    isco = sgx.kerr_isco_prograde(1.0, spin)
    sc = sgx.Scene(spin_a_over_M=spin, disc_inner_M=isco, disc_outer_M=30.0, disc_peak_T_K=1e4,
                   render_supersample=spp, max_steps=max_steps)
    cam = sgx.build_orbital_camera(dist, np.pi / 2 - np.radians(incl_deg), 0.0, fov)
    return sgx.pack_uniforms(sc, cam, w, h)


def test_adaptive_converges_to_fine_fixed_step(oracle, sgx):
    """FP64: adaptive at tol 1e-8 vs fixed-step RK4 at h = 0.01 give the same
    termination and colours for non-grazing rays."""
    u = _scene(sgx, 24, 14)
    fine = u.copy()
    fine.h_step = 0.01
    fine.max_steps = 400000
    n = u.width * u.height
    gy, gx = np.divmod(np.arange(n, dtype=np.uint32), u.width)
    s = np.zeros(n, np.uint32)
    h_ad, _, t_ad = oracle.trace(u, gx, gy, s, precision="f64", adaptive=oracle.adaptive_opts(tol=1e-8))
    h_fx, _, t_fx = oracle.trace(fine, gx, gy, s, precision="f64")
    same = t_ad == t_fx
    assert same.mean() >= 0.97, same.mean()
    # escaped rays land in the same starfield cell or neighbours: compare colours loosely
    close = np.all(np.abs(h_ad - h_fx) <= 1e-2 * np.maximum(1.0, np.abs(h_fx)), axis=1)
    assert (close | ~same).mean() >= 0.9


@pytest.mark.parametrize("mixed", [False, True])
def test_fp32_forms_match_fp64_within_target(oracle, sgx, mixed):
    """Mean per-channel error of the FP32 (and mixed) forms against FP64 <= 1e-3."""
    u = _scene(sgx, 64, 36, spp=2)
    a32 = oracle.adaptive_opts(mixed=mixed)
    a64 = oracle.adaptive_opts()
    img32, ldr32 = oracle.render(u, "f32", adaptive=a32)
    img64, ldr64 = oracle.render(u, "f64", adaptive=a64)
    err = np.abs(ldr32.astype(np.float64) - ldr64).mean()
    assert err <= 1e-3, err
    d8 = np.abs(img32[..., :3].astype(int) - img64[..., :3].astype(int))
    assert (d8.max(-1) <= 1).mean() >= 0.98


def test_carter_constant_drift(oracle, sgx):
    """Relative Carter drift |Q_end - Q0| / (|Q0| + L^2 + a^2 E^2) at tol 1e-6:
    median <= 1e-6 in FP32 and FP64 alike (truncation-limited, not precision-limited)."""
    u = _scene(sgx, 40, 24)
    n = u.width * u.height
    gy, gx = np.divmod(np.arange(n, dtype=np.uint32), u.width)
    s = np.zeros(n, np.uint32)
    med = {}
    for prec in ("f32", "f64"):
        _, _, term, d = oracle.trace(u, gx, gy, s, precision=prec, adaptive=oracle.adaptive_opts(), diag=True)
        ok = term != 5
        dq = np.array([abs(x.Q_end - x.Q0) / x.norm_Q for x in d])[ok]
        med[prec] = float(np.median(dq))
        assert np.isfinite(dq).all()
    assert med["f32"] <= 1e-6 and med["f64"] <= 1e-6, med
    assert med["f32"] <= 5 * med["f64"] + 1e-7, med


def test_fewer_steps_than_reference_fixed_step(oracle, sgx):
    u = _scene(sgx, 32, 18)
    n = u.width * u.height
    gy, gx = np.divmod(np.arange(n, dtype=np.uint32), u.width)
    s = np.zeros(n, np.uint32)
    fixed = u.copy()
    fixed.max_steps = 2500
    _, st_ad, _ = oracle.trace(u, gx, gy, s, adaptive=oracle.adaptive_opts())
    _, st_fx, _ = oracle.trace(fixed, gx, gy, s)
    assert st_ad.mean() * 2 < st_fx.mean(), (st_ad.mean(), st_fx.mean())


def test_photon_orbit_radius_known_answers(oracle):
    """xi(r) round trip and the a = 0 limit (3M); prograde/retrograde ends.
    12 halvings of [r_pro, r_ret] (< 3M wide) resolve r_c to 3.7e-4 M, well
    inside the 0.05 M band the mixed form needs."""
    import ctypes as C
    L = oracle.lib()
    L.oracle_photon_orbit_radius.restype = C.c_double
    L.oracle_photon_orbit_radius.argtypes = [C.c_double, C.c_double, C.c_double]
    assert L.oracle_photon_orbit_radius(0.0, 1.0, 5.0) == pytest.approx(3.0)
    a = 0.94
    for r in (1.6, 2.0, 2.8, 3.5):
        xi = (r * r * (3 - r) - a * a * (r + 1)) / (a * (r - 1))
        assert L.oracle_photon_orbit_radius(a, 1.0, xi) == pytest.approx(r, abs=4e-4)
    assert np.isnan(L.oracle_photon_orbit_radius(a, 1.0, 100.0))


def test_schwarzschild_metric_keeps_fixed_step(oracle, sgx):
    """The adaptive form is Kerr-only; a Schwarzschild-metric scene keeps the
    reference integrator, bit for bit."""
    sc = sgx.Scene(metric=sgx.MetricType.Schwarzschild, spin_a_over_M=0.0, disc_inner_M=6, disc_outer_M=20)
    u = sgx.pack_uniforms(sc, sgx.build_orbital_camera(30.0, 0.174533, 0.0, 40.0), 16, 16)
    a, _ = oracle.render(u, adaptive=oracle.adaptive_opts())
    b, _ = oracle.render(u)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("spin,incl,dist", [(0.94, 75.0, 40.0), (0.0, 60.0, 20.0), (0.998, 30.0, 15.0), (0.6, 85.0, 60.0)])
def test_early_capture_changes_no_result(oracle, sgx, spin, incl, dist):
    """A ray inside both its photon-orbit radius (less 0.05 M) and the disc's
    inner edge, moving inward with Q >= 0, ends as captured: the same
    termination and colour as tracing on to the reference's 1.02 r_+ cut,
    in fewer attempts."""
    u = _scene(sgx, 96, 54, spin=spin, dist=dist, incl_deg=incl, fov=45.0, max_steps=4000)
    n = u.width * u.height
    gy, gx = np.divmod(np.arange(n, dtype=np.uint32), u.width)
    s = np.zeros(n, np.uint32)
    for prec, mixed in (("f32", False), ("f32", True), ("f64", False)):
        on = oracle.trace(u, gx, gy, s, precision=prec, adaptive=oracle.adaptive_opts(mixed=mixed))
        off = oracle.trace(u, gx, gy, s, precision=prec, adaptive=oracle.adaptive_opts(mixed=mixed,
                                                                                      early_capture=False))
        np.testing.assert_array_equal(on[2], off[2])
        np.testing.assert_array_equal(on[0], off[0])
        assert np.all(on[1] <= off[1])
        captured = on[2] == 0
        if captured.any():
            assert on[1][captured].mean() < off[1][captured].mean()
