"""CPU checks of the differentiable render form's specification
(oracle/diff_oracle.hpp): it reduces to the reference's render when its
smoothing is turned off, and its loss is smooth enough in the four parameters
for central differences to settle (the property the adjoint relies on)."""

from __future__ import annotations

import math

import numpy as np

from singularity_gb300 import _native as N


def _scene(S, w, h, spp):
    return S.workloads.differentiation_base(w, h, spp)


def test_form_reduces_to_reference_render(oracle):
    """Crossing model, soft edge -> 0, no fade: the reference's first-hit
    render with the starfield off (orbital camera at elevation pi/2 - i,
    azimuth 0).  Pixels may differ only where the blackbody blend band
    (6500-6700 K) is hit or a ray ends inside the photon orbit."""
    import singularity_gb300 as S
    a, i, rin, ts = 0.7, math.radians(60.0), S.kerr_isco_prograde(1.0, 0.7), 1.0
    w, h = 64, 40
    cam = S.build_orbital_camera(40.0, math.pi / 2 - i, 0.0, 30.0)
    sc = S.Scene(spin_a_over_M=a, disc_inner_M=rin, disc_outer_M=30.0, disc_peak_T_K=1e4 * ts,
                 render_supersample=2, h_step=0.2, max_steps=2000)
    u = S.pack_uniforms(sc, cam, w, h)
    u.flags &= ~N.SGX_FLAG_STARFIELD_ON
    _, ref = oracle.render(u, precision="f64")
    form = oracle.diff_render(_scene(S, w, h, 2), (a, i, rin, ts), eps=1e-5, fade=(0.0, 1.0),
                              model=oracle.DIFF_MODEL_CROSSING)
    e = np.abs(form - ref.reshape(h, w, 3))
    assert e.mean() <= 1e-5
    assert (e.max(axis=-1) <= 1e-6).mean() >= 0.95


def test_fp32_form_tracks_fp64(oracle):
    import singularity_gb300 as S
    base = _scene(S, 48, 32, 2)
    p = S.workloads.differentiation_params(S.workloads.differentiation_target())
    d = np.abs(oracle.diff_render(base, p, precision="f32") - oracle.diff_render(base, p))
    assert d.mean() <= 1e-5 and d.max() <= 1e-3


def test_central_differences_settle(oracle):
    """Slab model (the default): FD of the image loss at steps 1e-3 and 3e-4
    agree to 2e-3 in all four parameters; the form has no jumps.  (The
    remaining difference is the O(step) bias of the clamps' kinks.)"""
    import singularity_gb300 as S
    W = S.workloads
    base = _scene(S, 64, 48, 2)
    target = oracle.diff_render(base, W.differentiation_params(W.differentiation_target()))
    guess = W.differentiation_params(W.differentiation_guess())
    g1 = oracle.diff_fd_gradient(base, guess, target, step=1e-3)
    g2 = oracle.diff_fd_gradient(base, guess, target, step=3e-4)
    assert np.all(np.abs(g1 - g2) <= 2e-3 * np.abs(g2)), (g1, g2)


def test_crossing_model_smooth_in_radius_and_temperature(oracle):
    """The crossing model is smooth in r_in and t_scale only: rays grazing the
    plane make its image jump in spin and inclination, which is why the slab
    is the default.  Pinned so a change of either model shows up here."""
    import singularity_gb300 as S
    W = S.workloads
    base = _scene(S, 48, 32, 2)
    form = dict(model=oracle.DIFF_MODEL_CROSSING)
    target = oracle.diff_render(base, W.differentiation_params(W.differentiation_target()), **form)
    guess = W.differentiation_params(W.differentiation_guess())
    g1 = oracle.diff_fd_gradient(base, guess, target, step=1e-3, **form)
    g2 = oracle.diff_fd_gradient(base, guess, target, step=3e-4, **form)
    for k in (2, 3):
        assert abs(g1[k] - g2[k]) <= 0.02 * abs(g1[k]), (k, g1, g2)


def test_dual_gradient_matches_central_differences(oracle):
    """The oracle's forward-mode gradient against its own central differences
    (the two independent ways the oracle differentiates the form).  The bar
    is the differences' own error: the clamps of ACES and the blackbody fit
    are kinks, which bias a central difference by O(step) (2.4e-3 on the
    temperature scale at this size and step)."""
    import singularity_gb300 as S
    W = S.workloads
    base = _scene(S, 48, 32, 2)
    target = oracle.diff_render(base, W.differentiation_params(W.differentiation_target()))
    guess = W.differentiation_params(W.differentiation_guess())
    img = oracle.diff_render(base, guess)
    g, img2 = oracle.diff_grad(base, guess, 2.0 * (img - target) / img.size)
    np.testing.assert_array_equal(img2, img)
    fd = oracle.diff_fd_gradient(base, guess, target, step=3e-4)
    assert np.all(np.abs(g - fd) <= 3e-3 * np.abs(fd)), (g, fd)
