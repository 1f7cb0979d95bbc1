"""GPU parity of the error-controlled Kerr integrator (FP32, mixed, FP64 forms)
against its CPU specification (oracle/adaptive_oracle.hpp), through the C ABI.

Tolerances: per-sample — same termination and |rel| <= 1e-3 for >= 97 % of
samples; images — mean per-channel error <= 2e-3 of full scale.  The
precision target (FP32 vs FP64 mean per-channel error <= 1e-3) is
checked GPU-against-GPU and GPU-against-FP64-oracle.
"""

from __future__ import annotations

import numpy as np
import pytest

from imgmetrics import channel_error

pytestmark = pytest.mark.gpu

SAMPLE_FRAC = 0.97


def _scene(sgx, w=96, h=54, spp=4, spin=0.94, dist=40.0, incl_deg=75.0, fov=30.0, max_steps=2500):
    isco = sgx.kerr_isco_prograde(1.0, spin)
    sc = sgx.Scene(spin_a_over_M=spin, disc_inner_M=isco, disc_outer_M=30.0, disc_peak_T_K=1e4,
                   render_supersample=spp, max_steps=max_steps)
    cam = sgx.build_orbital_camera(dist, np.pi / 2 - np.radians(incl_deg), 0.0, fov)
    return sgx.pack_uniforms(sc, cam, w, h)


PREC = {"f32": 0, "mixed": 1, "f64": 2}


def _opts(sgx, prec):
    return sgx.default_opts(integrator=1, precision=PREC[prec])


def _oracle_opts(oracle, prec):
    return oracle.adaptive_opts(mixed=(prec == "mixed"))


@pytest.mark.parametrize("prec", ["f32", "mixed", "f64"])
@pytest.mark.parametrize("spin,incl", [(0.94, 75.0), (0.5, 60.0), (0.0, 85.0), (0.998, 20.0), (0.94, 1.0)])
def test_probe_matches_adaptive_oracle(renderer, oracle, sgx, prec, spin, incl):
    u = _scene(sgx, 64, 36, spp=4, spin=spin, incl_deg=incl)
    rng = np.random.default_rng(3)
    n = 2048
    gx = rng.integers(0, u.width, n).astype(np.uint32)
    gy = rng.integers(0, u.height, n).astype(np.uint32)
    s = rng.integers(0, 4, n).astype(np.uint32)
    hdr, steps, term = renderer.trace_samples(u, gx, gy, s, _opts(sgx, prec))
    o_prec = "f64" if prec == "f64" else "f32"
    ref, o_steps, o_term = oracle.trace(u, gx, gy, s, precision=o_prec, adaptive=_oracle_opts(oracle, prec))
    ref = ref.astype(np.float32)
    same = term == o_term
    close = np.all(np.abs(hdr - ref) <= np.maximum(1e-5, 1e-3 * np.maximum(np.abs(hdr), np.abs(ref))), axis=1)
    ok = same & close
    print(f"{prec} a={spin} i={incl}: same_term={same.mean():.4f} ok={ok.mean():.4f} "
          f"steps gpu={steps.mean():.2f} oracle={o_steps.mean():.2f} same_steps={(steps == o_steps).mean():.3f}")
    assert ok.mean() >= SAMPLE_FRAC
    assert abs(steps.mean() - o_steps.mean()) <= 0.02 * o_steps.mean() + 0.5


@pytest.mark.parametrize("prec", ["f32", "mixed", "f64"])
def test_render_matches_adaptive_oracle(renderer, oracle, sgx, prec):
    u = _scene(sgx, 96, 54, spp=4)
    img = renderer.render_image(u, _opts(sgx, prec))
    ref, _ = oracle.render(u, "f64" if prec == "f64" else "f32", adaptive=_oracle_opts(oracle, prec))
    e = channel_error(img, ref)
    print(prec, e)
    assert e["mean"] <= 2e-3, e
    assert e["le1_frac"] >= 0.97, e


def test_fp32_vs_fp64_precision_target(renderer, oracle, sgx):
    """FP32 and mixed forms against the FP64 GPU form and the FP64 CPU oracle:
    mean per-channel error (RGBA32F, full scale) <= 1e-3."""
    N = sgx._native
    u = _scene(sgx, 128, 72, spp=8)
    f64 = renderer.render_image(u, _opts(sgx, "f64"), fmt=N.FORMAT_RGBA32F)[..., :3].astype(np.float64)
    _, ldr64 = oracle.render(u, "f64", adaptive=oracle.adaptive_opts())
    assert np.abs(f64 - ldr64).mean() <= 1e-4
    for prec in ("f32", "mixed"):
        img = renderer.render_image(u, _opts(sgx, prec), fmt=N.FORMAT_RGBA32F)[..., :3].astype(np.float64)
        e_gpu = np.abs(img - f64).mean()
        e_cpu = np.abs(img - ldr64).mean()
        print(f"{prec}: mean |fp32 - fp64 gpu| = {e_gpu:.2e}, vs fp64 oracle = {e_cpu:.2e}")
        assert e_gpu <= 1e-3 and e_cpu <= 1e-3


def test_trig_forms_coincide_for_adaptive(renderer, sgx):
    """The error-controlled form carries (sin theta, cos theta) in its state and
    evaluates no sine or cosine per stage, so rhs_form 2 (which makes the
    fixed-step form carry them too) renders the same frame as form 0."""
    u = _scene(sgx, 64, 36, spp=4)
    a = renderer.render_image(u, sgx.default_opts(integrator=1, precision=0, rhs_form=0))
    b = renderer.render_image(u, sgx.default_opts(integrator=1, precision=0, rhs_form=2))
    np.testing.assert_array_equal(a, b)


def test_adaptive_stats_and_progressive(renderer, sgx):
    u = _scene(sgx, 80, 45, spp=8)
    o = _opts(sgx, "mixed")
    one = renderer.render_image(u, o)
    st = renderer.stats()
    assert st.rays == 80 * 45 * 8
    assert st.steps > st.rays and st.rejected > 0 and st.zone_steps > 0
    assert st.rejected < st.steps and st.zone_steps < st.steps
    for b in range(0, 8, 3):
        o2 = _opts(sgx, "mixed")
        o2.sample_begin, o2.sample_count = b, 3
        renderer.render(u, o2)
    np.testing.assert_array_equal(renderer.capture(), one)


def test_adaptive_rejects_bad_options(renderer, sgx):
    u = _scene(sgx, 8, 8, spp=1)
    for field, val in (("tolerance", 0.0), ("h_init_frac", -1.0), ("h_max_frac", 0.0), ("fp64_zone", -0.5)):
        o = _opts(sgx, "f32")
        setattr(o, field, val)
        with pytest.raises(sgx.SgxError):
            renderer.render(u, o)
    o = sgx.default_opts(precision=1)  # mixed form needs the adaptive integrator
    with pytest.raises(sgx.SgxError):
        renderer.render(u, o)


def _seeded_pixels(u, n_pix=4096, spp_used=16):
    """The 4096 pixels of numpy.random.default_rng(0).choice(W*H, 4096,
    replace=False), each with its first `spp_used` samples."""
    rng = np.random.default_rng(0)
    pix = rng.choice(u.width * u.height, n_pix, replace=False).astype(np.uint32)
    gx = np.repeat(pix % u.width, spp_used).astype(np.uint32)
    gy = np.repeat(pix // u.width, spp_used).astype(np.uint32)
    s = np.tile(np.arange(spp_used, dtype=np.uint32), n_pix)
    return gx, gy, s


@pytest.mark.parametrize("prec", ["f32", "mixed", "f64"])
def test_carter_drift_on_the_gpu(renderer, oracle, sgx, prec):
    """Relative drift of Carter's constant, |Q_end - Q0| / (|Q0| + L^2 + a^2 E^2),
    of the rays the GPU traced in the 4K Kerr a = 0.94 workload (the seeded
    4096 pixels x 16 samples): <= 1e-6 at the 99th percentile and at the
    maximum, with p_theta projected back onto Q after each accepted step
    (the default).  Without the projection the integrator's own drift
    exceeds 1e-6 in the tail, as the CPU oracle of the same integrator shows;
    E, L_z and Q0 equal the oracle's."""
    u = sgx.workloads.kerr_4k_256spp()
    gx, gy, s = _seeded_pixels(u)
    inv, term = renderer.trace_invariants(u, gx, gy, s, _opts(sgx, prec))
    dq = sgx.carter_drift(inv, u.spin_a)
    assert dq.size >= 0.99 * gx.size
    p50, p99, mx = np.median(dq), np.percentile(dq, 99), dq.max()
    h2 = np.abs(inv[:, 4]) / inv[:, 0] ** 2
    print(f"{prec}: Carter drift median {p50:.2e} p99 {p99:.2e} max {mx:.2e}; "
          f"|2H|/E^2 median {np.nanmedian(h2):.2e} p99 {np.nanpercentile(h2, 99):.2e}")
    assert p99 <= 1e-6 and mx <= 1e-6
    # the oracle of the same integrator: the same constants at launch
    o_prec = "f64" if prec == "f64" else "f32"
    n = 8192
    _, _, o_term, diag = oracle.trace(u, gx[:n], gy[:n], s[:n], precision=o_prec,
                                      adaptive=_oracle_opts(oracle, prec), diag=True)
    E = np.array([d.E for d in diag])
    L = np.array([d.L for d in diag])
    Q0 = np.array([d.Q0 for d in diag])
    ok = o_term != 5
    np.testing.assert_allclose(inv[:n, 0][ok], E[ok], rtol=2e-6)
    np.testing.assert_allclose(inv[:n, 1][ok], L[ok], rtol=2e-6, atol=2e-6)
    norm = np.abs(Q0) + L * L + (u.spin_a * E) ** 2
    assert np.max(np.abs(inv[:n, 2] - Q0)[ok] / norm[ok]) <= 2e-6
    # projection off: the plain integrator's tail drift, as in the oracle
    o = _opts(sgx, prec)
    o.projection = 0
    inv0, _ = renderer.trace_invariants(u, gx, gy, s, o)
    dq0 = sgx.carter_drift(inv0, u.spin_a)
    _, _, _, d0 = oracle.trace(u, gx, gy, s, precision=o_prec,
                               adaptive=oracle.adaptive_opts(mixed=(prec == "mixed"), projection=False), diag=True)
    dq0_cpu = np.array([abs(d.Q_end - d.Q0) / d.norm_Q for d in d0])
    print(f"{prec} no projection: GPU p99 {np.percentile(dq0, 99):.2e}, oracle p99 "
          f"{np.nanpercentile(dq0_cpu, 99):.2e}")
    assert np.percentile(dq0, 99) > 1e-6
    assert 0.5 <= np.percentile(dq0, 99) / np.nanpercentile(dq0_cpu, 99) <= 2.0


def test_projection_keeps_the_image(renderer, oracle, sgx):
    """The projection moves p_theta by the integrator's truncation error only:
    per sample, the HDR colour with it and without it (the probe's
    diagnostic switch) agree to the parity bar of the oracle tests, and the
    rendered frame (renders always project) matches the FP64 oracle to
    <= 1e-3 mean per-channel error.  A render asked to skip the projection
    is refused."""
    N = sgx._native
    u = _scene(sgx, 96, 54, spp=4)
    rng = np.random.default_rng(5)
    n = 4096
    gx = rng.integers(0, u.width, n).astype(np.uint32)
    gy = rng.integers(0, u.height, n).astype(np.uint32)
    s = rng.integers(0, 4, n).astype(np.uint32)
    on, _, t_on = renderer.trace_samples(u, gx, gy, s, _opts(sgx, "mixed"))
    o = _opts(sgx, "mixed")
    o.projection = 0
    off, _, t_off = renderer.trace_samples(u, gx, gy, s, o)
    close = np.all(np.abs(on - off) <= np.maximum(1e-5, 1e-3 * np.maximum(np.abs(on), np.abs(off))), axis=1)
    print(f"projection on vs off: same termination {(t_on == t_off).mean():.4f}, close {close.mean():.4f}")
    assert ((t_on == t_off) & close).mean() >= SAMPLE_FRAC
    img = renderer.render_image(u, _opts(sgx, "mixed"), fmt=N.FORMAT_RGBA32F)[..., :3].astype(np.float64)
    _, ldr64 = oracle.render(u, "f64", adaptive=oracle.adaptive_opts())
    assert np.abs(img - ldr64).mean() <= 1e-3
    with pytest.raises(sgx.SgxError):
        renderer.render(u, o)


def test_invariants_and_projection_options_are_checked(renderer, sgx):
    """sgx_trace_invariants reports the error-controlled Kerr form only (the
    fixed step or Schwarzschild uniforms are refused); an empty sample list
    is a no-op; a batch refuses projection = 0 like a render."""
    N = sgx._native
    u = _scene(sgx, 16, 16, spp=1)
    gx = np.zeros(4, np.uint32)
    with pytest.raises(sgx.SgxError):
        renderer.trace_invariants(u, gx, gx, gx, sgx.default_opts())  # fixed step
    sc = sgx.Scene(metric=sgx.MetricType.Schwarzschild, spin_a_over_M=0.0, disc_inner_M=6.0, disc_outer_M=20.0)
    us = sgx.pack_uniforms(sc, sgx.build_orbital_camera(30.0, 0.2, 0.0, 40.0), 16, 16)
    with pytest.raises(sgx.SgxError):
        renderer.trace_invariants(us, gx, gx, gx, _opts(sgx, "f32"))
    inv, term = renderer.trace_invariants(u, gx[:0], gx[:0], gx[:0], _opts(sgx, "f32"))
    assert inv.shape == (0, 5) and term.shape == (0,)
    o = _opts(sgx, "f32")
    o.projection = 0
    with pytest.raises(sgx.SgxError):
        sgx.Batch(renderer, [u, u], o)
    o.projection = 1
    o.slice_count, o.slice_index = 2, 0
    with pytest.raises(sgx.SgxError):
        sgx.Batch(renderer, [u, u], o)
