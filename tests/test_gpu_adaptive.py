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
