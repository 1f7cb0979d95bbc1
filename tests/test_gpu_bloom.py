"""HDR output and the bloom/blit post-process on the GPU against their CPU
restatements (oracle/bloom_oracle.py; the HDR mean against the geodesic
oracle).  Tolerances: HDR mean within half-precision rounding plus the
tracer's FP32 tolerance; post-process within 2e-3 of full scale (half-precision
intermediates, CUDA vs numpy rounding)."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(sgx, w=96, h=54, spp=4):
    isco = sgx.kerr_isco_prograde(1.0, 0.94)
    sc = sgx.Scene(spin_a_over_M=0.94, disc_inner_M=isco, disc_outer_M=30.0, disc_peak_T_K=1e4,
                   render_supersample=spp)
    return sgx.pack_uniforms(sc, sgx.build_orbital_camera(40.0, 0.261799, 0.0, 30.0), w, h)


def test_hdr_mean_matches_oracle(renderer, oracle, sgx):
    N = sgx._native
    u = _scene(sgx)
    hdr = renderer.render_image(u, sgx.default_opts(format=N.FORMAT_RGBA16F_HDR), fmt=N.FORMAT_RGBA16F_HDR)
    assert hdr.dtype == np.float16 and hdr.shape == (54, 96, 4)
    n = u.width * u.height
    gy, gx = np.divmod(np.arange(n, dtype=np.uint32), u.width)
    spp = u.supersample
    sums = np.zeros((n, 3), np.float32)
    for s in range(spp):
        h, _, _ = oracle.trace(u, gx, gy, np.full(n, s, np.uint32))
        sums = sums + h
    mean = (sums * np.float32(1.0 / spp)).reshape(u.height, u.width, 3)
    got = hdr[..., :3].astype(np.float32)
    close = np.abs(got - mean) <= 2e-3 * np.maximum(1.0, np.abs(mean))
    assert close.all(axis=-1).mean() >= 0.98
    assert np.all(hdr[..., 3] == 1.0)


@pytest.mark.parametrize("sigma", [0.0, 8.0, 3.0])
@pytest.mark.parametrize("fmt", [0, 1])
def test_bloom_matches_cpu_restatement(renderer, sgx, sigma, fmt):
    from oracle import bloom_oracle as B
    N = sgx._native
    u = _scene(sgx, 128, 70)
    hdr = renderer.render_image(u, sgx.default_opts(format=N.FORMAT_RGBA16F_HDR), fmt=N.FORMAT_RGBA16F_HDR)
    out = renderer.bloom(sigma_px=sigma, fmt=fmt)
    ref = B.bloom_pipeline(hdr, u.bloom_threshold, u.bloom_strength, u.exposure, sigma)
    if fmt == N.FORMAT_RGBA32F:
        d = np.abs(out[..., :3] - ref)
        print(f"sigma={sigma}: mean {d.mean():.2e} max {d.max():.2e}")
        assert d.mean() <= 2e-4 and d.max() <= 2e-3
    else:
        d = np.abs(out[..., :3].astype(int) - B.to_srgb_u8(ref).astype(int))
        assert d.max() <= 1 and (d == 0).mean() >= 0.98
    # the raw HDR frame stays capturable after the post-process
    np.testing.assert_array_equal(renderer.capture(N.FORMAT_RGBA16F_HDR), hdr)


def test_bloom_spreads_light(renderer, sgx):
    """A wider sigma spreads the disc's glow: more lit pixels far from the disc."""
    N = sgx._native
    u = _scene(sgx, 160, 90)
    renderer.render(u, sgx.default_opts(format=N.FORMAT_RGBA16F_HDR))
    narrow = renderer.bloom(sigma_px=2.0, strength=1.0, fmt=N.FORMAT_RGBA32F)[..., :3].sum()
    wide = renderer.bloom(sigma_px=16.0, strength=1.0, fmt=N.FORMAT_RGBA32F)[..., :3].sum()
    none = renderer.bloom(sigma_px=8.0, strength=0.0, fmt=N.FORMAT_RGBA32F)[..., :3].sum()
    assert none < narrow and abs(wide - narrow) / narrow < 0.5


def test_bloom_errors(renderer, sgx):
    N = sgx._native
    u = _scene(sgx, 32, 18)
    renderer.render(u)  # an LDR frame
    with pytest.raises(sgx.SgxError):
        renderer.bloom()
    renderer.render(u, sgx.default_opts(format=N.FORMAT_RGBA16F_HDR))
    with pytest.raises(sgx.SgxError):  # no composed image yet in RGBA8
        renderer.capture(N.FORMAT_RGBA8_SRGB)
    with pytest.raises(sgx.SgxError):
        renderer.bloom(fmt=N.FORMAT_RGBA16F_HDR)


@pytest.mark.parametrize("w,h,precision", [(128, 70, 0), (97, 55, 0), (64, 37, 2)])
def test_fused_extract_equals_the_separate_pass(renderer, sgx, w, h, precision):
    """An HDR render into the context's image writes the bloom extract in its
    last accumulation pass, so the first sgx_bloom after it blurs and
    composes only; a threshold of the caller's own makes sgx_bloom extract
    again from the stored frame.  Both composites are the same, the fused
    pass's HDR frame equals the plain accumulation's (sgx_render_device into a
    caller buffer, which does not fuse), and progressive passes fuse on their
    last pass.  Odd sizes exercise the pixels outside the 2x2 blocks."""
    import ctypes as C
    import torch
    N = sgx._native
    u = _scene(sgx, w, h, spp=4)
    opts = sgx.default_opts(format=N.FORMAT_RGBA16F_HDR, precision=precision)
    hdr = renderer.render_image(u, opts, fmt=N.FORMAT_RGBA16F_HDR)
    fused = renderer.bloom(sigma_px=8.0, fmt=N.FORMAT_RGBA32F)
    separate = renderer.bloom(sigma_px=8.0, threshold=u.bloom_threshold, fmt=N.FORMAT_RGBA32F)
    np.testing.assert_array_equal(fused, separate)
    again = renderer.bloom(sigma_px=8.0, fmt=N.FORMAT_RGBA32F)  # a second call extracts again
    np.testing.assert_array_equal(again, fused)
    dev = torch.zeros(w * h * 8, dtype=torch.uint8, device="cuda")
    lib = N.load()
    st = lib.sgx_render_device(renderer.handle, C.byref(u), C.byref(opts), C.c_void_p(dev.data_ptr()),
                               N.FORMAT_RGBA16F_HDR, None)
    assert st == 0, lib.sgx_last_error(renderer.handle).decode()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy().view(np.float16).reshape(h, w, 4), hdr)
    for b in (0, 3):
        o = sgx.default_opts(format=N.FORMAT_RGBA16F_HDR, precision=precision, sample_begin=b,
                             sample_count=3 if b == 0 else 1)
        renderer.render(u, o)
    np.testing.assert_array_equal(renderer.capture(N.FORMAT_RGBA16F_HDR), hdr)
    np.testing.assert_array_equal(renderer.bloom(sigma_px=8.0, fmt=N.FORMAT_RGBA32F), fused)
