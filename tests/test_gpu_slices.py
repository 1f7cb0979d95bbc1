"""One frame split into row slices (the multi-GPU partition of a frame), on
one GPU: each slice rendered through sgx_render_device with opts.slice_*,
then assembled, equals the whole-frame render bit for bit — every pixel is
traced and accumulated exactly as in the whole frame, in the reference's
per-pixel sample order.  The multi-process gather itself is tested with gloo
ranks on the CPU (tests/test_dist.py)."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render_device(sgx, r, u, opts, rows, fmt):
    import torch
    from singularity_gb300 import _native as N
    bpp = 4 if fmt == N.FORMAT_RGBA8_SRGB else 16
    out = torch.zeros(u.width * rows * bpp, dtype=torch.uint8, device="cuda")
    st = N.load().sgx_render_device(r.handle, C.byref(u), C.byref(opts), C.c_void_p(out.data_ptr()), fmt, None)
    assert st == 0, N.load().sgx_last_error(r.handle).decode()
    torch.cuda.synchronize()
    a = out.cpu().numpy()
    return a.reshape(rows, u.width, 4) if bpp == 4 else a.view(np.float32).reshape(rows, u.width, 4)


FORMS = {
    "fixed_f32": dict(),
    "fixed_f64": dict(precision=2),
    "adaptive_mixed": dict(integrator=1, precision=1),
    "adaptive_f32_tiled": dict(integrator=1, precision=0, tile_w=8, tile_h=4),
}


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("count,band", [(2, 8), (3, 5), (8, 1)])
def test_slices_assemble_to_the_whole_frame(renderer, sgx, form, count, band):
    from singularity_gb300 import _native as N
    from singularity_gb300 import dist as D
    isco = sgx.kerr_isco_prograde(1.0, 0.94)
    sc = sgx.Scene(spin_a_over_M=0.94, disc_inner_M=isco, disc_outer_M=30.0, disc_peak_T_K=1e4,
                   render_supersample=4)
    u = sgx.pack_uniforms(sc, sgx.build_orbital_camera(40.0, 0.261799, 0.0, 30.0), 72, 43)
    fmt = N.FORMAT_RGBA32F if form == "fixed_f64" else N.FORMAT_RGBA8_SRGB
    whole = _render_device(sgx, renderer, u, sgx.default_opts(**FORMS[form]), u.height, fmt)
    parts = []
    for i in range(count):
        o = sgx.default_opts(slice_count=count, slice_index=i, slice_band=band, **FORMS[form])
        rows = D.slice_rows(u.height, band, count, i)
        parts.append(_render_device(sgx, renderer, u, o, rows, fmt))
        st = renderer.stats()
        assert st.rays == u.width * rows * 4
    np.testing.assert_array_equal(D.assemble_slices(parts, u.height, band), whole)


def test_slice_with_progressive_passes(renderer, sgx):
    """A slice rendered in progressive sample passes equals the slice in one pass."""
    from singularity_gb300 import _native as N
    from singularity_gb300 import dist as D
    u = sgx.workloads.kerr_1080p_16spp()
    u.width, u.height, u.supersample = 160, 90, 8
    base = dict(integrator=1, precision=1, slice_count=4, slice_index=1, slice_band=8)
    rows = D.slice_rows(u.height, 8, 4, 1)
    one = _render_device(sgx, renderer, u, sgx.default_opts(**base), rows, N.FORMAT_RGBA8_SRGB)
    for b in (0, 3, 6):
        o = sgx.default_opts(sample_begin=b, sample_count=3, **base)
        got = _render_device(sgx, renderer, u, o, rows, N.FORMAT_RGBA8_SRGB)
    np.testing.assert_array_equal(got, one)


def test_slice_options_are_checked(renderer, sgx):
    u = sgx.workloads.kerr_1080p_16spp()
    u.width, u.height, u.supersample = 16, 16, 1
    with pytest.raises(sgx.SgxError):
        renderer.render(u, sgx.default_opts(slice_count=2, slice_index=0))  # slices go through sgx_render_device
    import torch
    from singularity_gb300 import _native as N
    out = torch.zeros(16 * 16 * 4, dtype=torch.uint8, device="cuda")
    lib = N.load()
    for bad in (dict(slice_count=2, slice_index=2), dict(slice_count=3, slice_index=2, slice_band=16)):
        o = sgx.default_opts(**bad)
        st = lib.sgx_render_device(renderer.handle, C.byref(u), C.byref(o), C.c_void_p(out.data_ptr()), 0, None)
        assert st == 1, bad  # index beyond count; a slice with no rows
