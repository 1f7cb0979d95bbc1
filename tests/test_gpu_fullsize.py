"""Size-independent properties at the benchmark's full size (Kerr a = 0.94,
3840x2160, the precision form): the frame split into 8 slices of 8-row
bands assembles to the whole frame bit for bit, and a frame rendered in
explicit progressive passes equals the one render that the library splits
into passes itself (48 samples of 16-byte records, 6.4 GB, need more than
the 4 GiB per-pass workspace, so it takes two)."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 3840, 2160


def _u(sgx, spp):
    isco = sgx.kerr_isco_prograde(1.0, 0.94)
    sc = sgx.Scene(spin_a_over_M=0.94, disc_inner_M=isco, disc_outer_M=30.0, disc_peak_T_K=1e4,
                   render_supersample=spp)
    return sgx.pack_uniforms(sc, sgx.build_orbital_camera(40.0, 0.261799, 0.0, 30.0), W, H, 7.0 / 30.0)


def _device_render(sgx, renderer, u, opts, rows):
    import torch
    from singularity_gb300 import _native as N
    out = torch.zeros(rows * W * 4, dtype=torch.uint8, device="cuda")
    lib = N.load()
    st = lib.sgx_render_device(renderer.handle, C.byref(u), C.byref(opts), C.c_void_p(out.data_ptr()),
                               N.FORMAT_RGBA8_SRGB, None)
    assert st == 0, lib.sgx_last_error(renderer.handle).decode()
    torch.cuda.synchronize()
    return out.view(rows, W, 4)


def test_4k_slices_assemble_to_the_whole_frame(renderer, sgx):
    from singularity_gb300 import dist as D
    from singularity_gb300 import _native as N
    u = _u(sgx, 16)
    base = dict(integrator=N.INTEGRATOR_ADAPTIVE, precision=N.PRECISION_MIXED)
    whole = _device_render(sgx, renderer, u, sgx.default_opts(**base), H).cpu()
    parts = []
    for i in range(8):
        o = sgx.default_opts(slice_count=8, slice_index=i, slice_band=8, **base)
        parts.append(_device_render(sgx, renderer, u, o, D.slice_rows(H, 8, 8, i)).cpu())
    assert all(p.shape[0] in (264, 272) for p in parts)
    assert bool((D.assemble_slices(parts, H, 8) == whole).all())


def test_4k_progressive_passes_equal_the_split_render(renderer, sgx):
    from singularity_gb300 import _native as N
    u = _u(sgx, 48)
    base = dict(integrator=N.INTEGRATOR_ADAPTIVE, precision=N.PRECISION_MIXED)
    one = renderer.render_image(u, sgx.default_opts(**base))
    assert renderer.stats().rays == W * H * 48  # counters summed over the library's passes
    for b in range(0, 48, 16):
        renderer.render(u, sgx.default_opts(sample_begin=b, sample_count=16, **base))
    np.testing.assert_array_equal(renderer.capture(), one)
