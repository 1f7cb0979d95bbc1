"""The C-ABI library: loads without a GPU and exports every declared symbol."""

from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(sgx_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(sgx):
    from singularity_gb300 import _native as N
    lib = C.CDLL(str(N.LIB_PATH))
    declared = declared_functions()
    assert len(declared) >= 20
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    bound = {name for name, _, _ in N.SIGNATURES}
    assert declared == bound, (declared ^ bound)


def test_struct_layouts(sgx):
    from singularity_gb300 import _native as N
    assert C.sizeof(N.Uniforms) == 160
    offs = {"cam_pos": 0, "cam_fwd": 16, "cam_right": 32, "cam_up": 48, "mass_M": 64, "spin_a": 68, "rs": 72,
            "tan_half_fov": 76, "disc_r_inner": 80, "disc_r_outer": 84, "disc_peak_T": 88, "aspect": 92,
            "h_step": 96, "escape_r": 100, "horizon_cut": 104, "time_sec": 108, "width": 112, "height": 116,
            "metric_type": 120, "flags": 124, "max_steps": 128, "frame_index": 132, "supersample": 136,
            "pad_b": 140, "exposure": 144, "bloom_threshold": 148, "bloom_strength": 152,
            "disc_turbulence": 156}
    for k, v in offs.items():
        assert getattr(N.Uniforms, k).offset == v, k
    assert C.sizeof(N.RenderOpts) == 80
    assert N.RenderOpts.projection.offset == 64 and N.RenderOpts.slice_band.offset == 76
    o = sgx.default_opts()
    assert o.struct_size == 80 and o.precision == 0 and o.integrator == 0 and o.format == 0
    assert abs(o.tolerance - 1e-6) < 1e-12 and o.sample_count == 0
    # the projection belongs to the (opt-in) error-controlled integrator; no frame slice
    assert o.projection == 1 and o.slice_count == 0 and o.slice_index == 0 and o.slice_band == 0


def test_host_helpers_without_gpu(sgx):
    from singularity_gb300 import _native as N
    lib = N.load()
    assert lib.sgx_abi_version() == 1
    assert lib.sgx_status_string(0) == b"ok"
    s = N.SceneC()
    lib.sgx_scene_default(C.byref(s))
    assert s.metric == 1 and abs(s.spin_a_over_M - 0.6) < 1e-7 and s.render_supersample == 1
    assert abs(s.disc_peak_T_K - 4500.0) < 1e-3


def test_create_fails_cleanly_without_device(sgx):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from singularity_gb300 import _native as N
    h = C.c_void_p()
    st = N.load().sgx_create(0, C.byref(h))
    assert st == 2 and not h.value  # SGX_ERR_CUDA, no context
    with pytest.raises(sgx.SgxError):
        sgx.Renderer()
    be = sgx.CudaBackend()
    assert be.initialize(None, sgx.RenderConfig(8, 8)) is False
    assert be.capture_frame().pixels_rgba == b""
