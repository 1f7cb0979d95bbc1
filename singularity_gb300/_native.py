"""ctypes view of the C ABI in include/sgx.h.

The structures below mirror the C structs field for field; `check_layout()`
compares their sizes with the library's own expectations.  Loading fails
loudly when ``libsgx.so`` has not been built: there is no fallback path.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libsgx.so"

SGX_FLAG_DOPPLER_ON = 1 << 0
SGX_FLAG_REDSHIFT_ON = 1 << 1
SGX_FLAG_DISC_ON = 1 << 2
SGX_FLAG_STARFIELD_ON = 1 << 3
SGX_FLAG_ADAPTIVE_STEP = 1 << 4

SGX_METRIC_SCHWARZSCHILD = 0
SGX_METRIC_KERR = 1

SGX_OK = 0
NOALLOC_SCRATCH_BYTES = 64 << 20
SLICE_BAND_DEFAULT = 8
STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
                4: "no frame rendered", 5: "unsupported"}

FORMAT_RGBA8_SRGB = 0
FORMAT_RGBA32F = 1
FORMAT_RGBA16F_HDR = 2

PRECISION_FP32 = 0
PRECISION_MIXED = 1
PRECISION_FP64 = 2

INTEGRATOR_FIXED = 0
INTEGRATOR_ADAPTIVE = 1

TERM_NAMES = {0: "horizon", 1: "escape", 2: "disc", 3: "budget", 4: "cold-disc", 5: "no-root"}


class Vec4(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("w", C.c_float)]


class Uniforms(C.Structure):
    """sgx_uniforms — the reference's 160-byte Uniforms (shared_shader/uniforms.h:54-95)."""

    _fields_ = [
        ("cam_pos", Vec4), ("cam_fwd", Vec4), ("cam_right", Vec4), ("cam_up", Vec4),
        ("mass_M", C.c_float), ("spin_a", C.c_float), ("rs", C.c_float), ("tan_half_fov", C.c_float),
        ("disc_r_inner", C.c_float), ("disc_r_outer", C.c_float), ("disc_peak_T", C.c_float),
        ("aspect", C.c_float),
        ("h_step", C.c_float), ("escape_r", C.c_float), ("horizon_cut", C.c_float), ("time_sec", C.c_float),
        ("width", C.c_uint32), ("height", C.c_uint32), ("metric_type", C.c_uint32), ("flags", C.c_uint32),
        ("max_steps", C.c_uint32), ("frame_index", C.c_uint32), ("supersample", C.c_uint32),
        ("pad_b", C.c_uint32),
        ("exposure", C.c_float), ("bloom_threshold", C.c_float), ("bloom_strength", C.c_float),
        ("disc_turbulence", C.c_float),
    ]

    def copy(self) -> "Uniforms":
        u = Uniforms()
        C.memmove(C.byref(u), C.byref(self), C.sizeof(Uniforms))
        return u

    def to_bytes(self) -> bytes:
        return bytes(C.string_at(C.byref(self), C.sizeof(Uniforms)))


class RenderOpts(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("precision", C.c_uint32), ("integrator", C.c_uint32),
        ("format", C.c_uint32),
        ("tolerance", C.c_float), ("h_init_frac", C.c_float), ("h_max_frac", C.c_float),
        ("fp64_zone", C.c_float),
        ("sample_begin", C.c_uint32), ("sample_count", C.c_uint32), ("block_threads", C.c_uint32),
        ("blocks_per_sm", C.c_uint32), ("refill_interval", C.c_uint32), ("rhs_form", C.c_uint32),
        ("tile_w", C.c_uint32), ("tile_h", C.c_uint32), ("projection", C.c_uint32),
        ("slice_count", C.c_uint32), ("slice_index", C.c_uint32), ("slice_band", C.c_uint32),
    ]


class RenderStats(C.Structure):
    _fields_ = [
        ("rays", C.c_uint64), ("steps", C.c_uint64), ("rejected", C.c_uint64), ("zone_steps", C.c_uint64),
        ("budget_hits", C.c_uint64), ("trace_ms", C.c_float), ("total_ms", C.c_float),
    ]


class SceneC(C.Structure):
    """sgx_scene — the reference's Scene (render/include/render_backend.hpp:46-82)."""

    _fields_ = [
        ("metric", C.c_uint32), ("mass_solar", C.c_float), ("spin_a_over_M", C.c_float),
        ("disc_inner_M", C.c_float), ("disc_outer_M", C.c_float),
        ("disc_doppler_on", C.c_uint32), ("disc_redshift_on", C.c_uint32), ("disc_texture_on", C.c_uint32),
        ("show_overlay", C.c_uint32), ("render_supersample", C.c_uint32),
        ("exposure", C.c_float), ("bloom_threshold", C.c_float), ("bloom_strength", C.c_float),
        ("disc_turbulence", C.c_float), ("disc_peak_T_K", C.c_float),
        ("max_steps", C.c_uint32), ("h_step", C.c_float), ("adaptive_step_on", C.c_uint32),
    ]


class CameraC(C.Structure):
    """sgx_camera — the reference's CameraState (render_backend.hpp:84-99)."""

    _fields_ = [("position", C.c_float * 3), ("basis", C.c_float * 9), ("fov_y_radians", C.c_float)]


class SceneConfigC(C.Structure):
    """sgx_scene_config — the reference's SceneConfig (core/include/scene/scene_config.hpp:39-58)."""

    _fields_ = [
        ("mass", C.c_float), ("spin", C.c_float), ("disc_r_inner", C.c_float), ("disc_r_outer", C.c_float),
        ("disc_doppler_on", C.c_uint32), ("disc_redshift_on", C.c_uint32),
        ("camera_fov_deg", C.c_float), ("camera_distance", C.c_float), ("camera_elevation", C.c_float),
        ("h_step", C.c_float), ("max_steps", C.c_int32),
    ]


class BloomOpts(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("sigma_px", C.c_float), ("threshold", C.c_float),
                ("strength", C.c_float), ("format", C.c_uint32)]


class DiffParams(C.Structure):
    _fields_ = [("spin", C.c_double), ("incl", C.c_double), ("r_in", C.c_double), ("t_scale", C.c_double)]


class DiffOpts(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("precision", C.c_uint32), ("edge_width", C.c_float),
                ("fade_start", C.c_float), ("fade_width", C.c_float), ("model", C.c_uint32),
                ("half_thickness", C.c_float), ("tau_perp", C.c_float), ("adjoint_form", C.c_uint32),
                ("checkpoint_interval", C.c_uint32)]


DIFF_MODEL_CROSSING, DIFF_MODEL_SLAB = 0, 1
DIFF_ADJOINT_REVERSE, DIFF_ADJOINT_DUAL = 0, 1


_P = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_F32P = C.POINTER(C.c_float)

# (name, restype, argtypes) for every symbol in include/sgx.h.
SIGNATURES = [
    ("sgx_abi_version", C.c_int, []),
    ("sgx_status_string", C.c_char_p, [C.c_int]),
    ("sgx_render_opts_default", None, [C.POINTER(RenderOpts)]),
    ("sgx_scene_default", None, [C.POINTER(SceneC)]),
    ("sgx_build_orbital_camera", None, [C.POINTER(CameraC), C.c_float, C.c_float, C.c_float, C.c_float]),
    ("sgx_pack_uniforms", None, [C.POINTER(SceneC), C.POINTER(CameraC), C.c_uint32, C.c_uint32, C.c_float,
                                 C.POINTER(Uniforms)]),
    ("sgx_scene_config_default", None, [C.POINTER(SceneConfigC)]),
    ("sgx_scene_config_load_file", C.c_int, [C.c_char_p, C.POINTER(SceneConfigC), C.POINTER(C.c_int),
                                             C.c_char_p, C.c_size_t]),
    ("sgx_scene_config_load_string", C.c_int, [C.c_char_p, C.POINTER(SceneConfigC), C.POINTER(C.c_int),
                                               C.c_char_p, C.c_size_t]),
    ("sgx_kerr_isco_prograde", C.c_float, [C.c_float, C.c_float]),
    ("sgx_create", C.c_int, [C.c_int, C.POINTER(_P)]),
    ("sgx_destroy", None, [_P]),
    ("sgx_resize", C.c_int, [_P, C.c_uint32, C.c_uint32]),
    ("sgx_render", C.c_int, [_P, C.POINTER(Uniforms), C.POINTER(RenderOpts)]),
    ("sgx_capture", C.c_int, [_P, _P, C.c_size_t, C.c_uint32]),
    ("sgx_get_stats", C.c_int, [_P, C.POINTER(RenderStats)]),
    ("sgx_last_error", C.c_char_p, [_P]),
    ("sgx_render_device", C.c_int, [_P, C.POINTER(Uniforms), C.POINTER(RenderOpts), _P, C.c_uint32, _P]),
    ("sgx_render_noalloc", C.c_int, [C.POINTER(Uniforms), C.POINTER(RenderOpts), _P, C.c_uint32, _P, C.c_char_p,
                                     C.c_size_t]),
    ("sgx_bloom", C.c_int, [_P, C.POINTER(BloomOpts)]),
    ("sgx_batch_create", C.c_int, [_P, C.POINTER(Uniforms), C.c_uint32, C.POINTER(RenderOpts), C.c_uint32,
                                   C.POINTER(_P)]),
    ("sgx_batch_update", C.c_int, [_P, C.POINTER(Uniforms)]),
    ("sgx_batch_launch", C.c_int, [_P, _P]),
    ("sgx_batch_wait", C.c_int, [_P, C.POINTER(RenderStats)]),
    ("sgx_batch_output", C.c_int, [_P, C.POINTER(_P), C.POINTER(C.c_uint64)]),
    ("sgx_batch_capture", C.c_int, [_P, C.c_uint32, _P, C.c_size_t]),
    ("sgx_batch_destroy", None, [_P]),
    ("sgx_autotune", C.c_int, [_P, C.POINTER(Uniforms), C.c_uint32, C.POINTER(RenderOpts), C.c_uint32,
                               C.POINTER(RenderOpts), C.POINTER(C.c_float)]),
    ("sgx_diff_opts_default", None, [C.POINTER(DiffOpts)]),
    ("sgx_diff_forward", C.c_int, [_P, C.POINTER(Uniforms), C.POINTER(DiffParams), C.POINTER(DiffOpts), _P, _P]),
    ("sgx_diff_backward", C.c_int, [_P, _P, C.POINTER(C.c_double), _P]),
    ("sgx_diff_stats", C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("sgx_diff_checkpoint_steps", C.c_uint32, [_P]),
    ("sgx_measure_fp32_peak", C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
    ("sgx_trace_samples", C.c_int, [_P, C.POINTER(Uniforms), C.POINTER(RenderOpts), C.c_uint64, _U32P, _U32P,
                                    _U32P, _F32P, _U32P, _U32P]),
    ("sgx_trace_invariants", C.c_int, [_P, C.POINTER(Uniforms), C.POINTER(RenderOpts), C.c_uint64, _U32P, _U32P,
                                       _U32P, C.POINTER(C.c_double), _U32P]),
    ("sgx_slice_rows", C.c_uint32, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
    ("sgx_slice_row", C.c_uint32, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
]

_lib = None


class NativeLibraryMissing(RuntimeError):
    pass


def load() -> C.CDLL:
    """Load libsgx.so (built by singularity_gb300.build); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise NativeLibraryMissing(
            f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(LIB_PATH))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check_layout() -> None:
    assert C.sizeof(Uniforms) == 160, C.sizeof(Uniforms)
    assert Uniforms.exposure.offset == 144
    assert Uniforms.max_steps.offset == 128


check_layout()
