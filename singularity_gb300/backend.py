"""Python host mirror of the reference's render interface, over the C ABI.

Names, fields and behaviour follow the reference so code written against it
reads the same:

* ``Scene``, ``CameraState``, ``ImageData``, ``RenderConfig``
  — render/include/render_backend.hpp:37-105
* ``build_orbital_camera`` — cuda_cli/main.cpp:68-109
* ``pack_uniforms`` — render/cuda/cuda_backend.cu:45-101
* ``SceneConfig`` / ``load_scene_config_from_file`` — core/include/scene/scene_config.hpp
* ``CudaBackend`` — render/cuda/cuda_backend.{hpp,cu}: initialize / shutdown /
  resize / render_frame / capture_frame / name, with the reference's error
  behaviour (failures print to stderr, ``initialize`` returns False,
  ``capture_frame`` returns an empty ImageData) and its 1/30 s frame clock.

``Renderer`` is the same machinery with exceptions and every option of the
library exposed (precision form, integrator, progressive passes, formats).
All arithmetic that defines the uniform bytes runs in the C++ library so the
packed block equals the reference's bit for bit.
"""

from __future__ import annotations

import ctypes as C
import enum
import sys
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _native as N


class SgxError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{N.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# ---------------------------------------------------------------------------
# Value types (render_backend.hpp:37-105)
# ---------------------------------------------------------------------------
class MetricType(enum.IntEnum):
    Schwarzschild = 0
    Kerr = 1


@dataclass
class RenderConfig:
    width: int = 1280
    height: int = 720
    vsync_enabled: bool = True


@dataclass
class Scene:
    metric: MetricType = MetricType.Kerr
    mass_solar: float = 1.0
    spin_a_over_M: float = 0.6
    disc_inner_M: float = 3.83
    disc_outer_M: float = 25.0
    disc_doppler_on: bool = True
    disc_redshift_on: bool = True
    disc_texture_on: bool = True
    show_overlay: bool = False
    render_supersample: int = 1
    exposure: float = 1.8
    bloom_threshold: float = 0.8
    bloom_strength: float = 0.55
    disc_turbulence: float = 0.5
    disc_peak_T_K: float = 4500.0
    max_steps: int = 0
    h_step: float = 0.0
    adaptive_step_on: bool = False

    def to_c(self) -> N.SceneC:
        s = N.SceneC()
        for name, _ in N.SceneC._fields_:
            v = getattr(self, name)
            setattr(s, name, int(v) if isinstance(v, (bool, enum.IntEnum)) else v)
        return s


@dataclass
class CameraState:
    position: list = field(default_factory=lambda: [0.0, 0.0, 30.0])
    basis: list = field(default_factory=lambda: [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0])
    fov_y_radians: float = 1.047

    def to_c(self) -> N.CameraC:
        c = N.CameraC()
        for i in range(3):
            c.position[i] = self.position[i]
        for i in range(9):
            c.basis[i] = self.basis[i]
        c.fov_y_radians = self.fov_y_radians
        return c


@dataclass
class ImageData:
    pixels_rgba: bytes = b""
    width: int = 0
    height: int = 0

    def as_array(self) -> np.ndarray:
        return np.frombuffer(self.pixels_rgba, dtype=np.uint8).reshape(self.height, self.width, 4)


def build_orbital_camera(distance_M: float, elevation_rad: float, azimuth_rad: float,
                         fov_y_deg: float) -> CameraState:
    lib = N.load()
    c = N.CameraC()
    lib.sgx_build_orbital_camera(C.byref(c), distance_M, elevation_rad, azimuth_rad, fov_y_deg)
    return CameraState(list(c.position), list(c.basis), c.fov_y_radians)


def pack_uniforms(scene: Scene, camera: CameraState, width: int, height: int,
                  time_sec: float = 0.0) -> N.Uniforms:
    lib = N.load()
    u = N.Uniforms()
    s, cam = scene.to_c(), camera.to_c()
    lib.sgx_pack_uniforms(C.byref(s), C.byref(cam), width, height, time_sec, C.byref(u))
    return u


def kerr_isco_prograde(mass: float, spin: float) -> float:
    return float(N.load().sgx_kerr_isco_prograde(mass, spin))


# ---------------------------------------------------------------------------
# .scene files (core/include/scene/scene_config.hpp)
# ---------------------------------------------------------------------------
class SceneLoadStatus(enum.IntEnum):
    Ok = 0
    FileNotFound = 1
    ParseError = 2
    UnknownKey = 3


@dataclass
class SceneConfig:
    mass: float = 1.0
    spin: float = 0.0
    disc_r_inner: float = -1.0
    disc_r_outer: float = 20.0
    disc_doppler_on: bool = True
    disc_redshift_on: bool = True
    camera_fov_deg: float = 60.0
    camera_distance: float = 30.0
    camera_elevation: float = 0.0
    h_step: float = 0.1
    max_steps: int = 5000


@dataclass
class SceneLoadResult:
    status: SceneLoadStatus
    error_line: str
    line_number: int


def _cfg_from_c(c: N.SceneConfigC) -> SceneConfig:
    return SceneConfig(c.mass, c.spin, c.disc_r_inner, c.disc_r_outer, bool(c.disc_doppler_on),
                       bool(c.disc_redshift_on), c.camera_fov_deg, c.camera_distance, c.camera_elevation,
                       c.h_step, c.max_steps)


def _load(fn, arg: bytes) -> tuple[SceneLoadResult, SceneConfig]:
    c = N.SceneConfigC()
    N.load().sgx_scene_config_default(C.byref(c))
    line = C.c_int(0)
    buf = C.create_string_buffer(1024)
    st = fn(arg, C.byref(c), C.byref(line), buf, len(buf))
    return SceneLoadResult(SceneLoadStatus(st), buf.value.decode(errors="replace"), line.value), _cfg_from_c(c)


def load_scene_config_from_file(path: str) -> tuple[SceneLoadResult, SceneConfig]:
    return _load(N.load().sgx_scene_config_load_file, str(path).encode())


def load_scene_config_from_string(text: str) -> tuple[SceneLoadResult, SceneConfig]:
    return _load(N.load().sgx_scene_config_load_string, text.encode())


# ---------------------------------------------------------------------------
# Rendering
# ---------------------------------------------------------------------------
def default_opts(**kw) -> N.RenderOpts:
    o = N.RenderOpts()
    N.load().sgx_render_opts_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(f"unknown render option {k}")
        setattr(o, k, v)
    return o


class Renderer:
    """One device context (sgx_context).  Raises SgxError on failure."""

    def __init__(self, device: int = -1):
        self._lib = N.load()
        h = C.c_void_p()
        st = self._lib.sgx_create(device, C.byref(h))
        if st != N.SGX_OK:
            raise SgxError(st, "sgx_create failed (is a CUDA device visible?)")
        self._h = h

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sgx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int) -> None:
        if st != N.SGX_OK:
            raise SgxError(st, self._lib.sgx_last_error(self._h).decode(errors="replace"))

    def resize(self, width: int, height: int) -> None:
        self._check(self._lib.sgx_resize(self._h, width, height))

    def render(self, u: N.Uniforms, opts: Optional[N.RenderOpts] = None) -> None:
        self._size = (u.width, u.height)
        self._check(self._lib.sgx_render(self._h, C.byref(u), C.byref(opts) if opts is not None else None))

    def capture(self, fmt: int = N.FORMAT_RGBA8_SRGB) -> np.ndarray:
        w, h = self._size
        if fmt == N.FORMAT_RGBA8_SRGB:
            out = np.empty((h, w, 4), dtype=np.uint8)
        elif fmt == N.FORMAT_RGBA32F:
            out = np.empty((h, w, 4), dtype=np.float32)
        else:
            out = np.empty((h, w, 4), dtype=np.float16)
        self._check(self._lib.sgx_capture(self._h, out.ctypes.data_as(C.c_void_p), out.nbytes, fmt))
        return out

    def render_image(self, u: N.Uniforms, opts: Optional[N.RenderOpts] = None,
                     fmt: int = N.FORMAT_RGBA8_SRGB) -> np.ndarray:
        self.render(u, opts)
        return self.capture(fmt)

    def bloom(self, sigma_px: float = 0.0, threshold: float = -1.0, strength: float = -1.0,
              fmt: int = N.FORMAT_RGBA8_SRGB) -> np.ndarray:
        """Bloom + ACES on the last frame (rendered with FORMAT_RGBA16F_HDR)."""
        o = N.BloomOpts(C.sizeof(N.BloomOpts), sigma_px, threshold, strength, fmt)
        self._check(self._lib.sgx_bloom(self._h, C.byref(o)))
        return self.capture(fmt)

    def stats(self) -> N.RenderStats:
        s = N.RenderStats()
        self._check(self._lib.sgx_get_stats(self._h, C.byref(s)))
        return s

    def trace_samples(self, u: N.Uniforms, gx, gy, s, opts: Optional[N.RenderOpts] = None):
        """Per-sample HDR colour, steps and termination (parity probe)."""
        gx = np.ascontiguousarray(gx, dtype=np.uint32)
        gy = np.ascontiguousarray(gy, dtype=np.uint32)
        s = np.ascontiguousarray(s, dtype=np.uint32)
        n = gx.size
        hdr = np.zeros((n, 3), dtype=np.float32)
        steps = np.zeros(n, dtype=np.uint32)
        term = np.zeros(n, dtype=np.uint32)
        u32 = C.POINTER(C.c_uint32)
        f32 = C.POINTER(C.c_float)
        self._check(self._lib.sgx_trace_samples(
            self._h, C.byref(u), C.byref(opts) if opts is not None else None, n,
            gx.ctypes.data_as(u32), gy.ctypes.data_as(u32), s.ctypes.data_as(u32),
            hdr.ctypes.data_as(f32), steps.ctypes.data_as(u32), term.ctypes.data_as(u32)))
        return hdr, steps, term

    def trace_invariants(self, u: N.Uniforms, gx, gy, s, opts: Optional[N.RenderOpts] = None):
        """Constants of motion of listed samples of the error-controlled form:
        (n, 5) float64 [E, L_z, Q0, Q_end, 2H_end] and the termination kinds."""
        gx = np.ascontiguousarray(gx, dtype=np.uint32)
        gy = np.ascontiguousarray(gy, dtype=np.uint32)
        s = np.ascontiguousarray(s, dtype=np.uint32)
        n = gx.size
        inv = np.zeros((n, 5), dtype=np.float64)
        term = np.zeros(n, dtype=np.uint32)
        u32 = C.POINTER(C.c_uint32)
        self._check(self._lib.sgx_trace_invariants(
            self._h, C.byref(u), C.byref(opts) if opts is not None else None, n,
            gx.ctypes.data_as(u32), gy.ctypes.data_as(u32), s.ctypes.data_as(u32),
            inv.ctypes.data_as(C.POINTER(C.c_double)), term.ctypes.data_as(u32)))
        return inv, term


def carter_drift(inv: np.ndarray, spin_a: float) -> np.ndarray:
    """|Q_end - Q0| / (|Q0| + L^2 + a^2 E^2) per sample from trace_invariants'
    rows (NaN rows, samples without a camera root, dropped)."""
    E, L, Q0, Q1 = inv[:, 0], inv[:, 1], inv[:, 2], inv[:, 3]
    ok = np.isfinite(inv).all(axis=1)
    norm = np.abs(Q0) + L * L + (spin_a * E) ** 2
    return (np.abs(Q1 - Q0) / norm)[ok]


class Batch:
    """Many views in one persistent launch replayed from a CUDA graph (sgx_batch)."""

    def __init__(self, renderer: Renderer, views, opts: Optional[N.RenderOpts] = None,
                 fmt: int = N.FORMAT_RGBA8_SRGB):
        self._r = renderer
        self._lib = renderer._lib
        self.n = len(views)
        self.fmt = fmt
        self._views = (N.Uniforms * self.n)(*views)
        self.sizes = [(v.width, v.height) for v in views]
        h = C.c_void_p()
        st = self._lib.sgx_batch_create(renderer.handle, self._views, self.n,
                                        C.byref(opts) if opts is not None else None, fmt, C.byref(h))
        renderer._check(st)
        self._h = h

    def update(self, views) -> None:
        self._views = (N.Uniforms * self.n)(*views)
        self._r._check(self._lib.sgx_batch_update(self._h, self._views))

    def launch(self, stream_ptr: int = 0) -> None:
        self._r._check(self._lib.sgx_batch_launch(self._h, C.c_void_p(stream_ptr) if stream_ptr else None))

    def wait(self) -> N.RenderStats:
        s = N.RenderStats()
        self._r._check(self._lib.sgx_batch_wait(self._h, C.byref(s)))
        return s

    def output(self):
        ptr = C.c_void_p()
        offs = (C.c_uint64 * (self.n + 1))()
        self._r._check(self._lib.sgx_batch_output(self._h, C.byref(ptr), offs))
        return ptr.value, list(offs)

    def capture(self, view: int) -> np.ndarray:
        w, h = self.sizes[view]
        out = (np.empty((h, w, 4), dtype=np.uint8) if self.fmt == N.FORMAT_RGBA8_SRGB
               else np.empty((h, w, 4), dtype=np.float32))
        self._r._check(self._lib.sgx_batch_capture(self._h, view, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sgx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(renderer: Renderer, views, base: Optional[N.RenderOpts] = None, sample_cap: int = 4):
    """Fastest launch shape for these views (sgx_autotune): (opts, ms)."""
    arr = (N.Uniforms * len(views))(*views)
    best = N.RenderOpts()
    ms = C.c_float()
    renderer._check(renderer._lib.sgx_autotune(renderer.handle, arr, len(views),
                                                C.byref(base) if base is not None else None, sample_cap,
                                                C.byref(best), C.byref(ms)))
    return best, ms.value


class CudaBackend:
    """The reference's CudaBackend (render/cuda/cuda_backend.hpp:17-46)."""

    def __init__(self):
        self._r: Optional[Renderer] = None
        self._w = 0
        self._h = 0
        self._frame_time_sec = 0.0
        self._rendered = False
        self.opts: Optional[N.RenderOpts] = None  # extension: None = reference behaviour

    def name(self) -> str:
        return "CUDA"

    def initialize(self, window=None, config: RenderConfig = RenderConfig()) -> bool:
        self._w, self._h = int(config.width), int(config.height)
        self._frame_time_sec = 0.0
        try:
            if self._r is None:
                self._r = Renderer()
            self._r.resize(self._w, self._h)
        except (SgxError, N.NativeLibraryMissing) as e:
            print(f"singularity CUDA backend: initialize failed: {e}", file=sys.stderr)
            self._r = None
            return False
        return True

    def shutdown(self) -> None:
        if self._r is not None:
            self._r.close()
        self._r = None
        self._w = self._h = 0
        self._rendered = False

    def resize(self, width: int, height: int) -> None:
        if width == self._w and height == self._h:
            return
        self.shutdown()
        self.initialize(None, RenderConfig(width, height))

    def render_frame(self, scene: Scene, camera: CameraState) -> None:
        if self._r is None:
            return
        u = pack_uniforms(scene, camera, self._w, self._h, np.float32(self._frame_time_sec))
        try:
            self._r.render(u, self.opts)
            self._rendered = True
        except SgxError as e:
            print(f"singularity CUDA backend: render failed: {e}", file=sys.stderr)
        self._frame_time_sec = float(np.float32(np.float32(self._frame_time_sec) + np.float32(1.0 / 30.0)))

    def capture_frame(self) -> ImageData:
        out = ImageData(b"", self._w, self._h)
        if self._r is None or not self._rendered:
            return out
        try:
            img = self._r.capture(N.FORMAT_RGBA8_SRGB)
        except SgxError as e:
            print(f"singularity CUDA backend: capture failed: {e}", file=sys.stderr)
            return out
        out.pixels_rgba = img.tobytes()
        return out
