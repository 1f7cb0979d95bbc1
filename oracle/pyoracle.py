"""TEST INFRASTRUCTURE — ctypes front end of the CPU oracle.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module, and only as the checker.  It loads:

* ``oracle/_build/liboracle.so`` — the restatement (geodesic_oracle.hpp,
  adaptive_oracle.hpp), built by ``make -C oracle``;
* ``oracle/_ref/libref_host.so`` — the reference's own kernel source compiled
  for the host CPU (``make -C oracle ref``), present only where the reference
  sources are.

Where the reference sources are: ``reference_root()`` — the checkout named by
the environment variable SGX_REFERENCE_ROOT; else the snapshot
``oracle/_ref/src`` that ``make -C oracle snapshot`` leaves beside the
builds (the reference files the recipes compile, so that a machine without the
checkout, such as the GPU host, can build them).
"""

from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_host.so"
SNAPSHOT = HERE / "_ref" / "src"


def _has_sources(root: Path) -> bool:
    return (root / "render" / "cuda" / "kernels" / "geodesic_kernel.cu").exists()


def reference_checkout() -> Path | None:
    """The full checkout of the reference named by SGX_REFERENCE_ROOT, if any."""
    env = os.environ.get("SGX_REFERENCE_ROOT")
    if env and _has_sources(Path(env)):
        return Path(env)
    return None


def reference_root() -> Path | None:
    """The reference sources to compile: a checkout, else the snapshot, else None."""
    root = reference_checkout()
    if root is not None:
        return root
    return SNAPSHOT if _has_sources(SNAPSHOT) else None


class AdaptiveOpts(C.Structure):
    _fields_ = [("tol", C.c_float), ("h_init_frac", C.c_float), ("h_max_frac", C.c_float), ("zone", C.c_float),
                ("max_steps", C.c_uint32), ("mixed", C.c_uint32), ("no_early_capture", C.c_uint32),
                ("no_projection", C.c_uint32)]


def adaptive_opts(tol=1e-6, h_init_frac=0.1, h_max_frac=0.1, zone=0.05, max_steps=0, mixed=False,
                  early_capture=True, projection=True) -> "AdaptiveOpts":
    """The adaptive integrator's options (defaults = the library's defaults)."""
    return AdaptiveOpts(tol, h_init_frac, h_max_frac, zone, max_steps, int(bool(mixed)), int(not early_capture),
                        int(not projection))


class RayDiag(C.Structure):
    _fields_ = [("E", C.c_double), ("L", C.c_double), ("Q0", C.c_double), ("Q_end", C.c_double),
                ("H2_end", C.c_double), ("norm_Q", C.c_double), ("accepted", C.c_uint32),
                ("rejected", C.c_uint32), ("zone_steps", C.c_uint32), ("pad", C.c_uint32)]


class DiffParams(C.Structure):
    _fields_ = [("spin", C.c_double), ("incl", C.c_double), ("r_in", C.c_double), ("t_scale", C.c_double)]


class DiffOpts(C.Structure):
    _fields_ = [("eps", C.c_float), ("fade_start", C.c_float), ("fade_width", C.c_float), ("model", C.c_uint32),
                ("half_thickness", C.c_float), ("tau_perp", C.c_float), ("pad0", C.c_float), ("pad1", C.c_float)]


DIFF_MODEL_CROSSING, DIFF_MODEL_SLAB = 0, 1


DIFF_FADE = (0.625 * math.pi, 0.125 * math.pi)  # the library's default winding fade (start, width), rad


def diff_render(u, params, eps: float = 0.1, precision: str = "f64", threads: int | None = None,
                fade=DIFF_FADE, model: int = 1, half_thickness: float = 0.3, tau_perp: float = 4.0) -> np.ndarray:
    """LDR image (H, W, 3) of the differentiable form at params = (spin, incl_rad, r_in, t_scale).
    fade = (start, width) of the winding fade; start <= 0 turns it off."""
    threads = threads or default_threads()
    p = DiffParams(*[float(x) for x in params])
    o = DiffOpts(eps, fade[0], fade[1], model, half_thickness, tau_perp, 0.0, 0.0)
    dt = np.float32 if precision == "f32" else np.float64
    out = np.zeros((u.height, u.width, 3), dtype=dt)
    fn = lib().oracle_diff_render_f32 if precision == "f32" else lib().oracle_diff_render_f64
    rc = fn(_u(u), C.byref(p), C.byref(o), _p(out), C.c_int(threads))
    if rc != 0:
        raise RuntimeError("oracle diff render failed")
    return out


def diff_trace(u, params, gx, gy, s, eps: float = 0.1, fade=DIFF_FADE, model: int = 1, half_thickness: float = 0.3,
               tau_perp: float = 4.0, threads: int | None = None):
    """Per-sample FP64 HDR colour, steps and emitting events of the differentiable form."""
    threads = threads or default_threads()
    gx = np.ascontiguousarray(gx, dtype=np.uint32)
    gy = np.ascontiguousarray(gy, dtype=np.uint32)
    s = np.ascontiguousarray(s, dtype=np.uint32)
    n = gx.size
    p = DiffParams(*[float(x) for x in params])
    o = DiffOpts(eps, fade[0], fade[1], model, half_thickness, tau_perp, 0.0, 0.0)
    hdr = np.zeros((n, 3), dtype=np.float64)
    steps = np.zeros(n, dtype=np.uint32)
    events = np.zeros(n, dtype=np.uint32)
    rc = lib().oracle_diff_trace_f64(_u(u), C.byref(p), C.byref(o), C.c_int64(n), _p(gx), _p(gy), _p(s), _p(hdr),
                                     _p(steps), _p(events), C.c_int(threads))
    if rc != 0:
        raise RuntimeError("oracle diff trace failed")
    return hdr, steps, events


def diff_grad(u, params, dLdI: np.ndarray, eps: float = 0.1, fade=DIFF_FADE, model: int = 1,
              half_thickness: float = 0.3, tau_perp: float = 4.0, threads: int | None = None):
    """FP64 gradient of sum(dLdI * I) w.r.t. (spin, incl, r_in, t_scale) by forward-mode dual
    numbers through the oracle's form, and the FP64 image I."""
    threads = threads or default_threads()
    p = DiffParams(*[float(x) for x in params])
    o = DiffOpts(eps, fade[0], fade[1], model, half_thickness, tau_perp, 0.0, 0.0)
    g = np.ascontiguousarray(dLdI, dtype=np.float64)
    assert g.shape == (u.height, u.width, 3)
    out = np.zeros(4, dtype=np.float64)
    img = np.zeros((u.height, u.width, 3), dtype=np.float64)
    rc = lib().oracle_diff_grad_f64(_u(u), C.byref(p), C.byref(o), _p(g), _p(out), _p(img), C.c_int(threads))
    if rc != 0:
        raise RuntimeError("oracle diff grad failed")
    return out, img


def diff_fd_gradient(u, params, target: np.ndarray, step: float = 1e-3, eps: float = 0.1,
                     precision: str = "f64", fade=DIFF_FADE, **form) -> np.ndarray:
    """Central finite differences (step in each parameter) of mean((I - target)^2)."""
    params = np.asarray(params, dtype=np.float64)
    g = np.zeros(4)
    for k in range(4):
        d = np.zeros(4)
        d[k] = step
        lp = np.mean((diff_render(u, params + d, eps, precision, fade=fade, **form).astype(np.float64) - target) ** 2)
        lm = np.mean((diff_render(u, params - d, eps, precision, fade=fade, **form).astype(np.float64) - target) ** 2)
        g[k] = (lp - lm) / (2 * step)
    return g


def schw_integrate(y8, h_base: float, rs: float, r_out: float, adaptive: bool, budget: int = 400000):
    """FP32 Schwarzschild integration to r > r_out, fixed or radius-adaptive
    step: (final state, steps or -1, max |dE/E|, max |dL/L|)."""
    y = np.ascontiguousarray(y8, dtype=np.float32).copy()
    me, ml = C.c_float(), C.c_float()
    n = lib().oracle_schw_integrate_f32(_p(y), C.c_float(h_base), C.c_float(rs), C.c_float(r_out),
                                        C.c_int(int(adaptive)), C.c_int(budget), C.byref(me), C.byref(ml))
    return y, n, me.value, ml.value


def schw_rk4_n(y8, h: float, rs: float, n: int = 1) -> np.ndarray:
    """n FP32 Schwarzschild RK4 steps of (t, r, theta, phi, u^t, u^r, u^theta, u^phi)."""
    y = np.ascontiguousarray(y8, dtype=np.float32).copy()
    lib().oracle_schw_rk4_n_f32(_p(y), C.c_float(h), C.c_float(rs), C.c_int64(n))
    return y


def kerr_rhs(y6, c5) -> np.ndarray:
    """FP32 Kerr Hamiltonian RHS of (t, r, theta, phi, p_r, p_theta); c5 = (E, L, Q, a, M)."""
    y = np.ascontiguousarray(y6, dtype=np.float32)
    c = np.ascontiguousarray(c5, dtype=np.float32)
    d = np.zeros(6, dtype=np.float32)
    lib().oracle_kerr_rhs_f32(_p(y), _p(c), _p(d))
    return d


def kerr_two_H(r, th, pr, pth, c5) -> float:
    c = np.ascontiguousarray(c5, dtype=np.float32)
    fn = lib().oracle_kerr_two_H_f32
    fn.restype = C.c_float
    return float(fn(C.c_float(r), C.c_float(th), C.c_float(pr), C.c_float(pth), _p(c)))


def kerr_rk4_n(y6, h: float, c5, n: int = 1) -> np.ndarray:
    """n FP32 fixed-step Kerr RK4 steps (with the pole damping)."""
    y = np.ascontiguousarray(y6, dtype=np.float32).copy()
    c = np.ascontiguousarray(c5, dtype=np.float32)
    lib().oracle_kerr_rk4_n_f32(_p(y), C.c_float(h), _p(c), C.c_int64(n))
    return y


def crossing(th_prev: float, th_curr: float):
    """(crossed, frac) of the equatorial-crossing test in FP32."""
    frac = C.c_float()
    x = lib().oracle_crossing_f32(C.c_float(th_prev), C.c_float(th_curr), C.byref(frac))
    return bool(x), frac.value


def build(ref: bool = True) -> None:
    """Compile the oracle, and with ref=True the reference's own kernel source
    for the host and as PTX when its sources exist (refreshing the snapshot
    from a checkout)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if not ref:
        return
    checkout = reference_checkout()
    if checkout is not None:
        subprocess.run(["make", "-s", "-C", str(HERE), "snapshot", f"REFERENCE_ROOT={checkout}"], check=True)
    root = reference_root()
    if root is not None:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REFERENCE_ROOT={root}"], check=True)


def build_relink() -> Path | None:
    """The reference's unmodified cuda_cli/main.cpp compiled against this
    library's CudaBackend shim and linked with libsgx.so (needs the library
    built and the reference sources); None without the sources."""
    root = reference_root()
    if root is None:
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "relink", f"REFERENCE_ROOT={root}"], check=True)
    return HERE / "_ref" / "ref_cuda_cli_relinked"


_lib = None
_ref = {}
REF_RELEASE_LIB = HERE / "_ref" / "libref_host_release.so"


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build(ref=False)
        _lib = C.CDLL(str(LIB))
    return _lib


def ref_available() -> bool:
    return REF_LIB.exists()


def ref_lib(release: bool = False) -> C.CDLL:
    """The reference's kernel source compiled for the host: the exact-flag
    build (parity pins), or with release=True the reference's own Release
    flags, -O3 -ffast-math (CMakeLists.txt:121-122; timing)."""
    key = bool(release)
    if key not in _ref:
        _ref[key] = C.CDLL(str(REF_RELEASE_LIB if release else REF_LIB))
    return _ref[key]


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _u(u) -> C.c_void_p:
    return C.cast(C.pointer(u), C.c_void_p)


def default_threads() -> int:
    return os.cpu_count() or 1


def render(u, precision: str = "f32", pixels: np.ndarray | None = None, threads: int | None = None,
           adaptive: AdaptiveOpts | None = None):
    """RGBA8 image (or the listed pixels) and the LDR mean, as the reference kernel computes them."""
    threads = threads or default_threads()
    npix = u.width * u.height if pixels is None else len(pixels)
    rgba = np.zeros((npix, 4), dtype=np.uint8)
    dt = np.float32 if precision == "f32" else np.float64
    ldr = np.zeros((npix, 3), dtype=dt)
    pix = None if pixels is None else np.ascontiguousarray(pixels, dtype=np.uint32)
    L = lib()
    if adaptive is None:
        fn = L.oracle_render_f32 if precision == "f32" else L.oracle_render_f64
        rc = fn(_u(u), C.c_int64(npix), _p(pix), _p(rgba), _p(ldr), C.c_int(threads))
    else:
        fn = L.oracle_render_adaptive_f32 if precision == "f32" else L.oracle_render_adaptive_f64
        rc = fn(_u(u), C.byref(adaptive), C.c_int64(npix), _p(pix), _p(rgba), _p(ldr), C.c_int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle render failed ({rc})")
    if pixels is None:
        return rgba.reshape(u.height, u.width, 4), ldr.reshape(u.height, u.width, 3)
    return rgba, ldr


def trace(u, gx, gy, s, precision: str = "f32", threads: int | None = None, adaptive: AdaptiveOpts | None = None,
          diag: bool = False):
    """Per-sample HDR colour, steps and termination kind."""
    threads = threads or default_threads()
    gx = np.ascontiguousarray(gx, dtype=np.uint32)
    gy = np.ascontiguousarray(gy, dtype=np.uint32)
    s = np.ascontiguousarray(s, dtype=np.uint32)
    n = gx.size
    dt = np.float32 if precision == "f32" else np.float64
    hdr = np.zeros((n, 3), dtype=dt)
    steps = np.zeros(n, dtype=np.uint32)
    term = np.zeros(n, dtype=np.uint32)
    L = lib()
    if adaptive is None:
        fn = L.oracle_trace_f32 if precision == "f32" else L.oracle_trace_f64
        rc = fn(_u(u), C.c_int64(n), _p(gx), _p(gy), _p(s), _p(hdr), _p(steps), _p(term), C.c_int(threads))
        d = None
    else:
        d = (RayDiag * n)() if diag else None
        fn = L.oracle_trace_adaptive_f32 if precision == "f32" else L.oracle_trace_adaptive_f64
        rc = fn(_u(u), C.byref(adaptive), C.c_int64(n), _p(gx), _p(gy), _p(s), _p(hdr), _p(steps), _p(term),
                d, C.c_int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle trace failed ({rc})")
    if diag:
        return hdr, steps, term, d
    return hdr, steps, term


def count_ops(u, gx, gy, s, adaptive: AdaptiveOpts | None = None):
    """Per-sample algorithmic FP32 operation counts of the reference formulas."""
    gx = np.ascontiguousarray(gx, dtype=np.uint32)
    gy = np.ascontiguousarray(gy, dtype=np.uint32)
    s = np.ascontiguousarray(s, dtype=np.uint32)
    n = gx.size
    ops = np.zeros(n, dtype=np.uint64)
    steps = np.zeros(n, dtype=np.uint32)
    term = np.zeros(n, dtype=np.uint32)
    rc = lib().oracle_count_ops(_u(u), C.c_int64(n), _p(gx), _p(gy), _p(s), _p(ops), _p(steps), _p(term),
                                C.byref(adaptive) if adaptive is not None else None)
    if rc != 0:
        raise RuntimeError("oracle count failed")
    return ops, steps, term


# ---- the reference itself, compiled for the host (present only here) ----
def ref_render(u, threads: int | None = None) -> np.ndarray:
    threads = threads or default_threads()
    out = np.zeros((u.height, u.width, 4), dtype=np.uint8)
    ref_lib().ref_render_rgba8(_u(u), _p(out), C.c_int(threads))
    return out


def ref_trace(u, gx, gy, s, threads: int | None = None, release: bool = False) -> np.ndarray:
    threads = threads or default_threads()
    gx = np.ascontiguousarray(gx, dtype=np.uint32)
    gy = np.ascontiguousarray(gy, dtype=np.uint32)
    s = np.ascontiguousarray(s, dtype=np.uint32)
    hdr = np.zeros((gx.size, 3), dtype=np.float32)
    ref_lib(release).ref_trace_hdr(_u(u), C.c_int64(gx.size), _p(gx), _p(gy), _p(s), _p(hdr), C.c_int(threads))
    return hdr


class RefUniforms(C.Structure):
    """The reference's 160-byte Uniforms block (shared_shader/uniforms.h:54-95)."""

    _fields_ = [("cam_pos", C.c_float * 4), ("cam_fwd", C.c_float * 4), ("cam_right", C.c_float * 4),
                ("cam_up", C.c_float * 4), ("mass_M", C.c_float), ("spin_a", C.c_float), ("rs", C.c_float),
                ("tan_half_fov", C.c_float), ("disc_r_inner", C.c_float), ("disc_r_outer", C.c_float),
                ("disc_peak_T", C.c_float), ("aspect", C.c_float), ("h_step", C.c_float), ("escape_r", C.c_float),
                ("horizon_cut", C.c_float), ("time_sec", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32),
                ("metric_type", C.c_uint32), ("flags", C.c_uint32), ("max_steps", C.c_uint32),
                ("frame_index", C.c_uint32), ("supersample", C.c_uint32), ("pad_b", C.c_uint32),
                ("exposure", C.c_float), ("bloom_threshold", C.c_float), ("bloom_strength", C.c_float),
                ("disc_turbulence", C.c_float)]


# field order of the reference's Scene (render/include/render_backend.hpp:46-82)
REF_SCENE_FIELDS = ("metric", "mass_solar", "spin_a_over_M", "disc_inner_M", "disc_outer_M", "disc_doppler_on",
                    "disc_redshift_on", "disc_texture_on", "show_overlay", "render_supersample", "exposure",
                    "bloom_threshold", "bloom_strength", "disc_turbulence", "disc_peak_T_K", "max_steps", "h_step")


def ref_scene(**fields) -> np.ndarray:
    """The reference's Scene{} defaults with `fields` replaced (metric: 1 Kerr, 0 Schwarzschild)."""
    sc = np.zeros(17, dtype=np.float32)
    ref_lib().ref_scene_default(_p(sc))
    for k, v in fields.items():
        sc[REF_SCENE_FIELDS.index(k)] = float(v)
    return sc


def ref_isco_prograde(mass: float, spin: float) -> float:
    fn = ref_lib().ref_kerr_isco_prograde
    fn.restype = C.c_float
    fn.argtypes = [C.c_float, C.c_float]
    return float(fn(mass, spin))


def ref_pack_uniforms(scene17: np.ndarray, cam13: np.ndarray, width: int, height: int,
                      time_sec: float = 0.0) -> RefUniforms:
    """The uniform block CudaBackend::render_frame packs (render/cuda/cuda_backend.cu:45-101)."""
    u = RefUniforms()
    sc = np.ascontiguousarray(scene17, dtype=np.float32)
    cam = np.ascontiguousarray(cam13, dtype=np.float32)
    ref_lib().ref_pack_uniforms(_p(sc), _p(cam), C.c_uint32(width), C.c_uint32(height), C.c_float(time_sec),
                                C.byref(u))
    return u


def ref_headline_uniforms(width: int = 3840, height: int = 2160, spp: int = 256,
                          time_sec: float = 7.0 / 30.0) -> RefUniforms:
    """The Kerr a/M = 0.94 benchmark scene through the reference's own code: its
    orbital camera at r = 40 M, elevation 0.261799 rad (inclination 75 deg),
    azimuth 0, FOV 30 deg; disc from its prograde ISCO to 30 M at 1e4 K; its
    uniform packing (fixed step h = 0.4, 2500 steps)."""
    isco = ref_isco_prograde(1.0, 0.94)
    sc = ref_scene(metric=1, spin_a_over_M=0.94, disc_inner_M=isco, disc_outer_M=30.0, disc_peak_T_K=1e4,
                   render_supersample=spp)
    return ref_pack_uniforms(sc, ref_orbital_camera(40.0, 0.261799, 0.0, 30.0), width, height, time_sec)


def ref_orbital_camera(distance, elevation, azimuth, fov_deg) -> np.ndarray:
    out = np.zeros(13, dtype=np.float32)
    ref_lib().ref_build_orbital_camera(C.c_float(distance), C.c_float(elevation), C.c_float(azimuth),
                                       C.c_float(fov_deg), _p(out))
    return out


def ref_load_scene_text(text: str):
    out = np.zeros(11, dtype=np.float32)
    line = C.c_int(0)
    st = ref_lib().ref_load_scene_text(text.encode(), _p(out), C.byref(line))
    return st, out, line.value
