"""The named scenes of the benchmark configurations, as uniform blocks.

All synthetic and procedural (the reference has no dataset).  Inclination i
maps to the orbital camera's elevation pi/2 - i at azimuth 0; anything not
stated keeps the reference defaults (exposure 1.8, turbulence 0.5, escape
200 M, capture 1.02 r_+).
"""

from __future__ import annotations

import math

import numpy as np

from . import backend as B


# Band-phase seed of the disc turbulence (the reference has no seed): seed s
# renders the bands at time s / 30 s, the phase the reference's 1/30 s frame
# clock reaches at frame s (cuda_backend.cu:149-151).
TURBULENCE_SEED = 7


def turbulence_time(seed: int = TURBULENCE_SEED) -> float:
    return seed / 30.0


def _kerr(spin, r_obs, incl_deg, fov_deg, w, h, spp, peak_T=1e4, r_out=30.0, r_in=None, max_steps=0, time_sec=0.0):
    isco = B.kerr_isco_prograde(1.0, spin)
    sc = B.Scene(spin_a_over_M=spin, disc_inner_M=isco if r_in is None else r_in, disc_outer_M=r_out,
                 disc_peak_T_K=peak_T, render_supersample=spp, max_steps=max_steps)
    cam = B.build_orbital_camera(r_obs, math.pi / 2 - math.radians(incl_deg), 0.0, fov_deg)
    return B.pack_uniforms(sc, cam, w, h, time_sec)


def schwarzschild_256():
    """Schwarzschild (a = 0), 256x256, 1 spp at pixel centres, fixed step h = 0.05, 4000 steps,
    r_obs = 30 M, inclination 80 deg, FOV 40 deg, disc 6-20 M, Doppler and redshift on."""
    sc = B.Scene(metric=B.MetricType.Schwarzschild, spin_a_over_M=0.0, disc_inner_M=6.0, disc_outer_M=20.0,
                 render_supersample=1, h_step=0.05, max_steps=4000)
    cam = B.build_orbital_camera(30.0, math.pi / 2 - math.radians(80.0), 0.0, 40.0)
    return B.pack_uniforms(sc, cam, 256, 256, 0.0)


def kerr_1080p_16spp(seed: int = TURBULENCE_SEED):
    """Kerr a = 0.94, 1920x1080, 16 spp, r_obs 40 M, i = 75 deg, FOV 30, disc ISCO-30 M, 1e4 K,
    turbulence band phase of seed 7."""
    return _kerr(0.94, 40.0, 75.0, 30.0, 1920, 1080, 16, time_sec=turbulence_time(seed))


def kerr_4k_256spp(seed: int = TURBULENCE_SEED):
    """The 1080p Kerr a = 0.94 scene at 3840x2160 and 256 spp."""
    return _kerr(0.94, 40.0, 75.0, 30.0, 3840, 2160, 256, time_sec=turbulence_time(seed))


def batch_64_views(seed: int = 0):
    """64 square views drawn with numpy.random.default_rng(seed), per view in the
    order side in {128, 192, ..., 1024}, spin U[0, 0.998], inclination U[10, 89] deg,
    r_obs U[20, 60] M, spp in {1..64}; disc ISCO(a)-30 M; FOV 30 deg.
    seed 0 gives 31,272,960 pixels and 1,039,998,976 rays."""
    rng = np.random.default_rng(seed)
    views = []
    for _ in range(64):
        side = 128 + 64 * int(rng.integers(0, 15))
        spin = float(rng.uniform(0.0, 0.998))
        incl = float(rng.uniform(10.0, 89.0))
        r_obs = float(rng.uniform(20.0, 60.0))
        spp = int(rng.integers(1, 65))
        views.append(_kerr(spin, r_obs, incl, 30.0, side, side, spp))
    return views


def differentiation_target(w=512, h=512, spp=4):
    """Parameter-recovery target: a = 0.7, i = 60 deg, disc inner radius ISCO(0.7), temperature scale 1.0."""
    return dict(spin=0.7, incl_deg=60.0, r_in=B.kerr_isco_prograde(1.0, 0.7), t_scale=1.0, w=w, h=h, spp=spp)


def differentiation_guess(w=512, h=512, spp=4):
    """Parameter-recovery initial guess: a = 0.5, i = 50 deg, r_in = 1.2 ISCO(0.5), temperature scale 0.8."""
    return dict(spin=0.5, incl_deg=50.0, r_in=1.2 * B.kerr_isco_prograde(1.0, 0.5), t_scale=0.8, w=w, h=h, spp=spp)


def differentiation_base(w=512, h=512, spp=4, distance=40.0, fov_deg=30.0, h_step=0.2, max_steps=2000):
    """Uniform block of the parameter-recovery scene: camera at 40 M with a 30 degree
    field of view, disc out to 30 M at 10^4 K, step 0.2, 2000 steps.  The
    differentiable form takes spin, inclination, inner radius and temperature
    scale from its parameters, everything else from this block."""
    sc = B.Scene(spin_a_over_M=0.7, disc_outer_M=30.0, disc_peak_T_K=1e4, render_supersample=spp, h_step=h_step,
                 max_steps=max_steps)
    return B.pack_uniforms(sc, B.build_orbital_camera(distance, 0.3, 0.0, fov_deg), w, h)


def differentiation_params(d):
    """(spin, inclination in rad, r_in, t_scale) of a differentiation_target/guess dict."""
    return (d["spin"], math.radians(d["incl_deg"]), d["r_in"], d["t_scale"])
