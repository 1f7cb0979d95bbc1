"""Pins of the CPU oracle against the reference (no GPU).

* bit-exact against the reference kernel source compiled for the host
  (committed vectors from tests/golden/make_golden.py, plus live comparisons
  on random scenes where the reference tree is present);
* the reference's own CUDA goldens by the pHash rule of
  verification/test_cuda_goldens.py:32 (distance <= 4);
* the .scene loader and the orbital camera against the reference's code.
"""

from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, uniforms_from_bytes
from imgmetrics import phash_distance


def test_oracle_bit_exact_against_reference_host_vectors(oracle, host_vectors):
    z, names = host_vectors
    assert len(names) >= 9
    for name in names:
        u = uniforms_from_bytes(z[f"{name}_uniforms"])
        rgba, _ = oracle.render(u)
        np.testing.assert_array_equal(rgba, z[f"{name}_rgba8"], err_msg=name)
        hdr, _, _ = oracle.trace(u, z[f"{name}_gx"], z[f"{name}_gy"], z[f"{name}_s"])
        ref = z[f"{name}_hdr"]
        assert np.array_equal(hdr.view(np.uint32), ref.view(np.uint32)), name


def _random_uniforms(rng, sgx):
    metric = sgx.MetricType(int(rng.integers(0, 2)))
    spin = 0.0 if metric == sgx.MetricType.Schwarzschild else float(rng.uniform(0.0, 0.99))
    sc = sgx.Scene(metric=metric, spin_a_over_M=spin, disc_inner_M=float(rng.uniform(1.5, 7)),
                   disc_outer_M=float(rng.uniform(10, 35)), disc_peak_T_K=float(rng.uniform(2000, 30000)),
                   render_supersample=int(rng.integers(1, 5)), disc_doppler_on=bool(rng.integers(0, 2)),
                   disc_redshift_on=bool(rng.integers(0, 2)), disc_turbulence=float(rng.uniform(0, 1)),
                   exposure=float(rng.uniform(0.5, 3)), max_steps=int(rng.integers(200, 1500)),
                   h_step=float(rng.uniform(0.1, 0.6)))
    cam = sgx.build_orbital_camera(float(rng.uniform(12, 45)), float(rng.uniform(-1.4, 1.4)),
                                   float(rng.uniform(0, 6.28)), float(rng.uniform(20, 90)))
    return sgx.pack_uniforms(sc, cam, int(rng.integers(4, 24)), int(rng.integers(4, 24)),
                             float(rng.uniform(0, 3)))


def test_oracle_bit_exact_against_reference_live(oracle, sgx):
    if not oracle.ref_available():
        pytest.skip("reference sources not present on this host (pinned by the committed vectors instead)")
    rng = np.random.default_rng(7)
    for _ in range(12):
        u = _random_uniforms(rng, sgx)
        np.testing.assert_array_equal(oracle.render(u)[0], oracle.ref_render(u))


def test_oracle_against_reference_cuda_goldens(oracle, cuda_goldens):
    """The reference's golden rule: pHash distance <= 4 against its CUDA goldens.

    The committed Kerr goldens agree with the current reference source
    (distance 2).  `schw.png` predates the current default scene (a Kerr
    a = 0.6 scene since render_backend.hpp:52-55, rendered with a hotter disc
    and a lighter sky); the current reference source itself, reproduced bit
    for bit by the oracle, lies far from it, so only its distance is recorded.
    """
    d = {}
    for name in ("schw", "kerr_a05", "kerr_a094"):
        u = uniforms_from_bytes(cuda_goldens[f"{name}_uniforms"])
        rgba, _ = oracle.render(u)
        d[name] = phash_distance(rgba, cuda_goldens[f"{name}_rgba8"])
    assert d["kerr_a05"] <= 4, d
    assert d["kerr_a094"] <= 4, d
    assert d["schw"] > 4, d  # stale golden, see docstring


def test_scene_loader_matches_reference(sgx):
    cases = json.loads((GOLDEN / "reference_host_scene_cases.json").read_text())["scene_texts"]
    for key, c in cases.items():
        res, cfg = sgx.load_scene_config_from_string(c["text"])
        assert int(res.status) == c["status"], key
        assert res.line_number == c["line"], key
        got = [cfg.mass, cfg.spin, cfg.disc_r_inner, cfg.disc_r_outer, float(cfg.disc_doppler_on),
               float(cfg.disc_redshift_on), cfg.camera_fov_deg, cfg.camera_distance, cfg.camera_elevation,
               cfg.h_step, float(cfg.max_steps)]
        np.testing.assert_array_equal(np.float32(got), np.float32(c["fields"]), err_msg=key)


def test_scene_loader_file_not_found(sgx, tmp_path):
    res, _ = sgx.load_scene_config_from_file(str(tmp_path / "missing.scene"))
    assert res.status == sgx.SceneLoadStatus.FileNotFound
    assert res.line_number == 0
    assert res.error_line.endswith("missing.scene")


def test_orbital_camera_matches_reference(sgx):
    cams = json.loads((GOLDEN / "reference_host_scene_cases.json").read_text())["orbital_camera"]
    for c in cams:
        cam = sgx.build_orbital_camera(*c["args"])
        got = np.float32(cam.position + cam.basis + [cam.fov_y_radians])
        np.testing.assert_array_equal(got, np.float32(c["out"]), err_msg=str(c["args"]))


def test_pack_uniforms_reference_defaults(sgx):
    """pack_uniforms_cuda (cuda_backend.cu:45-101) defaults and derived fields."""
    cam = sgx.build_orbital_camera(30.0, 0.15, 0.0, 60.0)
    u = sgx.pack_uniforms(sgx.Scene(), cam, 256, 128, 0.25)
    assert u.metric_type == 1 and u.width == 256 and u.height == 128
    assert u.h_step == np.float32(0.4) and u.max_steps == 2500
    assert u.escape_r == 200.0 and u.horizon_cut == np.float32(1.02) * np.float32(2.0)
    assert u.flags == 0b1111  # STARFIELD | DISC | DOPPLER | REDSHIFT
    assert u.supersample == 1 and u.frame_index == 0 and u.pad_b == 0
    assert u.spin_a == np.float32(0.6) and u.rs == 2.0
    assert u.aspect == np.float32(2.0) and u.time_sec == np.float32(0.25)
    assert u.tan_half_fov == np.float32(np.tan(np.float32(0.5) * np.float32(cam.fov_y_radians)))
    assert (u.cam_fwd.x, u.cam_fwd.y, u.cam_fwd.z) == tuple(-np.float32(cam.basis[6:9]))
    assert u.exposure == np.float32(1.8) and u.disc_turbulence == np.float32(0.5)
    assert u.disc_peak_T == 4500.0 and u.disc_r_inner == np.float32(3.83)
    # Scene overrides and flags off.
    sc = sgx.Scene(metric=sgx.MetricType.Schwarzschild, h_step=0.05, max_steps=4000, render_supersample=0,
                   disc_texture_on=False, disc_doppler_on=False, disc_redshift_on=True, mass_solar=2.0)
    u = sgx.pack_uniforms(sc, cam, 8, 8)
    assert u.metric_type == 0 and u.h_step == np.float32(0.05) and u.max_steps == 4000
    assert u.supersample == 1 and u.flags == (8 | 2)
    assert u.escape_r == 400.0 and u.rs == 4.0 and u.disc_r_outer == 50.0


def test_isco_known_answers(sgx):
    """kerr_isco_prograde limits (tests/test_kerr.cpp: a=0 -> 6M, a=M -> M)."""
    assert sgx.kerr_isco_prograde(1.0, 0.0) == pytest.approx(6.0, abs=1e-5)
    assert sgx.kerr_isco_prograde(1.0, 1.0) == pytest.approx(1.0, abs=1e-3)
    assert sgx.kerr_isco_prograde(1.0, 0.94) == pytest.approx(2.023593, abs=2e-5)
    assert sgx.kerr_isco_prograde(1.0, 0.7) == pytest.approx(3.393129, abs=2e-5)
    assert sgx.kerr_isco_prograde(2.0, 0.0) == pytest.approx(12.0, abs=1e-4)


def test_reference_arm_uniforms_equal_the_product_packing(sgx, oracle):
    """The reference arm of bench.py builds its uniform block with the
    reference's own orbital camera, ISCO and Scene defaults and the harness's
    restatement of pack_uniforms_cuda (render/cuda/cuda_backend.cu:45-101), no
    product code; it is byte-identical to the product's sgx_pack_uniforms for
    the benchmark scene and for the reference's default scene."""
    import ctypes as C
    if not oracle.ref_available():
        pytest.skip("the host build of the reference kernel is not present")
    ref = oracle.ref_headline_uniforms(3840, 2160, 256, 7.0 / 30.0)
    isco = sgx.kerr_isco_prograde(1.0, 0.94)
    assert oracle.ref_isco_prograde(1.0, 0.94) == isco
    prod = sgx.pack_uniforms(sgx.Scene(spin_a_over_M=0.94, disc_inner_M=isco, disc_outer_M=30.0,
                                       disc_peak_T_K=1e4, render_supersample=256),
                             sgx.build_orbital_camera(40.0, 0.261799, 0.0, 30.0), 3840, 2160, 7.0 / 30.0)
    assert bytes(C.string_at(C.byref(ref), 160)) == prod.to_bytes()
    cam = oracle.ref_orbital_camera(30.0, 0.15, 0.0, 60.0)
    for w, h in ((256, 256), (1280, 720)):
        ref = oracle.ref_pack_uniforms(oracle.ref_scene(), cam, w, h)
        prod = sgx.pack_uniforms(sgx.Scene(), sgx.build_orbital_camera(30.0, 0.15, 0.0, 60.0), w, h)
        assert bytes(C.string_at(C.byref(ref), 160)) == prod.to_bytes()
