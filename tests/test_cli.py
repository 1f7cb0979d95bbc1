"""singularity_cuda_cli: flag set, messages and exit codes of the reference's
cuda_cli/main.cpp, and its renders (GPU).  Mirrors the reference's
verification/test_cli_interface.py and test_cuda_goldens.py (multi-frame orbit)."""

from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import uniforms_from_bytes
from imgmetrics import phash_distance, read_png

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="session")
def cli(sgx):
    p = ROOT / "singularity_gb300" / "_build" / "singularity_cuda_cli"
    assert p.exists(), "CLI not built"
    return p


def run(cli, *args, timeout=120):
    return subprocess.run([str(cli), *map(str, args)], capture_output=True, text=True, timeout=timeout)


def test_help(cli):
    r = run(cli, "--help")
    assert r.returncode == 0
    for flag in ("--scene", "--output", "--res", "--samples-per-pixel", "--camera-distance", "--camera-elevation",
                 "--camera-azimuth", "--fov-y-deg", "--frames", "--output-pattern", "--encode-mp4", "--mp4-fps"):
        assert flag in r.stdout, flag


@pytest.mark.parametrize("args,msg", [
    (["--res", "256"], "--res expects WxH, got 256"),
    (["--res", "2x2"], "--res too small"),
    (["--samples-per-pixel", "0"], "--samples-per-pixel must be in [1, 1024]"),
    (["--samples-per-pixel", "1025"], "--samples-per-pixel must be in [1, 1024]"),
    (["--frames", "0"], "--frames must be in [1, 100000]"),
    (["--mp4-fps", "500"], "--mp4-fps must be in [1, 240]"),
    (["--bogus"], "unknown argument: --bogus"),
    (["--frames", "3"], "--frames > 1 requires --output-pattern"),
    (["--frames", "3", "--output-pattern", "frame.png"], "--output-pattern must contain a printf placeholder"),
    (["--encode-mp4", "x.mp4"], "--encode-mp4 requires --frames > 1"),
    (["--integrator", "euler"], "--integrator must be fixed or adaptive"),
    (["--bloom-sigma", "100"], "--bloom-sigma must be in [0, 64]"),
    (["--rhs-form", "3"], "--rhs-form must be 0, 1 or 2"),
])
def test_usage_errors_exit_2(cli, args, msg):
    r = run(cli, *args)
    assert r.returncode == 2, (r.returncode, r.stderr)
    assert msg in r.stderr


def test_scene_errors_exit_2(cli, tmp_path):
    r = run(cli, "--scene", tmp_path / "missing.scene")
    assert r.returncode == 2 and "scene load failed (file-not-found, line 0)" in r.stderr
    bad = tmp_path / "bad.scene"
    bad.write_text("mass = 1\nbogus = 3\n")
    r = run(cli, "--scene", bad)
    assert r.returncode == 2 and "scene load failed (unknown-key, line 2): bogus" in r.stderr
    bad.write_text("spin = x\n")
    r = run(cli, "--scene", bad)
    assert r.returncode == 2 and "parse-error, line 1" in r.stderr


def test_no_gpu_is_a_runtime_error(cli, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run(cli, "--output", tmp_path / "x.png", "--res", "8x8")
    assert r.returncode == 1 and "backend initialize failed" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name,scene", [("schw", None), ("kerr_a05", "kerr_a05.scene"),
                                        ("kerr_a094", "kerr_a094.scene")])
def test_cli_golden_scenes(cli, sgx, renderer, cuda_goldens, tmp_path, name, scene):
    """The reference's golden commands (`--res 256x256 [--scene ...]`): the CLI's PNG
    equals the library render of the same uniforms, and sits at the same pHash
    distance from the reference's golden as the library does."""
    args = ["--output", tmp_path / "o.png", "--res", "256x256"]
    if scene is not None:
        text = {"kerr_a05.scene": "mass = 1.0\nspin = 0.5\ndisc_r_inner = 4.0\ndisc_r_outer = 30.0\n",
                "kerr_a094.scene": ("mass = 1.0\nspin = 0.94\ndisc_r_inner = 1.7\ndisc_r_outer = 30.0\n"
                                    "disc_doppler_on = 1\ndisc_redshift_on = 1\n")}[scene]
        (tmp_path / scene).write_text(text)
        args += ["--scene", tmp_path / scene]
    r = run(cli, *args)
    assert r.returncode == 0, r.stderr
    assert "wrote" in r.stdout and "(256x256, CUDA)" in r.stdout
    img = read_png(tmp_path / "o.png")
    u = uniforms_from_bytes(cuda_goldens[f"{name}_uniforms"])
    np.testing.assert_array_equal(img, renderer.render_image(u))
    if name != "schw":
        assert phash_distance(img, cuda_goldens[f"{name}_rgba8"]) <= 4


@pytest.mark.gpu
def test_cli_multi_frame_orbit(cli, tmp_path):
    """verification/test_cuda_goldens.py:84-129: 4 frames, the camera advances 90 deg."""
    scene = tmp_path / "k.scene"
    scene.write_text("mass = 1.0\nspin = 0.94\ndisc_r_inner = 1.7\ndisc_r_outer = 30.0\n")
    r = run(cli, "--frames", "4", "--output-pattern", tmp_path / "frame_%02d.png", "--res", "64x64",
            "--samples-per-pixel", "1", "--scene", scene)
    assert r.returncode == 0, r.stderr
    paths = sorted(tmp_path.glob("frame_*.png"))
    assert len(paths) == 4
    assert r.stdout.count("wrote") == 4 and "frame 4/4" in r.stdout
    f0, f2 = read_png(paths[0]), read_png(paths[2])
    assert phash_distance(f0, f2) > 0


@pytest.mark.gpu
def test_cli_extensions(cli, tmp_path):
    r = run(cli, "--output", tmp_path / "a.png", "--res", "96x54", "--samples-per-pixel", "4", "--integrator",
            "adaptive", "--precision", "mixed", "--disc-inner-isco", "--peak-temp", "10000", "--pfm")
    assert r.returncode == 0, r.stderr
    img = read_png(tmp_path / "a.png")
    assert img.shape == (54, 96, 4)
    data = (tmp_path / "a.pfm").read_bytes()
    assert data.startswith(b"PF\n96 54\n-1.0\n")
    f = np.frombuffer(data[len(b"PF\n96 54\n-1.0\n"):], dtype="<f4").reshape(54, 96, 3)[::-1]
    srgb = np.where(f <= 0.0031308, 12.92 * f, 1.055 * np.power(np.clip(f, 0, 1), 1 / 2.4) - 0.055)
    u8 = np.clip(srgb * 255 + 0.5, 0, 255).astype(np.uint8)
    assert np.abs(u8.astype(int) - img[..., :3].astype(int)).max() <= 1


@pytest.mark.gpu
def test_cli_adaptive_step_flag(cli, tmp_path, sgx, oracle):
    """--adaptive-step packs SGX_FLAG_ADAPTIVE_STEP (the radius-adaptive step of
    geodesic_math.h:91-96); the CLI's image matches the oracle with that flag."""
    scene = tmp_path / "s.scene"
    scene.write_text("mass = 1.0\nspin = 0.0\ndisc_r_inner = 6.0\ndisc_r_outer = 20.0\n")
    r = run(cli, "--output", tmp_path / "a.png", "--res", "64x48", "--scene", scene, "--adaptive-step")
    assert r.returncode == 0, r.stderr
    img = read_png(tmp_path / "a.png")
    sc = sgx.Scene(metric=sgx.MetricType.Schwarzschild, spin_a_over_M=0.0, disc_inner_M=6.0, disc_outer_M=20.0,
                   adaptive_step_on=True)
    u = sgx.pack_uniforms(sc, sgx.build_orbital_camera(30.0, 0.15, 0.0, 60.0), 64, 48)
    ref, _ = oracle.render(u)
    d = np.abs(img[..., :3].astype(int) - ref[..., :3].astype(int))
    assert d.mean() <= 0.5 and (d.max(axis=-1) <= 1).mean() >= 0.97


@pytest.mark.gpu
def test_cli_bloom_and_seed(cli, tmp_path, sgx, renderer):
    """--bloom-sigma renders the half-float HDR frame and writes the bloom +
    ACES composite; --turbulence-seed sets the first frame's band phase. The
    PNG equals the library's HDR render + sgx_bloom of the same scene."""
    N = sgx._native
    r = run(cli, "--output", tmp_path / "b.png", "--res", "96x54", "--samples-per-pixel", "2",
            "--bloom-sigma", "8", "--turbulence-seed", "7")
    assert r.returncode == 0, r.stderr
    img = read_png(tmp_path / "b.png")
    sc = sgx.Scene(render_supersample=2)
    u = sgx.pack_uniforms(sc, sgx.build_orbital_camera(30.0, 0.15, 0.0, 60.0), 96, 54, 7.0 / 30.0)
    renderer.render(u, sgx.default_opts(format=N.FORMAT_RGBA16F_HDR))
    ref = renderer.bloom(sigma_px=8.0, fmt=N.FORMAT_RGBA8_SRGB)
    np.testing.assert_array_equal(img, ref)
    plain = run(cli, "--output", tmp_path / "p.png", "--res", "96x54", "--samples-per-pixel", "2",
                "--turbulence-seed", "7")
    assert plain.returncode == 0
    assert not np.array_equal(read_png(tmp_path / "p.png"), img)


@pytest.mark.gpu
def test_cli_rhs_form(cli, tmp_path, sgx, renderer):
    """--rhs-form 2 renders the library's rhs_form 2 frame of the same scene
    (sin/cos of theta carried in the fixed-step state), close to form 0."""
    r = run(cli, "--output", tmp_path / "f2.png", "--res", "96x54", "--samples-per-pixel", "2", "--rhs-form", "2")
    assert r.returncode == 0, r.stderr
    img = read_png(tmp_path / "f2.png")
    u = sgx.pack_uniforms(sgx.Scene(render_supersample=2), sgx.build_orbital_camera(30.0, 0.15, 0.0, 60.0), 96, 54)
    np.testing.assert_array_equal(img, renderer.render_image(u, sgx.default_opts(rhs_form=2)))
    f0 = renderer.render_image(u, sgx.default_opts())
    assert (np.abs(img.astype(int) - f0.astype(int)).max(axis=-1) <= 1).mean() >= 0.99


SCENE_WITH_CAMERA_AND_STEPS = ("mass = 1.0\nspin = 0.9\ndisc_r_inner = 2.5\ndisc_r_outer = 25.0\n"
                               "camera_distance = 22.0\ncamera_elevation = 0.4\ncamera_fov_deg = 45.0\n"
                               "h_step = 0.25\nmax_steps = 900\n")


@pytest.mark.gpu
@pytest.mark.parametrize("use_camera,use_integrator", [(False, False), (True, False), (False, True), (True, True)])
def test_cli_scene_opt_ins(cli, sgx, renderer, tmp_path, use_camera, use_integrator):
    """--use-scene-camera / --use-scene-integrator (extensions, off by default):
    the .scene file's camera_distance, camera_elevation, camera_fov_deg and
    h_step, max_steps keys reach the render only when asked for; by default
    they are ignored as the reference's cuda_cli ignores them
    (cuda_cli/main.cpp:209-217) and the CLI's default camera (30 M, 0.15 rad,
    60 deg) and the backend's step (0.4, 2500 steps) apply.  The PNG equals
    the library render of the uniforms those choices imply."""
    scene = tmp_path / "s.scene"
    scene.write_text(SCENE_WITH_CAMERA_AND_STEPS)
    args = ["--output", tmp_path / "o.png", "--res", "96x64", "--scene", scene]
    if use_camera:
        args.append("--use-scene-camera")
    if use_integrator:
        args.append("--use-scene-integrator")
    r = run(cli, *args)
    assert r.returncode == 0, r.stderr
    img = read_png(tmp_path / "o.png")
    sc = sgx.Scene(spin_a_over_M=0.9, disc_inner_M=2.5, disc_outer_M=25.0,
                   h_step=0.25 if use_integrator else 0.0, max_steps=900 if use_integrator else 0)
    cam = (sgx.build_orbital_camera(22.0, 0.4, 0.0, 45.0) if use_camera
           else sgx.build_orbital_camera(30.0, 0.15, 0.0, 60.0))
    u = sgx.pack_uniforms(sc, cam, 96, 64)
    assert abs(u.h_step - (0.25 if use_integrator else 0.4)) < 1e-7
    assert u.max_steps == (900 if use_integrator else 2500)
    np.testing.assert_array_equal(img, renderer.render_image(u))
    if use_camera or use_integrator:
        plain = run(cli, "--output", tmp_path / "p.png", "--res", "96x64", "--scene", scene)
        assert plain.returncode == 0
        assert not np.array_equal(read_png(tmp_path / "p.png"), img)
