"""The drop-in relink: the reference's own, unmodified cuda_cli/main.cpp
compiled against this library's CudaBackend shim
(singularity_gb300/csrc/cuda_backend.hpp, which takes Scene, CameraState,
ImageData, WindowHandle, RenderConfig and RenderBackend from the reference's
render/include/render_backend.hpp) and linked with libsgx.so
(`make -C oracle relink`, oracle/pyoracle.py build_relink).

CPU: it compiles and links with no source change, binds libsgx.so, and
behaves as the reference CLI does without a GPU.  GPU: on the reference's
three golden commands its PNG equals singularity_cuda_cli's.
"""

from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from imgmetrics import read_png

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="session")
def relinked(sgx, oracle):
    p = oracle.build_relink()
    if p is None:
        pytest.skip("no reference sources (checkout or oracle/_ref/src snapshot) on this machine")
    return p


def run(exe, *args, timeout=120):
    return subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, timeout=timeout)


def test_reference_cli_relinks_against_the_shim(relinked):
    # the executable binds this library, not the reference's kernel
    maps = subprocess.run(["ldd", str(relinked)], capture_output=True, text=True).stdout
    assert "libsgx.so" in maps
    syms = subprocess.run(["nm", "-C", str(relinked)], capture_output=True, text=True).stdout
    assert "singularity_geodesic_kernel" not in syms
    assert "singularity::CudaBackend::render_frame" in syms
    r = run(relinked, "--help")
    assert r.returncode == 0 and "--samples-per-pixel" in r.stdout
    r = run(relinked, "--bogus")
    assert r.returncode == 2 and "unknown argument: --bogus" in r.stderr


def test_relinked_cli_without_gpu(relinked, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run(relinked, "--res", "8x8", "--output", tmp_path / "x.png")
    assert r.returncode == 1 and "backend initialize failed" in r.stderr


GOLDEN_SCENES = {
    "schw": None,
    "kerr_a05": "mass = 1.0\nspin = 0.5\ndisc_r_inner = 4.0\ndisc_r_outer = 30.0\n",
    "kerr_a094": "mass = 1.0\nspin = 0.94\ndisc_r_inner = 1.7\ndisc_r_outer = 30.0\ndisc_doppler_on = 1\n"
                 "disc_redshift_on = 1\n",
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GOLDEN_SCENES))
def test_relinked_cli_png_equals_ours(relinked, tmp_path, name):
    """verification/test_cuda_goldens.py's commands (`--res 256x256 [--scene
    scenes/<name>.scene]`) through the relinked reference CLI and through
    singularity_cuda_cli: the same pixels."""
    ours = ROOT / "singularity_gb300" / "_build" / "singularity_cuda_cli"
    args = ["--res", "256x256"]
    if GOLDEN_SCENES[name] is not None:
        scene = tmp_path / f"{name}.scene"
        scene.write_text(GOLDEN_SCENES[name])
        args += ["--scene", scene]
    a = run(relinked, *args, "--output", tmp_path / "ref.png")
    b = run(ours, *args, "--output", tmp_path / "ours.png")
    assert a.returncode == 0, a.stderr
    assert b.returncode == 0, b.stderr
    assert "(256x256, CUDA)" in a.stdout
    np.testing.assert_array_equal(read_png(tmp_path / "ref.png"), read_png(tmp_path / "ours.png"))


def test_png_reader_handles_every_row_filter(tmp_path):
    """The test-side PNG reader decodes all five row filters (the reference
    CLI's stb_image_write picks one per row)."""
    import struct
    import zlib
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    rows = img.reshape(5, 28).astype(np.int32)
    raw = b""
    prev = np.zeros(28, dtype=np.int32)
    for y, f in enumerate((0, 1, 2, 3, 4)):
        cur = rows[y]
        left = np.concatenate([np.zeros(4, np.int32), cur[:-4]])
        upleft = np.concatenate([np.zeros(4, np.int32), prev[:-4]])
        if f == 0:
            enc = cur
        elif f == 1:
            enc = cur - left
        elif f == 2:
            enc = cur - prev
        elif f == 3:
            enc = cur - ((left + prev) >> 1)
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            enc = cur - np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
        raw += bytes([f]) + (enc & 255).astype(np.uint8).tobytes()
        prev = cur

    def chunk(t, b):
        return struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xFFFFFFFF)
    path = tmp_path / "f.png"
    path.write_bytes(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 7, 5, 8, 6, 0, 0, 0))
                     + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))
    np.testing.assert_array_equal(read_png(path), img)


@pytest.mark.gpu
def test_relinked_cli_multi_frame_orbit_equals_ours(relinked, tmp_path):
    """The reference's multi-frame mode (`--frames 4 --output-pattern`, the
    camera orbiting 2 pi and the disc clock advancing 1/30 s a frame,
    cuda_cli/main.cpp:251-338) through the relinked reference CLI and
    through singularity_cuda_cli: the same four frames."""
    ours = ROOT / "singularity_gb300" / "_build" / "singularity_cuda_cli"
    scene = tmp_path / "k.scene"
    scene.write_text(GOLDEN_SCENES["kerr_a094"])
    for exe, name in ((relinked, "ref"), (ours, "ours")):
        r = run(exe, "--frames", "4", "--output-pattern", tmp_path / f"{name}_%02d.png", "--res", "96x64",
                "--samples-per-pixel", "2", "--scene", scene)
        assert r.returncode == 0, r.stderr
        assert r.stdout.count("wrote") == 4
    for k in range(4):
        a, b = read_png(tmp_path / f"ref_{k:02d}.png"), read_png(tmp_path / f"ours_{k:02d}.png")
        np.testing.assert_array_equal(a, b)
    assert not np.array_equal(read_png(tmp_path / "ours_00.png"), read_png(tmp_path / "ours_02.png"))
