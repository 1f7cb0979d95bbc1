"""Generate the committed golden fixtures from the reference tree.

Run where a full reference checkout is, named by $SGX_REFERENCE_ROOT
(oracle.pyoracle.reference_checkout()).  Nothing at test
time reads the reference tree; the tests read only the files this script
writes:

* ``reference_cuda_goldens.npz`` — the reference's own CUDA golden images
  (verification/golden/cuda/{schw,kerr_a05,kerr_a094}.png, 256x256 RGBA8, made
  by singularity_cuda_cli on an RTX 30-series GPU), decoded to arrays, with
  the uniform block the reference CLI packs for each (default camera,
  --res 256x256, the scene files of scenes/).
* ``reference_host_vectors.npz`` — outputs of the reference kernel source
  compiled for the host CPU (oracle/_ref): full RGBA8 images and per-sample
  HDR colours for a set of small scenes, with their uniform blocks.
* ``reference_host_scene_cases.json`` — the reference .scene loader and
  orbital camera on a set of inputs.
"""

from __future__ import annotations

import json
import os
import struct
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

def _checkout() -> Path:
    from oracle import pyoracle
    root = pyoracle.reference_checkout()
    if root is None:
        raise SystemExit("no reference checkout: set SGX_REFERENCE_ROOT")
    return root


REF = _checkout()


def decode_png_rgba8(path: Path) -> np.ndarray:
    """Minimal PNG decoder: 8-bit RGB/RGBA, non-interlaced, the five filters."""
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG"
    pos, idat, w = 8, b"", 0
    while pos < len(data):
        ln, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + ln]
        if typ == b"IHDR":
            w, h, depth, ctype, _, _, inter = struct.unpack(">IIBBBBB", body)
            assert depth == 8 and ctype in (2, 6) and inter == 0
            ch = 4 if ctype == 6 else 3
        elif typ == b"IDAT":
            idat += body
        pos += 12 + ln
    raw = zlib.decompress(idat)
    stride = w * ch
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, dtype=np.uint8, count=stride, offset=y * (stride + 1) + 1).astype(np.int32)
        cur = np.zeros(stride, dtype=np.int32)
        for x in range(stride):
            a = cur[x - ch] if x >= ch else 0
            b = prev[x]
            c = prev[x - ch] if x >= ch else 0
            if f == 0:
                v = line[x]
            elif f == 1:
                v = line[x] + a
            elif f == 2:
                v = line[x] + b
            elif f == 3:
                v = line[x] + ((a + b) >> 1)
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                v = line[x] + (a if (pa <= pb and pa <= pc) else (b if pb <= pc else c))
            cur[x] = v & 0xFF
        out[y] = cur
        prev = cur
    img = out.reshape(h, w, ch)
    if ch == 3:
        img = np.concatenate([img, np.full((h, w, 1), 255, np.uint8)], axis=2)
    return img


def cli_uniforms(scene_file: str | None, width=256, height=256, spp=1, dist=30.0, elev=0.15, az=0.0, fov=60.0):
    """The uniform block singularity_cuda_cli packs (cuda_cli/main.cpp:193-258)."""
    import singularity_gb300 as S
    scene = S.Scene()
    if scene_file is not None:
        res, cfg = S.load_scene_config_from_file(str(REF / scene_file))
        assert res.status == S.SceneLoadStatus.Ok
        scene.mass_solar = cfg.mass
        scene.spin_a_over_M = cfg.spin
        scene.disc_inner_M = cfg.disc_r_inner
        scene.disc_outer_M = cfg.disc_r_outer
        scene.disc_doppler_on = cfg.disc_doppler_on
        scene.disc_redshift_on = cfg.disc_redshift_on
        scene.metric = S.MetricType.Kerr if cfg.spin > 0 else S.MetricType.Schwarzschild
    scene.render_supersample = spp
    cam = S.build_orbital_camera(dist, elev, az, fov)
    return S.pack_uniforms(scene, cam, width, height, 0.0)


def host_cases():
    """Small scenes covering both metrics, every flag path, spp > 1 and edges."""
    import singularity_gb300 as S
    cases = []
    # The three CLI golden scenes at 64x48 (both metrics via the scene files).
    for name, f in [("schw_default", None), ("kerr_a05", "scenes/kerr_a05.scene"),
                    ("kerr_a094", "scenes/kerr_a094.scene")]:
        cases.append((name, cli_uniforms(f, 64, 48)))
    # Schwarzschild metric proper (spin 0 scene), disc 6-20, h 0.05, 4000 steps, fov 40, r 30, i 80 deg.
    sc = S.Scene(metric=S.MetricType.Schwarzschild, spin_a_over_M=0.0, disc_inner_M=6.0, disc_outer_M=20.0,
                 max_steps=4000, h_step=0.05)
    cases.append(("schw_a0_fov40_small", S.pack_uniforms(sc, S.build_orbital_camera(30.0, 0.174533, 0.0, 40.0), 40, 40)))
    # Kerr 0.94, 4 spp Halton, r 40, i 75, fov 30, disc ISCO..30, T 1e4.
    isco = S.kerr_isco_prograde(1.0, 0.94)
    sc = S.Scene(spin_a_over_M=0.94, disc_inner_M=isco, disc_outer_M=30.0, disc_peak_T_K=1e4, render_supersample=4)
    cases.append(("kerr094_spp4", S.pack_uniforms(sc, S.build_orbital_camera(40.0, 0.261799, 0.0, 30.0), 32, 24)))
    # Flags off (no Doppler / redshift), time animation, exposure and turbulence changes.
    sc = S.Scene(spin_a_over_M=0.3, disc_doppler_on=False, disc_redshift_on=False, exposure=0.7,
                 disc_turbulence=1.0)
    cases.append(("kerr03_flags", S.pack_uniforms(sc, S.build_orbital_camera(25.0, 0.4, 1.0, 50.0), 32, 32, 0.5)))
    # Disc off (starfield + shadow only), odd size.
    sc = S.Scene(spin_a_over_M=0.8, disc_texture_on=False)
    cases.append(("kerr08_nodisc", S.pack_uniforms(sc, S.build_orbital_camera(20.0, -0.3, 2.0, 70.0), 17, 13)))
    # Tiny step budget: rays run out (budget black).
    sc = S.Scene(spin_a_over_M=0.6, max_steps=30)
    cases.append(("kerr06_budget", S.pack_uniforms(sc, S.build_orbital_camera(30.0, 0.15, 0.0, 60.0), 16, 16)))
    # Near-polar view (pole damping path).
    sc = S.Scene(spin_a_over_M=0.9)
    cases.append(("kerr09_polar", S.pack_uniforms(sc, S.build_orbital_camera(30.0, 1.50, 0.0, 40.0), 24, 24)))
    return cases


def main() -> None:
    from oracle import pyoracle as O
    O.build(ref=True)
    assert O.ref_available(), "the host build of the reference kernel is required"

    # 1. the reference's CUDA goldens.
    arrays, meta = {}, {}
    for name, scene_file in [("schw", None), ("kerr_a05", "scenes/kerr_a05.scene"),
                             ("kerr_a094", "scenes/kerr_a094.scene")]:
        img = decode_png_rgba8(REF / "verification" / "golden" / "cuda" / f"{name}.png")
        u = cli_uniforms(scene_file)
        arrays[f"{name}_rgba8"] = img
        arrays[f"{name}_uniforms"] = np.frombuffer(u.to_bytes(), dtype=np.uint8)
        meta[name] = {"scene": scene_file, "res": "256x256", "spp": 1}
    np.savez_compressed(HERE / "reference_cuda_goldens.npz", **arrays, meta=json.dumps(meta))

    # 2. reference-host vectors.
    vec = {}
    rng = np.random.default_rng(1234)
    names = []
    for name, u in host_cases():
        names.append(name)
        vec[f"{name}_uniforms"] = np.frombuffer(u.to_bytes(), dtype=np.uint8)
        vec[f"{name}_rgba8"] = O.ref_render(u)
        spp = max(1, min(u.supersample, 1024))
        n = min(512, u.width * u.height * spp)
        gx = rng.integers(0, u.width, n).astype(np.uint32)
        gy = rng.integers(0, u.height, n).astype(np.uint32)
        s = rng.integers(0, spp, n).astype(np.uint32)
        vec[f"{name}_gx"], vec[f"{name}_gy"], vec[f"{name}_s"] = gx, gy, s
        vec[f"{name}_hdr"] = O.ref_trace(u, gx, gy, s)
    np.savez_compressed(HERE / "reference_host_vectors.npz", **vec, names=json.dumps(names))

    # 3. scene loader and camera.
    texts = {
        "kerr_a094": (REF / "scenes" / "kerr_a094.scene").read_text(),
        "kerr_a05": (REF / "scenes" / "kerr_a05.scene").read_text(),
        "comments_ws": "  # c\n\n mass = 2.5   # trailing\nspin=0.3\n  disc_doppler_on = OFF\ndisc_redshift_on=Yes\n",
        "all_keys": ("mass=1\nspin=0.9\ndisc_r_inner=2.3\ndisc_r_outer=25\ndisc_doppler_on=true\n"
                     "disc_redshift_on=0\ncamera_fov_deg=45\ncamera_distance=35\ncamera_elevation=0.2\n"
                     "h_step=0.05\nmax_steps=4000\n"),
        "unknown_key": "mass = 1\nbogus = 3\n",
        "no_equals": "mass 1\n",
        "empty_value": "mass =\n",
        "bad_float": "spin = 0.5x\n",
        "bad_bool": "disc_doppler_on = maybe\n",
        "bad_int": "max_steps = 12.5\n",
        "trailing_space_num": "spin = 0.25   \n",
        "partial_then_error": "spin = 0.7\nmass = abc\n",
        "empty": "",
    }
    scene_cases = {}
    for k, t in texts.items():
        st, fields, line = O.ref_load_scene_text(t)
        scene_cases[k] = {"text": t, "status": int(st), "fields": [float(x) for x in fields], "line": int(line)}
    cams = []
    for args in [(30.0, 0.15, 0.0, 60.0), (40.0, 0.261799, 0.0, 30.0), (30.0, 0.174533, 0.0, 40.0),
                 (25.0, 0.4, 1.0, 50.0), (20.0, -0.3, 2.0, 70.0), (30.0, 1.5707964, 0.0, 60.0),
                 (12.5, 0.9, 4.5, 90.0)]:
        cams.append({"args": list(args), "out": [float(x) for x in O.ref_orbital_camera(*args)]})
    (HERE / "reference_host_scene_cases.json").write_text(
        json.dumps({"scene_texts": scene_cases, "orbital_camera": cams}, indent=1))
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")), "and reference_host_scene_cases.json")


if __name__ == "__main__":
    main()
