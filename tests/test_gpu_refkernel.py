"""Our kernels against the reference's own CUDA kernel on the same GB300.

The reference kernel (render/cuda/kernels/geodesic_kernel.cu, compiled to PTX
from the reference tree by `make -C oracle ref`) is launched the way
CudaBackend::render_frame launches it (oracle/ref_gpu.py).  Parity: the same
RGBA8 frame on the pinned scenes — at least 99.5 % identical pixels and none
off by more than one level (both are FP32 CUDA; the few differing pixels are
near-polar rays where the two compilations' FMA contractions diverge).  Speed: the reference's
one-thread-per-pixel fixed-step kernel against our fixed-step kernel and our
precision form on the same scene, printed (and ours required faster)."""

from __future__ import annotations

import time

import numpy as np
import pytest

from conftest import uniforms_from_bytes
from imgmetrics import channel_error

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refk(sgx, renderer):
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("reference kernel PTX not built (make -C oracle ref needs the reference tree)")
    import torch
    torch.zeros(1, device="cuda")  # the primary context current on this thread
    k = ref_gpu.RefKernel()
    yield k
    k.close()


def _ref_frame(refk, u):
    import torch
    out = torch.zeros(u.width * u.height * 4, dtype=torch.uint8, device="cuda")
    refk.launch(out.data_ptr(), u)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(u.height, u.width, 4)


@pytest.mark.parametrize("rhs_form", [0, 1])
def test_matches_reference_cuda_kernel(renderer, sgx, host_vectors, refk, rhs_form):
    z, names = host_vectors
    for name in names:
        u = uniforms_from_bytes(z[f"{name}_uniforms"])
        ref = _ref_frame(refk, u)
        img = renderer.render_image(u, sgx.default_opts(rhs_form=rhs_form))
        e = channel_error(img, ref)
        exact = float((img == ref).all(axis=-1).mean())
        print(f"{name} rhs_form={rhs_form}: exact pixels {exact:.4f} {e}")
        # measured: identical frames on 8 of the 9 scenes, 99.8 % identical
        # pixels (others one level off) on the near-polar one
        assert exact >= 0.995 and e["max"] <= 1, (name, e)
        np.testing.assert_array_equal(ref, _ref_frame(refk, u))  # the reference kernel is deterministic


def test_faster_than_reference_cuda_kernel(renderer, sgx, refk):
    import torch
    N = sgx._native
    u = sgx.workloads.kerr_1080p_16spp()
    rays = u.width * u.height * u.supersample
    out = torch.zeros(u.width * u.height * 4, dtype=torch.uint8, device="cuda")
    refk.launch(out.data_ptr(), u)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(2):
        refk.launch(out.data_ptr(), u)
    torch.cuda.synchronize()
    t_ref = (time.perf_counter() - t0) / 2
    res = {}
    for name, opts in (("fixed", sgx.default_opts()),
                       ("precision_form", sgx.default_opts(integrator=N.INTEGRATOR_ADAPTIVE,
                                                           precision=N.PRECISION_MIXED))):
        renderer.render(u, opts)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(2):
            renderer.render(u, opts)
        torch.cuda.synchronize()
        res[name] = (time.perf_counter() - t0) / 2
    print(f"1080p x 16 spp: reference CUDA kernel {rays / t_ref / 1e6:.1f} Mrays/s, ours fixed step "
          f"{rays / res['fixed'] / 1e6:.1f}, ours precision form {rays / res['precision_form'] / 1e6:.1f}")
    assert res["fixed"] < t_ref


def test_random_scenes_match_reference_cuda_kernel(renderer, sgx, refk):
    """Seeded random scenes (metric, spin, camera, FOV, flags, disc, spp, step,
    budget) through both kernels."""
    N = sgx._native
    rng = np.random.default_rng(11)
    exact_all = []
    for i in range(24):
        kerr = bool(rng.integers(0, 2))
        spin = float(rng.uniform(0.0, 0.998)) if kerr else 0.0
        sc = sgx.Scene(metric=sgx.MetricType.Kerr if kerr else sgx.MetricType.Schwarzschild, spin_a_over_M=spin,
                       disc_inner_M=float(rng.uniform(1.5, 8.0)), disc_outer_M=float(rng.uniform(12.0, 40.0)),
                       disc_peak_T_K=float(rng.uniform(3000.0, 20000.0)), render_supersample=int(rng.integers(1, 5)),
                       h_step=float(rng.choice([0.2, 0.4])), max_steps=int(rng.choice([500, 2500])),
                       disc_doppler_on=bool(rng.integers(0, 2)), disc_redshift_on=bool(rng.integers(0, 2)))
        cam = sgx.build_orbital_camera(float(rng.uniform(15.0, 60.0)), float(rng.uniform(-1.4, 1.4)),
                                       float(rng.uniform(0.0, 6.28)), float(rng.uniform(20.0, 70.0)))
        u = sgx.pack_uniforms(sc, cam, int(rng.integers(8, 80)), int(rng.integers(8, 60)), float(rng.uniform(0, 2)))
        ref = _ref_frame(refk, u)
        img = renderer.render_image(u)
        e = channel_error(img, ref)
        exact = float((img == ref).all(axis=-1).mean())
        exact_all.append(exact)
        print(f"scene {i} kerr={kerr} a={spin:.3f} {u.width}x{u.height}x{u.supersample}: exact {exact:.4f} max {e['max']}")
        assert e["mean"] <= 2e-3 and e["le1_frac"] >= 0.97, (i, e)
    print(f"mean identical pixels {np.mean(exact_all):.4f}")
    assert np.mean(exact_all) >= 0.99


def test_schwarzschild_256_workload(renderer, sgx, oracle, refk):
    """The plain Schwarzschild workload (256x256, 1 spp at pixel centres, h = 0.05 M,
    4000 steps, r 30 M, i 80 deg, FOV 40, disc 6-20 M, FP32 RGBA float output):
    RGBA8 against the reference CUDA kernel, RGBA32F against the FP32 oracle."""
    N = sgx._native
    u = sgx.workloads.schwarzschild_256()
    ref = _ref_frame(refk, u)
    img = renderer.render_image(u)
    exact = float((img == ref).all(axis=-1).mean())
    f32 = renderer.capture(N.FORMAT_RGBA32F)[..., :3]
    _, ldr = oracle.render(u)
    d = np.abs(f32 - ldr.reshape(u.height, u.width, 3))
    print(f"schwarzschild_256: identical RGBA8 pixels vs reference kernel {exact:.4f}; "
          f"RGBA32F vs oracle mean {d.mean():.2e} max {d.max():.2e}")
    assert exact >= 0.995
    # GPU against host math: the few photon-ring rays where CUDA's and the C
    # library's last-ulp sin/pow differ end differently (measured: mean 1.2e-5)
    assert d.mean() <= 1e-4 and (d.max(axis=-1) <= 1e-3).mean() >= 0.999
