"""The differentiable render form and its adjoint on the GPU, through the C ABI.

Forward: the GPU image against the oracle's image of the same form
(oracle/diff_oracle.hpp) in the same precision.  Adjoint: the GPU's gradient
of an image loss against central differences of the oracle's FP64 image
(steps 1e-3 and 3e-4) and the FP32 adjoint against the FP64 adjoint.
Tolerances are stated per test."""

from __future__ import annotations

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FD_STEP = 1e-3


@pytest.fixture(scope="module")
def diff(sgx, renderer):
    from singularity_gb300 import diff as D
    return D.DiffRenderer(renderer)


def _setup(sgx, w=64, h=48, spp=2):
    W = sgx.workloads
    base = W.differentiation_base(w, h, spp)
    tgt = W.differentiation_params(W.differentiation_target())
    guess = W.differentiation_params(W.differentiation_guess())
    return base, tgt, guess


def _loss_grad_image(img, target):
    import torch
    return 2.0 * (img - target) / img.numel()


@pytest.mark.parametrize("model", [1, 0])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_forward_matches_oracle(diff, sgx, oracle, prec, model):
    from singularity_gb300 import diff as D
    N = sgx._native
    base, tgt, guess = _setup(sgx)
    opts = D.DiffOptions(precision=N.PRECISION_FP32 if prec == "f32" else N.PRECISION_FP64, model=model)
    for p in (tgt, guess):
        img = diff.forward(base, p, opts).cpu().numpy()
        ref = oracle.diff_render(base, p, precision=prec, **opts.oracle_form()).astype(np.float32)
        e = np.abs(img - ref)
        print(f"model {model} {prec} {p}: mean {e.mean():.2e} max {e.max():.2e}")
        if prec == "f64":
            assert e.mean() <= 1e-6 and e.max() <= 1e-4
        else:
            assert e.mean() <= 2e-5 and (e <= 1e-3).mean() >= 0.999


def _adjoint_and_fd(diff, sgx, oracle, model, steps=(FD_STEP,)):
    import torch
    from singularity_gb300 import diff as D
    N = sgx._native
    base, tgt, guess = _setup(sgx)
    form = D.DiffOptions(model=model).oracle_form()
    target = oracle.diff_render(base, tgt, **form)
    fds = [oracle.diff_fd_gradient(base, guess, target, step=st, **form) for st in steps]
    t_dev = torch.as_tensor(target.astype(np.float32), device="cuda")
    out = {}
    for prec in (N.PRECISION_FP64, N.PRECISION_FP32):
        img = diff.forward(base, guess, D.DiffOptions(precision=prec, model=model))
        out[prec] = diff.backward(_loss_grad_image(img, t_dev))
    return fds, out[N.PRECISION_FP64], out[N.PRECISION_FP32]


def test_adjoint_matches_central_differences(diff, sgx, oracle):
    """Slab model: the FP64 adjoint against central differences of the FP64
    oracle (steps 1e-3 and 3e-4), all four parameters; the FP32 adjoint
    against the FP64 adjoint."""
    (fd3, fd4), g64, g32 = _adjoint_and_fd(diff, sgx, oracle, 1, steps=(1e-3, 3e-4))
    rel3 = np.abs(g64 - fd3) / np.abs(fd3)
    rel4 = np.abs(g64 - fd4) / np.abs(fd4)
    rel32 = np.abs(g32 - g64) / np.abs(g64)
    print("fd 1e-3", fd3)
    print("fd 3e-4", fd4)
    print("fp64   ", g64, "rel vs fd 1e-3", rel3, "vs 3e-4", rel4)
    print("fp32   ", g32, "rel vs fp64", rel32)
    # FD at 1e-3 carries O(step^2) truncation and O(step) kink bias of a few
    # 1e-4; the better of the two steps must agree to 1e-3
    assert np.all(np.minimum(rel3, rel4) <= 1e-3), (rel3, rel4)
    assert np.all(rel32 <= 1e-3), rel32


def test_crossing_adjoint_smooth_parameters(diff, sgx, oracle):
    """Crossing model: r_in and t_scale (the parameters it is smooth in)."""
    (fd,), g64, g32 = _adjoint_and_fd(diff, sgx, oracle, 0)
    rel = np.abs(g64 - fd) / np.abs(fd)
    print("fd", fd, "fp64", g64, "rel", rel, "fp32", g32)
    assert rel[2] <= 1e-3 and rel[3] <= 1e-3, rel
    assert np.all(np.abs(g32[2:] - g64[2:]) <= 1e-3 * np.abs(g64[2:]))


@pytest.mark.parametrize("model", [1, 0])
def test_adjoint_matches_oracle_dual_gradient(diff, sgx, oracle, model):
    """The GPU adjoint against the oracle's forward-mode dual-number gradient of
    the same image loss (same dL/dI): FP64 to 1e-9, FP32 to 1e-3."""
    import torch
    from singularity_gb300 import diff as D
    N = sgx._native
    base, tgt, guess = _setup(sgx)
    form = D.DiffOptions(model=model).oracle_form()
    target = torch.as_tensor(oracle.diff_render(base, tgt, **form).astype(np.float32), device="cuda")
    got = {}
    for prec in (N.PRECISION_FP64, N.PRECISION_FP32):
        img = diff.forward(base, guess, D.DiffOptions(precision=prec, model=model))
        seed = _loss_grad_image(img, target)
        got[prec] = diff.backward(seed)
        if prec == N.PRECISION_FP64:
            ref, _ = oracle.diff_grad(base, guess, seed.cpu().numpy().astype(np.float64), **form)
    r64 = np.abs(got[N.PRECISION_FP64] - ref) / np.abs(ref)
    r32 = np.abs(got[N.PRECISION_FP32] - ref) / np.abs(ref)
    print(f"model {model}: oracle dual {ref} gpu fp64 rel {r64} gpu fp32 rel {r32}")
    assert np.all(r64 <= 1e-9), r64
    assert np.all(r32 <= 1e-3), r32


@pytest.mark.parametrize("model", [1, 0])
@pytest.mark.parametrize("prec", [0, 2])
def test_reverse_pass_matches_dual_jacobians(diff, sgx, prec, model):
    """The hand-derived reverse pass of a step against the step Jacobian built
    with dual numbers: the same gradient to rounding."""
    import torch
    from singularity_gb300 import diff as D
    base, tgt, guess = _setup(sgx, 48, 32, 2)
    target = diff.forward(base, tgt, D.DiffOptions(precision=prec, model=model)).clone()
    out = []
    for form in (sgx._native.DIFF_ADJOINT_REVERSE, sgx._native.DIFF_ADJOINT_DUAL):
        o = D.DiffOptions(precision=prec, model=model, adjoint_form=form)
        img = diff.forward(base, guess, o)
        out.append(diff.backward(_loss_grad_image(img, target)))
    rel = np.abs(out[0] - out[1]) / np.abs(out[1])
    print(f"prec {prec} model {model}: reverse {out[0]} dual {out[1]} rel {rel}")
    assert np.all(rel <= (1e-9 if prec == 2 else 1e-4)), rel


@pytest.mark.parametrize("model", [1, 0])
def test_dense_and_sparse_checkpoints_agree(diff, sgx, model):
    """FP32 adjoint from 10-step checkpoints (segment recomputed into shared
    memory) against 64-step checkpoints (thread-local segment): the same
    recomputed states and reverse pass, so the same gradient to rounding."""
    from singularity_gb300 import diff as D
    base, tgt, guess = _setup(sgx, 48, 32, 2)
    target = diff.forward(base, tgt, D.DiffOptions(model=model)).clone()
    out = []
    for ck in (10, 64):
        img = diff.forward(base, guess, D.DiffOptions(model=model, checkpoint_interval=ck))
        assert diff.stats()["checkpoint_steps"] == ck
        out.append(diff.backward(_loss_grad_image(img, target)))
    rel = np.abs(out[0] - out[1]) / np.abs(out[1])
    print(f"model {model}: 10-step {out[0]} 64-step {out[1]} rel {rel} identical {np.array_equal(out[0], out[1])}")
    assert np.all(rel <= 1e-6), rel


def test_checkpoint_interval_options(diff, sgx):
    from singularity_gb300 import diff as D
    N = sgx._native
    base, tgt, guess = _setup(sgx, 16, 16, 1)
    for bad in (D.DiffOptions(checkpoint_interval=7),
                D.DiffOptions(checkpoint_interval=10, precision=N.PRECISION_FP64),
                D.DiffOptions(checkpoint_interval=10, adjoint_form=N.DIFF_ADJOINT_DUAL)):
        with pytest.raises(sgx.SgxError):
            diff.forward(base, guess, bad)
    # automatic: 10 for FP32 with the reverse pass (records fit the budget), else 64
    for ok, want in ((D.DiffOptions(), 10), (D.DiffOptions(precision=N.PRECISION_FP64), 64),
                     (D.DiffOptions(checkpoint_interval=64, precision=N.PRECISION_FP64), 64),
                     (D.DiffOptions(adjoint_form=N.DIFF_ADJOINT_DUAL), 64)):
        diff.forward(base, guess, ok)
        assert diff.stats()["checkpoint_steps"] == want


def test_backward_is_deterministic(diff, sgx):
    import torch
    base, tgt, guess = _setup(sgx, 40, 30, 2)
    img = diff.forward(base, guess)
    g = torch.ones_like(img) * 1e-3
    a = diff.backward(g)
    b = diff.backward(g)
    np.testing.assert_array_equal(a, b)
    assert diff.stats()["crossing_overflow"] == 0


def test_autograd_function(diff, sgx):
    import torch
    from singularity_gb300 import diff as D
    base, tgt, guess = _setup(sgx, 40, 30, 2)
    target = diff.forward(base, tgt).clone()
    p = torch.tensor(guess, dtype=torch.float64, requires_grad=True)
    img = D.render(p, diff, base)
    loss = torch.mean((img - target) ** 2)
    loss.backward()
    direct_img = diff.forward(base, guess)
    direct = diff.backward(2.0 * (direct_img - target) / direct_img.numel())
    np.testing.assert_allclose(p.grad.numpy(), direct, rtol=1e-6, atol=1e-12)
    # a forward in between: the function recomputes its records
    p.grad = None
    img = D.render(p, diff, base)
    diff.forward(base, tgt)
    torch.mean((img - target) ** 2).backward()
    np.testing.assert_allclose(p.grad.numpy(), direct, rtol=1e-6, atol=1e-12)


def test_errors(diff, sgx):
    import torch
    from singularity_gb300 import diff as D
    base, tgt, guess = _setup(sgx, 16, 16, 1)
    with pytest.raises(sgx.SgxError):
        diff.forward(base, (1.5, 1.0, 5.0, 1.0))
    with pytest.raises(sgx.SgxError):
        diff.forward(base, guess, D.DiffOptions(precision=sgx._native.PRECISION_MIXED))
    schw = base.copy()
    schw.metric_type = 0
    with pytest.raises(sgx.SgxError):
        diff.forward(schw, guess)


def test_adam_reduces_loss(diff, sgx):
    """A short recovery run: the loss falls and every parameter moves toward the target."""
    from singularity_gb300 import diff as D
    base, tgt, guess = _setup(sgx, 64, 64, 1)
    target = diff.forward(base, tgt).clone()
    res = D.fit(diff, base, target, guess, steps=40)
    print("loss", res.loss[0], "->", res.loss[-1])
    print("params", res.params[-1], "target", tgt)
    assert res.loss[-1] < 0.25 * res.loss[0]
    d0 = np.abs(np.array(guess) - np.array(tgt))
    d1 = np.abs(res.params[-1] - np.array(tgt))
    assert np.sum(d1 / d0) < np.sum(np.ones(4))
