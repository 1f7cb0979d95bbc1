"""The reference's physics known-answer tests, restated on the oracle
(the FP32 formulas the kernels share).

Radius-adaptive step: tests/test_adaptive_step.cpp:65-150 — a photon launched
tangentially at 8 M keeps its deflection within 0.5 % of a fine fixed-step
integration, conserves E and L to 3e-4, and escapes in >= 5x fewer steps.
"""

from __future__ import annotations

import math

import numpy as np


def _tangential_photon(r0, rs):
    # state (t, r, theta, phi, u^t, u^r, u^theta, u^phi) at periapsis r0 in the
    # equatorial plane; null condition with u^r = u^theta = 0
    ut = 1.0 / (1.0 - rs / r0)
    uphi = math.sqrt(1.0 - rs / r0) * ut / r0
    return np.array([0.0, r0, 0.5 * math.pi, 0.0, ut, 0.0, 0.0, uphi], dtype=np.float32)


def _motion_angle(y):
    cp, sp = math.cos(y[3]), math.sin(y[3])
    vx = y[5] * cp - y[1] * y[7] * sp
    vy = y[5] * sp + y[1] * y[7] * cp
    return math.atan2(vy, vx)


def test_adaptive_step_preserves_deflection(oracle):
    rs, r0, r_out = 2.0, 8.0, 400.0
    ref, n_ref, _, _ = oracle.schw_integrate(_tangential_photon(r0, rs), 0.01, rs, r_out, False)
    ad, n_ad, _, _ = oracle.schw_integrate(_tangential_photon(r0, rs), 0.12, rs, r_out, True)
    assert n_ref > 0 and n_ad > 0
    psi_ref, psi_ad = _motion_angle(ref), _motion_angle(ad)
    deflection = abs(psi_ref - 0.5 * math.pi)
    assert deflection > 0.1
    assert abs(psi_ad - psi_ref) < 0.005 * max(deflection, 1.0)


def test_adaptive_step_conserves_e_and_l(oracle):
    _, n, max_e, max_l = oracle.schw_integrate(_tangential_photon(8.0, 2.0), 0.12, 2.0, 400.0, True, budget=100000)
    assert n > 0
    assert max_e < 3e-4 and max_l < 3e-4


def test_adaptive_step_takes_5x_fewer_steps(oracle):
    _, n_fixed, _, _ = oracle.schw_integrate(_tangential_photon(8.0, 2.0), 0.12, 2.0, 200.0, False)
    _, n_ad, _, _ = oracle.schw_integrate(_tangential_photon(8.0, 2.0), 0.12, 2.0, 200.0, True)
    assert n_fixed > 0 and n_ad > 0
    assert n_ad * 5 <= n_fixed
