"""TEST INFRASTRUCTURE — CPU oracle of the HDR bloom and display transform.

A numpy restatement (float32 arithmetic, float16 storage between stages, as
the reference's rgba16f targets) of the realtime backends' post-process:
render/vulkan/shaders/bloom.hlsl:19-77 (Karis extract with soft knee, 7-tap
separable blur with clamp-to-edge) and blit.hlsl:43-57 (hdr + bloom *
strength, exposure, ACES).  The blur takes either the reference's weights or
a normalised Gaussian of sigma_px / 2 half-resolution texels.  Only tests/
use it, as the checker of singularity_gb300/csrc/sgx_post.cu.
"""

from __future__ import annotations

import math

import numpy as np

REF_WEIGHTS = np.array([0.071303, 0.131514, 0.189879, 0.214607, 0.189879, 0.131514, 0.071303], np.float32)
LUMA = np.array([0.2126, 0.7152, 0.0722], np.float32)


def weights(sigma_px: float) -> np.ndarray:
    if not sigma_px > 0:
        return REF_WEIGHTS
    s = sigma_px * 0.5
    r = min(max(int(math.ceil(3.0 * s)), 1), 32)
    k = np.exp(-0.5 * np.arange(-r, r + 1, dtype=np.float64) ** 2 / (s * s))
    return (k / k.sum()).astype(np.float32)


def _luma(x: np.ndarray) -> np.ndarray:
    return (x[..., 0] * LUMA[0] + x[..., 1] * LUMA[1] + x[..., 2] * LUMA[2]).astype(np.float32)


def extract(hdr: np.ndarray, threshold: float) -> np.ndarray:
    """hdr: (H, W, >=3) float16/float32 -> (H//2, W//2, 3) float16."""
    h = hdr[..., :3].astype(np.float32)
    H, W = h.shape[:2]
    bh, bw = max(1, H // 2), max(1, W // 2)
    a = h[0:2 * bh:2, 0:2 * bw:2]
    b = h[0:2 * bh:2, 1:2 * bw:2]
    c = h[1:2 * bh:2, 0:2 * bw:2]
    d = h[1:2 * bh:2, 1:2 * bw:2]
    one = np.float32(1)
    la, lb, lc, ld = (one / (one + _luma(x)) for x in (a, b, c, d))
    wden = np.maximum(la + lb + lc + ld, np.float32(1e-6))
    avg = (a * la[..., None] + b * lb[..., None] + c * lc[..., None] + d * ld[..., None]) / wden[..., None]
    l = _luma(avg)
    knee = (l * l) / np.maximum(l + np.float32(threshold), np.float32(1e-4))
    k = np.where(l > np.float32(1e-4), knee / np.where(l > 0, l, one), np.float32(0))
    return (avg * k[..., None]).astype(np.float16)


def blur(src: np.ndarray, w: np.ndarray, axis: int) -> np.ndarray:
    x = src.astype(np.float32)
    r = (len(w) - 1) // 2
    n = x.shape[axis]
    out = np.zeros_like(x)
    for i in range(-r, r + 1):
        idx = np.clip(np.arange(n) + i, 0, n - 1)
        out = out + np.take(x, idx, axis=axis) * w[i + r]
    return out.astype(np.float16)


def aces(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.float32)
    return np.clip((x * (np.float32(2.51) * x + np.float32(0.03))) / (x * (np.float32(2.43) * x + np.float32(0.59))
                                                                     + np.float32(0.14)), 0, 1)


def compose(hdr: np.ndarray, bloom: np.ndarray, strength: float, exposure: float) -> np.ndarray:
    """Bilinear (clamp to edge) half-res bloom at full-res pixel centres; returns ACES output, float32."""
    h = hdr[..., :3].astype(np.float32)
    H, W = h.shape[:2]
    bh, bw = bloom.shape[:2]
    b = bloom.astype(np.float32)
    tx = (np.arange(W, dtype=np.float32) + np.float32(0.5)) / np.float32(W) * np.float32(bw) - np.float32(0.5)
    ty = (np.arange(H, dtype=np.float32) + np.float32(0.5)) / np.float32(H) * np.float32(bh) - np.float32(0.5)
    fx0, fy0 = np.floor(tx), np.floor(ty)
    fx, fy = (tx - fx0)[None, :, None], (ty - fy0)[:, None, None]
    x0 = np.clip(fx0.astype(int), 0, bw - 1)
    x1 = np.clip(fx0.astype(int) + 1, 0, bw - 1)
    y0 = np.clip(fy0.astype(int), 0, bh - 1)
    y1 = np.clip(fy0.astype(int) + 1, 0, bh - 1)
    b00, b10 = b[y0][:, x0], b[y0][:, x1]
    b01, b11 = b[y1][:, x0], b[y1][:, x1]
    top = b00 + fx * (b10 - b00)
    bot = b01 + fx * (b11 - b01)
    bl = top + fy * (bot - top)
    c = (h + bl * np.float32(strength)) * np.float32(exposure)
    return aces(c)


def to_srgb_u8(c: np.ndarray) -> np.ndarray:
    c = np.clip(c.astype(np.float32), 0, 1)
    s = np.where(c <= np.float32(0.0031308), np.float32(12.92) * c,
                 np.float32(1.055) * np.power(c, np.float32(1 / 2.4)) - np.float32(0.055))
    return np.clip(s * np.float32(255) + np.float32(0.5), 0, 255).astype(np.uint8)


def bloom_pipeline(hdr: np.ndarray, threshold: float, strength: float, exposure: float,
                   sigma_px: float = 0.0) -> np.ndarray:
    """Full post-process of an HDR frame; returns the linear ACES output (H, W, 3) float32."""
    w = weights(sigma_px)
    a = extract(hdr, threshold)
    b = blur(a, w, axis=1)
    a = blur(b, w, axis=0)
    return compose(hdr, a, strength, exposure)
