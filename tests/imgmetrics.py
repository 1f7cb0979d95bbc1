"""Image comparison helpers for the tests.

``phash`` restates the perceptual hash the reference's golden tests use
(imagehash.phash with hash_size 8, verification/test_cuda_goldens.py:74-76):
luma conversion, a 32x32 Lanczos-windowed downsample, a 2-D DCT-II, the 8x8
low-frequency block thresholded at its median.  PIL's resampler is not
reproduced bit for bit, so distances are close to, not identical with, the
reference harness's.
"""

from __future__ import annotations

import struct
import zlib

import numpy as np


def _lanczos_weights(n_in: int, n_out: int, a: int = 3) -> np.ndarray:
    scale = n_in / n_out
    support = a * max(scale, 1.0)
    w = np.zeros((n_out, n_in))
    for i in range(n_out):
        center = (i + 0.5) * scale
        lo = int(np.floor(center - support))
        hi = int(np.ceil(center + support))
        xs = np.arange(max(lo, 0), min(hi, n_in))
        t = (xs + 0.5 - center) / max(scale, 1.0)
        k = np.sinc(t) * np.sinc(t / a)
        k[np.abs(t) >= a] = 0.0
        if k.sum() != 0:
            k = k / k.sum()
        w[i, xs] = k
    return w


def _dct_ii(x: np.ndarray, axis: int) -> np.ndarray:
    n = x.shape[axis]
    k = np.arange(n)
    basis = np.cos(np.pi * (2 * k[None, :] + 1) * k[:, None] / (2 * n)) * 2.0
    return np.moveaxis(np.tensordot(basis, np.moveaxis(x, axis, 0), axes=(1, 0)), 0, axis)


def phash(rgba: np.ndarray, hash_size: int = 8, highfreq_factor: int = 4) -> np.ndarray:
    img = np.asarray(rgba)[..., :3].astype(np.float64)
    luma = np.floor((img[..., 0] * 299 + img[..., 1] * 587 + img[..., 2] * 114) / 1000 + 0.5)
    n = hash_size * highfreq_factor
    small = _lanczos_weights(luma.shape[0], n) @ luma @ _lanczos_weights(luma.shape[1], n).T
    small = np.clip(np.floor(small + 0.5), 0, 255)
    d = _dct_ii(_dct_ii(small, 0), 1)
    low = d[:hash_size, :hash_size]
    return (low > np.median(low)).ravel()


def phash_distance(a: np.ndarray, b: np.ndarray) -> int:
    return int(np.count_nonzero(phash(a) != phash(b)))


def channel_error(a: np.ndarray, b: np.ndarray) -> dict:
    """Per-channel error of two RGBA8 images in units of 1/255 (RGB only)."""
    d = np.abs(a[..., :3].astype(np.int32) - b[..., :3].astype(np.int32))
    px = d.max(axis=-1)
    return {
        "mean": float(d.mean() / 255.0),
        "max": int(d.max()),
        "exact_frac": float((px == 0).mean()),
        "le1_frac": float((px <= 1).mean()),
        "gt16_frac": float((px > 16).mean()),
    }


def write_png(path, img: np.ndarray) -> None:
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w, c = img.shape
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    ct = {3: 2, 4: 6}[c]
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ct, 0, 0, 0))
                + chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def read_png(path) -> np.ndarray:
    """Decoder for the 8-bit RGB(A) PNGs this project and the CLI write."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
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
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, w * ch + 1)
    filt = raw[:, 0]
    if np.all(filt == 0):
        return raw[:, 1:].reshape(h, w, ch).copy()
    # the five PNG row filters (None, Sub, Up, Average, Paeth; PNG spec 9.2),
    # as stb_image_write (the reference CLI's writer) uses them
    out = np.zeros((h, w * ch), dtype=np.uint8)
    prev = np.zeros(w * ch, dtype=np.int32)
    for y in range(h):
        line = raw[y, 1:].astype(np.int32)
        f = int(filt[y])
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(w * ch, dtype=np.int32)
            ln, pv = line.tolist(), prev.tolist()
            cl = [0] * (w * ch)
            for x in range(w * ch):
                a = cl[x - ch] if x >= ch else 0
                b = pv[x]
                c = pv[x - ch] if x >= ch else 0
                if f == 1:
                    pred = a
                elif f == 3:
                    pred = (a + b) >> 1
                else:
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cl[x] = (ln[x] + pred) & 255
            cur = np.array(cl, dtype=np.int32)
        out[y] = cur
        prev = cur
    return out.reshape(h, w, ch)
