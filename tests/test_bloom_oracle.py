"""The bloom oracle's own invariants (no GPU): kernel weights and the soft knee."""

import numpy as np


def test_weights():
    from oracle import bloom_oracle as B
    assert np.isclose(B.REF_WEIGHTS.sum(), 1.0, atol=1e-5)
    for s in (1.0, 4.0, 8.0, 16.0):
        w = B.weights(s)
        assert np.isclose(w.sum(), 1.0, atol=1e-6) and len(w) % 2 == 1 and np.allclose(w, w[::-1])
    assert len(B.weights(8.0)) == 25  # sigma 4 half-res texels, radius 12


def test_extract_threshold_and_black():
    from oracle import bloom_oracle as B
    hdr = np.zeros((8, 8, 4), np.float16)
    assert np.all(B.extract(hdr, 0.8) == 0)
    hdr[..., :3] = 10.0
    e = B.extract(hdr, 0.8).astype(np.float32)
    # uniform input: the Karis average is the input, scaled by l / (l + threshold)
    assert np.allclose(e, 10.0 * 10.0 / 10.8, rtol=2e-3)
    out = B.bloom_pipeline(hdr, 0.8, 0.55, 1.8)
    assert out.shape == (8, 8, 3) and np.all((out >= 0) & (out <= 1))
