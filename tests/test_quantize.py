"""The noise-gradient quantisation (quantize_unit in csrc/preprocess.cu), restated on the CPU.

The reference converts each unit gradient component c to a byte as
(unsigned char)(((double)c + 1.0) / 2.0 * 255.0) (gradient.cpp:466-477).  The kernel computes
t = fma(c, 127.5, 127.5) in float and returns floor(t) unless t lies within 1e-4 of an integer,
where it evaluates the double expression itself.  These tests check that the two agree on every
float32 within 2^14 ulps of each of the 256 integer crossings, on both signs of zero and the
interval ends, and on random components.  The float FMA is emulated as one rounding of the
product-sum formed in float64 (c * 127.5 + 127.5 is exact there); Python floats are IEEE doubles
with round-to-nearest, as the device's double arithmetic."""
import numpy as np

F32 = np.float32


def reference(c: np.ndarray) -> np.ndarray:
    d = ((c.astype(np.float64) + 1.0) / 2.0) * 255.0
    return np.trunc(d).astype(np.int64)  # values in (-1, 256): truncation toward zero


def kernel(c: np.ndarray) -> np.ndarray:
    t = (c.astype(np.float64) * 127.5 + 127.5).astype(F32)
    f = np.floor(t)
    r = t - f
    fast = (r > F32(1e-4)) & (r < F32(1.0) - F32(1e-4))
    return np.where(fast, f.astype(np.int64), reference(c))


def near_crossings(span: int = 1 << 14) -> np.ndarray:
    # c_k = 2k / 255 - 1 is where (c + 1) * 127.5 = k; every float32 within `span` ulps of it
    out = []
    for k in range(256):
        ck = F32(2.0 * k / 255.0 - 1.0)
        bits = np.array([ck], F32).view(np.int32)[0]
        offs = np.arange(-span, span + 1, dtype=np.int64)
        if ck == 0:
            continue
        cand = (bits + offs).astype(np.int32).view(F32)
        out.append(cand[np.isfinite(cand) & (np.abs(cand) <= 1.0)])
    return np.concatenate(out)


def test_quantisation_agrees_near_every_integer_crossing():
    c = near_crossings()
    assert c.size > 250 * (1 << 14)
    np.testing.assert_array_equal(kernel(c), reference(c))
    # the double fallback is taken only close to a crossing
    t = (c.astype(np.float64) * 127.5 + 127.5).astype(F32)
    r = t - np.floor(t)
    assert 0 < np.count_nonzero((r <= 1e-4) | (r >= 1 - 1e-4)) < c.size


def test_quantisation_agrees_on_ends_zeros_and_random_components():
    special = np.array([-1.0, 1.0, 0.0, -0.0, np.nextafter(F32(1), F32(2)), np.nextafter(F32(-1), F32(-2)),
                        np.nextafter(F32(0), F32(1)), np.nextafter(F32(0), F32(-1))], F32)
    np.testing.assert_array_equal(kernel(special), reference(special))
    rng = np.random.default_rng(466)
    c = (rng.random(4_000_000, dtype=np.float32) * F32(2) - F32(1)).astype(F32)
    np.testing.assert_array_equal(kernel(c), reference(c))
    # normalised gradients: components of unit vectors, as the filter pass produces them
    v = rng.standard_normal((1_000_000, 3)).astype(F32)
    v /= np.sqrt((v * v).sum(axis=1, keepdims=True)).astype(F32)
    np.testing.assert_array_equal(kernel(v.ravel()), reference(v.ravel()))
