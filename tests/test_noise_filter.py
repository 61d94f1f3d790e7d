"""The HYBRID sampler's noise filter (NoiseCells<false> in csrc/vvlic_device.cuh), restated in
FP32 on the CPU: each noise byte enters the 8-weight trilinear sum as the float 32768 + b and
the bias is subtracted once at the end.  Its error against the exact trilinear, in noise steps
(1/255 of the unit range), is bounded by 0.011 (max) with no bias; the exact form (NoiseCells<true>,
CELL) stays at float rounding.  fp32 FMA is emulated as one rounding of the product-sum formed
in float64 (the product of two floats is exact there)."""
import numpy as np

F32 = np.float32


def fma32(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F32)


def filters(n=400_000, seed=5):
    rng = np.random.default_rng(seed)
    ax, ay, az = (rng.random(n, dtype=np.float32) for _ in range(3))
    b = rng.integers(0, 256, (8, n)).astype(F32)
    one = F32(1)
    bx, by, bz = one - ax, one - ay, one - az
    w00, w10, w01, w11 = by * bz, ay * bz, by * az, ay * az
    w = [bx * w00, ax * w00, bx * w10, ax * w10, bx * w01, ax * w01, bx * w11, ax * w11]
    exact_form = np.zeros(n, F32)
    biased = np.zeros(n, F32)
    for i in range(8):
        exact_form = fma32(w[i], b[i], exact_form)
        biased = fma32(w[i], b[i] + F32(32768), biased)
    biased = biased - F32(32768)
    ref = np.zeros(n)
    for i in range(8):
        wx = ax.astype(np.float64) if i & 1 else 1.0 - ax.astype(np.float64)
        wy = ay.astype(np.float64) if i & 2 else 1.0 - ay.astype(np.float64)
        wz = az.astype(np.float64) if i & 4 else 1.0 - az.astype(np.float64)
        ref += wx * wy * wz * b[i]
    return exact_form.astype(np.float64) - ref, biased.astype(np.float64) - ref


def test_bias_bytes_are_exact():
    # 0x4700bb00 is 2^15 * (1 + b * 2^8 / 2^23) = 32768 + b for every byte b
    b = np.arange(256, dtype=np.uint32)
    v = (np.uint32(0x47000000) | (b << np.uint32(8))).view(np.float32)
    np.testing.assert_array_equal(v, 32768.0 + b.astype(np.float32))


def test_biased_filter_error_bound():
    e_exact, e_biased = filters()
    assert np.abs(e_exact).max() < 1e-4
    assert np.abs(e_biased).max() < 0.011
    assert np.sqrt(np.mean(e_biased ** 2)) < 0.0025
    assert abs(float(e_biased.mean())) < 2e-4
