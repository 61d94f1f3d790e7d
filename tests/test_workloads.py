"""The seeded synthetic inputs standing in for the reference's missing datasets."""
import numpy as np

from vectorvisualization_gb300 import workloads as wl


def test_spectral_field_is_unit_rms_and_solenoidal():
    f = wl.spectral_field(32, seed=5).astype(np.float64)
    mag = np.sqrt((f ** 2).sum(-1))
    assert abs(np.sqrt((mag ** 2).mean()) - 1.0) < 1e-5
    # the encoder zeroes vectors shorter than 1e-5: almost none may be that short
    assert (mag < 1e-5).mean() < 1e-4
    # divergence in Fourier space: k . u_hat = 0 for every mode (layout (z, y, x, [x, y, z]))
    U = [np.fft.fftn(f[..., d]) for d in range(3)]
    k = np.fft.fftfreq(32, 1.0 / 32)
    KZ, KY, KX = np.meshgrid(k, k, k, indexing="ij")
    div = KX * U[0] + KY * U[1] + KZ * U[2]
    # Nyquist planes (|k| = n/2) have no sign and no spectral derivative: left out
    inner = (np.abs(KX) < 16) & (np.abs(KY) < 16) & (np.abs(KZ) < 16)
    assert np.abs(div[inner]).max() <= 1e-6 * np.abs(U[0]).max() * 32


def test_spectral_field_is_seeded():
    a = wl.spectral_field(16, seed=5)
    np.testing.assert_array_equal(a, wl.spectral_field(16, seed=5))
    assert not np.array_equal(a, wl.spectral_field(16, seed=6))
