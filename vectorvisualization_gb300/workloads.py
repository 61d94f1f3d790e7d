"""Seeded synthetic inputs and the named render configurations.

The reference ships no datasets (its .dat/.raw volumes, noise files, filter PNGs and colour
tables are not in the repository), so fields, noise, filters and transfer functions are
generated here from seeded SplitMix64 streams:

* C1  64^3 ABC flow, sparse noise, Euler L=20, box filter, 256^2 orthographic, spacing 1/128.
* C2  256^3 drift + 8 Gaussian vortices, dense noise (freq 4.0), Heun L=40 h=0.005, Gaussian
      filter, 1024^2, spacing 1/256, central-difference gradient lighting; FP32/FP16/BF16 field.
* C4  128^3 vortex field, dense noise, Heun L=30, 512^2 x 4 views.
* C5  512^3 divergence-free spectral field (E(k) ~ k^-5/3, k in [2, 64]), RK4 L=60, h=1/512,
      2048^2, spacing 1/512, lighting.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import capi


class LibraryDefaults:
    """Parameter, view and filter-table defaults of libvvlic (vvlic_params_default,
    vvlic_view_default, vvlic_make_filter_table).  Every configuration below takes a `defaults`
    provider with these three callables; another provider (the oracle's own restatement) builds
    the same configuration without the library."""

    params = staticmethod(capi.params_default)
    view = staticmethod(capi.view_default)
    filter_table = staticmethod(capi.make_filter_table)


LIBRARY = LibraryDefaults()

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


class SplitMix64:
    """SplitMix64 stream: the k-th output mixes seed + k * golden (k = 1, 2, ...)."""

    def __init__(self, seed: int):
        self.seed = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.k = 0

    def u64(self, n: int) -> np.ndarray:
        idx = np.arange(self.k + 1, self.k + n + 1, dtype=np.uint64)
        self.k += n
        with np.errstate(over="ignore"):
            z = self.seed + idx * _GOLDEN
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            return z ^ (z >> np.uint64(31))

    def uniform(self, n: int) -> np.ndarray:
        """doubles in [0, 1)"""
        return (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def normal(self, n: int) -> np.ndarray:
        u1 = self.uniform(n)
        u2 = self.uniform(n)
        return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


# -------------------------------------------------------------------------------------------
# vector fields, shape (nz, ny, nx, 3) float32, sampled at voxel centres
# -------------------------------------------------------------------------------------------
def _centres(n: int) -> np.ndarray:
    return (np.arange(n, dtype=np.float64) + 0.5) / n


def abc_field(n, A=math.sqrt(3.0), B=math.sqrt(2.0), Cc=1.0) -> np.ndarray:
    """Arnold-Beltrami-Childress flow on [0, 2pi]^3."""
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    x = _centres(nx) * 2 * math.pi
    y = _centres(ny) * 2 * math.pi
    z = _centres(nz) * 2 * math.pi
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    v = np.empty(X.shape + (3,), np.float32)
    v[..., 0] = A * np.sin(Z) + Cc * np.cos(Y)
    v[..., 1] = B * np.sin(X) + A * np.cos(Z)
    v[..., 2] = Cc * np.sin(Y) + B * np.cos(X)
    return v


def vortex_field(n, seed: int, count: int = 8, drift=(0.2, 0.0, 0.0)) -> np.ndarray:
    """Uniform drift plus `count` Gaussian vortices: s * exp(-r^2/R^2) * (a x (x - c))."""
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    rng = SplitMix64(seed)
    c = rng.uniform(3 * count).reshape(count, 3)
    R = 0.05 + 0.15 * rng.uniform(count)
    s = rng.normal(count)
    a = rng.normal(3 * count).reshape(count, 3)
    a /= np.linalg.norm(a, axis=1, keepdims=True)
    x, y, z = _centres(nx), _centres(ny), _centres(nz)
    v = np.empty((nz, ny, nx, 3), np.float32)
    Y, X = np.meshgrid(y, x, indexing="ij")
    for k in range(nz):
        vz = np.zeros((ny, nx, 3), np.float64)
        vz[..., 0] += drift[0]
        vz[..., 1] += drift[1]
        vz[..., 2] += drift[2]
        for i in range(count):
            d = np.stack([X - c[i, 0], Y - c[i, 1], np.full_like(X, z[k] - c[i, 2])], axis=-1)
            g = s[i] * np.exp(-np.sum(d * d, axis=-1) / (R[i] * R[i]))
            vz += g[..., None] * np.cross(a[i], d)
        v[k] = vz
    return v


def spectral_field(n: int, seed: int, kmin: float = 2.0, kmax: float = 64.0, device: str | None = None) -> np.ndarray:
    """Divergence-free random-phase field with E(k) ~ k^(-5/3) on kmin <= |k| <= kmax.

    Complex Gaussian modes are scaled so that the shell energy follows k^(-5/3), projected onto
    the plane orthogonal to k (solenoidal) and inverse-transformed (torch.fft on `device` when
    given, numpy otherwise), then scaled to unit RMS magnitude: the unnormalised inverse
    transform shrinks as n^-3 (about 1e-7 at 512^3), below the 1e-5 zero-vector threshold of the
    field encoding.  Returns (n, n, n, 3) float32."""
    rng = SplitMix64(seed)
    kx = np.fft.fftfreq(n, 1.0 / n)
    kz = np.fft.rfftfreq(n, 1.0 / n)
    K = [kx[:, None, None], kx[None, :, None], kz[None, None, :]]  # axes (x, y, z-half)
    shape = (n, n, n // 2 + 1)
    k2 = K[0] ** 2 + K[1] ** 2 + K[2] ** 2
    kmag = np.sqrt(k2)
    band = (kmag >= kmin) & (kmag <= kmax)
    # E(k) ~ k^-5/3 over shells of area ~k^2: per-mode amplitude ~ k^(-11/6)
    amp = np.where(band, np.power(np.maximum(kmag, 1e-12), -11.0 / 6.0), 0.0).astype(np.float32)
    size = int(np.prod(shape))
    comps = []
    for _ in range(3):
        re = rng.normal(size).reshape(shape).astype(np.float32)
        im = rng.normal(size).reshape(shape).astype(np.float32)
        comps.append((re + 1j * im).astype(np.complex64) * amp)
    # solenoidal projection: u - k (k.u)/|k|^2
    kdotu = K[0] * comps[0] + K[1] * comps[1] + K[2] * comps[2]
    inv = np.where(k2 > 0, 1.0 / np.maximum(k2, 1e-12), 0.0).astype(np.float32)
    out = np.empty((n, n, n, 3), np.float32)
    for d in range(3):
        u = (comps[d] - K[d] * kdotu * inv).astype(np.complex64)
        if device is not None:
            import torch

            t = torch.fft.irfftn(torch.from_numpy(u).to(device), s=(n, n, n))
            r = t.float().cpu().numpy()
        else:
            r = np.fft.irfftn(u, s=(n, n, n), axes=(0, 1, 2)).astype(np.float32)
        # array axes are (x, y, z); the field layout is (z, y, x)
        out[..., d] = np.transpose(r, (2, 1, 0))
    rms = float(np.sqrt(np.einsum("zyxc,zyxc->", out, out, dtype=np.float64) / (n ** 3)))
    if rms > 0:
        out *= np.float32(1.0 / rms)
    return out


# -------------------------------------------------------------------------------------------
# noise, transfer functions
# -------------------------------------------------------------------------------------------
def sparse_noise(m, seed: int, p: float = 0.05) -> np.ndarray:
    mx, my, mz = (m, m, m) if np.isscalar(m) else m
    u = SplitMix64(seed).uniform(mx * my * mz)
    return np.where(u < p, 255, 0).astype(np.uint8).reshape(mz, my, mx)


def dense_noise(m, seed: int) -> np.ndarray:
    mx, my, mz = (m, m, m) if np.isscalar(m) else m
    u = SplitMix64(seed).uniform(mx * my * mz)
    return np.minimum(np.floor(u * 256.0), 255).astype(np.uint8).reshape(mz, my, mx)


def default_tf() -> tuple[np.ndarray, np.ndarray]:
    """TransferEdit's default tables (transferEdit.cpp:76-82): rgb = i, alpha = opacity =
    max(0, i - 20), divided by 255.  With tf_index = magnitude this is the linear ramp on |v|."""
    i = np.arange(capi.TF_ENTRIES, dtype=np.float32)
    rgba = np.empty((capi.TF_ENTRIES, 4), np.float32)
    rgba[:, 0] = rgba[:, 1] = rgba[:, 2] = i / 255.0
    ao = np.where(i < 20, 0, i - 20).astype(np.float32) / 255.0
    rgba[:, 3] = ao
    return rgba, ao.copy()


def random_tf(seed: int, knots: int = 8) -> tuple[np.ndarray, np.ndarray]:
    """A smooth seeded TF: piecewise-linear through `knots` random control points per channel."""
    rng = SplitMix64(seed)
    xs = np.linspace(0, 1, knots)
    t = (np.arange(capi.TF_ENTRIES) + 0.5) / capi.TF_ENTRIES
    rgba = np.empty((capi.TF_ENTRIES, 4), np.float32)
    for ch in range(4):
        ys = rng.uniform(knots)
        rgba[:, ch] = np.interp(t, xs, ys)
    op = np.interp(t, xs, rng.uniform(knots)).astype(np.float32)
    return rgba, op


# -------------------------------------------------------------------------------------------
# views
# -------------------------------------------------------------------------------------------
def quat_axis_angle(axis, deg: float) -> tuple[float, float, float, float]:
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    h = math.radians(deg) / 2.0
    s = math.sin(h)
    return (a[0] * s, a[1] * s, a[2] * s, math.cos(h))


def quat_mul(q, r):
    x1, y1, z1, w1 = q
    x2, y2, z2, w2 = r
    return (
        w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
        w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2,
        w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2,
        w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2,
    )


def ortho_view(center=(0.5, 0.5, 0.5), right=(0.5, 0.0, 0.0), up=(0.0, 0.5, 0.0), direction=(0.0, 0.0, 1.0),
               defaults=LIBRARY) -> capi.View:
    v = defaults.view()
    v.projection = capi.ORTHOGRAPHIC
    for i in range(3):
        v.ortho_center[i] = center[i]
        v.ortho_right[i] = right[i]
        v.ortho_up[i] = up[i]
        v.ortho_dir[i] = direction[i]
    return v


def perspective_view(quat=(0.0, 0.0, 0.0, 1.0), distance: float = 4.0, fovy: float = 35.0, pan=(0.0, 0.0, 0.0),
                     defaults=LIBRARY) -> capi.View:
    v = defaults.view()
    v.projection = capi.PERSPECTIVE
    for i in range(4):
        v.quat[i] = quat[i]
    for i in range(3):
        v.pan[i] = pan[i]
    v.distance = distance
    v.fovy_deg = fovy
    return v


def orbit_view(frame: int, frames: int, distance: float = 2.2, tilt: float = 25.0, defaults=LIBRARY) -> capi.View:
    q = quat_mul(quat_axis_angle((1, 0, 0), tilt), quat_axis_angle((0, 1, 0), 360.0 * frame / frames))
    return perspective_view(q, distance, defaults=defaults)


def random_view(rng: SplitMix64, distance: float = 2.4, defaults=LIBRARY) -> capi.View:
    u = rng.uniform(3)
    q = quat_mul(quat_axis_angle((1, 0, 0), 80.0 * (u[0] - 0.5)), quat_axis_angle((0, 1, 0), 360.0 * u[1]))
    return perspective_view(q, distance * (0.9 + 0.2 * u[2]), defaults=defaults)


# -------------------------------------------------------------------------------------------
# named configurations
# -------------------------------------------------------------------------------------------
@dataclass
class Workload:
    name: str
    field: np.ndarray                 # (nz, ny, nx, 3) float32
    noise: np.ndarray                 # (mz, my, mx) uint8
    noise_mode: int
    filter_table: np.ndarray
    filter_kind: str
    tf_rgba: np.ndarray
    tf_opac: np.ndarray
    params: capi.Params
    views: list = field(default_factory=list)
    width: int = 256
    height: int = 256
    storage: str = "f32"
    seeds: dict = field(default_factory=dict)

    def describe(self) -> dict:
        p = self.params
        nz, ny, nx = self.field.shape[:3]
        return {
            "workload": self.name,
            "field": f"{nx}x{ny}x{nz}",
            "noise": "x".join(str(s) for s in self.noise.shape[::-1]),
            "image": f"{self.width}x{self.height}",
            "views": len(self.views),
            "integrator": ["euler", "heun", "rk4"][p.integrator],
            "L": [int(p.steps_backward), int(p.steps_forward)],
            "step_lic": float(p.step_size_lic),
            "spacing": float(p.step_size_vol),
            "filter": self.filter_kind,
            "illum": ["none", "gradient", "zoeckler", "mallo"][p.illum],
            "storage": self.storage,
            "seeds": self.seeds,
        }


def c1(size: int = 64, image: int = 256, defaults=LIBRARY) -> Workload:
    """Plain method, small: the reference's CPU-runnable case."""
    p = defaults.params()
    p.integrator = capi.EULER
    p.steps_forward = p.steps_backward = 20
    p.step_size_lic = 0.01
    p.step_size_vol = 1.0 / 128.0
    p.tf_index = capi.TF_INDEX_MAGNITUDE
    p.illum = capi.ILLUM_NONE
    rgba, op = default_tf()
    return Workload(
        name=f"C1 ABC {size}^3 sparse-noise Euler L=20 box {image}^2 ortho",
        field=abc_field(size),
        noise=sparse_noise(size, seed=1),
        noise_mode=capi.NOISE_SCALAR,
        filter_table=defaults.filter_table("box", 256),
        filter_kind="box",
        tf_rgba=rgba,
        tf_opac=op,
        params=p,
        views=[ortho_view(defaults=defaults)],
        width=image,
        height=image,
        seeds={"noise": 1},
    )


def c2_view(defaults=LIBRARY) -> capi.View:
    q = quat_mul(quat_axis_angle((1, 0, 0), 20.0), quat_axis_angle((0, 1, 0), 30.0))
    return perspective_view(q, distance=2.3, defaults=defaults)


def c2(size: int = 256, image: int = 1024, storage: str = "f32", lighting: bool = True, defaults=LIBRARY) -> Workload:
    """Mid-size with lighting and precision."""
    p = defaults.params()
    p.integrator = capi.HEUN
    p.steps_forward = p.steps_backward = 40
    p.step_size_lic = 0.005
    p.step_size_vol = 1.0 / 256.0
    p.freq_scale = 4.0
    p.tf_index = capi.TF_INDEX_MAGNITUDE
    p.illum = capi.ILLUM_GRADIENT if lighting else capi.ILLUM_NONE
    rgba, op = default_tf()
    return Workload(
        name=f"C2 vortex {size}^3 dense-noise Heun L=40 gaussian {image}^2 {'lit' if lighting else 'unlit'} {storage}",
        field=vortex_field(size, seed=2),
        noise=dense_noise(size, seed=20),
        noise_mode=capi.NOISE_GRAD_CENTRAL if lighting else capi.NOISE_SCALAR,
        filter_table=defaults.filter_table("gaussian", 256),
        filter_kind="gaussian",
        tf_rgba=rgba,
        tf_opac=op,
        params=p,
        views=[c2_view(defaults)],
        width=image,
        height=image,
        storage=storage,
        seeds={"field": 2, "noise": 20},
    )


def c4(size: int = 128, image: int = 512, views: int = 4, defaults=LIBRARY) -> Workload:
    """Differentiable TF / filter fit setting (forward part)."""
    p = defaults.params()
    p.integrator = capi.HEUN
    p.steps_forward = p.steps_backward = 30
    p.step_size_lic = 0.01
    p.step_size_vol = 1.0 / 128.0
    p.tf_index = capi.TF_INDEX_MAGNITUDE
    rgba, op = random_tf(seed=404)
    rng = SplitMix64(44)
    return Workload(
        name=f"C4 vortex {size}^3 dense-noise Heun L=30 {image}^2 x{views}",
        field=vortex_field(size, seed=4),
        noise=dense_noise(size, seed=40),
        noise_mode=capi.NOISE_SCALAR,
        filter_table=defaults.filter_table("gaussian", 256),
        filter_kind="gaussian",
        tf_rgba=rgba,
        tf_opac=op,
        params=p,
        views=[random_view(rng, defaults=defaults) for _ in range(views)],
        width=image,
        height=image,
        seeds={"field": 4, "noise": 40, "tf": 404, "views": 44},
    )


@dataclass
class BatchVolume:
    field: np.ndarray
    kind: str
    seed: int
    views: list
    L: int
    filter_kind: str


def c3(volumes: int = 64, image: int = 512, seed: int = 3, max_views: int = 8, dims=tuple(range(64, 193, 16)),
       defaults=LIBRARY):
    """Batched uneven volumes: per-axis dims from {64, 80, ..., 192}, each an ABC or a vortex field
    from its own seed, 1..max_views random views at image^2, filters mixed box / triangle / cos^2,
    L in [15, 60].  Returns (volumes, shared noise, base params)."""
    rng = SplitMix64(seed)
    out = []
    kinds = ("box", "triangle", "cos2")
    for v in range(volumes):
        u = rng.uniform(7)
        n = tuple(int(dims[min(int(u[i] * len(dims)), len(dims) - 1)]) for i in range(3))
        vseed = 1000 + v
        kind = "abc" if u[3] < 0.5 else "vortex"
        field = abc_field(n) if kind == "abc" else vortex_field(n, seed=vseed)
        nviews = 1 + min(int(u[4] * max_views), max_views - 1)
        vr = SplitMix64(vseed * 7 + 1)
        views = [random_view(vr, defaults=defaults) for _ in range(nviews)]
        L = 15 + min(int(u[5] * 46), 45)
        out.append(BatchVolume(field, kind, vseed, views, L, kinds[min(int(u[6] * 3), 2)]))
    p = defaults.params()
    p.integrator = capi.HEUN
    p.step_size_lic = 0.01
    p.step_size_vol = 1.0 / 128.0
    p.tf_index = capi.TF_INDEX_MAGNITUDE
    return out, dense_noise(128, seed=seed * 10), p


def c3_jobs(vols, image: int = 512):
    """The batch's jobs in order, (volume, view) pairs, with a cost estimate per job for
    dealing them over replicas: pixels x taps (the random views' chords are alike)."""
    jobs = [(bv, v) for bv in vols for v in bv.views]
    return jobs, [image * image * (2 * bv.L + 1) for bv, _ in jobs]


def c5(size: int = 512, image: int = 2048, frames: int = 64, device: str | None = None,
       defaults=LIBRARY) -> Workload:
    """Large turbulence orbit (spectral field via torch.fft on `device`, numpy otherwise)."""
    p = defaults.params()
    p.integrator = capi.RK4
    p.steps_forward = p.steps_backward = 60
    p.step_size_lic = 1.0 / 512.0
    p.step_size_vol = 1.0 / 512.0
    p.tf_index = capi.TF_INDEX_MAGNITUDE
    p.illum = capi.ILLUM_GRADIENT
    rgba, op = default_tf()
    return Workload(
        name=f"C5 spectral {size}^3 RK4 L=60 {image}^2 orbit x{frames} lit f16",
        field=spectral_field(size, seed=5, device=device),
        noise=dense_noise(size, seed=50),
        noise_mode=capi.NOISE_GRAD_CENTRAL,
        filter_table=defaults.filter_table("gaussian", 256),
        filter_kind="gaussian",
        tf_rgba=rgba,
        tf_opac=op,
        params=p,
        views=[orbit_view(f, frames, defaults=defaults) for f in range(frames)],
        width=image,
        height=image,
        storage="f16",
        seeds={"field": 5, "noise": 50},
    )


def setup_context(ctx: capi.Context, w: Workload, storage: str | None = None) -> int:
    """Upload a workload into a context; returns the volume id."""
    vid = ctx.upload_field(w.field, storage=storage or w.storage)
    ctx.upload_noise(w.noise, w.noise_mode)
    ctx.set_filter_table(w.filter_table)
    ctx.set_tf(w.tf_rgba, w.tf_opac)
    ctx.set_params(w.params)
    ctx.set_view(w.views[0])
    return vid
