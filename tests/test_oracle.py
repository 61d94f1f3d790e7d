"""CPU tests of the oracle: pins against the reference's own code and GL-semantics unit tests.

The reference has no tests and ships none of its inputs, so its GLSL math cannot be run here
(it needs an OpenGL stack).  What can be pinned is pinned:
  * noise gradients against the reference's gradient.cpp (compiled by oracle/build_ref.sh when
    the reference checkout is present; the committed fixtures in tests/golden otherwise);
  * the restated GL sampler / integrator / blend semantics against closed-form cases.
"""
import math

import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

GOLDEN = None


def golden():
    global GOLDEN
    if GOLDEN is None:
        import os

        GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "noise_gradients.npz"))
    return GOLDEN


CASES = ["dense_11x13x17", "sparse_24", "dense_16_aniso", "tiny_3x4x5"]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode,tag", [(capi.NOISE_GRAD_SOBEL, "sobel"), (capi.NOISE_GRAD_CENTRAL, "central")])
def test_noise_gradients_match_reference_fixture(oracle, case, mode, tag):
    g = golden()
    noise = g[f"{case}/noise"]
    got = oracle.noise_gradients(noise, mode, g[f"{case}/slice_dist"])
    np.testing.assert_array_equal(got, g[f"{case}/{tag}"])


def test_golden_noise_regenerates(oracle):
    """The fixtures' noise volumes come from the seeded generator (no hidden inputs)."""
    g = golden()
    np.testing.assert_array_equal(g["dense_11x13x17/noise"], wl.dense_noise((11, 13, 17), 3))
    np.testing.assert_array_equal(g["sparse_24/noise"], wl.sparse_noise(24, 7))


@pytest.mark.parametrize("mode", [capi.NOISE_GRAD_SOBEL, capi.NOISE_GRAD_CENTRAL])
def test_noise_gradients_match_compiled_reference(oracle, mode):
    if not oracle.ref_available():
        pytest.skip("reference gradient code not built here (oracle/build_ref.sh)")
    for dims, seed in [((20, 9, 14), 21), ((33, 32, 31), 22)]:
        noise = wl.dense_noise(dims, seed)
        np.testing.assert_array_equal(oracle.noise_gradients(noise, mode), oracle.ref_noise_gradients(noise, mode))


def test_noise_filter_weights(oracle):
    w = oracle.noise_filter_weights()
    assert w.shape == (27,)
    assert abs(float(w.sum()) - 1.0) < 1e-6
    # index (k, j, i) over [-2, 0]^3; the largest weight sits at offset (0, 0, 0)
    assert int(np.argmax(w)) == 26
    r2 = np.array([i * i + j * j + k * k for k in range(-2, 1) for j in range(-2, 1) for i in range(-2, 1)], float)
    np.testing.assert_allclose(w / w[26], np.exp(-r2 / 5.0), rtol=1e-6)


def test_encode_field_closed_form(oracle):
    v = np.zeros((2, 2, 3, 3), np.float32)
    v[0, 0, 0] = (3.0, 0.0, 4.0)   # |v| = 5 (the maximum)
    v[0, 0, 1] = (0.0, -2.0, 0.0)  # |v| = 2
    v[1, 1, 2] = (1e-7, 0, 0)      # below EPS: zero vector
    rgba = oracle.encode_field(v)
    np.testing.assert_allclose(rgba[0, 0, 0], [0.5 + 0.5 * 0.6, 0.5, 0.5 + 0.5 * 0.8, 1.0], rtol=1e-7)
    np.testing.assert_allclose(rgba[0, 0, 1], [0.5, 0.0, 0.5, 0.4], rtol=1e-7)
    np.testing.assert_array_equal(rgba[1, 1, 2], [0.5, 0.5, 0.5, 0.0])
    np.testing.assert_array_equal(rgba[1, 0, 0], [0.5, 0.5, 0.5, 0.0])


def test_encode_uint8_wraps_like_reference(oracle):
    # dataset.cpp subtracts 128 from unsigned char: 0 -> 128, 128 -> 0, 255 -> 127
    v = np.array([[[[0, 128, 128], [128, 255, 128]]]], np.uint8)
    rgba = oracle.encode_field(v)
    np.testing.assert_allclose(rgba[0, 0, 0], [1.0, 0.5, 0.5, 1.0], rtol=1e-7)
    np.testing.assert_allclose(rgba[0, 0, 1, :3], [0.5, 1.0, 0.5], rtol=1e-7)
    assert abs(rgba[0, 0, 1, 3] - 127.0 / 128.0) < 1e-7


def test_encode_interp_lerp_closed_form(oracle):
    # t = index/size, each component data + t*(next - data) in float32 (dataset.cpp:593)
    rng = np.random.default_rng(5)
    a0 = rng.standard_normal((3, 4, 5, 3)).astype(np.float32)
    a1 = rng.standard_normal((3, 4, 5, 3)).astype(np.float32)
    for index, size in ((0, 1), (1, 3), (7, 8)):
        t = np.float32(index) / np.float32(size)
        lerp = a0 + t * (a1 - a0)
        np.testing.assert_array_equal(oracle.encode_field_interp(a0, a1, index, size), oracle.encode_field(lerp))
    np.testing.assert_array_equal(oracle.encode_field_interp(a0, a1, 0, 4), oracle.encode_field(a0))


def test_encode_interp_uint8_truncates(oracle):
    # bytes 130 and 135 are 2 and 7 after the -128 wrap; at t = 1/2: 2 + 0.5*5 = 4.5 -> 4 (byte 132)
    a0 = np.full((1, 1, 2, 3), 128, np.uint8)
    a1 = a0.copy()
    a0[0, 0, 0, 0], a1[0, 0, 0, 0] = 130, 135
    a0[0, 0, 1, 1], a1[0, 0, 1, 1] = 0, 255   # 128 and 127 (the wrap): 128 - 0.5 = 127.5 -> 127
    want = a0.copy()
    want[0, 0, 0, 0] = 132
    want[0, 0, 1, 1] = 255
    np.testing.assert_array_equal(oracle.encode_field_interp(a0, a1, 1, 2), oracle.encode_field(want))


def _unorm8(v):
    return np.floor(np.clip(np.asarray(v, np.float32).astype(np.float64), 0, 1) * 255 + 0.5).astype(np.int64)


def test_zoeckler_table_matches_numpy_restatement(oracle):
    # illumination.cpp:96-172 with the default LineMat, vectorised in numpy (float64 throughout,
    # ambient*lightColor and the 0.9 factor in float32 as in the reference)
    luts = oracle.illum_luts()
    assert luts.shape == (3, 256, 256, 4)
    x = np.arange(256)
    lt = 2.0 * (x * (1.0 / 255)) - 1.0
    LT, VT = np.meshgrid(lt, lt)
    diff = np.sqrt(1 - LT * LT) ** 2.0
    dp = np.clip(LT * VT - np.sqrt(1 - LT * LT) * np.sqrt(1 - VT * VT), -1, 1)
    td = np.clip((float(np.float32(0.1)) + diff * float(np.float32(0.5))) * 0.5, 0, 1)
    ts = np.clip(np.abs(dp) ** 40.0 * float(np.float32(0.8)) * 0.5, 0, 1)
    z = luts[0].astype(np.int64)
    assert np.abs(z[..., 0] - _unorm8(td)).max() <= 1
    assert np.abs(z[..., 3] - _unorm8(ts.astype(np.float32) * np.float32(0.9))).max() <= 1
    np.testing.assert_array_equal(z[..., 0], z[..., 1])  # LUMINANCE_ALPHA reads (L, L, L, A)
    # lt = +-1: no diffuse term, only ambient 0.1 halved -> round(12.75) = 13
    assert (z[:, 0, 0] == 13).all() and (z[:, 255, 0] == 13).all()


def test_mallo_tables_match_numpy_restatement(oracle):
    luts = oracle.illum_luts()
    s = (np.arange(256) + 0.5) / 256
    alpha = np.arccos(2 * s - 1)[None, :]
    beta = np.arccos(2 * s - 1)[:, None]
    lt = (2 * s - 1)[:, None]
    fd = np.sqrt(1 - lt * lt) * (np.sin(alpha) + (np.pi - alpha) * np.cos(alpha)) * 0.25
    # Simpson, 20 intervals over [alpha - pi/2, pi/2] of max(0, cos(th - beta))^40 cos(th) / 2
    a = alpha - np.pi / 2
    hstep = (np.pi / 2 - a) / 20
    f = lambda th: np.maximum(np.cos(th - beta), 0) ** 40.0 * (np.cos(th) / 2)
    acc = sum((2.0 if i % 2 == 0 else 4.0) * f(a + i * hstep) for i in range(20)) + f(a + 20 * hstep) - f(a)
    fs = 3.5 * acc * (hstep / 3)
    md, ms = luts[1].astype(np.int64), luts[2].astype(np.int64)
    for c in range(4):
        assert np.abs(md[..., c] - _unorm8(np.clip(fd * float(np.float32(0.5)), 0, 1))).max() <= 1
        assert np.abs(ms[..., c] - _unorm8(np.clip(fs * float(np.float32(0.8)), 0, 1))).max() <= 1
    # the Simpson sum approximates the exact integral (a smooth check on the specular table)
    from scipy.integrate import quad

    for i, j in [(40, 200), (128, 128), (220, 60)]:
        al, be = float(alpha[0, i]), float(beta[j, 0])
        exact, _ = quad(lambda th: max(np.cos(th - be), 0) ** 40 * np.cos(th) / 2, al - np.pi / 2, np.pi / 2)
        assert abs(fs[j, i] / 3.5 - exact) <= 0.02 * max(exact, 1e-3) + 1e-4


def test_line_material_size_rounds_to_power_of_two(oracle):
    from vectorvisualization_gb300 import capi

    m = capi.line_material_default()
    m.width, m.height = 100, 60
    assert oracle.illum_luts(m).shape == (3, 64, 128, 4)


def test_storage_rounding_matches_numpy(oracle):
    x = np.concatenate([np.linspace(0, 1, 10001, dtype=np.float32), np.float32([1e-5, 6.1e-5, 3.3e-7, 0.999999])])
    np.testing.assert_array_equal(oracle.round_storage(x, "f16"), x.astype(np.float16).astype(np.float32))
    import torch

    np.testing.assert_array_equal(oracle.round_storage(x, "bf16"), torch.from_numpy(x).bfloat16().float().numpy())


def test_filter_taps_gl_clamp_border(oracle):
    box = capi.make_filter_table("box", 256)
    assert box.size == 256 and np.all(box == 255)
    t = oracle.filter_taps(box, 20, 20)
    # the outermost taps sit at s = 0 and s = 1 and blend half with the zero border
    assert abs(t[0] - 0.5) < 1e-12 and abs(t[-1] - 0.5) < 1e-12
    np.testing.assert_allclose(t[1:-1], 1.0)
    t2 = oracle.filter_taps(box, 20, 20, capi.KERNEL_CLAMP_EDGE)
    np.testing.assert_allclose(t2, 1.0)
    assert oracle.filter_inv_area(box, True) == 0.5


def test_filter_tables_shapes():
    for kind in ("triangle", "cos2", "gaussian"):
        t = capi.make_filter_table(kind, 256)
        assert t.size == 256
        assert t[127] >= 250 and t[128] >= 250  # peak at the centre
        assert t[0] < t[64] < t[127]
        np.testing.assert_array_equal(t, t[::-1])  # symmetric
    assert capi.make_filter_table("box", 100).size == 128  # nextPowerTwo


def test_geometry_matches_reference_formulas(oracle):
    g = oracle.geometry([64, 80, 128])
    np.testing.assert_allclose(g["extent"], [0.5, 0.625, 1.0])
    np.testing.assert_allclose(g["scale"], [2.0, 1.6, 1.0])
    np.testing.assert_allclose(g["tex_max"], [1.0, 1.0, 1.0])
    np.testing.assert_allclose(g["center"], [0.25, 0.3125, 0.5])


def _constant_scene(oracle, direction, n=8, noise=None, tf=None):
    d = np.asarray(direction, np.float32)
    v = np.broadcast_to(d, (n, n, n, 3)).copy()
    rgba = oracle.encode_field(v)
    if noise is None:
        noise = np.full((n, n, n), 255, np.uint8)
    rgba_tf, op = tf if tf is not None else wl.default_tf()
    return oracle.Scene(rgba, noise, rgba_tf, op, filter_table=capi.make_filter_table("box", 256))


def test_ortho_ray_sample_count(oracle):
    sc = _constant_scene(oracle, (1, 0, 0))
    p = capi.params_default()
    p.steps_forward = p.steps_backward = 2
    p.step_size_vol = 1.0 / 16.0
    p.gradient_scale = 0.0  # transparent: no early termination
    img, smp = sc.render(p, wl.ortho_view(), 4, 4)
    # z = 0, 1/16, ..., 16/16: 17 samples per ray, the last one exactly on the far face
    assert np.all(smp == 17)
    np.testing.assert_array_equal(img, 0.0)


def test_perspective_rays_hit_and_miss(oracle):
    sc = _constant_scene(oracle, (1, 0, 0))
    p = capi.params_default()
    p.steps_forward = p.steps_backward = 1
    p.gradient_scale = 0.0
    img, smp = sc.render(p, wl.perspective_view(distance=4.0), 32, 32)
    assert smp[0, 0] == 0 and smp[16, 16] > 0  # corners miss, centre hits
    assert smp.sum() > 0


def test_constant_noise_lic_intensity(oracle):
    """With noise 255 everywhere, I = sum(taps) * invArea / (Lf+Lb) * gradientScale."""
    sc = _constant_scene(oracle, (0, 0, 1))
    p = capi.params_default()
    L = 5
    p.steps_forward = p.steps_backward = L
    p.gradient_scale = 1.0
    p.illum_scale = 1.0
    p.step_size_vol = 1.0  # a single sample at z=0, then outside
    p.tf_index = capi.TF_INDEX_MAGNITUDE
    ones = np.ones((256, 4), np.float32)
    sc2 = oracle.Scene(sc.field, sc.noise, ones, np.ones(256, np.float32), filter_table=capi.make_filter_table("box", 256))
    img, smp = sc2.render(p, wl.ortho_view(), 2, 2)
    assert np.all(smp == 1)
    taps_sum = (2 * L - 1) + 2 * 0.5 + 0  # interior 1.0, two end taps 0.5; centre 1.0
    taps_sum = (2 * L + 1 - 2) * 1.0 + 2 * 0.5
    I = taps_sum * 0.5 / (2 * L) * 1.0
    a = 1.0 - (1.0 - 1.0) ** 128.0  # opacity table 1, tf.a 1 -> alpha 1
    np.testing.assert_allclose(img[0, 0], [I * a, I * a, I * a, a], rtol=1e-6)


def test_heun_streamline_in_uniform_field(oracle):
    """In a uniform field the LIC positions advance by exactly h_eff per step; with a noise that
    is a linear ramp in x the LIC average equals the ramp at the centre (symmetric taps)."""
    n = 32
    v = np.zeros((n, n, n, 3), np.float32)
    v[..., 0] = 1.0
    rgba = oracle.encode_field(v)
    xs = (np.arange(n) + 0.5) / n
    noise = np.broadcast_to(np.round(xs * 200).astype(np.uint8)[None, None, :], (n, n, n)).copy()
    ones = np.ones((256, 4), np.float32)
    sc = oracle.Scene(rgba, noise, ones, np.ones(256, np.float32), filter_table=capi.make_filter_table("box", 256),
                      filter_clamp=capi.KERNEL_CLAMP_EDGE)
    p = capi.params_default()
    p.steps_forward = p.steps_backward = 4
    p.step_size_lic = 0.01
    p.gradient_scale = 1.0
    p.step_size_vol = 1.0
    view = wl.ortho_view(center=(0.5, 0.5, 0.5))
    img, smp = sc.render(p, view, 1, 1)
    # one sample at (0.5, 0.5, 0); noise is linear across the streamline support (0.5 +- 0.012)
    x0 = 0.5 * n - 0.5
    ramp = np.interp(x0, np.arange(n), noise[0, 0].astype(float)) / 255.0
    I = ramp * 9 * 0.5 / 8
    np.testing.assert_allclose(img[0, 0, 3], 1.0, rtol=0, atol=0)  # alpha saturates (opacity 1)
    np.testing.assert_allclose(img[0, 0, 0], I, rtol=2e-3)


def test_oracle_f32_close_to_f64(oracle):
    w = wl.c1(size=16, image=24)
    rgba = oracle.encode_field(w.field)
    sc = oracle.Scene(rgba, w.noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)
    a, sa = sc.render(w.params, w.views[0], 24, 24, precision=64)
    b, sb = sc.render(w.params, w.views[0], 24, 24, precision=32)
    np.testing.assert_array_equal(sa, sb)
    assert float(np.sqrt(np.mean((a - b) ** 2))) < 1e-5


def test_row_subset_matches_full(oracle):
    w = wl.c1(size=16, image=20)
    rgba = oracle.encode_field(w.field)
    sc = oracle.Scene(rgba, w.noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)
    full, _ = sc.render(w.params, w.views[0], 20, 20)
    rows = [0, 7, 19]
    sub, _ = sc.render(w.params, w.views[0], 20, 20, rows=rows)
    np.testing.assert_array_equal(sub, full[rows])


# ---------------------------------------------------------------------------------------------
# the FP64 adjoint against central finite differences of the FP64 forward
# ---------------------------------------------------------------------------------------------
def _adjoint_case(oracle, lit=False, integrator=capi.HEUN):
    w = wl.c1(size=12, image=14)
    w.field = wl.vortex_field((12, 12, 12), seed=6)
    w.noise = wl.dense_noise(12, seed=61)
    if lit == "gradient":  # illumGradient on central-difference noise gradients
        w.noise = oracle.noise_gradients(w.noise, capi.NOISE_GRAD_CENTRAL)
        w.params.illum = capi.ILLUM_GRADIENT
        w.params.light_pos[:] = (0.2, 1.4, 1.1)
    elif lit:
        w.params.illum = {"zoeckler": capi.ILLUM_ZOECKLER, "mallo": capi.ILLUM_MALLO}[lit]
        w.params.light_pos[:] = (0.2, 1.4, 1.1)
    w.params.integrator = integrator
    w.params.steps_forward = w.params.steps_backward = 4
    w.params.gradient_scale = 6.0
    w.params.step_size_vol = 1.0 / 24.0
    rgba, op = wl.random_tf(seed=7)
    taps = np.linspace(0.6, 1.0, 9)
    view = wl.perspective_view(wl.quat_axis_angle((1, 1, 0), 25.0), distance=2.2)
    enc = oracle.encode_field(w.field)

    def render(rgba_, op_, taps_):
        sc = oracle.Scene(enc, w.noise, rgba_, op_, taps=taps_, inv_filter_area=0.8)
        return sc.render(w.params, view, w.width, w.height)[0].astype(np.float64), sc

    target, _ = render(*wl.random_tf(seed=8), taps[::-1].copy())
    return w, view, enc, rgba, op, taps, target, render


@pytest.mark.parametrize("lit,integrator", [(False, capi.HEUN), ("gradient", capi.HEUN), ("zoeckler", capi.HEUN),
                                             ("mallo", capi.HEUN), (False, capi.RK4), ("gradient", capi.RK4),
                                             ("gradient", capi.EULER)])
def test_oracle_adjoint_matches_finite_differences(oracle, lit, integrator):
    w, view, enc, rgba, op, taps, target, render = _adjoint_case(oracle, lit, integrator)
    img, sc = render(rgba, op, taps)
    g = (2.0 * (img - target)).astype(np.float32)
    d_tf, d_op, d_taps = oracle.adjoint(sc, w.params, view, w.width, w.height, g)

    def loss(rgba_, op_, taps_):
        im, _ = render(rgba_, op_, taps_)
        return float(np.sum((im - target) ** 2))

    h = 1e-4
    checked = 0
    # the most sensitive entries of each parameter group
    for idx in np.argsort(-np.abs(d_tf.reshape(-1)))[:6]:
        e, ch = divmod(int(idx), 4)
        p1, p2 = rgba.copy(), rgba.copy()
        p1[e, ch] += h
        p2[e, ch] -= h
        fd = (loss(p1, op, taps) - loss(p2, op, taps)) / (2 * h)
        assert abs(fd - d_tf[e, ch]) <= 2e-3 * max(1.0, abs(fd)), (e, ch, fd, d_tf[e, ch])
        checked += 1
    for e in np.argsort(-np.abs(d_op))[:4]:
        p1, p2 = op.copy(), op.copy()
        p1[e] += h
        p2[e] -= h
        fd = (loss(rgba, p1, taps) - loss(rgba, p2, taps)) / (2 * h)
        assert abs(fd - d_op[e]) <= 2e-3 * max(1.0, abs(fd)), (e, fd, d_op[e])
        checked += 1
    for j in range(taps.size):
        t1, t2 = taps.copy(), taps.copy()
        t1[j] += h
        t2[j] -= h
        fd = (loss(rgba, op, t1) - loss(rgba, op, t2)) / (2 * h)
        assert abs(fd - d_taps[j]) <= 2e-3 * max(1.0, abs(fd)), (j, fd, d_taps[j])
        checked += 1
    assert checked == 6 + 4 + taps.size
    assert np.abs(d_tf).max() > 0 and np.abs(d_taps).max() > 0
