"""GPU parity: the CUDA kernels, called through the C ABI, against the FP64 oracle on the same
seeded inputs.

Tolerances (per image, RGBA in [0, 1]):
  * RMSE <= 1e-3 against the FP64 oracle for every FP32 configuration (the project's bar);
  * reduced-precision storage is compared with an oracle that reads the same FP16 / BF16
    rounded field (same bar), and its error against the full-precision oracle is reported;
  * per-pixel max-abs is bounded separately (MAXABS below): a sample that lands within float
    rounding of the volume boundary may be taken by one side and not the other.
Preprocessing (field encoding, noise gradients) is integer/float-exact work: bit-exact.
"""
import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

pytestmark = pytest.mark.gpu

RMSE_TOL = 1e-3
MAXABS = 0.25


def rmse(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


def torch_cuda():
    import torch

    return torch


def oracle_scene(oracle, w: wl.Workload, storage="f32", noise_rgba=None):
    rgba = oracle.encode_field(w.field)
    if storage != "f32":
        rgba = oracle.round_storage(rgba, storage)
    noise = w.noise
    if w.noise_mode != capi.NOISE_SCALAR:
        noise = noise_rgba if noise_rgba is not None else oracle.noise_gradients(w.noise, w.noise_mode)
    return oracle.Scene(rgba, noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)


def render_gpu(ctx, w: wl.Workload, sampler="cell", storage=None, view=None, samples=False):
    vid = wl.setup_context(ctx, w, storage=storage)
    p = w.params
    p.sampler = capi.SAMPLER[sampler]
    ctx.set_params(p)
    if view is not None:
        ctx.set_view(view)
    if not samples:
        return ctx.render(vid, w.width, w.height), None
    torch = torch_cuda()
    out = torch.empty((w.height, w.width, 4), dtype=torch.float32, device="cuda")
    smp = torch.zeros((w.height, w.width), dtype=torch.int32, device="cuda")
    ctx.render_device(vid, out.data_ptr(), w.width, w.height, smp.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy(), smp.cpu().numpy().astype(np.uint32)


# ---------------------------------------------------------------------------------------------
# preprocessing: bit-exact
# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("storage", ["f32", "f16", "bf16", "u8"])
def test_field_encoding_bit_exact(ctx, oracle, storage):
    for field in (wl.vortex_field((24, 17, 9), seed=3), wl.abc_field((8, 8, 8))):
        vid = ctx.upload_field(field, storage=storage)
        got = ctx.download_field(vid, field.shape[2::-1], storage)
        want = oracle.round_storage(oracle.encode_field(field), storage)
        np.testing.assert_array_equal(got, want)


def test_field_encoding_uint8_bit_exact(ctx, oracle):
    rng = wl.SplitMix64(77)
    field = (rng.uniform(6 * 5 * 4 * 3) * 256).astype(np.uint8).reshape(4, 5, 6, 3)
    vid = ctx.upload_field(field)
    np.testing.assert_array_equal(ctx.download_field(vid, (6, 5, 4), "f32"), oracle.encode_field(field))


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_field_interp_bit_exact(ctx, oracle, storage):
    a0 = wl.vortex_field((24, 17, 9), seed=3)
    a1 = wl.abc_field((24, 17, 9))
    for index, size in ((0, 5), (3, 5), (47, 48)):
        vid = ctx.upload_field_interp(a0, a1, index, size, storage=storage)
        got = ctx.download_field(vid, (24, 17, 9), storage)
        want = oracle.round_storage(oracle.encode_field_interp(a0, a1, index, size), storage)
        np.testing.assert_array_equal(got, want)
        ctx.free_volume(vid)


def test_field_interp_uint8_bit_exact(ctx, oracle):
    rng = wl.SplitMix64(78)
    a0 = (rng.uniform(7 * 6 * 5 * 3) * 256).astype(np.uint8).reshape(5, 6, 7, 3)
    a1 = (rng.uniform(7 * 6 * 5 * 3) * 256).astype(np.uint8).reshape(5, 6, 7, 3)
    for index, size in ((1, 2), (2, 7)):
        vid = ctx.upload_field_interp(a0, a1, index, size)
        np.testing.assert_array_equal(ctx.download_field(vid, (7, 6, 5), "f32"),
                                      oracle.encode_field_interp(a0, a1, index, size))
        ctx.free_volume(vid)


def test_field_interp_rejects_bad_index(ctx):
    a0 = wl.abc_field((8, 8, 8))
    for index, size in ((2, 2), (-1, 4), (0, 0)):
        with pytest.raises(capi.VVLICError):
            ctx.upload_field_interp(a0, a0, index, size)


def test_field_encoding_zero_field(ctx, oracle):
    field = np.zeros((3, 4, 5, 3), np.float32)
    vid = ctx.upload_field(field)
    got = ctx.download_field(vid, (5, 4, 3), "f32")
    np.testing.assert_array_equal(got, oracle.encode_field(field))
    np.testing.assert_array_equal(got[..., 3], 0.0)


@pytest.mark.parametrize("mode", [capi.NOISE_GRAD_SOBEL, capi.NOISE_GRAD_CENTRAL])
def test_noise_gradients_bit_exact_vs_reference_fixture(ctx, mode):
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "noise_gradients.npz"))
    tag = "sobel" if mode == capi.NOISE_GRAD_SOBEL else "central"
    for case in ["dense_11x13x17", "sparse_24", "tiny_3x4x5"]:
        noise = g[f"{case}/noise"]
        ctx.upload_noise(noise, mode)
        got = ctx.download_noise(noise.shape[::-1], 4)
        np.testing.assert_array_equal(got, g[f"{case}/{tag}"])


def test_noise_gradients_device_entry(vvlic_lib, oracle):
    torch = torch_cuda()
    noise = wl.dense_noise((40, 33, 29), seed=5)
    sd = (1.0, 0.5, 2.0)
    d_in = torch.from_numpy(noise).cuda()
    d_out = torch.empty(noise.shape + (4,), dtype=torch.uint8, device="cuda")
    dims = noise.shape[::-1]  # (mx, my, mz)
    assert dims == (40, 33, 29)
    for mode in (capi.NOISE_GRAD_SOBEL, capi.NOISE_GRAD_CENTRAL):
        capi.noise_gradients_device(d_in.data_ptr(), dims, mode, d_out.data_ptr(), slice_dist=sd)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d_out.cpu().numpy(), oracle.noise_gradients(noise, mode, sd))


# ---------------------------------------------------------------------------------------------
# C1: plain method, small (the full configuration)
# ---------------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def c1_ref(oracle):
    w = wl.c1()
    sc = oracle_scene(oracle, w)
    img, smp = sc.render(w.params, w.views[0], w.width, w.height)
    return w, img, smp


SAMPLERS = ["gather", "cell", "texture", "hybrid"]
STORAGES = ["f32", "f16", "bf16", "u8"]


@pytest.mark.parametrize("sampler", SAMPLERS)
def test_c1_parity(ctx, c1_ref, sampler):
    """The FP32 C1 frame: per-pixel sample counts identical, RMSE within the bar.  TEXTURE and
    HYBRID filter with the texture unit's 8-bit fractional weights."""
    w, ref, ref_smp = c1_ref
    img, smp = render_gpu(ctx, wl.c1(), sampler=sampler, samples=True)
    np.testing.assert_array_equal(smp, ref_smp)
    e = rmse(img, ref)
    print(f"C1 {sampler}: RMSE {e:.2e} max-abs {float(np.abs(img - ref).max()):.2e}")
    assert e <= RMSE_TOL, e
    assert float(np.abs(img - ref).max()) <= MAXABS
    st = ctx.stats()
    assert st.samples == int(ref_smp.sum()) and st.sample_steps == st.samples * 40 and st.rays == 256 * 256


@pytest.mark.parametrize("sampler", SAMPLERS)
def test_schedules_agree_bitwise(ctx, sampler):
    """Each pixel's computation does not depend on the work distribution."""
    w = c2_small()
    vid = wl.setup_context(ctx, w)
    imgs = []
    for sch in ("queue", "static"):
        p = w.params
        p.sampler = capi.SAMPLER[sampler]
        p.schedule = capi.SCHEDULE[sch]
        ctx.set_params(p)
        imgs.append(ctx.render(vid, w.width, w.height))
        imgs.append(ctx.stats().samples)
    np.testing.assert_array_equal(imgs[0], imgs[2])
    assert imgs[1] == imgs[3]


# ---------------------------------------------------------------------------------------------
# C2 at reduced size: lighting, Heun, Gaussian filter, perspective view, every storage
# ---------------------------------------------------------------------------------------------
def c2_small():
    w = wl.c2(size=48, image=96)
    w.params.steps_forward = w.params.steps_backward = 12
    return w


@pytest.fixture(scope="module")
def c2_refs(oracle):
    w = c2_small()
    noise_rgba = oracle.noise_gradients(w.noise, w.noise_mode)
    out = {}
    for st in STORAGES:
        sc = oracle_scene(oracle, w, st, noise_rgba)
        out[st] = sc.render(w.params, w.views[0], w.width, w.height)
    return out


@pytest.mark.parametrize("storage", STORAGES)
@pytest.mark.parametrize("sampler", SAMPLERS)
def test_c2_small_parity(ctx, c2_refs, storage, sampler):
    img, smp = render_gpu(ctx, c2_small(), sampler=sampler, storage=storage, samples=True)
    ref, ref_smp = c2_refs[storage]
    e = rmse(img, ref)
    assert e <= RMSE_TOL, e
    assert float(np.abs(img - ref).max()) <= MAXABS
    assert np.mean(smp != ref_smp) < 1e-3
    full = rmse(img, c2_refs["f32"][0])
    print(f"C2-small {storage}/{sampler}: RMSE vs same-storage oracle {e:.2e}, vs FP32-field oracle {full:.2e}")


# ---------------------------------------------------------------------------------------------
# variants and edge cases
# ---------------------------------------------------------------------------------------------
def small(integrator=capi.HEUN, **kw):
    w = wl.c1(size=24, image=40)
    w.params.integrator = integrator
    w.params.steps_forward = w.params.steps_backward = 6
    for k, v in kw.items():
        setattr(w.params, k, v)
    return w


def axis_aligned_field(shape, seed):
    """Vectors along +-x, +-y or +-z with lengths k/4 (k = 1..4): every encoded texel component
    (0, 1/2, 1 and k/4) is exact in FP16 and BF16 alike."""
    rng = np.random.default_rng(seed)
    axis = rng.integers(0, 3, shape)
    val = (rng.choice([-1.0, 1.0], shape) * rng.integers(1, 5, shape) / 4.0).astype(np.float32)
    f = np.zeros(tuple(shape) + (3,), np.float32)
    np.put_along_axis(f, axis[..., None], val[..., None], axis=3)
    f[0, 0, 0] = (1.0, 0.0, 0.0)
    return f


@pytest.mark.parametrize("sampler", ["texture", "hybrid"])
def test_bf16_texture_holds_the_bf16_texels(ctx, sampler):
    # the texture of a BF16 volume is a half4 copy of its BF16 texels: where both formats hold
    # the texels exactly, BF16 and FP16 storage give the same image bit for bit
    w = small()
    w.field = axis_aligned_field(w.field.shape[:3], seed=17)
    a, _ = render_gpu(ctx, w, sampler=sampler, storage="f16")
    b, _ = render_gpu(ctx, w, sampler=sampler, storage="bf16")
    np.testing.assert_array_equal(a, b)
    assert float(a[..., 3].max()) > 0.05


def check_small(ctx, oracle, w, sampler="cell", view=None, tol=RMSE_TOL):
    sc = oracle_scene(oracle, w)
    v = view or w.views[0]
    ref, ref_smp = sc.render(w.params, v, w.width, w.height)
    img, smp = render_gpu(ctx, w, sampler=sampler, view=v, samples=True)
    e = rmse(img, ref)
    assert e <= tol, e
    assert np.mean(smp != ref_smp) < 1e-2
    return img, ref


@pytest.mark.parametrize("integ", [capi.EULER, capi.HEUN, capi.RK4])
def test_integrators(ctx, oracle, integ):
    check_small(ctx, oracle, small(integ))


def test_speed_of_flow_and_dir_z_index(ctx, oracle):
    check_small(ctx, oracle, small(speed_of_flow=1, tf_index=capi.TF_INDEX_DIR_Z))


def test_low_res_preview(ctx, oracle):
    check_small(ctx, oracle, small(low_res=1))


def test_luminance_quirk_flat_lic(ctx, oracle):
    w = small(quirks=capi.QUIRKS_REFERENCE | capi.QUIRK_LUMINANCE_NOISE)
    check_small(ctx, oracle, w)


def test_perspective_views(ctx, oracle):
    w = small()
    for q in [(0, 0, 0, 1), wl.quat_axis_angle((1, 1, 0), 40.0), wl.quat_axis_angle((0, 1, 0), 135.0)]:
        check_small(ctx, oracle, w, view=wl.perspective_view(q, distance=2.5))


def test_uneven_volume(ctx, oracle):
    w = small()
    w.field = wl.vortex_field((40, 24, 32), seed=8)
    check_small(ctx, oracle, w, view=wl.perspective_view(wl.quat_axis_angle((1, 2, 0), 30.0), distance=2.4))


def test_lighting_uniform_scale_bug_off(ctx, oracle):
    w = c2_small()
    w.params.quirks = 0
    w.width = w.height = 48
    check_small(ctx, oracle, w)


def test_scalar_gate(ctx, oracle):
    w = small(scalar_gate=1, sampler=capi.SAMPLER["cell"])
    nz, ny, nx = w.field.shape[:3]
    zz = (np.arange(nz) + 0.5) / nz
    scalar = np.broadcast_to(zz[:, None, None], (nz, ny, nx)).astype(np.float32).copy() * 0.5
    sc = oracle.Scene(oracle.encode_field(w.field), w.noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table,
                      scalar=scalar)
    ref, _ = sc.render(w.params, w.views[0], w.width, w.height)
    vid = wl.setup_context(ctx, w)
    ctx.upload_scalar(scalar)
    img = ctx.render(vid, w.width, w.height)
    assert rmse(img, ref) <= RMSE_TOL


def test_table_updates_wait_for_renders_in_flight(ctx):
    """set_tf right after an asynchronous render on another stream applies to later renders only."""
    import torch

    w = small()
    w.width = w.height = 192
    w.params.steps_forward = w.params.steps_backward = 24
    vid = wl.setup_context(ctx, w)
    ref = ctx.render(vid, w.width, w.height)
    stream = torch.cuda.Stream()
    out = torch.empty((w.height, w.width, 4), dtype=torch.float32, device="cuda")
    other = wl.random_tf(seed=3)
    for _ in range(3):
        ctx.render_device(vid, out.data_ptr(), w.width, w.height, None, stream.cuda_stream)
        ctx.set_tf(*other)  # must not reach the render above
        stream.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), ref)
        ctx.set_tf(w.tf_rgba, w.tf_opac)


def test_views_that_miss_give_zero(ctx, oracle):
    w = small()
    vid = wl.setup_context(ctx, w)
    ctx.set_view(wl.ortho_view(center=(5.0, 5.0, 0.5)))
    img = ctx.render(vid, 17, 9)
    np.testing.assert_array_equal(img, 0.0)
    assert ctx.stats().rays == 0


def test_num_iterations_bounds(ctx, oracle):
    for it in (0, 1, 3):
        w = small(num_iterations=it)
        img, ref = check_small(ctx, oracle, w)
        if it == 0:
            np.testing.assert_array_equal(img, 0.0)


def test_one_sided_streamlines(ctx, oracle):
    check_small(ctx, oracle, small(steps_forward=0, steps_backward=7))
    check_small(ctx, oracle, small(steps_forward=5, steps_backward=0))


def test_longest_streamlines(ctx, oracle):
    """L_f = L_b = VVLIC_MAX_STEPS (513 taps), asymmetric lengths at the limit, every integrator."""
    for integ, lb, lf in ((capi.HEUN, capi.MAX_STEPS, capi.MAX_STEPS), (capi.RK4, capi.MAX_STEPS, 3),
                          (capi.EULER, 1, capi.MAX_STEPS)):
        w = small(integ, steps_backward=lb, steps_forward=lf)
        w.width, w.height = 12, 10
        check_small(ctx, oracle, w)
    with pytest.raises(capi.VVLICError):
        ctx.set_params(small(steps_forward=capi.MAX_STEPS + 1).params)


def test_tiny_images_and_volumes(ctx, oracle):
    w = small()
    w.width, w.height = 1, 1
    check_small(ctx, oracle, w)
    w = small()
    w.field = wl.abc_field((1, 2, 3))
    w.width, w.height = 7, 5
    check_small(ctx, oracle, w)


def test_filters_and_clamp_modes(ctx, oracle):
    for kind in ("triangle", "cos2", "gaussian"):
        w = small()
        w.filter_table = capi.make_filter_table(kind, 256)
        check_small(ctx, oracle, w)


def test_explicit_taps(ctx, oracle):
    w = small(sampler=capi.SAMPLER["cell"])
    taps = np.linspace(0.2, 1.0, 13).astype(np.float64)
    sc = oracle.Scene(oracle.encode_field(w.field), w.noise, w.tf_rgba, w.tf_opac, taps=taps, inv_filter_area=0.7)
    ref, _ = sc.render(w.params, w.views[0], w.width, w.height)
    vid = wl.setup_context(ctx, w)
    ctx.set_filter_taps(taps.astype(np.float32), 6, 6, 0.7)
    np.testing.assert_allclose(ctx.filter_taps()[0], taps, rtol=1e-7)
    img = ctx.render(vid, w.width, w.height)
    assert rmse(img, ref) <= RMSE_TOL


def test_filter_taps_match_oracle(ctx, oracle):
    w = small()
    wl.setup_context(ctx, w)
    for kind in ("box", "gaussian", "cos2"):
        t = capi.make_filter_table(kind, 256)
        ctx.set_filter_table(t)
        got, ia = ctx.filter_taps()
        np.testing.assert_allclose(got, oracle.filter_taps(t, 6, 6), rtol=1e-6, atol=1e-7)
        assert abs(ia - oracle.filter_inv_area(t, kind == "box")) < 1e-6


def test_view_rays_match_oracle(ctx, oracle):
    w = small()
    vid = wl.setup_context(ctx, w)
    v = wl.perspective_view(wl.quat_axis_angle((1, 2, 3), 77.0), distance=3.1, pan=(0.1, -0.2, 0.3))
    ctx.set_view(v)
    np.testing.assert_allclose(ctx.view_rays(vid, 64, 48), oracle.view_rays(v, [24, 24, 24], 64, 48), rtol=1e-12,
                               atol=1e-12)


def test_errors_are_reported(ctx):
    w = small()
    vid = ctx.upload_field(w.field)
    with pytest.raises(capi.VVLICError) as e:
        ctx.render(vid, 8, 8)  # no noise yet
    assert e.value.status == capi.ERR_NOT_READY
    ctx.upload_noise(w.noise)
    p = capi.params_default()
    p.steps_forward = p.steps_backward = 0
    with pytest.raises(capi.VVLICError) as e:
        ctx.set_params(p)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    p = capi.params_default()
    p.illum = capi.ILLUM_GRADIENT
    ctx.set_params(p)
    with pytest.raises(capi.VVLICError) as e:
        ctx.render(vid, 8, 8)  # gradient lighting with value-only noise
    assert e.value.status == capi.ERR_NOT_READY
    ctx.free_volume(vid)
    with pytest.raises(capi.VVLICError):
        ctx.render(vid, 8, 8)


def test_contexts_are_independent_across_threads(oracle):
    """Contexts used from separate host threads at the same time (ctypes releases the GIL
    during each call) render exactly what they render alone."""
    import threading

    cases = [small(capi.HEUN), small(capi.RK4, illum=capi.ILLUM_GRADIENT), small(capi.EULER, speed_of_flow=1)]
    cases[1].noise_mode = capi.NOISE_GRAD_CENTRAL
    alone = []
    for w in cases:
        with capi.Context(0) as c:
            vid = wl.setup_context(c, w)
            alone.append(c.render(vid, w.width, w.height))
    results = [None] * len(cases)
    errors = []

    def run(k):
        try:
            with capi.Context(0) as c:
                vid = wl.setup_context(c, cases[k])
                for _ in range(3):
                    results[k] = c.render(vid, cases[k].width, cases[k].height)
        except Exception as e:  # surfaced below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(k,)) for k in range(len(cases))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for got, want in zip(results, alone):
        np.testing.assert_array_equal(got, want)
