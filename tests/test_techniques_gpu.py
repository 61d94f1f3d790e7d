"""The reference's other render techniques against the FP64 oracle: view-aligned SLICING
(lic3d_slicing_fragment.glsl), vector-field DVR (VOLUME, vectorfield_fragment.glsl) and the
LIC-volume precompute + DVR (LICVOLUME, lic3d_volume_fragment.glsl / raycast_lic3d_fragment.glsl).
Bar: RMSE <= 1e-3 per image; the LIC volume itself to 1e-5 RMSE."""
import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

pytestmark = pytest.mark.gpu


def rmse(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


def case(technique, sampler="cell", lit=False, size=24, image=40):
    w = wl.c1(size=size, image=image)
    w.field = wl.vortex_field((size, size, size), seed=12)
    w.noise = wl.dense_noise(size, seed=121)
    p = w.params
    p.integrator = capi.HEUN
    p.steps_forward = p.steps_backward = 6
    p.gradient_scale = 10.0
    p.technique = capi.TECHNIQUE[technique]
    p.sampler = capi.SAMPLER[sampler]
    if lit:
        p.illum = capi.ILLUM_GRADIENT
        w.noise_mode = capi.NOISE_GRAD_CENTRAL
    return w


def oracle_scene(oracle, w):
    noise = w.noise if w.noise_mode == capi.NOISE_SCALAR else oracle.noise_gradients(w.noise, w.noise_mode)
    return oracle.Scene(oracle.encode_field(w.field), noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)


VIEWS = [wl.ortho_view(), wl.perspective_view(wl.quat_axis_angle((1, 1, 0), 35.0), distance=2.4),
         wl.perspective_view(wl.quat_axis_angle((0, 1, 0), 120.0), distance=2.2)]


@pytest.mark.parametrize("sampler", ["cell", "hybrid"])
@pytest.mark.parametrize("lit", [False, True])
def test_slicing_matches_oracle(ctx, oracle, sampler, lit):
    w = case("slicing", sampler, lit)
    sc = oracle_scene(oracle, w)
    vid = wl.setup_context(ctx, w)
    for v in VIEWS:
        ctx.set_view(v)
        img = ctx.render(vid, w.width, w.height)
        ref, smp = sc.render(w.params, v, w.width, w.height)
        e = rmse(img, ref)
        assert e <= 1e-3, (e, v.projection)
        assert ctx.stats().samples > 0 and abs(int(ctx.stats().samples) - int(smp.sum())) <= 0.01 * smp.sum() + 2
        assert float(img[..., 3].max()) > 0


def test_slicing_orthographic_planes_are_the_ray_samples(ctx, oracle):
    """Along +z the slabs are z = (i + 1/2) / N: the same planes a ray-cast with that spacing
    would sample, offset by half a slab."""
    w = case("slicing")
    vid = wl.setup_context(ctx, w)
    ctx.set_view(wl.ortho_view())
    ctx.render(vid, 8, 8)
    n = int(1.0 / w.params.step_size_vol) + 1
    assert ctx.stats().samples <= 64 * n


@pytest.mark.parametrize("sampler", ["gather", "hybrid"])
def test_vector_field_dvr_matches_oracle(ctx, oracle, sampler):
    w = case("volume", sampler)
    sc = oracle_scene(oracle, w)
    vid = wl.setup_context(ctx, w)
    for v in VIEWS:
        ctx.set_view(v)
        img = ctx.render(vid, w.width, w.height)
        ref, _ = sc.render(w.params, v, w.width, w.height)
        assert rmse(img, ref) <= 1e-3


# the precompute's warps take 8x4 voxel tiles: dims that are not multiples of the tile (and an
# odd z) leave partial tiles on every face
@pytest.mark.parametrize("sampler,integrator,dims", [("cell", capi.HEUN, (20, 18, 16)), ("hybrid", capi.HEUN, (20, 18, 16)),
                                                     ("cell", capi.RK4, (21, 13, 15)), ("hybrid", capi.RK4, (16, 12, 9))])
def test_lic_volume_and_its_dvr_match_oracle(ctx, oracle, sampler, integrator, dims):
    w = case("licvolume", sampler)
    w.params.integrator = integrator
    sc = oracle_scene(oracle, w)
    vid = wl.setup_context(ctx, w)
    ctx.compute_lic_volume(vid, dims)
    got = ctx.download_lic_volume(vid, dims)
    ref_vol = sc.lic_volume(w.params, dims)
    scale = max(float(np.abs(ref_vol).max()), 1e-6)
    tol = 1e-5 if sampler == "cell" else 5e-3
    assert rmse(got, ref_vol) <= tol * scale
    sc.attach_lic_volume(ref_vol)
    for v in VIEWS:
        ctx.set_view(v)
        img = ctx.render(vid, w.width, w.height)
        ref, _ = sc.render(w.params, v, w.width, w.height)
        assert rmse(img, ref) <= 1e-3


def test_licvolume_requires_precompute(ctx):
    w = case("licvolume")
    vid = wl.setup_context(ctx, w)
    with pytest.raises(capi.VVLICError) as e:
        ctx.render(vid, 8, 8)
    assert e.value.status == capi.ERR_NOT_READY
