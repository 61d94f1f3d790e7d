"""Illuminated-streamline shading (illumZoeckler / illumMallo, inc_illum.glsl:46-154) against the
FP64 oracle.  The tables are integer work (bit-exact); the images meet the RMSE <= 1e-3 bar."""
import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

pytestmark = pytest.mark.gpu

ILLUM = {"zoeckler": capi.ILLUM_ZOECKLER, "mallo": capi.ILLUM_MALLO}


def rmse(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


def case(illum, sampler="cell", technique="raycast", size=24, image=40):
    w = wl.c1(size=size, image=image)
    w.field = wl.vortex_field((size, size, size), seed=14)
    w.noise = wl.dense_noise(size, seed=141)
    p = w.params
    p.integrator = capi.HEUN
    p.steps_forward = p.steps_backward = 6
    p.gradient_scale = 10.0
    p.illum = ILLUM[illum]
    p.sampler = capi.SAMPLER[sampler]
    p.technique = capi.TECHNIQUE[technique]
    return w


VIEWS = [wl.ortho_view(), wl.perspective_view(wl.quat_axis_angle((1, 1, 0), 35.0), distance=2.4),
         wl.perspective_view(wl.quat_axis_angle((0, 1, 0), 120.0), distance=2.2)]


def test_tables_bit_exact(ctx, oracle):
    np.testing.assert_array_equal(ctx.illum_luts(), oracle.illum_luts())
    m = capi.line_material_default()
    m.width, m.height = 100, 60
    m.diffuse[:] = (0.9, 0.6, 0.3, 1.0)
    m.specular[:] = (0.2, 0.5, 1.0, 1.0)
    m.light_color[:] = (1.0, 0.8, 0.9, 1.0)
    m.ambient[0] = 0.25
    m.spec_exp, m.diff_exp = 12.0, 3.0
    ctx.set_line_material(m)
    got = ctx.illum_luts()
    assert got.shape == (3, 64, 128, 4)
    np.testing.assert_array_equal(got, oracle.illum_luts(m))


@pytest.mark.parametrize("illum", ["zoeckler", "mallo"])
@pytest.mark.parametrize("sampler", ["cell", "hybrid"])
def test_raycast_matches_oracle(ctx, oracle, illum, sampler):
    w = case(illum, sampler)
    sc = oracle.Scene(oracle.encode_field(w.field), w.noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)
    vid = wl.setup_context(ctx, w)
    unlit = case("zoeckler", sampler).params
    unlit.illum = capi.ILLUM_NONE
    for v in VIEWS:
        ctx.set_view(v)
        ctx.set_params(w.params)
        img = ctx.render(vid, w.width, w.height)
        ref, smp = sc.render(w.params, v, w.width, w.height)
        e = rmse(img, ref)
        assert e <= 1e-3, (illum, sampler, e)
        assert abs(int(ctx.stats().samples) - int(smp.sum())) <= 0.01 * smp.sum() + 2
        ctx.set_params(unlit)
        plain = ctx.render(vid, w.width, w.height)
        assert rmse(img, plain) > 1e-2  # the shading model changes the image


def test_zoeckler_luminance_quirk(ctx, oracle):
    w = case("zoeckler")
    sc = oracle.Scene(oracle.encode_field(w.field), w.noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)
    vid = wl.setup_context(ctx, w)
    v = VIEWS[1]
    ctx.set_view(v)
    imgs = []
    for q in (capi.QUIRKS_REFERENCE, capi.QUIRKS_REFERENCE & ~capi.QUIRK_ZOECKLER_LUMINANCE):
        w.params.quirks = q
        ctx.set_params(w.params)
        img = ctx.render(vid, w.width, w.height)
        ref, _ = sc.render(w.params, v, w.width, w.height)
        assert rmse(img, ref) <= 1e-3
        imgs.append(img)
    assert rmse(imgs[0], imgs[1]) > 1e-3


@pytest.mark.parametrize("illum", ["zoeckler", "mallo"])
def test_slicing_matches_oracle(ctx, oracle, illum):
    w = case(illum, technique="slicing")
    sc = oracle.Scene(oracle.encode_field(w.field), w.noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)
    vid = wl.setup_context(ctx, w)
    for v in VIEWS[:2]:
        ctx.set_view(v)
        img = ctx.render(vid, w.width, w.height)
        ref, _ = sc.render(w.params, v, w.width, w.height)
        assert rmse(img, ref) <= 1e-3


def test_custom_material_render(ctx, oracle):
    w = case("mallo")
    m = capi.line_material_default()
    m.specular[:] = (0.3, 0.3, 0.3, 1.0)
    m.spec_exp = 8.0
    m.width = m.height = 64
    ctx.set_line_material(m)
    w.params.spec_exp = 8.0
    sc = oracle.Scene(oracle.encode_field(w.field), w.noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)
    sc.attach_line_material(m)
    vid = wl.setup_context(ctx, w)
    ctx.set_view(VIEWS[1])
    img = ctx.render(vid, w.width, w.height)
    ref, _ = sc.render(w.params, VIEWS[1], w.width, w.height)
    assert rmse(img, ref) <= 1e-3


def test_bad_material_rejected(ctx):
    m = capi.line_material_default()
    m.width = 1
    with pytest.raises(capi.VVLICError):
        ctx.set_line_material(m)
    m = capi.line_material_default()
    m.spec_exp = float("nan")
    with pytest.raises(capi.VVLICError):
        ctx.set_line_material(m)
