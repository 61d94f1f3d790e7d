"""The BRICK sampler (field and noise bricks staged into shared memory by TMA): images equal the
GATHER sampler's (the same arithmetic, read from shared memory; tolerance 2e-6 for the
compiler's FMA contraction choices) and the FP64 oracle's (RMSE <= 1e-3), with no brick wait
running out.  Covered: the small plain configuration (64^3 FP32, Euler, box filter,
orthographic), perspective views, every storage, every integrator, gradient lighting, a long
kernel whose reach exceeds the brick (fetches fall back to global memory), and the cases the
sampler refuses."""
import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

pytestmark = pytest.mark.gpu


def render(ctx, w, vid, sampler):
    p = capi.Params.from_buffer_copy(w.params)
    p.sampler = capi.SAMPLER[sampler]
    if sampler == "brick":
        p.schedule = capi.SCHEDULE["static"]
    ctx.set_params(p)
    img = ctx.render(vid, w.width, w.height)
    st = ctx.stats()
    return img, st


def compare(ctx, oracle, w, storage="f32", views=None):
    vid = wl.setup_context(ctx, w, storage=storage)
    enc = oracle.encode_field(w.field)
    if storage != "f32":
        enc = oracle.round_storage(enc, storage)
    noise = w.noise if w.noise_mode == capi.NOISE_SCALAR else oracle.noise_gradients(w.noise, w.noise_mode)
    sc = oracle.Scene(enc, noise, w.tf_rgba, w.tf_opac, filter_table=oracle.filter_table(w.filter_kind, 256))
    for v in views or w.views:
        ctx.set_view(v)
        got, st = render(ctx, w, vid, "brick")
        assert st.check_flags == 0, st.check_flags
        ref_g, st_g = render(ctx, w, vid, "gather")
        np.testing.assert_allclose(got, ref_g, rtol=0, atol=2e-6)
        assert st.samples == st_g.samples and st.samples > 0
        ref, _ = sc.render(w.params, v, w.width, w.height)
        e = float(np.sqrt(np.mean((got.astype(np.float64) - ref) ** 2)))
        assert e <= 1e-3, e
    ctx.free_volume(vid)


def test_brick_plain_small_configuration(ctx, oracle):
    w = wl.c1()  # 64^3 FP32 ABC flow, sparse noise, Euler L=20, box filter, 256^2 orthographic
    compare(ctx, oracle, w, "f32")


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16", "u8"])
def test_brick_storages_and_perspective(ctx, oracle, storage):
    w = wl.c1(size=48, image=64)
    w.params.integrator = capi.HEUN
    w.params.steps_forward = w.params.steps_backward = 10
    views = [wl.perspective_view(wl.quat_axis_angle((1, 2, 0), 40.0), distance=1.8),
             wl.ortho_view(direction=(0.0, 1.0, 0.0), up=(0.0, 0.0, 0.5))]
    compare(ctx, oracle, w, storage, views)


@pytest.mark.parametrize("integ", [capi.EULER, capi.HEUN, capi.RK4])
def test_brick_integrators_and_lighting(ctx, oracle, integ):
    w = wl.c2(size=32, image=48, storage="f16")
    w.params.integrator = integ
    w.params.steps_forward = w.params.steps_backward = 6
    w.params.step_size_vol = 1.0 / 48.0
    compare(ctx, oracle, w, "f16")


def test_brick_reach_beyond_the_brick_falls_back(ctx, oracle):
    """L = 200 at step 0.02 reaches 77 texels of a 64^3 field each way: the brick cannot hold
    the box and most fetches read global memory; the image is still GATHER's."""
    w = wl.c1(size=64, image=48)
    w.params.steps_forward = w.params.steps_backward = 200
    w.params.step_size_lic = 0.02
    w.params.step_size_vol = 1.0 / 32.0
    compare(ctx, oracle, w, "f16")


def test_brick_refusals(ctx):
    import torch

    w = wl.c1(size=16, image=16)
    w.field = wl.abc_field((15, 16, 16))  # 15 x 8 bytes per F16 row: not a multiple of 16
    vid = wl.setup_context(ctx, w, storage="f16")
    p = capi.Params.from_buffer_copy(w.params)
    p.sampler = capi.SAMPLER["brick"]
    ctx.set_params(p)
    with pytest.raises(capi.VVLICError) as e:
        ctx.render(vid, 16, 16)
    assert e.value.status == capi.ERR_UNSUPPORTED
    vid2 = ctx.upload_field(wl.abc_field(16), storage="f16")
    p.record_tape = 1
    ctx.set_params(p)
    with pytest.raises(capi.VVLICError) as e:
        ctx.render(vid2, 16, 16)
    assert e.value.status == capi.ERR_UNSUPPORTED
    p.record_tape = 0
    out = torch.empty((16, 16, 4), dtype=torch.float32, device="cuda")
    job = capi.make_job(vid2, out.data_ptr(), 16, 16, w.views[0], p, w.filter_table)
    with pytest.raises(capi.VVLICError) as e:
        ctx.batch_render([job])
    assert e.value.status == capi.ERR_UNSUPPORTED
