"""In-place input updates: vvlic_update_field / vvlic_update_field_interp (the reference's per-frame
createTextureIterp of its animation loop, 3DLIC.cpp:129-145) and a same-shape vvlic_upload_noise.
After an update every layout the volume or noise already had (cells, texture copy) must hold the
new data: images equal those of a freshly uploaded volume bit for bit, on every sampler and
storage.  Stale derived state (LIC volume, adjoint tape) is refused rather than used."""
import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

pytestmark = pytest.mark.gpu

SAMPLERS = ["gather", "cell", "texture", "hybrid"]


def small():
    w = wl.c1(size=24, image=40)
    w.params.steps_forward = w.params.steps_backward = 6
    return w


def render(ctx, vid, w, sampler):
    p = w.params
    p.sampler = capi.SAMPLER[sampler]
    ctx.set_params(p)
    return ctx.render(vid, w.width, w.height)


def other_field(w, seed):
    return wl.vortex_field(w.field.shape[2::-1], seed=seed).astype(np.float32)


@pytest.mark.parametrize("storage", ["f16", "bf16", "u8"])
def test_update_field_equals_fresh_upload(ctx, storage):
    w = small()
    vid = wl.setup_context(ctx, w, storage=storage)
    for sm in SAMPLERS:  # build every layout of the old field
        render(ctx, vid, w, sm)
    new = other_field(w, seed=77)
    ctx.update_field(vid, new)
    fresh = ctx.upload_field(new, storage=storage)
    for sm in SAMPLERS:
        a = render(ctx, vid, w, sm)
        b = render(ctx, fresh, w, sm)
        np.testing.assert_array_equal(a, b, err_msg=f"{storage}/{sm}")
    nz, ny, nx = new.shape[:3]
    np.testing.assert_array_equal(ctx.download_field(vid, (nx, ny, nz), storage),
                                  ctx.download_field(fresh, (nx, ny, nz), storage))
    ctx.free_volume(fresh)
    ctx.free_volume(vid)


@pytest.mark.parametrize("storage", ["f32", "f16", "u8"])
def test_update_field_device_equals_fresh_upload(ctx, storage):
    """vvlic_update_field_device (float32 xyz already on the device, ordered on a stream) leaves
    the volume bit for bit as a fresh upload of the same field, in every layout; the LIC volume
    turns stale as with the host update."""
    import torch

    w = small()
    vid = wl.setup_context(ctx, w, storage=storage)
    for sm in SAMPLERS:
        render(ctx, vid, w, sm)
    ctx.compute_lic_volume(vid, (24, 24, 24))
    new = other_field(w, seed=78)
    d_new = torch.from_numpy(np.ascontiguousarray(new)).cuda()
    stream = torch.cuda.Stream()
    nz, ny, nx = new.shape[:3]
    ctx.update_field_device(vid, d_new.data_ptr(), (nx, ny, nz), stream.cuda_stream)
    stream.synchronize()
    fresh = ctx.upload_field(new, storage=storage)
    for sm in SAMPLERS:
        np.testing.assert_array_equal(render(ctx, vid, w, sm), render(ctx, fresh, w, sm), err_msg=f"{storage}/{sm}")
    np.testing.assert_array_equal(ctx.download_field(vid, (nx, ny, nz), storage),
                                  ctx.download_field(fresh, (nx, ny, nz), storage))
    p = w.params
    p.technique = capi.TECHNIQUE["licvolume"]
    ctx.set_params(p)
    with pytest.raises(capi.VVLICError) as e:
        ctx.render(vid, w.width, w.height)
    assert e.value.status == capi.ERR_NOT_READY
    p.technique = capi.TECHNIQUE["raycast"]
    ctx.set_params(p)
    with pytest.raises(capi.VVLICError) as e:
        ctx.update_field_device(vid, d_new.data_ptr(), (nx, ny, nz + 1), stream.cuda_stream)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    ctx.free_volume(fresh)
    ctx.free_volume(vid)


def test_lic_volume_stats(ctx):
    """vvlic_get_stats after vvlic_compute_lic_volume: one sample per voxel, L_b + L_f steps each,
    the kernel time."""
    w = small()
    vid = wl.setup_context(ctx, w)
    ctx.compute_lic_volume(vid, (24, 20, 16))
    st = ctx.stats()
    assert st.samples == 24 * 20 * 16
    assert st.sample_steps == st.samples * (w.params.steps_backward + w.params.steps_forward)
    assert st.rays == 0 and st.kernel_ms > 0 and st.check_flags == 0
    ctx.free_volume(vid)


def test_update_field_interp_equals_upload_field_interp(ctx):
    w = small()
    f0, f1 = w.field, other_field(w, seed=5)
    vid = wl.setup_context(ctx, w, storage="f16")
    render(ctx, vid, w, "hybrid")
    for index in (1, 3):
        ctx.update_field_interp(vid, f0, f1, index, 4)
        fresh = ctx.upload_field_interp(f0, f1, index, 4, storage="f16")
        np.testing.assert_array_equal(render(ctx, vid, w, "hybrid"), render(ctx, fresh, w, "hybrid"))
        ctx.free_volume(fresh)
    ctx.free_volume(vid)


def test_update_field_rejects_other_dimensions(ctx):
    w = small()
    vid = wl.setup_context(ctx, w)
    bad = np.zeros((w.field.shape[0] + 1,) + w.field.shape[1:], np.float32)
    with pytest.raises(capi.VVLICError) as e:
        ctx.update_field(vid, bad)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    with pytest.raises(capi.VVLICError) as e:
        ctx.update_field(vid + 1000, w.field)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    ctx.free_volume(vid)


def test_lic_volume_is_stale_after_update(ctx):
    w = small()
    vid = wl.setup_context(ctx, w)
    ctx.compute_lic_volume(vid, (24, 24, 24))
    p = w.params
    p.technique = capi.TECHNIQUE["licvolume"]
    ctx.set_params(p)
    ctx.render(vid, w.width, w.height)
    ctx.update_field(vid, other_field(w, seed=3))
    with pytest.raises(capi.VVLICError) as e:
        ctx.render(vid, w.width, w.height)
    assert e.value.status == capi.ERR_NOT_READY
    p.technique = capi.TECHNIQUE["raycast"]
    ctx.set_params(p)
    ctx.compute_lic_volume(vid, (24, 24, 24))
    fresh = ctx.upload_field(other_field(w, seed=3))
    ctx.compute_lic_volume(fresh, (24, 24, 24))
    p.technique = capi.TECHNIQUE["licvolume"]
    ctx.set_params(p)
    np.testing.assert_array_equal(ctx.render(vid, w.width, w.height), ctx.render(fresh, w.width, w.height))
    p.technique = capi.TECHNIQUE["raycast"]
    ctx.set_params(p)
    ctx.free_volume(fresh)
    ctx.free_volume(vid)


@pytest.mark.parametrize("sampler", ["cell", "texture", "hybrid"])
def test_same_shape_noise_upload_rewrites_every_layout(sampler):
    w = small()
    rng = np.random.default_rng(12)
    noise2 = rng.integers(0, 256, w.noise.shape, dtype=np.uint8)
    with capi.Context(0) as a, capi.Context(0) as b:
        va = wl.setup_context(a, w)
        render(a, va, w, sampler)  # builds the noise layout of the first noise
        a.upload_noise(noise2, w.noise_mode)
        got = render(a, va, w, sampler)
        vb = wl.setup_context(b, w)
        b.upload_noise(noise2, w.noise_mode)
        np.testing.assert_array_equal(got, render(b, vb, w, sampler))


def test_adjoint_tape_dropped_by_input_changes(ctx):
    import torch

    w = small()
    vid = wl.setup_context(ctx, w, storage="f16")
    g = torch.zeros((w.height, w.width, 4), dtype=torch.float32, device="cuda")
    d = [torch.zeros(n, dtype=torch.float32, device="cuda") for n in (1024, 256, 2 * 6 + 1)]

    def record():
        p = w.params
        p.sampler = capi.SAMPLER["hybrid"]
        p.record_tape = 1
        ctx.set_params(p)
        ctx.render(vid, w.width, w.height)
        p.record_tape = 0
        ctx.set_params(p)

    def adjoint():
        ctx.render_adjoint(vid, g.data_ptr(), w.width, w.height, *(x.data_ptr() for x in d))
        torch.cuda.synchronize()

    record()
    adjoint()  # a valid tape
    ctx.update_field(vid, other_field(w, seed=9))
    with pytest.raises(capi.VVLICError) as e:
        adjoint()
    assert e.value.status == capi.ERR_NOT_READY
    record()
    ctx.upload_noise(w.noise, w.noise_mode)
    with pytest.raises(capi.VVLICError) as e:
        adjoint()
    assert e.value.status == capi.ERR_NOT_READY
    record()
    ctx.free_volume(vid)
    with pytest.raises(capi.VVLICError) as e:
        adjoint()
    assert e.value.status in (capi.ERR_NOT_READY, capi.ERR_INVALID_ARGUMENT)


def test_batch_replay_follows_an_updated_field(ctx):
    import torch

    w = small()
    vid = wl.setup_context(ctx, w, storage="f16")
    p = w.params
    p.sampler = capi.SAMPLER["hybrid"]
    outs = [torch.zeros((w.height, w.width, 4), dtype=torch.float32, device="cuda") for _ in range(2)]
    views = [w.views[0], wl.perspective_view(wl.quat_axis_angle((0, 1, 0), 40.0), distance=2.2)]
    jobs = [capi.make_job(vid, o.data_ptr(), w.width, w.height, v, p, w.filter_table) for o, v in zip(outs, views)]
    stream = torch.cuda.Stream()
    ctx.batch_render(jobs, stream.cuda_stream)  # captures the graph
    stream.synchronize()
    ctx.update_field(vid, other_field(w, seed=21))
    ctx.batch_render(jobs, stream.cuda_stream)
    stream.synchronize()
    ctx.set_filter_table(w.filter_table)
    ctx.set_params(p)
    for o, v in zip(outs, views):
        ctx.set_view(v)
        np.testing.assert_array_equal(o.cpu().numpy(), ctx.render(vid, w.width, w.height))
    ctx.free_volume(vid)


def test_repeated_updates_allocate_nothing(ctx):
    # 96^3 FP16 field (7 MB texels, 57 MB cells, 7 MB texture array): a reallocation of any of
    # them would move the device's free memory by megabytes
    import torch

    w = wl.c1(size=96, image=64)
    w.params.steps_forward = w.params.steps_backward = 4
    vid = wl.setup_context(ctx, w, storage="f16")
    for sm in SAMPLERS:  # every layout exists before the updates
        render(ctx, vid, w, sm)
    ctx.update_field(vid, other_field(w, seed=40))  # grows the staging buffers once
    ctx.upload_noise(w.noise, w.noise_mode)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for k in range(3):
        ctx.update_field(vid, other_field(w, seed=41 + k))
        ctx.upload_noise(w.noise, w.noise_mode)
        for sm in SAMPLERS:
            render(ctx, vid, w, sm)
    torch.cuda.synchronize()
    assert abs(torch.cuda.mem_get_info()[0] - free0) < (1 << 20)
    ctx.free_volume(vid)


@pytest.mark.parametrize("lit", [False, True])
def test_stream_ordered_animation_equals_synchronous_steps(ctx, lit):
    """vvlic_update_field_async + vvlic_upload_noise_async + vvlic_render_to_host_async on one
    stream, all frames enqueued before a single wait, give the images of the synchronous
    update / upload / render sequence bit for bit (every copy overlaps the previous render)."""
    import torch

    w = small()
    if lit:
        w.params.illum = capi.ILLUM_GRADIENT
        w.noise_mode = capi.NOISE_GRAD_CENTRAL
    fields = [other_field(w, seed=s) for s in (11, 12, 13)]
    noises = [wl.dense_noise(w.noise.shape[::-1], seed=s) for s in (21, 22, 23)]
    views = [wl.perspective_view(wl.quat_axis_angle((0, 1, 0), a), distance=2.2) for a in (0.0, 40.0, 80.0)]
    W, H = w.width, w.height
    vid = wl.setup_context(ctx, w, storage="f16")
    p = w.params
    p.sampler = capi.SAMPLER["hybrid"]
    ctx.set_params(p)
    want = []
    for f, n, v in zip(fields, noises, views):
        ctx.update_field(vid, f)
        ctx.upload_noise(n, w.noise_mode)
        ctx.set_view(v)
        want.append(ctx.render(vid, W, H))
    ctx.update_field(vid, w.field)  # back to the first state
    hf = [torch.from_numpy(np.ascontiguousarray(f)).pin_memory() for f in fields]
    hn = [torch.from_numpy(np.ascontiguousarray(n)).pin_memory() for n in noises]
    out = [torch.empty((H, W, 4), dtype=torch.float32).pin_memory() for _ in fields]
    stream = torch.cuda.Stream()
    nz, ny, nx = w.field.shape[:3]
    for k, v in enumerate(views):
        ctx.update_field_async(vid, hf[k].data_ptr(), (nx, ny, nz), stream.cuda_stream)
        ctx.upload_noise_async(hn[k].data_ptr(), noises[k].shape[::-1], w.noise_mode, stream.cuda_stream)
        ctx.set_view(v)
        ctx.render_to_host_async(vid, out[k].data_ptr(), W, H, stream.cuda_stream)
    assert ctx.synchronize(stream.cuda_stream, timeout_ms=120000)
    for k in range(len(views)):
        np.testing.assert_array_equal(out[k].numpy(), want[k], err_msg=f"frame {k}")
    ctx.free_volume(vid)


def test_async_noise_needs_a_same_shape_noise(ctx):
    import torch

    w = small()
    wl.setup_context(ctx, w, storage="f16")
    other = wl.dense_noise((8, 8, 8), seed=3)
    h = torch.from_numpy(other).pin_memory()
    with pytest.raises(capi.VVLICError) as e:
        ctx.upload_noise_async(h.data_ptr(), (8, 8, 8), capi.NOISE_SCALAR, 0)
    assert e.value.status == capi.ERR_NOT_READY
