"""The VVLIC_BOUNDS_CHECK build (the sanitizer substitute): every gather index, tape slot and
image pixel of the render and adjoint kernels is checked against its buffer, and an
out-of-range access would set a VVLIC_CHECK_* bit in the render's stats instead of touching
memory.  Small cases over every sampler, storage, integrator, shading model, technique, the
adjoint and a batch must report no such access and produce the default build's images."""
import numpy as np
import pytest

from vectorvisualization_gb300 import build, capi, workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked_lib():
    return capi.load(build.build(extra=["-DVVLIC_BOUNDS_CHECK=1"], variant="boundscheck"))


def small(integ=capi.HEUN, illum=capi.ILLUM_NONE, size=(20, 17, 14), image=(37, 29)):
    w = wl.c1(size=16, image=32)
    w.field = wl.vortex_field(size, seed=21)
    w.noise = wl.dense_noise(12, seed=22)[:, :, :11].copy()  # odd noise extent: the modulo path
    w.width, w.height = image
    p = w.params
    p.integrator = integ
    p.steps_forward, p.steps_backward = 5, 7
    p.illum = illum
    if illum == capi.ILLUM_GRADIENT:
        w.noise_mode = capi.NOISE_GRAD_CENTRAL
    return w


def render(lib, w, sampler, storage, view, technique="raycast", record=False):
    import torch

    with capi.Context(0, lib=lib) as ctx:
        vid = wl.setup_context(ctx, w, storage=storage)
        p = capi.Params.from_buffer_copy(w.params)
        p.sampler = capi.SAMPLER[sampler]
        p.technique = capi.TECHNIQUE[technique]
        p.record_tape = int(record)
        ctx.set_params(p)
        ctx.set_view(view)
        if technique == "licvolume":
            ctx.compute_lic_volume(vid, (9, 10, 11))
        out = torch.zeros((w.height, w.width, 4), dtype=torch.float32, device="cuda")
        ctx.render_device(vid, out.data_ptr(), w.width, w.height)
        torch.cuda.synchronize()
        flags = ctx.stats().check_flags
        grads = None
        if record:
            g = torch.ones_like(out)
            n = p.steps_forward + p.steps_backward + 1
            d = [torch.zeros(k, device="cuda") for k in (1024, 256, n)]
            ctx.render_adjoint(vid, g.data_ptr(), w.width, w.height, *(x.data_ptr() for x in d))
            torch.cuda.synchronize()
            flags |= ctx.stats().check_flags
            grads = [x.cpu().numpy() for x in d]
        return out.cpu().numpy(), flags, grads


VIEWS = [wl.ortho_view(), wl.perspective_view(wl.quat_axis_angle((1, 2, 0), 50.0), distance=1.6),
         wl.perspective_view(wl.quat_axis_angle((0, 1, 0), 200.0), distance=2.5)]


@pytest.mark.parametrize("sampler,storage", [("gather", "f32"), ("cell", "f16"), ("cell", "bf16"), ("cell", "u8"),
                                             ("texture", "f16"), ("hybrid", "u8"), ("hybrid", "f32"),
                                             ("hybrid", "bf16")])
def test_no_out_of_range_access_and_same_images(checked_lib, sampler, storage):
    default = capi.load()
    for integ, illum in ((capi.EULER, capi.ILLUM_NONE), (capi.RK4, capi.ILLUM_GRADIENT),
                         (capi.HEUN, capi.ILLUM_MALLO)):
        w = small(integ, illum)
        for v in VIEWS:
            img, flags, _ = render(checked_lib, w, sampler, storage, v)
            assert flags == 0, (sampler, storage, integ, illum, flags)
            ref, _, _ = render(default, w, sampler, storage, v)
            # the checks change no arithmetic; allow for a different contraction choice
            np.testing.assert_allclose(img, ref, rtol=0, atol=2e-6)


@pytest.mark.parametrize("technique", ["slicing", "volume", "licvolume"])
def test_techniques_in_range(checked_lib, technique):
    w = small()
    for v in VIEWS:
        _, flags, _ = render(checked_lib, w, "cell", "f16", v, technique=technique)
        assert flags == 0, (technique, flags)


@pytest.mark.parametrize("illum", [capi.ILLUM_NONE, capi.ILLUM_GRADIENT])
def test_adjoint_in_range(checked_lib, illum):
    w = small(capi.HEUN, illum)
    for v in VIEWS:
        _, flags, grads = render(checked_lib, w, "hybrid", "f16", v, record=True)
        assert flags == 0, flags
        _, _, ref = render(capi.load(), w, "hybrid", "f16", v, record=True)
        for got, want in zip(grads, ref):
            np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-4 * float(np.abs(want).max()))


def test_watchdog_times_out_then_completes(ctx):
    """vvlic_synchronize gives up at its deadline while a long render runs, then waits it out."""
    import torch

    w = wl.c2(size=128, image=768)
    vid = wl.setup_context(ctx, w)
    stream = torch.cuda.Stream()
    out = torch.empty((768, 768, 4), dtype=torch.float32, device="cuda")
    ctx.render_device(vid, out.data_ptr(), 768, 768, None, stream.cuda_stream)
    assert ctx.synchronize(stream.cuda_stream, timeout_ms=0) is False
    assert ctx.synchronize(stream.cuda_stream, timeout_ms=120000) is True
    assert float(out[..., 3].mean()) > 0
