"""Batched rendering (vvlic_batch_render): every job of a batch of uneven volumes, views, LIC
lengths and filters equals the same job rendered alone bit for bit (the per-pixel computation
does not depend on the work distribution), and a sampled job matches the FP64 oracle.  The
graph replay path, a changed view between replays and the autotuner are exercised."""
import numpy as np
import pytest

from vectorvisualization_gb300 import capi, workloads as wl

pytestmark = pytest.mark.gpu


def small_batch(ctx, n_vol=5, image=48, storage="f16", sampler="hybrid"):
    import torch

    vols, noise, base = wl.c3(volumes=n_vol, image=image, max_views=3, dims=(16, 24, 32))
    ctx.upload_noise(noise)
    rgba, op = wl.default_tf()
    ctx.set_tf(rgba, op)
    jobs, outs, specs = [], [], []
    for bv in vols:
        vid = ctx.upload_field(bv.field, storage=storage)
        table = capi.make_filter_table(bv.filter_kind, 256)
        for v in bv.views:
            p = capi.Params.from_buffer_copy(base)
            p.steps_forward = p.steps_backward = bv.L // 4  # keep the test short
            p.sampler = capi.SAMPLER[sampler]
            out = torch.zeros((image, image, 4), dtype=torch.float32, device="cuda")
            outs.append(out)
            jobs.append(capi.make_job(vid, out.data_ptr(), image, image, v, p, table))
            specs.append((vid, v, p, table, bv))
    return jobs, outs, specs


@pytest.mark.parametrize("storage", ["f16", "bf16"])
def test_batch_equals_single_renders(ctx, storage):
    import torch

    jobs, outs, specs = small_batch(ctx, storage=storage)
    stream = torch.cuda.Stream()
    ctx.batch_render(jobs, stream.cuda_stream)
    stream.synchronize()
    st = ctx.stats()
    total_steps = 0
    for out, (vid, v, p, table, bv) in zip(outs, specs):
        ctx.set_filter_table(table)
        ctx.set_params(p)
        ctx.set_view(v)
        img = ctx.render(vid, out.shape[1], out.shape[0])
        total_steps += ctx.stats().sample_steps
        np.testing.assert_array_equal(out.cpu().numpy(), img)
    assert st.sample_steps == total_steps and st.sample_steps > 0


def test_batch_graph_replay_follows_changed_views(ctx):
    import torch

    jobs, outs, specs = small_batch(ctx, n_vol=3)
    stream = torch.cuda.Stream()
    ctx.batch_render(jobs, stream.cuda_stream)  # captures the graph
    stream.synchronize()
    # same shape, different views: the replay must pick up the new job table
    rng = wl.SplitMix64(99)
    for j in jobs:
        j.view = wl.random_view(rng)
    ctx.batch_render(jobs, stream.cuda_stream)
    stream.synchronize()
    for j, out, (vid, v, p, table, bv) in zip(jobs, outs, specs):
        ctx.set_filter_table(table)
        ctx.set_params(p)
        ctx.set_view(j.view)
        np.testing.assert_array_equal(out.cpu().numpy(), ctx.render(vid, out.shape[1], out.shape[0]))


def test_batch_job_matches_oracle(ctx, oracle):
    import torch

    jobs, outs, specs = small_batch(ctx, n_vol=2, storage="f32", sampler="cell")
    stream = torch.cuda.Stream()
    ctx.batch_render(jobs, stream.cuda_stream)
    stream.synchronize()
    rgba, op = wl.default_tf()
    noise = wl.c3(volumes=2, image=48, max_views=3, dims=(16, 24, 32))[1]
    for out, (vid, v, p, table, bv) in list(zip(outs, specs))[:3]:
        sc = oracle.Scene(oracle.encode_field(bv.field), noise, rgba, op, filter_table=table)
        ref, _ = sc.render(p, v, out.shape[1], out.shape[0])
        e = float(np.sqrt(np.mean((out.cpu().numpy().astype(np.float64) - ref) ** 2)))
        assert e <= 1e-3, e


def test_batch_autotune_and_validation(ctx):
    import torch

    jobs, outs, specs = small_batch(ctx, n_vol=2)
    stream = torch.cuda.Stream()
    tw, smp, ms = ctx.batch_autotune(jobs, stream.cuda_stream)
    assert tw in (4, 8, 16, 32) and smp in (capi.SAMPLER["hybrid"], capi.SAMPLER["cell"]) and ms > 0
    ctx.batch_render(jobs, stream.cuda_stream)
    stream.synchronize()
    for out, (vid, v, p, table, bv) in zip(outs, specs):
        ctx.set_filter_table(table)
        p2 = capi.Params.from_buffer_copy(p)
        p2.sampler = smp
        ctx.set_params(p2)
        ctx.set_view(v)
        np.testing.assert_array_equal(out.cpu().numpy(), ctx.render(vid, out.shape[1], out.shape[0]))
    # mixed integrators in one batch are rejected
    bad = [jobs[0], jobs[1]]
    p = capi.Params.from_buffer_copy(bad[1].params)
    p.integrator = capi.RK4
    bad[1] = capi.make_job(bad[1].vol_id, bad[1].d_out, bad[1].w, bad[1].h, bad[1].view, p)
    with pytest.raises(capi.VVLICError) as e:
        ctx.batch_render(bad, stream.cuda_stream)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
