"""torch.autograd.Function over the C ABI's recording render and adjoint (test harness only).

forward: upload the TF / opacity tables and explicit filter taps, render with
params.record_tape = 1 into a device image.  backward: vvlic_render_adjoint with the image
cotangent gives the gradients of the TF table, the opacity table and the taps.
"""
import torch

from vectorvisualization_gb300 import capi


class LICRender(torch.autograd.Function):
    @staticmethod
    def forward(ctx_fn, tf_rgba, tf_opac, taps, vctx: capi.Context, vid: int, params: capi.Params, w: int, h: int,
                inv_area: float):
        p = params
        p.record_tape = 1
        vctx.set_params(p)
        vctx.set_tf(tf_rgba.detach().cpu().numpy(), tf_opac.detach().cpu().numpy())
        vctx.set_filter_taps(taps.detach().cpu().numpy(), p.steps_backward, p.steps_forward, inv_area)
        out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
        vctx.render_device(vid, out.data_ptr(), w, h, None, torch.cuda.current_stream().cuda_stream)
        ctx_fn.vctx, ctx_fn.vid, ctx_fn.w, ctx_fn.h = vctx, vid, w, h
        ctx_fn.ntaps = taps.numel()
        return out

    @staticmethod
    def backward(ctx_fn, g_img):
        g = g_img.contiguous().float()
        d_tf = torch.empty((256, 4), dtype=torch.float32, device="cuda")
        d_op = torch.empty(256, dtype=torch.float32, device="cuda")
        d_taps = torch.empty(ctx_fn.ntaps, dtype=torch.float32, device="cuda")
        ctx_fn.vctx.render_adjoint(ctx_fn.vid, g.data_ptr(), ctx_fn.w, ctx_fn.h, d_tf.data_ptr(), d_op.data_ptr(),
                                   d_taps.data_ptr(), torch.cuda.current_stream().cuda_stream)
        return d_tf, d_op, d_taps, None, None, None, None, None, None


def render(tf_rgba, tf_opac, taps, vctx, vid, params, w, h, inv_area=0.5):
    return LICRender.apply(tf_rgba, tf_opac, taps, vctx, vid, params, w, h, inv_area)
