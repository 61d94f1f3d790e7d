"""Benchmark of the LIC volume ray-cast hot path (one JSON line on stdout).

Workload (default): the mid-size configuration with lighting and precision — a 256^3 field of a
uniform drift plus 8 seeded Gaussian vortices, dense uint8 noise (frequency 4.0) with
central-difference gradients, Heun streamlines L = 40 each way at step 0.005, Gaussian filter,
1024^2 image, ray spacing 1/256, gradient Phong lighting, FP16 field storage (FP32 and BF16 are
measured alongside).  A step is one frame.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is device throughput in Gsample-steps/s (one LIC integration step at one ray sample),
whole job over all ranks; `e2e` is the same metric through the C ABI with host buffers
(field + noise upload, preprocessing, render, image download inside the timed region).
`--impl reference` times the CPU restatement of the reference's path (the reference itself is
GLSL and cannot run without an OpenGL stack) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gsample-steps/s & frames/s, fwd and fwd+adjoint, at RMSE<=1e-3 vs FP64 oracle"
UNIT = "Gsample-steps/s"
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--storage", default="f16", choices=["f32", "f16", "bf16", "u8"])
    ap.add_argument("--sampler", default="hybrid", choices=["gather", "cell", "texture", "hybrid"])
    ap.add_argument("--schedule", default="queue", choices=["queue", "static"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--image", type=int, default=1024)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    # the batch (C3) and the large orbit (C5) run by default; --no-c3 / --no-c5 skip them
    ap.add_argument("--c3", dest="c3", action="store_true")
    ap.add_argument("--no-c3", dest="c3", action="store_false", help="skip the 64-volume batch")
    ap.add_argument("--c3-volumes", type=int, default=64)
    ap.add_argument("--c5", dest="c5", action="store_true")
    ap.add_argument("--no-c5", dest="c5", action="store_false", help="skip the 512^3 RK4 lit orbit")
    ap.add_argument("--c5-frames", type=int, default=2)
    ap.set_defaults(c3=True, c5=True)
    ap.add_argument("--c5-size", type=int, default=512)
    ap.add_argument("--c5-image", type=int, default=2048)
    return ap.parse_args()


# ---------------------------------------------------------------------------------------------
# distributed plumbing (one process per GPU; replicas of the same workload, no data exchange)
# ---------------------------------------------------------------------------------------------
def Dist(init: bool = True):
    from vectorvisualization_gb300.replicas import Replicas

    return Replicas(backend="nccl", init=init)


# ---------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="vvlic_clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ---------------------------------------------------------------------------------------------
def bytes_per_texel(storage: str) -> int:
    return 16 if storage == "f32" else 8


def algorithmic_bytes(stats, params, storage: str, lit: bool, pixels: int) -> float:
    """Cacheless trilinear-gather model: 8*(k*s_F + s_N) per sample-step, 8*s_F per sample for
    the compositing fetch, 16 B per output pixel."""
    k = {0: 1, 1: 2, 2: 4}[params.integrator]
    sF = bytes_per_texel(storage)
    sN = 4 if lit else 1
    return stats.sample_steps * 8 * (k * sF + sN) + stats.samples * 8 * sF + pixels * 16


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(workload_key: str):
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        d = json.load(fh)
    e = d.get(workload_key)
    return None if e is None else e.get("bytes_per_launch")


def make_workload(args):
    from vectorvisualization_gb300 import workloads as wl

    return wl.c2(size=args.size, image=args.image, storage=args.storage)


def cpu_sample(w, seconds: float, threads: int = 0, rows_offset: int = 0):
    """FP32 OpenMP CPU restatement on a stratified row subset sized to ~`seconds`."""
    from oracle import pyoracle
    from vectorvisualization_gb300 import capi

    rgba = pyoracle.round_storage(pyoracle.encode_field(w.field), w.storage)
    noise = w.noise if w.noise_mode == capi.NOISE_SCALAR else pyoracle.noise_gradients(w.noise, w.noise_mode)
    sc = pyoracle.Scene(rgba, noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)
    H = w.height
    # probe one row, then size the stratified subset
    probe_row = [H // 2 + rows_offset % max(1, H // 2)]
    t0 = time.perf_counter()
    _, s = sc.render(w.params, w.views[0], w.width, H, rows=probe_row, precision=32, threads=threads)
    dt = max(time.perf_counter() - t0, 1e-3)
    nrows = int(max(1, min(H, seconds / dt)))
    stride = max(1, H // nrows)
    rows = list(range((rows_offset % stride), H, stride))[:nrows]
    t0 = time.perf_counter()
    img, smp = sc.render(w.params, w.views[0], w.width, H, rows=rows, precision=32, threads=threads)
    dt = time.perf_counter() - t0
    steps = float(smp.astype(np.float64).sum()) * (w.params.steps_forward + w.params.steps_backward)
    return {"rate": steps / dt / 1e9, "seconds": dt, "rows": rows, "img": img, "sample_steps": steps,
            "threads": pyoracle.max_threads() if threads <= 0 else threads}


def run_reference(args, dist):
    """CPU restatement of the reference path, all host threads, bounded sample per step."""
    if dist.rank != 0:
        return 0
    w = make_workload(args)
    per_step = max(1.0, min(args.cpu_seconds, 20.0))
    for i in range(args.warmup):
        cpu_sample(w, per_step / 4, rows_offset=i)
    rates, secs, steps = [], 0.0, 0.0
    res = None
    for i in range(args.steps):
        res = cpu_sample(w, per_step, rows_offset=i + args.warmup)
        rates.append(res["rate"])
        secs += res["seconds"]
        steps += res["sample_steps"]
    value = steps / secs / 1e9
    full_frame_steps = None
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 vortex field and noise)",
        "config": {**w.describe(), "cpu_rows_per_step": len(res["rows"]) if res else 0},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": res["threads"] if res else 0, "kind": "port",
                         "sample": f"{len(res['rows']) if res else 0} stratified rows of the {w.width}x{w.height} "
                                   f"frame per step (FP32 OpenMP restatement of the GLSL path; the reference "
                                   f"itself runs only through OpenGL)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    del full_frame_steps
    print(json.dumps(line), flush=True)
    return 0


def bench_adjoint(ctx, torch, stream, flush, args):
    """C4: 128^3 vortex field, dense noise, Heun L=30 (61 taps), 512^2 x 4 views, L2 loss to a
    target rendered from a hidden seeded TF; gradients w.r.t. TF (256x4), opacity (256) and the
    61 taps.  Times the plain forward, the recording forward and the adjoint per view."""
    from vectorvisualization_gb300 import capi, workloads as wl

    w = wl.c4()
    w.storage = args.storage
    vid = wl.setup_context(ctx, w)
    L = w.params.steps_forward
    taps, inv_area = ctx.filter_taps()
    W, H = w.width, w.height
    p = w.params
    p.sampler = capi.SAMPLER[args.sampler]
    p.schedule = capi.SCHEDULE[args.schedule]
    sh = stream.cuda_stream
    img = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    # the hidden target: the same views rendered with another seeded TF
    ctx.set_tf(*wl.random_tf(seed=4040))
    ctx.set_params(p)
    targets = []
    for v in w.views:
        ctx.set_view(v)
        ctx.render_device(vid, img.data_ptr(), W, H, None, sh)
        stream.synchronize()
        targets.append(img.clone())
    ctx.set_tf(w.tf_rgba, w.tf_opac)
    d_tf = torch.empty((256, 4), dtype=torch.float32, device="cuda")
    d_op = torch.empty(256, dtype=torch.float32, device="cuda")
    d_taps = torch.empty(2 * L + 1, dtype=torch.float32, device="cuda")
    g = torch.empty_like(img)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            fn()
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    fwd_ms, rec_ms, adj_ms, steps = 0.0, 0.0, 0.0, 0
    for rep in range(2):  # first pass warms up
        f_ms = r_ms = a_ms = 0.0
        for v, tgt in zip(w.views, targets):
            ctx.set_view(v)
            p.record_tape = 0
            ctx.set_params(p)
            f_ms += timed(lambda: ctx.render_device(vid, img.data_ptr(), W, H, None, sh))
            steps_v = ctx.stats().sample_steps
            p.record_tape = 1
            ctx.set_params(p)
            r_ms += timed(lambda: ctx.render_device(vid, img.data_ptr(), W, H, None, sh))
            torch.mul(img - tgt, 2.0, out=g)

            def adj():
                ctx.render_adjoint(vid, g.data_ptr(), W, H, d_tf.data_ptr(), d_op.data_ptr(), d_taps.data_ptr(), sh)

            a_ms += timed(adj)
            if rep == 1:
                steps += steps_v
        fwd_ms, rec_ms, adj_ms = f_ms, r_ms, a_ms
    p.record_tape = 0
    ctx.set_params(p)
    ctx.free_volume(vid)
    return {
        "workload": "C4 vortex 128^3 dense-noise Heun L=30 (61 taps) 512^2 x 4 views, L2 to hidden-TF target",
        "storage": w.storage, "sampler": args.sampler,
        "fwd_ms": fwd_ms, "fwd_recording_ms": rec_ms, "adjoint_ms": adj_ms,
        "fwd_plus_adjoint_over_fwd": (rec_ms + adj_ms) / fwd_ms,
        "gss_fwd": steps / (fwd_ms / 1e3) / 1e9,
        "gss_fwd_adjoint": steps / ((rec_ms + adj_ms) / 1e3) / 1e9,
        "grad_norms": {"tf": float(d_tf.norm()), "opacity": float(d_op.norm()), "taps": float(d_taps.norm())},
    }


def bench_batch(ctx, torch, stream, flush, args):
    """C3: 64 volumes with per-axis dims from {64, 80, ..., 192} (ABC or vortex, own seeds), 1-8
    random views each at 512^2, filters mixed box / triangle / cos^2, L in [15, 60], FP16
    storage, Heun; one persistent launch per batch, replayed from a CUDA graph."""
    from vectorvisualization_gb300 import capi, workloads as wl

    t0 = time.perf_counter()
    vols, noise, base = wl.c3(volumes=args.c3_volumes)
    gen_s = time.perf_counter() - t0
    ctx.upload_noise(noise)
    ctx.set_tf(*wl.default_tf())
    jobs, outs = [], []
    voxels = 0
    for bv in vols:
        vid = ctx.upload_field(bv.field, storage=args.storage)
        voxels += bv.field.shape[0] * bv.field.shape[1] * bv.field.shape[2]
        table = capi.make_filter_table(bv.filter_kind, 256)
        for v in bv.views:
            p = capi.Params.from_buffer_copy(base)
            p.steps_forward = p.steps_backward = bv.L
            p.sampler = capi.SAMPLER[args.sampler]
            out = torch.empty((512, 512, 4), dtype=torch.float32, device="cuda")
            outs.append(out)
            jobs.append(capi.make_job(vid, out.data_ptr(), 512, 512, v, p, table))
    sh = stream.cuda_stream
    tw, smp, tune_ms = ctx.batch_autotune(jobs, sh)
    ctx.batch_render(jobs, sh)  # capture with the tuned shape
    stream.synchronize()
    times = []
    for _ in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            ctx.batch_render(jobs, sh)
            e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    st = ctx.stats()
    ms = min(times)
    # cacheless model for the unlit Heun batch: 8 (2 s_F + 1) B per sample-step
    sF = bytes_per_texel(args.storage)
    alg = st.sample_steps * 8 * (2 * sF + 1) + st.samples * 8 * sF + len(jobs) * 512 * 512 * 16
    peak, peak_kind = load_peaks()
    achieved = alg / (ms / 1e3) / 1e9
    # the plain FP32 form: the same jobs from FP32 texels with the gather sampler, one launch
    plain_ms = None
    with capi.Context(torch.cuda.current_device()) as pctx:
        pctx.upload_noise(noise)
        pctx.set_tf(*wl.default_tf())
        pjobs = []
        k = 0
        for bv in vols:
            pvid = pctx.upload_field(bv.field, storage="f32")
            table = capi.make_filter_table(bv.filter_kind, 256)
            for v in bv.views:
                p = capi.Params.from_buffer_copy(base)
                p.steps_forward = p.steps_backward = bv.L
                p.sampler = capi.SAMPLER["gather"]
                pjobs.append(capi.make_job(pvid, outs[k].data_ptr(), 512, 512, v, p, table))
                k += 1
        pctx.batch_render(pjobs, sh)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            pctx.batch_render(pjobs, sh)
            e1.record(stream)
        torch.cuda.synchronize()
        plain_ms = e0.elapsed_time(e1)
    return {
        "workload": f"C3 {len(vols)} volumes (dims 64..192 per axis), {len(jobs)} views at 512^2, L 15..60, "
                    f"mixed box/triangle/cos2, {args.storage}",
        "jobs": len(jobs), "voxels": voxels, "ms_per_batch": ms, "frames_per_s": len(jobs) / (ms / 1e3),
        "gss": st.sample_steps / (ms / 1e3) / 1e9, "sample_steps": int(st.sample_steps),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "algorithmic_bytes_per_batch": alg},
        "plain_f32_gather_ms": plain_ms, "speedup_vs_plain_f32": plain_ms / ms,
        "autotune": {"tile": f"{tw}x{32 // tw}", "sampler": [k for k, v in capi.SAMPLER.items() if v == smp][0],
                     "best_ms": tune_ms},
        "cuda_graph": True, "generation_s": gen_s,
    }


def bench_orbit(ctx, torch, stream, flush, args, dist):
    """C5: 512^3 FP16 solenoidal spectral field, dense gradient noise, RK4 L=60, step 1/512,
    2048^2, gradient lighting; `--c5-frames` frames of the 64-frame orbit per GPU (frames dealt
    round-robin over the ranks, each holding its own copy of the inputs), one launch each, L2
    flushed between frames (the 1.5 GiB field + noise working set exceeds L2 anyway)."""
    from vectorvisualization_gb300 import capi, workloads as wl

    t0 = time.perf_counter()
    w = wl.c5(size=args.c5_size, image=args.c5_image, frames=64, device="cuda")
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    vid = wl.setup_context(ctx, w)
    p = w.params
    p.sampler = capi.SAMPLER[args.sampler]
    p.schedule = capi.SCHEDULE[args.schedule]
    ctx.set_params(p)
    setup_s = time.perf_counter() - t0
    W, H = w.width, w.height
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    sh = stream.cuda_stream
    per_rank = max(1, min(args.c5_frames, 64 // dist.world))
    mine = dist.shard(per_rank * dist.world)
    frames = len(mine)
    with torch.cuda.stream(stream):
        ctx.render_device(vid, out.data_ptr(), W, H, None, sh)  # warm-up (cell layouts, tables)
    stream.synchronize()
    ms, steps, samples = [], 0, 0
    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    dist.barrier()
    for f in mine:
        ctx.set_view(w.views[f])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            ctx.render_device(vid, out.data_ptr(), W, H, None, sh)
            e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        st = ctx.stats()
        steps += int(st.sample_steps)
        samples += int(st.samples)
    clk = clocks.stop()
    adjoint = None
    if not args.no_adjoint:
        adjoint = orbit_adjoint(ctx, torch, stream, flush, w, vid, out, mine[0])
    total_ms = dist.max(sum(ms))
    steps, samples = dist.sum(float(steps)), dist.sum(float(samples))
    frames = per_rank * dist.world
    peak, peak_kind = load_peaks()

    class _S:
        pass

    agg = _S()
    agg.sample_steps, agg.samples = steps, samples
    alg = algorithmic_bytes(agg, p, w.storage, True, W * H * frames)
    achieved = alg / (total_ms / 1e3) / 1e9 / dist.world  # per GPU, against one GPU's peak
    key = f"c5/{w.storage}/{args.sampler}/{args.c5_size}/{args.c5_image}"
    traffic = load_traffic(key)
    return {
        "workload": w.name, "frames": frames, "ms_per_frame": total_ms / frames,
        "frames_per_s": frames / (total_ms / 1e3), "gss": steps / (total_ms / 1e3) / 1e9,
        "sample_steps_per_frame": steps / frames, "samples_per_frame": samples / frames,
        "sampler": args.sampler, "storage": w.storage,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind, "algorithmic_bytes_per_frame": alg / frames},
        "clocks": clk, "generation_s": gen_s, "setup_s": setup_s,
        "image_alpha_mean": float(out[..., 3].mean()),
        "fwd_adjoint": adjoint,
    }


def orbit_adjoint(ctx, torch, stream, flush, w, vid, out, frame):
    """Forward (recording) + adjoint of one lit C5 frame: L2 loss to the same frame rendered with
    another transfer function; gradients for the TF, opacity and 121 taps."""
    from vectorvisualization_gb300 import workloads as wl

    W, H = w.width, w.height
    sh = stream.cuda_stream
    p = w.params
    ctx.set_view(w.views[frame])
    target = torch.empty_like(out)
    ctx.set_tf(*wl.random_tf(seed=505))
    ctx.render_device(vid, target.data_ptr(), W, H, None, sh)
    ctx.set_tf(w.tf_rgba, w.tf_opac)
    stream.synchronize()
    ntaps = p.steps_forward + p.steps_backward + 1
    d_tf = torch.empty((256, 4), dtype=torch.float32, device="cuda")
    d_op = torch.empty(256, dtype=torch.float32, device="cuda")
    d_taps = torch.empty(ntaps, dtype=torch.float32, device="cuda")
    g = torch.empty_like(out)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0.record(stream)
            fn()
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    p.record_tape = 0
    ctx.set_params(p)
    fwd_ms = timed(lambda: ctx.render_device(vid, out.data_ptr(), W, H, None, sh))
    steps = ctx.stats().sample_steps
    p.record_tape = 1
    ctx.set_params(p)
    rec_ms = timed(lambda: ctx.render_device(vid, out.data_ptr(), W, H, None, sh))
    with torch.cuda.stream(stream):
        torch.mul(out - target, 2.0, out=g)
    adj_ms = timed(lambda: ctx.render_adjoint(vid, g.data_ptr(), W, H, d_tf.data_ptr(), d_op.data_ptr(),
                                              d_taps.data_ptr(), sh))
    p.record_tape = 0
    ctx.set_params(p)
    return {"frame": frame, "fwd_ms": fwd_ms, "fwd_recording_ms": rec_ms, "adjoint_ms": adj_ms,
            "fwd_plus_adjoint_over_fwd": (rec_ms + adj_ms) / fwd_ms,
            "gss_fwd": steps / (fwd_ms / 1e3) / 1e9, "gss_fwd_adjoint": steps / ((rec_ms + adj_ms) / 1e3) / 1e9,
            "finite": bool(torch.isfinite(d_tf).all() and torch.isfinite(d_taps).all()),
            "grad_norms": {"tf": float(d_tf.norm()), "opacity": float(d_op.norm()), "taps": float(d_taps.norm())}}


def run_ours(args, dist):
    import torch

    from vectorvisualization_gb300 import build, capi, workloads as wl

    build.build()
    dev = dist.local
    torch.cuda.set_device(dev)
    w = make_workload(args)
    lit = w.params.illum == capi.ILLUM_GRADIENT
    ctx = capi.Context(dev)
    vid = wl.setup_context(ctx, w)
    p = w.params
    p.sampler = capi.SAMPLER[args.sampler]
    p.schedule = capi.SCHEDULE[args.schedule]
    ctx.set_params(p)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    W, H = w.width, w.height
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def frame():
        ctx.render_device(vid, out.data_ptr(), W, H, None, sh)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            frame()
    stream.synchronize()
    st0 = ctx.stats()

    clocks = Clocks(dev)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()  # L2 flush between frames, outside the event pair
            starts[k].record(stream)
            frame()
            ends[k].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    dist.barrier()
    clk = clocks.stop()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    st = ctx.stats()
    assert st.sample_steps == st0.sample_steps
    kernel_ms = sum(times)
    steps_rank = st.sample_steps * args.steps
    total_steps = dist.sum(float(steps_rank))
    max_ms = dist.max(kernel_ms)
    value = total_steps / (max_ms / 1e3) / 1e9
    ms_per_step = max_ms / args.steps

    peak, peak_kind = load_peaks()
    alg = algorithmic_bytes(st, p, w.storage, lit, W * H)
    achieved = alg / (ms_per_step / 1e3) / 1e9
    key = f"c2/{w.storage}/{args.sampler}/{args.size}/{args.image}"
    traffic = load_traffic(key)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": alg,
                "model": "8*(k*s_F+s_N) B per sample-step + 8*s_F per sample + 16 B per pixel"}

    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "frames_per_s": 1e3 / ms_per_step * dist.world,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 vortex field and noise; the reference ships no datasets)",
        "config": {**w.describe(), "sampler": args.sampler, "schedule": args.schedule,
                   "l2": "flushed between frames (256 MiB write); inputs > L2",
                   "sample_steps_per_frame": int(st.sample_steps), "samples_per_frame": int(st.samples),
                   "rays": int(st.rays), "parallelism": f"replicas x{dist.world}"},
        "wall_ms_per_step": t_wall / args.steps * 1e3,
        "image_alpha_mean": float(out[..., 3].mean()),
        "roofline": roofline,
        # per frame: the queue schedule's tile order (cost, bucket scan, scatter) + the ray-cast
        "gpu_launches": args.steps * (4 if args.schedule == "queue" else 1),
        "clocks": clk,
    }

    # reduced / full precision storage alongside (same frame, same sampler)
    if not args.no_variants and dist.rank == 0:
        variants = {}
        for storage in ("f32", "f16", "bf16"):
            if storage == w.storage:
                variants[storage] = {"gss": value / dist.world, "ms": ms_per_step}
                continue
            vid2 = ctx.upload_field(w.field, storage=storage)
            with torch.cuda.stream(stream):
                frame2 = lambda: ctx.render_device(vid2, out.data_ptr(), W, H, None, sh)  # noqa: E731
                frame2()
                stream.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                flush.zero_()
                e0.record(stream)
                frame2()
                e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            s2 = ctx.stats()
            variants[storage] = {"gss": s2.sample_steps / (ms / 1e3) / 1e9, "ms": ms}
            ctx.free_volume(vid2)
        line["storage_variants"] = variants

    # forward + adjoint on the differentiable-fit configuration (unlit; 4 views)
    if not args.no_adjoint and dist.rank == 0:
        with capi.Context(dev) as actx:
            line["fwd_adjoint"] = bench_adjoint(actx, torch, stream, flush, args)
    if args.c3 and dist.rank == 0:
        with capi.Context(dev) as bctx:
            line["batch"] = bench_batch(bctx, torch, stream, flush, args)
    if args.c5:
        with capi.Context(dev) as octx:
            orbit = bench_orbit(octx, torch, stream, flush, args, dist)
        if dist.rank == 0:
            line["orbit"] = orbit

    # end to end through the C ABI with host buffers
    if not args.no_e2e:
        field_h = torch.from_numpy(np.ascontiguousarray(w.field)).pin_memory()
        noise_h = torch.from_numpy(np.ascontiguousarray(w.noise)).pin_memory()
        img_h = torch.empty((H, W, 4), dtype=torch.float32).pin_memory()
        lib = capi.load()
        nz, ny, nx = w.field.shape[:3]
        mz, my, mx = w.noise.shape
        e2e_steps = max(1, min(args.steps, 3))
        e2e_vid = None

        def e2e_step():
            # the animation path (a new field and noise every frame): the first step creates the
            # volume, later steps rewrite it in place (vvlic_update_field; the same-shape noise
            # upload is in place too); every step copies both from pinned host memory, encodes,
            # recomputes the noise gradients and cell / texture layouts, renders and downloads
            nonlocal e2e_vid
            if e2e_vid is None:
                v = capi._I(0)
                ctx._check(lib.vvlic_upload_field(ctx.h, field_h.data_ptr(), capi.DTYPE_FLOAT32, nx, ny, nz, None,
                                                  capi.STORAGE[w.storage], capi.C.byref(v)), "upload_field")
                e2e_vid = v.value
            else:
                ctx._check(lib.vvlic_update_field(ctx.h, e2e_vid, field_h.data_ptr(), capi.DTYPE_FLOAT32, nx, ny, nz),
                           "update_field")
            ctx._check(lib.vvlic_upload_noise(ctx.h, noise_h.data_ptr(), mx, my, mz, w.noise_mode), "upload_noise")
            ctx._check(lib.vvlic_render(ctx.h, e2e_vid, img_h.data_ptr(), W, H), "render")

        e2e_step()
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        t = time.perf_counter() - t0
        t = dist.max(t)
        s3 = ctx.stats()
        line["e2e"] = {"value": dist.sum(float(s3.sample_steps * e2e_steps)) / t / 1e9, "unit": UNIT,
                       "h2d_bytes_per_step": int(field_h.numel() * 4 + noise_h.numel()),
                       "d2h_bytes_per_step": int(img_h.numel() * 4),
                       "ms_per_step": t / e2e_steps * 1e3,
                       "includes": "field upload+encode (in place), noise upload+gradients, cell and texture "
                                   "layout rebuilds, render, image download"}
        ctx.free_volume(e2e_vid)

    # CPU baseline (rank 0, N=1 only): the FP32 OpenMP restatement on a bounded sample
    if not args.no_cpu and dist.rank == 0 and dist.world == 1:
        res = cpu_sample(w, args.cpu_seconds)
        gpu_rows = out.cpu().numpy()[res["rows"]]
        line["cpu_baseline"] = {
            "value": res["rate"], "unit": UNIT, "cores": res["threads"], "kind": "port",
            "sample": f"{len(res['rows'])} stratified rows of the {W}x{H} frame ({res['seconds']:.1f} s, "
                      f"FP32 OpenMP restatement of the reference GLSL path)",
            "rmse_gpu_vs_cpu_rows": float(np.sqrt(np.mean((gpu_rows.astype(np.float64) - res["img"]) ** 2))),
        }
    ctx.close()
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    # the reference arm runs on rank 0 only and needs no process group
    dist = Dist(init=args.impl == "ours")
    try:
        if args.impl == "reference":
            return run_reference(args, dist)
        return run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
