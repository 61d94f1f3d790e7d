"""Benchmark of the LIC volume ray-cast hot path (one JSON line on stdout).

Headline workload: the large turbulence orbit — a 512^3 FP16 divergence-free spectral field
(random-phase Fourier modes, E(k) ~ k^-5/3 for k in [2, 64], seed 5), dense uint8 noise with
central-difference gradients, RK4 streamlines L = 60 each way at step 1/512, Gaussian filter,
2048^2 image at ray spacing 1/512, gradient Phong lighting, a 64-frame orbit.  A step is one
frame; K steps render K frames spread evenly over the orbit (all 64 when K = 64).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is device throughput in Gsample-steps/s (one LIC integration step at one ray sample),
whole job over all ranks (replicas: every rank renders its own share of frames).  `e2e` is the
same metric through the C ABI with host buffers: every step copies the field and the noise from
pinned host memory, re-encodes the field, recomputes the noise gradients and layouts, renders
and downloads the image.  `roofline` compares the kernel's fetch rate with the measured L1TEX
fetch ceiling of the GPU (vvlic_measure_fetch_ceiling); DRAM figures are reported beside it.
Extra keys: the mid-size lit frame with FP32/FP16/BF16 storage (`c2`), the 64-volume batch
(`batch`), the differentiable-fit forward+adjoint (`fwd_adjoint`), the orbit's forward+adjoint
(`orbit_adjoint`), the TMA-staged brick sampler against the texture and gather samplers
(`brick_ab`), and the techniques and preprocessing beside the ray-cast on the orbit's volume —
slicing, LIC-volume precompute and ray-cast, vector-field DVR, device field update, noise
gradients — each against its bound (`rows`).

`--impl reference` times the CPU restatement of the reference's path (the reference itself is
GLSL and runs only through OpenGL) on all host cores, on stratified rows of the same orbit
frames, with inputs built by the oracle alone (libvvlic is not loaded).
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
ORBIT_FRAMES = 64


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--sampler", default="hybrid", choices=["gather", "cell", "texture", "hybrid"])
    ap.add_argument("--schedule", default="auto", choices=["auto", "queue", "static"],
                    help="auto: the schedule measured faster per workload (static for the orbit frames, "
                         "queue for the others)")
    ap.add_argument("--size", type=int, default=512, help="orbit field size per axis")
    ap.add_argument("--image", type=int, default=2048, help="orbit image size")
    ap.add_argument("--c2-size", type=int, default=256)
    ap.add_argument("--c2-image", type=int, default=1024)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-c3", action="store_true", help="skip the 64-volume batch")
    ap.add_argument("--no-c4", action="store_true", help="skip the differentiable-fit forward+adjoint")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the orbit's forward+adjoint")
    ap.add_argument("--no-rows", action="store_true",
                    help="skip the techniques and preprocessing beside the ray-cast (on the orbit's volume)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ceiling", action="store_true", help="skip the L1TEX fetch-ceiling measurement")
    ap.add_argument("--c3-volumes", type=int, default=64)
    ap.add_argument("--only", default="all", choices=["all", "c5", "c2", "c3", "c4", "brick"],
                    help="run one section alone (profiling); its results are the only keys printed")
    return ap.parse_args()


def schedule(args, workload: str) -> str:
    """The work distribution of a section.  Measured on one GB300 (ms per frame): the orbit's
    2048^2 RK4 frames run about 3 % faster on the static raster grid (1230 / 1419 / 1491 against
    1268 / 1455 / 1540 for frames 0 / 16 / 40), the lit 1024^2 Heun frame about 3 % faster on
    the longest-first queue; `auto` takes the faster per workload."""
    if args.schedule != "auto":
        return args.schedule
    return "static" if workload == "orbit" else "queue"


def orbit_frames(steps: int, world: int, rank: int) -> list[int]:
    """Frames of the 64-frame orbit that `rank` renders: the steps*world global steps spread
    evenly over the orbit, dealt round-robin."""
    total = steps * world
    return [((k * world + rank) * ORBIT_FRAMES // total) % ORBIT_FRAMES for k in range(steps)]


# ---------------------------------------------------------------------------------------------
# distributed plumbing (one process per GPU; replicas of the workload, no data exchange)
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
# roofline helpers
# ---------------------------------------------------------------------------------------------
FIELD_EVALS = {0: 1, 1: 2, 2: 4}  # field evaluations per streamline step: Euler, Heun, RK4
GROUP_KEY = {0: "euler", 1: "heun", 2: "rk4"}


def bytes_per_texel(storage: str) -> int:
    """RGBA texel bytes of a field storage: FP32 16, FP16 / BF16 8, UNORM8 4."""
    return {"f32": 16, "f16": 8, "bf16": 8, "u8": 4}[storage]


def cacheless_bytes(sample_steps: float, samples: float, integrator: int, storage: str, lit: bool,
                    pixels: int) -> float:
    """Cacheless trilinear-gather model: 8*(k*s_F + s_N) per sample-step, 8*s_F per sample for
    the compositing fetch, 16 B per output pixel."""
    k = FIELD_EVALS[integrator]
    sF = bytes_per_texel(storage)
    sN = 4 if lit else 1
    return sample_steps * 8 * (k * sF + sN) + samples * 8 * sF + pixels * 16


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(workload_key: str):
    """DRAM bytes per launch of the workload's render kernel from the committed ncu capture, if
    that capture was made with the current kernel sources (else None: the figure is stale)."""
    from vectorvisualization_gb300 import build

    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        d = json.load(fh)
    e = d.get(workload_key)
    if e is None or e.get("source_digest") != build.source_digest():
        return None
    return e.get("bytes_per_launch")


def roofline(steps: float, samples: float, ms: float, integrator: int, storage: str, lit: bool, pixels: int,
             ceiling: dict | None, traffic_key: str) -> dict:
    """The render kernel against the L1TEX fetch ceiling (the bound that applies: the field comes
    through the texture unit, the noise cells through 256-bit loads, and both hit L1 or L2), with
    DRAM beside it.  A fetch group is one noise-cell load plus the k field fetches of one
    streamline step; per launch there are samples*(L_b+L_f+1) noise taps = steps + samples."""
    peak_hbm, peak_kind = load_peaks()
    secs = ms / 1e3
    groups = steps + samples
    k = FIELD_EVALS[integrator]
    traffic = load_traffic(traffic_key)
    alg = cacheless_bytes(steps, samples, integrator, storage, lit, pixels)
    hbm = {"peak_gbs": peak_hbm, "peak_kind": peak_kind,
           "dram_bytes_per_launch": traffic,
           "dram_gbs": None if traffic is None else traffic / secs / 1e9,
           "dram_frac": None if traffic is None else traffic / secs / 1e9 / peak_hbm,
           "cacheless_model_bytes_per_launch": alg,
           "cacheless_model_ratio": alg / secs / 1e9 / peak_hbm,
           "note": "cacheless_model_ratio counts every texel of every trilinear as DRAM bytes; it "
                   "measures cache reuse, not HBM use"}
    r = {"bound": "l1tex", "unit": "G fetch-groups/s", "traffic": traffic,
         "fetch_group": f"one 256-bit noise-cell load + {k} trilinear field fetches (one streamline step)",
         "per_launch": {"noise_cell_loads": groups, "field_fetches": k * steps + samples, "kernel_ms": ms},
         "achieved": groups / secs / 1e9, "hbm": hbm}
    if ceiling:
        peak = ceiling["group_per_s"][GROUP_KEY[integrator]] / 1e9
        r.update({"peak": peak, "frac": r["achieved"] / peak, "peak_kind": "measured (vvlic_measure_fetch_ceiling)"})
    else:
        r.update({"peak": None, "frac": None, "peak_kind": "not measured"})
    return r


# ---------------------------------------------------------------------------------------------
# CPU restatement (oracle) on stratified rows
# ---------------------------------------------------------------------------------------------
def cpu_scene(w):
    """Oracle scene of a workload: the field encoded and rounded to its storage by the oracle,
    the noise gradients computed by the oracle."""
    from oracle import pyoracle
    from vectorvisualization_gb300 import capi

    rgba = pyoracle.encode_field(w.field)
    if w.storage != "f32":
        rgba = pyoracle.round_storage(rgba, w.storage)
    noise = w.noise if w.noise_mode == capi.NOISE_SCALAR else pyoracle.noise_gradients(w.noise, w.noise_mode)
    return pyoracle.Scene(rgba, noise, w.tf_rgba, w.tf_opac, filter_table=w.filter_table)


def cpu_sample(sc, w, view, seconds: float, threads: int = 0, rows_offset: int = 0, row_seconds=None):
    """FP32 OpenMP CPU restatement on about `seconds` of stratified rows: evenly spaced over the
    whole frame (the k-th of n rows at (k + f) H / n, f shifted per call by the golden ratio), so
    that dense centre rows and sparse edge rows enter in their proportion.  `row_seconds` is the
    time of one central row (measured here when not given)."""
    from oracle import pyoracle

    H = w.height
    if row_seconds is None:
        t0 = time.perf_counter()
        sc.render(w.params, view, w.width, H, rows=[H // 2], precision=32, threads=threads)
        row_seconds = max(time.perf_counter() - t0, 1e-3)
    nrows = int(max(1, min(H, seconds / row_seconds)))
    f = (0.5 + 0.6180339887 * rows_offset) % 1.0
    rows = sorted({min(H - 1, int((k + f) * H / nrows)) for k in range(nrows)})
    t0 = time.perf_counter()
    img, smp = sc.render(w.params, view, w.width, H, rows=rows, precision=32, threads=threads)
    dt = time.perf_counter() - t0
    steps = float(smp.astype(np.float64).sum()) * (w.params.steps_forward + w.params.steps_backward)
    return {"rate": steps / dt / 1e9, "seconds": dt, "rows": rows, "img": img, "sample_steps": steps,
            "row_seconds": row_seconds, "threads": pyoracle.max_threads() if threads <= 0 else threads}


def run_reference(args, dist):
    """The CPU restatement of the reference path on all host threads, on stratified rows of the
    same orbit frames as the GPU arm; the workload is built by the oracle (no libvvlic)."""
    if dist.rank != 0:
        return 0
    from oracle import pyoracle
    from vectorvisualization_gb300 import workloads as wl

    t0 = time.perf_counter()
    w = wl.c5(size=args.size, image=args.image, frames=ORBIT_FRAMES, defaults=pyoracle.DEFAULTS)
    sc = cpu_scene(w)
    prep_s = time.perf_counter() - t0
    frames = orbit_frames(args.steps, 1, 0)
    # the whole run stays within a few minutes: about 120 s of timed CPU work in all
    per_step = max(1.0, min(args.cpu_seconds, 120.0 / max(1, args.steps)))
    row_s = None
    for i in range(args.warmup):
        row_s = cpu_sample(sc, w, w.views[frames[i % len(frames)]], per_step / 4, rows_offset=i,
                           row_seconds=row_s)["row_seconds"]
    secs, steps, rows = 0.0, 0.0, 0
    res = None
    for i, f in enumerate(frames):
        res = cpu_sample(sc, w, w.views[f], per_step, rows_offset=i + args.warmup, row_seconds=row_s)
        secs += res["seconds"]
        steps += res["sample_steps"]
        rows += len(res["rows"])
    value = steps / secs / 1e9
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
        "data": "synthetic (seeded SplitMix64 spectral field and noise; the reference ships no datasets)",
        "config": {**w.describe(), "frames": frames, "cpu_rows_per_step": rows / max(1, len(frames)),
                   "input_build_s": prep_s},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": res["threads"] if res else 0, "kind": "port",
                         "sample": f"about {rows // max(1, len(frames))} stratified rows of each {w.width}x{w.height} "
                                   f"orbit frame per step (FP32 OpenMP restatement of the GLSL path; the reference "
                                   f"itself runs only through OpenGL)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------
# sections of the GPU arm
# ---------------------------------------------------------------------------------------------
def timed(torch, stream, flush, fn) -> float:
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        flush.zero_()
        e0.record(stream)
        fn()
        e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def bench_c2(ctx, torch, stream, flush, args, ceiling):
    """C2: 256^3 drift + 8 vortices, dense noise (freq 4) with central-difference gradients, Heun
    L = 40 at 0.005, Gaussian filter, 1024^2, spacing 1/256, gradient lighting; f16 field, with
    the f32 and bf16 storage of the same frame beside it."""
    from vectorvisualization_gb300 import capi, workloads as wl

    w = wl.c2(size=args.c2_size, image=args.c2_image, storage="f16")
    vid = wl.setup_context(ctx, w)
    p = w.params
    p.sampler = capi.SAMPLER[args.sampler]
    p.schedule = capi.SCHEDULE[schedule(args, "c2")]
    ctx.set_params(p)
    W, H = w.width, w.height
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    sh = stream.cuda_stream
    frame = lambda v: ctx.render_device(v, out.data_ptr(), W, H, None, sh)  # noqa: E731
    for _ in range(2):
        timed(torch, stream, flush, lambda: frame(vid))
    n = max(3, min(args.steps, 10))
    ms = [timed(torch, stream, flush, lambda: frame(vid)) for _ in range(n)]
    st = ctx.stats()
    mean = sum(ms) / len(ms)
    res = {"workload": w.name, "frames": n, "ms_per_frame": mean, "gss": st.sample_steps / (mean / 1e3) / 1e9,
           "sample_steps_per_frame": int(st.sample_steps), "samples_per_frame": int(st.samples),
           "image_alpha_mean": float(out[..., 3].mean()),
           "roofline": roofline(st.sample_steps, st.samples, mean, p.integrator, "f16", True, W * H, ceiling,
                                f"c2/f16/{args.sampler}/{args.c2_size}/{args.c2_image}")}
    variants = {"f16": {"gss": res["gss"], "ms": mean}}
    for storage in ("f32", "bf16"):
        vid2 = ctx.upload_field(w.field, storage=storage)
        timed(torch, stream, flush, lambda: frame(vid2))
        ms2 = timed(torch, stream, flush, lambda: frame(vid2))
        s2 = ctx.stats()
        variants[storage] = {"gss": s2.sample_steps / (ms2 / 1e3) / 1e9, "ms": ms2}
        ctx.free_volume(vid2)
    variants["bf16"]["note"] = ("bf16 texels via their f16 texture copy: the texture and hybrid samplers read a "
                                "half4 texture, so this is the f16 kernel on bf16-valued data")
    res["storage_variants"] = variants
    ctx.free_volume(vid)
    return res


def bench_brick(ctx, torch, stream, flush, args):
    """The BRICK sampler (field and noise bricks staged in shared memory by TMA) against the
    hardware-trilinear texture path and the gathers, on the configurations where a brick holds
    a segment's streamline reach (the plain 64^3 case: Euler L = 20 reaches 4 texels) and where
    it does not (the fit's 128^3 Heun L = 30 frame: 12 texels each way)."""
    from vectorvisualization_gb300 import capi, workloads as wl

    res = {}
    for name, w, storage in (("C1 64^3 f32 Euler L=20 box 256^2 ortho", wl.c1(), "f32"),
                             ("C4 128^3 f16 Heun L=30 512^2 view 0", wl.c4(), "f16")):
        vid = wl.setup_context(ctx, w, storage=storage)
        W, H = w.width, w.height
        out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        row = {}
        for sampler in ("brick", "gather", "cell", "texture", "hybrid"):
            p = capi.Params.from_buffer_copy(w.params)
            p.sampler = capi.SAMPLER[sampler]
            p.schedule = capi.SCHEDULE["static" if sampler == "brick" else schedule(args, "brick_ab")]
            ctx.set_params(p)
            frame = lambda: ctx.render_device(vid, out.data_ptr(), W, H, None, stream.cuda_stream)  # noqa: E731
            timed(torch, stream, flush, frame)
            ms = min(timed(torch, stream, flush, frame) for _ in range(5))
            st = ctx.stats()
            row[sampler] = {"ms": ms, "gss": st.sample_steps / (ms / 1e3) / 1e9, "check_flags": int(st.check_flags)}
        res[name] = row
        ctx.free_volume(vid)
    return res


def bench_c4(ctx, torch, stream, flush, args):
    """C4: 128^3 vortex field, dense noise, Heun L=30 (61 taps), 512^2 x 4 views, L2 loss to a
    target rendered from a hidden seeded TF; gradients w.r.t. TF (256x4), opacity (256) and the
    61 taps.  Times the plain forward, the recording forward and the adjoint per view."""
    from vectorvisualization_gb300 import capi, workloads as wl

    w = wl.c4()
    w.storage = "f16"
    vid = wl.setup_context(ctx, w)
    L = w.params.steps_forward
    W, H = w.width, w.height
    p = w.params
    p.sampler = capi.SAMPLER[args.sampler]
    p.schedule = capi.SCHEDULE[schedule(args, "c4")]
    sh = stream.cuda_stream
    img = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    ctx.set_tf(*wl.random_tf(seed=4040))  # the hidden target TF
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
    fwd_ms, rec_ms, adj_ms, steps = 0.0, 0.0, 0.0, 0
    for rep in range(2):  # the first pass warms up
        f_ms = r_ms = a_ms = 0.0
        for v, tgt in zip(w.views, targets):
            ctx.set_view(v)
            p.record_tape = 0
            ctx.set_params(p)
            f_ms += timed(torch, stream, flush, lambda: ctx.render_device(vid, img.data_ptr(), W, H, None, sh))
            steps_v = ctx.stats().sample_steps
            p.record_tape = 1
            ctx.set_params(p)
            r_ms += timed(torch, stream, flush, lambda: ctx.render_device(vid, img.data_ptr(), W, H, None, sh))
            torch.mul(img - tgt, 2.0, out=g)
            a_ms += timed(torch, stream, flush, lambda: ctx.render_adjoint(
                vid, g.data_ptr(), W, H, d_tf.data_ptr(), d_op.data_ptr(), d_taps.data_ptr(), sh))
            if rep == 1:
                steps += steps_v
        fwd_ms, rec_ms, adj_ms = f_ms, r_ms, a_ms
    flags = ctx.stats().check_flags
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
        "tape_overflow": bool(flags & capi.CHECK_TAPE_OVERFLOW),
        "grad_norms": {"tf": float(d_tf.norm()), "opacity": float(d_op.norm()), "taps": float(d_taps.norm())},
    }


def bench_batch(ctx, torch, stream, flush, args, dist):
    """C3: 64 volumes with per-axis dims from {64, 80, ..., 192} (ABC or vortex, own seeds), 1-8
    random views each at 512^2, filters mixed box / triangle / cos^2, L in [15, 60], FP16
    storage, Heun; one persistent launch per batch, replayed from a CUDA graph.  Under N ranks
    every rank renders its cost-balanced share of the jobs (replicas, no exchange)."""
    from vectorvisualization_gb300 import capi, workloads as wl
    from vectorvisualization_gb300.replicas import shard_by_cost

    t0 = time.perf_counter()
    vols, noise, base = wl.c3(volumes=args.c3_volumes)
    gen_s = time.perf_counter() - t0
    specs, costs = wl.c3_jobs(vols)
    mine = shard_by_cost(costs, dist.rank, dist.world)
    ctx.upload_noise(noise)
    ctx.set_tf(*wl.default_tf())

    def make_jobs(c, storage, sampler, outs):
        vids, jobs = {}, []
        for k, i in enumerate(mine):
            bv, v = specs[i]
            if id(bv) not in vids:
                vids[id(bv)] = c.upload_field(bv.field, storage=storage)
            p = capi.Params.from_buffer_copy(base)
            p.steps_forward = p.steps_backward = bv.L
            p.sampler = capi.SAMPLER[sampler]
            jobs.append(capi.make_job(vids[id(bv)], outs[k].data_ptr(), 512, 512, v, p,
                                      capi.make_filter_table(bv.filter_kind, 256)))
        return jobs, vids

    outs = [torch.empty((512, 512, 4), dtype=torch.float32, device="cuda") for _ in mine]
    jobs, vids = make_jobs(ctx, "f16", args.sampler, outs)
    voxels = sum(int(np.prod(bv.field.shape[:3])) for bv in vols if id(bv) in vids)
    sh = stream.cuda_stream
    tw, smp, tune_ms = ctx.batch_autotune(jobs, sh)
    ctx.batch_render(jobs, sh)  # capture with the tuned shape
    stream.synchronize()
    dist.barrier()
    ms = min(timed(torch, stream, flush, lambda: ctx.batch_render(jobs, sh)) for _ in range(2))
    st = ctx.stats()
    ms_all = dist.max(ms)
    steps_all = dist.sum(float(st.sample_steps))
    jobs_all = int(dist.sum(float(len(jobs))))
    res = {
        "workload": f"C3 {len(vols)} volumes (dims 64..192 per axis), {len(specs)} views at 512^2, L 15..60, "
                    f"mixed box/triangle/cos2, f16",
        "jobs": jobs_all, "jobs_this_rank": len(jobs), "voxels_this_rank": voxels, "ms_per_batch": ms_all,
        "frames_per_s": jobs_all / (ms_all / 1e3), "gss": steps_all / (ms_all / 1e3) / 1e9,
        "sample_steps": int(steps_all), "sharding": f"shard_by_cost over {dist.world} rank(s)",
        "autotune": {"tile": f"{tw}x{32 // tw}", "sampler": [k for k, v in capi.SAMPLER.items() if v == smp][0],
                     "best_ms": tune_ms},
        "cuda_graph": True, "generation_s": gen_s,
    }
    # the plain FP32 form: the same jobs from FP32 texels with the gather sampler, one launch
    with capi.Context(torch.cuda.current_device()) as pctx:
        pctx.upload_noise(noise)
        pctx.set_tf(*wl.default_tf())
        pjobs, _ = make_jobs(pctx, "f32", "gather", outs)
        pctx.batch_render(pjobs, sh)
        stream.synchronize()
        plain_ms = timed(torch, stream, flush, lambda: pctx.batch_render(pjobs, sh))
    res["plain_f32_gather_ms"] = dist.max(plain_ms)
    res["speedup_vs_plain_f32"] = res["plain_f32_gather_ms"] / ms_all
    return res


def bench_orbit_adjoint(ctx, torch, stream, flush, w, vid, out, frame):
    """Forward (recording) + adjoint of one lit orbit frame: L2 loss to the same frame rendered
    with another transfer function; gradients for the TF, opacity and 121 taps."""
    from vectorvisualization_gb300 import capi, workloads as wl

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
    p.record_tape = 0
    ctx.set_params(p)
    fwd_ms = timed(torch, stream, flush, lambda: ctx.render_device(vid, out.data_ptr(), W, H, None, sh))
    steps = ctx.stats().sample_steps
    p.record_tape = 1
    ctx.set_params(p)
    rec_ms = timed(torch, stream, flush, lambda: ctx.render_device(vid, out.data_ptr(), W, H, None, sh))
    with torch.cuda.stream(stream):
        torch.mul(out - target, 2.0, out=g)
    adj_ms = timed(torch, stream, flush, lambda: ctx.render_adjoint(
        vid, g.data_ptr(), W, H, d_tf.data_ptr(), d_op.data_ptr(), d_taps.data_ptr(), sh))
    flags = ctx.stats().check_flags
    p.record_tape = 0
    ctx.set_params(p)
    return {"frame": frame, "fwd_ms": fwd_ms, "fwd_recording_ms": rec_ms, "adjoint_ms": adj_ms,
            "fwd_plus_adjoint_over_fwd": (rec_ms + adj_ms) / fwd_ms,
            "gss_fwd": steps / (fwd_ms / 1e3) / 1e9, "gss_fwd_adjoint": steps / ((rec_ms + adj_ms) / 1e3) / 1e9,
            "tape_overflow": bool(flags & capi.CHECK_TAPE_OVERFLOW),
            "finite": bool(torch.isfinite(d_tf).all() and torch.isfinite(d_taps).all()),
            "grad_norms": {"tf": float(d_tf.norm()), "opacity": float(d_op.norm()), "taps": float(d_taps.norm())}}


def bench_rows(ctx, torch, stream, flush, w, vid, ceiling, frame, args):
    """The techniques and preprocessing beside the ray-cast, on the orbit's field, noise and
    parameters (512^3, RK4 L = 60 each way, 2048^2, orbit frame `frame`), each timed with CUDA
    events after a warm-up and an L2 flush, against the bound that applies:
      licvolume_precompute  vvlic_compute_lic_volume at 512^3 voxels (the reference's size): one
                            LIC per voxel, the ray-cast's fetch groups -> L1TEX fetch ceiling;
      licvolume_dvr         the LIC-volume ray-cast: one trilinear field fetch + one 8-load
                            gather of the LIC volume per sample -> texture fetch rate;
      vector_dvr            the vector-field DVR: one trilinear field fetch per sample;
      slicing               LIC on view-aligned slices -> L1TEX fetch ceiling;
      field_update_device   vvlic_update_field_device of the float32 field (encode + texture
                            copy) -> HBM;
      noise_gradients       vvlic_noise_gradients_device of the 512^3 noise -> HBM."""
    from vectorvisualization_gb300 import capi

    W, H = w.width, w.height
    sh = stream.cuda_stream
    p = capi.Params.from_buffer_copy(w.params)
    peak_hbm, hbm_kind = load_peaks()
    tex_peak = ceiling["tex_per_s"] / 1e9 if ceiling else None
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    ctx.set_view(w.views[frame])
    res = {"frame": frame}

    def settle():
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()

    # LIC-volume precompute (synchronous on the context's stream; its stats carry the kernel time)
    n = args.size
    ctx.set_params(p)
    ctx.compute_lic_volume(vid, (n, n, n))
    settle()
    ctx.compute_lic_volume(vid, (n, n, n))
    st = ctx.stats()
    res["licvolume_precompute"] = {
        "voxels": int(st.samples), "kernel_ms": st.kernel_ms,
        "gss": st.sample_steps / (st.kernel_ms / 1e3) / 1e9,
        "roofline": roofline(st.sample_steps, st.samples, st.kernel_ms, p.integrator, w.storage, False, 0, ceiling,
                             "")}

    def dvr(technique):
        q = capi.Params.from_buffer_copy(p)
        q.technique = capi.TECHNIQUE[technique]
        ctx.set_params(q)
        frame_fn = lambda: ctx.render_device(vid, out.data_ptr(), W, H, None, sh)  # noqa: E731
        timed(torch, stream, flush, frame_fn)
        ms = min(timed(torch, stream, flush, frame_fn) for _ in range(3))
        return ms, ctx.stats()

    for key, technique in (("licvolume_dvr", "licvolume"), ("vector_dvr", "volume")):
        ms, st = dvr(technique)
        rate = st.samples / (ms / 1e3) / 1e9
        res[key] = {"ms": ms, "samples": int(st.samples), "gsamples_per_s": rate,
                    "roofline": {"bound": "l1tex", "unit": "G samples/s", "achieved": rate, "peak": tex_peak,
                                 "frac": rate / tex_peak if tex_peak else None,
                                 "peak_kind": "measured trilinear fetch rate (vvlic_measure_fetch_ceiling)",
                                 "note": "one trilinear field fetch per sample through the texture unit"
                                         + (" plus an 8-load gather of the FP32 LIC volume"
                                            if technique == "licvolume" else "")}}
    ms, st = dvr("slicing")
    res["slicing"] = {"ms": ms, "samples": int(st.samples), "gss": st.sample_steps / (ms / 1e3) / 1e9,
                      "roofline": roofline(st.sample_steps, st.samples, ms, p.integrator, w.storage, True, W * H,
                                           ceiling, "")}
    ctx.set_params(p)

    # field update from device memory: the same field, so the volume is unchanged afterwards
    d_xyz = torch.from_numpy(np.ascontiguousarray(w.field)).cuda()
    nz, ny, nx = w.field.shape[:3]
    upd = lambda: ctx.update_field_device(vid, d_xyz.data_ptr(), (nx, ny, nz), sh)  # noqa: E731
    timed(torch, stream, flush, upd)
    ms = min(timed(torch, stream, flush, upd) for _ in range(3))
    vox = nx * ny * nz
    vbytes = ctx.volume_bytes(vid)
    texels = vox * bytes_per_texel(w.storage)
    # two passes over the float32 field, every layout of the volume written once, the texels read
    # once more to build the derived layouts
    alg = vox * 24 + vbytes + (texels if vbytes > texels else 0)
    res["field_update_device"] = {
        "ms": ms, "voxels": vox, "volume_bytes": vbytes,
        "roofline": {"bound": "hbm", "unit": "GB/s", "achieved": alg / (ms / 1e3) / 1e9, "peak": peak_hbm,
                     "frac": alg / (ms / 1e3) / 1e9 / peak_hbm, "peak_kind": hbm_kind, "traffic": None,
                     "algorithmic_bytes": alg,
                     "bytes": "24 B per voxel read (the length pass and the encode pass over float32 xyz) + "
                              "the volume's layouts written (texels, texture copy, cells if any) + the "
                              "texels read once to build the derived layouts"}}
    del d_xyz

    # noise gradients: 4 calls per timed region, the first untimed, so that the stream-ordered
    # scratch of calls 2-4 comes from the pool's free list
    mz, my, mx = w.noise.shape
    d_noise = torch.from_numpy(np.ascontiguousarray(w.noise)).cuda()
    d_rgba = torch.empty(mx * my * mz * 4, dtype=torch.uint8, device="cuda")
    ng = lambda: capi.noise_gradients_device(d_noise.data_ptr(), (mx, my, mz), w.noise_mode,  # noqa: E731
                                             d_rgba.data_ptr(), None, sh)
    best = 1e30
    for _ in range(3):
        with torch.cuda.stream(stream):
            flush.zero_()
            ng()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(3):
                ng()
            e1.record(stream)
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 3)
    nvox = mx * my * mz
    alg = nvox * 30  # raw pass: 1 B read, 12 B written; filter pass: 12 B + 1 B read, 4 B written
    res["noise_gradients"] = {
        "ms": best, "voxels": nvox,
        "roofline": {"bound": "hbm", "unit": "GB/s", "achieved": alg / (best / 1e3) / 1e9, "peak": peak_hbm,
                     "frac": alg / (best / 1e3) / 1e9 / peak_hbm, "peak_kind": hbm_kind, "traffic": None,
                     "algorithmic_bytes": alg,
                     "bytes": "30 B per voxel: the raw-gradient pass reads the noise byte (its 27-voxel "
                              "stencil from L1) and writes 12 B; the filter pass reads 12 B (27-voxel "
                              "stencil from L1) and the noise byte and writes 4 B RGBA"}}
    del d_noise, d_rgba
    return res


def run_ours(args, dist):
    import torch

    from vectorvisualization_gb300 import build, capi

    build.build()
    dev = dist.local
    torch.cuda.set_device(dev)
    ceiling = None if args.no_ceiling else capi.measure_fetch_ceiling(dev, 1)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    line = headline(args, dist, torch, stream, flush, ceiling) if args.only in ("all", "c5") else {}
    if args.only in ("all", "c2") and dist.rank == 0:
        with capi.Context(dev) as c2ctx:
            line["c2"] = bench_c2(c2ctx, torch, stream, flush, args, ceiling)
    if args.only in ("all", "c4") and not args.no_c4 and dist.rank == 0:
        with capi.Context(dev) as actx:
            line["fwd_adjoint"] = bench_c4(actx, torch, stream, flush, args)
    if args.only in ("all", "brick") and dist.rank == 0:
        with capi.Context(dev) as bctx:
            line["brick_ab"] = bench_brick(bctx, torch, stream, flush, args)
    if args.only in ("all", "c3") and not args.no_c3:
        with capi.Context(dev) as bctx:
            batch = bench_batch(bctx, torch, stream, flush, args, dist)
        if dist.rank == 0:
            line["batch"] = batch
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def headline(args, dist, torch, stream, flush, ceiling) -> dict:
    """The orbit frames: device-timed steps, e2e steps, the orbit's adjoint, the CPU baseline."""
    from vectorvisualization_gb300 import capi, workloads as wl

    dev = dist.local

    t0 = time.perf_counter()
    w = wl.c5(size=args.size, image=args.image, frames=ORBIT_FRAMES, device="cuda")
    gen_s = time.perf_counter() - t0
    ctx = capi.Context(dev)
    t0 = time.perf_counter()
    vid = wl.setup_context(ctx, w)
    p = w.params
    p.sampler = capi.SAMPLER[args.sampler]
    p.schedule = capi.SCHEDULE[schedule(args, "orbit")]
    ctx.set_params(p)
    setup_s = time.perf_counter() - t0
    sh = stream.cuda_stream
    W, H = w.width, w.height
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    frames = orbit_frames(args.steps, dist.world, dist.rank)

    def frame(f):
        ctx.set_view(w.views[f])
        ctx.render_device(vid, out.data_ptr(), W, H, None, sh)

    for i in range(args.warmup):
        timed(torch, stream, flush, lambda: frame(frames[i % len(frames)]))

    # timed region: K frames, each bracketed by events on the render stream, L2 flushed between
    clocks = Clocks(dev)
    starts = [torch.cuda.Event(enable_timing=True) for _ in frames]
    ends = [torch.cuda.Event(enable_timing=True) for _ in frames]
    steps_f, samples_f = [], []
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall0 = time.perf_counter()
    for k, f in enumerate(frames):
        ctx.set_view(w.views[f])
        with torch.cuda.stream(stream):
            flush.zero_()
            starts[k].record(stream)
            ctx.render_device(vid, out.data_ptr(), W, H, None, sh)
            ends[k].record(stream)
        st = ctx.stats()  # waits for this frame; counts of its samples
        steps_f.append(int(st.sample_steps))
        samples_f.append(int(st.samples))
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    dist.barrier()
    clk = clocks.stop()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    kernel_ms = sum(times)
    max_ms = dist.max(kernel_ms)
    total_steps = dist.sum(float(sum(steps_f)))
    total_samples = dist.sum(float(sum(samples_f)))
    value = total_steps / (max_ms / 1e3) / 1e9
    ms_per_step = max_ms / args.steps
    roof = roofline(sum(steps_f), sum(samples_f), kernel_ms, p.integrator, w.storage, True, W * H * len(frames),
                    ceiling, f"c5/{w.storage}/{args.sampler}/{args.size}/{args.image}")
    # per launch figures (the roofline's traffic is per launch)
    roof["per_launch"] = {kk: v / len(frames) for kk, v in roof["per_launch"].items()}
    if roof["traffic"] is not None:
        roof["hbm"]["dram_gbs"] = roof["traffic"] / (kernel_ms / len(frames) / 1e3) / 1e9
        roof["hbm"]["dram_frac"] = roof["hbm"]["dram_gbs"] / roof["hbm"]["peak_gbs"]
    roof["hbm"]["cacheless_model_bytes_per_launch"] /= len(frames)
    if ceiling:
        roof["ceiling"] = {"tex_per_s": ceiling["tex_per_s"], "ld256_per_s": ceiling["ld256_per_s"],
                           "group_per_s": ceiling["group_per_s"], "spread_texels": ceiling["spread_texels"]}

    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "frames_per_s": len(frames) * dist.world / (max_ms / 1e3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 spectral field and noise; the reference ships no datasets)",
        "config": {**w.describe(), "sampler": args.sampler, "schedule": schedule(args, "orbit"), "frames": frames,
                   "l2": "inputs > L2 (1 GiB field texture, 4.3 GB noise cells); L2 also flushed between frames "
                         "(256 MiB write)",
                   "sample_steps_per_frame": sum(steps_f) / len(frames),
                   "samples_per_frame": sum(samples_f) / len(frames),
                   "parallelism": f"replicas x{dist.world}", "generation_s": gen_s, "setup_s": setup_s},
        "wall_ms_per_step": t_wall / args.steps * 1e3,
        "image_alpha_mean": float(out[..., 3].mean()),
        "roofline": roof,
        # per frame: the ray-cast (+ the queue schedule's tile order: cost, bucket scan, scatter)
        "gpu_launches": args.steps * (4 if schedule(args, "orbit") == "queue" else 1),
        "clocks": clk,
    }
    del total_samples

    # end to end through the C ABI with host buffers.  Every step copies the field and the noise
    # from pinned host memory, re-encodes the field, recomputes the noise gradients and layouts,
    # renders and downloads the image.  `e2e` runs the steps as the stream-ordered animation
    # step (vvlic_update_field_async, vvlic_upload_noise_async, vvlic_render_to_host_async on
    # one stream, one wait at the end), so each step's host copies overlap the previous render;
    # `e2e_synchronous` runs the first steps with the synchronous calls for comparison.
    if not args.no_e2e:
        field_h = torch.from_numpy(np.ascontiguousarray(w.field)).pin_memory()
        noise_h = torch.from_numpy(np.ascontiguousarray(w.noise)).pin_memory()
        img_h = torch.empty((H, W, 4), dtype=torch.float32).pin_memory()
        nz, ny, nx = w.field.shape[:3]
        mz, my, mx = w.noise.shape
        lib = capi.load()

        def step_async(f):
            ctx.update_field_async(vid, field_h.data_ptr(), (nx, ny, nz), sh)
            ctx.upload_noise_async(noise_h.data_ptr(), (mx, my, mz), w.noise_mode, sh)
            ctx.set_view(w.views[f])
            ctx.render_to_host_async(vid, img_h.data_ptr(), W, H, sh)

        step_async(frames[0])
        stream.synchronize()
        dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for f in frames:
            step_async(f)
        ctx._check(lib.vvlic_synchronize(ctx.h, sh, 600000), "synchronize")
        torch.cuda.synchronize()
        t = dist.max(time.perf_counter() - t0)
        last = ctx.stats()
        line["e2e"] = {"value": total_steps / t / 1e9, "unit": UNIT,
                       "h2d_bytes_per_step": int(field_h.numel() * 4 + noise_h.numel()),
                       "d2h_bytes_per_step": int(img_h.numel() * 4),
                       "ms_per_step": t / args.steps * 1e3,
                       "same_sample_steps_as_device_timed": int(last.sample_steps) == steps_f[-1],
                       "includes": "per step: field copy from pinned host memory + in-place encode, noise copy + "
                                   "gradients, cell and texture layout rebuilds, view, render, image copy to pinned "
                                   "host memory; stream-ordered calls, the next step's copies overlapping the "
                                   "render; the same frames as the device-timed steps"}
        # the same steps with the synchronous calls (each returns when its work is done)
        ns = min(len(frames), 4)
        t0 = time.perf_counter()
        steps_sync = 0
        for f in frames[:ns]:
            ctx._check(lib.vvlic_update_field(ctx.h, vid, field_h.data_ptr(), capi.DTYPE_FLOAT32, nx, ny, nz),
                       "update_field")
            ctx._check(lib.vvlic_upload_noise(ctx.h, noise_h.data_ptr(), mx, my, mz, w.noise_mode), "upload_noise")
            ctx.set_view(w.views[f])
            ctx._check(lib.vvlic_render(ctx.h, vid, img_h.data_ptr(), W, H), "render")
            steps_sync += ctx.stats().sample_steps
        t = time.perf_counter() - t0
        line["e2e_synchronous"] = {"value": steps_sync / t / 1e9, "unit": UNIT, "steps": ns,
                                   "ms_per_step": t / ns * 1e3}

    if not args.no_adjoint and dist.rank == 0:
        line["orbit_adjoint"] = bench_orbit_adjoint(ctx, torch, stream, flush, w, vid, out, frames[0])

    if not args.no_rows and dist.rank == 0:
        line["rows"] = bench_rows(ctx, torch, stream, flush, w, vid, ceiling, frames[0], args)

    # CPU baseline (rank 0, N=1 only): the FP32 OpenMP restatement on a bounded row sample of
    # the last timed frame, compared with the GPU's rows of that frame
    if not args.no_cpu and dist.rank == 0 and dist.world == 1:
        ctx.set_view(w.views[frames[-1]])
        ctx.render_device(vid, out.data_ptr(), W, H, None, sh)
        stream.synchronize()
        gpu_img = out.cpu().numpy()
        t0 = time.perf_counter()
        sc = cpu_scene(w)
        prep_s = time.perf_counter() - t0
        res = cpu_sample(sc, w, w.views[frames[-1]], args.cpu_seconds)
        gpu_rows = gpu_img[res["rows"]]
        line["cpu_baseline"] = {
            "value": res["rate"], "unit": UNIT, "cores": res["threads"], "kind": "port",
            "sample": f"{len(res['rows'])} stratified rows of orbit frame {frames[-1]} ({W}x{H}; "
                      f"{res['seconds']:.1f} s; FP32 OpenMP restatement of the reference GLSL path)",
            "rmse_gpu_vs_cpu_rows": float(np.sqrt(np.mean((gpu_rows.astype(np.float64) - res["img"]) ** 2))),
            "input_build_s": prep_s,
        }
        del sc
    ctx.free_volume(vid)
    ctx.close()
    return line


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
