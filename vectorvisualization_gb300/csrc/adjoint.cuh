// Adjoint of the LIC ray-cast (any shading model + front-to-back blend) with respect
// to the transfer-function table (256 RGBA), the opacity table (256) and the filter taps.
//
// The forward render records a tape: per sample (intensity I, TF coordinate), with gradient
// lighting also the LIC gradient sum G (4 halves), and every kSegment samples a checkpoint
// (position, dest before the sample).  Per ray this kernel walks the segments last to first: it
// recomputes the segment's compositing states from its checkpoint into a local array (cheap:
// no streamline work), then backpropagates sample by sample through clamp, blend, alpha
// correction, the opacity lookup, the shading (illumZoeckler / illumMallo factors recomputed
// from the field sample) and the TF lookup.  The cotangents of I and G are
// pushed onto the filter taps by walking the sample's streamlines once more
// (dL/dw_j = sum_k S dL/dI_k n_kj + dL/dG_k . g_kj).
//
// Reductions are deterministic: per-tap sums are formed by a fixed-order warp butterfly, and
// every contribution enters 64-bit fixed-point accumulators (scale 2^30) by integer atomics,
// which are associative — so the result does not depend on scheduling.
#pragma once

#include "render_fwd.cuh"

namespace vvlic {

// Minimum resident CTAs per SM requested for the adjoint kernels (register cap 65536 / (128 * n)):
// 6 (80 registers, a few spilled bytes) measured 1786 ms against 1951 ms for 5 (93 registers)
// on the lit 512^3 RK4 frame with one sample per pass and one warp butterfly per tap sum.
#ifndef VVLIC_ADJ_MIN_BLOCKS
#define VVLIC_ADJ_MIN_BLOCKS 6
#endif
// Samples whose streamlines one thread re-walks together in the RK4 adjoint: 1 or 2 (four
// independent gather chains, as the forward's trace_pixel2).  On frames 0 / 40 of the lit 512^3
// RK4 orbit (2048^2) the adjoint took 1309 / 1532 ms with two samples at 6 CTAs per SM (80
// registers, 100 spilled bytes), 1335 / 1550 ms at 5 (96 registers), 1353 / 1579 ms at 4 (127
// registers) and 1518 / 1762 ms with one sample at 6.  Two samples per pass measured slower for
// the Heun forward, so the other integrators keep one.
#ifndef VVLIC_ADJ_RK4_SAMPLES_PER_PASS
#define VVLIC_ADJ_RK4_SAMPLES_PER_PASS 2
#endif

template <int INTEG> __host__ __device__ constexpr int adj_samples_per_pass() {
  return INTEG == VVLIC_RK4 ? VVLIC_ADJ_RK4_SAMPLES_PER_PASS : 1;
}

constexpr float kFixedScale = 1073741824.0f;  // 2^30
constexpr int kAccTF = 0, kAccOpac = 4 * VVLIC_TF_ENTRIES, kAccTaps = 5 * VVLIC_TF_ENTRIES;
constexpr int kAccSize = kAccTaps + kMaxTaps;

__device__ __forceinline__ void fixed_add(long long* slot, float v) {
  if (v != 0.0f) atomicAdd(reinterpret_cast<unsigned long long*>(slot), (unsigned long long)__float2ll_rn(v * kFixedScale));
}

// Sum over the warp (fixed butterfly order); lane 0 adds it to the block accumulator.
__device__ __forceinline__ void warp_fixed_add(long long* slot, float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) fixed_add(slot, v);
}

// Two warp sums in five shuffles (fixed order): the first exchange leaves lanes 0-15 holding
// pair sums of `va` and lanes 16-31 pair sums of `vb`; each half then reduces on its own.  Lane 0
// adds the sum of `va` to slot_a (when use_a), lane 16 the sum of `vb` to slot_b (when use_b).
__device__ __forceinline__ void warp_fixed_add2(long long* slot_a, bool use_a, float va, long long* slot_b, bool use_b,
                                                float vb) {
  const int lane = threadIdx.x & 31;
  const bool lo = lane < 16;
  float x = (lo ? va : vb) + __shfl_xor_sync(0xffffffffu, lo ? vb : va, 16);
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((lane == 0 && use_a) || (lane == 16 && use_b)) fixed_add(lo ? slot_a : slot_b, x);
}

// 1D LINEAR + CLAMP_TO_EDGE lookup decomposed: entries i0, i1, weight t of i1, and whether the
// coordinate lies strictly inside the interpolation range (derivative in s = 256 there, else 0).
struct Lut {
  int i0, i1;
  float t;
  bool inside;
};
__device__ __forceinline__ Lut lut(float s) {
  Lut L;
  float u = fmaf(s, (float)VVLIC_TF_ENTRIES, -0.5f);
  L.inside = u >= 0.0f && u < (float)(VVLIC_TF_ENTRIES - 1);
  u = fminf(fmaxf(u, -1.0f), (float)VVLIC_TF_ENTRIES);
  const float fl = floorf(u);
  L.t = u - fl;
  const int b = (int)fl;
  L.i0 = min(max(b, 0), VVLIC_TF_ENTRIES - 1);
  L.i1 = min(max(b + 1, 0), VVLIC_TF_ENTRIES - 1);
  return L;
}

// Unlit source of one sample from its tape record (illumLIC, inc_illum.glsl:158-172).
struct Src {
  Lut lt, lo;
  float4 tf;
  float op, base, alpha;
  float3 col;
};
__device__ __forceinline__ Src unlit_source(const RenderArgs& a, const float* s_tf, float I, float tfc) {
  Src r;
  r.lt = lut(tfc);
  const float4 t0 = reinterpret_cast<const float4*>(s_tf)[r.lt.i0], t1 = reinterpret_cast<const float4*>(s_tf)[r.lt.i1];
  r.tf = lerp4(t0, t1, r.lt.t);
  r.lo = lut(I * 1.3f);
  const float* op = s_tf + 4 * VVLIC_TF_ENTRIES;
  r.op = lerpf(op[r.lo.i0], op[r.lo.i1], r.lo.t);
  const float a0 = r.op * r.tf.w;
  r.base = 1.0f - a0;
  r.alpha = 1.0f - powf(fmaxf(r.base, 0.0f), a.alpha_corr);
  r.col = f3(I * r.tf.x * a.illum_scale, I * r.tf.y * a.illum_scale, I * r.tf.z * a.illum_scale);
  return r;
}
__device__ __forceinline__ float4 premultiplied(const Src& s) {
  return make_float4(s.col.x * s.alpha, s.col.y * s.alpha, s.col.z * s.alpha, s.alpha);
}
// The source as blend() takes it (colour not yet multiplied by alpha), matching shade().
__device__ __forceinline__ float4 unlit_source_rgba(const RenderArgs& a, const float* s_tf, float I, float tfc) {
  const Src s = unlit_source(a, s_tf, I, tfc);
  return make_float4(s.col.x, s.col.y, s.col.z, s.alpha);
}

// illumGradient (inc_illum.glsl:1-41) intermediates: N = n(-G), R = n(2 (L.N) N - L),
// df = sat(L.N) * illumScale, spf = sat(R.V)^e.
struct LitT {
  float3 L, V, N, Rv;
  float mlen, rlen, ln, rv, df, spf;
};
__device__ __forceinline__ LitT lit_setup(const RenderArgs& a, float3 G, float3 pos, float3 dir) {
  LitT t;
  t.L = light_dir(a, pos);
  t.V = norm3(scl3(dir, -1.0f));
  const float3 m = f3(-G.x, -G.y, -G.z);
  t.mlen = sqrtf(dot3(m, m));
  t.N = norm3(m);
  t.ln = dot3(t.L, t.N);
  const float3 r = sub3(scl3(t.N, 2.0f * t.ln), t.L);
  t.rlen = sqrtf(dot3(r, r));
  t.Rv = norm3(r);
  t.rv = dot3(t.Rv, t.V);
  t.spf = powf(__saturatef(t.rv), a.spec_exp);
  t.df = __saturatef(t.ln) * a.illum_scale;
  return t;
}
__device__ __forceinline__ float3 lit_color(const RenderArgs& a, const LitT& t, float4 tf, float I) {
  return f3((tf.x * I * (a.light_diff[0] * t.df + 0.3f + a.light_amb[0]) + a.light_spec[0] * t.spf * I) * a.illum_scale,
            (tf.y * I * (a.light_diff[1] * t.df + 0.3f + a.light_amb[1]) + a.light_spec[1] * t.spf * I) * a.illum_scale,
            (tf.z * I * (a.light_diff[2] * t.df + 0.3f + a.light_amb[2]) + a.light_spec[2] * t.spf * I) * a.illum_scale);
}
// Reverse mode of lit_color for a colour cotangent dcol: dL/dtf.rgb, dL/dI, dL/dG.  sat() has
// derivative 1 strictly inside (0, 1).
__device__ __forceinline__ void lit_vjp(const RenderArgs& a, const LitT& t, float4 tf, float I, float3 dcol,
                                        float dtf[3], float* dI, float3* dG) {
  const float is = a.illum_scale;
  const float d[3] = {dcol.x, dcol.y, dcol.z}, tfc[3] = {tf.x, tf.y, tf.z};
  float cdf = 0.0f, cspf = 0.0f, di = 0.0f;
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    const float k = a.light_diff[ch] * t.df + 0.3f + a.light_amb[ch];
    dtf[ch] = d[ch] * I * k * is;
    di += d[ch] * (tfc[ch] * k + a.light_spec[ch] * t.spf) * is;
    cdf += d[ch] * tfc[ch] * I * a.light_diff[ch] * is;
    cspf += d[ch] * a.light_spec[ch] * I * is;
  }
  *dI = di;
  float3 gN = f3(0.f, 0.f, 0.f);
  if (t.ln > 0.0f && t.ln < 1.0f) gN = scl3(t.L, cdf * is);
  if (t.rv > 0.0f && t.rv < 1.0f && t.rlen > 0.0f && cspf != 0.0f) {
    const float dspf = cspf * a.spec_exp * powf(t.rv, a.spec_exp - 1.0f);
    const float3 gR = scl3(t.V, dspf);
    const float3 gr = scl3(sub3(gR, scl3(t.Rv, dot3(t.Rv, gR))), 1.0f / t.rlen);
    gN = add3(gN, add3(scl3(t.L, 2.0f * dot3(t.N, gr)), scl3(gr, 2.0f * t.ln)));
  }
  *dG = t.mlen > 0.0f ? scl3(sub3(gN, scl3(t.N, dot3(t.N, gN))), -1.0f / t.mlen) : f3(0.f, 0.f, 0.f);
}
__device__ __forceinline__ float3 tape_gradient(const RenderArgs& a, size_t idx) {
  const uint2 v = a.tape_g[idx];
  const float2 xy = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
  const float2 z0 = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
  return f3(xy.x, xy.y, z0.x);
}

// Walk the streamlines of the LIC at `pos` once more and add gI * n_j (+ gG . g_j with noise
// gradients) to the tap accumulators.  Every lane of the warp takes part in each reduction;
// lanes with zero cotangents skip the fetches.
template <int ST, int FL, int NL, int INTEG, bool GRAD>
__device__ __forceinline__ float tap_dot(float4 n, float gI, float3 gG) {
  return GRAD ? fmaf(gI, n.w, gG.x * n.x + gG.y * n.y + gG.z * n.z) : gI * n.w;
}
template <int ST, int FL, int NL, int INTEG, bool GRAD>
__device__ __forceinline__ void tap_gradients(const RenderArgs& a, float3 pos, float gI, float3 gG, long long* s_taps) {
  const bool act = gI != 0.0f || (GRAD && (gG.x != 0.0f || gG.y != 0.0f || gG.z != 0.0f));
  const int lb = a.lb, lf = a.lf, L = max(lb, lf);
  float4 f0 = make_float4(0.f, 0.f, 0.f, 0.f);
  float v0 = 0.0f;
  if (act) {
    f0 = Field<ST, FL>::sample(a, pos);
    v0 = tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, pos), gI, gG);
  }
  warp_fixed_add(s_taps + lb, v0);
  float3 pb = pos, pf = pos;
  float4 sb = f0, sf = f0;
  for (int i = 1; i <= L; ++i) {
    float vb = 0.0f, vf = 0.0f;
    if (act) {
      if (i <= lb) {
        pb = lic_step<ST, FL, INTEG>(a, pb, sb, -1.0f);
        vb = tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, pb), gI, gG);
      }
      if (i <= lf) {
        pf = lic_step<ST, FL, INTEG>(a, pf, sf, 1.0f);
        vf = tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, pf), gI, gG);
      }
    }
    warp_fixed_add2(s_taps + lb - i, i <= lb, vb, s_taps + lb + i, i <= lf, vf);
  }
}

// tap_gradients of two samples at once: four independent streamline chains per thread, and
// per tap the two samples' contributions are added in the lane before the warp sum.  A lane
// walks both samples' streamlines when either has a non-zero cotangent; the other sample's
// terms are then zero (its cotangents are zero and its noise values finite).
template <int ST, int FL, int NL, int INTEG, bool GRAD>
__device__ __forceinline__ void tap_gradients2(const RenderArgs& a, float3 pa, float gIa, float3 gGa, float3 pc,
                                               float gIc, float3 gGc, long long* s_taps) {
  const bool act = gIa != 0.0f || gIc != 0.0f ||
                   (GRAD && (gGa.x != 0.0f || gGa.y != 0.0f || gGa.z != 0.0f || gGc.x != 0.0f || gGc.y != 0.0f ||
                             gGc.z != 0.0f));
  const int lb = a.lb, lf = a.lf, L = max(lb, lf);
  float4 fa = make_float4(0.f, 0.f, 0.f, 0.f), fc = fa;
  float v0 = 0.0f;
  if (act) {
    fa = Field<ST, FL>::sample(a, pa);
    fc = Field<ST, FL>::sample(a, pc);
    v0 = tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, pa), gIa, gGa) +
         tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, pc), gIc, gGc);
  }
  warp_fixed_add(s_taps + lb, v0);
  float3 p0 = pa, p1 = pa, p2 = pc, p3 = pc;
  float4 s0 = fa, s1 = fa, s2 = fc, s3 = fc;
  const int both = min(lb, lf);
  int i = 1;
  for (; i <= both; ++i) {
    float vb = 0.0f, vf = 0.0f;
    if (act) {
      p0 = lic_step<ST, FL, INTEG>(a, p0, s0, -1.0f);
      p1 = lic_step<ST, FL, INTEG>(a, p1, s1, 1.0f);
      p2 = lic_step<ST, FL, INTEG>(a, p2, s2, -1.0f);
      p3 = lic_step<ST, FL, INTEG>(a, p3, s3, 1.0f);
      vb = tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, p0), gIa, gGa) +
           tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, p2), gIc, gGc);
      vf = tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, p1), gIa, gGa) +
           tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, p3), gIc, gGc);
    }
    warp_fixed_add2(s_taps + lb - i, true, vb, s_taps + lb + i, true, vf);
  }
  for (; i <= L; ++i) {
    float vb = 0.0f, vf = 0.0f;
    if (act) {
      if (i <= lb) {
        p0 = lic_step<ST, FL, INTEG>(a, p0, s0, -1.0f);
        p2 = lic_step<ST, FL, INTEG>(a, p2, s2, -1.0f);
        vb = tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, p0), gIa, gGa) +
             tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, p2), gIc, gGc);
      }
      if (i <= lf) {
        p1 = lic_step<ST, FL, INTEG>(a, p1, s1, 1.0f);
        p3 = lic_step<ST, FL, INTEG>(a, p3, s3, 1.0f);
        vf = tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, p1), gIa, gGa) +
             tap_dot<ST, FL, NL, INTEG, GRAD>(noise_tap<NL, GRAD>(a, p3), gIc, gGc);
      }
    }
    warp_fixed_add2(s_taps + lb - i, i <= lb, vb, s_taps + lb + i, i <= lf, vf);
  }
}

// Reverse step through one sample (kk of segment seg): clamp, blend, alpha correction, opacity
// and TF lookups and the shading, from the recomputed compositing state Dloc[kk].  Adds the TF
// and opacity cotangents to the block accumulators, updates the image cotangent g to the one
// before the sample and returns the cotangents of the sample's LIC intensity (gIraw, already
// scaled by the intensity scale) and gradient sum (gG), and its position.  Samples at or past
// cnt leave everything zero.
template <int ST, int FL, bool GRAD>
__device__ __forceinline__ void sample_cotangent(const RenderArgs& a, const float* s_tf, bool line, float3 dir,
                                                 const float4* Dloc, const float3* Ploc, int px, int py, int seg,
                                                 int kk, int cnt, float4& g, long long* s_acc, float& gIraw,
                                                 float3& gG, float3& pk) {
  gIraw = 0.0f;
  gG = f3(0.f, 0.f, 0.f);
  pk = f3(0.f, 0.f, 0.f);
  if (kk < 0 || kk >= cnt) return;
  const size_t idx = tape_entry_checked(a, px, py, seg * kSegment + kk);
  const float2 rec = a.tape_is[idx];
  const float I = rec.x;
  Src s = unlit_source(a, s_tf, I, rec.y);
  LitT lt;
  float3 ld = f3(0.f, 0.f, 0.f);
  if (GRAD) {
    lt = lit_setup(a, tape_gradient(a, idx), Ploc[kk], dir);
    s.col = lit_color(a, lt, s.tf, I);
  } else if (line) {  // colour = tf.rgb * I * d + s (d, s independent of TF, taps and I)
    float3 sf;
    line_factors(a, Ploc[kk], dir, Field<ST, FL>::sample(a, Ploc[kk]), ld, sf);
    s.col = f3(s.tf.x * I * ld.x + sf.x, s.tf.y * I * ld.y + sf.y, s.tf.z * I * ld.z + sf.z);
  }
  const float4 sv = premultiplied(s);
  const float4 Dp = Dloc[kk];
  pk = Ploc[kk];
  const float om = 1.0f - Dp.w;
  // clamp((1 - Dp.a) * s + Dp) per channel: derivative 1 on [0, 1]
  const float ux = fmaf(om, sv.x, Dp.x), uy = fmaf(om, sv.y, Dp.y), uz = fmaf(om, sv.z, Dp.z),
              uw = fmaf(om, sv.w, Dp.w);
  const float gx = (ux >= 0.f && ux <= 1.f) ? g.x : 0.f, gy = (uy >= 0.f && uy <= 1.f) ? g.y : 0.f,
              gz = (uz >= 0.f && uz <= 1.f) ? g.z : 0.f, gw = (uw >= 0.f && uw <= 1.f) ? g.w : 0.f;
  const float4 ds = make_float4(om * gx, om * gy, om * gz, om * gw);
  float4 gp = make_float4(gx, gy, gz, gw);
  gp.w -= gx * sv.x + gy * sv.y + gz * sv.z + gw * sv.w;
  // s = (col * alpha, alpha)
  const float dcx = ds.x * s.alpha, dcy = ds.y * s.alpha, dcz = ds.z * s.alpha;
  const float dalpha = ds.x * s.col.x + ds.y * s.col.y + ds.z * s.col.z + ds.w;
  const float dba = s.base > 0.0f ? a.alpha_corr * powf(s.base, a.alpha_corr - 1.0f) : 0.0f;
  const float da0 = dalpha * dba;
  // a0 = opacity(1.3 I) * tf.a
  const float dop = da0 * s.tf.w, dtfa = da0 * s.op;
  fixed_add(s_acc + kAccOpac + s.lo.i0, dop * (1.0f - s.lo.t));
  fixed_add(s_acc + kAccOpac + s.lo.i1, dop * s.lo.t);
  const float* op = s_tf + 4 * VVLIC_TF_ENTRIES;
  float dI = s.lo.inside ? dop * (op[s.lo.i1] - op[s.lo.i0]) * (float)VVLIC_TF_ENTRIES * 1.3f : 0.0f;
  float dtf[4];
  dtf[3] = dtfa;
  if (GRAD) {
    float dIc;
    lit_vjp(a, lt, s.tf, I, f3(dcx, dcy, dcz), dtf, &dIc, &gG);
    dI += dIc;
  } else if (line) {
    dtf[0] = dcx * I * ld.x;
    dtf[1] = dcy * I * ld.y;
    dtf[2] = dcz * I * ld.z;
    dI += dcx * s.tf.x * ld.x + dcy * s.tf.y * ld.y + dcz * s.tf.z * ld.z;
  } else {  // col = I * tf.rgb * illumScale
    const float ci = I * a.illum_scale;
    dtf[0] = dcx * ci;
    dtf[1] = dcy * ci;
    dtf[2] = dcz * ci;
    dI += (dcx * s.tf.x + dcy * s.tf.y + dcz * s.tf.z) * a.illum_scale;
  }
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    fixed_add(s_acc + kAccTF + 4 * s.lt.i0 + ch, dtf[ch] * (1.0f - s.lt.t));
    fixed_add(s_acc + kAccTF + 4 * s.lt.i1 + ch, dtf[ch] * s.lt.t);
  }
  gIraw = dI * a.intensity_scale;
  g = gp;
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
__global__ void __launch_bounds__(kThreads, VVLIC_ADJ_MIN_BLOCKS) adjoint_kernel(const __grid_constant__ RenderArgs a,
                                                           const float4* __restrict__ g_img, long long* acc,
                                                           const uint32_t* __restrict__ order, int ntiles,
                                                           unsigned* __restrict__ next) {
  __shared__ __align__(16) float s_tf[5 * VVLIC_TF_ENTRIES];
  __shared__ long long s_acc[kAccSize];
  for (int i = threadIdx.x; i < kAccSize; i += blockDim.x) s_acc[i] = 0;
  load_tf(a, s_tf);  // includes __syncthreads
  const int lane = threadIdx.x & 31;
  const int tiles_x = (a.W + kWarpTileW - 1) / kWarpTileW;
  const bool line = !GRAD && (a.illum == VVLIC_ILLUM_ZOECKLER || a.illum == VVLIC_ILLUM_MALLO);
  float4 Dloc[kSegment];
  float3 Ploc[kSegment];
  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(next, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= (unsigned)ntiles) break;
    const unsigned tile = __ldg(order + t);
    const int px = (int)(tile % tiles_x) * kWarpTileW + (lane & (kWarpTileW - 1));
    const int py = (int)(tile / tiles_x) * kWarpTileH + (lane / kWarpTileW);
    const bool in_image = px < a.W && py < a.H;
    const size_t ray = in_image ? (size_t)py * a.W + px : 0;
    float3 pos0 = f3(0.f, 0.f, 0.f), dir = f3(0.f, 0.f, 0.f);
    int S = 0;
    float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
    if (in_image && ray_setup(a, px, py, pos0, dir)) {
      S = (int)min(a.tape_n[ray], (uint32_t)a.tape_stride);
      g = g_img[ray];
    }
    const int nseg = (S + kSegment - 1) / kSegment;
    const int nseg_warp = __reduce_max_sync(0xffffffffu, (unsigned)nseg);
    for (int seg = nseg_warp - 1; seg >= 0; --seg) {
      const bool act_seg = seg < nseg;
      int cnt = 0;
      if (act_seg) {
        size_t ce = tape_ck_entry(a, px, py, seg);
        if (!in_range(a, (long long)ce + 32, tape_ck_entries(a), VVLIC_CHECK_TAPE)) ce = 0;
        const float4* ck = a.tape_ck + ce;
        const float4 p4 = ck[0];
        float3 p = f3(p4.x, p4.y, p4.z);
        float4 D = ck[32];
        cnt = min(kSegment, S - seg * kSegment);
        for (int kk = 0; kk < cnt; ++kk) {
          Ploc[kk] = p;
          Dloc[kk] = D;
          const size_t idx = tape_entry_checked(a, px, py, seg * kSegment + kk);
          const float2 rec = a.tape_is[idx];
          float4 src;
          if (GRAD) {
            const Src us = unlit_source(a, s_tf, rec.x, rec.y);
            const float3 col = lit_color(a, lit_setup(a, tape_gradient(a, idx), p, dir), us.tf, rec.x);
            src = make_float4(col.x, col.y, col.z, us.alpha);
          } else if (line) {
            const Src us = unlit_source(a, s_tf, rec.x, rec.y);
            float3 d, sf;
            line_factors(a, p, dir, Field<ST, FL>::sample(a, p), d, sf);
            src = make_float4(us.tf.x * rec.x * d.x + sf.x, us.tf.y * rec.x * d.y + sf.y, us.tf.z * rec.x * d.z + sf.z,
                              us.alpha);
          } else {
            src = unlit_source_rgba(a, s_tf, rec.x, rec.y);
          }
          D = blend(D, src);
          p = add3(p, scl3(dir, a.step_size));
        }
      }
      for (int kk = kSegment - 1; kk >= 0; kk -= adj_samples_per_pass<INTEG>()) {
        float gIraw;
        float3 gG, pk;
        sample_cotangent<ST, FL, GRAD>(a, s_tf, line, dir, Dloc, Ploc, px, py, seg, kk, cnt, g, s_acc, gIraw, gG, pk);
        bool need = gIraw != 0.0f || (GRAD && (gG.x != 0.0f || gG.y != 0.0f || gG.z != 0.0f));
        if constexpr (adj_samples_per_pass<INTEG>() == 2) {
          float gIraw1;
          float3 gG1, pk1;
          sample_cotangent<ST, FL, GRAD>(a, s_tf, line, dir, Dloc, Ploc, px, py, seg, kk - 1, cnt, g, s_acc, gIraw1,
                                         gG1, pk1);
          need = need || gIraw1 != 0.0f || (GRAD && (gG1.x != 0.0f || gG1.y != 0.0f || gG1.z != 0.0f));
          if (__any_sync(0xffffffffu, need))
            tap_gradients2<ST, FL, NL, INTEG, GRAD>(a, pk, gIraw, gG, pk1, gIraw1, gG1, s_acc + kAccTaps);
        } else {
          if (__any_sync(0xffffffffu, need)) tap_gradients<ST, FL, NL, INTEG, GRAD>(a, pk, gIraw, gG, s_acc + kAccTaps);
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kAccSize; i += blockDim.x)
    if (s_acc[i] != 0) atomicAdd(reinterpret_cast<unsigned long long*>(acc + i), (unsigned long long)s_acc[i]);
}

template <int ST, int FL, int NL, int INTEG, bool GRAD>
static cudaError_t launch_adjoint_one(const RenderArgs& a, const float4* g_img, long long* acc, const Schedule& sch,
                                      cudaStream_t s) {
  auto kern = adjoint_kernel<ST, FL, NL, INTEG, GRAD>;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, 0);
  if (e != cudaSuccess) return e;
  kern<<<std::max(1, per_sm) * sch.num_sms, kThreads, 0, s>>>(a, g_img, acc, sch.order, sch.ntiles, sch.next);
  return cudaGetLastError();
}

template <int ST, int FL, int NL, bool GRAD>
static cudaError_t launch_adjoint_integ(const RenderArgs& a, int integ, const float4* g_img, long long* acc,
                                        const Schedule& sch, cudaStream_t s) {
  if (integ == VVLIC_EULER) return launch_adjoint_one<ST, FL, NL, VVLIC_EULER, GRAD>(a, g_img, acc, sch, s);
  if (integ == VVLIC_HEUN) return launch_adjoint_one<ST, FL, NL, VVLIC_HEUN, GRAD>(a, g_img, acc, sch, s);
  return launch_adjoint_one<ST, FL, NL, VVLIC_RK4, GRAD>(a, g_img, acc, sch, s);
}

template <int ST, int FL, int NL>
static cudaError_t launch_adjoint_layout(const RenderArgs& a, int integ, bool lit, const float4* g_img,
                                         long long* acc, const Schedule& sch, cudaStream_t s) {
  return lit ? launch_adjoint_integ<ST, FL, NL, true>(a, integ, g_img, acc, sch, s)
             : launch_adjoint_integ<ST, FL, NL, false>(a, integ, g_img, acc, sch, s);
}

template <int ST>
static cudaError_t launch_adjoint_storage(const RenderArgs& a, int sampler, int integ, bool lit, const float4* g_img,
                                          long long* acc, const Schedule& sch, cudaStream_t s) {
  switch (sampler) {
    case VVLIC_SAMPLER_GATHER: return launch_adjoint_layout<ST, kGather, kGather>(a, integ, lit, g_img, acc, sch, s);
    case VVLIC_SAMPLER_CELL: return launch_adjoint_layout<ST, kCell, kCell>(a, integ, lit, g_img, acc, sch, s);
    case VVLIC_SAMPLER_TEXTURE:
      if constexpr (ST == VVLIC_STORAGE_BF16) return cudaErrorNotSupported;  // runs as F16 (kernel_storage)
      else return launch_adjoint_layout<ST, kTexture, kTexture>(a, integ, lit, g_img, acc, sch, s);
    case VVLIC_SAMPLER_HYBRID:
      if constexpr (ST == VVLIC_STORAGE_BF16) return cudaErrorNotSupported;
      else return launch_adjoint_layout<ST, kTexture, kCellFast>(a, integ, lit, g_img, acc, sch, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vvlic
