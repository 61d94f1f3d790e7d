// BRICK sampler: field and noise texels staged per CTA into shared memory by TMA.
//
// A CTA owns a 16x8 pixel tile and marches its 128 rays together in segments of `seg`
// samples.  Before each segment one thread works out the texel box that the segment's ray
// samples and their streamlines can reach — the samples of a ray lie on a line, and a
// streamline moves at most h_eff per step along each texture axis (the encoded direction
// components are in [-1, 1], inc_lic.glsl:114-125), so L * h_eff bounds the reach — and loads
// that box of the field (x-fastest RGBA texels) and of the noise with one
// cp.async.bulk.tensor.3d each, completing on an mbarrier.  Every trilinear fetch whose eight
// texels lie in the brick reads shared memory; any other fetch (a box larger than the brick,
// the noise's REPEAT wrap) reads global memory.  Both paths run the GATHER sampler's
// arithmetic, so BRICK images equal GATHER images up to the compiler's choice of FMA
// contractions in the two kernels.
//
// The tensor maps cover this GPU's own memory only and use no cluster multicast.  Every wait on
// the mbarrier is bounded: a wait that runs out records VVLIC_CHECK_BRICK in the render's
// stats and the CTA waits (bounded again) for its copy before it returns.
#pragma once

#include <cuda.h>

#include "vvlic_device.cuh"

namespace vvlic {

constexpr int kBrickTileW = 16, kBrickTileH = 8, kBrickThreads = 128;

// Launch constants of a BRICK render: the two tensor maps and the brick shapes.
struct BrickArgs {
  CUtensorMap fmap;   // field texels as 32-bit words: dims (n0 * tw, n1, n2), box (fb0 * tw, fb1, fb2)
  CUtensorMap nmap;   // noise bytes: dims (m0 * ch, m1, m2), box (nb0 * ch, nb1, nb2)
  int fb[3];          // field brick extent (texels)
  int nb[3];          // noise brick extent (texels)
  int tw;             // 32-bit words per field texel
  int falign, nalign; // x origin alignment (texels) of the field and noise boxes
  int seg;            // ray samples per segment
  float fr[3];        // streamline reach (field texels) per axis, trilinear neighbour included
  float nr[3];        // streamline reach (noise texels) per axis
  unsigned fbytes, nbytes;  // bytes of one field / noise brick (the TMA transaction size)
};

// Per-CTA state at the start of dynamic shared memory (the bricks follow, 128-byte aligned).
struct BrickState {
  unsigned long long bar;  // mbarrier of the current segment's two copies
  int fo[3];               // field brick origin (texels)
  int no[3];               // noise brick origin (texels)
  int fb[3], nb[3];        // brick extents (copied from BrickArgs for the samplers)
  int noff;                // byte offset of the noise brick in dynamic shared memory
  int any;                 // some ray of the CTA is still marching
  int lo[4][6];            // per-warp lower box corners: field xyz, noise xyz (texels)
  int hi[4][6];            // per-warp upper box corners
};
// Dynamic shared memory: [BrickState][TF table: 5 x 256 floats][field brick][noise brick].
constexpr int kBrickStateBytes = 384;  // sizeof(BrickState) rounded up to a multiple of 128
static_assert(sizeof(BrickState) <= kBrickStateBytes, "brick state");
constexpr int kBrickTfOff = kBrickStateBytes;
constexpr int kBrickFieldOff = kBrickTfOff + 5 * VVLIC_TF_ENTRIES * 4;  // 5504
static_assert(kBrickFieldOff % 128 == 0, "TMA destinations must be 128-byte aligned");

extern __shared__ __align__(128) unsigned char vvlic_brick_smem[];

__device__ __forceinline__ BrickState& brick_state() { return *reinterpret_cast<BrickState*>(vvlic_brick_smem); }
__device__ __forceinline__ const unsigned char* brick_field_smem() { return vvlic_brick_smem + kBrickFieldOff; }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Texel decode from shared memory (the same values Texel<ST>::load reads from global memory).
template <int ST> struct TexelS;
template <> struct TexelS<VVLIC_STORAGE_F32> {
  static __device__ __forceinline__ float4 load(const unsigned char* b, int i) { return reinterpret_cast<const float4*>(b)[i]; }
};
template <> struct TexelS<VVLIC_STORAGE_F16> {
  static __device__ __forceinline__ float4 load(const unsigned char* b, int i) {
    return Texel<VVLIC_STORAGE_F16>::decode(reinterpret_cast<const uint2*>(b)[i]);
  }
};
template <> struct TexelS<VVLIC_STORAGE_BF16> {
  static __device__ __forceinline__ float4 load(const unsigned char* b, int i) {
    return Texel<VVLIC_STORAGE_BF16>::decode(reinterpret_cast<const uint2*>(b)[i]);
  }
};
template <> struct TexelS<VVLIC_STORAGE_UNORM8> {
  static __device__ __forceinline__ float4 load(const unsigned char* b, int i) {
    return unorm8x4(reinterpret_cast<const uint32_t*>(b)[i]);
  }
};

constexpr int kBrick = 4;  // layout id of the BRICK samplers (Field / Noise specialisations)

template <int ST> struct Field<ST, kBrick> {
  static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 s) {
    int x0, x1, y0, y1, z0, z1;
    float ax, ay, az;
    clamp_axis(s.x, a.n[0], x0, x1, ax);
    clamp_axis(s.y, a.n[1], y0, y1, ay);
    clamp_axis(s.z, a.n[2], z0, z1, az);
    const BrickState& st = brick_state();
    const int lx0 = x0 - st.fo[0], lx1 = x1 - st.fo[0], ly0 = y0 - st.fo[1], ly1 = y1 - st.fo[1];
    const int lz0 = z0 - st.fo[2], lz1 = z1 - st.fo[2];
    const int bx = st.fb[0], by = st.fb[1], bz = st.fb[2];
    if ((unsigned)lx0 < (unsigned)bx && (unsigned)lx1 < (unsigned)bx && (unsigned)ly0 < (unsigned)by &&
        (unsigned)ly1 < (unsigned)by && (unsigned)lz0 < (unsigned)bz && (unsigned)lz1 < (unsigned)bz) {
      const unsigned char* f = brick_field_smem();
      const int r00 = (lz0 * by + ly0) * bx, r10 = (lz0 * by + ly1) * bx, r01 = (lz1 * by + ly0) * bx,
                r11 = (lz1 * by + ly1) * bx;
      return trilerp(TexelS<ST>::load(f, r00 + lx0), TexelS<ST>::load(f, r00 + lx1), TexelS<ST>::load(f, r10 + lx0),
                     TexelS<ST>::load(f, r10 + lx1), TexelS<ST>::load(f, r01 + lx0), TexelS<ST>::load(f, r01 + lx1),
                     TexelS<ST>::load(f, r11 + lx0), TexelS<ST>::load(f, r11 + lx1), ax, ay, az);
    }
    return Field<ST, kGather>::sample(a, s);
  }
};

template <> struct Noise<kBrick> {
  template <bool RGBA, bool GRADC> static __device__ __forceinline__ float4 sample(const RenderArgs& a, float3 p) {
    const float3 s = noise_coord<GRADC>(a, p);
    int x0, x1, y0, y1, z0, z1;
    float ax, ay, az;
    repeat_axis(s.x, a.m[0], x0, x1, ax);
    repeat_axis(s.y, a.m[1], y0, y1, ay);
    repeat_axis(s.z, a.m[2], z0, z1, az);
    const BrickState& st = brick_state();
    const int lx0 = x0 - st.no[0], lx1 = x1 - st.no[0], ly0 = y0 - st.no[1], ly1 = y1 - st.no[1];
    const int lz0 = z0 - st.no[2], lz1 = z1 - st.no[2];
    const int bx = st.nb[0], by = st.nb[1], bz = st.nb[2];
    if (!((unsigned)lx0 < (unsigned)bx && (unsigned)lx1 < (unsigned)bx && (unsigned)ly0 < (unsigned)by &&
          (unsigned)ly1 < (unsigned)by && (unsigned)lz0 < (unsigned)bz && (unsigned)lz1 < (unsigned)bz))
      return Noise<kGather>::template sample<RGBA, GRADC>(a, p);
    const float k = 1.0f / 255.0f;
    const unsigned char* nb = vvlic_brick_smem + st.noff;  // the noise brick follows the field brick
    const int r00 = (lz0 * by + ly0) * bx, r10 = (lz0 * by + ly1) * bx, r01 = (lz1 * by + ly0) * bx,
              r11 = (lz1 * by + ly1) * bx;
    if (RGBA) {
      const uint32_t* t = reinterpret_cast<const uint32_t*>(nb);
      const uint32_t t000 = t[r00 + lx0], t100 = t[r00 + lx1], t010 = t[r10 + lx0], t110 = t[r10 + lx1],
                     t001 = t[r01 + lx0], t101 = t[r01 + lx1], t011 = t[r11 + lx0], t111 = t[r11 + lx1];
      float4 r;
      float* rp = &r.x;
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        float c00 = lerpf(bytef(t000, ch), bytef(t100, ch), ax), c10 = lerpf(bytef(t010, ch), bytef(t110, ch), ax);
        float c01 = lerpf(bytef(t001, ch), bytef(t101, ch), ax), c11 = lerpf(bytef(t011, ch), bytef(t111, ch), ax);
        rp[ch] = lerpf(lerpf(c00, c10, ay), lerpf(c01, c11, ay), az) * k;
      }
      return r;
    }
    float c00 = lerpf((float)nb[r00 + lx0], (float)nb[r00 + lx1], ax);
    float c10 = lerpf((float)nb[r10 + lx0], (float)nb[r10 + lx1], ax);
    float c01 = lerpf((float)nb[r01 + lx0], (float)nb[r01 + lx1], ax);
    float c11 = lerpf((float)nb[r11 + lx0], (float)nb[r11 + lx1], ax);
    return make_float4(0.f, 0.f, 0.f, lerpf(lerpf(c00, c10, ay), lerpf(c01, c11, ay), az) * k);
  }
};

}  // namespace vvlic
