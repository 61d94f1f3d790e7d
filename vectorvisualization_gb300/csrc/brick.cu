// BRICK sampler: the ray-cast with field and noise bricks staged in shared memory by TMA (see
// brick.cuh), its tensor maps and its launch.  One CTA per 16x8 pixel tile; rays march in
// segments of BrickArgs::seg samples; before each segment thread 0 places the two bricks over
// the texel box the segment can reach and loads them with cp.async.bulk.tensor.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/vvlic.h"
#include "brick.cuh"
#include "render_fwd.cuh"
#include "vvlic_host.hpp"
#include "vvlic_launch.hpp"

namespace vvlic {
namespace {

constexpr int kTfOff = kBrickTfOff;
constexpr int kFieldOff = kBrickFieldOff;
constexpr unsigned kWaitPolls = 1u << 22;  // mbarrier polls before a wait gives up

__host__ __device__ constexpr unsigned round128(unsigned b) { return (b + 127u) & ~127u; }

__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned phase) {
  for (unsigned i = 0; i < kWaitPolls; ++i)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}
// One 3D tile of `map` at element coordinates (x, y, z) into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_3d(const void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Brick origin along one axis: the box [lo, hi] of needed texels (hi < lo: nothing needed),
// an extent `cap`, the axis length n and the origin alignment.  A box that fits lies inside the
// brick; a larger one gets the brick centred on it.  Origins stay in [0, n - cap] when n >= cap
// and are rounded down to the alignment (the extents carry that much slack).
__device__ __forceinline__ int place(int lo, int hi, int cap, int n, int align) {
  if (hi < lo) return 0;
  lo = max(lo, 0);
  hi = min(hi, n - 1);
  int o = (hi - lo + 1 <= cap - (align - 1)) ? lo : (lo + hi + 1) / 2 - cap / 2;
  o = min(o, n - cap);
  o = max(o, 0);
  return o - o % align;
}

// Texel box (lo, hi) along one axis of the positions between a and b, dilated by `reach`, for a
// texture axis of `scale` texels per unit (u = p * scale - 1/2).
__device__ __forceinline__ void axis_box(float a, float b, float scale, float reach, int& lo, int& hi) {
  const float u0 = fminf(a, b) * scale - 0.5f, u1 = fmaxf(a, b) * scale - 0.5f;
  lo = (int)floorf(fmaxf(u0 - reach, -1.0e6f));
  hi = (int)floorf(fminf(u1 + reach, 1.0e6f)) + 1;
}

template <int ST, int INTEG, bool GRAD>
__global__ void __launch_bounds__(kBrickThreads) brick_kernel(const __grid_constant__ RenderArgs a,
                                                              const __grid_constant__ BrickArgs b) {
  BrickState& st = brick_state();
  float* s_tf = reinterpret_cast<float*>(vvlic_brick_smem + kTfOff);
  unsigned char* fbrick = vvlic_brick_smem + kFieldOff;
  unsigned char* nbrick = vvlic_brick_smem + kFieldOff + round128(b.fbytes);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < 5 * VVLIC_TF_ENTRIES; i += kBrickThreads) s_tf[i] = __ldg(a.tf + i);
  // TMA writes need 128-byte aligned destinations; a launch without them runs every fetch from
  // global memory (empty bricks) and reports VVLIC_CHECK_BRICK
  const bool use_tma = ((smem_u32(fbrick) | smem_u32(nbrick)) & 127u) == 0;
  if (tid == 0) {
    for (int i = 0; i < 3; ++i) {
      st.fb[i] = use_tma ? b.fb[i] : 0;
      st.nb[i] = use_tma ? b.nb[i] : 0;
    }
    st.noff = kFieldOff + (int)round128(b.fbytes);
    mbar_init(&st.bar);
    if (!use_tma) atomicOr(a.counters + 3, (unsigned long long)VVLIC_CHECK_BRICK);
  }
  __syncthreads();

  const int px = blockIdx.x * kBrickTileW + (tid % kBrickTileW), py = blockIdx.y * kBrickTileH + (tid / kBrickTileW);
  float3 pos = f3(0.f, 0.f, 0.f), dir = f3(0.f, 0.f, 0.f);
  bool alive = px < a.W && py < a.H && ray_setup(a, px, py, pos, dir);
  const uint32_t hit = alive ? 1u : 0u;
  const float3 dstep = scl3(dir, a.step_size);
  const uint32_t max_samples = (uint32_t)a.num_iter * (uint32_t)a.num_iter;
  if (max_samples == 0) alive = false;
  float4 dest = make_float4(0.f, 0.f, 0.f, 0.f);
  uint32_t samples = 0, phase = 0;
  const float* nsc = GRAD ? a.nscale_grad : a.nscale;
  for (;;) {
    // 1. the texel boxes this segment's samples and streamlines can reach
    int box[12];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      box[i] = INT_MAX;       // lo: field xyz, noise xyz
      box[6 + i] = INT_MIN;   // hi
    }
    if (alive) {
      const float3 pe = add3(pos, scl3(dstep, (float)(b.seg - 1)));
      const float p0[3] = {pos.x, pos.y, pos.z}, p1[3] = {pe.x, pe.y, pe.z};
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        axis_box(p0[i], p1[i], (float)a.n[i], b.fr[i], box[i], box[6 + i]);
        axis_box(p0[i], p1[i], nsc[i], b.nr[i], box[3 + i], box[9 + i]);
      }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      box[i] = __reduce_min_sync(0xffffffffu, box[i]);
      box[6 + i] = __reduce_max_sync(0xffffffffu, box[6 + i]);
    }
    if (lane == 0)
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        st.lo[warp][i] = box[i];
        st.hi[warp][i] = box[6 + i];
      }
    if (!__syncthreads_or(alive)) break;
    if (tid == 0 && use_tma) {
      int lo[6], hi[6];
      for (int i = 0; i < 6; ++i) {
        lo[i] = st.lo[0][i];
        hi[i] = st.hi[0][i];
        for (int w = 1; w < kBrickThreads / 32; ++w) {
          lo[i] = min(lo[i], st.lo[w][i]);
          hi[i] = max(hi[i], st.hi[w][i]);
        }
      }
      for (int i = 0; i < 3; ++i) {
        st.fo[i] = place(lo[i], hi[i], b.fb[i], a.n[i], i == 0 ? b.falign : 1);
        st.no[i] = place(lo[3 + i], hi[3 + i], b.nb[i], a.m[i], i == 0 ? b.nalign : 1);
      }
      // the previous segment's shared-memory reads are ordered before the copies' writes
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&st.bar, b.fbytes + b.nbytes);
      tma_load_3d(fbrick, &b.fmap, st.fo[0] * b.tw, st.fo[1], st.fo[2], &st.bar);
      tma_load_3d(nbrick, &b.nmap, st.no[0] * a.noise_ch, st.no[1], st.no[2], &st.bar);
    }
    __syncthreads();
    // 2. wait for both bricks (bounded; the decision to go on is the whole CTA's)
    if (use_tma) {
      if (!__syncthreads_and(mbar_wait(&st.bar, phase))) {
        if (tid == 0) atomicOr(a.counters + 3, (unsigned long long)VVLIC_CHECK_BRICK);
        mbar_wait(&st.bar, phase);  // the copy may still land: a second bounded wait before leaving
        break;
      }
      phase ^= 1u;
    }
    // 3. march the segment (lic3d_fragment.glsl:38-95 per sample)
    for (int k = 0; k < b.seg && alive; ++k) {
      const float4 f = Field<ST, kBrick>::sample(a, pos);
      const float tfc = a.tf_index == VVLIC_TF_INDEX_MAGNITUDE ? f.w : f.z;
      const float4 tf = tf_rgba(s_tf, tfc);
      float4 il = compute_lic<ST, kBrick, kBrick, INTEG, GRAD>(a, pos, f);
      il.w *= a.intensity_scale;
      ++samples;
      const float4 src = shade<GRAD>(a, s_tf, il, tf, pos, dir, f);
      dest = blend(dest, src);
      pos = add3(pos, dstep);
      alive = !(outside_box(a, pos) || src.w > a.alpha_thr) && samples < max_samples;
    }
    // 4. every thread is done with the bricks before the next copies overwrite them
    __syncthreads();
  }
  if (px < a.W && py < a.H) store_pixel(a, px, py, dest, samples);
  flush_counters(a, samples, hit);
}

template <int ST, int INTEG, bool GRAD>
cudaError_t launch_one_brick(const RenderArgs& a, const BrickArgs& b, cudaStream_t s) {
  const size_t smem = kFieldOff + round128(b.fbytes) + round128(b.nbytes);
  auto kern = brick_kernel<ST, INTEG, GRAD>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((a.W + kBrickTileW - 1) / kBrickTileW, (a.H + kBrickTileH - 1) / kBrickTileH);
  kern<<<grid, kBrickThreads, smem, s>>>(a, b);
  return cudaGetLastError();
}

template <int ST>
cudaError_t launch_brick_storage(const RenderArgs& a, const BrickArgs& b, int integ, bool grad, cudaStream_t s) {
  if (grad) {
    if (integ == VVLIC_EULER) return launch_one_brick<ST, VVLIC_EULER, true>(a, b, s);
    if (integ == VVLIC_HEUN) return launch_one_brick<ST, VVLIC_HEUN, true>(a, b, s);
    return launch_one_brick<ST, VVLIC_RK4, true>(a, b, s);
  }
  if (integ == VVLIC_EULER) return launch_one_brick<ST, VVLIC_EULER, false>(a, b, s);
  if (integ == VVLIC_HEUN) return launch_one_brick<ST, VVLIC_HEUN, false>(a, b, s);
  return launch_one_brick<ST, VVLIC_RK4, false>(a, b, s);
}

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda).
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 3D tiled map over `base` (dims and box in elements, x fastest, rows of row_bytes).
bool encode_map(CUtensorMap* map, CUtensorMapDataType type, void* base, const uint64_t dims[3], uint64_t row_bytes,
                uint64_t slice_bytes, const uint32_t box[3]) {
  auto fn = encode_tiled();
  if (!fn) return false;
  const cuuint64_t gdim[3] = {dims[0], dims[1], dims[2]};
  const cuuint64_t gstride[2] = {row_bytes, slice_bytes};
  const cuuint32_t bdim[3] = {box[0], box[1], box[2]};
  const cuuint32_t estride[3] = {1, 1, 1};
  return fn(map, type, 3, base, gdim, gstride, bdim, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int round_up(int v, int m) { return (v + m - 1) / m * m; }

}  // namespace

// Brick shapes and tensor maps of a BRICK render of volume v with the argument block a.
vvlic_status prepare_brick(vvlic_ctx* c, Volume& v, const RenderArgs& a, bool grad, BrickArgs& b) {
  std::memset(&b, 0, sizeof b);
  NoiseTex& nz = c->noise;
  const int tw = texel_bytes(v.storage) / 4;
  const int ch = nz.ch;
  if (((size_t)v.n[0] * tw) % 4 != 0)
    return fail(c, VVLIC_ERR_UNSUPPORTED, "BRICK sampler: field rows must be a multiple of 16 bytes (nx = %d)", v.n[0]);
  if (((size_t)nz.m[0] * ch) % 16 != 0)
    return fail(c, VVLIC_ERR_UNSUPPORTED, "BRICK sampler: noise rows must be a multiple of 16 bytes (mx = %d)",
                nz.m[0]);
  b.tw = tw;
  b.falign = 4 / tw;     // x * tw words start on 16 bytes
  b.nalign = 16 / ch;    // x * ch bytes start on 16 bytes
  b.seg = 8;
  const float* nsc = grad ? a.nscale_grad : a.nscale;
  const double reach = (double)std::max(a.lb, a.lf) * a.h_eff * 1.001;  // texture units per axis
  const double march = (double)(b.seg - 1) * a.step_size;              // one segment along a ray
  int fb[3], nb[3];
  for (int i = 0; i < 3; ++i) {
    b.fr[i] = (float)(reach * a.n[i] + 1.0);
    b.nr[i] = (float)(reach * nsc[i] + 1.0);
    // a segment's samples of a 16x8 ray tile (about 4 texels across) plus its streamline reach
    fb[i] = (int)std::ceil(2.0 * b.fr[i] + march * a.scale_vol[i] * a.n[i] + 6.0);
    nb[i] = (int)std::ceil(2.0 * b.nr[i] + march * a.scale_vol[i] * nsc[i] + 6.0);
  }
  fb[0] += b.falign - 1;
  nb[0] += b.nalign - 1;
  // TMA boxes: at most 256 elements per dimension, inner extent a multiple of 16 bytes
  const int fmax[3] = {256 / tw, 256, 256}, nmax[3] = {256 / ch, 256, 256};
  for (int i = 0; i < 3; ++i) {
    fb[i] = std::min(std::min(fb[i], round_up(v.n[i], i == 0 ? b.falign : 1)), fmax[i]);
    nb[i] = std::min(std::min(nb[i], round_up(nz.m[i], i == 0 ? b.nalign : 1)), nmax[i]);
  }
  fb[0] = round_up(fb[0], b.falign);
  nb[0] = round_up(nb[0], b.nalign);
  // shared-memory budget: shrink the largest extent until both bricks fit beside the TF table
  const size_t budget = 200 * 1024 - kFieldOff;
  auto bytes = [&](const int* e, int unit) { return (size_t)e[0] * e[1] * e[2] * unit; };
  while (round128((unsigned)bytes(fb, tw * 4)) + round128((unsigned)bytes(nb, ch)) > budget) {
    int* big = bytes(fb, tw * 4) >= bytes(nb, ch) ? fb : nb;
    const int al = big == fb ? b.falign : b.nalign;
    int k = 0;
    for (int i = 1; i < 3; ++i)
      if (big[i] > big[k]) k = i;
    big[k] = k == 0 ? std::max(al, big[k] - al) : std::max(2, big[k] - 1);
  }
  for (int i = 0; i < 3; ++i) {
    b.fb[i] = fb[i];
    b.nb[i] = nb[i];
  }
  b.fbytes = (unsigned)bytes(fb, tw * 4);
  b.nbytes = (unsigned)bytes(nb, ch);
  // tensor maps, re-encoded when the box changes (addresses are stable across in-place updates)
  if (std::memcmp(v.brick_box, fb, sizeof fb) != 0) {
    const uint64_t dims[3] = {(uint64_t)v.n[0] * tw, (uint64_t)v.n[1], (uint64_t)v.n[2]};
    const uint32_t box[3] = {(uint32_t)(fb[0] * tw), (uint32_t)fb[1], (uint32_t)fb[2]};
    const uint64_t row = (uint64_t)v.n[0] * tw * 4;
    if (!encode_map(&v.brick_map, CU_TENSOR_MAP_DATA_TYPE_UINT32, v.d_texels, dims, row, row * v.n[1], box))
      return fail(c, VVLIC_ERR_CUDA, "BRICK sampler: field tensor map");
    std::memcpy(v.brick_box, fb, sizeof fb);
  }
  if (std::memcmp(nz.brick_box, nb, sizeof nb) != 0) {
    const uint64_t dims[3] = {(uint64_t)nz.m[0] * ch, (uint64_t)nz.m[1], (uint64_t)nz.m[2]};
    const uint32_t box[3] = {(uint32_t)(nb[0] * ch), (uint32_t)nb[1], (uint32_t)nb[2]};
    const uint64_t row = (uint64_t)nz.m[0] * ch;
    if (!encode_map(&nz.brick_map, CU_TENSOR_MAP_DATA_TYPE_UINT8, nz.d_texels, dims, row, row * nz.m[1], box))
      return fail(c, VVLIC_ERR_CUDA, "BRICK sampler: noise tensor map");
    std::memcpy(nz.brick_box, nb, sizeof nb);
  }
  b.fmap = v.brick_map;
  b.nmap = nz.brick_map;
  return VVLIC_OK;
}

cudaError_t launch_brick(int storage, const RenderArgs& a, const BrickArgs& b, int integ, bool grad, cudaStream_t s) {
  switch (storage) {
    case VVLIC_STORAGE_F32: return launch_brick_storage<VVLIC_STORAGE_F32>(a, b, integ, grad, s);
    case VVLIC_STORAGE_F16: return launch_brick_storage<VVLIC_STORAGE_F16>(a, b, integ, grad, s);
    case VVLIC_STORAGE_BF16: return launch_brick_storage<VVLIC_STORAGE_BF16>(a, b, integ, grad, s);
    default: return launch_brick_storage<VVLIC_STORAGE_UNORM8>(a, b, integ, grad, s);
  }
}

}  // namespace vvlic
