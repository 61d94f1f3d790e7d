// Measured fetch ceiling of the L1TEX unit: how many trilinear texture fetches and 256-bit
// read-only loads per second this GPU serves when every access hits L1.
//
// The ray-cast kernels spend their time in exactly these two operations — a hardware-trilinear
// tex3D of the RGBA16F field (k per streamline step: Euler 1, Heun 2, RK4 4, plus one per ray
// sample) and one 256-bit load of a corner-packed noise cell per tap — with L1 hit rates of
// 80-99 % and DRAM nearly idle.  HBM bandwidth is therefore not the bound that applies; the
// rate at which the L1TEX unit can serve these fetches is.  These kernels measure that rate
// with the access pattern of the render kernels' warps (an 8x4 ray tile whose lanes sit a
// fraction of a texel apart and advance a fraction of a texel per step), on data small enough
// to stay in L1, and with as little other work as possible.
//
// No counterpart in the reference.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/vvlic.h"
#include "vvlic_host.hpp"

namespace {

constexpr int kTexN = 16;          // 16^3 half4 texels: 32 KB, L1-resident
constexpr int kCells = 512;        // 8^3 cells of 32 bytes: 16 KB, L1-resident
constexpr int kThreads = 256;
constexpr int kBlocksPerSM = 8;    // 2048 threads per SM: full occupancy

__device__ __forceinline__ void ld256(const void* p, uint32_t (&r)[8]) {
  asm volatile("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "l"(p));
}

// NTEX trilinear fetches and NLD 256-bit loads per iteration.  `spread4` is the distance between
// neighbouring lanes of the 8x4 tile in quarter texels (1 = a quarter texel, the ray spacing of
// the 2048^2 / 512^3 frame).  Every access stays inside its buffer: the texture wraps (WRAP
// addressing) and cell indices are masked to kCells.
template <int NTEX, int NLD>
__global__ void __launch_bounds__(kThreads) fetch_kernel(cudaTextureObject_t tex, const uint4* __restrict__ cells,
                                                         int iters, int spread4, float* sink) {
  const int lane = threadIdx.x & 31;
  const unsigned warp = blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  // warp start: spread over the volume by a multiplicative hash
  const unsigned h = warp * 2654435761u;
  const float t = 1.0f / kTexN;
  float x = ((h & 1023u) * (1.0f / 1024.0f)) + (float)((lane & 7) * spread4) * 0.25f * t;
  float y = (((h >> 10) & 1023u) * (1.0f / 1024.0f)) + (float)((lane >> 3) * spread4) * 0.25f * t;
  float z = ((h >> 20) & 1023u) * (1.0f / 1024.0f);
  const float dx = 0.21f * t, dy = 0.13f * t, dz = 0.07f * t;  // about a quarter texel per step
  unsigned c = ((h >> 7) + ((((lane & 7) * spread4) >> 2) + (((lane >> 3) * spread4) >> 2) * 8)) & (kCells - 1);
  float acc0 = 0.f, acc1 = 0.f;
  uint32_t accl = 0;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < NTEX; ++k) {
      // permuted coordinates: distinct positions without extra arithmetic
      const float4 v = k == 0 ? tex3D<float4>(tex, x, y, z)
                       : k == 1 ? tex3D<float4>(tex, y, z, x)
                       : k == 2 ? tex3D<float4>(tex, z, x, y)
                                : tex3D<float4>(tex, x, z, y);
      acc0 = fmaf(v.x, v.y, acc0);
      acc1 = fmaf(v.z, v.w, acc1);
    }
    x += dx;
    y += dy;
    z += dz;
#pragma unroll
    for (int k = 0; k < NLD; ++k) {
      uint32_t r[8];
      ld256(cells + 2 * ((c + 73u * k) & (kCells - 1)), r);
      accl ^= r[0] ^ r[7];
    }
    ++c;
  }
  // a data-dependent store the compiler cannot fold away keeps every fetch alive
  if (__float_as_uint(acc0 + acc1) == (accl ^ 0x9e3779b9u)) sink[0] = acc0;
}

template <int NTEX, int NLD>
cudaError_t time_kernel(cudaTextureObject_t tex, const uint4* cells, float* sink, int blocks, int iters, int spread4,
                        cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, int repeats, float* best_ms) {
  *best_ms = 1e30f;
  fetch_kernel<NTEX, NLD><<<blocks, kThreads, 0, s>>>(tex, cells, iters / 8, spread4, sink);  // warm-up
  for (int r = 0; r < repeats; ++r) {
    cudaEventRecord(e0, s);
    fetch_kernel<NTEX, NLD><<<blocks, kThreads, 0, s>>>(tex, cells, iters, spread4, sink);
    cudaEventRecord(e1, s);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) return e;
    float ms = 0.f;
    if ((e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) return e;
    *best_ms = std::min(*best_ms, ms);
  }
  return cudaGetLastError();
}

}  // namespace

extern "C" vvlic_status vvlic_measure_fetch_ceiling(int32_t device, int32_t spread4, vvlic_fetch_ceiling* out) {
  if (!out || spread4 < 0 || spread4 > 64) return VVLIC_ERR_INVALID_ARGUMENT;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return VVLIC_ERR_NO_DEVICE;
  vvlic::DeviceGuard g(device);
  std::memset(out, 0, sizeof *out);
  int sms = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return VVLIC_ERR_CUDA;
  cudaArray_t arr = nullptr;
  cudaTextureObject_t tex = 0;
  uint4* cells = nullptr;
  float* sink = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  vvlic_status st = VVLIC_OK;
  do {
    // texels in [0, 1] (the encoded field's range) and arbitrary cell bytes
    std::vector<__half> host(4 * kTexN * kTexN * kTexN);
    for (size_t i = 0; i < host.size(); ++i) host[i] = __float2half((float)((i * 37u) % 251u) / 250.0f);
    cudaChannelFormatDesc desc = cudaCreateChannelDescHalf4();
    if ((e = cudaMalloc3DArray(&arr, &desc, make_cudaExtent(kTexN, kTexN, kTexN))) != cudaSuccess) break;
    cudaMemcpy3DParms cp;
    std::memset(&cp, 0, sizeof cp);
    cp.srcPtr = make_cudaPitchedPtr(host.data(), kTexN * 8, kTexN, kTexN);
    cp.dstArray = arr;
    cp.extent = make_cudaExtent(kTexN, kTexN, kTexN);
    cp.kind = cudaMemcpyHostToDevice;
    if ((e = cudaMemcpy3D(&cp)) != cudaSuccess) break;
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof rd);
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof td);
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    if ((e = cudaCreateTextureObject(&tex, &rd, &td, nullptr)) != cudaSuccess) break;
    if ((e = cudaMalloc(&cells, kCells * 32)) != cudaSuccess) break;
    if ((e = cudaMemset(cells, 0x5a, kCells * 32)) != cudaSuccess) break;
    if ((e = cudaMalloc(&sink, sizeof(float))) != cudaSuccess) break;
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) break;
    const int blocks = sms * kBlocksPerSM;
    const int iters = 2048, repeats = 5;
    const double threads = (double)blocks * kThreads * iters;
    float ms;
    if ((e = time_kernel<4, 0>(tex, cells, sink, blocks, iters, spread4, s, e0, e1, repeats, &ms)) != cudaSuccess) break;
    out->tex_per_s = threads * 4 / (ms * 1e-3);
    out->ms[0] = ms;
    if ((e = time_kernel<0, 4>(tex, cells, sink, blocks, iters, spread4, s, e0, e1, repeats, &ms)) != cudaSuccess) break;
    out->ld256_per_s = threads * 4 / (ms * 1e-3);
    out->ms[1] = ms;
    if ((e = time_kernel<1, 1>(tex, cells, sink, blocks, iters, spread4, s, e0, e1, repeats, &ms)) != cudaSuccess) break;
    out->group_per_s[0] = threads / (ms * 1e-3);
    out->ms[2] = ms;
    if ((e = time_kernel<2, 1>(tex, cells, sink, blocks, iters, spread4, s, e0, e1, repeats, &ms)) != cudaSuccess) break;
    out->group_per_s[1] = threads / (ms * 1e-3);
    out->ms[3] = ms;
    if ((e = time_kernel<4, 1>(tex, cells, sink, blocks, iters, spread4, s, e0, e1, repeats, &ms)) != cudaSuccess) break;
    out->group_per_s[2] = threads / (ms * 1e-3);
    out->ms[4] = ms;
    out->num_sms = sms;
    out->spread4 = spread4;
  } while (false);
  if (e != cudaSuccess) st = e == cudaErrorMemoryAllocation ? VVLIC_ERR_OUT_OF_MEMORY : VVLIC_ERR_CUDA;
  if (s) cudaStreamSynchronize(s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  if (tex) cudaDestroyTextureObject(tex);
  if (arr) cudaFreeArray(arr);
  if (cells) cudaFree(cells);
  if (sink) cudaFree(sink);
  return st;
}
