// Device preprocessing: field encoding (dataset.cpp:533-635), noise gradients
// (gradient.cpp:190-531 + dataset.cpp:1270-1286) and the corner-packed cell arrays.
//
// This file is compiled with -fmad=false: every float expression rounds like the reference's
// CPU code (no fused multiply-add), so the encoded field and the quantised gradients are
// bit-identical to the reference's own arithmetic.  The one explicit fma (quantize_unit) only
// decides a byte where it provably equals the reference's double expression.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>

#include "../../include/vvlic.h"
#include "vvlic_device.cuh"
#include "vvlic_launch.hpp"

namespace vvlic {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float vlen_f32(const float* f) { return sqrtf(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]); }

// Magnitude of voxel a as fillTexDataFloatInterp computes it (0 below EPS = 1e-5f).
__device__ __forceinline__ float voxel_len(const void* xyz, int dtype, size_t a, unsigned char t[3]) {
  float len;
  if (dtype == VVLIC_DTYPE_UINT8) {
    const uint8_t* u = reinterpret_cast<const uint8_t*>(xyz) + 3 * a;
    // `dataU -= 128` on unsigned char wraps modulo 256 (dataset.cpp:565-569)
    for (int c = 0; c < 3; ++c) t[c] = (unsigned char)(u[c] - 128);
    len = sqrtf((float)((int)t[0] * t[0]) + (float)((int)t[1] * t[1]) + (float)((int)t[2] * t[2]));
  } else {
    len = vlen_f32(reinterpret_cast<const float*>(xyz) + 3 * a);
  }
  return len < 1e-5f ? 0.0f : len;
}

__global__ void field_maxlen_kernel(const void* xyz, int dtype, size_t count, unsigned* maxbits) {
  float m = 0.0f;
  for (size_t a = blockIdx.x * (size_t)blockDim.x + threadIdx.x; a < count; a += (size_t)gridDim.x * blockDim.x) {
    unsigned char t[3];
    m = fmaxf(m, voxel_len(xyz, dtype, a, t));
  }
  // non-negative floats order like their bit patterns
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxbits, __float_as_uint(m));
}

template <int ST>
__device__ __forceinline__ void store_texel(void* out, size_t a, float r, float g, float b, float al) {
  if (ST == VVLIC_STORAGE_F32) {
    reinterpret_cast<float4*>(out)[a] = make_float4(r, g, b, al);
  } else if (ST == VVLIC_STORAGE_F16) {
    __half2 lo = __halves2half2(__float2half_rn(r), __float2half_rn(g));
    __half2 hi = __halves2half2(__float2half_rn(b), __float2half_rn(al));
    uint2 v;
    v.x = *reinterpret_cast<unsigned*>(&lo);
    v.y = *reinterpret_cast<unsigned*>(&hi);
    reinterpret_cast<uint2*>(out)[a] = v;
  } else if (ST == VVLIC_STORAGE_UNORM8) {
    // nearest multiple of 1/255 (x*255 rounded in float, then to nearest integer)
    const unsigned q0 = __float2uint_rn(r * 255.0f), q1 = __float2uint_rn(g * 255.0f),
                   q2 = __float2uint_rn(b * 255.0f), q3 = __float2uint_rn(al * 255.0f);
    reinterpret_cast<uint32_t*>(out)[a] = min(q0, 255u) | (min(q1, 255u) << 8) | (min(q2, 255u) << 16) |
                                          (min(q3, 255u) << 24);
  } else {
    __nv_bfloat16 br = __float2bfloat16_rn(r), bg = __float2bfloat16_rn(g), bb = __float2bfloat16_rn(b),
                  ba = __float2bfloat16_rn(al);
    uint2 v;
    v.x = (unsigned)*reinterpret_cast<unsigned short*>(&br) | ((unsigned)*reinterpret_cast<unsigned short*>(&bg) << 16);
    v.y = (unsigned)*reinterpret_cast<unsigned short*>(&bb) | ((unsigned)*reinterpret_cast<unsigned short*>(&ba) << 16);
    reinterpret_cast<uint2*>(out)[a] = v;
  }
}

template <int ST>
__global__ void field_encode_kernel(const void* xyz, int dtype, size_t count, const unsigned* maxbits, void* out) {
  const float max_len = __uint_as_float(*maxbits);
  for (size_t a = blockIdx.x * (size_t)blockDim.x + threadIdx.x; a < count; a += (size_t)gridDim.x * blockDim.x) {
    unsigned char t[3];
    float len = voxel_len(xyz, dtype, a, t);
    float r, g, b;
    if (len == 0.0f) {
      r = g = b = 0.5f;
    } else if (dtype == VVLIC_DTYPE_UINT8) {
      r = 0.5f * (float)t[0] / len + 0.5f;
      g = 0.5f * (float)t[1] / len + 0.5f;
      b = 0.5f * (float)t[2] / len + 0.5f;
    } else {
      const float* f = reinterpret_cast<const float*>(xyz) + 3 * a;
      r = 0.5f * f[0] / len + 0.5f;
      g = 0.5f * f[1] / len + 0.5f;
      b = 0.5f * f[2] / len + 0.5f;
    }
    float al = max_len > 0.0f ? len / max_len : 0.0f;
    al = (al > 1.0f) ? 1.0f : ((al < 0.0f) ? 0.0f : al);
    store_texel<ST>(out, a, r, g, b, al);
  }
}

__device__ __forceinline__ float nv(const uint8_t* v, int nx, int ny, int x, int y, int z) {
  return (float)v[((size_t)z * ny + y) * nx + x];
}

// The noise-gradient kernels run one thread per x voxel on a (ceil(nx / kThreads), ny, nz) grid,
// the y and z extents capped at the grid limit (the kernels step over the rest): a voxel's
// coordinates come from the block and thread indices without integer division.
constexpr int kGridYZ = 65535;
inline dim3 voxel_grid(const int m[3]) {
  return dim3((unsigned)((m[0] + kThreads - 1) / kThreads), (unsigned)std::min(m[1], kGridYZ),
              (unsigned)std::min(m[2], kGridYZ));
}

// computeGradients (gradient.cpp:190-374) for one voxel.
__global__ void noise_grad_raw_kernel(const uint8_t* v, int nx, int ny, int nz, int mode, float sd0, float sd1,
                                      float sd2, float4* g) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nx) return;
  for (int z = blockIdx.z; z < nz; z += gridDim.z)
  for (int y = blockIdx.y; y < ny; y += gridDim.y) {
    const size_t a = ((size_t)z * ny + y) * nx + x;
    const float sd[3] = {sd0, sd1, sd2};
    float gp[3];
    if (mode == VVLIC_NOISE_GRAD_SOBEL && x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1) {
      // weights[dir][i+1][j+1][k+1]: the 3x3x3 Sobel masks (gradient.cpp:199-224), summed in
      // the reference's i, j, k order
      const int s1[3] = {1, 3, 1}, s2[3] = {3, 6, 3};
      // the 27 neighbours once; the three masks then run over them in the same i, j, k order
      float nb[27];
#pragma unroll
      for (int i = -1; i < 2; i++)
#pragma unroll
        for (int j = -1; j < 2; j++)
#pragma unroll
          for (int k = -1; k < 2; k++) nb[((i + 1) * 3 + (j + 1)) * 3 + (k + 1)] = nv(v, nx, ny, x + i, y + j, z + k);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        float acc = 0.0f;
#pragma unroll
        for (int i = -1; i < 2; i++)
#pragma unroll
          for (int j = -1; j < 2; j++)
#pragma unroll
            for (int k = -1; k < 2; k++) {
              const int o[3] = {i, j, k};
              const int e = o[d];  // derivative axis offset
              const int p = o[(d + 1) % 3], q = o[(d + 2) % 3];
              // mask = sign(e) * w(p) * w(q) with w = (1,3,1) cross (1,3,1) pattern (1,3,1;3,6,3;1,3,1)
              int w = e == 0 ? 0 : e * ((p == 0 ? s2 : s1)[q + 1]);
              acc += (float)w * nb[((i + 1) * 3 + (j + 1)) * 3 + (k + 1)];
            }
        gp[d] = acc / (2.0f * sd[d]);
      }
    } else {
      // the voxel's neighbours along axis d lie `st[d]` bytes away
      const uint8_t* cp = v + a;
      const float c = (float)cp[0];
      const size_t st[3] = {1, (size_t)nx, (size_t)nx * ny};
      const int P[3] = {x, y, z}, N[3] = {nx, ny, nz};
      if (mode == VVLIC_NOISE_GRAD_SOBEL) {
        // one-sided differences on the border of the Sobel mode
#pragma unroll
        for (int d = 0; d < 3; ++d)
          gp[d] = (P[d] < 1) ? ((float)cp[st[d]] - c) / sd[d] : (c - (float)*(cp - st[d])) / sd[d];
      } else {
        // central differences (SOBEL 0 branch); the last slice per axis uses a one-sided
        // difference — those values are never read by the smoothing window below
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          if (P[d] < 1) gp[d] = ((float)cp[st[d]] - c) / sd[d];
          else if (P[d] >= N[d] - 1) gp[d] = (c - (float)*(cp - st[d])) / sd[d];
          else gp[d] = ((float)cp[st[d]] - (float)*(cp - st[d])) / sd[d] * 0.5f;
        }
      }
    }
    g[a] = make_float4(gp[0], gp[1], gp[2], 0.0f);  // padded to 16 bytes: one vector load per filter tap
  }
}

struct W27 {
  float w[27];
};

// (unsigned char)(((double)c + 1.0) / 2.0 * 255.0), quantizeGradients' conversion of a unit
// component c (gradient.cpp:466-477), without double arithmetic for almost every input.  The
// float t = fma(c, 127.5, 127.5) is within 2^-17 of the exact (c + 1) * 127.5 and the double
// expression within 2^-44 of it; the exact value is an integer only at c = -1 and c = 1, so
// when t lies more than 1e-4 from an integer both truncate to floor(t).  Inputs nearer an
// integer (about 2 in 10^4) take the double expression itself, in a call of its own so that the
// compiler cannot evaluate it speculatively for every voxel (GB300's FP64 rate is a small
// fraction of its FP32 rate).
__device__ __noinline__ unsigned char quantize_unit_double(float c) {
  return (unsigned char)(((double)c + 1.0) / 2.0 * 255.0);
}
__device__ __forceinline__ unsigned char quantize_unit(float c) {
  const float t = fmaf(c, 127.5f, 127.5f);
  const float f = floorf(t);
  const float r = t - f;
  if (r > 1e-4f && r < 1.0f - 1e-4f) return (unsigned char)(int)f;
  return quantize_unit_double(c);
}

// filterGradients + quantize8 + RGBA pack (gradient.cpp:377-478, dataset.cpp:1270-1286).
__global__ void noise_grad_filter_kernel(const uint8_t* v, const float4* g, int nx, int ny, int nz,
                                         const __grid_constant__ W27 fw27,
                                         uint8_t* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nx) return;
  for (int z = blockIdx.z; z < nz; z += gridDim.z)
  for (int y = blockIdx.y; y < ny; y += gridDim.y) {
    const size_t a = ((size_t)z * ny + y) * nx + x;
    int bd = min(min(min(x, nx - x - 1), min(y, ny - y - 1)), min(z, nz - z - 1));
    const int fw = min(2, bd);
    // One pass over the window with the three channel sums side by side: each channel adds its
    // terms in the reference's (k, j, i) order, so the sums are the per-channel loops' bit for bit.
    float acc[3] = {0.0f, 0.0f, 0.0f};
    if (fw == 2) {  // interior: k, j, i in {-2, -1, 0}, table entries (k+2, j+2, i+2)
#pragma unroll
      for (int k = -2; k < 1; ++k)
#pragma unroll
        for (int j = -2; j < 1; ++j) {
          const float4* row = g + ((size_t)(z + k) * ny + (y + j)) * nx + x;
#pragma unroll
          for (int i = -2; i < 1; ++i) {
            const float w = fw27.w[((k + 2) * 3 + (j + 2)) * 3 + (i + 2)];
            const float4 q = row[i];
            acc[0] += w * q.x;
            acc[1] += w * q.y;
            acc[2] += w * q.z;
          }
        }
    } else {
      for (int k = -fw; k < fw - 1; ++k)
        for (int j = -fw; j < fw - 1; ++j)
          for (int i = -fw; i < fw - 1; ++i) {
            // the reference indexes its 5x5x5 table with the shrunken fw; only entries with
            // all three indices in [0, 2] are ever used
            const int wk = fw + k, wj = fw + j, wi = fw + i;
            const float w = fw27.w[(wk * 3 + wj) * 3 + wi];
            const float4 q = g[((size_t)(z + k) * ny + (y + j)) * nx + (x + i)];
            acc[0] += w * q.x;
            acc[1] += w * q.y;
            acc[2] += w * q.z;
          }
    }
    float len = sqrtf(acc[0] * acc[0] + acc[1] * acc[1] + acc[2] * acc[2]);
    if (len < 1e-5f) {
      acc[0] = acc[1] = acc[2] = 0.0f;
    } else {
      acc[0] /= len;
      acc[1] /= len;
      acc[2] /= len;
    }
    uchar4 o;
    o.x = quantize_unit(acc[0]);
    o.y = quantize_unit(acc[1]);
    o.z = quantize_unit(acc[2]);
    o.w = v[a];
    reinterpret_cast<uchar4*>(out)[a] = o;
  }
}


// cell c per axis covers texels clamp(c-1), clamp(c): (n+1)^3 cells of 8 texels
template <int ST>
__global__ void field_cells_kernel(const void* texels, int nx, int ny, int nz, void* cells) {
  using T = typename std::conditional<ST == VVLIC_STORAGE_F32, float4,
                                      typename std::conditional<ST == VVLIC_STORAGE_UNORM8, uint32_t, uint2>::type>::type;
  const T* t = reinterpret_cast<const T*>(texels);
  T* c = reinterpret_cast<T*>(cells);
  const int cx = nx + 1, cy = ny + 1, cz = nz + 1;
  const size_t count = (size_t)cx * cy * cz;
  for (size_t a = blockIdx.x * (size_t)blockDim.x + threadIdx.x; a < count; a += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(a % cx), y = (int)((a / cx) % cy), z = (int)(a / ((size_t)cx * cy));
    const int x0 = max(x - 1, 0), x1 = min(x, nx - 1), y0 = max(y - 1, 0), y1 = min(y, ny - 1), z0 = max(z - 1, 0),
              z1 = min(z, nz - 1);
    const int xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      c[8 * a + k] = t[((size_t)zs[(k >> 2) & 1] * ny + ys[(k >> 1) & 1]) * nx + xs[k & 1]];
    }
  }
}

// noise cell i per axis covers texels i and (i+1) mod m (REPEAT): m^3 cells
__global__ void noise_cells_kernel(const uint8_t* texels, int mx, int my, int mz, int ch, uint8_t* cells) {
  const size_t count = (size_t)mx * my * mz;
  const int m[3] = {mx, my, mz};
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < count; v += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(v % mx), y = (int)((v / mx) % my), z = (int)(v / ((size_t)mx * my));
    const size_t a = noise_cell_index(x, y, z, m);
    const int xs[2] = {x, x + 1 == mx ? 0 : x + 1}, ys[2] = {y, y + 1 == my ? 0 : y + 1},
              zs[2] = {z, z + 1 == mz ? 0 : z + 1};
    // the cell is assembled in registers and written with 16-byte (RGBA: 32-byte cells) or one
    // 8-byte (value: 8-byte cells) stores; cells are 32- / 8-byte aligned
    if (ch == 4) {
      const uint32_t* t = reinterpret_cast<const uint32_t*>(texels);
      uint32_t q[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) q[k] = t[((size_t)zs[(k >> 2) & 1] * my + ys[(k >> 1) & 1]) * mx + xs[k & 1]];
      uint4* c = reinterpret_cast<uint4*>(cells) + 2 * a;
      c[0] = make_uint4(q[0], q[1], q[2], q[3]);
      c[1] = make_uint4(q[4], q[5], q[6], q[7]);
    } else {
      uint32_t lo = 0, hi = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        lo |= (uint32_t)texels[((size_t)zs[(k >> 2) & 1] * my + ys[(k >> 1) & 1]) * mx + xs[k & 1]] << (8 * k);
        hi |= (uint32_t)texels[((size_t)zs[1] * my + ys[(k >> 1) & 1]) * mx + xs[k & 1]] << (8 * k);
      }
      reinterpret_cast<uint2*>(cells)[a] = make_uint2(lo, hi);
    }
  }
}

inline int grid_for(size_t count) {
  size_t b = (count + kThreads - 1) / kThreads;
  return (int)(b < 152 * 64 ? (b == 0 ? 1 : b) : 152 * 64);
}

// One RGBA texel per iteration: four bf16 values (8 bytes) -> four halves (8 bytes), the
// component order kept (x in the low half of the first word).
__global__ void bf16_to_half_kernel(const uint2* in, size_t count, uint2* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
    const uint2 r = in[i];
    __half2 lo = __floats2half2_rn(__uint_as_float(r.x << 16), __uint_as_float(r.x & 0xffff0000u));
    __half2 hi = __floats2half2_rn(__uint_as_float(r.y << 16), __uint_as_float(r.y & 0xffff0000u));
    out[i] = make_uint2(*reinterpret_cast<uint32_t*>(&lo), *reinterpret_cast<uint32_t*>(&hi));
  }
}

}  // namespace

namespace {
// Time interpolation of fillTexData*Interp (dataset.cpp:555-585): t = interpIndex / InterpSize,
// FLOAT3: data + t * (next - data); UCHAR3: the same on the 128-shifted bytes, stored back
// un-shifted so the encoding's own shift recovers the interpolated value.
__global__ void field_interp_kernel(const void* a0, const void* a1, int dtype, size_t count3, float t, void* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count3; i += (size_t)gridDim.x * blockDim.x) {
    if (dtype == VVLIC_DTYPE_UINT8) {
      const unsigned char d = (unsigned char)(reinterpret_cast<const uint8_t*>(a0)[i] - 128);
      const unsigned char nx = (unsigned char)(reinterpret_cast<const uint8_t*>(a1)[i] - 128);
      const unsigned char v = (unsigned char)((float)d + t * (float)((int)nx - (int)d));
      reinterpret_cast<uint8_t*>(out)[i] = (uint8_t)(v + 128);
    } else {
      const float d = reinterpret_cast<const float*>(a0)[i], nx = reinterpret_cast<const float*>(a1)[i];
      reinterpret_cast<float*>(out)[i] = d + t * (nx - d);
    }
  }
}
}  // namespace

cudaError_t launch_interp_field(const void* d_a0, const void* d_a1, int dtype, const int n[3], float t, void* d_out,
                                cudaStream_t s) {
  const size_t count3 = (size_t)n[0] * n[1] * n[2] * 3;
  field_interp_kernel<<<grid_for(count3), kThreads, 0, s>>>(d_a0, d_a1, dtype, count3, t, d_out);
  return cudaGetLastError();
}

cudaError_t launch_encode_field(const void* d_xyz, int dtype, const int n[3], int storage, void* d_texels,
                                unsigned* d_maxbits, cudaStream_t s) {
  const size_t count = (size_t)n[0] * n[1] * n[2];
  cudaError_t e = cudaMemsetAsync(d_maxbits, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  field_maxlen_kernel<<<grid_for(count), kThreads, 0, s>>>(d_xyz, dtype, count, d_maxbits);
  if (storage == VVLIC_STORAGE_F32)
    field_encode_kernel<VVLIC_STORAGE_F32><<<grid_for(count), kThreads, 0, s>>>(d_xyz, dtype, count, d_maxbits, d_texels);
  else if (storage == VVLIC_STORAGE_F16)
    field_encode_kernel<VVLIC_STORAGE_F16><<<grid_for(count), kThreads, 0, s>>>(d_xyz, dtype, count, d_maxbits, d_texels);
  else if (storage == VVLIC_STORAGE_UNORM8)
    field_encode_kernel<VVLIC_STORAGE_UNORM8><<<grid_for(count), kThreads, 0, s>>>(d_xyz, dtype, count, d_maxbits,
                                                                                    d_texels);
  else
    field_encode_kernel<VVLIC_STORAGE_BF16><<<grid_for(count), kThreads, 0, s>>>(d_xyz, dtype, count, d_maxbits, d_texels);
  return cudaGetLastError();
}

cudaError_t launch_noise_gradients(const uint8_t* d_noise, const int m[3], int mode, const float sd[3], float* d_grad,
                                   uint8_t* d_rgba, const float w27[27], cudaStream_t s) {
  float4* g4 = reinterpret_cast<float4*>(d_grad);
  noise_grad_raw_kernel<<<voxel_grid(m), kThreads, 0, s>>>(d_noise, m[0], m[1], m[2], mode, sd[0], sd[1], sd[2], g4);
  W27 w;
  for (int i = 0; i < 27; ++i) w.w[i] = w27[i];
  noise_grad_filter_kernel<<<voxel_grid(m), kThreads, 0, s>>>(d_noise, g4, m[0], m[1], m[2], w, d_rgba);
  return cudaGetLastError();
}

cudaError_t launch_build_field_cells(const void* d_texels, const int n[3], int storage, void* d_cells,
                                     cudaStream_t s) {
  const size_t count = (size_t)(n[0] + 1) * (n[1] + 1) * (n[2] + 1);
  if (storage == VVLIC_STORAGE_F32)
    field_cells_kernel<VVLIC_STORAGE_F32><<<grid_for(count), kThreads, 0, s>>>(d_texels, n[0], n[1], n[2], d_cells);
  else if (storage == VVLIC_STORAGE_F16)
    field_cells_kernel<VVLIC_STORAGE_F16><<<grid_for(count), kThreads, 0, s>>>(d_texels, n[0], n[1], n[2], d_cells);
  else if (storage == VVLIC_STORAGE_UNORM8)
    field_cells_kernel<VVLIC_STORAGE_UNORM8><<<grid_for(count), kThreads, 0, s>>>(d_texels, n[0], n[1], n[2], d_cells);
  else
    field_cells_kernel<VVLIC_STORAGE_BF16><<<grid_for(count), kThreads, 0, s>>>(d_texels, n[0], n[1], n[2], d_cells);
  return cudaGetLastError();
}

cudaError_t launch_bf16_to_half(const void* d_bf16, size_t count, void* d_half, cudaStream_t s) {
  bf16_to_half_kernel<<<grid_for(count), kThreads, 0, s>>>(reinterpret_cast<const uint2*>(d_bf16), count,
                                                          reinterpret_cast<uint2*>(d_half));
  return cudaGetLastError();
}

cudaError_t launch_build_noise_cells(const uint8_t* d_texels, const int m[3], int ch, uint8_t* d_cells,
                                     cudaStream_t s) {
  const size_t count = (size_t)m[0] * m[1] * m[2];
  noise_cells_kernel<<<grid_for(count), kThreads, 0, s>>>(d_texels, m[0], m[1], m[2], ch, d_cells);
  return cudaGetLastError();
}

}  // namespace vvlic
