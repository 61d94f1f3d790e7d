// Batched rendering: job table, job-major (job, tile) order over the whole batch, the
// CUDA-graph-captured launch sequence and the tile-shape / sampler autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/vvlic.h"
#include "vvlic_device.cuh"
#include "vvlic_host.hpp"
#include "vvlic_launch.hpp"

using namespace vvlic;

namespace vvlic_batch_order {

__device__ __forceinline__ int job_of(const unsigned* start, int njobs, unsigned g) {
  int lo = 0, hi = njobs - 1;  // largest j with start[j] <= g
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Item g of the batch: job j = the job whose tiles contain g, tile g - start[j].  Jobs run in
// submission order and each job's tiles in raster order, so the warps in flight work on one or
// two volumes at a time and share their texels in L1 and L2.  Measured on the 64-volume batch
// (297 views at 512^2): 1065 ms per batch against 1252 ms for a longest-first order over all
// (job, tile) items, which spreads the warps in flight over every volume; the tail this order
// leaves is at most one job's last tiles.
__global__ void batch_order_kernel(const unsigned* start, int njobs, int ntiles, uint2* order) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ntiles; g += gridDim.x * blockDim.x) {
    const int j = job_of(start, njobs, (unsigned)g);
    order[g] = make_uint2((unsigned)j, (unsigned)g - start[j]);
  }
}

}  // namespace vvlic_batch_order

namespace vvlic {

cudaError_t launch_batch_order(const BatchScratch& b, int njobs, int ntiles, cudaStream_t s) {
  using namespace vvlic_batch_order;
  batch_order_kernel<<<std::max(1, std::min((ntiles + 255) / 256, 152 * 8)), 256, 0, s>>>(b.start, njobs, ntiles,
                                                                                          b.order);
  return cudaGetLastError();
}

}  // namespace vvlic

namespace {

vvlic_status grow_device(vvlic_ctx* c, void** p, size_t* cap, size_t bytes, const char* what) {
  if (*cap >= bytes) return VVLIC_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  *cap = bytes;
  return VVLIC_OK;
}

void drop_graph(vvlic_ctx* c) {
  if (c->batch_graph) cudaGraphExecDestroy(c->batch_graph);
  c->batch_graph = nullptr;
  std::memset(c->batch_key, 0, sizeof c->batch_key);
}

cudaError_t launch_batch(int storage, const BatchLaunch& b, int sampler, int integ, bool grad, cudaStream_t s) {
  switch (kernel_storage(storage, sampler)) {
    case VVLIC_STORAGE_F32: return launch_batch_f32(b, sampler, integ, grad, s);
    case VVLIC_STORAGE_F16: return launch_batch_f16(b, sampler, integ, grad, s);
    case VVLIC_STORAGE_UNORM8: return launch_batch_u8(b, sampler, integ, grad, s);
    default: return launch_batch_bf16(b, sampler, integ, grad, s);
  }
}

// Validates the jobs, builds their argument blocks into the pinned staging table and the
// per-job tile starts; returns the batch-wide variant and the tile count.
vvlic_status prepare_batch(vvlic_ctx* c, const vvlic_job* jobs, int n, int tw, int sampler_override, cudaStream_t s,
                           int* storage, int* sampler, int* integ, bool* grad, int* ntiles,
                           std::vector<unsigned>& start) {
  if (!jobs || n < 1 || n > 65536) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "batch: need 1..65536 jobs");
  // the staging table may still be in flight from the previous batch
  if (c->ev_jobs) cudaEventSynchronize(c->ev_jobs);
  const size_t table = (size_t)n * sizeof(RenderArgs);
  if (c->h_jobs_cap < table) {
    if (c->h_jobs) cudaFreeHost(c->h_jobs);
    c->h_jobs = nullptr;
    c->h_jobs_cap = 0;
    cudaError_t e = cudaHostAlloc((void**)&c->h_jobs, table, cudaHostAllocDefault);
    if (e != cudaSuccess) return cuda_fail(c, e, "batch staging allocation");
    c->h_jobs_cap = table;
  }
  start.assign(n + 1, 0);
  double total = 0.0;
  for (int j = 0; j < n; ++j) {
    const vvlic_job& jb = jobs[j];
    auto it = c->vols.find(jb.vol_id);
    if (it == c->vols.end()) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "batch: job %d: unknown volume %d", j, jb.vol_id);
    if (!jb.d_out || jb.w < 1 || jb.h < 1 || jb.w > 32768 || jb.h > 32768)
      return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "batch: job %d: bad image", j);
    vvlic_params p = jb.params;
    if (sampler_override >= 0) p.sampler = sampler_override;
    if (p.sampler == VVLIC_SAMPLER_BRICK)
      return fail(c, VVLIC_ERR_UNSUPPORTED, "batch: job %d: the BRICK sampler renders single images only", j);
    p.record_tape = 0;
    const vvlic_params& p0 = jobs[0].params;
    const int smp0 = sampler_override >= 0 ? sampler_override : p0.sampler;
    if (it->second.storage != c->vols[jobs[0].vol_id].storage || p.sampler != smp0 || p.integrator != p0.integrator ||
        (p.illum == VVLIC_ILLUM_GRADIENT) != (p0.illum == VVLIC_ILLUM_GRADIENT))
      return fail(c, VVLIC_ERR_INVALID_ARGUMENT,
                  "batch: job %d differs from job 0 in field storage, sampler, integrator or lighting", j);
    if (jb.view.projection != VVLIC_PERSPECTIVE && jb.view.projection != VVLIC_ORTHOGRAPHIC)
      return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "batch: job %d: projection", j);
    JobFilter jf;
    uint8_t tab[1024];
    if (jb.filter_table) {
      if (jb.filter_width < 1 || jb.filter_width > 1024)
        return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "batch: job %d: filter width", j);
      jf.width = centre_filter_table(jb.filter_table, jb.filter_width, tab, &jf.is_box);
      jf.table = tab;
      jf.clamp = jb.filter_clamp;
    }
    vvlic_status st = build_render_args_ex(c, it->second, jb.w, jb.h, s, p, jb.view, jb.filter_table ? &jf : nullptr,
                                           c->h_jobs[j]);
    if (st) return st;
    RenderArgs& a = c->h_jobs[j];
    a.out = jb.d_out;
    a.counters = c->d_counters;
    const int th = 32 / tw;
    const double tiles = (double)((jb.w + tw - 1) / tw) * (double)((jb.h + th - 1) / th);
    start[j] = (unsigned)total;
    total += tiles;
    if (total > 4.0e9) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "batch: too many tiles");
  }
  start[n] = (unsigned)total;
  *ntiles = (int)total;
  *storage = c->vols[jobs[0].vol_id].storage;
  *sampler = sampler_override >= 0 ? sampler_override : jobs[0].params.sampler;
  *integ = jobs[0].params.integrator;
  *grad = jobs[0].params.illum == VVLIC_ILLUM_GRADIENT;
  return VVLIC_OK;
}

vvlic_status batch_render(vvlic_ctx* c, const vvlic_job* jobs, int n, cudaStream_t s, int tw, int sampler_override) {
  int storage, sampler, integ, ntiles;
  bool grad;
  std::vector<unsigned> start;
  vvlic_status st = prepare_batch(c, jobs, n, tw, sampler_override, s, &storage, &sampler, &integ, &grad, &ntiles,
                                  start);
  if (st) return st;
  // device buffers; a reallocation invalidates the captured graph
  const void* old_jobs = c->d_jobs;
  const void* old_batch = c->d_batch;
  if ((st = grow_device(c, (void**)&c->d_jobs, &c->d_jobs_cap, (size_t)n * sizeof(RenderArgs), "batch job table")))
    return st;
  const size_t words = batch_scratch(nullptr, n, ntiles).words;
  size_t cap_bytes = c->batch_cap * sizeof(unsigned);
  if ((st = grow_device(c, (void**)&c->d_batch, &cap_bytes, words * sizeof(unsigned), "batch scratch"))) return st;
  c->batch_cap = cap_bytes / sizeof(unsigned);
  if (old_jobs != c->d_jobs || old_batch != c->d_batch) drop_graph(c);
  const BatchScratch bs = batch_scratch(c->d_batch, n, ntiles);
  unsigned* d_start = bs.start;
  // upload the job table and tile starts (outside the graph)
  cudaError_t e = cudaMemcpyAsync(c->d_jobs, c->h_jobs, (size_t)n * sizeof(RenderArgs), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_start, start.data(), (n + 1) * sizeof(unsigned), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    if (!c->ev_jobs) e = cudaEventCreateWithFlags(&c->ev_jobs, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_jobs, s);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "batch upload");
  const uint64_t key[8] = {(uint64_t)n, (uint64_t)ntiles, (uint64_t)storage, (uint64_t)sampler, (uint64_t)integ,
                           (uint64_t)grad, (uint64_t)tw, 0};
  if (!c->batch_graph || std::memcmp(key, c->batch_key, sizeof key) != 0) {
    drop_graph(c);
    // capture: counters reset, order pass, queue reset, the persistent launch
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(c, e, "batch graph capture (a non-default stream is required)");
    cudaError_t ec = cudaMemsetAsync(c->d_counters, 0, 4 * sizeof(unsigned long long), s);
    if (ec == cudaSuccess) ec = launch_batch_order(bs, n, ntiles, s);
    if (ec == cudaSuccess) ec = cudaMemsetAsync(bs.next, 0, sizeof(unsigned), s);
    if (ec == cudaSuccess) {
      BatchLaunch b{c->d_jobs, bs.order, ntiles, bs.next, c->d_tf, c->d_counters, tw, c->num_sms};
      ec = launch_batch(storage, b, sampler, integ, grad, s);
    }
    e = cudaStreamEndCapture(s, &graph);
    if (ec != cudaSuccess || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return cuda_fail(c, ec != cudaSuccess ? ec : e, "batch graph capture");
    }
    e = cudaGraphInstantiate(&c->batch_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      c->batch_graph = nullptr;
      return cuda_fail(c, e, "batch graph instantiate");
    }
    std::memcpy(c->batch_key, key, sizeof key);
  }
  e = cudaEventRecord(c->ev0, s);
  if (e == cudaSuccess) e = cudaGraphLaunch(c->batch_graph, s);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev1, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "batch launch");
  c->stats_pending = true;
  c->tape_flag_pending = false;
  c->last_was_batch = true;
  c->tape_valid = false;
  return VVLIC_OK;
}

}  // namespace

extern "C" vvlic_status vvlic_batch_render(vvlic_ctx* c, const vvlic_job* jobs, int32_t n, void* stream) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  DeviceGuard g(c->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  return batch_render(c, jobs, n, s, c->batch_tile_w, c->batch_sampler_override);
}

extern "C" vvlic_status vvlic_batch_autotune(vvlic_ctx* c, const vvlic_job* jobs, int32_t n, void* stream,
                                            int32_t* best_tile_w, int32_t* best_sampler, float* best_ms) {
  if (!c) return VVLIC_ERR_BAD_HANDLE;
  if (!jobs || n < 1) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "batch_autotune: no jobs");
  DeviceGuard g(c->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  auto it = c->vols.find(jobs[0].vol_id);
  if (it == c->vols.end()) return fail(c, VVLIC_ERR_INVALID_ARGUMENT, "batch_autotune: unknown volume");
  std::vector<int> samplers = {VVLIC_SAMPLER_HYBRID, VVLIC_SAMPLER_CELL};
  const int tws[4] = {8, 4, 16, 32};
  float best = 1e30f;
  int bt = c->batch_tile_w, bs = jobs[0].params.sampler;
  for (int smp : samplers) {
    for (int tw : tws) {
      float ms = 0.f;
      for (int rep = 0; rep < 2; ++rep) {  // the first render builds layouts and the graph
        vvlic_status st = batch_render(c, jobs, n, s, tw, smp);
        if (st) return st;
        cudaError_t e = cudaEventSynchronize(c->ev1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        if (e != cudaSuccess) return cuda_fail(c, e, "batch_autotune");
      }
      if (ms < best) {
        best = ms;
        bt = tw;
        bs = smp;
      }
    }
  }
  c->batch_tile_w = bt;
  c->batch_sampler_override = bs;
  drop_graph(c);
  if (best_tile_w) *best_tile_w = bt;
  if (best_sampler) *best_sampler = bs;
  if (best_ms) *best_ms = best;
  return VVLIC_OK;
}
