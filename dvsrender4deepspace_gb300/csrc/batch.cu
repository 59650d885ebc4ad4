// Multi-sensor batch kernels of the GB300 DVS path (sm_103a).
//
// A batch advances many sensors over one shared scene geometry in lockstep
// (the batching workload: many uneven trajectories over one terrain).  Each
// step traces every sensor's cells in ONE persistent launch: a grid of
// resident blocks that pull runs of work items -- one warp packet (32/CW
// pixels x CW cells of one sensor) per warp -- from a device counter, so
// sensors of different sizes share the GPU without a tail per sensor; then one
// circuit launch integrates every sensor's pixels.  The host captures the
// whole step (uploads, these launches, the per-sensor event compaction and
// status copies) into a CUDA graph and replays it while the sensors' batch
// shapes stay the same.  Items execute the one-sensor kernels' per-item code
// (trace_item.cuh), so a sensor's results are the same alone or in a batch.
// Built with -fmad=false like kernels.cu.
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.h"
#include "trace_item.cuh"

namespace dvsgb {
namespace {

// The job holding an item or block: the last j with first[j] <= x (first[0] = 0).
template <class T>
__device__ __forceinline__ int job_of(const T *first, int n_jobs, T x) {
  int lo = 0, hi = n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (first[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The job table travels as the launch's parameter block (__grid_constant__: no
// copy), so a warp reads its job's view -- the same job for all its lanes --
// through the constant cache, as the one-sensor kernel reads its view.
template <int kRays, int kGeo>
__global__ void __launch_bounds__(128, kRays == 2 ? DVS_TRACE_PAIR_MIN_BLOCKS : DVS_TRACE_MIN_BLOCKS)
    trace_jobs_kernel(const __grid_constant__ TraceJobs P) {
  __shared__ int s_code[kWarpsPerBlock][kStackSlots];
  __shared__ float s_t[kWarpsPerBlock][kStackSlots];
  __shared__ SubraySample s_subrays[kWarpsPerBlock][kSubrayTable];
  __shared__ long long s_first[kMaxBatchJobs];
  __shared__ long long s_base;
  for (int j = threadIdx.x; j < P.n_jobs; j += blockDim.x) s_first[j] = P.jobs[j].first_item;
  const int wib = threadIdx.x >> 5;
  // A block takes kWarpsPerBlock consecutive items at a time (one per warp),
  // as a block of the one-sensor kernel holds consecutive packets: the warps
  // of an SM then trace neighbouring pixels, whose nodes stay in its L1.
  while (true) {
    __syncthreads();  // every warp is done with the previous s_base
    if (threadIdx.x == 0) s_base = (long long)atomicAdd(P.next_item, (unsigned long long)kWarpsPerBlock);
    __syncthreads();
    const long long base = s_base;
    if (base >= P.total_items) break;  // block-uniform
    const long long item = base + wib;
    if (item < P.total_items) {        // warp-uniform
      const int j = job_of<long long>(s_first, P.n_jobs, item);
      const TraceJob &J = P.jobs[j];
      trace_cells_item<kRadiance, kRays, kGeo>(J.view, J.n_pix, nullptr, J.poses, J.c0, J.nc, J.cw_log2,
                                               J.radiance, nullptr, J.counters, item - s_first[j], s_code[wib],
                                               s_t[wib], s_subrays[wib]);
    }
  }
}

template <bool kF32, bool kPhilox>
__global__ void __launch_bounds__(128) circuit_jobs_kernel(const CircuitJob *__restrict__ jobs, int n_jobs) {
  __shared__ int s_first[kMaxBatchJobs];
  for (int j = threadIdx.x; j < n_jobs; j += blockDim.x) s_first[j] = jobs[j].first_block;
  __syncthreads();
  const CircuitJob &J = jobs[job_of<int>(s_first, n_jobs, (int)blockIdx.x)];
  const int r = ((int)blockIdx.x - J.first_block) * blockDim.x + threadIdx.x;
  if (r >= J.n) return;
  circuit_rank<kF32, kPhilox>(r, J.n, nullptr, J.cells, J.c0, J.nc, J.radiance, J.p, J.photo, J.max_events, J.st,
                              J.ev_count, J.slab_t, J.slab_p, J.error, J.counters);
}

template <int kRays, int kGeo>
cudaError_t trace_jobs_geo(const TraceJobs &jobs, cudaStream_t s) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_jobs_kernel<kRays, kGeo>, 128, 0);
  // resident blocks only (a persistent grid), fewer when there are fewer items than warps
  const long long resident = (long long)sms * (per_sm > 0 ? per_sm : 1);
  const long long needed = (jobs.total_items + kWarpsPerBlock - 1) / kWarpsPerBlock;
  const long long grid = needed < resident ? needed : resident;
  trace_jobs_kernel<kRays, kGeo><<<(int)grid, 128, 0, s>>>(jobs);
  return cudaGetLastError();
}

template <int kRays>
cudaError_t trace_jobs_rays(const TraceJobs &jobs, int geometry, cudaStream_t s) {
  switch (geometry) {
    case kGeoHalfBounds: return trace_jobs_geo<kRays, kGeoHalfBounds>(jobs, s);
    case kGeoWatertight: return trace_jobs_geo<kRays, kGeoWatertight>(jobs, s);
    case kGeoHalfBounds | kGeoWatertight: return trace_jobs_geo<kRays, kGeoHalfBounds | kGeoWatertight>(jobs, s);
    default: return trace_jobs_geo<kRays, kGeoReference>(jobs, s);
  }
}

}  // namespace

long long trace_job_items(int n_pix, int nc, int cw_log2) {
  const int cw = 1 << cw_log2, ppw = 32 >> cw_log2;
  return (long long)((n_pix + ppw - 1) / ppw) * ((nc + cw - 1) / cw);
}

cudaError_t launch_trace_jobs(const TraceJobs &jobs, int rays, int geometry, cudaStream_t s) {
  if (jobs.n_jobs <= 0 || jobs.total_items <= 0) return cudaSuccess;
  if (jobs.n_jobs > kMaxBatchJobs) return cudaErrorInvalidValue;
  return rays == 2 ? trace_jobs_rays<2>(jobs, geometry, s) : trace_jobs_rays<1>(jobs, geometry, s);
}

cudaError_t launch_circuit_jobs(const CircuitJob *jobs, int n_jobs, int total_blocks, bool fp32, bool philox,
                                cudaStream_t s) {
  if (n_jobs <= 0 || total_blocks <= 0) return cudaSuccess;
  if (n_jobs > kMaxBatchJobs) return cudaErrorInvalidValue;
  if (fp32 && philox)
    circuit_jobs_kernel<true, true><<<total_blocks, 128, 0, s>>>(jobs, n_jobs);
  else if (fp32)
    circuit_jobs_kernel<true, false><<<total_blocks, 128, 0, s>>>(jobs, n_jobs);
  else
    circuit_jobs_kernel<false, false><<<total_blocks, 128, 0, s>>>(jobs, n_jobs);
  return cudaGetLastError();
}

}  // namespace dvsgb
