// Device event readout of the GB300 DVS path: the reference's finite FIFO
// (EventReadout::submit/drain, src/event_readout.cpp:6-34) on the GPU.
//
//   1. Order: a stable LSD radix sort of the batch by (t, y, x) -- 8-bit
//      digits over the 30-bit (y, x) key, then over the 64 order-preserving
//      bits of t.  A pass whose digit is the same for every event (the high
//      bytes of t within a batch, the high byte of y) moves nothing and is
//      skipped on the device.
//   2. Completions: with bandwidth B the FIFO's serial recurrence
//      c_k = max(c_{k-1}, t_k) + 1/B (c_{-1} = the carried availability A)
//      equals the max-plus scan c_k = (k+1)/B + max(A, max_{j<=k} (t_j - j/B)):
//      a prefix maximum, exact, computed in parallel.  Delivery is c_k + latency.
//   3. Occupancy: at arrival k the queue holds the carried and the accepted
//      events delivered after t_k; both are sorted by delivery, so each
//      arrival finds its occupancy by binary search, and the peak is the
//      largest occupancy + 1.  When no arrival sees a full queue nothing is
//      dropped and steps 2-3 are the FIFO's result; otherwise one device
//      thread replays the batch serially with the drops (a loop bounded by
//      the batch size; nothing waits).
//   4. Release: events delivered by `now` leave in queue order (carried first)
//      into the output array; the rest stay in the pending ring buffer (device
//      memory, a power of two >= the capacity) for the next batch.
// Order, drops and peak are the serial FIFO's; delivery times are the same
// sums grouped as a scan (equal up to the rounding of the FP64 additions).
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.h"

namespace dvsgb {
namespace {

constexpr int kSortThreads = 256;
constexpr int kDigits = 256;
__device__ __forceinline__ double neg_inf() { return __longlong_as_double(0xfff0000000000000ll); }

__device__ __forceinline__ unsigned long long time_key(double t) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(t);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ unsigned digit_of(int pass, unsigned long long kt, unsigned kyx) {
  return pass < 4 ? (kyx >> (8 * pass)) & 0xffu : (unsigned)(kt >> (8 * (pass - 4))) & 0xffu;
}
// [begin, end) of block b's tile when n items are split over gridDim.x blocks.
__device__ __forceinline__ void tile_of(int n, int b, int &begin, int &end) {
  const int per = (n + (int)gridDim.x - 1) / (int)gridDim.x;
  begin = min(n, b * per);
  end = min(n, begin + per);
}
__device__ __forceinline__ unsigned long long ring_index(const ReadoutFifo &f, unsigned long long c) {
  return c & (f.ring_size - 1);
}

// ---- sort ---------------------------------------------------------------------------
__global__ void ro_keys_kernel(const DevEvent *events, const int32_t *count, ReadoutSort s) {
  const int n = *count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const DevEvent e = events[i];
    s.kt[0][i] = time_key(e.t);
    s.kyx[0][i] = ((unsigned)(uint16_t)e.y << 16) | (unsigned)(uint16_t)e.x;
    s.idx[0][i] = (unsigned)i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *s.cur = 0;
}

// Per block: the histogram of the pass's digit over its tile, digit-major
// (hist[d * grid + b]) for the exclusive scan.
__global__ void __launch_bounds__(kSortThreads) ro_hist_kernel(int pass, const int32_t *count, ReadoutSort s) {
  __shared__ unsigned h[kDigits];
  const int n = *count, cur = *s.cur;
  h[threadIdx.x] = 0;
  __syncthreads();
  int begin, end;
  tile_of(n, blockIdx.x, begin, end);
  for (int i = begin + threadIdx.x; i < end; i += blockDim.x)
    atomicAdd(&h[digit_of(pass, s.kt[cur][i], s.kyx[cur][i])], 1u);
  __syncthreads();
  s.hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// One block of 1024 threads: *skip = 1 when one digit holds all n keys (or
// n == 0), else the exclusive scan of the grid x 256 counts in place.
__global__ void __launch_bounds__(1024) ro_scan_kernel(int grid, const int32_t *count, ReadoutSort s) {
  __shared__ unsigned partial[1024];
  __shared__ int skip;
  const int n = *count, total = grid * kDigits;
  if (threadIdx.x == 0) skip = n == 0;
  __syncthreads();
  if (threadIdx.x < kDigits) {
    unsigned d_total = 0;
    for (int b = 0; b < grid; ++b) d_total += s.hist[threadIdx.x * grid + b];
    if (d_total == (unsigned)n) skip = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) *s.skip = skip;
  if (skip) return;  // block-uniform
  const int per = (total + (int)blockDim.x - 1) / (int)blockDim.x;
  const int begin = min(total, (int)threadIdx.x * per), end = min(total, begin + per);
  unsigned sum = 0;
  for (int i = begin; i < end; ++i) sum += s.hist[i];
  partial[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < (int)blockDim.x; off <<= 1) {  // inclusive scan of the partial sums
    const unsigned v = threadIdx.x >= (unsigned)off ? partial[threadIdx.x - off] : 0u;
    __syncthreads();
    partial[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned run = threadIdx.x ? partial[threadIdx.x - 1] : 0u;
  for (int i = begin; i < end; ++i) {
    const unsigned c = s.hist[i];
    s.hist[i] = run;
    run += c;
  }
}

// Stable scatter: each block walks its tile in rounds of 256 keys in order;
// a key's destination is its digit's offset for this block, plus the keys of
// its digit in earlier rounds, in earlier warps of its round and in earlier
// lanes of its warp.
__global__ void __launch_bounds__(kSortThreads) ro_scatter_kernel(int pass, const int32_t *count, ReadoutSort s) {
  __shared__ unsigned base[kDigits];
  __shared__ unsigned warp_count[kSortThreads / 32][kDigits];
  if (*s.skip) return;  // grid-uniform
  const int n = *count, cur = *s.cur;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  base[threadIdx.x] = s.hist[threadIdx.x * gridDim.x + blockIdx.x];
  int begin, end;
  tile_of(n, blockIdx.x, begin, end);
  for (int r0 = begin; r0 < end; r0 += kSortThreads) {  // block-uniform rounds
    for (int w = 0; w < kSortThreads / 32; ++w) warp_count[w][threadIdx.x] = 0;
    __syncthreads();
    const int i = r0 + (int)threadIdx.x;
    const bool live = i < end;
    unsigned long long kt = 0;
    unsigned kyx = 0, idx = 0, d = 0xffffffffu;  // dead lanes share a digit no key has
    if (live) {
      kt = s.kt[cur][i];
      kyx = s.kyx[cur][i];
      idx = s.idx[cur][i];
      d = digit_of(pass, kt, kyx);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned rank_in_warp = __popc(peers & ((1u << lane) - 1u));
    if (live && rank_in_warp == 0) warp_count[warp][d] = __popc(peers);
    __syncthreads();
    if (live) {
      unsigned before = 0;
      for (int w = 0; w < warp; ++w) before += warp_count[w][d];
      const unsigned dst = base[d] + before + rank_in_warp;
      s.kt[1 - cur][dst] = kt;
      s.kyx[1 - cur][dst] = kyx;
      s.idx[1 - cur][dst] = idx;
    }
    __syncthreads();
    unsigned round_total = 0;
    for (int w = 0; w < kSortThreads / 32; ++w) round_total += warp_count[w][threadIdx.x];
    base[threadIdx.x] += round_total;
    __syncthreads();
  }
}

__global__ void ro_flip_kernel(ReadoutSort s) {
  if (!*s.skip) *s.cur = 1 - *s.cur;
}

// ---- FIFO ---------------------------------------------------------------------------
// Carried entries (ring [head, tail)) delivered after t, by binary search.
__device__ __forceinline__ long long carried_after(const ReadoutFifo &f, unsigned long long head,
                                                   unsigned long long tail, double t) {
  unsigned long long lo = head, hi = tail;
  while (lo < hi) {
    const unsigned long long mid = lo + (hi - lo) / 2;
    if (f.ring[ring_index(f, mid)].t <= t) lo = mid + 1; else hi = mid;
  }
  return (long long)(tail - lo);
}

// Per block: the maximum of u_k = t_k - k/B over its tile.
__global__ void __launch_bounds__(256) ro_fifo_max_kernel(const DevEvent *events, const int32_t *count,
                                                           ReadoutSort s, ReadoutFifo f) {
  __shared__ double red[256];
  const int n = *count, cur = *s.cur;
  int begin, end;
  tile_of(n, blockIdx.x, begin, end);
  double m = neg_inf();
  for (int k = begin + threadIdx.x; k < end; k += blockDim.x)
    m = fmax(m, events[s.idx[cur][k]].t - (double)k * f.step);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int off = 128; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + off]);
    __syncthreads();
  }
  if (threadIdx.x == 0) f.block_max[blockIdx.x] = red[0];
}

// Per block: the prefix maximum from the carried availability and the earlier
// blocks' maxima, then the completion and delivery time of every arrival.
__global__ void __launch_bounds__(256) ro_fifo_scan_kernel(const DevEvent *events, const int32_t *count,
                                                            ReadoutSort s, ReadoutFifo f) {
  __shared__ double chunk[256];
  const int n = *count, cur = *s.cur;
  int begin, end;
  tile_of(n, blockIdx.x, begin, end);
  double carry = *f.available;
  for (int b = 0; b < (int)blockIdx.x; ++b) carry = fmax(carry, f.block_max[b]);
  for (int r0 = begin; r0 < end; r0 += blockDim.x) {  // block-uniform rounds
    const int k = r0 + (int)threadIdx.x;
    const bool live = k < end;
    chunk[threadIdx.x] = live ? events[s.idx[cur][k]].t - (double)k * f.step : neg_inf();
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {  // inclusive prefix maximum
      const double v = threadIdx.x >= (unsigned)off ? chunk[threadIdx.x - off] : neg_inf();
      __syncthreads();
      chunk[threadIdx.x] = fmax(chunk[threadIdx.x], v);
      __syncthreads();
    }
    if (live) {
      const double c = (double)(k + 1) * f.step + fmax(carry, chunk[threadIdx.x]);
      f.completion[k] = c;
      f.delivery[k] = c + f.latency;
    }
    carry = fmax(carry, chunk[blockDim.x - 1]);
    __syncthreads();
  }
}

// Occupancy at every arrival: the overflow flag and the batch's peak.
__global__ void ro_fifo_occupancy_kernel(const DevEvent *events, const int32_t *count, ReadoutSort s,
                                         ReadoutFifo f) {
  const int n = *count, cur = *s.cur;
  const unsigned long long head = *f.head, tail = *f.tail;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double t = events[s.idx[cur][k]].t;
    int lo = 0, hi = k;  // first j < k delivered after t (deliveries are nondecreasing)
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (f.delivery[mid] <= t) lo = mid + 1; else hi = mid;
    }
    const long long occ = carried_after(f, head, tail, t) + (k - lo);
    if (occ >= (long long)f.capacity) atomicOr(f.overflow, 1);
    atomicMax(f.peak_batch, (unsigned long long)(occ + 1));
  }
}

// One thread.  No FIFO delay: everything is released in order.  No overflow:
// the release plan (carried released, batch released, batch accepted), the
// availability and the peak.  Overflow: the serial FIFO with its drops
// (event_readout.cpp:13-30), writing the output and the ring directly.
__global__ void ro_fifo_commit_kernel(const DevEvent *events, const int32_t *count, ReadoutSort s, ReadoutFifo f,
                                      const double *now_at) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double now = *now_at;
  if (f.gate && *f.gate) {  // the batch failed: the FIFO neither takes nor releases anything
    f.plan[0] = -1;
    *f.out_count = 0;
    return;
  }
  const int n = *count, cur = *s.cur;
  unsigned long long head = *f.head, tail = *f.tail;
  if (f.step <= 0) {
    f.plan[0] = 0;
    f.plan[1] = n;
    f.plan[2] = n;
    *f.out_count = n;
    return;
  }
  if (!*f.overflow) {
    // An entry leaves when an arrival after it or `now` reaches its delivery
    // time; deliveries only grow along the queue and an event is delivered
    // after its own arrival, so both releases are prefixes at the threshold
    // max(now, last arrival).
    const double until = n > 0 ? fmax(now, events[s.idx[cur][n - 1]].t) : now;
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (f.delivery[mid] <= until) lo = mid + 1; else hi = mid;
    }
    const long long carried_out = (long long)(tail - head) - carried_after(f, head, tail, until);
    if ((long long)(tail - head) - carried_out + (n - lo) > (long long)f.ring_size) {
      *f.status = 1;  // the pending events would not fit the ring (capacity above its size)
      f.plan[0] = -1;
      *f.out_count = 0;
      return;
    }
    f.plan[0] = carried_out;
    f.plan[1] = lo;
    f.plan[2] = n;
    *f.out_count = (int32_t)(carried_out + lo);
    if (n > 0) *f.available = f.completion[n - 1];
    if (*f.peak_batch > *f.peak) *f.peak = *f.peak_batch;
    return;
  }
  int out = 0;
  double available = *f.available;
  unsigned long long peak = *f.peak, dropped = *f.dropped;
  for (int k = 0; k < n; ++k) {
    const DevEvent e = events[s.idx[cur][k]];
    while (head < tail && f.ring[ring_index(f, head)].t <= e.t) f.out[out++] = f.ring[ring_index(f, head++)];
    if (tail - head >= f.capacity) {
      ++dropped;
      continue;
    }
    if (tail - head >= f.ring_size) {  // a capacity above the ring's size: stop, report, keep the ring intact
      *f.status = 1;
      break;
    }
    const double completed = fmax(available, e.t) + f.step;
    available = completed;
    DevEvent d = e;
    d.t = completed + f.latency;
    f.ring[ring_index(f, tail++)] = d;
    if (tail - head > peak) peak = tail - head;
  }
  while (head < tail && f.ring[ring_index(f, head)].t <= now) f.out[out++] = f.ring[ring_index(f, head++)];
  *f.available = available;
  *f.peak = peak;
  *f.dropped = dropped;
  *f.head = head;
  *f.tail = tail;
  *f.out_count = out;
  f.plan[0] = -1;  // done serially
}

// The plan's copies: released carried entries and batch events to the output
// (queue order), the batch's later deliveries to the ring.
__global__ void ro_fifo_release_kernel(const DevEvent *events, ReadoutSort s, ReadoutFifo f) {
  const long long carried_out = f.plan[0], batch_out = f.plan[1], accepted = f.plan[2];
  if (carried_out < 0) return;
  const int cur = *s.cur;
  const unsigned long long head = *f.head, tail = *f.tail;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < carried_out + accepted; i += stride) {
    if (i < carried_out) {
      f.out[i] = f.ring[ring_index(f, head + i)];
    } else {
      const long long k = i - carried_out;
      DevEvent d = events[s.idx[cur][k]];
      if (f.step > 0) d.t = f.delivery[k];
      if (k < batch_out) f.out[carried_out + k] = d;
      else f.ring[ring_index(f, tail + (k - batch_out))] = d;
    }
  }
}

__global__ void ro_fifo_advance_kernel(ReadoutFifo f) {
  if (f.plan[0] < 0) return;
  *f.head += (unsigned long long)f.plan[0];
  *f.tail += (unsigned long long)(f.plan[2] - f.plan[1]);
}

// drain (event_readout.cpp:31-34): every pending entry, in order.
__global__ void ro_drain_kernel(ReadoutFifo f) {
  const unsigned long long head = *f.head, tail = *f.tail;
  for (unsigned long long i = head + blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < tail;
       i += (unsigned long long)gridDim.x * blockDim.x)
    f.out[i - head] = f.ring[ring_index(f, i)];
}
__global__ void ro_drain_commit_kernel(ReadoutFifo f) {
  *f.out_count = (int32_t)(*f.tail - *f.head);
  *f.head = *f.tail;
}

}  // namespace

cudaError_t launch_readout_submit(const DevEvent *events, const int32_t *count, ReadoutSort s, ReadoutFifo f,
                                  const double *now, int grid, cudaStream_t st) {
  ro_keys_kernel<<<grid, 256, 0, st>>>(events, count, s);
  for (int pass = 0; pass < 12; ++pass) {
    ro_hist_kernel<<<grid, kSortThreads, 0, st>>>(pass, count, s);
    ro_scan_kernel<<<1, 1024, 0, st>>>(grid, count, s);
    ro_scatter_kernel<<<grid, kSortThreads, 0, st>>>(pass, count, s);
    ro_flip_kernel<<<1, 1, 0, st>>>(s);
  }
  cudaError_t e = cudaMemsetAsync(f.overflow, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(f.peak_batch, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  if (f.step > 0) {
    ro_fifo_max_kernel<<<grid, 256, 0, st>>>(events, count, s, f);
    ro_fifo_scan_kernel<<<grid, 256, 0, st>>>(events, count, s, f);
    ro_fifo_occupancy_kernel<<<grid, 256, 0, st>>>(events, count, s, f);
  }
  ro_fifo_commit_kernel<<<1, 32, 0, st>>>(events, count, s, f, now);
  ro_fifo_release_kernel<<<grid, 256, 0, st>>>(events, s, f);
  ro_fifo_advance_kernel<<<1, 1, 0, st>>>(f);
  return cudaGetLastError();
}

cudaError_t launch_readout_drain(ReadoutFifo f, int grid, cudaStream_t st) {
  ro_drain_kernel<<<grid, 256, 0, st>>>(f);
  ro_drain_commit_kernel<<<1, 1, 0, st>>>(f);
  return cudaGetLastError();
}

}  // namespace dvsgb
