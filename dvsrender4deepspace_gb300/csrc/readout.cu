// Device event readout of the GB300 DVS path: the reference's finite FIFO
// (EventReadout::submit/drain, src/event_readout.cpp:6-34) on the GPU.
//
//   1. Order: a stable LSD radix sort of the batch by (t, y, x) -- 8-bit
//      digits over the 32-bit (y, x) key, then over the 64 order-preserving
//      bits of t.  The key kernel ORs every key against the first event's, so
//      the bits that vary within the batch are known before any pass.  Bits
//      that never vary decide nothing: when the varying ranges of t, y and x
//      fit 64 bits (a 64 us batch of a 1280x720 sensor: 38 + 10 + 11), they
//      are packed into one key and the (y, x) key is not moved at all; a
//      digit that is the same for every key makes its pass do nothing; and
//      every kernel derives from the same words which of the two key buffers
//      its pass reads.  Per active pass: a digit histogram per block, one
//      block per digit scanning that digit's counts over the blocks, and a
//      stable scatter whose blocks add the digits' totals.
//   2. Completions: with bandwidth B the FIFO's serial recurrence
//      c_k = max(c_{k-1}, t_k) + 1/B (c_{-1} = the carried availability A)
//      equals the max-plus scan c_k = (k+1)/B + max(A, max_{j<=k} (t_j - j/B)):
//      a prefix maximum, exact, computed in parallel from the sorted keys.
//      Delivery is c_k + latency.
//   3. Occupancy: at arrival k the queue holds the carried and the accepted
//      events delivered after t_k; both are sorted by delivery, so each
//      arrival finds its occupancy by a search (galloping back from k: a short
//      queue costs a load or two), and the peak is the largest occupancy + 1.
//      When no arrival sees a full queue nothing is dropped and steps 2-3 are
//      the FIFO's result; otherwise one device thread replays the batch
//      serially with the drops (a loop bounded by the batch size; nothing waits).
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
constexpr int kPasses = 12;          // 4 bytes of the (y, x) key, then 8 of the time key
constexpr int kScanThreads = 1024;   // one thread per sort block in the per-digit scan
constexpr unsigned kFull = 0xffffffffu;

// Order-preserving bits of a double (the sort key of t) and back.
__device__ __forceinline__ unsigned long long time_key(double t) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(t);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_time(unsigned long long k) {
  const unsigned long long u = (k & 0x8000000000000000ull) ? (k ^ 0x8000000000000000ull) : ~k;
  return __longlong_as_double((long long)u);
}
__device__ __forceinline__ unsigned yx_key(const DevEvent &e) {
  return ((unsigned)(uint16_t)e.y << 16) | (unsigned)(uint16_t)e.x;
}
// Key buffer b (0 or 1), chosen by a select: indexing the parameter's
// arrays with a run-time value would copy them to the stack.
__device__ __forceinline__ unsigned long long *kt_of(const ReadoutSort &s, int b) { return b ? s.kt[1] : s.kt[0]; }
__device__ __forceinline__ unsigned *kyx_of(const ReadoutSort &s, int b) { return b ? s.kyx[1] : s.kyx[0]; }
__device__ __forceinline__ unsigned *idx_of(const ReadoutSort &s, int b) { return b ? s.idx[1] : s.idx[0]; }
// The sort key of a batch.  Bits that are the same for every event of the
// batch decide no comparison, so dropping them keeps the (t, y, x) order:
// when the varying ranges of the time key (its low bt bits: all higher bits
// are the first event's), of y (low by bits) and of x (low bx bits) fit 64
// bits together, the batch sorts on one packed key t' << (by + bx) | y' << bx
// | x' in the time-key buffers (passes 4-11, the (y, x) buffers unused);
// otherwise on the time key and the (y, x) key (passes 0-3 over (y, x), 4-11
// over t).  Every kernel derives the same layout from `varying`.
__device__ __forceinline__ int bits_of(unsigned long long v) { return v ? 64 - __clzll((long long)v) : 0; }
__device__ __forceinline__ unsigned long long low_mask(int b) { return b >= 64 ? ~0ull : (1ull << b) - 1ull; }
struct KeyLayout {
  bool packed;
  int xbits, shift;              // packed: bits of x', and of y' and x' together
  unsigned long long tmask;      // packed: the varying range of the time key
  unsigned long long thigh;      // packed: the time key's bits above it (the first event's)
  unsigned xmask, ymask;
  unsigned long long vary_t;     // varying bits of the time-key buffers' keys (packed: of the packed key)
  unsigned long long vary_yx;    // varying bits of the (y, x) keys (0 when packed)
  unsigned mask;                 // bit p: pass p's digit differs between events
};
__device__ __forceinline__ unsigned long long pack_key(const KeyLayout &L, unsigned long long kt, unsigned kyx) {
  return ((kt & L.tmask) << L.shift) | ((unsigned long long)((kyx >> 16) & L.ymask) << L.xbits) | (kyx & L.xmask);
}
__device__ __forceinline__ KeyLayout key_layout(const ReadoutSort &s) {
  const unsigned long long vt = s.varying[0], vyx = s.varying[1];
  const int bt = bits_of(vt), bx = bits_of(vyx & 0xffffull), by = bits_of(vyx >> 16);
  KeyLayout L;
  L.packed = bt + bx + by <= 64;
  L.xbits = bx;
  L.shift = bx + by;
  L.tmask = low_mask(bt);
  L.thigh = s.varying[2] & ~L.tmask;
  L.xmask = (unsigned)low_mask(bx);
  L.ymask = (unsigned)low_mask(by);
  L.vary_t = L.packed ? pack_key(L, vt, (unsigned)vyx) : vt;
  L.vary_yx = L.packed ? 0ull : vyx;
  unsigned m = 0;
#pragma unroll
  for (int p = 0; p < 4; ++p)
    if ((L.vary_yx >> (8 * p)) & 0xffull) m |= 1u << p;
#pragma unroll
  for (int p = 0; p < 8; ++p)
    if ((L.vary_t >> (8 * p)) & 0xffull) m |= 1u << (4 + p);
  L.mask = m;
  return L;
}
// The time key of a sorted key.
__device__ __forceinline__ unsigned long long time_key_of(const KeyLayout &L, unsigned long long k) {
  return L.packed ? L.thigh | ((k >> L.shift) & L.tmask) : k;
}
// The key buffer pass p reads: each active pass before it moved the keys once.
__device__ __forceinline__ int buffer_before(unsigned mask, int pass) { return __popc(mask & ((1u << pass) - 1u)) & 1; }
__device__ __forceinline__ int sorted_buffer(const KeyLayout &L) { return __popc(L.mask) & 1; }
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
// First j in [0, k) with a[j] > t (k if none), for a nondecreasing a: galloping
// back from k, then a binary search of the last bracket.
__device__ __forceinline__ long long first_after(const double *a, long long k, double t) {
  long long lo = 0, hi = k, step = 1;
  while (true) {
    const long long j = hi - step;
    if (j < 0) break;             // the answer is in [0, hi]
    if (a[j] > t) {
      hi = j;                     // a[hi..k) > t
      step <<= 1;
    } else {
      lo = j + 1;                 // the answer is in [j + 1, hi]
      break;
    }
  }
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (a[mid] <= t) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// ---- sort ---------------------------------------------------------------------------
// Keys of the batch in arrival order, the OR of every key against the first
// event's (varying[0..1], zeroed before the launch) and the first event's time
// key (varying[2]).  256 threads.
__global__ void __launch_bounds__(256) ro_keys_kernel(const DevEvent *events, const int32_t *count, ReadoutSort s) {
  __shared__ unsigned long long red[256 / 32][2];
  const int n = *count;
  if (n <= 0) return;  // grid-uniform
  const DevEvent first = events[0];
  const unsigned long long kt0 = time_key(first.t);
  const unsigned kyx0 = yx_key(first);
  unsigned long long dt = 0;
  unsigned dyx = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const DevEvent e = events[i];
    const unsigned long long kt = time_key(e.t);
    const unsigned kyx = yx_key(e);
    s.kt[0][i] = kt;
    s.kyx[0][i] = kyx;
    s.idx[0][i] = (unsigned)i;
    dt |= kt ^ kt0;
    dyx |= kyx ^ kyx0;
  }
  const unsigned lo = __reduce_or_sync(kFull, (unsigned)dt), hi = __reduce_or_sync(kFull, (unsigned)(dt >> 32));
  const unsigned yx = __reduce_or_sync(kFull, dyx);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[warp][0] = ((unsigned long long)hi << 32) | lo;
    red[warp][1] = yx;
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0) s.varying[2] = kt0;
  if (threadIdx.x == 0) {
    unsigned long long a = 0, b = 0;
    for (int w = 0; w < 256 / 32; ++w) {
      a |= red[w][0];
      b |= red[w][1];
    }
    if (a) atomicOr(s.varying, a);
    if (b) atomicOr(s.varying + 1, b);
  }
}

// Packed layout: the packed key replaces the time key, in place.
__global__ void __launch_bounds__(256) ro_pack_kernel(const int32_t *count, ReadoutSort s) {
  const KeyLayout L = key_layout(s);
  if (!L.packed) return;  // grid-uniform
  const int n = *count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s.kt[0][i] = pack_key(L, s.kt[0][i], s.kyx[0][i]);
}

// A pass whose digit takes few values (at most 3 varying bits: <= 8 values,
// e.g. the high byte of y) counts with lanes of the same digit adding once
// (match_any), so they do not serialize on one shared counter; other passes
// count with one shared atomic per key.
__device__ __forceinline__ bool few_digit_values(const KeyLayout &L, int pass) {
  const unsigned long long v = pass < 4 ? L.vary_yx >> (8 * pass) : L.vary_t >> (8 * (pass - 4));
  return __popcll(v & 0xffull) <= 3;
}
// Adds one key of digit d (live) to h; called by every lane of the warp.
__device__ __forceinline__ void count_digit(unsigned *h, unsigned d, bool live, bool aggregate) {
  if (aggregate) {
    const unsigned peers = __match_any_sync(kFull, live ? d : kFull);
    if (live && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&h[d], (unsigned)__popc(peers));
  } else if (live) {
    atomicAdd(&h[d], 1u);
  }
}
// Exclusive scan of one value per thread over a block of 256 threads.
__device__ __forceinline__ unsigned block_exclusive_scan_256(unsigned v, unsigned *warp_total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned incl = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned u = __shfl_up_sync(kFull, incl, off);
    if (lane >= off) incl += u;
  }
  if (lane == 31) warp_total[warp] = incl;
  __syncthreads();
  unsigned excl = incl - v;
  for (int w = 0; w < warp; ++w) excl += warp_total[w];
  __syncthreads();  // warp_total is free for the next scan
  return excl;
}

// Per block: the histogram of the pass's digit over its tile, digit-major
// (hist[d * grid + b]).
__global__ void __launch_bounds__(kSortThreads) ro_hist_kernel(int pass, const int32_t *count, ReadoutSort s) {
  constexpr int kPer = 4;  // keys per thread and round: their loads are in flight together
  __shared__ unsigned h[kDigits];
  const KeyLayout L = key_layout(s);
  if (!((L.mask >> pass) & 1u)) return;  // grid-uniform: the digit is every key's
  const int n = *count, cur = buffer_before(L.mask, pass);
  const bool aggregate = few_digit_values(L, pass);
  const unsigned long long *kt = kt_of(s, cur);
  const unsigned *kyx = kyx_of(s, cur);
  h[threadIdx.x] = 0;
  __syncthreads();
  int begin, end;
  tile_of(n, blockIdx.x, begin, end);
  for (int r0 = begin; r0 < end; r0 += kPer * kSortThreads) {  // block-uniform rounds: every lane reaches the match
    unsigned d[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int i = r0 + j * kSortThreads + (int)threadIdx.x;
      d[j] = kFull;
      if (i < end) d[j] = pass < 4 ? (kyx[i] >> (8 * pass)) & 0xffu : (unsigned)(kt[i] >> (8 * (pass - 4))) & 0xffu;
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) count_digit(h, d[j], d[j] != kFull, aggregate);
  }
  __syncthreads();
  s.hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Block d (one per digit, grid <= 1024 sort blocks, one thread each): the
// exclusive scan of digit d's counts over the blocks, in place, and the
// digit's total.
__global__ void __launch_bounds__(kScanThreads) ro_scan_kernel(int pass, int grid, ReadoutSort s) {
  __shared__ unsigned warp_sum[kScanThreads / 32];
  if (!((key_layout(s).mask >> pass) & 1u)) return;  // grid-uniform
  const int b = threadIdx.x, lane = b & 31, warp = b >> 5;
  unsigned *row = s.hist + (size_t)blockIdx.x * grid;
  const unsigned v = b < grid ? row[b] : 0u;
  unsigned incl = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned u = __shfl_up_sync(kFull, incl, off);
    if (lane >= off) incl += u;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  if (warp == 0) {  // kScanThreads / 32 == 32 warp sums, one per lane
    const unsigned ws = warp_sum[lane];
    unsigned wi = ws;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned u = __shfl_up_sync(kFull, wi, off);
      if (lane >= off) wi += u;
    }
    warp_sum[lane] = wi - ws;
  }
  __syncthreads();
  if (b < grid) row[b] = warp_sum[warp] + incl - v;
  if (b == kScanThreads - 1) s.digit_total[blockIdx.x] = warp_sum[warp] + incl;
}

// Stable scatter in tiles of 1024 keys (4 per thread, in arrival order).  A
// key's place in the output is the keys of smaller digits (the exclusive scan
// of the digit totals), plus its digit's keys in earlier blocks and earlier
// tiles of its block, plus its rank among its digit's keys in the tile.  The
// tile is first ordered by digit in shared memory -- rank = the digit's
// offset in the tile + its keys in earlier quarters, warps and lanes -- and
// then written out in that order, so a digit's keys of one tile land in one
// run of consecutive addresses instead of one scattered store each.
constexpr int kTileKeys = 4 * kSortThreads;
__global__ void __launch_bounds__(kSortThreads) ro_scatter_kernel(int pass, const int32_t *count, ReadoutSort s) {
  constexpr int kWarps = kSortThreads / 32, kPer = kTileKeys / kSortThreads;
  __shared__ unsigned base[kDigits], tcount[kDigits], toff[kDigits], run[kDigits];
  __shared__ unsigned warp_total[kWarps];
  __shared__ unsigned warp_count[2][kWarps][kDigits];
  __shared__ unsigned long long skt[kTileKeys];
  __shared__ unsigned skyx[kTileKeys], sidx[kTileKeys];
  const KeyLayout L = key_layout(s);
  if (!((L.mask >> pass) & 1u)) return;  // grid-uniform
  const int n = *count, cur = buffer_before(L.mask, pass);
  const bool aggregate = few_digit_values(L, pass), yx = !L.packed;  // packed: no (y, x) keys to move
  const unsigned long long *kt_in = kt_of(s, cur);
  const unsigned *kyx_in = kyx_of(s, cur), *idx_in = idx_of(s, cur);
  unsigned long long *kt_out = kt_of(s, 1 - cur);
  unsigned *kyx_out = kyx_of(s, 1 - cur), *idx_out = idx_of(s, 1 - cur);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  base[t] = block_exclusive_scan_256(s.digit_total[t], warp_total) + s.hist[t * gridDim.x + blockIdx.x];
  int begin, end;
  tile_of(n, blockIdx.x, begin, end);
  for (int c0 = begin; c0 < end; c0 += kTileKeys) {  // block-uniform tiles
    const int tn = min(kTileKeys, end - c0);
    unsigned long long k_t[kPer];
    unsigned k_yx[kPer], k_i[kPer], dg[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int q = j * kSortThreads + t;
      k_t[j] = 0;
      k_yx[j] = 0;
      k_i[j] = 0;
      dg[j] = kFull;  // no key
      if (q < tn) {
        k_t[j] = kt_in[c0 + q];
        if (yx) k_yx[j] = kyx_in[c0 + q];
        k_i[j] = idx_in[c0 + q];
        dg[j] = digit_of(pass, k_t[j], k_yx[j]);
      }
    }
    tcount[t] = 0;
    run[t] = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) warp_count[0][w][t] = 0;
    __syncthreads();  // also publishes base[] of the prologue or the previous tile
#pragma unroll
    for (int j = 0; j < kPer; ++j) count_digit(tcount, dg[j], dg[j] != kFull, aggregate);
    __syncthreads();
    const unsigned my_count = tcount[t];
    toff[t] = block_exclusive_scan_256(my_count, warp_total);
    __syncthreads();
    int buf = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) {  // quarters of the tile in arrival order
      const unsigned d = dg[j];
      const bool live = d != kFull;
      const unsigned peers = __match_any_sync(kFull, d);
      const unsigned rank_in_warp = __popc(peers & ((1u << lane) - 1u));
      if (live && rank_in_warp == 0) warp_count[buf][warp][d] = __popc(peers);
      __syncthreads();  // the quarter's counts are visible
      if (live) {
        unsigned before = 0;
        for (int w = 0; w < warp; ++w) before += warp_count[buf][w][d];
        const unsigned local = toff[d] + run[d] + before + rank_in_warp;
        skt[local] = k_t[j];
        if (yx) skyx[local] = k_yx[j];
        sidx[local] = k_i[j];
      }
      unsigned quarter_total = 0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        quarter_total += warp_count[buf][w][t];
        warp_count[buf ^ 1][w][t] = 0;  // the next quarter's counts
      }
      __syncthreads();  // every thread has read run[] and the quarter's counts; the keys are in place
      run[t] += quarter_total;
      buf ^= 1;
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) {  // out in digit order: runs of consecutive addresses
      const int q = j * kSortThreads + t;
      if (q < tn) {
        const unsigned long long a = skt[q];
        const unsigned b = yx ? skyx[q] : 0u;
        const unsigned d = digit_of(pass, a, b);
        const unsigned g = base[d] + (unsigned)q - toff[d];
        kt_out[g] = a;
        if (yx) kyx_out[g] = b;
        idx_out[g] = sidx[q];
      }
    }
    __syncthreads();  // every thread has read base[], toff[] and the staged keys
    base[t] += my_count;
  }
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

// The prefix maxima of the FIFO scan run on the order-preserving keys of the
// FP64 values (integer maxima: GB300's FP64 pipe is narrow); only u_k and the
// completion sums are FP64 arithmetic.  Key 0 is below every key of a number.
__device__ __forceinline__ unsigned long long u64_max(unsigned long long a, unsigned long long b) { return a > b ? a : b; }
__device__ __forceinline__ unsigned long long warp_max_key(unsigned long long v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = u64_max(v, __shfl_xor_sync(kFull, v, off));
  return v;
}
// Key of u_k = t_k - k/B, t_k from the sorted key.
__device__ __forceinline__ unsigned long long slack_key(const KeyLayout &L, unsigned long long key, int k, double step) {
  return time_key(key_time(time_key_of(L, key)) - (double)k * step);
}

// Per block: the maximum of u_k over its tile.
__global__ void __launch_bounds__(256) ro_fifo_max_kernel(const int32_t *count, ReadoutSort s, ReadoutFifo f) {
  __shared__ unsigned long long red[256 / 32];
  const KeyLayout L = key_layout(s);
  const int n = *count, cur = sorted_buffer(L);
  const unsigned long long *kt = kt_of(s, cur);
  int begin, end;
  tile_of(n, blockIdx.x, begin, end);
  unsigned long long m = 0;
  for (int k = begin + threadIdx.x; k < end; k += blockDim.x) m = u64_max(m, slack_key(L, kt[k], k, f.step));
  m = warp_max_key(m);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = red[0];
    for (int w = 1; w < 256 / 32; ++w) b = u64_max(b, red[w]);
    f.block_max[blockIdx.x] = b;
  }
}

// Per block: the prefix maximum from the carried availability and the earlier
// blocks' maxima, then the completion and delivery time of every arrival.
__global__ void __launch_bounds__(256) ro_fifo_scan_kernel(const int32_t *count, ReadoutSort s, ReadoutFifo f) {
  constexpr int kWarps = 256 / 32;
  __shared__ unsigned long long wmax[kWarps];
  __shared__ unsigned long long carry_in;
  const KeyLayout L = key_layout(s);
  const int n = *count, cur = sorted_buffer(L);
  const unsigned long long *kt = kt_of(s, cur);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int begin, end;
  tile_of(n, blockIdx.x, begin, end);
  unsigned long long c = threadIdx.x == 0 ? time_key(*f.available) : 0ull;
  for (int b = threadIdx.x; b < (int)blockIdx.x; b += blockDim.x) c = u64_max(c, f.block_max[b]);
  c = warp_max_key(c);
  if (lane == 0) wmax[warp] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = wmax[0];
    for (int w = 1; w < kWarps; ++w) m = u64_max(m, wmax[w]);
    carry_in = m;
  }
  __syncthreads();
  unsigned long long carry = carry_in;
  for (int r0 = begin; r0 < end; r0 += blockDim.x) {  // block-uniform rounds
    const int k = r0 + (int)threadIdx.x;
    const bool live = k < end;
    unsigned long long incl = live ? slack_key(L, kt[k], k, f.step) : 0ull;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {  // inclusive prefix maximum within the warp
      const unsigned long long v = __shfl_up_sync(kFull, incl, off);
      if (lane >= off) incl = u64_max(incl, v);
    }
    if (lane == 31) wmax[warp] = incl;
    __syncthreads();
    unsigned long long prior = carry;
    for (int w = 0; w < warp; ++w) prior = u64_max(prior, wmax[w]);
    if (live) {
      const double cc = (double)(k + 1) * f.step + key_time(u64_max(prior, incl));
      f.completion[k] = cc;
      f.delivery[k] = cc + f.latency;
    }
    for (int w = 0; w < kWarps; ++w) carry = u64_max(carry, wmax[w]);
    __syncthreads();  // wmax is rewritten by the next round
  }
}

// Occupancy at every arrival: the overflow flag and the batch's peak, reduced
// per warp and per block first (one atomic per block, not per event).
__global__ void __launch_bounds__(256) ro_fifo_occupancy_kernel(const int32_t *count, ReadoutSort s, ReadoutFifo f) {
  __shared__ unsigned red_peak[256 / 32];
  __shared__ int red_over[256 / 32];
  const KeyLayout L = key_layout(s);
  const int n = *count, cur = sorted_buffer(L);
  const unsigned long long *kt = kt_of(s, cur);
  const unsigned long long head = *f.head, tail = *f.tail;
  // occupancy + 1 <= ring entries (< 2^25) + batch events (< 2^31): fits 32 bits
  unsigned peak = 0;
  int over = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double t = key_time(time_key_of(L, kt[k]));
    const long long lo = first_after(f.delivery, k, t);  // earlier arrivals still queued at t: [lo, k)
    const long long occ = carried_after(f, head, tail, t) + (k - lo);
    over |= occ >= (long long)f.capacity;
    peak = max(peak, (unsigned)(occ + 1));
  }
  peak = __reduce_max_sync(kFull, peak);
  over = __any_sync(kFull, over);
  if ((threadIdx.x & 31) == 0) {
    red_peak[threadIdx.x >> 5] = peak;
    red_over[threadIdx.x >> 5] = over;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned p = 0;
    int o = 0;
    for (int w = 0; w < 256 / 32; ++w) {
      p = max(p, red_peak[w]);
      o |= red_over[w];
    }
    if (o) atomicOr(f.overflow, 1);
    if (p) atomicMax(f.peak_batch, (unsigned long long)p);
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
  const KeyLayout L = key_layout(s);
  const int n = *count, cur = sorted_buffer(L);
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
    const double until = n > 0 ? fmax(now, key_time(time_key_of(L, kt_of(s, cur)[n - 1]))) : now;
    const long long lo = first_after(f.delivery, n, until);
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
    const DevEvent e = events[idx_of(s, cur)[k]];
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
  const int cur = sorted_buffer(key_layout(s));
  const unsigned long long head = *f.head, tail = *f.tail;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < carried_out + accepted; i += stride) {
    if (i < carried_out) {
      f.out[i] = f.ring[ring_index(f, head + i)];
    } else {
      const long long k = i - carried_out;
      DevEvent d = events[idx_of(s, cur)[k]];
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

int readout_submit_launches(bool delayed) { return 2 + kPasses * 3 + (delayed ? 3 : 0) + 3; }

cudaError_t launch_readout_submit(const DevEvent *events, const int32_t *count, ReadoutSort s, ReadoutFifo f,
                                  const double *now, int grid, cudaStream_t st) {
  if (grid < 1 || grid > kScanThreads) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(s.varying, 0, 3 * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  ro_keys_kernel<<<grid, 256, 0, st>>>(events, count, s);
  ro_pack_kernel<<<grid, 256, 0, st>>>(count, s);
  for (int pass = 0; pass < kPasses; ++pass) {
    ro_hist_kernel<<<grid, kSortThreads, 0, st>>>(pass, count, s);
    ro_scan_kernel<<<kDigits, kScanThreads, 0, st>>>(pass, grid, s);
    ro_scatter_kernel<<<grid, kSortThreads, 0, st>>>(pass, count, s);
  }
  e = cudaMemsetAsync(f.overflow, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(f.peak_batch, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  if (f.step > 0) {
    ro_fifo_max_kernel<<<grid, 256, 0, st>>>(count, s, f);
    ro_fifo_scan_kernel<<<grid, 256, 0, st>>>(count, s, f);
    ro_fifo_occupancy_kernel<<<grid, 256, 0, st>>>(count, s, f);
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
