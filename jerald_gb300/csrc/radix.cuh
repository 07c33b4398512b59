// Stable least-significant-digit radix sort of (uint32 key, int32 value)
// pairs on sm_103a: the sort by integer cell key that the sorted paint uses.
//
// Each pass orders the pairs by `bits` (<= 9) key bits starting at `shift`,
// keeping the order of equal digits, so after the passes over all key bits
// the pairs are in key order with ties in input order (numpy's
// argsort(kind="stable")).  A pass is three steps:
//   1. radix_count_kernel: per tile of 4096 pairs, a digit histogram
//      (warp-aggregated shared-memory counts), stored digit-major,
//      counts[d * ntiles + tile];
//   2. scan_*: exclusive scan of that array, so counts[d * ntiles + tile]
//      becomes the first output slot of digit d in tile `tile`;
//   3. radix_scatter_kernel: each warp ranks its contiguous 512 pairs in
//      element order (__match_any_sync per 32-pair round plus warp-private
//      digit counters), the tile orders its pairs by digit in shared memory,
//      and writes them back with consecutive threads on consecutive slots.
// Every step reads and writes only within its buffers: no waits, no
// cross-CTA flags.
#pragma once

#include "common.cuh"

namespace jld {

constexpr int kRadixThreads = 256;
constexpr int kRadixWarps = kRadixThreads / 32;
constexpr int kRadixItems = 16;                        // per thread and pass
constexpr int kRadixTile = kRadixThreads * kRadixItems;  // 4096 pairs per tile
constexpr int kRadixWarpSpan = 32 * kRadixItems;         // 512 pairs per warp
constexpr int kRadixMaxBits = 9;
constexpr int kRadixMaxBuckets = 1 << kRadixMaxBits;
constexpr int kScanItems = 16;
constexpr int kScanChunk = kRadixThreads * kScanItems;  // 4096 counts per scan block

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Step 1: digit histogram of one tile, stored digit-major.
__global__ void __launch_bounds__(kRadixThreads)
radix_count_kernel(const uint32_t* __restrict__ keys, int64_t n, int shift, int bits, int ntiles,
                   uint32_t* __restrict__ counts) {
  __shared__ uint32_t h[kRadixMaxBuckets];
  const int nb = 1 << bits;
  const uint32_t mask = (uint32_t)nb - 1u;
  for (int i = threadIdx.x; i < nb; i += kRadixThreads) h[i] = 0u;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t base = (int64_t)blockIdx.x * kRadixTile;
#pragma unroll 4
  for (int r = 0; r < kRadixItems; ++r) {
    const int64_t e = base + (int64_t)r * kRadixThreads + threadIdx.x;
    const bool live = e < n;
    const uint32_t d = live ? (__ldg(keys + e) >> shift) & mask : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    if (live && lane == __ffs(peers) - 1) atomicAdd(&h[d], (uint32_t)__popc(peers));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += kRadixThreads) counts[(int64_t)i * ntiles + blockIdx.x] = h[i];
}

// Block-wide exclusive scan of one value per thread (256 threads); returns
// the thread's exclusive prefix, *total gets the block sum.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot, uint32_t* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  uint32_t before = 0, all = 0;
#pragma unroll
  for (int i = 0; i < kRadixWarps; ++i) {
    const uint32_t t = warp_tot[i];
    if (i < w) before += t;
    all += t;
  }
  __syncthreads();
  *total = all;
  return before + x - v;
}

// Step 2a: sum of each 4096-count chunk.
__global__ void __launch_bounds__(kRadixThreads)
scan_reduce_kernel(const uint32_t* __restrict__ a, int64_t m, uint32_t* __restrict__ part) {
  __shared__ uint32_t wt[kRadixWarps];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < m) s += a[base + i];
  uint32_t tot;
  block_exclusive_scan(s, wt, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// Step 2b: exclusive scan of the chunk sums (one block, sequential over
// groups of 256).
__global__ void __launch_bounds__(kRadixThreads)
scan_part_kernel(uint32_t* __restrict__ part, int64_t nparts) {
  __shared__ uint32_t wt[kRadixWarps];
  uint32_t carry = 0;
  for (int64_t b = 0; b < nparts; b += kRadixThreads) {
    const int64_t i = b + threadIdx.x;
    const uint32_t v = i < nparts ? part[i] : 0u;
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan(v, wt, &tot);
    if (i < nparts) part[i] = carry + ex;
    carry += tot;
  }
}

// Step 2c: exclusive scan of each chunk in place, offset by its chunk prefix.
__global__ void __launch_bounds__(kRadixThreads)
scan_apply_kernel(uint32_t* __restrict__ a, int64_t m, const uint32_t* __restrict__ part) {
  __shared__ uint32_t wt[kRadixWarps];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = base + i < m ? a[base + i] : 0u;
    s += v[i];
  }
  uint32_t tot;
  uint32_t run = block_exclusive_scan(s, wt, &tot) + part[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < m) a[base + i] = run;
    run += v[i];
  }
}

// Step 3: stable scatter of one tile by digit.
__global__ void __launch_bounds__(kRadixThreads)
radix_scatter_kernel(const uint32_t* __restrict__ kin, const int32_t* __restrict__ vin, int64_t n, int shift,
                     int bits, int ntiles, const uint32_t* __restrict__ offsets, uint32_t* __restrict__ kout,
                     int32_t* __restrict__ vout) {
  // wcnt (per-warp digit counters, then their warp prefixes) and the
  // tile's keys in digit order share one buffer: the counters are dead
  // once every pair knows its slot.
  __shared__ uint32_t sbuf[kRadixWarps * kRadixMaxBuckets];  // == kRadixTile
  __shared__ int32_t svals[kRadixTile];
  __shared__ uint32_t dstart[kRadixMaxBuckets];
  __shared__ uint32_t gofs[kRadixMaxBuckets];
  __shared__ uint32_t wt[kRadixWarps];
  static_assert(kRadixWarps * kRadixMaxBuckets == kRadixTile, "shared buffer sizes");
  const int nb = 1 << bits;
  const uint32_t mask = (uint32_t)nb - 1u;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t* wcnt = sbuf + w * kRadixMaxBuckets;
  for (int i = lane; i < nb; i += 32) wcnt[i] = 0u;
  __syncwarp();
  const int64_t tile0 = (int64_t)blockIdx.x * kRadixTile;
  const int64_t wbase = tile0 + (int64_t)w * kRadixWarpSpan;
  uint32_t key[kRadixItems];
  int32_t val[kRadixItems];
  uint32_t rk[kRadixItems];  // rank among equal digits in this warp's span
  const unsigned lt = lanemask_lt();
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    const int64_t e = wbase + r * 32 + lane;
    const bool live = e < n;
    key[r] = live ? __ldg(kin + e) : 0xffffffffu;
    val[r] = live ? __ldg(vin + e) : 0;
    const uint32_t d = live ? (key[r] >> shift) & mask : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t c = 0;
    if (live) c = wcnt[d];
    rk[r] = c + (uint32_t)__popc(peers & lt);
    __syncwarp();
    if (live && lane == __ffs(peers) - 1) wcnt[d] = c + (uint32_t)__popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: prefix over warps (in place), tile count, global slot
  const int64_t tile_n = n - tile0 < kRadixTile ? n - tile0 : kRadixTile;
  uint32_t cnt[kRadixMaxBuckets / kRadixThreads];
#pragma unroll
  for (int j = 0; j < kRadixMaxBuckets / kRadixThreads; ++j) {
    const int d = threadIdx.x * (kRadixMaxBuckets / kRadixThreads) + j;
    uint32_t run = 0;
    if (d < nb) {
#pragma unroll
      for (int i = 0; i < kRadixWarps; ++i) {
        const uint32_t c = sbuf[i * kRadixMaxBuckets + d];
        sbuf[i * kRadixMaxBuckets + d] = run;
        run += c;
      }
      gofs[d] = offsets[(int64_t)d * ntiles + blockIdx.x];
    }
    cnt[j] = run;
  }
  uint32_t s = 0;
#pragma unroll
  for (int j = 0; j < kRadixMaxBuckets / kRadixThreads; ++j) s += cnt[j];
  uint32_t tot;
  uint32_t ex = block_exclusive_scan(s, wt, &tot);
#pragma unroll
  for (int j = 0; j < kRadixMaxBuckets / kRadixThreads; ++j) {
    const int d = threadIdx.x * (kRadixMaxBuckets / kRadixThreads) + j;
    if (d < nb) dstart[d] = ex;
    ex += cnt[j];
  }
  __syncthreads();
  uint32_t slot[kRadixItems];
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    const int64_t e = wbase + r * 32 + lane;
    slot[r] = 0xffffffffu;
    if (e < n) {
      const uint32_t d = (key[r] >> shift) & mask;
      slot[r] = dstart[d] + sbuf[w * kRadixMaxBuckets + d] + rk[r];
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRadixItems; ++r) {
    if (slot[r] != 0xffffffffu) {
      sbuf[slot[r]] = key[r];
      svals[slot[r]] = val[r];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < tile_n; i += kRadixThreads) {
    const uint32_t k = sbuf[i];
    const uint32_t d = (k >> shift) & mask;
    const int64_t o = (int64_t)gofs[d] + (int64_t)(i - (int)dstart[d]);
    kout[o] = k;
    vout[o] = svals[i];
  }
}

// Pass plan for keys below 2^key_bits: the fewest passes of <= 9 bits.
struct RadixPlan {
  int passes, bits[4], shift[4];
};

inline RadixPlan radix_plan(int key_bits) {
  RadixPlan p{};
  if (key_bits < 1) key_bits = 1;
  p.passes = (key_bits + kRadixMaxBits - 1) / kRadixMaxBits;
  int sh = 0;
  for (int i = 0; i < p.passes; ++i) {
    const int b = (key_bits - sh + (p.passes - i) - 1) / (p.passes - i);
    p.bits[i] = b;
    p.shift[i] = sh;
    sh += b;
  }
  return p;
}

inline int64_t radix_ntiles(int64_t n) { return (n + kRadixTile - 1) / kRadixTile; }

// Workspace of radix_sort_pairs: the other key/value buffer pair, the
// digit counts and the scan's chunk sums, each 256-byte aligned.
inline size_t radix_workspace(int64_t n) {
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const int64_t nt = radix_ntiles(n);
  const int64_t m = nt * kRadixMaxBuckets;
  return al((size_t)n * 4) * 2 + al((size_t)m * 4) + al((size_t)((m + kScanChunk - 1) / kScanChunk + 1) * 4);
}

// Sorts (ka, va) by the low key_bits of the keys; the result lands in
// (ka, va) (the workspace holds the other buffer pair).  n < 2^31.
inline int radix_sort_pairs(cudaStream_t st, uint32_t* ka, int32_t* va, int64_t n, int key_bits, void* ws,
                            size_t ws_bytes, const char* who) {
  if (n <= 1) return JLD_OK;
  if (ws_bytes < radix_workspace(n)) return set_error(JLD_ERR_WORKSPACE, "%s: sort workspace too small", who);
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  const int64_t nt = radix_ntiles(n);
  const int64_t m = nt * kRadixMaxBuckets;
  char* w = (char*)ws;
  uint32_t* kb = (uint32_t*)w;
  w += al((size_t)n * 4);
  int32_t* vb = (int32_t*)w;
  w += al((size_t)n * 4);
  uint32_t* counts = (uint32_t*)w;
  w += al((size_t)m * 4);
  uint32_t* part = (uint32_t*)w;
  const RadixPlan p = radix_plan(key_bits);
  uint32_t *src_k = ka, *dst_k = kb;
  int32_t *src_v = va, *dst_v = vb;
  for (int i = 0; i < p.passes; ++i) {
    const int64_t mm = nt << p.bits[i];
    const int64_t nchunk = (mm + kScanChunk - 1) / kScanChunk;
    radix_count_kernel<<<(unsigned)nt, kRadixThreads, 0, st>>>(src_k, n, p.shift[i], p.bits[i], (int)nt, counts);
    scan_reduce_kernel<<<(unsigned)nchunk, kRadixThreads, 0, st>>>(counts, mm, part);
    scan_part_kernel<<<1, kRadixThreads, 0, st>>>(part, nchunk);
    scan_apply_kernel<<<(unsigned)nchunk, kRadixThreads, 0, st>>>(counts, mm, part);
    radix_scatter_kernel<<<(unsigned)nt, kRadixThreads, 0, st>>>(src_k, src_v, n, p.shift[i], p.bits[i], (int)nt,
                                                                counts, dst_k, dst_v);
    JLD_LAUNCH_CHECK(who);
    uint32_t* tk = src_k; src_k = dst_k; dst_k = tk;
    int32_t* tv = src_v; src_v = dst_v; dst_v = tv;
  }
  if (src_k != ka) {
    JLD_CUDA_TRY(cudaMemcpyAsync(ka, src_k, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
    JLD_CUDA_TRY(cudaMemcpyAsync(va, src_v, (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
  }
  return JLD_OK;
}

}  // namespace jld
