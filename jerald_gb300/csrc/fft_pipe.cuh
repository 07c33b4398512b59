// Pipelined pencil-FFT passes for line lengths 2^k and 3 x 2^k (sm_103a).
//
// Persistent CTAs walk a stream of "items" (one input tile each).  A ring of
// shared-memory staging slots is filled by the Tensor Memory Accelerator:
// cp.async.bulk.tensor (2-D/3-D tiles of strided pencils) or cp.async.bulk
// (contiguous rows), each completing on an mbarrier with its byte count.
// While a CTA transforms item i, the loads of items i+1 .. i+NSLOT-1 are in
// flight.  The transform itself uses a compile-time radix schedule (P2<...>):
// its first stage reads the staging slot (or any functor), its middle stages
// go through a work buffer, its last stage hands every value to an output
// functor (usually a direct, coalesced global store with the elementwise
// epilogue of the pass applied in registers).
//
// Every mbarrier wait is bounded: after kWaitLimit polls the CTA records an
// error in the pass's error word and stops, so a lost copy cannot hang the GPU.
#pragma once

#include <cuda.h>  // CUtensorMap (type only; the encoder is resolved at run time)

#include "fft_core.cuh"

namespace jld {

// ---------------------------------------------------------------------------
// PTX helpers.

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

constexpr int kWaitLimit = 1 << 22;

// Bounded wait on `parity` of an mbarrier; false after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit = kWaitLimit) {
  for (int it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Tile order of the persistent passes.  A CTA's first tile is blockIdx.x.
// With a per-launch counter `tick` (zero before the launch) every later tile
// is the counter's next value past the grid, so a CTA that starts late (its
// SM partly held by other work: a copy kernel, another box's step) takes
// fewer tiles instead of holding the pass up by a whole share.  Without a
// counter the order is the static blockIdx.x + i * gridDim.x.
__device__ __forceinline__ int next_tile(int* tick, int t) {
  return tick ? (int)gridDim.x + atomicAdd(tick, 1) : t + (int)gridDim.x;
}

// Orders earlier generic-proxy accesses of shared memory before a later TMA
// (async-proxy) write into it.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// ---------------------------------------------------------------------------
// Compile-time radix schedules (radix of the first stage first): powers of
// two, and 3 x a power of two with one radix-3 stage last.
constexpr int cgcd(int a, int b) { return b == 0 ? a : cgcd(b, a % b); }
constexpr int clcm_pack(int a) { return a; }
template <class... Ts>
constexpr int clcm_pack(int a, Ts... r) {
  const int b = clcm_pack(r...);
  return a / cgcd(a, b) * b;
}
constexpr int clog2(int v) {
  int s = 0;
  while ((1 << s) < v) ++s;
  return s;
}

template <int... Rs>
struct P2 {
  static constexpr int nst = sizeof...(Rs);
  static constexpr int rad[nst] = {Rs...};
  static constexpr int n = (1 * ... * Rs);
  // values per thread per line: a multiple of every radix (the largest
  // radix for a power-of-two schedule)
  static constexpr int E = clcm_pack(Rs...);
  static constexpr int pre(int s) {
    int p = 1;
    for (int i = 0; i < s; ++i) p *= rad[i];
    return p;
  }
};

// Work-buffer layouts.
//   ColWork: element (c, j) at j * cols + c   (strided passes: threads c-fastest)
//   RowWork: element (c, j) at c * ldw + j + (j >> PSH) (row passes: j-fastest;
//            the padding keeps the first stage's stride-R writes conflict-free)
struct ColWork {
  float2* p;
  int cols;
  __device__ __forceinline__ float2& at(int c, int j) const { return p[j * cols + c]; }
};
template <int PSH>
struct RowWork {
  float2* p;
  int ldw;
  __device__ __forceinline__ float2& at(int c, int j) const { return p[c * ldw + j + (j >> PSH)]; }
};

// One stage S of schedule Sch over all columns of the tile.  COL selects the
// thread mapping (c-fastest for strided tiles, j-fastest for rows).  With
// SYNC_MID the stage loads everything, synchronises, then stores (in place).
template <class Sch, int S, bool COL, bool SYNC_MID, class Ld, class St, class Mid>
__device__ __forceinline__ void p2_stage(const Ld& ld, const St& st, const float2* __restrict__ tw, int sgn,
                                         int cshift, int tid, int nthr, const Mid& mid) {
  constexpr int R = Sch::rad[S];
  constexpr int P = Sch::pre(S);
  constexpr int N = Sch::n;
  constexpr int T = N / R;
  constexpr int Q = Sch::E / R;
  constexpr int TWS = N / (P * R);
  float2 u[Q][R];
  int cc[Q], bb[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int id = tid + q * nthr;
    int c, b;
    if constexpr (COL) {
      c = id & ((1 << cshift) - 1);
      b = id >> cshift;
    } else {
      // unsigned division by constants: shifts and masks when T is a power
      // of two
      b = (int)((unsigned)id % (unsigned)T);
      c = (int)((unsigned)id / (unsigned)T);
    }
    cc[q] = c;
    bb[q] = b;
#pragma unroll
    for (int r = 0; r < R; ++r) u[q][r] = ld(c, b + r * T);
  }
  if constexpr (SYNC_MID) {
    __syncthreads();
    mid();
  }
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = bb[q], c = cc[q];
    static_assert((P & (P - 1)) == 0, "only the last stage of a schedule may have a radix other than 2^k");
    const int k = b & (P - 1);
    if constexpr (P > 1) {
      if (k != 0) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          float2 w = __ldg(tw + r * k * TWS);
          if (sgn > 0) w.y = -w.y;
          u[q][r] = cmul(u[q][r], w);
        }
      }
    }
    dftR<R>(u[q], sgn);
    const int j = (b - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) st(c, j + r * P, u[q][r]);
  }
}

// Whole transform of a tile: in(c, j) -> [work] -> out(c, j, v).  `rel` runs
// (on every thread) right after the barrier that follows the first stage,
// i.e. once no thread reads `in` any more: the place to recycle the input's
// staging slot.  The caller synchronises before (work / input free) and
// after (if the output lands in shared memory that other threads read).
struct NoRelease {
  __device__ __forceinline__ void operator()() const {}
};

template <class Sch, bool COL, class W, class In, class Out, class Rel>
__device__ __forceinline__ void p2_run_rel(const W& work, const In& in, const Out& out, const Rel& rel,
                                           const float2* __restrict__ tw, int sgn, int cshift, int tid,
                                           int nthr) {
  auto wld = [&](int c, int j) { return work.at(c, j); };
  auto wst = [&](int c, int j, float2 v) { work.at(c, j) = v; };
  if constexpr (Sch::nst == 1) {
    p2_stage<Sch, 0, COL, true>(in, out, tw, sgn, cshift, tid, nthr, rel);
  } else {
    p2_stage<Sch, 0, COL, false>(in, wst, tw, sgn, cshift, tid, nthr, NoRelease{});
    __syncthreads();
    rel();
    if constexpr (Sch::nst >= 3) {
      p2_stage<Sch, 1, COL, true>(wld, wst, tw, sgn, cshift, tid, nthr, NoRelease{});
      __syncthreads();
    }
    if constexpr (Sch::nst >= 4) {
      p2_stage<Sch, 2, COL, true>(wld, wst, tw, sgn, cshift, tid, nthr, NoRelease{});
      __syncthreads();
    }
    p2_stage<Sch, Sch::nst - 1, COL, false>(wld, out, tw, sgn, cshift, tid, nthr, NoRelease{});
  }
}

template <class Sch, bool COL, class W, class In, class Out>
__device__ __forceinline__ void p2_run(const W& work, const In& in, const Out& out, const float2* __restrict__ tw,
                                       int sgn, int cshift, int tid, int nthr) {
  p2_run_rel<Sch, COL>(work, in, out, NoRelease{}, tw, sgn, cshift, tid, nthr);
}

// Schedules used for each power-of-two length: radix-16 stages and one
// smaller tail, E = 16 elements per thread per column.
template <int N> struct P2For;
template <> struct P2For<16> { using type = P2<16>; };
template <> struct P2For<32> { using type = P2<16, 2>; };
template <> struct P2For<64> { using type = P2<16, 4>; };
template <> struct P2For<128> { using type = P2<16, 8>; };
template <> struct P2For<256> { using type = P2<16, 16>; };
template <> struct P2For<512> { using type = P2<16, 16, 2>; };
template <> struct P2For<1024> { using type = P2<16, 16, 4>; };
template <> struct P2For<2048> { using type = P2<16, 16, 8>; };
// 3 x 2^k (meshes of 96 and 192 cells per axis and their half lengths): the
// radix-4 and radix-2 stages first, one radix-3 stage last, E = 12 values
// per thread per line (the lcm of the radices; radix-8 stages would make it
// 24 and spill in the kernels capped at 64-96 registers).
template <> struct P2For<48> { using type = P2<4, 4, 3>; };
template <> struct P2For<96> { using type = P2<4, 4, 2, 3>; };
template <> struct P2For<192> { using type = P2<4, 4, 4, 3>; };

// Radix-8 family: 8 values per thread per line, so a kernel can stay under
// 64 registers and keep twice the warps resident (used by the x passes,
// whose three transforms per tile otherwise hold 128 registers).
template <int N> struct P2For8;
template <> struct P2For8<16> { using type = P2<8, 2>; };
template <> struct P2For8<32> { using type = P2<8, 4>; };
template <> struct P2For8<64> { using type = P2<8, 8>; };
template <> struct P2For8<128> { using type = P2<8, 8, 2>; };
template <> struct P2For8<256> { using type = P2<8, 8, 4>; };
template <> struct P2For8<512> { using type = P2<8, 8, 8>; };
template <> struct P2For8<1024> { using type = P2<8, 8, 8, 2>; };
template <> struct P2For8<2048> { using type = P2<8, 8, 8, 4>; };

template <class F>
inline int with_p2_8(int n, F&& body) {
  switch (n) {
    case 16: return body(P2For8<16>::type{});
    case 32: return body(P2For8<32>::type{});
    case 64: return body(P2For8<64>::type{});
    case 128: return body(P2For8<128>::type{});
    case 256: return body(P2For8<256>::type{});
    case 512: return body(P2For8<512>::type{});
    case 1024: return body(P2For8<1024>::type{});
    case 2048: return body(P2For8<2048>::type{});
    default: return -1;
  }
}

// Calls body(P2For<N>::type{}) for a supported length (a power of two from
// 16 to 2048, or 48, 96, 192); returns -1 if n has no pipelined schedule.
template <class F>
inline int with_p2(int n, F&& body) {
  switch (n) {
    case 48: return body(P2For<48>::type{});
    case 96: return body(P2For<96>::type{});
    case 192: return body(P2For<192>::type{});
    case 16: return body(P2For<16>::type{});
    case 32: return body(P2For<32>::type{});
    case 64: return body(P2For<64>::type{});
    case 128: return body(P2For<128>::type{});
    case 256: return body(P2For<256>::type{});
    case 512: return body(P2For<512>::type{});
    case 1024: return body(P2For<1024>::type{});
    case 2048: return body(P2For<2048>::type{});
    default: return -1;
  }
}

// Values per thread per line (E) and first-stage shift (PSH of the row
// work buffer) of the P2For schedule of length n; false if there is none.
inline bool p2_shape(int n, int* E, int* psh) {
  return with_p2(n, [&](auto sch) {
           using Sch = decltype(sch);
           *E = Sch::E;
           *psh = clog2(Sch::rad[0]);
           return 0;
         }) == 0;
}

}  // namespace jld
