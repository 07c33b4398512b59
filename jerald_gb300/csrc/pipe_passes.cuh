// Pipelined strided passes over the main block of the internal half
// spectrum (main[x][y][kz], kz < h) for power-of-two line lengths.  The nyq
// plane (kz = h) is small and keeps the generic kernels.
//
// Tiles are `cols` consecutive kz (y passes) or (y, kz) columns (x passes) by
// the whole line; a tile is one TMA load (two or more 256-line boxes).  Each
// CTA is persistent over tiles (blockIdx.x first, then the order of
// next_tile) and keeps one staging slot: the load of its next tile is issued
// as soon as the first FFT stage of the current one has copied the slot into
// the work buffer, so it overlaps the remaining stages and the epilogue.
#pragma once

#include "fft_pipe.cuh"

namespace jld {

// Geometry of a strided pass (AX = 1: along y; AX = 0: along x).
struct SGeom {
  int nx, ny, h;
  int cols, cshift;  // tile width (power of two dividing h)
  int lines;         // transform length: ny (AX 1) or nx (AX 0)
  int ntiles;        // tiles in the main block
  int64_t es;        // element stride along a line (complex units)
};

// First element (column 0, line 0) of tile t.
template <int AX>
__device__ __forceinline__ int64_t tile_base(const SGeom& g, int t) {
  if (AX == 1) {
    const int tpp = g.h >> g.cshift;
    const int x = t / tpp;
    return (int64_t)x * g.ny * g.h + ((int64_t)(t - x * tpp) << g.cshift);
  }
  return (int64_t)t << g.cshift;
}

// Issues the TMA load of tile t of tensor `map` into dst (all lines).
template <int AX>
__device__ __forceinline__ void issue_tile(const CUtensorMap* map, float2* dst, uint64_t* bar, const SGeom& g,
                                           int t) {
  const int chunk = g.lines < 256 ? g.lines : 256;
  mbar_arrive_expect_tx(bar, (uint32_t)g.lines * g.cols * 8u);
  if (AX == 1) {
    const int tpp = g.h >> g.cshift;
    const int x = t / tpp;
    const int kz0 = (t - x * tpp) << g.cshift;
    for (int y0 = 0; y0 < g.lines; y0 += chunk) tma_load_3d(dst + y0 * g.cols, map, 2 * kz0, y0, x, bar);
  } else {
    const int col0 = t << g.cshift;
    for (int x0 = 0; x0 < g.lines; x0 += chunk) tma_load_2d(dst + x0 * g.cols, map, 2 * col0, x0, bar);
  }
}

// Shared-memory carve-up of the pipelined kernels: staging slot(s), work
// buffer, optional accumulator tiles, then one mbarrier per staging slot.
struct PipeSmem {
  float2* slot[3];
  float2* work;
  float2* acc;
  uint64_t* bar;
};
__device__ __forceinline__ PipeSmem pipe_smem(unsigned char* raw, int tile_elems, int nslot, int nacc) {
  PipeSmem s;
  float2* p = reinterpret_cast<float2*>(raw);
  for (int i = 0; i < 3; ++i) s.slot[i] = i < nslot ? p + (size_t)i * tile_elems : nullptr;
  s.work = p + (size_t)nslot * tile_elems;
  s.acc = nacc ? s.work + tile_elems : nullptr;
  s.bar = reinterpret_cast<uint64_t*>(s.work + (size_t)(1 + nacc) * tile_elems);
  return s;
}

__device__ __forceinline__ void pipe_error(int* err, int code) {
  if (err) atomicExch(err, code);
}

// ---------------------------------------------------------------------------
// Single-input pass in place (y or x FFT, either sign): out may equal the
// tensor's buffer.
template <class Sch, int AX, int SGN>
__global__ void __launch_bounds__(512)
spass_kernel(const __grid_constant__ CUtensorMap m_in, float2* out, SGeom g, const float2* __restrict__ tw,
             int* err, int* tick) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int s_next;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int tile_elems = g.lines * g.cols;
  PipeSmem s = pipe_smem(smraw, tile_elems, 1, 0);
  if (tid == 0) {
    mbar_init(s.bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  int t = blockIdx.x;
  if (tid == 0 && t < g.ntiles) issue_tile<AX>(&m_in, s.slot[0], s.bar, g, t);
  ColWork wk{s.work, g.cols};
  for (int i = 0; t < g.ntiles; ++i) {
    bool ok = mbar_wait_bounded(s.bar, (uint32_t)(i & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 1); return; }
    const float2* slot = s.slot[0];
    const int64_t base = tile_base<AX>(g, t);
    auto in = [&](int c, int j) { return slot[j * g.cols + c]; };
    auto st = [&](int c, int j, float2 v) { out[base + c + (int64_t)j * g.es] = v; };
    auto release = [&]() {
      if (tid == 0) {
        const int nt = next_tile(tick, t);
        s_next = nt;
        if (nt < g.ntiles) {
          fence_proxy_async_smem();
          issue_tile<AX>(&m_in, s.slot[0], s.bar, g, nt);
        }
      }
    };
    p2_run_rel<Sch, true>(wk, in, st, release, tw, SGN, g.cshift, tid, nthr);
    __syncthreads();
    t = s_next;
  }
}

}  // namespace jld

namespace jld {

// ---------------------------------------------------------------------------
// x pass (AX 0) of the main block with the result written in the caller's
// half-spectrum layout (nx, ny, h+1): interleaved complex (out_c) or split
// real / imaginary arrays (out_re, out_im).  A tile's columns are `cols`
// consecutive kz of one y (cols divides h), so each line's stores are one
// contiguous run.
template <class Sch, int SGN>
__global__ void __launch_bounds__(512)
xref_pipe_kernel(const __grid_constant__ CUtensorMap m_in, float2* __restrict__ out_c, float* __restrict__ out_re,
                 float* __restrict__ out_im, SGeom g, const float2* __restrict__ tw, int* err) {
  extern __shared__ __align__(128) unsigned char smraw[];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int tile_elems = g.lines * g.cols;
  PipeSmem s = pipe_smem(smraw, tile_elems, 1, 0);
  if (tid == 0) {
    mbar_init(s.bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  const int ntl = (g.ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  if (tid == 0 && ntl > 0) issue_tile<0>(&m_in, s.slot[0], s.bar, g, blockIdx.x);
  ColWork wk{s.work, g.cols};
  const int64_t row = (int64_t)g.ny * (g.h + 1);  // caller-layout stride between x lines
  for (int i = 0; i < ntl; ++i) {
    const int t = blockIdx.x + i * gridDim.x;
    bool ok = mbar_wait_bounded(s.bar, (uint32_t)(i & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 11); return; }
    const float2* slot = s.slot[0];
    const int64_t col0 = (int64_t)t << g.cshift;  // (y, kz) column index y * h + kz
    const int64_t y = col0 / g.h, kz0 = col0 - y * g.h;
    const int64_t o0 = y * (g.h + 1) + kz0;
    const bool more = i + 1 < ntl;
    auto in = [&](int c, int j) { return slot[j * g.cols + c]; };
    auto st = [&](int c, int j, float2 v) {
      const int64_t o = o0 + c + (int64_t)j * row;
      if (out_c) {
        out_c[o] = v;
      } else {
        out_re[o] = v.x;
        out_im[o] = v.y;
      }
    };
    auto release = [&]() {
      if (tid == 0 && more) {
        fence_proxy_async_smem();
        issue_tile<0>(&m_in, s.slot[0], s.bar, g, t + gridDim.x);
      }
    };
    p2_run_rel<Sch, true>(wk, in, st, release, tw, SGN, g.cshift, tid, nthr);
    __syncthreads();
  }
}

}  // namespace jld
