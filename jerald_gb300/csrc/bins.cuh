// Spatial binning of particles into mesh tiles and tile-privatized CIC
// scatters (sm_103a).
//
// Binning is a counting sort of the particles by the tile that contains
// their cell (the cell of int(p) on each axis after the box prelude, the
// same cell the paint uses): a warp-aggregated histogram over tiles, an
// exclusive scan, and a warp-aggregated scatter.  The order of particles
// inside a tile follows the atomics; it only affects the order in which
// float contributions are summed.
//
// A tiled scatter gives each CTA whole tiles: the CTA accumulates its
// particles' corner weights with shared-memory atomics into a window
// covering the tile, `halo` cells on each side and the +1 corner, then adds
// the window to the mesh with one global atomic per nonzero cell.  Corners
// outside the window (particles that drifted since binning) go straight to
// global atomics, so the result does not depend on the drift.
#pragma once

#include "common.cuh"

namespace jld {

struct TileGeom {
  int tx, ty, tz;     // tile size (cells)
  int ntx, nty, ntz;  // tiles per axis
  int halo;           // window margin below and above the tile
  int wx, wy, wz;     // window extent: t + 2*halo + 1
  __host__ __device__ int ntiles() const { return ntx * nty * ntz; }
  __host__ __device__ int wcells() const { return wx * wy * wz; }
};

inline TileGeom make_tile_geom(int nx, int ny, int nz, int t, int halo) {
  TileGeom tg;
  tg.tx = nx < t ? nx : t;
  tg.ty = ny < t ? ny : t;
  tg.tz = nz < t ? nz : t;
  tg.ntx = (nx + tg.tx - 1) / tg.tx;
  tg.nty = (ny + tg.ty - 1) / tg.ty;
  tg.ntz = (nz + tg.tz - 1) / tg.tz;
  tg.halo = halo;
  tg.wx = tg.tx + 2 * halo + 1;
  tg.wy = tg.ty + 2 * halo + 1;
  tg.wz = tg.tz + 2 * halo + 1;
  return tg;
}

// Lower cell index of the CIC stencil on one axis, wrapped into [0, n).
__device__ __forceinline__ int wrap_cell(float q, int n) {
  int i = (int)q % n;
  return i < 0 ? i + n : i;
}

__device__ __forceinline__ int tile_of(const float q[3], const Grid3& g, const TileGeom& tg) {
  const int i = wrap_cell(q[0], g.nx), j = wrap_cell(q[1], g.ny), k = wrap_cell(q[2], g.nz);
  return ((i / tg.tx) * tg.nty + (j / tg.ty)) * tg.ntz + (k / tg.tz);
}

// Warp-aggregated increment of counters[key]: returns this lane's slot among
// all lanes of the warp with the same key, added to the counter's old value.
__device__ __forceinline__ int warp_agg_inc(int* counters, int key, bool live) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int k = live ? key : -1;
  const unsigned peers = __match_any_sync(full, k);
  const int leader = __ffs(peers) - 1;
  const int rank = __popc(peers & ((1u << lane) - 1u));
  int base = 0;
  if (lane == leader && live) base = atomicAdd(counters + key, __popc(peers));
  base = __shfl_sync(full, base, leader);
  return base + rank;
}

}  // namespace jld

namespace jld {

// Per-axis CIC cell indices (lower corner and its periodic neighbour, both
// wrapped as the paint wraps them) plus validity flags and fraction.
struct CicIdx {
  int lo[3], hi[3];
  bool ok[3][2];
  float d[3];
};

__device__ __forceinline__ void cic_idx(const float q[3], const Grid3& g, CicIdx& c) {
  const int n[3] = {g.nx, g.ny, g.nz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int i = (int)q[a];
    c.d[a] = __fsub_rn(q[a], (float)i);
    if ((unsigned)i < (unsigned)n[a]) {
      c.lo[a] = i;
      c.hi[a] = (i + 1 == n[a]) ? 0 : i + 1;
      c.ok[a][0] = true;
      c.ok[a][1] = true;
    } else {
      int ip1 = (i + 1) % n[a];
      c.ok[a][0] = false;
      c.ok[a][1] = (unsigned)ip1 < (unsigned)n[a];
      c.lo[a] = abs(i % n[a]);
      c.hi[a] = abs(ip1 % n[a]);
    }
  }
}

// Offset of global cell index v (in [0, n)) inside a window starting at o
// (o may be negative or past n: the mesh is periodic); >= w means outside.
__device__ __forceinline__ int win_coord(int v, int o, int n) {
  int d = v - o;
  if (d < 0) d += n;
  if (d >= n) d -= n;
  return d;
}

// Pass 1 of the binning: tile key of every particle and the tile histogram.
__global__ void __launch_bounds__(256)
bin_count_kernel(const float* __restrict__ X, int64_t n, float3 box, float3 cell, Grid3 g, TileGeom tg,
                 int* __restrict__ keys, int* __restrict__ counts) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
    const int64_t p = base + (threadIdx.x & 31);
    const bool live = p < n;
    int key = 0;
    if (live) {
      float q[3] = {box_to_mesh(__ldg(X + 3 * p), box.x, cell.x), box_to_mesh(__ldg(X + 3 * p + 1), box.y, cell.y),
                    box_to_mesh(__ldg(X + 3 * p + 2), box.z, cell.z)};
      key = tile_of(q, g, tg);
      keys[p] = key;
    }
    warp_agg_inc(counts, key, live);
  }
}

// Pass 2: exclusive scan of the tile counts (one block of 1024 threads):
// starts[t] = sum of counts[< t], starts[ntiles] = total; fill = starts.
__global__ void __launch_bounds__(1024)
bin_scan_kernel(const int* __restrict__ counts, int ntiles, int* __restrict__ starts, int* __restrict__ fill) {
  __shared__ int part[1024];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int chunk = (ntiles + nthr - 1) / nthr;
  const int b = tid * chunk, e = min(ntiles, b + chunk);
  int s = 0;
  for (int i = b; i < e; ++i) s += counts[i];
  part[tid] = s;
  __syncthreads();
  if (tid == 0) {
    int acc = 0;
    for (int i = 0; i < nthr; ++i) { int v = part[i]; part[i] = acc; acc += v; }
    starts[ntiles] = acc;
  }
  __syncthreads();
  int acc = part[tid];
  for (int i = b; i < e; ++i) { starts[i] = acc; fill[i] = acc; acc += counts[i]; }
}

// Pass 3: scatter particles into tile order: Xs[slot] = X[p], perm[slot] = p.
__global__ void __launch_bounds__(256)
bin_scatter_kernel(const float* __restrict__ X, int64_t n, const int* __restrict__ keys, int* __restrict__ fill,
                   float* __restrict__ Xs, int* __restrict__ perm) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
    const int64_t p = base + (threadIdx.x & 31);
    const bool live = p < n;
    const int key = live ? __ldg(keys + p) : 0;
    const int slot = warp_agg_inc(fill, key, live);
    if (live) {
      Xs[3 * (int64_t)slot] = __ldg(X + 3 * p);
      Xs[3 * (int64_t)slot + 1] = __ldg(X + 3 * p + 1);
      Xs[3 * (int64_t)slot + 2] = __ldg(X + 3 * p + 2);
      perm[slot] = (int)p;
    }
  }
}

// Tile origin (lowest window cell) of tile t.
__device__ __forceinline__ void tile_origin(const TileGeom& tg, int t, int o[3]) {
  const int tk = t % tg.ntz, tj = (t / tg.ntz) % tg.nty, ti = t / (tg.ntz * tg.nty);
  o[0] = ti * tg.tx - tg.halo;
  o[1] = tj * tg.ty - tg.halo;
  o[2] = tk * tg.tz - tg.halo;
}

__device__ __forceinline__ int wrap_idx(int v, int n) {
  v %= n;
  return v < 0 ? v + n : v;
}

}  // namespace jld

namespace jld {

// Tile-privatized unit-mass paint of tile-ordered positions Xs (box units).
// One window of floats per CTA in dynamic shared memory.
__global__ void __launch_bounds__(256)
tiled_paint_kernel(const float* __restrict__ Xs, const int* __restrict__ starts, TileGeom tg, float3 box,
                   float3 cell, Grid3 g, float* __restrict__ rho) {
  extern __shared__ float win[];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int ntiles = tg.ntiles(), wc = tg.wcells();
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int p0 = __ldg(starts + t), p1 = __ldg(starts + t + 1);
    if (p0 == p1) continue;
    int o[3];
    tile_origin(tg, t, o);
    for (int c = tid; c < wc; c += nthr) win[c] = 0.f;
    __syncthreads();
    for (int p = p0 + tid; p < p1; p += nthr) {
      float q[3] = {box_to_mesh(__ldg(Xs + 3 * (int64_t)p), box.x, cell.x),
                    box_to_mesh(__ldg(Xs + 3 * (int64_t)p + 1), box.y, cell.y),
                    box_to_mesh(__ldg(Xs + 3 * (int64_t)p + 2), box.z, cell.z)};
      CicIdx ci;
      cic_idx(q, g, ci);
      float lo[3], hi[3];
      int wl[3], wh[3];
      const int n[3] = {g.nx, g.ny, g.nz};
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        hi[a] = ci.d[a];
        lo[a] = __fsub_rn(1.f, ci.d[a]);
        wl[a] = win_coord(ci.lo[a], o[a], n[a]);
        wh[a] = win_coord(ci.hi[a], o[a], n[a]);
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int bits = corner_axis_bits(k);
        const int bx = bits & 1, by = (bits >> 1) & 1, bz = (bits >> 2) & 1;
        if (!(ci.ok[0][bx] && ci.ok[1][by] && ci.ok[2][bz])) continue;
        const float w = __fmul_rn(__fmul_rn(bx ? hi[0] : lo[0], by ? hi[1] : lo[1]), bz ? hi[2] : lo[2]);
        const int x = bx ? wh[0] : wl[0], y = by ? wh[1] : wl[1], z = bz ? wh[2] : wl[2];
        if (x < tg.wx && y < tg.wy && z < tg.wz) {
          atomicAdd(win + (x * tg.wy + y) * tg.wz + z, w);
        } else {
          const int gx = bx ? ci.hi[0] : ci.lo[0], gy = by ? ci.hi[1] : ci.lo[1], gz = bz ? ci.hi[2] : ci.lo[2];
          atomicAdd(rho + (int64_t)gx * g.sx + (int64_t)gy * g.sy + gz, w);
        }
      }
    }
    __syncthreads();
    for (int c = tid; c < wc; c += nthr) {
      const float v = win[c];
      if (v != 0.f) {
        const int z = c % tg.wz, y = (c / tg.wz) % tg.wy, x = c / (tg.wz * tg.wy);
        const int gx = wrap_idx(o[0] + x, g.nx), gy = wrap_idx(o[1] + y, g.ny), gz = wrap_idx(o[2] + z, g.nz);
        atomicAdd(rho + (int64_t)gx * g.sx + (int64_t)gy * g.sy + gz, v);
      }
    }
    __syncthreads();
  }
}

// Adjoint of one layer's readout on tile-ordered particles: Xb = Xb1 +
// J^T Xb1 (gather of the float4 force mesh with CIC weight gradients) and the
// three-channel scatter of Xb1 into the float4 cotangent mesh through a
// shared-memory window (three floats per window cell).  GATHER = false
// does the scatter only (the first layer).
template <bool GATHER>
__global__ void __launch_bounds__(256)
tiled_bwd_kernel(const float* __restrict__ Xs, const float* __restrict__ Xb1, const int* __restrict__ starts,
                 TileGeom tg, float3 box, float3 cell, float3 dw, Grid3 g, const float4* __restrict__ g4,
                 float4* __restrict__ gb4, float* __restrict__ Xb) {
  extern __shared__ float win3[];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int ntiles = tg.ntiles(), wc = tg.wcells();
  const float dwv[3] = {dw.x, dw.y, dw.z};
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int p0 = __ldg(starts + t), p1 = __ldg(starts + t + 1);
    if (p0 == p1) continue;
    int o[3];
    tile_origin(tg, t, o);
    for (int c = tid; c < 3 * wc; c += nthr) win3[c] = 0.f;
    __syncthreads();
    for (int p = p0 + tid; p < p1; p += nthr) {
      const int64_t p3 = 3 * (int64_t)p;
      float q[3] = {box_to_mesh(__ldg(Xs + p3), box.x, cell.x), box_to_mesh(__ldg(Xs + p3 + 1), box.y, cell.y),
                    box_to_mesh(__ldg(Xs + p3 + 2), box.z, cell.z)};
      const float v[3] = {__ldg(Xb1 + p3), __ldg(Xb1 + p3 + 1), __ldg(Xb1 + p3 + 2)};
      CicIdx ci;
      cic_idx(q, g, ci);
      float lo[3], hi[3];
      int wl[3], wh[3];
      const int n[3] = {g.nx, g.ny, g.nz};
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        hi[a] = ci.d[a];
        lo[a] = __fsub_rn(1.f, ci.d[a]);
        wl[a] = win_coord(ci.lo[a], o[a], n[a]);
        wh[a] = win_coord(ci.hi[a], o[a], n[a]);
      }
      float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int bits = corner_axis_bits(k);
        const int bx = bits & 1, by = (bits >> 1) & 1, bz = (bits >> 2) & 1;
        if (!(ci.ok[0][bx] && ci.ok[1][by] && ci.ok[2][bz])) continue;
        const int gx = bx ? ci.hi[0] : ci.lo[0], gy = by ? ci.hi[1] : ci.lo[1], gz = bz ? ci.hi[2] : ci.lo[2];
        const int64_t off = (int64_t)gx * g.sx + (int64_t)gy * g.sy + gz;
        const float wx = bx ? hi[0] : lo[0], wy = by ? hi[1] : lo[1], wz = bz ? hi[2] : lo[2];
        if (GATHER) {
          const float4 gv = __ldg(g4 + off);
          const float u = v[0] * gv.x + v[1] * gv.y + v[2] * gv.z;
          acc[0] += u * ((bx ? dwv[0] : -dwv[0]) * wy * wz);
          acc[1] += u * (wx * (by ? dwv[1] : -dwv[1]) * wz);
          acc[2] += u * (wx * wy * (bz ? dwv[2] : -dwv[2]));
        }
        const float w = __fmul_rn(__fmul_rn(wx, wy), wz);
        const int x = bx ? wh[0] : wl[0], y = by ? wh[1] : wl[1], z = bz ? wh[2] : wl[2];
        if (x < tg.wx && y < tg.wy && z < tg.wz) {
          float* cellp = win3 + 3 * ((x * tg.wy + y) * tg.wz + z);
          atomicAdd(cellp, v[0] * w);
          atomicAdd(cellp + 1, v[1] * w);
          atomicAdd(cellp + 2, v[2] * w);
        } else {
          atomicAdd(gb4 + off, make_float4(v[0] * w, v[1] * w, v[2] * w, 0.f));
        }
      }
      if (GATHER) {
#pragma unroll
        for (int e = 0; e < 3; ++e) Xb[p3 + e] = v[e] + acc[e];
      }
    }
    __syncthreads();
    for (int c = tid; c < wc; c += nthr) {
      const float a0 = win3[3 * c], a1 = win3[3 * c + 1], a2 = win3[3 * c + 2];
      if (a0 != 0.f || a1 != 0.f || a2 != 0.f) {
        const int z = c % tg.wz, y = (c / tg.wz) % tg.wy, x = c / (tg.wz * tg.wy);
        const int gx = wrap_idx(o[0] + x, g.nx), gy = wrap_idx(o[1] + y, g.ny), gz = wrap_idx(o[2] + z, g.nz);
        atomicAdd(gb4 + (int64_t)gx * g.sx + (int64_t)gy * g.sy + gz, make_float4(a0, a1, a2, 0.f));
      }
    }
    __syncthreads();
  }
}

}  // namespace jld
