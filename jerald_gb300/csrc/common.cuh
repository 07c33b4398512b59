// Shared helpers for the sm_103a kernels: status/error plumbing, the
// mesh-coordinate prelude and the cloud-in-cell (CIC) corner arithmetic.
#pragma once

#include <cuda_runtime.h>
#include <algorithm>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>

#include "../../include/jld.h"

namespace jld {

// ---------------------------------------------------------------------------
// Error reporting.  Every C entry point returns a status and leaves a
// human-readable message in a thread-local buffer.
int set_error(int status, const char* fmt, ...);
void clear_error();

#define JLD_CUDA_TRY(expr)                                                      \
  do {                                                                          \
    cudaError_t _e = (expr);                                                    \
    if (_e != cudaSuccess)                                                      \
      return ::jld::set_error(JLD_ERR_CUDA, "%s failed: %s (%s:%d)", #expr,     \
                              cudaGetErrorString(_e), __FILE__, __LINE__);      \
  } while (0)

// Checks the launch that was just issued on the current thread.
#define JLD_LAUNCH_CHECK(name)                                                  \
  do {                                                                          \
    cudaError_t _e = cudaGetLastError();                                        \
    if (_e != cudaSuccess)                                                      \
      return ::jld::set_error(JLD_ERR_CUDA, "launch of %s failed: %s", name,    \
                              cudaGetErrorString(_e));                          \
  } while (0)

// Number of SMs of the current device (cached per device).
int sm_count();

// Grid size for a grid-stride loop over n items with the given block size:
// enough CTAs to fill every SM `per_sm` times, never more than needed.
inline unsigned grid_for(int64_t n, int block, int per_sm = 8) {
  int64_t need = (n + block - 1) / block;
  int64_t cap = (int64_t)sm_count() * per_sm;
  if (need < 1) need = 1;
  return (unsigned)(need < cap ? need : cap);
}

// CTAs of `func` (a __global__ function) that fit on one SM at this block
// size and dynamic shared memory (cached per device and configuration).
int resident_blocks_ptr(const void* func, int block, size_t smem);

// Grid of a grid-stride loop over n items that runs in exactly one wave:
// every SM holds as many CTAs as fit (from the kernel's registers and shared
// memory), never more CTAs than items need.  A grid of more CTAs than fit
// runs a partial second wave in which most SMs idle, because every CTA of
// a grid-stride loop carries the same amount of work.
template <typename K>
inline unsigned resident_grid(K* func, int64_t n, int block, size_t smem = 0) {
  int64_t need = (n + block - 1) / block;
  int64_t cap = (int64_t)sm_count() * resident_blocks_ptr((const void*)func, block, smem);
  if (need < 1) need = 1;
  return (unsigned)(need < cap ? need : cap);
}

// Unit-mass CIC paint of box-unit positions into `out` (zeroed first); the
// same kernels as jld_ppaint_box_f32 (method 0 atomics, 1 warp-aggregated)
// with the division-free prelude (box_to_mesh_fast).  tick: the launch's
// WarpBatches counters (kTicksPerLaunch ints, zeroed) or nullptr.
int paint_unit_f32(cudaStream_t st, const float* pos, int64_t n, int64_t nx, int64_t ny,
                   int64_t nz, const float* box, int method, float* out, int* tick = nullptr);

// Batches of 32 consecutive particles walked by one warp of a persistent
// particle kernel; every lane calls first() and next() together.
// Without counters: the grid-stride order, batch w, w + W, w + 2W, ... for
// global warp w of W.  With counters (kTickRegions ints kTickStride apart,
// zero before the launch): units of kUnitBatches consecutive batches, unit u
// in region u % kTickRegions; a warp's first unit is static (the
// (w / kTickRegions)-th of region w % kTickRegions) and every later one is
// its region counter's next value past the region's warp count, so warps
// that start late (their SM partly held by other work: a host copy, another
// box's step) take fewer units instead of holding the kernel up by a whole
// share.  The regions keep the counters on separate cache lines.
// Units of up to 16 batches: 29.07 ms per 512^3 step against 29.14 (8) and
// 29.27 (4) on one box; 1 and 2 were slower still (31.20, 29.74 on another).
constexpr int kTickRegions = 32, kTickStride = 32, kUnitBatches = 16;
constexpr int kTicksPerLaunch = kTickRegions * kTickStride;
struct WarpBatches {
  int* tick;         // this warp's region counter, or nullptr (grid-stride order)
  int64_t unit_end;  // counters: end of the current unit
  int pending;       // counters, lane 0: the next unit's ticket, fetched a unit ahead
  int ub;            // counters: batches per unit
  // Only these stay live across a kernel's batch loop; the warp index,
  // region and stride are recomputed when needed (registers are the scarce
  // resource of the particle kernels).  The next ticket is fetched when a
  // unit starts and read when it ends, so the atomic's round trip overlaps
  // the unit's work (reading it at once cost the layer update 13 %).
  __device__ __forceinline__ static int64_t warps() { return (int64_t)gridDim.x * (blockDim.x >> 5); }
  __device__ __forceinline__ static int64_t warp() {
    return (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  }
  __device__ __forceinline__ int64_t unit_start(int64_t region, int64_t q) const {
    return (region + (int64_t)kTickRegions * q) * (32 * (int64_t)ub);
  }
  __device__ __forceinline__ void fetch() {
    if ((threadIdx.x & 31) == 0) {
      const int64_t region = warp() % kTickRegions;
      const int wr = (int)((warps() - region + kTickRegions - 1) / kTickRegions);
      pending = wr + atomicAdd(tick, 1);
    }
  }
  // n: particles of the launch.  A unit holds up to kUnitBatches batches,
  // fewer when there is too little work for every warp to get eight units
  // (a 64^3 box has 9e3 batches for 7e3 warps).
  __device__ __forceinline__ int64_t first(int* tick_, int64_t n) {
    const int64_t w = warp(), nw = warps();
    tick = nw >= kTickRegions ? tick_ + (w % kTickRegions) * kTickStride : nullptr;
    if (!tick) return 32 * w;
    const int64_t per = n / (32 * 8 * nw);
    ub = (int)(per < 1 ? 1 : per > kUnitBatches ? kUnitBatches : per);
    const int64_t b = unit_start(w % kTickRegions, w / kTickRegions);
    unit_end = b + 32 * (int64_t)ub;
    fetch();
    return b;
  }
  __device__ __forceinline__ int64_t next(int64_t base) {
    if (!tick) return base + 32 * warps();
    base += 32;
    if (base < unit_end) return base;
    const int q = __shfl_sync(0xffffffffu, pending, 0);
    const int64_t b = unit_start(warp() % kTickRegions, q);
    unit_end = b + 32 * (int64_t)ub;
    fetch();
    return b;
  }
};

// ---------------------------------------------------------------------------
// Mesh geometry passed by value to kernels.
struct Grid3 {
  int nx, ny, nz;      // mesh cells per axis
  int64_t sy, sx;      // strides of y and x in a (nx, ny, nz) row-major mesh
  __host__ __device__ int64_t cells() const { return sx * (int64_t)nx; }
};

inline Grid3 make_grid(int64_t nx, int64_t ny, int64_t nz) {
  Grid3 g;
  g.nx = (int)nx; g.ny = (int)ny; g.nz = (int)nz;
  g.sy = nz;
  g.sx = (int64_t)ny * nz;
  return g;
}

// Box-to-mesh prelude of jaxpops_bind.py:163-164 in the working dtype:
// r = x mod L with jnp.remainder semantics (C fmod, plus L when the signs of
// r and L differ and r is nonzero), then r / (L/N) with IEEE division.
// The common cases take exact shortcuts with identical results (box > 0):
//   0 <= x < L    fmod(x, L) = x
//   L <= x < 2L   fmod(x, L) = x - L, exact by Sterbenz' lemma
//   -L < x < 0    fmod(x, L) = x; the signs differ, so r = x + L (rounded)
// anything else (|x| >= 2L, x = -L, NaN) goes through fmod.
template <typename T>
__device__ __forceinline__ T box_to_mesh(T x, T box, T cell) {
  T r;
  if (x >= T(0) && x < box) {
    r = x;
  } else if (x >= box && x < T(2) * box) {
    r = x - box;
  } else if (x < T(0) && x > -box) {
    r = x + box;
  } else {
    r = fmod(x, box);
    if (r != T(0) && ((r < T(0)) != (box < T(0)))) r = r + box;
  }
  return r / cell;
}

// The same prelude with r * (N/L) instead of r / (L/N): one rounding more
// (q within one ulp of box_to_mesh's), no division.  For kernels whose
// results are compared within a tolerance (the fused step): the CIC weights
// are continuous in q, so painted and gathered values move by a few ulps.
// The cell (floor q) is box_to_mesh's for every float r when L/N = 25/16;
// with other cell sizes it can be one lower or higher for r on a cell
// boundary, where the weight moved across is an ulp of q.
__device__ __forceinline__ float box_to_mesh_fast(float x, float box, float inv_cell) {
  float r;
  if (x >= 0.f && x < box) {
    r = x;
  } else if (x >= box && x < 2.f * box) {
    r = x - box;
  } else if (x < 0.f && x > -box) {
    r = x + box;
  } else {
    r = fmodf(x, box);
    if (r != 0.f && ((r < 0.f) != (box < 0.f))) r = r + box;
  }
  return r * inv_cell;
}

// IEEE round-to-nearest products/sums without FMA contraction, so that the
// CIC weights and readout sums follow the reference's operation order
// (lib/parops_fast.h:376-409, 442-478) bit for bit.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// The eight CIC corners of one particle, in the order the reference visits
// them (lib/parops_fast.h:402-409): (i,j,k) (i+1,j,k) (i,j+1,k) (i,j,k+1)
// (i+1,j+1,k) (i+1,j,k+1) (i,j+1,k+1) (i+1,j+1,k+1).
// `lo[a]` / `hi[a]` are the per-axis weights of the lower / upper corner
// (t = 1-d and d in the reference), `ok_lo[a]` / `ok_hi[a]` the validity
// flags (inx.. / inpx..) and `cell_lo[a]` / `cell_hi[a]` the wrapped
// indices.  At world size one the rank edges are [0, N) on every axis.
// Offsets are 32-bit: the CIC entry points require Nx*Ny*Nz < 2^32.
template <typename T>
struct Corners {
  uint32_t o[3][2];  // per-axis offset (index * stride) of the lower / upper corner
  bool ok[3][2];     // per-axis validity flags (inx / inpx ...)
  T d[3];            // fractional offsets p - int(p)
};

template <typename T>
__device__ __forceinline__ void cic_corners(const T p[3], const Grid3& g,
                                            Corners<T>& c) {
  const int n[3] = {g.nx, g.ny, g.nz};
  const uint32_t st[3] = {(uint32_t)g.sx, (uint32_t)g.sy, 1u};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int i = (int)p[a];                 // C++ int(): truncation toward zero
    c.d[a] = sub_rn(p[a], (T)i);
    int lo, hi;
    if ((unsigned)i < (unsigned)n[a]) {  // in range: i % n = i, (i+1) % n = i+1 or 0
      lo = i;
      hi = (i + 1 == n[a]) ? 0 : i + 1;
      c.ok[a][0] = true;
      c.ok[a][1] = true;
    } else {                             // C remainder semantics of the reference
      int ip1 = (i + 1) % n[a];
      c.ok[a][0] = false;
      c.ok[a][1] = (unsigned)ip1 < (unsigned)n[a];
      lo = abs(i % n[a]);
      hi = abs(ip1 % n[a]);
    }
    c.o[a][0] = (uint32_t)lo * st[a];
    c.o[a][1] = (uint32_t)hi * st[a];
  }
}

// cic_corners for a point known to lie inside the mesh (0 <= int(p) < n on
// every axis): the same offsets, every corner valid.
template <typename T>
__device__ __forceinline__ void cic_corners_inrange(const T p[3], const Grid3& g, Corners<T>& c) {
  const int n[3] = {g.nx, g.ny, g.nz};
  const uint32_t st[3] = {(uint32_t)g.sx, (uint32_t)g.sy, 1u};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int i = (int)p[a];
    c.d[a] = sub_rn(p[a], (T)i);
    c.o[a][0] = (uint32_t)i * st[a];
    c.o[a][1] = (uint32_t)(i + 1 == n[a] ? 0 : i + 1) * st[a];
    c.ok[a][0] = c.ok[a][1] = true;
  }
}

// Flattened cell offset of corner q (0..7, reference order).
__device__ __forceinline__ int corner_axis_bits(int q) {
  // bit a set => upper corner along axis a
  // order: 000 100 010 001 110 101 011 111 (x is bit 0)
  const int tab = (0) | (1 << 3) | (2 << 6) | (4 << 9) | (3 << 12) | (5 << 15) |
                  (6 << 18) | (7 << 21);
  return (tab >> (3 * q)) & 7;
}

template <typename T>
__device__ __forceinline__ uint32_t corner_offset(const Corners<T>& c, int bits,
                                                  const Grid3&) {
  return c.o[0][bits & 1] + c.o[1][(bits >> 1) & 1] + c.o[2][(bits >> 2) & 1];
}

template <typename T>
__device__ __forceinline__ bool corner_ok(const Corners<T>& c, int bits) {
  return c.ok[0][bits & 1] && c.ok[1][(bits >> 1) & 1] && c.ok[2][(bits >> 2) & 1];
}

// Pairing of neighbouring particles for scatters.  A warp takes 32
// consecutive particles.  A particle whose stencil does not wrap on any
// axis gets the key "offset of its lower corner", others kNoPair.  If lane
// l has key K and lane l-1 key K-1, lane l-1's upper-z face (corners 001
// 101 011 111) is lane l's lower-z face (000 100 010 110): lane l adds those
// four values to its own and lane l-1 skips their atomics.  Every value is
// added by exactly one lane, so the result never depends on the pairing
// rate; particles in lattice order (z fastest) pair most of the time, which
// removes about half of their atomics.
constexpr uint32_t kNoPair = 0xffffffffu;

template <typename T>
__device__ __forceinline__ uint32_t pair_key(const Corners<T>& c, const Grid3& g) {
  const bool canon = c.o[0][1] == c.o[0][0] + (uint32_t)g.sx && c.o[1][1] == c.o[1][0] + (uint32_t)g.sy &&
                     c.o[2][1] == c.o[2][0] + 1u;
  return canon ? c.o[0][0] + c.o[1][0] + c.o[2][0] : kNoPair;
}

struct Pairing {
  bool tz, gz;    // takes / gives the upper-z face
};

// Warp-collective (all 32 lanes): lane l absorbs lane l-1's upper-z face.
__device__ __forceinline__ Pairing zpair32_flags(uint32_t key) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t kz = __shfl_up_sync(full, key, 1);
  Pairing p;
  p.tz = lane > 0 && key != kNoPair && kz != kNoPair && key == kz + 1u;
  const unsigned bz = __ballot_sync(full, p.tz);
  p.gz = lane < 31 && ((bz >> (lane + 1)) & 1u);
  return p;
}

// Reference corner order k -> axis bits (x = bit 0): the upper-z corners
// k = 3, 5, 6, 7 pair with the lower-z corners k = 0, 1, 2, 4.
__device__ __forceinline__ constexpr int zpair_hi(int j) { return j == 0 ? 3 : j == 1 ? 5 : j == 2 ? 6 : 7; }
__device__ __forceinline__ constexpr int zpair_lo(int j) { return j == 0 ? 0 : j == 1 ? 1 : j == 2 ? 2 : 4; }

// Whether corner k is still added by this lane after pairing.
__device__ __forceinline__ bool pair_keeps(const Pairing& p, int k) {
  return (k == 0 || k == 1 || k == 2 || k == 4) ? true : !p.gz;
}

}  // namespace jld
