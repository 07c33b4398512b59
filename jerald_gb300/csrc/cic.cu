// Cloud-in-cell paint and readout on sm_103a.
//
// Device restatement of the single-rank CIC loops of the reference:
//   lpaint     lib/parops_fast.h:354-411    -> paint_kernel
//   lreadout   lib/parops_fast.h:414-481    -> readout_kernel
//   lpaint3D   lib/parops_fast.h:616-676    -> paint3_kernel
//   lreadout3D lib/parops_fast.h:730-821    -> readout3_kernel
// At world size one the decomposition/exchange/gather steps
// (lib/parops_fast.h:52-351) keep every particle local and in input order,
// so each kernel walks the caller's particle array directly.
//
// Paint scatters with global float/double atomics (red.global.add), one per
// corner.  The warp-aggregated variant first merges lanes of a warp that hit
// the same cell (__match_any_sync) so clustered inputs issue fewer atomics.
// Readouts gather the eight corners; weights and sums use explicit
// round-to-nearest intrinsics so they follow the reference's operation order.

#include <cstdlib>

#include "common.cuh"
#include "radix.cuh"

namespace jld {

template <typename T>
struct PosSrc {
  const T* pos;   // (N, 3) row-major
  T box[3];       // used when BOX
  T cell[3];      // box / N per axis, in T
  T inv[3];       // N / box per axis (fast prelude)
  int fast;       // 1: box_to_mesh_fast (the fused step's paints, float only)
};

template <typename T, bool BOX>
__device__ __forceinline__ void load_pos(const PosSrc<T>& s, int64_t p, T q[3]) {
  const T* src = s.pos + 3 * p;
  T x = __ldg(src), y = __ldg(src + 1), z = __ldg(src + 2);
  if (BOX) {
    if constexpr (sizeof(T) == 4) {
      if (s.fast) {
        q[0] = box_to_mesh_fast(x, s.box[0], s.inv[0]);
        q[1] = box_to_mesh_fast(y, s.box[1], s.inv[1]);
        q[2] = box_to_mesh_fast(z, s.box[2], s.inv[2]);
        return;
      }
    }
    q[0] = box_to_mesh(x, s.box[0], s.cell[0]);
    q[1] = box_to_mesh(y, s.box[1], s.cell[1]);
    q[2] = box_to_mesh(z, s.box[2], s.cell[2]);
  } else {
    q[0] = x; q[1] = y; q[2] = z;
  }
}

// Per-axis weights of corner `bits`: lower corner t = 1 - d, upper corner d.
template <typename T>
__device__ __forceinline__ T corner_weight(const T lo[3], const T hi[3], int bits) {
  T wx = (bits & 1) ? hi[0] : lo[0];
  T wy = (bits & 2) ? hi[1] : lo[1];
  T wz = (bits & 4) ? hi[2] : lo[2];
  return mul_rn(mul_rn(wx, wy), wz);
}

// ---------------------------------------------------------------------------
// Paint (single channel).  mass == nullptr => every particle weighs mscalar.
// Warps walk 32 consecutive particles at a time (all lanes stay in the loop
// for the shuffles); lanes whose stencils share a z face merge it before
// the atomics (zpair32_flags); batches whose stencils fall in a 4 x 4 x 4
// cell window (halo clumps) go through a shared-memory window instead.
// Also measured and slower here: a 16 x 2 lane layout that pairs y faces as
// well (a scalar atomic costs less than the extra shuffles and ballots), 8-
// and 16-byte vector atomics over the z runs, and 8 x 8 x 8 windows kept
// across a warp's batches.
// Six CTAs of 256 threads per SM in single precision (40 registers): on the
// 512^3 clustered step five and six tie, seven and eight (32 registers, full
// occupancy) are 0.7 ms slower, more warps queueing on the same atomics.
#ifndef JLD_PAINT_MIN_CTAS
#define JLD_PAINT_MIN_CTAS 6
#endif
// STAGED (float, 16-byte aligned positions and masses): each warp copies
// the positions (and masses) of its batches two batches ahead into its own
// shared-memory buffers with cp.async, so a batch's loads are in flight
// while the warp paints the batch before it (ncu on the unstaged paint at
// 256^3: long_scoreboard the top stall, DRAM at 21 % of peak).  A partial
// last batch reads global memory directly.  Measured slower than the
// unstaged kernel at 512^3 (1.82 against 1.68 ms); kept selectable.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// UNIT: every particle weighs exactly 1 (mass == nullptr, mscalar == 1): the
// product with the mass is the identity and is left out, and an invalid
// corner's weight is selected to 0 rather than multiplied by 0 (the same
// values: the weights are non-negative).  The paint is issue-bound (ncu at
// 256^3: 73 % of the issue slots busy), so the 16 multiplies per particle
// this saves matter.
template <typename T, bool BOX, bool STAGED = false, bool UNIT = false>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? JLD_PAINT_MIN_CTAS : 3)
paint_kernel(PosSrc<T> src, int64_t n, const T* __restrict__ mass, T mscalar,
             Grid3 g, T* __restrict__ out, int* tick) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  // Clumps: a batch whose lower corners span at most three cells per axis
  // adds its 8 x 32 corner values into a 4 x 4 x 4 shared-memory window
  // first; the window then goes to the mesh with one atomic per nonzero
  // cell, lanes on consecutive cells (few sectors per instruction, where
  // the lanes' own atomics would touch a dozen).
  __shared__ T wins[8][64];
  T* win = wins[threadIdx.x >> 5];
  // per warp, two buffers of 32 positions (96 floats) and 32 masses
  __shared__ __align__(16) float stage[STAGED ? 8 : 1][2][128];
  float* stg = stage[STAGED ? (threadIdx.x >> 5) : 0][0];
  const int nax[3] = {g.nx, g.ny, g.nz};
  // the staged copies run two batches ahead in the grid-stride order
  WarpBatches wb;
  const int64_t base0 = wb.first(STAGED ? nullptr : tick, n);
  const int64_t stride = 32 * WarpBatches::warps();
  auto issue = [&](int64_t b, int buf) {
    if (b + 32 <= n) {
      float* d = stg + buf * 128;
      if (lane < 24) cp_async16(d + 4 * lane, reinterpret_cast<const char*>(src.pos + 3 * b) + 16 * lane);
      else if (mass) cp_async16(d + 96 + 4 * (lane - 24), reinterpret_cast<const char*>(mass + b) + 16 * (lane - 24));
    }
    cp_async_commit();
  };
  if constexpr (STAGED) {
    issue(base0, 0);
    issue(base0 + stride, 1);
  }
  int kb = 0;
  for (int64_t base = base0; base < n; base = wb.next(base), ++kb) {
    const int64_t p = base + lane;
    const bool live = p < n;
    T q[3] = {T(0), T(0), T(0)};
    T m = T(0);
    if constexpr (STAGED) {
      cp_async_wait_1();
      __syncwarp();
      if (base + 32 <= n) {
        const float* d = stg + (kb & 1) * 128;
        const float x = d[3 * lane], y = d[3 * lane + 1], z = d[3 * lane + 2];
        if (BOX) {
          if (src.fast) {
            q[0] = box_to_mesh_fast(x, src.box[0], src.inv[0]);
            q[1] = box_to_mesh_fast(y, src.box[1], src.inv[1]);
            q[2] = box_to_mesh_fast(z, src.box[2], src.inv[2]);
          } else {
            q[0] = box_to_mesh(x, src.box[0], src.cell[0]);
            q[1] = box_to_mesh(y, src.box[1], src.cell[1]);
            q[2] = box_to_mesh(z, src.box[2], src.cell[2]);
          }
        } else {
          q[0] = x; q[1] = y; q[2] = z;
        }
        m = mass ? d[96 + lane] : mscalar;
      } else if (live) {
        load_pos<T, BOX>(src, p, q);
        m = mass ? __ldg(mass + p) : mscalar;
      }
      __syncwarp();
      issue(base + 2 * stride, kb & 1);
    } else if (live) {
      load_pos<T, BOX>(src, p, q);
      m = mass ? __ldg(mass + p) : mscalar;
    }
    // Batches whose 32 particles all lie inside the mesh (nearly all) take a
    // path without the per-corner validity flags that the reference's
    // out-of-range semantics need (the paint is issue-bound).
    bool inr_lane = live;
#pragma unroll
    for (int a = 0; a < 3; ++a) inr_lane = inr_lane && (unsigned)(int)q[a] < (unsigned)nax[a];
    auto scatter = [&](auto fast_tag) {
      constexpr bool FAST = decltype(fast_tag)::value;
      const bool lv = FAST || live;
      Corners<T> c;
      if constexpr (FAST) cic_corners_inrange(q, g, c);
      else cic_corners(q, g, c);
      T lo[3], hi[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) { hi[a] = c.d[a]; lo[a] = sub_rn(T(1), c.d[a]); }
      T w[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int bits = corner_axis_bits(k);
        if constexpr (FAST && UNIT) w[k] = corner_weight(lo, hi, bits);
        else if constexpr (FAST) w[k] = mul_rn(corner_weight(lo, hi, bits), m);
        else if constexpr (UNIT) w[k] = corner_ok(c, bits) ? corner_weight(lo, hi, bits) : T(0);
        else w[k] = mul_rn(mul_rn(corner_weight(lo, hi, bits), m), corner_ok(c, bits) ? T(1) : T(0));
      }
      // z span first: lattice-ordered batches (32 cells along z) leave here
      {
        unsigned mn[3], mx[3];
        int ii[3];
        bool clump = false;
        ii[2] = (int)q[2];
        mn[2] = __reduce_min_sync(full, lv ? (unsigned)ii[2] : 0xffffffffu);
        mx[2] = __reduce_max_sync(full, lv ? (unsigned)ii[2] : 0u);
        if (mx[2] - mn[2] <= 2u) {
          ii[0] = (int)q[0];
          ii[1] = (int)q[1];
#pragma unroll
          for (int a = 0; a < 2; ++a) {
            mn[a] = __reduce_min_sync(full, lv ? (unsigned)ii[a] : 0xffffffffu);
            mx[a] = __reduce_max_sync(full, lv ? (unsigned)ii[a] : 0u);
          }
          bool inr = FAST;
          if constexpr (!FAST) {
            inr = true;
#pragma unroll
            for (int a = 0; a < 3; ++a) inr = inr && (unsigned)ii[a] < (unsigned)nax[a];
            inr = __all_sync(full, inr || !live);
          }
          clump = inr && mx[0] - mn[0] <= 2u && mx[1] - mn[1] <= 2u;
        }
        if (clump) {
          win[lane] = T(0);
          win[lane + 32] = T(0);
          __syncwarp();
          if (lv) {
            const int wb = ((ii[0] - (int)mn[0]) * 4 + (ii[1] - (int)mn[1])) * 4 + (ii[2] - (int)mn[2]);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const int bits = corner_axis_bits(k);
              atomicAdd(win + wb + (bits & 1) * 16 + ((bits >> 1) & 1) * 4 + (bits >> 2), w[k]);
            }
          }
          __syncwarp();
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int sl = lane + 32 * h;
            const T v = win[sl];
            if (v != T(0)) {
              int gx = (int)mn[0] + (sl >> 4), gy = (int)mn[1] + ((sl >> 2) & 3), gz = (int)mn[2] + (sl & 3);
              if (gx >= g.nx) gx -= g.nx;
              if (gy >= g.ny) gy -= g.ny;
              if (gz >= g.nz) gz -= g.nz;
              atomicAdd(out + ((uint32_t)gx * (uint32_t)g.sx + (uint32_t)gy * (uint32_t)g.sy + (uint32_t)gz), v);
            }
          }
          __syncwarp();
          return;
        }
      }
      const Pairing pr = zpair32_flags(lv ? pair_key(c, g) : kNoPair);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const T t = __shfl_up_sync(full, w[zpair_hi(j)], 1);
        if (pr.tz) w[zpair_lo(j)] = add_rn(w[zpair_lo(j)], t);
      }
      if (lv) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (pair_keeps(pr, k)) atomicAdd(out + corner_offset(c, corner_axis_bits(k), g), w[k]);
      }
    };
    if (__all_sync(full, inr_lane)) scatter(std::true_type{});
    else scatter(std::false_type{});
  }
}

// Warp-aggregated paint: lanes of a warp whose corner falls in the same cell
// add their weights (in ascending lane order) and one leader lane issues the
// atomic.  Every lane of the warp runs the loop body so the warp-wide
// intrinsics see a full mask; out-of-range lanes carry weight 0 at cell -1.
template <typename T, bool BOX>
__global__ void __launch_bounds__(256)
paint_warpagg_kernel(PosSrc<T> src, int64_t n, const T* __restrict__ mass,
                     T mscalar, Grid3 g, T* __restrict__ out) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t base0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31);
  for (int64_t base = base0; base < n; base += stride) {
    int64_t p = base + lane;
    bool live = p < n;
    T q[3] = {T(0), T(0), T(0)};
    T m = T(0);
    if (live) {
      load_pos<T, BOX>(src, p, q);
      m = mass ? __ldg(mass + p) : mscalar;
    }
    Corners<T> c;
    cic_corners(q, g, c);
    T lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) { hi[a] = c.d[a]; lo[a] = sub_rn(T(1), c.d[a]); }
#pragma unroll 1
    for (int k = 0; k < 8; ++k) {
      int bits = corner_axis_bits(k);
      T w = mul_rn(corner_weight(lo, hi, bits), m);
      w = mul_rn(w, corner_ok(c, bits) ? T(1) : T(0));
      long long cell = live ? (long long)corner_offset(c, bits, g) : -1ll;
      unsigned peers = __match_any_sync(full, cell);
      int leader = __ffs(peers) - 1;
      T sum = T(0);
      unsigned rem = peers;
      while (__any_sync(full, rem != 0u)) {
        int srcl = rem ? (__ffs(rem) - 1) : lane;
        T t = __shfl_sync(full, w, srcl);
        if (rem) { sum = sum + t; rem &= rem - 1u; }
      }
      if (lane == leader && cell >= 0) atomicAdd(out + cell, sum);
    }
  }
}

// ---------------------------------------------------------------------------
// Three-channel paint: mass (N,3) row-major, out (3, C).
template <typename T, bool BOX>
__global__ void __launch_bounds__(256)
paint3_kernel(PosSrc<T> src, int64_t n, const T* __restrict__ mass, Grid3 g,
              T* __restrict__ out) {
  const int64_t C = g.cells();
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    T q[3];
    load_pos<T, BOX>(src, p, q);
    Corners<T> c;
    cic_corners(q, g, c);
    T lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) { hi[a] = c.d[a]; lo[a] = sub_rn(T(1), c.d[a]); }
    T m3[3] = {__ldg(mass + 3 * p), __ldg(mass + 3 * p + 1), __ldg(mass + 3 * p + 2)};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        int bits = corner_axis_bits(k);
        T w = mul_rn(corner_weight(lo, hi, bits), m3[d]);
        w = mul_rn(w, corner_ok(c, bits) ? T(1) : T(0));
        atomicAdd(out + d * C + corner_offset(c, bits, g), w);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Readout of one field; vjpdim in {-1, 0, 1, 2}.
template <typename T, bool BOX>
__global__ void __launch_bounds__(256)
readout_kernel(PosSrc<T> src, int64_t n, const T* __restrict__ field, Grid3 g,
               int vjpdim, T dweight, T* __restrict__ out) {
  // Two particles per iteration (p and p + S): their sixteen gathers are in
  // flight together, which matters for this latency-bound loop.
  const int64_t S = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p0 < n; p0 += 2 * S) {
    const int64_t pp[2] = {p0, p0 + S < n ? p0 + S : p0};
    Corners<T> c[2];
    T lo[2][3], hi[2][3], v[2][8];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      T q[3];
      load_pos<T, BOX>(src, pp[i], q);
      cic_corners(q, g, c[i]);
#pragma unroll
      for (int a = 0; a < 3; ++a) { hi[i][a] = c[i].d[a]; lo[i][a] = sub_rn(T(1), c[i].d[a]); }
      if (vjpdim >= 0) { hi[i][vjpdim] = dweight; lo[i][vjpdim] = -dweight; }
#pragma unroll
      for (int k = 0; k < 8; ++k) v[i][k] = __ldg(field + corner_offset(c[i], corner_axis_bits(k), g));
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      T acc = T(0);
      // a particle inside the mesh has every corner valid: the products
      // with the validity flag are the identity (bit for bit) and are left
      // out; others keep the reference's out-of-range semantics
      if (c[i].ok[0][0] && c[i].ok[1][0] && c[i].ok[2][0]) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const T t = mul_rn(corner_weight(lo[i], hi[i], corner_axis_bits(k)), v[i][k]);
          acc = (k == 0) ? t : add_rn(acc, t);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int bits = corner_axis_bits(k);
          T t = mul_rn(mul_rn(corner_weight(lo[i], hi[i], bits), v[i][k]), corner_ok(c[i], bits) ? T(1) : T(0));
          acc = (k == 0) ? t : add_rn(acc, t);
        }
      }
      if (i == 0 || p0 + S < n) out[pp[i]] = acc;
    }
  }
}

// Three-channel readout.  vjp == 0: out[p,d] reads channel d of a (3, C)
// field.  vjp == 1: out[p,d] is the weight gradient along d of one field.
template <typename T, bool BOX>
__global__ void __launch_bounds__(256)
readout3_kernel(PosSrc<T> src, int64_t n, const T* __restrict__ field, Grid3 g,
                int vjp, T dw0, T dw1, T dw2, T* __restrict__ out) {
  const int64_t C = g.cells();
  const T dw[3] = {dw0, dw1, dw2};
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    T q[3];
    load_pos<T, BOX>(src, p, q);
    Corners<T> c;
    cic_corners(q, g, c);
    T lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) { hi[a] = c.d[a]; lo[a] = sub_rn(T(1), c.d[a]); }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      T lo_d[3] = {lo[0], lo[1], lo[2]};
      T hi_d[3] = {hi[0], hi[1], hi[2]};
      const T* f = field;
      if (vjp) { hi_d[d] = dw[d]; lo_d[d] = -dw[d]; }
      else f = field + d * C;
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        int bits = corner_axis_bits(k);
        T v = __ldg(f + corner_offset(c, bits, g));
        T t = mul_rn(mul_rn(corner_weight(lo_d, hi_d, bits), v),
                     corner_ok(c, bits) ? T(1) : T(0));
        acc = (k == 0) ? t : add_rn(acc, t);
      }
      out[3 * p + d] = acc;
    }
  }
}

// ---------------------------------------------------------------------------
// Cell keys: flattened index of int(p) % N per axis, the key the reference's
// decomposition computes for each particle (lib/parops_fast.h:91-93).
template <typename T, bool BOX>
__global__ void __launch_bounds__(256)
keys_kernel(PosSrc<T> src, int64_t n, Grid3 g, int32_t* __restrict__ keys) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    T q[3];
    load_pos<T, BOX>(src, p, q);
    int i = (int)q[0] % g.nx, j = (int)q[1] % g.ny, k = (int)q[2] % g.nz;
    keys[p] = (int32_t)(((int64_t)i * g.ny + j) * g.nz + k);
  }
}

// ---------------------------------------------------------------------------
// Sort by cell key, and the paint that walks that order.
//
// The key of a particle is the reference's decomposition key, int(p) % N per
// axis flattened z fastest (lib/parops_fast.h:91-93), on positions that the
// box prelude (jaxpops_bind.py:161-164) has put in [0, N]: every key lies in
// [0, Nx*Ny*Nz).  radix.cuh sorts (key, particle index) pairs stably, so the
// order equals numpy.argsort(keys, kind="stable").
//
// Sorted paint: the particles of one cell form a run of equal keys.  A warp
// walks kSortedSpan consecutive sorted slots in rounds of 32 (lane = slot):
// each lane computes its particle's eight corner weights, a segmented
// shuffle scan sums them per run within the round (runs are contiguous
// lanes), and the lane that ends a run holds the run's sums.  A run that
// reaches past the round's last lane stays open and its sums are carried to
// the next round -- in FP64 once it holds kDenseRun particles, so a dense
// cell (halo cores hold thousands of particles) is summed in FP64 and
// rounded once, whatever its length; a run only splits where a warp's span
// ends.  FP64 arithmetic runs only in rounds that continue such a run
// (GB300 runs FP64 at a small fraction of its FP32 rate: a first version
// that converted every run's sums to FP64 took 13 ms at 512^3).  Each
// closed run adds its lower-z face to the mesh with one atomic per corner;
// its upper-z face goes into the next run's lower-z face when that run is
// the next cell of the same z row (the two faces are the same four cells),
// else to the mesh.  For particles in cell order the end lanes of a round's
// runs sit on consecutive cells, so its atomics touch a few 32-byte sectors
// (a thread-per-chunk version, whose lanes' atomics lay 8 cells apart, took
// 29 ms).  The corner cells of a run follow from any of its particles (all
// particles of a cell share them); the per-particle validity flags (the
// x mod L -> L edge, where int(p) = N) are applied to each particle's
// weights, as in lpaint.
constexpr int kSortedSpan = 32 * 64;
constexpr int kDenseRun = 32;

__device__ __forceinline__ unsigned lanemask_le() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_le;" : "=r"(m));
  return m;
}

template <bool BOX>
__global__ void __launch_bounds__(256)
sort_keys_kernel(PosSrc<float> src, int64_t n, Grid3 g, uint32_t* __restrict__ keys, int32_t* __restrict__ order) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    float q[3];
    load_pos<float, BOX>(src, p, q);
    const int i = (int)q[0] % g.nx, j = (int)q[1] % g.ny, k = (int)q[2] % g.nz;
    keys[p] = (uint32_t)(((int64_t)i * g.ny + j) * g.nz + k);
    order[p] = (int32_t)p;
  }
}

// Eight corner weights of one particle (index = bx | by << 1 | bz << 2),
// each the lpaint product of the three axis weights, the mass and the
// corner's validity flag; also the particle's corner offsets.
template <bool BOX>
__device__ __forceinline__ void particle_corners(const PosSrc<float>& src, int64_t p, const float* mass,
                                                 float mscalar, const Grid3& g, float w[8], Corners<float>& c) {
  float q[3];
  load_pos<float, BOX>(src, p, q);
  const float m = mass ? __ldg(mass + p) : mscalar;
  cic_corners(q, g, c);
  float lo[3], hi[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) { hi[a] = c.d[a]; lo[a] = sub_rn(1.f, c.d[a]); }
#pragma unroll
  for (int b = 0; b < 8; ++b) w[b] = mul_rn(mul_rn(corner_weight(lo, hi, b), m), corner_ok(c, b) ? 1.f : 0.f);
}

template <bool BOX>
__global__ void __launch_bounds__(256)
sorted_paint_kernel(PosSrc<float> src, const uint32_t* __restrict__ keys, const int32_t* __restrict__ order,
                    int64_t n, const float* __restrict__ mass, float mscalar, Grid3 g, float* __restrict__ out) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned le = lanemask_le();
  const uint32_t nz = (uint32_t)g.nz;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w0 = warp * kSortedSpan; w0 < n; w0 += nwarps * kSortedSpan) {
    const int64_t w1 = w0 + kSortedSpan < n ? w0 + kSortedSpan : n;
    // The open run carried from the previous round, the same in every lane:
    // key, corner offsets, particle count, and sums -- FP32 (pend_f) while
    // the run is shorter than kDenseRun particles, FP64 (pend_d) from then on.
    bool has_pend = false, pend_dense = false;
    uint32_t pend_key = 0u;
    int pend_cnt = 0;
    float pend_f[8];
    double pend_d[8];
    uint32_t pend_off[8];
#pragma unroll
    for (int b = 0; b < 8; ++b) { pend_f[b] = 0.f; pend_d[b] = 0.0; pend_off[b] = 0u; }
    for (int64_t base = w0; base < w1; base += 32) {
      const int64_t i = base + lane;
      const bool live = i < w1;
      const bool last_round = base + 32 >= w1;
      const uint32_t key = live ? __ldg(keys + i) : 0xffffffffu;
      float w[8];
      uint32_t off[8];
#pragma unroll
      for (int b = 0; b < 8; ++b) { w[b] = 0.f; off[b] = 0u; }
      if (live) {
        Corners<float> c;
        particle_corners<BOX>(src, __ldg(order + i), mass, mscalar, g, w, c);
#pragma unroll
        for (int b = 0; b < 8; ++b) off[b] = corner_offset(c, b, g);
      }
      const uint32_t kprev = __shfl_up_sync(full, key, 1);
      const bool head = live && (lane == 0 ? !(has_pend && pend_key == key) : kprev != key);
      const unsigned heads = __ballot_sync(full, head);
      const unsigned lives = __ballot_sync(full, live);
      const int last_live = 31 - __clz(lives);
      const unsigned hb = heads & le;
      const int sstart = hb ? 31 - __clz(hb) : -1;  // -1: this lane continues the open run
      const int s0 = sstart < 0 ? 0 : sstart;
      if (heads != lives) {  // some run covers more than one lane: segmented scan
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
          for (int b = 0; b < 8; ++b) {
            const float t = __shfl_up_sync(full, w[b], o);
            if (lane - o >= s0) w[b] = add_rn(w[b], t);
          }
        }
      }
      const bool next_head = lane < 31 && ((heads >> (lane + 1)) & 1u);
      const bool is_end = live && (lane == last_live || next_head);
      const uint32_t kn = __shfl_down_sync(full, key, 1);
      const bool chain_next = next_head && kn == key + 1u && (kn % nz) != 0u;
      const bool lane0_head = heads & 1u;
      const uint32_t key0 = __shfl_sync(full, key, 0);
      // upper face of the run ending at each lane (read by the next run)
      float up[4];
#pragma unroll
      for (int b = 0; b < 4; ++b) up[b] = w[b + 4];
      // 1. the open run closed before lane 0 (lane 0 starts another run):
      //    lanes 0..7 flush it, its upper face into lane 0's run when that
      //    is the next cell of the row
      bool chain0 = false;
      if (has_pend && lane0_head) {
        chain0 = key0 == pend_key + 1u && (key0 % nz) != 0u;
        float v = 0.f;
        if (pend_dense) {
#pragma unroll
          for (int b = 0; b < 8; ++b)
            if (lane == b) v = (float)pend_d[b];
#pragma unroll
          for (int b = 0; b < 4; ++b) pend_f[b + 4] = (float)pend_d[b + 4];
        } else {
#pragma unroll
          for (int b = 0; b < 8; ++b)
            if (lane == b) v = pend_f[b];
        }
        uint32_t o = pend_off[0];
#pragma unroll
        for (int b = 1; b < 8; ++b)
          if (lane == b) o = pend_off[b];
        if (lane < 8 && (lane < 4 || !chain0) && v != 0.f) atomicAdd(out + o, v);
      }
      // 2. lanes before the first head continue the open run, up to lane ce
      const bool has_cont = has_pend && !lane0_head;
      const unsigned before_head = heads ? ((1u << (__ffs(heads) - 1)) - 1u) : full;
      const unsigned cont_lanes = lives & before_head;
      const int ce = has_cont ? 31 - __clz(cont_lanes) : -1;
      const bool cont_open = has_cont && ce == last_live && !last_round;
      const int cnt_total = pend_cnt + ce + 1;
      const bool cont_dense = has_cont && (pend_dense || cnt_total >= kDenseRun);
      float cont_f[8];
      double cont_d[8];
#pragma unroll
      for (int b = 0; b < 8; ++b) { cont_f[b] = 0.f; cont_d[b] = 0.0; }
      if (has_cont) {
        float wc[8];
#pragma unroll
        for (int b = 0; b < 8; ++b) wc[b] = __shfl_sync(full, w[b], ce);
        if (cont_dense) {
#pragma unroll
          for (int b = 0; b < 8; ++b) {
            cont_d[b] = __dadd_rn(pend_dense ? pend_d[b] : (double)pend_f[b], (double)wc[b]);
            cont_f[b] = (float)cont_d[b];
          }
        } else {
#pragma unroll
          for (int b = 0; b < 8; ++b) cont_f[b] = add_rn(pend_f[b], wc[b]);
        }
        if (lane == ce) {
#pragma unroll
          for (int b = 0; b < 4; ++b) up[b] = cont_f[b + 4];
        }
        if (!cont_open) {  // the continued run closes at ce: lanes 0..7 flush it
          const bool cn = __shfl_sync(full, chain_next ? 1 : 0, ce) != 0;
          float v = 0.f;
#pragma unroll
          for (int b = 0; b < 8; ++b)
            if (lane == b) v = cont_f[b];
          uint32_t o = pend_off[0];
#pragma unroll
          for (int b = 1; b < 8; ++b)
            if (lane == b) o = pend_off[b];
          if (lane < 8 && (lane < 4 || !cn) && v != 0.f) atomicAdd(out + o, v);
        }
      }
      // 3. runs that start in this round: lower face (plus the previous
      //    run's upper face when chained), upper face unless chained onward
      const int pl = sstart > 0 ? sstart - 1 : 0;
      const uint32_t kp = __shfl_sync(full, key, pl);
      float pu[4];
#pragma unroll
      for (int b = 0; b < 4; ++b) pu[b] = __shfl_sync(full, up[b], pl);
      if (sstart >= 0) {
        const bool chain_prev = sstart > 0 ? (kp + 1u == key && (key % nz) != 0u) : chain0;
        if (chain_prev) {
#pragma unroll
          for (int b = 0; b < 4; ++b) w[b] = add_rn(w[b], sstart > 0 ? pu[b] : pend_f[b + 4]);
        }
      }
      const bool open = is_end && lane == last_live && !last_round && sstart >= 0;
      if (is_end && sstart >= 0 && !open) {
#pragma unroll
        for (int b = 0; b < 4; ++b)
          if (w[b] != 0.f) atomicAdd(out + off[b], w[b]);
        if (!chain_next) {
#pragma unroll
          for (int b = 4; b < 8; ++b)
            if (w[b] != 0.f) atomicAdd(out + off[b], w[b]);
        }
      }
      // 4. the run open at the round's end is carried
      if (cont_open) {
        pend_cnt = cnt_total;
        if (cont_dense) {
#pragma unroll
          for (int b = 0; b < 8; ++b) pend_d[b] = cont_d[b];
        } else {
#pragma unroll
          for (int b = 0; b < 8; ++b) pend_f[b] = cont_f[b];
        }
        pend_dense = cont_dense;
        has_pend = true;
      } else {
        const bool any_open = __shfl_sync(full, open ? 1 : 0, last_live) != 0;
        if (any_open) {
          pend_key = __shfl_sync(full, key, last_live);
          pend_cnt = last_live - __shfl_sync(full, sstart, last_live) + 1;
#pragma unroll
          for (int b = 0; b < 8; ++b) {
            pend_f[b] = __shfl_sync(full, w[b], last_live);
            pend_off[b] = __shfl_sync(full, off[b], last_live);
          }
          pend_dense = false;
        }
        has_pend = any_open;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Host side.

template <typename T>
static int check_common(const void* pos, int64_t nparts, const void* out,
                        int64_t nx, int64_t ny, int64_t nz, const char* who) {
  if (nparts < 0) return set_error(JLD_ERR_ARG, "%s: nparts < 0", who);
  if (nparts > 0 && !pos) return set_error(JLD_ERR_ARG, "%s: pos is NULL", who);
  if (!out) return set_error(JLD_ERR_ARG, "%s: output is NULL", who);
  if (nx <= 0 || ny <= 0 || nz <= 0)
    return set_error(JLD_ERR_ARG, "%s: mesh sizes must be positive", who);
  if (nx > (1 << 30) || ny > (1 << 30) || nz > (1 << 30) ||
      (double)nx * (double)ny * (double)nz >= 4294967296.0)
    return set_error(JLD_ERR_UNSUPPORTED, "%s: mesh too large (needs fewer than 2^32 cells)", who);
  return JLD_OK;
}

template <typename T>
static PosSrc<T> make_src(const T* pos, const T* box, int64_t nx, int64_t ny,
                          int64_t nz) {
  PosSrc<T> s;
  s.pos = pos;
  const int64_t n[3] = {nx, ny, nz};
  for (int a = 0; a < 3; ++a) {
    s.box[a] = box ? box[a] : T(1);
    s.cell[a] = box ? (T)(box[a] / (T)n[a]) : T(1);
    s.inv[a] = box ? (T)((T)n[a] / box[a]) : T(1);
  }
  s.fast = 0;
  return s;
}

template <typename T>
static int paint_impl(cudaStream_t st, const T* pos, int64_t nparts, const T* mass,
                      T mscalar, int64_t nx, int64_t ny, int64_t nz, const T* box,
                      int method, T* out, const char* who, bool fast = false, bool clear = true,
                      int* tick = nullptr) {
  int s = check_common<T>(pos, nparts, out, nx, ny, nz, who);
  if (s) return s;
  if (box && !(box[0] > 0 && box[1] > 0 && box[2] > 0))
    return set_error(JLD_ERR_ARG, "%s: box sizes must be positive", who);
  Grid3 g = make_grid(nx, ny, nz);
  if (clear) JLD_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(T) * g.cells(), st));
  if (nparts == 0) return JLD_OK;
  PosSrc<T> src = make_src<T>(pos, box, nx, ny, nz);
  src.fast = fast ? 1 : 0;
  const int block = 256;
  if (method == 1) {
    const unsigned grid = resident_grid(paint_warpagg_kernel<T, true>, nparts, block);
    if (box) paint_warpagg_kernel<T, true><<<grid, block, 0, st>>>(src, nparts, mass, mscalar, g, out);
    else paint_warpagg_kernel<T, false><<<grid, block, 0, st>>>(src, nparts, mass, mscalar, g, out);
  } else {
    // The cp.async-staged kernel measured slower at 512^3 (paint primitive
    // 1.82 against 1.68 ms, fused step 29.3 against 28.9 ms): the unstaged
    // kernel is the default; JLD_PAINT_STAGED=1 selects the staged one.
    static const bool use_staged = [] {
      const char* e = getenv("JLD_PAINT_STAGED");
      return e && e[0] == '1';
    }();
    bool staged = false;
    if constexpr (sizeof(T) == 4) {
      staged = use_staged && ((uintptr_t)pos & 15u) == 0 && ((uintptr_t)mass & 15u) == 0;
      if (staged) {
        const unsigned grid = resident_grid(paint_kernel<T, true, true>, nparts, block);
        if (box) paint_kernel<T, true, true><<<grid, block, 0, st>>>(src, nparts, mass, mscalar, g, out, nullptr);
        else paint_kernel<T, false, true><<<grid, block, 0, st>>>(src, nparts, mass, mscalar, g, out, nullptr);
      }
    }
    if (!staged) {
      const unsigned grid = resident_grid(paint_kernel<T, true>, nparts, block);
      if (!mass && mscalar == T(1)) {
        if (box) paint_kernel<T, true, false, true><<<grid, block, 0, st>>>(src, nparts, mass, mscalar, g, out, tick);
        else paint_kernel<T, false, false, true><<<grid, block, 0, st>>>(src, nparts, mass, mscalar, g, out, tick);
      } else {
        if (box) paint_kernel<T, true><<<grid, block, 0, st>>>(src, nparts, mass, mscalar, g, out, tick);
        else paint_kernel<T, false><<<grid, block, 0, st>>>(src, nparts, mass, mscalar, g, out, tick);
      }
    }
  }
  JLD_LAUNCH_CHECK(who);
  return JLD_OK;
}

template <typename T>
static int paint3_impl(cudaStream_t st, const T* pos, int64_t nparts, const T* mass,
                       int64_t nx, int64_t ny, int64_t nz, const T* box, T* out,
                       const char* who) {
  int s = check_common<T>(pos, nparts, out, nx, ny, nz, who);
  if (s) return s;
  if (nparts > 0 && !mass) return set_error(JLD_ERR_ARG, "%s: mass is NULL", who);
  Grid3 g = make_grid(nx, ny, nz);
  JLD_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(T) * 3 * g.cells(), st));
  if (nparts == 0) return JLD_OK;
  PosSrc<T> src = make_src<T>(pos, box, nx, ny, nz);
  const int block = 256;
  if (box) paint3_kernel<T, true><<<resident_grid(paint3_kernel<T, true>, nparts, block), block, 0, st>>>(src, nparts, mass, g, out);
  else paint3_kernel<T, false><<<resident_grid(paint3_kernel<T, false>, nparts, block), block, 0, st>>>(src, nparts, mass, g, out);
  JLD_LAUNCH_CHECK(who);
  return JLD_OK;
}

template <typename T>
static int readout_impl(cudaStream_t st, const T* pos, int64_t nparts, const T* field,
                        int64_t nx, int64_t ny, int64_t nz, const T* box, bool boxpos,
                        int vjpdim, T* out, const char* who) {
  int s = check_common<T>(pos, nparts, out, nx, ny, nz, who);
  if (s) return s;
  if (!field) return set_error(JLD_ERR_ARG, "%s: field is NULL", who);
  if (vjpdim < -1 || vjpdim > 2)
    return set_error(JLD_ERR_ARG, "%s: vjpdim must be between -1 and 2", who);
  if (vjpdim >= 0 && !box) return set_error(JLD_ERR_ARG, "%s: vjp needs box", who);
  if (nparts == 0) return JLD_OK;
  Grid3 g = make_grid(nx, ny, nz);
  PosSrc<T> src = make_src<T>(pos, box, nx, ny, nz);
  const int64_t nm[3] = {nx, ny, nz};
  T dweight = vjpdim >= 0 ? (T)((T)nm[vjpdim] / box[vjpdim]) : T(0);
  const int block = 256;
  if (boxpos) readout_kernel<T, true><<<resident_grid(readout_kernel<T, true>, nparts, block), block, 0, st>>>(src, nparts, field, g, vjpdim, dweight, out);
  else readout_kernel<T, false><<<resident_grid(readout_kernel<T, false>, nparts, block), block, 0, st>>>(src, nparts, field, g, vjpdim, dweight, out);
  JLD_LAUNCH_CHECK(who);
  return JLD_OK;
}

template <typename T>
static int readout3_impl(cudaStream_t st, const T* pos, int64_t nparts, const T* field,
                         int64_t nx, int64_t ny, int64_t nz, const T* box, bool boxpos,
                         int vjp, T* out, const char* who) {
  int s = check_common<T>(pos, nparts, out, nx, ny, nz, who);
  if (s) return s;
  if (!field) return set_error(JLD_ERR_ARG, "%s: field is NULL", who);
  if (vjp != 0 && vjp != 1) return set_error(JLD_ERR_ARG, "%s: vjp must be 0 or 1", who);
  if (!box) return set_error(JLD_ERR_ARG, "%s: box is NULL", who);
  if (nparts == 0) return JLD_OK;
  Grid3 g = make_grid(nx, ny, nz);
  PosSrc<T> src = make_src<T>(pos, box, nx, ny, nz);
  T dw[3];
  const int64_t nm[3] = {nx, ny, nz};
  for (int a = 0; a < 3; ++a) dw[a] = (T)((T)nm[a] / box[a]);
  const int block = 256;
  if (boxpos) readout3_kernel<T, true><<<resident_grid(readout3_kernel<T, true>, nparts, block), block, 0, st>>>(src, nparts, field, g, vjp, dw[0], dw[1], dw[2], out);
  else readout3_kernel<T, false><<<resident_grid(readout3_kernel<T, false>, nparts, block), block, 0, st>>>(src, nparts, field, g, vjp, dw[0], dw[1], dw[2], out);
  JLD_LAUNCH_CHECK(who);
  return JLD_OK;
}

int paint_unit_f32(cudaStream_t st, const float* pos, int64_t n, int64_t nx, int64_t ny,
                   int64_t nz, const float* box, int method, float* out, int* tick) {
  return paint_impl<float>(st, pos, n, nullptr, 1.0f, nx, ny, nz, box, method, out, "fused paint", true, true,
                           tick);
}

template <typename T>
static int keys_impl(cudaStream_t st, const T* pos, int64_t nparts, int64_t nx, int64_t ny,
                     int64_t nz, const T* box, int32_t* keys, const char* who) {
  int s = check_common<T>(pos, nparts, keys, nx, ny, nz, who);
  if (s) return s;
  if (nx * ny * nz > INT32_MAX) return set_error(JLD_ERR_UNSUPPORTED, "%s: mesh too large for int32 keys", who);
  if (nparts == 0) return JLD_OK;
  Grid3 g = make_grid(nx, ny, nz);
  PosSrc<T> src = make_src<T>(pos, box, nx, ny, nz);
  const int block = 256;
  if (box) keys_kernel<T, true><<<resident_grid(keys_kernel<T, true>, nparts, block), block, 0, st>>>(src, nparts, g, keys);
  else keys_kernel<T, false><<<resident_grid(keys_kernel<T, false>, nparts, block), block, 0, st>>>(src, nparts, g, keys);
  JLD_LAUNCH_CHECK(who);
  return JLD_OK;
}

static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

static size_t sorted_paint_ws(int64_t n) { return 2 * al256((size_t)n * 4) + radix_workspace(n); }

static int key_bits_of(int64_t cells) {
  int b = 1;
  while (b < 31 && ((int64_t)1 << b) < cells) ++b;
  return b;
}

static int cell_sort_impl(cudaStream_t st, const float* pos, int64_t n, int64_t nx, int64_t ny, int64_t nz,
                          const float* box, int32_t* keys, int32_t* order, void* ws, size_t wsb, const char* who) {
  int s = check_common<float>(pos, n, keys, nx, ny, nz, who);
  if (s) return s;
  if (!order) return set_error(JLD_ERR_ARG, "%s: order is NULL", who);
  if (!box || !(box[0] > 0 && box[1] > 0 && box[2] > 0))
    return set_error(JLD_ERR_ARG, "%s: box sizes must be positive", who);
  if (n >= INT32_MAX) return set_error(JLD_ERR_UNSUPPORTED, "%s: at most 2^31 - 2 particles", who);
  if (nx * ny * nz > INT32_MAX) return set_error(JLD_ERR_UNSUPPORTED, "%s: mesh too large for int32 keys", who);
  if (n == 0) return JLD_OK;
  if (n > 1 && (!ws || wsb < radix_workspace(n))) return set_error(JLD_ERR_WORKSPACE, "%s: workspace too small", who);
  Grid3 g = make_grid(nx, ny, nz);
  PosSrc<float> src = make_src<float>(pos, box, nx, ny, nz);
  sort_keys_kernel<true><<<resident_grid(sort_keys_kernel<true>, n, 256), 256, 0, st>>>(src, n, g, (uint32_t*)keys,
                                                                                       order);
  JLD_LAUNCH_CHECK(who);
  return radix_sort_pairs(st, (uint32_t*)keys, order, n, key_bits_of(g.cells()), ws, wsb, who);
}

static int sorted_paint_impl(cudaStream_t st, const float* pos, int64_t n, const float* mass, float ms, int64_t nx,
                             int64_t ny, int64_t nz, const float* box, const int32_t* keys, const int32_t* order,
                             float* out, const char* who) {
  int s = check_common<float>(pos, n, out, nx, ny, nz, who);
  if (s) return s;
  if (!box || !(box[0] > 0 && box[1] > 0 && box[2] > 0))
    return set_error(JLD_ERR_ARG, "%s: box sizes must be positive", who);
  if (n > 0 && (!keys || !order)) return set_error(JLD_ERR_ARG, "%s: keys or order is NULL", who);
  Grid3 g = make_grid(nx, ny, nz);
  JLD_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * g.cells(), st));
  if (n == 0) return JLD_OK;
  PosSrc<float> src = make_src<float>(pos, box, nx, ny, nz);
  const int64_t spans = (n + kSortedSpan - 1) / kSortedSpan;
  sorted_paint_kernel<true><<<resident_grid(sorted_paint_kernel<true>, 32 * spans, 256), 256, 0, st>>>(
      src, (const uint32_t*)keys, order, n, mass, ms, g, out);
  JLD_LAUNCH_CHECK(who);
  return JLD_OK;
}

}  // namespace jld

using namespace jld;

#define ST(s) reinterpret_cast<cudaStream_t>(s)

extern "C" {

int jld_ppaint_f32(jld_stream_t s, const float* pos, int64_t n, const float* mass,
                   int32_t nx, int32_t ny, int32_t nz, float* out) {
  clear_error();
  if (n > 0 && !mass) return set_error(JLD_ERR_ARG, "jld_ppaint_f32: mass is NULL");
  return paint_impl<float>(ST(s), pos, n, mass, 0.f, nx, ny, nz, nullptr, 0, out, "jld_ppaint_f32");
}
int jld_ppaint_f64(jld_stream_t s, const double* pos, int64_t n, const double* mass,
                   int64_t nx, int64_t ny, int64_t nz, double* out) {
  clear_error();
  if (n > 0 && !mass) return set_error(JLD_ERR_ARG, "jld_ppaint_f64: mass is NULL");
  return paint_impl<double>(ST(s), pos, n, mass, 0.0, nx, ny, nz, nullptr, 0, out, "jld_ppaint_f64");
}
int jld_ppaint_box_f32(jld_stream_t s, const float* pos, int64_t n, const float* mass,
                       float ms, int32_t nx, int32_t ny, int32_t nz, const float box[3],
                       float* out) {
  clear_error();
  if (!box) return set_error(JLD_ERR_ARG, "jld_ppaint_box_f32: box is NULL");
  return paint_impl<float>(ST(s), pos, n, mass, ms, nx, ny, nz, box, 0, out, "jld_ppaint_box_f32");
}
int jld_ppaint_box_acc_f32(jld_stream_t s, const float* pos, int64_t n, const float* mass,
                           float ms, int32_t nx, int32_t ny, int32_t nz, const float box[3],
                           float* out) {
  clear_error();
  if (!box) return set_error(JLD_ERR_ARG, "jld_ppaint_box_acc_f32: box is NULL");
  return paint_impl<float>(ST(s), pos, n, mass, ms, nx, ny, nz, box, 0, out, "jld_ppaint_box_acc_f32",
                           false, false);
}
int jld_ppaint_box_f64(jld_stream_t s, const double* pos, int64_t n, const double* mass,
                       double ms, int64_t nx, int64_t ny, int64_t nz, const double box[3],
                       double* out) {
  clear_error();
  if (!box) return set_error(JLD_ERR_ARG, "jld_ppaint_box_f64: box is NULL");
  return paint_impl<double>(ST(s), pos, n, mass, ms, nx, ny, nz, box, 0, out, "jld_ppaint_box_f64");
}
int jld_ppaint_box_method_f32(jld_stream_t s, const float* pos, int64_t n,
                              const float* mass, float ms, int32_t nx, int32_t ny,
                              int32_t nz, const float box[3], int32_t method, float* out) {
  clear_error();
  if (!box) return set_error(JLD_ERR_ARG, "jld_ppaint_box_method_f32: box is NULL");
  if (method != 0 && method != 1)
    return set_error(JLD_ERR_ARG, "jld_ppaint_box_method_f32: method must be 0 or 1");
  return paint_impl<float>(ST(s), pos, n, mass, ms, nx, ny, nz, box, method, out,
                           "jld_ppaint_box_method_f32");
}

size_t jld_cell_sort_workspace(int64_t nparts) { return nparts > 1 ? radix_workspace(nparts) : 0; }

int jld_cell_sort_f32(jld_stream_t s, const float* pos, int64_t n, int32_t nx, int32_t ny, int32_t nz,
                      const float box[3], int32_t* keys, int32_t* order, void* ws, size_t ws_bytes) {
  clear_error();
  return cell_sort_impl(ST(s), pos, n, nx, ny, nz, box, keys, order, ws, ws_bytes, "jld_cell_sort_f32");
}

int jld_ppaint_sorted_f32(jld_stream_t s, const float* pos, int64_t n, const float* mass, float ms, int32_t nx,
                          int32_t ny, int32_t nz, const float box[3], const int32_t* keys, const int32_t* order,
                          float* out) {
  clear_error();
  return sorted_paint_impl(ST(s), pos, n, mass, ms, nx, ny, nz, box, keys, order, out, "jld_ppaint_sorted_f32");
}

size_t jld_ppaint_box_sorted_workspace(int64_t nparts) { return nparts > 0 ? sorted_paint_ws(nparts) : 0; }

int jld_ppaint_box_sorted_f32(jld_stream_t s, const float* pos, int64_t n, const float* mass, float ms, int32_t nx,
                              int32_t ny, int32_t nz, const float box[3], float* out, void* ws, size_t ws_bytes) {
  clear_error();
  const char* who = "jld_ppaint_box_sorted_f32";
  if (n > 0 && (!ws || ws_bytes < sorted_paint_ws(n))) return set_error(JLD_ERR_WORKSPACE, "%s: workspace too small", who);
  if (n == 0) return sorted_paint_impl(ST(s), pos, n, mass, ms, nx, ny, nz, box, nullptr, nullptr, out, who);
  int32_t* keys = (int32_t*)ws;
  int32_t* order = (int32_t*)((char*)ws + al256((size_t)n * 4));
  void* rws = (char*)ws + 2 * al256((size_t)n * 4);
  int st = cell_sort_impl(ST(s), pos, n, nx, ny, nz, box, keys, order, rws, ws_bytes - 2 * al256((size_t)n * 4), who);
  if (st) return st;
  return sorted_paint_impl(ST(s), pos, n, mass, ms, nx, ny, nz, box, keys, order, out, who);
}

int jld_preadout_f32(jld_stream_t s, const float* pos, int64_t n, const float* field,
                     int32_t nx, int32_t ny, int32_t nz, const float box[3],
                     int32_t vjpdim, float* out) {
  clear_error();
  return readout_impl<float>(ST(s), pos, n, field, nx, ny, nz, box, false, vjpdim, out, "jld_preadout_f32");
}
int jld_preadout_f64(jld_stream_t s, const double* pos, int64_t n, const double* field,
                     int64_t nx, int64_t ny, int64_t nz, const double box[3],
                     int32_t vjpdim, double* out) {
  clear_error();
  return readout_impl<double>(ST(s), pos, n, field, nx, ny, nz, box, false, vjpdim, out, "jld_preadout_f64");
}
int jld_preadout_box_f32(jld_stream_t s, const float* pos, int64_t n, const float* field,
                         int32_t nx, int32_t ny, int32_t nz, const float box[3],
                         int32_t vjpdim, float* out) {
  clear_error();
  if (!box) return set_error(JLD_ERR_ARG, "jld_preadout_box_f32: box is NULL");
  return readout_impl<float>(ST(s), pos, n, field, nx, ny, nz, box, true, vjpdim, out, "jld_preadout_box_f32");
}
int jld_preadout_box_f64(jld_stream_t s, const double* pos, int64_t n, const double* field,
                         int64_t nx, int64_t ny, int64_t nz, const double box[3],
                         int32_t vjpdim, double* out) {
  clear_error();
  if (!box) return set_error(JLD_ERR_ARG, "jld_preadout_box_f64: box is NULL");
  return readout_impl<double>(ST(s), pos, n, field, nx, ny, nz, box, true, vjpdim, out, "jld_preadout_box_f64");
}

int jld_ppaint3d_f32(jld_stream_t s, const float* pos, int64_t n, const float* mass,
                     int32_t nx, int32_t ny, int32_t nz, float* out) {
  clear_error();
  return paint3_impl<float>(ST(s), pos, n, mass, nx, ny, nz, nullptr, out, "jld_ppaint3d_f32");
}
int jld_ppaint3d_f64(jld_stream_t s, const double* pos, int64_t n, const double* mass,
                     int64_t nx, int64_t ny, int64_t nz, double* out) {
  clear_error();
  return paint3_impl<double>(ST(s), pos, n, mass, nx, ny, nz, nullptr, out, "jld_ppaint3d_f64");
}
int jld_ppaint3d_box_f32(jld_stream_t s, const float* pos, int64_t n, const float* mass,
                         int32_t nx, int32_t ny, int32_t nz, const float box[3], float* out) {
  clear_error();
  if (!box) return set_error(JLD_ERR_ARG, "jld_ppaint3d_box_f32: box is NULL");
  return paint3_impl<float>(ST(s), pos, n, mass, nx, ny, nz, box, out, "jld_ppaint3d_box_f32");
}
int jld_ppaint3d_box_f64(jld_stream_t s, const double* pos, int64_t n, const double* mass,
                         int64_t nx, int64_t ny, int64_t nz, const double box[3], double* out) {
  clear_error();
  if (!box) return set_error(JLD_ERR_ARG, "jld_ppaint3d_box_f64: box is NULL");
  return paint3_impl<double>(ST(s), pos, n, mass, nx, ny, nz, box, out, "jld_ppaint3d_box_f64");
}

int jld_preadout3d_f32(jld_stream_t s, const float* pos, int64_t n, const float* field,
                       int32_t nx, int32_t ny, int32_t nz, const float box[3], int32_t vjp,
                       float* out) {
  clear_error();
  return readout3_impl<float>(ST(s), pos, n, field, nx, ny, nz, box, false, vjp, out, "jld_preadout3d_f32");
}
int jld_preadout3d_f64(jld_stream_t s, const double* pos, int64_t n, const double* field,
                       int64_t nx, int64_t ny, int64_t nz, const double box[3], int32_t vjp,
                       double* out) {
  clear_error();
  return readout3_impl<double>(ST(s), pos, n, field, nx, ny, nz, box, false, vjp, out, "jld_preadout3d_f64");
}
int jld_preadout3d_box_f32(jld_stream_t s, const float* pos, int64_t n, const float* field,
                           int32_t nx, int32_t ny, int32_t nz, const float box[3],
                           int32_t vjp, float* out) {
  clear_error();
  return readout3_impl<float>(ST(s), pos, n, field, nx, ny, nz, box, true, vjp, out, "jld_preadout3d_box_f32");
}
int jld_preadout3d_box_f64(jld_stream_t s, const double* pos, int64_t n, const double* field,
                           int64_t nx, int64_t ny, int64_t nz, const double box[3],
                           int32_t vjp, double* out) {
  clear_error();
  return readout3_impl<double>(ST(s), pos, n, field, nx, ny, nz, box, true, vjp, out, "jld_preadout3d_box_f64");
}

int jld_cell_keys_f32(jld_stream_t s, const float* pos, int64_t n, int32_t nx, int32_t ny,
                      int32_t nz, const float* box, int32_t* keys) {
  clear_error();
  return keys_impl<float>(ST(s), pos, n, nx, ny, nz, box, keys, "jld_cell_keys_f32");
}
int jld_cell_keys_f64(jld_stream_t s, const double* pos, int64_t n, int64_t nx, int64_t ny,
                      int64_t nz, const double* box, int32_t* keys) {
  clear_error();
  return keys_impl<double>(ST(s), pos, n, nx, ny, nz, box, keys, "jld_cell_keys_f64");
}

}  // extern "C"
