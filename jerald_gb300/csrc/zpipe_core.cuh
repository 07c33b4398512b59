// Pipelined z (row) passes for power-of-two half-row lengths h = nz/2
// (sm_103a): shared pieces and the real-to-complex row pass.
//
// A tile is R whole rows of one or more meshes.  Rows are contiguous, so a
// tile arrives by a few cp.async.bulk copies into one staging slot,
// completing on an mbarrier.  Persistent CTAs walk the tiles; the copy of a
// CTA's next tile is issued as soon as the first FFT stage has read the slot,
// so it overlaps the remaining stages, the epilogue and the global stores.
// The packed transform of length h runs with the j-fastest ("row") thread
// mapping: line c of the tile is worked on by h/16 consecutive threads.  Its
// last stage writes back into the work buffer, and an epilogue reads whole
// rows from there (the r2c split X[k], X[h-k] from Z[k], Z[h-k], or the c2r
// output of the caller's pass).
#pragma once

#include "fft_pipe.cuh"

namespace jld {

// Tile geometry of a z pass: `lines` = R rows per mesh x `nin` meshes.
struct ZTile {
  int R;          // rows per tile
  int ntiles;     // rows / R
  int64_t rows;   // nx * ny
  int64_t nyq_off;  // nyq plane offset from a main block (complex elements)
};

template <class Sch>
struct ZShape {
  static constexpr int H = Sch::n;
  static constexpr int PSH = clog2(Sch::rad[0]);
  static constexpr int LDW = H + (H >> PSH);
};

// Runs all stages of Sch with the row mapping, reading stage 0 from `in`
// and leaving the result in the work buffer (last stage in place).  `rel`
// runs once every thread is past its reads of `in`.
template <class Sch, class W, class In, class Rel>
__device__ __forceinline__ void p2_rows_to_work(const W& work, const In& in, const Rel& rel,
                                                const float2* __restrict__ tw, int sgn, int tid, int nthr) {
  auto wld = [&](int c, int j) { return work.at(c, j); };
  auto wst = [&](int c, int j, float2 v) { work.at(c, j) = v; };
  if constexpr (Sch::nst == 1) {
    p2_stage<Sch, 0, false, true>(in, wst, tw, sgn, 0, tid, nthr, rel);
  } else {
    p2_stage<Sch, 0, false, false>(in, wst, tw, sgn, 0, tid, nthr, NoRelease{});
    __syncthreads();
    rel();
    if constexpr (Sch::nst >= 3) {
      p2_stage<Sch, 1, false, true>(wld, wst, tw, sgn, 0, tid, nthr, NoRelease{});
      __syncthreads();
    }
    if constexpr (Sch::nst >= 4) {
      p2_stage<Sch, 2, false, true>(wld, wst, tw, sgn, 0, tid, nthr, NoRelease{});
      __syncthreads();
    }
    p2_stage<Sch, Sch::nst - 1, false, true>(wld, wst, tw, sgn, 0, tid, nthr, NoRelease{});
  }
}

// Packed c2r input Z'[k] of line c from a staged main tile (h per line) and
// its nyq values (the same construction as c2r_pack).
__device__ __forceinline__ float2 c2r_pack_tile(const float2* slot, const float2* nq, int h, int c, int k,
                                                const float2* __restrict__ twr) {
  float2 xk = slot[c * h + k];
  float2 xh = (k == 0) ? nq[c] : slot[c * h + (h - k)];
  if (k == 0) { xk.y = 0.f; xh.y = 0.f; }
  const float2 xc = make_float2(xh.x, -xh.y);
  const float2 a = make_float2(xk.x + xc.x, xk.y + xc.y);
  const float2 b = make_float2(xk.x - xc.x, xk.y - xc.y);
  float2 w = __ldg(twr + k);
  w.y = -w.y;
  const float2 t = make_float2(w.x * b.x - w.y * b.y, w.x * b.y + w.y * b.x);
  return make_float2(a.x - t.y, a.y + t.x);
}

// ---------------------------------------------------------------------------
// Forward z pass (r2c) of real rows with the source map applied on load:
// main[row][k] (k < h) and nyq[row] = X[h].
constexpr int kZr2cThreads = 256;  // CTA size cap of its geometry
template <class Sch, class Src>
__global__ void __launch_bounds__(512)
zr2c_pipe_kernel(const float* __restrict__ in, Src src, ZTile zt, const float2* __restrict__ twr,
                 float2* __restrict__ main, const float2* __restrict__ tw, int* err, int* tick) {
  using Z = ZShape<Sch>;
  constexpr int H = Z::H;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int R = zt.R;
  float2* slot = reinterpret_cast<float2*>(smraw);
  float2* work = slot + R * H;
  uint64_t* bar = reinterpret_cast<uint64_t*>(work + R * Z::LDW);
  const int tid = threadIdx.x, nthr = blockDim.x;
  if (tid == 0) { mbar_init(bar, 1); mbar_fence_init(); }
  __syncthreads();
  const uint32_t bytes = (uint32_t)R * H * 8u;
  __shared__ int s_next;
  int t = blockIdx.x;
  auto issue = [&](int t) {
    mbar_arrive_expect_tx(bar, bytes);
    bulk_load_1d(slot, in + (int64_t)t * R * 2 * H, bytes, bar);
  };
  if (tid == 0 && t < zt.ntiles) issue(t);
  RowWork<Z::PSH> wk{work, Z::LDW};
  float2* nyq = main + zt.nyq_off;
  for (int i = 0; t < zt.ntiles; ++i) {
    const bool ok = mbar_wait_bounded(bar, (uint32_t)(i & 1));
    if (!__syncthreads_and(ok)) {
      if (tid == 0 && err) atomicExch(err, 6);
      return;
    }
    const int64_t e0 = (int64_t)t * R * 2 * H;  // real index of the tile's first value
    auto in0 = [&](int c, int j) {
      float2 v = slot[c * H + j];
      const int64_t e = e0 + 2 * ((int64_t)c * H + j);
      v.x = src(v.x, e);
      v.y = src(v.y, e + 1);
      return v;
    };
    auto rel = [&]() {
      if (tid == 0) {
        const int nt = next_tile(tick, t);
        s_next = nt;
        if (nt < zt.ntiles) {
          fence_proxy_async_smem();
          issue(nt);
        }
      }
    };
    p2_rows_to_work<Sch>(wk, in0, rel, tw, -1, tid, nthr);
    __syncthreads();
    constexpr int HH = H / 2 + 1;
    const int64_t row0 = (int64_t)t * R;
    for (int f = tid; f < R * HH; f += nthr) {
      const int c = f / HH, k = f - c * HH;
      const int64_t row = row0 + c;
      const float2 z = wk.at(c, k);  // k <= H/2 < H
      const float2 zm = wk.at(c, k == 0 ? 0 : H - k);
      const float2 zc = make_float2(zm.x, -zm.y);
      const float2 xe = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y));
      const float2 dd = make_float2(0.5f * (z.x - zc.x), 0.5f * (z.y - zc.y));
      const float2 xo = make_float2(dd.y, -dd.x);
      const float2 w = __ldg(twr + k);
      const float2 wxo = make_float2(w.x * xo.x - w.y * xo.y, w.x * xo.y + w.y * xo.x);
      main[row * H + k] = make_float2(xe.x + wxo.x, xe.y + wxo.y);
      const float2 xhk = make_float2(xe.x - wxo.x, -(xe.y - wxo.y));
      if (k == 0) nyq[row] = xhk;
      else if (H - k != k) main[row * H + (H - k)] = xhk;
    }
    __syncthreads();
    t = s_next;
  }
}

// Identity source map (plain r2c).
struct SrcIdentity {
  __device__ __forceinline__ float operator()(float v, int64_t) const { return v; }
};

// Inverse z pass (c2r) of one mesh into real rows out[row][2h].
template <class Sch>
__global__ void __launch_bounds__(512)
zc2r_pipe_kernel(const float2* __restrict__ V, ZTile zt, const float2* __restrict__ twr, float* __restrict__ out,
                 const float2* __restrict__ tw, int* err, int* tick) {
  using Z = ZShape<Sch>;
  constexpr int H = Z::H;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int R = zt.R;
  float2* slot = reinterpret_cast<float2*>(smraw);
  float2* nq = slot + R * H;
  float2* work = nq + R;
  uint64_t* bar = reinterpret_cast<uint64_t*>(work + R * Z::LDW);
  const int tid = threadIdx.x, nthr = blockDim.x;
  if (tid == 0) { mbar_init(bar, 1); mbar_fence_init(); }
  __syncthreads();
  __shared__ int s_next;
  int t = blockIdx.x;
  auto issue = [&](int t) {
    const uint32_t b0 = (uint32_t)R * H * 8u, b1 = (uint32_t)R * 8u;
    mbar_arrive_expect_tx(bar, b0 + b1);
    bulk_load_1d(slot, V + (int64_t)t * R * H, b0, bar);
    bulk_load_1d(nq, V + zt.nyq_off + (int64_t)t * R, b1, bar);
  };
  if (tid == 0 && t < zt.ntiles) issue(t);
  RowWork<Z::PSH> wk{work, Z::LDW};
  for (int i = 0; t < zt.ntiles; ++i) {
    const bool ok = mbar_wait_bounded(bar, (uint32_t)(i & 1));
    if (!__syncthreads_and(ok)) {
      if (tid == 0 && err) atomicExch(err, 10);
      return;
    }
    auto in0 = [&](int c, int k) { return c2r_pack_tile(slot, nq, H, c, k, twr); };
    auto rel = [&]() {
      if (tid == 0) {
        const int nt = next_tile(tick, t);
        s_next = nt;
        if (nt < zt.ntiles) {
          fence_proxy_async_smem();
          issue(nt);
        }
      }
    };
    p2_rows_to_work<Sch>(wk, in0, rel, tw, +1, tid, nthr);
    __syncthreads();
    float2* o = reinterpret_cast<float2*>(out) + (int64_t)t * R * H;
    for (int f = tid; f < R * H; f += nthr) {
      const int r = f / H, m = f - r * H;
      o[f] = wk.at(r, m);
    }
    __syncthreads();
    t = s_next;
  }
}

}  // namespace jld
