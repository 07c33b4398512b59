// Pipelined z (row) passes of the fused LDL step (the row-pass machinery is
// in zpipe_core.cuh): the c2r interleave of three force channels into the
// float4 mesh, the source-power adjoint with its reduction, and the r2c of
// the three cotangent channels of the float4 mesh.
#pragma once

#include "ldl_kernels.cuh"
#include "zpipe_core.cuh"

namespace jld {

// ---------------------------------------------------------------------------
// Inverse z pass of the forward: three c2r transforms (x, y, z force
// channels) interleaved into the float4 mesh g4[row][z] = (gx, gy, gz, 0).
// Lines 0..R-1 of a tile are channel x, R..2R-1 channel y, 2R..3R-1 z.
constexpr int kZc2r3Threads = 192;  // CTA size cap of its geometry
template <class Sch>
__global__ void __launch_bounds__(512)
zc2r3_pipe_kernel(const float2* __restrict__ Gx, const float2* __restrict__ Gy, const float2* __restrict__ Gz,
                  ZTile zt, const float2* __restrict__ twr, float4* __restrict__ g4,
                  const float2* __restrict__ tw, int* err, int* tick) {
  using Z = ZShape<Sch>;
  constexpr int H = Z::H;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int R = zt.R, L = 3 * zt.R;
  float2* slot = reinterpret_cast<float2*>(smraw);
  float2* nq = slot + L * H;
  float2* work = nq + L;
  uint64_t* bar = reinterpret_cast<uint64_t*>(work + L * Z::LDW);
  const int tid = threadIdx.x, nthr = blockDim.x;
  if (tid == 0) { mbar_init(bar, 1); mbar_fence_init(); }
  __syncthreads();
  const float2* src[3] = {Gx, Gy, Gz};
  __shared__ int s_next;
  int t = blockIdx.x;
  auto issue = [&](int t) {
    const uint32_t b0 = (uint32_t)R * H * 8u, b1 = (uint32_t)R * 8u;
    mbar_arrive_expect_tx(bar, 3u * (b0 + b1));
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      bulk_load_1d(slot + d * R * H, src[d] + (int64_t)t * R * H, b0, bar);
      bulk_load_1d(nq + d * R, src[d] + zt.nyq_off + (int64_t)t * R, b1, bar);
    }
  };
  if (tid == 0 && t < zt.ntiles) issue(t);
  RowWork<Z::PSH> wk{work, Z::LDW};
  for (int i = 0; t < zt.ntiles; ++i) {
    const bool ok = mbar_wait_bounded(bar, (uint32_t)(i & 1));
    if (!__syncthreads_and(ok)) {
      if (tid == 0 && err) atomicExch(err, 7);
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
    const int64_t row0 = (int64_t)t * R;
    for (int f = tid; f < R * H; f += nthr) {
      const int r = f / H, m = f - r * H;
      const float2 a = wk.at(r, m), b = wk.at(R + r, m), e = wk.at(2 * R + r, m);
      float4* o = g4 + (row0 + r) * (2 * (int64_t)H) + 2 * m;
      o[0] = make_float4(a.x, b.x, e.x, 0.f);
      o[1] = make_float4(a.y, b.y, e.y, 0.f);
    }
    __syncthreads();
    t = s_next;
  }
}

// ---------------------------------------------------------------------------
// Last adjoint z pass: c2r of the source cotangent V, then per real value
// rb = ct * gamma * base^(gamma-1) * fact (skipped when rb == nullptr) and
// the d gamma partial sum ct * base^gamma * log(base), base = fact*rho+1e-8.
// 128-thread CTAs capped at 80 registers, six per SM (at 128 registers
// four): 29.96 against 30.30 ms per 512^3 step; five (96 registers) 30.07.
constexpr int kZadjThreads = 128;
template <class Sch>
__global__ void __launch_bounds__(kZadjThreads, 6)
zc2r_adj_pipe_kernel(const float2* __restrict__ V, ZTile zt, const float2* __restrict__ twr,
                     const float* __restrict__ rho_paint, const float* __restrict__ params, float fact,
                     float* __restrict__ rb, double* __restrict__ partials, const float2* __restrict__ tw,
                     int* err, int* tick) {
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
  const float gamma = __ldg(params + 1);
  KahanF acc[1];
  for (int i = 0; t < zt.ntiles; ++i) {
    const bool ok = mbar_wait_bounded(bar, (uint32_t)(i & 1));
    if (!__syncthreads_and(ok)) {
      if (tid == 0 && err) atomicExch(err, 8);
      break;
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
    const int64_t e0 = (int64_t)t * R * 2 * H;
    for (int f = tid; f < R * H; f += nthr) {
      const int r = f / H, m = f - r * H;
      const float2 z = wk.at(r, m);
      const int64_t e = e0 + 2 * ((int64_t)r * H + m);
      const float2 rp = __ldg(reinterpret_cast<const float2*>(rho_paint + e));
      float o[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const float cts = q ? z.y : z.x;
        const float rho = __fmul_rn(q ? rp.y : rp.x, fact);
        const float base = __fadd_rn(rho, 1e-8f);
        float lb;
        const float s = pow_pos(base, gamma, &lb);
        acc[0].add(cts * s * lb);
        o[q] = cts * gamma * (s / base) * fact;
      }
      if (rb) *reinterpret_cast<float2*>(rb + e) = make_float2(o[0], o[1]);
    }
    __syncthreads();
    t = s_next;
  }
  block_reduce_kahan<1>(acc, partials, 1);
}

// ---------------------------------------------------------------------------
// First adjoint z pass: r2c of the three cotangent channels of the float4
// mesh gb4 (rows of 2h float4) into Ax, Ay and c_z(kz) * Az (main + nyq).
// Lines 0..R-1 of a tile are channel x, R..2R-1 channel y, 2R..3R-1 z; all
// three read the same staged float4 rows.
// 192-thread CTAs capped at 96 registers so that three fit per SM (at
// 128 registers only two did): 29.95 against 30.12 ms per 512^3 step.
constexpr int kZr2c3Threads = 192;
template <class Sch>
__global__ void __launch_bounds__(kZr2c3Threads, 3)
zr2c3_pipe_kernel(const float4* __restrict__ gb4, ZTile zt, const float2* __restrict__ twr,
                  const float* __restrict__ cz, float2* __restrict__ Ax, float2* __restrict__ Ay,
                  float2* __restrict__ Az, const float2* __restrict__ tw, int* err, int* tick) {
  using Z = ZShape<Sch>;
  constexpr int H = Z::H;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int R = zt.R;
  float4* slot = reinterpret_cast<float4*>(smraw);
  float2* work = reinterpret_cast<float2*>(slot + R * 2 * H);
  uint64_t* bar = reinterpret_cast<uint64_t*>(work + 3 * R * Z::LDW);
  const int tid = threadIdx.x, nthr = blockDim.x;
  if (tid == 0) { mbar_init(bar, 1); mbar_fence_init(); }
  __syncthreads();
  const uint32_t bytes = (uint32_t)R * 2 * H * 16u;
  __shared__ int s_next;
  int t = blockIdx.x;
  auto issue = [&](int t) {
    mbar_arrive_expect_tx(bar, bytes);
    bulk_load_1d(slot, gb4 + (int64_t)t * R * 2 * H, bytes, bar);
  };
  if (tid == 0 && t < zt.ntiles) issue(t);
  RowWork<Z::PSH> wk{work, Z::LDW};
  float2* dst[3] = {Ax, Ay, Az};
  for (int i = 0; t < zt.ntiles; ++i) {
    const bool ok = mbar_wait_bounded(bar, (uint32_t)(i & 1));
    if (!__syncthreads_and(ok)) {
      if (tid == 0 && err) atomicExch(err, 9);
      return;
    }
    auto in0 = [&](int c, int j) {
      const int d = c / R, r = c - d * R;
      const float4 a = slot[r * 2 * H + 2 * j], b = slot[r * 2 * H + 2 * j + 1];
      return d == 0 ? make_float2(a.x, b.x) : d == 1 ? make_float2(a.y, b.y) : make_float2(a.z, b.z);
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
    for (int f = tid; f < 3 * R * HH; f += nthr) {
      const int c = f / HH, k = f - c * HH;
      const int d = c / R, r = c - d * R;
      const int64_t row = row0 + r;
      const float2 z = wk.at(c, k);  // k <= H/2 < H
      const float2 zm = wk.at(c, k == 0 ? 0 : H - k);
      const float2 zc = make_float2(zm.x, -zm.y);
      const float2 xe = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y));
      const float2 dd = make_float2(0.5f * (z.x - zc.x), 0.5f * (z.y - zc.y));
      const float2 xo = make_float2(dd.y, -dd.x);
      const float2 w = __ldg(twr + k);
      const float2 wxo = make_float2(w.x * xo.x - w.y * xo.y, w.x * xo.y + w.y * xo.x);
      const float2 xk = make_float2(xe.x + wxo.x, xe.y + wxo.y);
      const float2 xhk = make_float2(xe.x - wxo.x, -(xe.y - wxo.y));
      const float s1 = d == 2 ? __ldg(cz + k) : 1.f;
      const float s2 = d == 2 ? __ldg(cz + (H - k)) : 1.f;
      float2* o = dst[d];
      o[row * H + k] = make_float2(xk.x * s1, xk.y * s1);
      if (k == 0) o[zt.nyq_off + row] = make_float2(xhk.x * s2, xhk.y * s2);
      else if (H - k != k) o[row * H + (H - k)] = make_float2(xhk.x * s2, xhk.y * s2);
    }
    __syncthreads();
    t = s_next;
  }
}

}  // namespace jld
