// Pipelined (TMA-staged, persistent) versions of the fused LDL step's strided
// spectral passes over the main block; see ldl_kernels.cuh for the math of
// each pass and pipe_passes.cuh for the staging scheme.  The nyq plane keeps
// the generic kernels.
#pragma once

#include "ldl_kernels.cuh"
#include "pipe_passes.cuh"

namespace jld {

// Column indices of the current x-pass tile: (ky, kz) of columns c < cols.
__device__ __forceinline__ void xcols(const SGeom& g, int t, int* ky, int* kz, int tid) {
  if (tid < g.cols) {
    const int col = (t << g.cshift) + tid;
    ky[tid] = col / g.h;
    kz[tid] = col - ky[tid] * g.h;
  }
}

// Forward x pass: S = FFT_x(A) (kept for the adjoint), P = 1e-2 alpha G S / Nc,
// T0 = iFFT_x(P), T1 = iFFT_x(-i c_x P).
template <class Sch, bool HI = false>
__global__ void __launch_bounds__(512, Sch::E == 8 ? 2 : 1)
xfilt_pipe_kernel(const __grid_constant__ CUtensorMap mA, SGeom g, KTables kt, const float* __restrict__ params,
                  int kind, float scale, float2* __restrict__ S, float2* __restrict__ T0,
                  float2* __restrict__ T1, const float2* __restrict__ tw, int* err,
                  const float2* __restrict__ S2, int* tick) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int cky[64], ckz[64];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int tile_elems = g.lines * g.cols;
  PipeSmem s = pipe_smem(smraw, tile_elems, 1, 1);
  if (tid == 0) { mbar_init(s.bar, 1); mbar_fence_init(); }
  __syncthreads();
  __shared__ int s_next;
  int t = blockIdx.x;
  if (tid == 0 && t < g.ntiles) issue_tile<0>(&mA, s.slot[0], s.bar, g, t);
  const float alpha = __ldg(params + 0), kh = __ldg(params + 2), kl = __ldg(params + 3), nu = __ldg(params + 4);
  const float a = pot_coef(kind) * alpha * scale;
  ColWork wk{s.work, g.cols};
  ColWork ac{s.acc, g.cols};
  for (int i = 0; t < g.ntiles; ++i) {
    bool ok = mbar_wait_bounded(s.bar, (uint32_t)(i & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 2); return; }
    xcols(g, t, cky, ckz, tid);
    const int64_t base = tile_base<0>(g, t);
    const float2* slot = s.slot[0];
    auto in = [&](int c, int j) { return slot[j * g.cols + c]; };
    auto keep = [&](int c, int j, float2 v) {
      S[base + c + (int64_t)j * g.es] = v;
      ac.at(c, j) = v;
    };
    auto rel = [&]() {
      if (tid == 0) {
        const int nt = next_tile(tick, t);
        s_next = nt;
        if (nt < g.ntiles) { fence_proxy_async_smem(); issue_tile<0>(&mA, s.slot[0], s.bar, g, nt); }
      }
    };
    p2_run_rel<Sch, true>(wk, in, keep, rel, tw, -1, g.cshift, tid, nthr);
    __syncthreads();
    for (int f = tid; f < tile_elems; f += nthr) {
      const int c = f & (g.cols - 1), j = f >> g.cshift;
      Green gr = green_fn(__ldg(kt.kx + j), __ldg(kt.ky + cky[c]), __ldg(kt.kz + ckz[c]), kind, kh, kl, nu);
      const float m = a * gr.g;
      float2 v = ac.at(c, j);
      float2 p = make_float2(v.x * m, v.y * m);
      if (HI) hi_add_src2(p, S2[base + c + (int64_t)j * g.es], params, scale, __ldg(kt.kx + j),
                          __ldg(kt.ky + cky[c]), __ldg(kt.kz + ckz[c]));
      ac.at(c, j) = p;
    }
    __syncthreads();
    auto inP = [&](int c, int j) { return ac.at(c, j); };
    auto st0 = [&](int c, int j, float2 v) { T0[base + c + (int64_t)j * g.es] = v; };
    p2_run<Sch, true>(wk, inP, st0, tw, +1, g.cshift, tid, nthr);
    __syncthreads();
    auto inQ = [&](int c, int j) {
      float2 p = ac.at(c, j);
      const float cx = __ldg(kt.cx + j);
      return make_float2(p.y * cx, -p.x * cx);
    };
    auto st1 = [&](int c, int j, float2 v) { T1[base + c + (int64_t)j * g.es] = v; };
    p2_run<Sch, true>(wk, inQ, st1, tw, +1, g.cshift, tid, nthr);
    __syncthreads();
    t = s_next;
  }
}

// Forward inverse y pass: Gy = iFFT_y(-i c_y T0), Gz = -i c_z iFFT_y(T0),
// Gx = iFFT_y(T1).  Items per tile: T0, T1.
template <class Sch>
__global__ void __launch_bounds__(512)
yinv3_pipe_kernel(const __grid_constant__ CUtensorMap mT0, const __grid_constant__ CUtensorMap mT1, SGeom g,
                  KTables kt, float2* __restrict__ Gx, float2* __restrict__ Gy, float2* __restrict__ Gz,
                  const float2* __restrict__ tw, int* err, int* tick) {
  extern __shared__ __align__(128) unsigned char smraw[];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int tile_elems = g.lines * g.cols;
  PipeSmem s = pipe_smem(smraw, tile_elems, 1, 0);
  if (tid == 0) { mbar_init(s.bar, 1); mbar_fence_init(); }
  __syncthreads();
  __shared__ int s_next;
  int t = blockIdx.x;
  if (tid == 0 && t < g.ntiles) issue_tile<1>(&mT0, s.slot[0], s.bar, g, t);
  ColWork wk{s.work, g.cols};
  const float2* slot = s.slot[0];
  int phase = 0;
  for (int i = 0; t < g.ntiles; ++i) {
    const int64_t base = tile_base<1>(g, t);
    const int kz0 = (int)(base % g.h);
    // item T0
    bool ok = mbar_wait_bounded(s.bar, (uint32_t)(phase++ & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 3); return; }
    auto inY = [&](int c, int j) {
      float2 v = slot[j * g.cols + c];
      const float cy = __ldg(kt.cy + j);
      return make_float2(v.y * cy, -v.x * cy);
    };
    auto stY = [&](int c, int j, float2 v) { Gy[base + c + (int64_t)j * g.es] = v; };
    p2_run<Sch, true>(wk, inY, stY, tw, +1, g.cshift, tid, nthr);
    __syncthreads();
    auto in0 = [&](int c, int j) { return slot[j * g.cols + c]; };
    auto stZ = [&](int c, int j, float2 v) {
      const float cz = __ldg(kt.cz + kz0 + c);
      Gz[base + c + (int64_t)j * g.es] = make_float2(v.y * cz, -v.x * cz);
    };
    auto relT1 = [&]() {
      if (tid == 0) { fence_proxy_async_smem(); issue_tile<1>(&mT1, s.slot[0], s.bar, g, t); }
    };
    p2_run_rel<Sch, true>(wk, in0, stZ, relT1, tw, +1, g.cshift, tid, nthr);
    __syncthreads();
    // item T1
    ok = mbar_wait_bounded(s.bar, (uint32_t)(phase++ & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 3); return; }
    auto stX = [&](int c, int j, float2 v) { Gx[base + c + (int64_t)j * g.es] = v; };
    auto relN = [&]() {
      if (tid == 0) {
        const int nt = next_tile(tick, t);
        s_next = nt;
        if (nt < g.ntiles) { fence_proxy_async_smem(); issue_tile<1>(&mT0, s.slot[0], s.bar, g, nt); }
      }
    };
    p2_run_rel<Sch, true>(wk, in0, stX, relN, tw, +1, g.cshift, tid, nthr);
    __syncthreads();    t = s_next;
  }
}

// Adjoint y pass: Bx = FFT_y(Ax) (in place), D = c_y FFT_y(Ay) + FFT_y(Az').
// Items per tile: Ax, Ay, Az'.
template <class Sch>
__global__ void __launch_bounds__(512)
yfwd_comb_pipe_kernel(const __grid_constant__ CUtensorMap mAx, const __grid_constant__ CUtensorMap mAy,
                      const __grid_constant__ CUtensorMap mAz, SGeom g, KTables kt, float2* __restrict__ Bx,
                      float2* __restrict__ D, const float2* __restrict__ tw, int* err, int* tick) {
  extern __shared__ __align__(128) unsigned char smraw[];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int tile_elems = g.lines * g.cols;
  PipeSmem s = pipe_smem(smraw, tile_elems, 1, 1);
  if (tid == 0) { mbar_init(s.bar, 1); mbar_fence_init(); }
  __syncthreads();
  __shared__ int s_next;
  int t = blockIdx.x;
  if (tid == 0 && t < g.ntiles) issue_tile<1>(&mAx, s.slot[0], s.bar, g, t);
  ColWork wk{s.work, g.cols};
  ColWork ac{s.acc, g.cols};
  const float2* slot = s.slot[0];
  auto in0 = [&](int c, int j) { return slot[j * g.cols + c]; };
  int phase = 0;
  for (int i = 0; t < g.ntiles; ++i) {
    const int64_t base = tile_base<1>(g, t);
    bool ok = mbar_wait_bounded(s.bar, (uint32_t)(phase++ & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 4); return; }
    auto stB = [&](int c, int j, float2 v) { Bx[base + c + (int64_t)j * g.es] = v; };
    auto relAy = [&]() { if (tid == 0) { fence_proxy_async_smem(); issue_tile<1>(&mAy, s.slot[0], s.bar, g, t); } };
    p2_run_rel<Sch, true>(wk, in0, stB, relAy, tw, -1, g.cshift, tid, nthr);
    __syncthreads();
    ok = mbar_wait_bounded(s.bar, (uint32_t)(phase++ & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 4); return; }
    auto stAcc = [&](int c, int j, float2 v) {
      const float cy = __ldg(kt.cy + j);
      ac.at(c, j) = make_float2(v.x * cy, v.y * cy);
    };
    auto relAz = [&]() { if (tid == 0) { fence_proxy_async_smem(); issue_tile<1>(&mAz, s.slot[0], s.bar, g, t); } };
    p2_run_rel<Sch, true>(wk, in0, stAcc, relAz, tw, -1, g.cshift, tid, nthr);
    __syncthreads();
    ok = mbar_wait_bounded(s.bar, (uint32_t)(phase++ & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 4); return; }
    auto stD = [&](int c, int j, float2 v) {
      float2 u = ac.at(c, j);
      D[base + c + (int64_t)j * g.es] = make_float2(u.x + v.x, u.y + v.y);
    };
    auto relN = [&]() {
      if (tid == 0) {
        const int nt = next_tile(tick, t);
        s_next = nt;
        if (nt < g.ntiles) { fence_proxy_async_smem(); issue_tile<1>(&mAx, s.slot[0], s.bar, g, nt); }
      }
    };
    p2_run_rel<Sch, true>(wk, in0, stD, relN, tw, -1, g.cshift, tid, nthr);
    __syncthreads();    t = s_next;
  }
}

// Adjoint x pass with the parameter-gradient reductions; items per tile:
// Bx, D, S.  Partials per block: [d alpha, d kh, d kl, d nu].
template <class Sch, bool HI = false>
__global__ void __launch_bounds__(512, Sch::E == 8 ? 2 : 1)
xbwd_pipe_kernel(const __grid_constant__ CUtensorMap mBx, const __grid_constant__ CUtensorMap mD,
                 const __grid_constant__ CUtensorMap mS, SGeom g, KTables kt, const float* __restrict__ params,
                 int kind, int mode, float scale, float2* __restrict__ Vout, double* __restrict__ partials,
                 const float2* __restrict__ tw, int* err, float2* __restrict__ Wout, int* tick) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int cky[64], ckz[64];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int tile_elems = g.lines * g.cols;
  PipeSmem s = pipe_smem(smraw, tile_elems, 1, 1);
  if (tid == 0) { mbar_init(s.bar, 1); mbar_fence_init(); }
  __syncthreads();
  __shared__ int s_next;
  int t = blockIdx.x;
  if (tid == 0 && t < g.ntiles) issue_tile<0>(&mBx, s.slot[0], s.bar, g, t);
  const float alpha = __ldg(params + 0), kh = __ldg(params + 2), kl = __ldg(params + 3), nu = __ldg(params + 4);
  const float pc = pot_coef(kind);
  const float a1 = pc * scale;
  const float vm0 = pc * alpha * scale;
  const int nz = 2 * g.h;
  ColWork wk{s.work, g.cols};
  ColWork ac{s.acc, g.cols};
  const float2* slot = s.slot[0];
  auto in0 = [&](int c, int j) { return slot[j * g.cols + c]; };
  KahanF acc[4];
  int phase = 0;
  bool failed = false;
  for (int i = 0; t < g.ntiles && !failed; ++i) {
    const int64_t base = tile_base<0>(g, t);
    bool ok = mbar_wait_bounded(s.bar, (uint32_t)(phase++ & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 5); failed = true; break; }
    xcols(g, t, cky, ckz, tid);
    auto stB = [&](int c, int j, float2 v) {
      const float cx = __ldg(kt.cx + j);
      ac.at(c, j) = make_float2(v.x * cx, v.y * cx);
    };
    auto relD = [&]() { if (tid == 0) { fence_proxy_async_smem(); issue_tile<0>(&mD, s.slot[0], s.bar, g, t); } };
    p2_run_rel<Sch, true>(wk, in0, stB, relD, tw, -1, g.cshift, tid, nthr);
    __syncthreads();
    ok = mbar_wait_bounded(s.bar, (uint32_t)(phase++ & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 5); failed = true; break; }
    auto stW = [&](int c, int j, float2 v) {
      float2 q = ac.at(c, j);
      q.x += v.x; q.y += v.y;
      ac.at(c, j) = make_float2(-q.y, q.x);  // W = i (c_x FFT(Bx) + FFT(D))
    };
    auto relS = [&]() { if (tid == 0) { fence_proxy_async_smem(); issue_tile<0>(&mS, s.slot[0], s.bar, g, t); } };
    p2_run_rel<Sch, true>(wk, in0, stW, relS, tw, -1, g.cshift, tid, nthr);
    __syncthreads();
    ok = mbar_wait_bounded(s.bar, (uint32_t)(phase++ & 1));
    if (!__syncthreads_and(ok)) { if (tid == 0) pipe_error(err, 5); failed = true; break; }
    for (int f = tid; f < tile_elems; f += nthr) {
      const int c = f & (g.cols - 1), j = f >> g.cshift;
      const int kz = ckz[c];
      const float2 W = ac.at(c, j);
      if (HI) Wout[base + c + (int64_t)j * g.es] = W;
      const float2 Sv = slot[j * g.cols + c];
      Green gr = green_fn(__ldg(kt.kx + j), __ldg(kt.ky + cky[c]), __ldg(kt.kz + kz), kind, kh, kl, nu);
      const float reWS = W.x * Sv.x + W.y * Sv.y;
      const float mk = (kz == 0 || (kz == g.h && (nz & 1) == 0)) ? 1.f : 2.f;
      const float m_alpha = mode == 1 ? mk : 1.f;
      const float m_green = mode == 1 ? mk : ((kz >= 1 && kz < g.ny / 2) ? 2.f : 1.f);
      acc[0].add(m_alpha * a1 * gr.g * reWS);
      const float qg = m_green * pc * alpha * scale * reWS;
      acc[1].add(qg * gr.dkh);
      acc[2].add(qg * gr.dkl);
      acc[3].add(qg * gr.dnu);
      const float vm = vm0 * gr.g;
      ac.at(c, j) = make_float2(W.x * vm, W.y * vm);
    }
    __syncthreads();
    if (tid == 0) {
      const int nt = next_tile(tick, t);
      s_next = nt;
      if (nt < g.ntiles) { fence_proxy_async_smem(); issue_tile<0>(&mBx, s.slot[0], s.bar, g, nt); }
    }
    auto inV = [&](int c, int j) { return ac.at(c, j); };
    auto stV = [&](int c, int j, float2 v) { Vout[base + c + (int64_t)j * g.es] = v; };
    p2_run<Sch, true>(wk, inV, stV, tw, +1, g.cshift, tid, nthr);
    __syncthreads();    t = s_next;
  }
  if (failed) return;
  block_reduce_kahan<4>(acc, partials, 4);
}

}  // namespace jld
