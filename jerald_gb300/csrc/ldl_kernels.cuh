// Fused LDL forward + adjoint step on sm_103a (FP32 data, FP64 reductions).
//
// Forward of one layer (model.py:186-212 "sm", 137-179 "dm"):
//   paint      rho = paint(X) (unit mass)                          paint_kernel
//   zfwd       s = (fact*rho + 1e-8)^gamma fused into the z r2c     rfft_z_kernel<SourcePow>
//   yfwd       y FFT in place                                       line_pass_kernel
//   xfilt      x FFT -> S (kept for the adjoint); P = 1e-2 alpha G S / Nc;
//              T0 = iFFT_x(P), T1 = iFFT_x(-i c_x P)                xfilt_kernel
//   yinv3      Gy = iFFT_y(-i c_y T0), Gz = -i c_z iFFT_y(T0), Gx = iFFT_y(T1)
//   zinv3      three c2r rows -> float4 force mesh (gx, gy, gz, 0)  zinv3_kernel
//   update     X' = X + CIC gather of the force mesh                update_kernel
// Final map and loss (model.py:311-403): paint, loss_kernel (bias, ReLU,
// L1/L2 with mask, its cotangent and d/d(mu, w, b)), gather_vjp_kernel
// (folded into bwd_fused_kernel on the plain-atomic path).
// The pipelined (TMA / bulk-copy) versions of the FFT passes are in
// ldl_pipe.cuh and zpipe.cuh.
// Adjoint of one layer, given Xbar' (the cotangent of X'):
//   bwd_fused  Xbar' completed with the paint adjoint of the next layer's
//              density, then Xbar = Xbar' + sum_d Xbar'_d grad g_d(X) (gather
//              of the float4 force mesh with CIC weight gradients) and the
//              3-channel scatter gbar_d = paint(X, Xbar'_d) as one float4
//              vector atomic per corner
//   zfwd3      r2c of gbar_x, gbar_y, gbar_z; the z channel is multiplied by c_z
//   yfwd_comb  Bx = FFT_y(Ax), D = c_y FFT_y(Ay) + FFT_y(c_z Az)
//   xbwd       W = i (c_x FFT_x(Bx) + FFT_x(D)); reductions for d/d(alpha,
//              kh, kl, nu); V = 1e-2 alpha G W / Nc; iFFT_x(V)
//   yinv       iFFT_y in place
//   zinv_adj   ct_s = c2r(V); d/d gamma reduction; rhobar = fact * ct_s *
//              gamma (rho + 1e-8)^(gamma-1)
//   gather     Xbar += CIC weight-gradient gather of rhobar (paint's adjoint)
// The gradient convention is selectable: mode 0 follows the reference's VJP
// rules (jaxpops_bind.py:699-701, 758-759 and the c2f rule of model.py:23-29),
// mode 1 is the exact adjoint.  They differ only in d/d alpha (the reference's
// pifft rule omits the half-spectrum multiplicity).
//
// All parameters are read from device memory so that one captured CUDA graph
// serves every parameter vector.

#pragma once

#include <vector>
#include <cmath>
#include <mutex>
#include <map>
#include <tuple>

#include "fft_core.cuh"
#include "fft_passes.cuh"

namespace jld {

// ---------------------------------------------------------------------------
// Per-axis wavevector tables (FP64 on the host, stored as float):
// k_a[i] = 2 pi fftfreq(N_a, L_a/N_a)[i], c_a[i] = (45 sin(k h) - 9 sin(2kh)
// + sin(3kh)) / (30 h), h = L_a/N_a; the z tables cover kz in [0, Nz/2] with
// the reference's negative Nyquist entry (pmesh.py:179-183).
struct KTables {
  const float* kx; const float* ky; const float* kz;
  const float* cx; const float* cy; const float* cz;
};

static std::mutex g_kt_mu;
static std::map<std::tuple<int, int, int, int, double, double, double>, float*> g_ktabs;

static int get_ktables(int nx, int ny, int nz, const float box[3], bool build, KTables* out) {
  int dev = 0;
  JLD_CUDA_TRY(cudaGetDevice(&dev));
  auto key = std::make_tuple(dev, nx, ny, nz, (double)box[0], (double)box[1], (double)box[2]);
  std::lock_guard<std::mutex> lock(g_kt_mu);
  auto it = g_ktabs.find(key);
  const int h = nz / 2;
  const int len[3] = {nx, ny, h + 1};
  if (it == g_ktabs.end()) {
    if (!build)
      return set_error(JLD_ERR_NOPLAN, "LDL tables missing; run the step once before stream capture");
    const int n[3] = {nx, ny, nz};
    std::vector<float> host(2 * (nx + ny + h + 1));
    size_t o = 0;
    for (int a = 0; a < 3; ++a) {
      double L = box[a], step = L / n[a];
      for (int i = 0; i < len[a]; ++i) {
        int m = (i < (n[a] - 1) / 2 + 1) ? i : i - n[a];  // numpy fftfreq order
        double k = 2.0 * 3.14159265358979323846 * m / (n[a] * step);
        host[o + i] = (float)k;
        host[o + len[0] + len[1] + len[2] + i] =
            (float)((45.0 * std::sin(k * step) - 9.0 * std::sin(2 * k * step) +
                     std::sin(3 * k * step)) / (30.0 * step));
      }
      o += len[a];
    }
    float* d = nullptr;
    JLD_CUDA_TRY(cudaMalloc(&d, host.size() * sizeof(float)));
    JLD_CUDA_TRY(cudaMemcpy(d, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice));
    it = g_ktabs.emplace(key, d).first;
  }
  float* d = it->second;
  const int tot = len[0] + len[1] + len[2];
  out->kx = d; out->ky = d + len[0]; out->kz = d + len[0] + len[1];
  out->cx = d + tot; out->cy = d + tot + len[0]; out->cz = d + tot + len[0] + len[1];
  return JLD_OK;
}

// Green's function G(|k|) and its derivatives, model.py:156 ("dm") / 195 ("sm").
struct Green {
  float g, dkh, dkl, dnu;
};
__device__ __forceinline__ Green green_fn(float kx, float ky, float kz, int kind, float kh,
                                          float kl, float nu) {
  // G = -exp(E) k^nu = -2^(E log2(e) + nu log2(k)): one logarithm and one
  // exponential per mode
  constexpr float kLog2e = 1.4426950408889634f, kLn2 = 0.6931471805599453f;
  float k = sqrtf(kx * kx + ky * ky + kz * kz);
  if (k == 0.f) k = 1e-8f;
  Green r;
  const float l2k = log2f(k);
  if (kind == 1) {  // dm
    r.g = -exp2f((-k / kl - kh / k) * kLog2e + nu * l2k);
    r.dkh = r.g * (-1.f / k);
    r.dkl = r.g * (k / (kl * kl));
  } else {          // sm
    const float k2 = k * k;
    r.g = -exp2f((-k2 / (kl * kl) - kh * kh / k2) * kLog2e + nu * l2k);
    r.dkh = r.g * (-2.f * kh / k2);
    r.dkl = r.g * (2.f * k2 / (kl * kl * kl));
  }
  r.dnu = r.g * (l2k * kLn2);
  return r;
}

// ---------------------------------------------------------------------------
// Tile helpers: `cols` columns of lines of length n in smem (sm[j*ld + c]).
// Column c of the tile has global base address colad[c] (-1 = padding);
// element j of a line lives at colad[c] + j * es.

template <typename C>
__device__ __forceinline__ void tile_load(C* sm, int ld, const C* __restrict__ g,
                                          const int64_t* colad, int64_t es, int n, int cols,
                                          int cshift, int tid, int nthr) {
  const int total = cols * n;
  const bool contig = es == 1;
  for (int f = tid; f < total; f += nthr) {
    int c, j;
    if (contig) { c = f / n; j = f - c * n; } else { c = f & (cols - 1); j = f >> cshift; }
    int64_t a = colad[c];
    C v;
    if (a >= 0) v = g[a + (int64_t)j * es];
    else { v.x = 0; v.y = 0; }
    sm[j * ld + c] = v;
  }
}

template <typename C>
__device__ __forceinline__ void tile_store(const C* sm, int ld, C* __restrict__ g,
                                           const int64_t* colad, int64_t es, int n, int cols,
                                           int cshift, int tid, int nthr) {
  const int total = cols * n;
  const bool contig = es == 1;
  for (int f = tid; f < total; f += nthr) {
    int c, j;
    if (contig) { c = f / n; j = f - c * n; } else { c = f & (cols - 1); j = f >> cshift; }
    int64_t a = colad[c];
    if (a >= 0) g[a + (int64_t)j * es] = sm[j * ld + c];
  }
}

// A pass over the internal half-spectrum layout (main rows of length h plus
// the nyq plane) along x (AX = 0) or y (AX = 1).  Tiles [0, tiles_main) cover
// main, the rest cover nyq.  For each tile column this gives its base address
// and its two fixed spectral indices: (ky, kz) for x passes, (x, kz) for y.
struct SpecPass {
  int nx, ny, h;
  int cols, cshift;
  int64_t tiles_main;
};

__device__ __forceinline__ void spec_columns(const SpecPass& sp, int ax, int64_t tile,
                                             int64_t* colad, int* ca, int* cb, int64_t* es,
                                             int64_t* off, int tid) {
  // off: element offset of the nyq plane relative to main (set by caller)
  const int64_t h = sp.h, ny = sp.ny, nx = sp.nx;
  bool nyq = tile >= sp.tiles_main;
  int64_t t = nyq ? tile - sp.tiles_main : tile;
  if (ax == 0) {  // lines along x
    *es = nyq ? ny : ny * h;
    if (tid < sp.cols) {
      int64_t c = t * sp.cols + tid;
      int64_t ncol = nyq ? ny : ny * h;
      if (c < ncol) {
        colad[tid] = nyq ? (*off + c) : c;
        ca[tid] = nyq ? (int)c : (int)(c / h);      // ky
        cb[tid] = nyq ? (int)h : (int)(c % h);      // kz
      } else { colad[tid] = -1; ca[tid] = 0; cb[tid] = 0; }
    }
  } else {        // lines along y
    *es = nyq ? 1 : h;
    if (tid < sp.cols) {
      int64_t c = t * sp.cols + tid;
      int64_t ncol = nyq ? nx : nx * h;
      if (c < ncol) {
        colad[tid] = nyq ? (*off + c * ny) : ((c / h) * ny * h + (c % h));
        ca[tid] = nyq ? (int)c : (int)(c / h);      // x
        cb[tid] = nyq ? (int)h : (int)(c % h);      // kz
      } else { colad[tid] = -1; ca[tid] = 0; cb[tid] = 0; }
    }
  }
}

// Potential prefactor: 1e-2 (kinds sm, dm; model.py:159,198), 1e-3 for the
// two-source HI kind (kind 2, model.py:232).
__device__ __forceinline__ float pot_coef(int kind) { return kind == 2 ? 1e-3f : 1e-2f; }

// HI kind: adds the star-map term 1e-3 a2 G2 S2 / Nc of the potential to p
// (a2, kh2, kl2, nu2 at params[5], [7], [8], [9]; G2 = +exp(-k^2/kl2^2 -
// kh2^2/k^2) k^nu2, the sm Green's function with the sign flipped).
__device__ __forceinline__ void hi_add_src2(float2& p, float2 s2, const float* __restrict__ params, float scale,
                                            float kx, float ky, float kz) {
  const Green g2 = green_fn(kx, ky, kz, 0, __ldg(params + 7), __ldg(params + 8), __ldg(params + 9));
  const float m = -1e-3f * __ldg(params + 5) * scale * g2.g;
  p.x += s2.x * m;
  p.y += s2.y * m;
}

// ---------------------------------------------------------------------------
// Forward kernels.

// base^e for base > 0 as exp2(e * log2(base)), optionally with ln(base):
// one logarithm and one exponential instead of powf's extended-precision
// path.  Relative error: a few ulp plus |e * log2(base)| * 2^-24, far
// inside the FP32 tolerance of the step.
__device__ __forceinline__ float pow_pos(float base, float e, float* ln_base = nullptr) {
  const float l2 = log2f(base);
  if (ln_base) *ln_base = l2 * 0.693147180559945f;
  return exp2f(e * l2);
}

struct SourcePow {
  const float* params;  // gamma at params[1]
  float fact;
  __device__ __forceinline__ float operator()(float v, int64_t) const {
    float gamma = __ldg(params + 1);
    float rho = __fmul_rn(v, fact);
    return pow_pos(__fadd_rn(rho, 1e-8f), gamma);
  }
};

// x pass of the forward: FFT_x, keep S, filter, two inverse outputs.
template <int SCHED>
__global__ void __launch_bounds__(512)
xfilt_kernel(LinePlan<float> pl, SpecPass sp, KTables kt, const float* __restrict__ params,
             int kind, float scale, const float2* __restrict__ A, float2* __restrict__ S,
             float2* __restrict__ T0, float2* __restrict__ T1, const float2* __restrict__ S2) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int64_t colad[64];
  __shared__ int ca[64], cb[64];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int cols = sp.cols, ld = cols + 1, n = pl.n;
  float2* s0 = reinterpret_cast<float2*>(smraw);
  float2* s1 = s0 + n * ld;
  int64_t es, off = (int64_t)sp.nx * sp.ny * sp.h;
  spec_columns(sp, 0, blockIdx.x, colad, ca, cb, &es, &off, tid);
  __syncthreads();
  tile_load(s0, ld, A, colad, es, n, cols, sp.cshift, tid, nthr);
  __syncthreads();
  fft_tile<float, SCHED>(s0, ld, pl, sp.cshift, -1, tid, nthr);
  tile_store(s0, ld, S, colad, es, n, cols, sp.cshift, tid, nthr);
  __syncthreads();
  const float alpha = __ldg(params + 0), kh = __ldg(params + 2), kl = __ldg(params + 3),
              nu = __ldg(params + 4);
  const float a = pot_coef(kind) * alpha * scale;
  for (int f = tid; f < cols * n; f += nthr) {
    int c = f & (cols - 1), j = f >> sp.cshift;
    float2 v = s0[j * ld + c];
    Green gr = green_fn(__ldg(kt.kx + j), __ldg(kt.ky + ca[c]), __ldg(kt.kz + cb[c]), kind, kh, kl, nu);
    float m = a * gr.g;
    float2 p = make_float2(v.x * m, v.y * m);
    if (S2 && colad[c] >= 0) hi_add_src2(p, S2[colad[c] + (int64_t)j * es], params, scale,
                                         __ldg(kt.kx + j), __ldg(kt.ky + ca[c]), __ldg(kt.kz + cb[c]));
    s0[j * ld + c] = p;
    float cxv = __ldg(kt.cx + j);
    s1[j * ld + c] = make_float2(p.y * cxv, -p.x * cxv);  // -i c_x P
  }
  __syncthreads();
  fft_tile<float, SCHED>(s0, ld, pl, sp.cshift, +1, tid, nthr);
  fft_tile<float, SCHED>(s1, ld, pl, sp.cshift, +1, tid, nthr);
  tile_store(s0, ld, T0, colad, es, n, cols, sp.cshift, tid, nthr);
  tile_store(s1, ld, T1, colad, es, n, cols, sp.cshift, tid, nthr);
}

// y pass of the forward inverse: three outputs from T0, T1.
template <int SCHED>
__global__ void __launch_bounds__(512)
yinv3_kernel(LinePlan<float> pl, SpecPass sp, KTables kt, const float2* __restrict__ T0,
             const float2* __restrict__ T1, float2* __restrict__ Gx, float2* __restrict__ Gy,
             float2* __restrict__ Gz) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int64_t colad[64];
  __shared__ int ca[64], cb[64];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int cols = sp.cols, ld = cols + 1, n = pl.n;
  float2* s0 = reinterpret_cast<float2*>(smraw);
  int64_t es, off = (int64_t)sp.nx * sp.ny * sp.h;
  spec_columns(sp, 1, blockIdx.x, colad, ca, cb, &es, &off, tid);
  __syncthreads();
  // Gy = iFFT_y(-i c_y(ky) T0)
  tile_load(s0, ld, T0, colad, es, n, cols, sp.cshift, tid, nthr);
  __syncthreads();
  for (int f = tid; f < cols * n; f += nthr) {
    int c = f & (cols - 1), j = f >> sp.cshift;
    float2 v = s0[j * ld + c];
    float cy = __ldg(kt.cy + j);
    s0[j * ld + c] = make_float2(v.y * cy, -v.x * cy);
  }
  __syncthreads();
  fft_tile<float, SCHED>(s0, ld, pl, sp.cshift, +1, tid, nthr);
  tile_store(s0, ld, Gy, colad, es, n, cols, sp.cshift, tid, nthr);
  __syncthreads();
  // Gz = -i c_z(kz) iFFT_y(T0)
  tile_load(s0, ld, T0, colad, es, n, cols, sp.cshift, tid, nthr);
  __syncthreads();
  fft_tile<float, SCHED>(s0, ld, pl, sp.cshift, +1, tid, nthr);
  for (int f = tid; f < cols * n; f += nthr) {
    int c = f & (cols - 1), j = f >> sp.cshift;
    int64_t a = colad[c];
    if (a >= 0) {
      float2 v = s0[j * ld + c];
      float cz = __ldg(kt.cz + cb[c]);
      Gz[a + (int64_t)j * es] = make_float2(v.y * cz, -v.x * cz);
    }
  }
  __syncthreads();
  // Gx = iFFT_y(T1)
  tile_load(s0, ld, T1, colad, es, n, cols, sp.cshift, tid, nthr);
  __syncthreads();
  fft_tile<float, SCHED>(s0, ld, pl, sp.cshift, +1, tid, nthr);
  tile_store(s0, ld, Gx, colad, es, n, cols, sp.cshift, tid, nthr);
}

// Builds the packed c2r input Z'[k] of one row element (see irfft_z_kernel).
__device__ __forceinline__ float2 c2r_pack(const float2* __restrict__ main,
                                           const float2* __restrict__ nyq, int64_t row, int h,
                                           int k, const float2* __restrict__ twr) {
  float2 xk = main[row * h + k];
  float2 xh = (k == 0) ? nyq[row] : main[row * h + (h - k)];
  if (k == 0) { xk.y = 0.f; xh.y = 0.f; }
  float2 xc = make_float2(xh.x, -xh.y);
  float2 a = make_float2(xk.x + xc.x, xk.y + xc.y);
  float2 b = make_float2(xk.x - xc.x, xk.y - xc.y);
  float2 w = __ldg(twr + k);
  w.y = -w.y;
  float2 t = make_float2(w.x * b.x - w.y * b.y, w.x * b.y + w.y * b.x);
  return make_float2(a.x - t.y, a.y + t.x);
}

// z pass of the forward inverse: three c2r transforms into a float4 mesh.
template <int SCHED>
__global__ void __launch_bounds__(512)
zinv3_kernel(LinePlan<float> pl, const float2* __restrict__ twr, const float2* __restrict__ Gx,
             const float2* __restrict__ Gy, const float2* __restrict__ Gz, int64_t nyq_off,
             float4* __restrict__ g4, int64_t rows, int cols, int cshift) {
  extern __shared__ __align__(128) unsigned char smraw[];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int h = pl.n, ld = cols + 1;
  float2* sm[3];
  sm[0] = reinterpret_cast<float2*>(smraw);
  sm[1] = sm[0] + h * ld;
  sm[2] = sm[1] + h * ld;
  const float2* src[3] = {Gx, Gy, Gz};
  const int64_t row0 = (int64_t)blockIdx.x * cols;
  for (int d = 0; d < 3; ++d) {
    for (int f = tid; f < cols * h; f += nthr) {
      int c = f / h, k = f - c * h;
      int64_t row = row0 + c;
      float2 v = make_float2(0.f, 0.f);
      if (row < rows) v = c2r_pack(src[d], src[d] + nyq_off, row, h, k, twr);
      sm[d][k * ld + c] = v;
    }
  }
  __syncthreads();
  for (int d = 0; d < 3; ++d) fft_tile<float, SCHED>(sm[d], ld, pl, cshift, +1, tid, nthr);
  for (int f = tid; f < cols * h; f += nthr) {
    int c = f / h, m = f - c * h;
    int64_t row = row0 + c;
    if (row < rows) {
      float2 a = sm[0][m * ld + c], b = sm[1][m * ld + c], e = sm[2][m * ld + c];
      float4* o = g4 + row * (2 * (int64_t)h) + 2 * m;
      o[0] = make_float4(a.x, b.x, e.x, 0.f);
      o[1] = make_float4(a.y, b.y, e.y, 0.f);
    }
  }
}

// ---------------------------------------------------------------------------
// Particle kernels.

struct BoxGeom {
  float box[3], cell[3], dw[3];  // dw = N/L, the CIC weight derivative
};

__device__ __forceinline__ void particle_setup(const float* __restrict__ X, int64_t p,
                                               const BoxGeom& bg, const Grid3& g, Corners<float>& c,
                                               float lo[3], float hi[3]) {
  float q[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) q[a] = box_to_mesh_fast(__ldg(X + 3 * p + a), bg.box[a], bg.dw[a]);
  cic_corners(q, g, c);
#pragma unroll
  for (int a = 0; a < 3; ++a) { hi[a] = c.d[a]; lo[a] = __fsub_rn(1.f, c.d[a]); }
}

// sum_k u_k grad w_k over the eight corners (u_k = 0 for invalid corners),
// factored by axis: d w_k / d x_0 = (b_x ? dw_0 : -dw_0) w_y[b_y] w_z[b_z]
// and likewise for y and z, so each axis costs four differences and four
// products of the other two axes' weights.
__device__ __forceinline__ void cic_grad(const float (&u)[8], const float lo[3], const float hi[3],
                                         const float dw[3], float out[3]) {
  float U[2][2][2];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int b = corner_axis_bits(k);
    U[b & 1][(b >> 1) & 1][(b >> 2) & 1] = u[k];
  }
  const float wx[2] = {lo[0], hi[0]}, wy[2] = {lo[1], hi[1]}, wz[2] = {lo[2], hi[2]};
  float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      sx += wy[i] * wz[j] * (U[1][i][j] - U[0][i][j]);
      sy += wx[i] * wz[j] * (U[i][1][j] - U[i][0][j]);
      sz += wx[i] * wy[j] * (U[i][j][1] - U[i][j][0]);
    }
  out[0] = dw[0] * sx;
  out[1] = dw[1] * sy;
  out[2] = dw[2] * sz;
}

__device__ __forceinline__ float wprod(const float lo[3], const float hi[3], int bits) {
  float wx = (bits & 1) ? hi[0] : lo[0];
  float wy = (bits & 2) ? hi[1] : lo[1];
  float wz = (bits & 4) ? hi[2] : lo[2];
  return __fmul_rn(__fmul_rn(wx, wy), wz);
}

// X' = X + readout of the float4 force mesh (three channels, the reference's
// per-channel summation order).  Five CTAs per SM (48 registers): on the
// 512^3 clustered step 29.9 ms against 30.1 at six (40 registers) and 31.8
// at seven (32 registers, spills).
#ifndef JLD_UPD_MIN_CTAS
#define JLD_UPD_MIN_CTAS 5
#endif
__global__ void __launch_bounds__(256, JLD_UPD_MIN_CTAS)
update_kernel(const float* __restrict__ X, int64_t n, BoxGeom bg, Grid3 g,
              const float4* __restrict__ g4, float* __restrict__ Xn, int* tick) {
  // warps walk batches of 32 particles (WarpBatches); the next batch's
  // position is loaded one batch ahead
  const int lane = threadIdx.x & 31;
  WarpBatches wb;
  int64_t base = wb.first(tick, n);
  float nr[3] = {0.f, 0.f, 0.f};
  if (base + lane < n) {
    const int64_t p = base + lane;
    nr[0] = __ldg(X + 3 * p); nr[1] = __ldg(X + 3 * p + 1); nr[2] = __ldg(X + 3 * p + 2);
  }
  for (; base < n;) {
    const int64_t p = base + lane;
    const float r[3] = {nr[0], nr[1], nr[2]};
    base = wb.next(base);
    const int64_t pn = base + lane;
    if (pn < n) { nr[0] = __ldg(X + 3 * pn); nr[1] = __ldg(X + 3 * pn + 1); nr[2] = __ldg(X + 3 * pn + 2); }
    if (p >= n) continue;
    Corners<float> c;
    float lo[3], hi[3];
    {
      float q[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) q[a] = box_to_mesh_fast(r[a], bg.box[a], bg.dw[a]);
      cic_corners(q, g, c);
#pragma unroll
      for (int a = 0; a < 3; ++a) { hi[a] = c.d[a]; lo[a] = __fsub_rn(1.f, c.d[a]); }
    }
    float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      int bits = corner_axis_bits(k);
      float4 v = __ldg(g4 + corner_offset(c, bits, g));
      float w = corner_ok(c, bits) ? wprod(lo, hi, bits) : 0.f;
      float t0 = __fmul_rn(w, v.x), t1 = __fmul_rn(w, v.y), t2 = __fmul_rn(w, v.z);
      if (k == 0) { acc[0] = t0; acc[1] = t1; acc[2] = t2; }
      else { acc[0] = __fadd_rn(acc[0], t0); acc[1] = __fadd_rn(acc[1], t1); acc[2] = __fadd_rn(acc[2], t2); }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) Xn[3 * p + a] = __fadd_rn(r[a], acc[a]);
  }
}

// Xbar += sum_c rb[c] grad w_c (the adjoint of a unit-mass paint,
// lib/parops_fast.h:730-821 with vjp = true); accumulate == 0 overwrites.
__global__ void __launch_bounds__(256)
gather_vjp_kernel(const float* __restrict__ X, int64_t n, BoxGeom bg, Grid3 g,
                  const float* __restrict__ rb, float* __restrict__ Xb, int accumulate) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    Corners<float> c;
    float lo[3], hi[3];
    particle_setup(X, p, bg, g, c, lo, hi);
    float a[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      int bits = corner_axis_bits(k);
      if (!corner_ok(c, bits)) continue;
      float r = __ldg(rb + corner_offset(c, bits, g));
#pragma unroll
      for (int e = 0; e < 3; ++e) {
        float l2[3] = {lo[0], lo[1], lo[2]}, h2[3] = {hi[0], hi[1], hi[2]};
        l2[e] = -bg.dw[e]; h2[e] = bg.dw[e];
        a[e] += r * wprod(l2, h2, bits);
      }
    }
#pragma unroll
    for (int e = 0; e < 3; ++e) Xb[3 * p + e] = accumulate ? Xb[3 * p + e] + a[e] : a[e];
  }
}

// ---------------------------------------------------------------------------
// Fused particle kernels (plain-atomic scatter path).

// Adjoint of layer l with the paint adjoint of layer l+1 folded in:
//   v = Xbp + sum_c rb[c] grad w_c(Xn)     (gather_vjp_kernel's arithmetic;
//                                           Xbp == nullptr: no partial)
//   Xb = v + J^T v at X (GATHER), gb4 += scatter of v (float4 atomics)
// Xn are the positions after layer l, X the positions before it.
// Warps walk 32 consecutive particles; lanes merge shared z faces before
// the float4 atomics (zpair32_flags).  Measured on the 512^3 clustered step:
// this layout at five CTAs per SM (48 registers) beats the 16 x 2 layout with
// y pairing as well at four (64 registers), 30.1 against 30.9 ms per step.
#ifndef JLD_BWD_MIN_CTAS
#define JLD_BWD_MIN_CTAS 5
#endif
template <bool GATHER>
__global__ void __launch_bounds__(256, JLD_BWD_MIN_CTAS)
bwd_fused_kernel(const float* __restrict__ Xn, const float* __restrict__ rb, const float* __restrict__ Xbp,
                 const float* __restrict__ X, int64_t n, BoxGeom bg, Grid3 g, const float4* __restrict__ g4,
                 float4* __restrict__ gb4, float* __restrict__ Xb, int* tick) {
  const unsigned full = 0xffffffffu;
  WarpBatches wb;
  const int nax[3] = {g.nx, g.ny, g.nz};
  // Warps whose 32 particles all lie inside the mesh (nearly all) skip the
  // per-corner validity flags, separately for the two stencils.
  auto inside = [&](const float q[3], bool live) {
    bool in = live;
#pragma unroll
    for (int a = 0; a < 3; ++a) in = in && (unsigned)(int)q[a] < (unsigned)nax[a];
    return __all_sync(full, in);
  };
  auto corners = [&](const float q[3], bool fast, Corners<float>& c, float lo[3], float hi[3]) {
    if (fast) cic_corners_inrange(q, g, c);
    else cic_corners(q, g, c);
#pragma unroll
    for (int a = 0; a < 3; ++a) { hi[a] = c.d[a]; lo[a] = __fsub_rn(1.f, c.d[a]); }
  };
  for (int64_t base = wb.first(tick, n); base < n; base = wb.next(base)) {
    const bool live = base + (threadIdx.x & 31) < n;
    const int64_t p = live ? base + (threadIdx.x & 31) : n - 1;
    float v[3];
    {
      float q[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) q[a] = box_to_mesh_fast(__ldg(Xn + 3 * p + a), bg.box[a], bg.dw[a]);
      const bool fast = inside(q, live);
      Corners<float> c;
      float lo[3], hi[3];
      corners(q, fast, c, lo, hi);
      float r[8];
      if (fast) {
#pragma unroll
        for (int k = 0; k < 8; ++k) r[k] = __ldg(rb + corner_offset(c, corner_axis_bits(k), g));
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int bits = corner_axis_bits(k);
          r[k] = corner_ok(c, bits) ? __ldg(rb + corner_offset(c, bits, g)) : 0.f;
        }
      }
      float a[3];
      cic_grad(r, lo, hi, bg.dw, a);
#pragma unroll
      for (int e = 0; e < 3; ++e) v[e] = live ? (Xbp ? __ldg(Xbp + 3 * p + e) + a[e] : a[e]) : 0.f;
    }
    float q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) q[a] = box_to_mesh_fast(__ldg(X + 3 * p + a), bg.box[a], bg.dw[a]);
    const bool fast = inside(q, live);
    Corners<float> c;
    float lo[3], hi[3];
    corners(q, fast, c, lo, hi);
    float a[3] = {0.f, 0.f, 0.f};
    float4 s4[8];
    if (GATHER) {
      float u[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int bits = corner_axis_bits(k);
        const float4 gv = __ldg(g4 + corner_offset(c, bits, g));
        u[k] = (fast || corner_ok(c, bits)) ? v[0] * gv.x + v[1] * gv.y + v[2] * gv.z : 0.f;
      }
      cic_grad(u, lo, hi, bg.dw, a);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int bits = corner_axis_bits(k);
      const float w = (fast || corner_ok(c, bits)) ? wprod(lo, hi, bits) : 0.f;
      s4[k] = make_float4(v[0] * w, v[1] * w, v[2] * w, 0.f);
    }
    const Pairing pr = zpair32_flags(live ? pair_key(c, g) : kNoPair);
    auto move = [&](int from, int to, int delta, bool take) {
      const float4 h = s4[from];
      const float tx = __shfl_up_sync(full, h.x, delta), ty = __shfl_up_sync(full, h.y, delta),
                  tz = __shfl_up_sync(full, h.z, delta);
      if (take) {
        float4& d = s4[to];
        d.x += tx; d.y += ty; d.z += tz;
      }
    };
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) move(zpair_hi(jj), zpair_lo(jj), 1, pr.tz);
    if (live) {
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (pair_keeps(pr, k)) atomicAdd(gb4 + corner_offset(c, corner_axis_bits(k), g), s4[k]);
      if (GATHER) {
#pragma unroll
        for (int e = 0; e < 3; ++e) Xb[3 * p + e] = v[e] + a[e];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Block reductions in FP64 into per-block partial slots (deterministic:
// the final sum runs in a fixed order in finish_kernel).

template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double* __restrict__ out,
                                                   int slot_stride) {
  __shared__ double red[32][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // lanes that exist in this warp (the last warp of a block may be partial)
  const int live = min(32, (int)blockDim.x - warp * 32);
  const unsigned mask = live == 32 ? 0xffffffffu : ((1u << live) - 1u);
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    double x = v[i];
    for (int o = 16; o > 0; o >>= 1) {
      double y = __shfl_down_sync(mask, x, o);
      if (lane + o < live) x += y;
    }
    if (lane == 0) red[warp][i] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0;
    int nw = (blockDim.x + 31) >> 5;
    for (int w = 0; w < nw; ++w) s += red[w][threadIdx.x];
    out[(int64_t)blockIdx.x * slot_stride + threadIdx.x] = s;
  }
}

// Compensated (Kahan) FP32 running sum for per-thread partials (a thread
// covers tens of elements); the cross-thread and cross-block sums are FP64.
// FP64 arithmetic per element would be slow on this part.
struct KahanF {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    float y = __fsub_rn(x, c);
    float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

template <int NV>
__device__ __forceinline__ void block_reduce_kahan(const KahanF (&k)[NV], double* __restrict__ out,
                                                   int slot_stride) {
  double v[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) v[i] = k[i].value();
  block_reduce_store<NV>(v, out, slot_stride);
}

// Final map, loss and its cotangent (model.py:311-403, 351-403, 416-465).
// F = ReLU(w (rho + 1e-8)^mu + b) (kind sm) or rho (kind dm); the loss map is
// Fp = F^index * field2 (model.py:357-361); diff = Fp - target, smoothed by
// c2r(r2c(diff) K) with K = |k|^-n + 1 when n > 0 (model.py:376-381, no c2f);
// loss = sum (mask |diff|)^p / Npixel, the validation loss the same with
// maskvalid (model.py:454-465).  rb = fact * d loss / d rho.
struct LossArgs {
  float mu, w, b, fact, inpx, index;
  int kind, L1;
};

struct MapCell {
  float F, u, pw, base, lnb;
};

__device__ __forceinline__ MapCell map_cell(const LossArgs& la, float rho_paint) {
  MapCell c;
  const float rho = __fmul_rn(rho_paint, la.fact);
  c.u = c.pw = c.base = c.lnb = 0.f;
  if (la.kind == 0) {
    c.base = __fadd_rn(rho, 1e-8f);
    c.pw = pow_pos(c.base, la.mu, &c.lnb);
    c.u = __fadd_rn(__fmul_rn(la.w, c.pw), la.b);
    c.F = c.u > 1e-12f ? c.u : 1e-12f;
  } else {
    c.F = rho;
  }
  return c;
}

// Fp = F^index * f2; *dFp = dFp/dF.
__device__ __forceinline__ float map_ext(const LossArgs& la, float F, float f2, float* dFp) {
  float Fp = F, d = 1.f;
  if (la.index != 1.f) {
    Fp = pow_pos(F, la.index);
    d = la.index * pow_pos(F, la.index - 1.f);
  }
  *dFp = d * f2;
  return Fp * f2;
}

// Adjoint of the map for ctF = dL/dF: (d mu, d w, d b) into acc3 (kind sm);
// returns fact * dL/drho.
__device__ __forceinline__ float map_adjoint(const LossArgs& la, const MapCell& c, float ctF, KahanF* acc3) {
  if (la.kind == 0) {
    const float ctu = c.u > 1e-12f ? ctF : 0.f;
    acc3[0].add(ctu * la.w * c.pw * c.lnb);
    acc3[1].add(ctu * c.pw);
    acc3[2].add(ctu);
    // base^(mu-1) = pw / base (base > 0)
    return ctu * la.w * la.mu * (c.pw / c.base) * la.fact;
  }
  return ctF * la.fact;
}

// Loss and validation-loss terms of one cell's residual; returns dL/d diff.
__device__ __forceinline__ float diff_terms(const LossArgs& la, float diff, float m, float mv, KahanF& lacc,
                                            KahanF& vacc) {
  const float ad = fabsf(diff) * m;
  lacc.add(la.L1 ? ad : ad * ad);
  const float av = fabsf(diff) * mv;
  vacc.add(la.L1 ? av : av * av);
  const float sg = diff >= 0.f ? 1.f : -1.f;
  return (la.L1 ? sg * m : 2.f * fabsf(diff) * m * m * sg) * la.inpx;
}

__device__ __forceinline__ LossArgs loss_args(const float* fparams, int kind, int L1, float fact, float index,
                                              const double* inv_npix) {
  LossArgs la;
  la.mu = kind == 0 ? __ldg(fparams + 0) : 0.f;
  la.w = kind == 0 ? __ldg(fparams + 1) : 0.f;
  la.b = kind == 0 ? __ldg(fparams + 2) : 0.f;
  la.fact = fact;
  la.inpx = inv_npix ? (float)(*inv_npix) : 0.f;
  la.index = index;
  la.kind = kind;
  la.L1 = L1;
  return la;
}

// The per-cell inputs of the loss (mask, field2, validation mask optional).
struct LossFields {
  const float* rho;
  const float* target;
  const float* mask;
  const float* field2;
  const float* maskvalid;
};

__device__ __forceinline__ float4 ld4_or(const float* p, int64_t e, float v) {
  return p ? __ldg(reinterpret_cast<const float4*>(p) + e) : make_float4(v, v, v, v);
}
__device__ __forceinline__ float ld_or(const float* p, int64_t e, float v) { return p ? __ldg(p + e) : v; }
__device__ __forceinline__ float f4c(const float4& v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }

// Unsmoothed loss in one pass.  Partials per block: [loss, d mu, d w, d b,
// validation loss].  Cells in float4 groups (vec4: every array 16-byte
// aligned, C a multiple of 4), the rest one by one.
__global__ void __launch_bounds__(256)
loss_kernel(LossFields lf, int64_t C, float fact, const float* __restrict__ fparams, int kind, int L1,
            float index, const double* __restrict__ inv_npix, float* __restrict__ rb,
            double* __restrict__ partials, int vec4) {
  const LossArgs la = loss_args(fparams, kind, L1, fact, index, inv_npix);
  KahanF acc[5];
  auto cell = [&](float r, float t, float m, float f2, float mv) {
    const MapCell c = map_cell(la, r);
    float dFp;
    const float Fp = map_ext(la, c.F, f2, &dFp);
    const float ct = diff_terms(la, Fp - t, m, mv, acc[0], acc[4]);
    return map_adjoint(la, c, ct * dFp, acc + 1);
  };
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  const int64_t c4 = vec4 ? C / 4 : 0;
  for (int64_t e = tid; e < c4; e += nth) {
    const float4 r = __ldg(reinterpret_cast<const float4*>(lf.rho) + e);
    const float4 t = __ldg(reinterpret_cast<const float4*>(lf.target) + e);
    const float4 m = ld4_or(lf.mask, e, 1.f), f2 = ld4_or(lf.field2, e, 1.f), mv = ld4_or(lf.maskvalid, e, 0.f);
    float o[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = cell(f4c(r, q), f4c(t, q), f4c(m, q), f4c(f2, q), f4c(mv, q));
    reinterpret_cast<float4*>(rb)[e] = make_float4(o[0], o[1], o[2], o[3]);
  }
  for (int64_t e = 4 * c4 + tid; e < C; e += nth)
    rb[e] = cell(__ldg(lf.rho + e), __ldg(lf.target + e), ld_or(lf.mask, e, 1.f), ld_or(lf.field2, e, 1.f),
                 ld_or(lf.maskvalid, e, 0.f));
  block_reduce_kahan<5>(acc, partials, 5);
}

// Smoothed loss, pass 1: rb = Fp - target.
__global__ void __launch_bounds__(256)
smooth_map_kernel(LossFields lf, int64_t C, float fact, const float* __restrict__ fparams, int kind,
                  float index, float* __restrict__ rb) {
  const LossArgs la = loss_args(fparams, kind, 1, fact, index, nullptr);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < C; e += (int64_t)gridDim.x * blockDim.x) {
    const MapCell c = map_cell(la, __ldg(lf.rho + e));
    float dFp;
    rb[e] = map_ext(la, c.F, ld_or(lf.field2, e, 1.f), &dFp) - __ldg(lf.target + e);
  }
}

// Smoothed loss, pass 2, on rb = the smoothed residual: partials per block
// [loss, validation loss]; rb = dL / d(smoothed residual).
__global__ void __launch_bounds__(256)
smooth_loss_kernel(LossFields lf, int64_t C, int L1, const double* __restrict__ inv_npix, float* __restrict__ rb,
                   double* __restrict__ partials) {
  LossArgs la = loss_args(nullptr, 1, L1, 1.f, 1.f, inv_npix);
  KahanF acc[2];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < C; e += (int64_t)gridDim.x * blockDim.x)
    rb[e] = diff_terms(la, rb[e], ld_or(lf.mask, e, 1.f), ld_or(lf.maskvalid, e, 0.f), acc[0], acc[1]);
  block_reduce_kahan<2>(acc, partials, 2);
}

// Smoothed loss, pass 3, on rb = dL/dFp: partials per block [d mu, d w, d b];
// rb = fact * dL/drho.
__global__ void __launch_bounds__(256)
smooth_adj_kernel(LossFields lf, int64_t C, float fact, const float* __restrict__ fparams, int kind, float index,
                  float* __restrict__ rb, double* __restrict__ partials) {
  const LossArgs la = loss_args(fparams, kind, 1, fact, index, nullptr);
  KahanF acc[3];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < C; e += (int64_t)gridDim.x * blockDim.x) {
    const MapCell c = map_cell(la, __ldg(lf.rho + e));
    float dFp;
    (void)map_ext(la, c.F, ld_or(lf.field2, e, 1.f), &dFp);
    rb[e] = map_adjoint(la, c, rb[e] * dFp, acc);
  }
  block_reduce_kahan<3>(acc, partials, 3);
}

// Smoothing kernel on an interleaved (Nx, Ny, Nz/2+1) half spectrum:
// spec *= (|k|^-n + 1) * scale with |k| = 0 read as 1e-8 (model.py:100-102,
// so the reference's |k| == 0 branch never applies).
__global__ void __launch_bounds__(256)
smooth_spec_kernel(float2* __restrict__ spec, int nx, int ny, int hh, KTables kt, float n, float scale) {
  const int64_t H = (int64_t)nx * ny * hh;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < H; e += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(e % hh);
    const int64_t r = e / hh;
    const int j = (int)(r % ny), i = (int)(r / ny);
    const float kx = __ldg(kt.kx + i), ky = __ldg(kt.ky + j), kz = __ldg(kt.kz + l);
    float k = sqrtf(kx * kx + ky * ky + kz * kz);
    if (k == 0.f) k = 1e-8f;
    const float K = __fadd_rn(exp2f(-n * log2f(k)), 1.f) * scale;
    const float2 v = spec[e];
    spec[e] = make_float2(v.x * K, v.y * K);
  }
}

// Adjoint z pass: ct_s = c2r(V); per element the source adjoint.
// Partials per block: [d gamma].
template <int SCHED>
__global__ void __launch_bounds__(512)
zinv_adj_kernel(LinePlan<float> pl, const float2* __restrict__ twr, const float2* __restrict__ V,
                int64_t nyq_off, const float* __restrict__ rho_paint, const float* __restrict__ params,
                float fact, float* __restrict__ rb, double* __restrict__ partials, int64_t rows,
                int cols, int cshift) {
  extern __shared__ __align__(128) unsigned char smraw[];
  float2* sm = reinterpret_cast<float2*>(smraw);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int h = pl.n, ld = cols + 1;
  const int64_t row0 = (int64_t)blockIdx.x * cols;
  for (int f = tid; f < cols * h; f += nthr) {
    int c = f / h, k = f - c * h;
    int64_t row = row0 + c;
    float2 v = make_float2(0.f, 0.f);
    if (row < rows) v = c2r_pack(V, V + nyq_off, row, h, k, twr);
    sm[k * ld + c] = v;
  }
  __syncthreads();
  fft_tile<float, SCHED>(sm, ld, pl, cshift, +1, tid, nthr);
  const float gamma = __ldg(params + 1);
  KahanF acc[1];
  for (int f = tid; f < cols * h; f += nthr) {
    int c = f / h, m = f - c * h;
    int64_t row = row0 + c;
    if (row < rows) {
      float2 z = sm[m * ld + c];
      int64_t e = row * 2 * (int64_t)h + 2 * m;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        float cts = q ? z.y : z.x;
        float rho = __fmul_rn(__ldg(rho_paint + e + q), fact);
        float base = __fadd_rn(rho, 1e-8f);
        float lb;
        float s = pow_pos(base, gamma, &lb);
        acc[0].add(cts * s * lb);
        // base^(gamma-1) = s / base (base > 0); rb == nullptr: the first
        // layer, whose paint cotangent feeds no position cotangent
        if (rb) rb[e + q] = cts * gamma * (s / base) * fact;
      }
    }
  }
  block_reduce_kahan<1>(acc, partials, 1);
}

// Adjoint z pass of the three cotangent channels: r2c rows of the float4 mesh.
// Outputs Ax, Ay and c_z(kz) * Az in the internal layout.
template <int SCHED>
__global__ void __launch_bounds__(512)
zfwd3_kernel(LinePlan<float> pl, const float2* __restrict__ twr, const float* __restrict__ cz,
             const float4* __restrict__ gb4, float2* __restrict__ Ax, float2* __restrict__ Ay,
             float2* __restrict__ Az, int64_t nyq_off, int64_t rows, int cols, int cshift) {
  extern __shared__ __align__(128) unsigned char smraw[];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int h = pl.n, ld = cols + 1;
  float2* sm[3];
  sm[0] = reinterpret_cast<float2*>(smraw);
  sm[1] = sm[0] + h * ld;
  sm[2] = sm[1] + h * ld;
  const int64_t row0 = (int64_t)blockIdx.x * cols;
  for (int f = tid; f < cols * h; f += nthr) {
    int c = f / h, j = f - c * h;
    int64_t row = row0 + c;
    float4 a = make_float4(0, 0, 0, 0), b = a;
    if (row < rows) {
      const float4* r = gb4 + row * 2 * (int64_t)h + 2 * j;
      a = r[0]; b = r[1];
    }
    sm[0][j * ld + c] = make_float2(a.x, b.x);
    sm[1][j * ld + c] = make_float2(a.y, b.y);
    sm[2][j * ld + c] = make_float2(a.z, b.z);
  }
  __syncthreads();
  for (int d = 0; d < 3; ++d) fft_tile<float, SCHED>(sm[d], ld, pl, cshift, -1, tid, nthr);
  float2* dst[3] = {Ax, Ay, Az};
  const int hh = h / 2 + 1;
  for (int d = 0; d < 3; ++d) {
    for (int f = tid; f < cols * hh; f += nthr) {
      int c = f / hh, k = f - c * hh;
      int64_t row = row0 + c;
      if (row >= rows) continue;
      float2 z = sm[d][(k % h) * ld + c];
      float2 zm = sm[d][((h - k) % h) * ld + c];
      float2 zc = make_float2(zm.x, -zm.y);
      float2 xe = make_float2(0.5f * (z.x + zc.x), 0.5f * (z.y + zc.y));
      float2 dd = make_float2(0.5f * (z.x - zc.x), 0.5f * (z.y - zc.y));
      float2 xo = make_float2(dd.y, -dd.x);
      float2 w = __ldg(twr + k);
      float2 wxo = make_float2(w.x * xo.x - w.y * xo.y, w.x * xo.y + w.y * xo.x);
      float2 xk = make_float2(xe.x + wxo.x, xe.y + wxo.y);
      float2 xhk = make_float2(xe.x - wxo.x, -(xe.y - wxo.y));
      float s1 = d == 2 ? __ldg(cz + k) : 1.f;
      float s2 = d == 2 ? __ldg(cz + (h - k)) : 1.f;
      dst[d][row * h + k] = make_float2(xk.x * s1, xk.y * s1);
      if (k == 0) dst[d][nyq_off + row] = make_float2(xhk.x * s2, xhk.y * s2);
      else if (h - k != k) dst[d][row * h + (h - k)] = make_float2(xhk.x * s2, xhk.y * s2);
    }
  }
}

// Adjoint y pass: Bx = FFT_y(Ax) (in place), D = c_y FFT_y(Ay) + FFT_y(Az').
template <int SCHED>
__global__ void __launch_bounds__(512)
yfwd_comb_kernel(LinePlan<float> pl, SpecPass sp, KTables kt, float2* __restrict__ Ax,
                 const float2* __restrict__ Ay, const float2* __restrict__ Az,
                 float2* __restrict__ D) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int64_t colad[64];
  __shared__ int ca[64], cb[64];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int cols = sp.cols, ld = cols + 1, n = pl.n;
  float2* s0 = reinterpret_cast<float2*>(smraw);
  float2* s1 = s0 + n * ld;
  int64_t es, off = (int64_t)sp.nx * sp.ny * sp.h;
  spec_columns(sp, 1, blockIdx.x, colad, ca, cb, &es, &off, tid);
  __syncthreads();
  tile_load(s0, ld, Ax, colad, es, n, cols, sp.cshift, tid, nthr);
  tile_load(s1, ld, Ay, colad, es, n, cols, sp.cshift, tid, nthr);
  __syncthreads();
  fft_tile<float, SCHED>(s0, ld, pl, sp.cshift, -1, tid, nthr);
  fft_tile<float, SCHED>(s1, ld, pl, sp.cshift, -1, tid, nthr);
  tile_store(s0, ld, Ax, colad, es, n, cols, sp.cshift, tid, nthr);
  for (int f = tid; f < cols * n; f += nthr) {
    int c = f & (cols - 1), j = f >> sp.cshift;
    float cy = __ldg(kt.cy + j);
    float2 v = s1[j * ld + c];
    s1[j * ld + c] = make_float2(v.x * cy, v.y * cy);
  }
  __syncthreads();
  tile_load(s0, ld, Az, colad, es, n, cols, sp.cshift, tid, nthr);
  __syncthreads();
  fft_tile<float, SCHED>(s0, ld, pl, sp.cshift, -1, tid, nthr);
  for (int f = tid; f < cols * n; f += nthr) {
    int c = f & (cols - 1), j = f >> sp.cshift;
    int64_t a = colad[c];
    if (a >= 0) {
      float2 u = s0[j * ld + c], v = s1[j * ld + c];
      D[a + (int64_t)j * es] = make_float2(u.x + v.x, u.y + v.y);
    }
  }
}

// Adjoint x pass with the parameter-gradient reductions.
// Partials per block: [d alpha, d kh, d kl, d nu].
template <int SCHED>
__global__ void __launch_bounds__(512)
xbwd_kernel(LinePlan<float> pl, SpecPass sp, KTables kt, const float* __restrict__ params, int kind,
            int mode, float scale, const float2* __restrict__ Bx, const float2* __restrict__ D,
            const float2* __restrict__ S, float2* __restrict__ Vout, double* __restrict__ partials,
            float2* __restrict__ Wout) {
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int64_t colad[64];
  __shared__ int ca[64], cb[64];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int cols = sp.cols, ld = cols + 1, n = pl.n;
  float2* s0 = reinterpret_cast<float2*>(smraw);
  float2* s1 = s0 + n * ld;
  int64_t es, off = (int64_t)sp.nx * sp.ny * sp.h;
  spec_columns(sp, 0, blockIdx.x, colad, ca, cb, &es, &off, tid);
  __syncthreads();
  tile_load(s0, ld, Bx, colad, es, n, cols, sp.cshift, tid, nthr);
  tile_load(s1, ld, D, colad, es, n, cols, sp.cshift, tid, nthr);
  __syncthreads();
  fft_tile<float, SCHED>(s0, ld, pl, sp.cshift, -1, tid, nthr);
  fft_tile<float, SCHED>(s1, ld, pl, sp.cshift, -1, tid, nthr);
  const float alpha = __ldg(params + 0), kh = __ldg(params + 2), kl = __ldg(params + 3),
              nu = __ldg(params + 4);
  const float pc = pot_coef(kind);
  const float a1 = pc * scale;  // d P / d alpha = 1e-2 G S / Nc (1e-3 for HI)
  const int nz = 2 * sp.h, nyy = sp.ny;
  KahanF acc[4];
  for (int f = tid; f < cols * n; f += nthr) {
    int c = f & (cols - 1), j = f >> sp.cshift;
    int64_t ad = colad[c];
    float2 v = make_float2(0.f, 0.f);
    if (ad >= 0) {
      int kz = cb[c];
      float2 bx = s0[j * ld + c], dd = s1[j * ld + c];
      float cx = __ldg(kt.cx + j);
      // W = i (c_x Bx + D)
      float2 q = make_float2(cx * bx.x + dd.x, cx * bx.y + dd.y);
      float2 W = make_float2(-q.y, q.x);
      if (Wout) Wout[ad + (int64_t)j * es] = W;
      float2 Sv = S[ad + (int64_t)j * es];
      Green gr = green_fn(__ldg(kt.kx + j), __ldg(kt.ky + ca[c]), __ldg(kt.kz + kz), kind, kh, kl, nu);
      // Re(conj(W) S)
      float reWS = W.x * Sv.x + W.y * Sv.y;
      float mk = (kz == 0 || (kz == sp.h && (nz & 1) == 0)) ? 1.f : 2.f;
      float m_alpha = mode == 1 ? mk : 1.f;
      float m_green = mode == 1 ? mk : ((kz >= 1 && kz < nyy / 2) ? 2.f : 1.f);
      acc[0].add(m_alpha * a1 * gr.g * reWS);
      float qg = m_green * pc * alpha * scale * reWS;
      acc[1].add(qg * gr.dkh);
      acc[2].add(qg * gr.dkl);
      acc[3].add(qg * gr.dnu);
      float vm = pc * alpha * scale * gr.g;
      v = make_float2(W.x * vm, W.y * vm);
    }
    s0[j * ld + c] = v;
  }
  __syncthreads();
  fft_tile<float, SCHED>(s0, ld, pl, sp.cshift, +1, tid, nthr);
  tile_store(s0, ld, Vout, colad, es, n, cols, sp.cshift, tid, nthr);
  block_reduce_kahan<4>(acc, partials, 4);
}

// Sums per-block partials in a fixed order: out[slot] = sum_b partials[b*stride + j].
// One block per value j, 256 threads, fixed summation order (strided
// per-thread sums, then a shared-memory tree), so results are reproducible.
// scale_ptr (device, may be null) multiplies the sum; invert != 0 stores 1/sum.
__global__ void __launch_bounds__(256)
finish_kernel(const double* __restrict__ partials, int nblocks, int stride, int nvals,
              double* __restrict__ out, int out_off, const double* __restrict__ scale_ptr,
              int invert) {
  __shared__ double sh[256];
  const int j = blockIdx.x;
  double s = 0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[(int64_t)b * stride + j];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0 && j < nvals) {
    double v = sh[0];
    if (scale_ptr) v *= scale_ptr[0];
    out[out_off + j] = invert ? 1.0 / v : v;
  }
}

// Sum of the mask in FP64 (Npixel) and its reciprocal.
__global__ void mask_count_kernel(const float* __restrict__ mask, int64_t C, double* __restrict__ partials) {
  KahanF acc[1];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < C;
       e += (int64_t)gridDim.x * blockDim.x)
    acc[0].add(__ldg(mask + e));
  block_reduce_kahan<1>(acc, partials, 1);
}
__global__ void set_scalar_kernel(double* out, double v) { out[0] = v; }

}  // namespace jld

