// Pass kernels of the 3-D real FFT (see fft.cu for the pipeline) and their
// launchers.  The z-pass kernels take functors so the fused LDL step can run
// its elementwise source/epilogue math inside the first and last passes.
#pragma once

#include <type_traits>

#include "fft_core.cuh"

namespace jld {

// Raises the dynamic shared-memory limit of kernel `func` on the current
// device (once per kernel and device) when a launch needs more than the
// 48 KB default.
int ensure_smem_ptr(const void* func, size_t bytes);

template <typename F>
inline int ensure_smem(F func, size_t bytes) {
  if (bytes <= 48 * 1024) return JLD_OK;
  return ensure_smem_ptr(reinterpret_cast<const void*>(func), bytes);
}

inline int ilog2i(int v) { int s = 0; while ((1 << s) < v) ++s; return s; }

// ---------------------------------------------------------------------------
// Generic line pass: each tile is `cols` columns of a strided line set.
// Element (column c, line position j) lives at
//   coff + (c / cdiv) * cmul + (c % cdiv) + j * es
// in the input and output (interleaved complex, or split re/im planes).
template <typename T>
struct LineJob {
  const cplx_t<T>* src = nullptr; const T* src_re = nullptr; const T* src_im = nullptr;
  cplx_t<T>* dst = nullptr; T* dst_re = nullptr; T* dst_im = nullptr;
  int64_t es_in = 1, es_out = 1;
  int64_t cdiv_in = INT64_MAX, cmul_in = 0, coff_in = 0;
  int64_t cdiv_out = INT64_MAX, cmul_out = 0, coff_out = 0;
  int64_t ncol = 0;
  int64_t tiles = 0;
};

template <typename T>
__device__ __forceinline__ int64_t job_col_in(const LineJob<T>& J, int64_t c) {
  return J.coff_in + (c / J.cdiv_in) * J.cmul_in + (c % J.cdiv_in);
}
template <typename T>
__device__ __forceinline__ int64_t job_col_out(const LineJob<T>& J, int64_t c) {
  return J.coff_out + (c / J.cdiv_out) * J.cmul_out + (c % J.cdiv_out);
}

template <typename T, int SCHED>
__global__ void __launch_bounds__(512)
line_pass_kernel(LinePlan<T> pl, LineJob<T> j0, LineJob<T> j1, int cols, int cshift, int sgn) {
  using C = cplx_t<T>;
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int64_t colin[64], colout[64];
  C* sm = reinterpret_cast<C*>(smraw);
  const int tid = threadIdx.x, nthr = blockDim.x;
  int64_t b = blockIdx.x;
  const bool second = b >= j0.tiles;
  const LineJob<T>& J = second ? j1 : j0;
  if (second) b -= j0.tiles;
  const int n = pl.n, ld = cols + 1;
  const int64_t c0 = b * cols;
  if (tid < cols) {
    int64_t cc = c0 + tid;
    colin[tid] = cc < J.ncol ? job_col_in(J, cc) : -1;
    colout[tid] = cc < J.ncol ? job_col_out(J, cc) : -1;
  }
  __syncthreads();
  const int total = cols * n;
  const bool contig_in = J.es_in == 1, contig_out = J.es_out == 1;
  for (int f = tid; f < total; f += nthr) {
    int c, jj;
    if (contig_in) { c = f / n; jj = f - c * n; } else { c = f & (cols - 1); jj = f >> cshift; }
    int64_t a = colin[c];
    C v;
    if (a >= 0) {
      a += (int64_t)jj * J.es_in;
      if (J.src) v = J.src[a];
      else { v.x = J.src_re[a]; v.y = J.src_im[a]; }
    } else { v.x = T(0); v.y = T(0); }
    sm[jj * ld + c] = v;
  }
  __syncthreads();
  fft_tile<T, SCHED>(sm, ld, pl, cshift, sgn, tid, nthr);
  for (int f = tid; f < total; f += nthr) {
    int c, jj;
    if (contig_out) { c = f / n; jj = f - c * n; } else { c = f & (cols - 1); jj = f >> cshift; }
    int64_t a = colout[c];
    if (a >= 0) {
      a += (int64_t)jj * J.es_out;
      C v = sm[jj * ld + c];
      if (J.dst) J.dst[a] = v;
      else { J.dst_re[a] = v.x; J.dst_im[a] = v.y; }
    }
  }
}

// ---------------------------------------------------------------------------
// z pass, forward r2c.  A real row of length nz = 2h is read as h complex
// values (even, odd samples), transformed, and split:
//   X[k] = Xe + W^k Xo,  X[h-k] = conj(Xe - W^k Xo),
//   Xe = (Z[k] + conj Z[h-k]) / 2,  Xo = -i (Z[k] - conj Z[h-k]) / 2,
// W = exp(-2 pi i / nz).  X[0..h-1] go to main, X[h] to nyq.
struct IdentitySrc {
  template <typename T>
  __device__ __forceinline__ T operator()(T v, int64_t) const { return v; }
};

template <typename T, int SCHED, class Src>
__global__ void __launch_bounds__(512)
rfft_z_kernel(LinePlan<T> pl, const cplx_t<T>* __restrict__ twr, const T* __restrict__ in,
              Src src, cplx_t<T>* __restrict__ main, cplx_t<T>* __restrict__ nyq,
              int64_t rows, int cols, int cshift) {
  using C = cplx_t<T>;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int h = pl.n, ld = cols + 1;
  const int64_t row0 = (int64_t)blockIdx.x * cols;
  const C* in2 = reinterpret_cast<const C*>(in);
  for (int f = tid; f < cols * h; f += nthr) {
    int c = f / h, j = f - c * h;
    int64_t row = row0 + c;
    C v;
    if (row < rows) {
      int64_t e = row * h + j;  // complex index == real index / 2
      v = __ldg(in2 + e);
      v.x = src(v.x, 2 * e);
      v.y = src(v.y, 2 * e + 1);
    } else { v.x = T(0); v.y = T(0); }
    sm[j * ld + c] = v;
  }
  __syncthreads();
  fft_tile<T, SCHED>(sm, ld, pl, cshift, -1, tid, nthr);
  const int hh = h / 2 + 1;
  for (int f = tid; f < cols * hh; f += nthr) {
    int c = f / hh, k = f - c * hh;
    int64_t row = row0 + c;
    if (row >= rows) continue;
    C z = sm[(k % h) * ld + c];
    C zm = sm[((h - k) % h) * ld + c];
    C zc = cconj(zm);
    C xe = cscale(cadd(z, zc), T(0.5));
    C d = cscale(csub(z, zc), T(0.5));
    C xo = cmake<C>(d.y, -d.x);  // -i * d
    C w = __ldg(twr + k);
    C wxo = cmul(w, xo);
    C xk = cadd(xe, wxo);
    C xhk = cconj(csub(xe, wxo));
    main[row * h + k] = xk;
    if (k == 0) nyq[row] = xhk;
    else if (h - k != k) main[row * h + (h - k)] = xhk;
  }
}

// ---------------------------------------------------------------------------
// z pass, inverse c2r.  Builds Z'[k] = (X[k] + conj X[h-k]) +
// i W^-k (X[k] - conj X[h-k]) with the imaginary parts of X[0] and X[h]
// dropped, inverse-transforms it, and hands (x[2m], x[2m+1]) = z[m] to dst.
struct RowStoreDst {
  template <typename T>
  __device__ __forceinline__ void operator()(T* out, int64_t row, int h, int m, T a, T b) const {
    cplx_t<T> v; v.x = a; v.y = b;
    reinterpret_cast<cplx_t<T>*>(out)[row * h + m] = v;
  }
};

template <typename T, int SCHED, class Dst>
__global__ void __launch_bounds__(512)
irfft_z_kernel(LinePlan<T> pl, const cplx_t<T>* __restrict__ twr,
               const cplx_t<T>* __restrict__ main, const cplx_t<T>* __restrict__ nyq,
               T* __restrict__ out, Dst dst, int64_t rows, int cols, int cshift) {
  using C = cplx_t<T>;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int h = pl.n, ld = cols + 1;
  const int64_t row0 = (int64_t)blockIdx.x * cols;
  for (int f = tid; f < cols * h; f += nthr) {
    int c = f / h, k = f - c * h;
    int64_t row = row0 + c;
    C v;
    if (row < rows) {
      C xk = main[row * h + k];
      C xh = (k == 0) ? nyq[row] : main[row * h + (h - k)];
      if (k == 0) { xk.y = T(0); xh.y = T(0); }
      C xc = cconj(xh);
      C a = cadd(xk, xc), bb = csub(xk, xc);
      C wi = cconj(__ldg(twr + k));
      C t = cmul(wi, bb);
      v = cmake<C>(a.x - t.y, a.y + t.x);  // a + i t
    } else { v.x = T(0); v.y = T(0); }
    sm[k * ld + c] = v;
  }
  __syncthreads();
  fft_tile<T, SCHED>(sm, ld, pl, cshift, +1, tid, nthr);
  for (int f = tid; f < cols * h; f += nthr) {
    int c = f / h, m = f - c * h;
    int64_t row = row0 + c;
    if (row < rows) {
      C z = sm[m * ld + c];
      dst(out, row, h, m, z.x, z.y);
    }
  }
}

// Calls body(std::integral_constant<int, SCHED>) for the schedule class of pl.
template <typename T, class F>
inline int with_sched(const LinePlan<T>& pl, F&& body) {
  switch (sched_of(pl)) {
    case 1: return body(std::integral_constant<int, 1>());
    case 2: return body(std::integral_constant<int, 2>());
    case 4: return body(std::integral_constant<int, 4>());
    case 8: return body(std::integral_constant<int, 8>());
    default: return body(std::integral_constant<int, kSchedGen>());
  }
}

// ---------------------------------------------------------------------------
// Launchers.

template <typename T, class Src>
int launch_rfft_z_src(cudaStream_t st, const Plan3<T>& pl, const T* data, Src src,
                      cplx_t<T>* main, cplx_t<T>* nyq) {
  const LinePlan<T>& lp = pl.pz;
  int cols = tile_cols(lp.n, lp.E, sizeof(cplx_t<T>));
  int nthr = cols * lp.n / lp.E;
  int64_t rows = (int64_t)pl.nx * pl.ny;
  unsigned grid = (unsigned)((rows + cols - 1) / cols);
  size_t smem = (size_t)lp.n * (cols + 1) * sizeof(cplx_t<T>);
  int s = with_sched(lp, [&](auto sc) {
    constexpr int S = decltype(sc)::value;
    int e = ensure_smem(rfft_z_kernel<T, S, Src>, smem);
    if (e) return e;
    rfft_z_kernel<T, S, Src><<<grid, nthr, smem, st>>>(lp, pl.twr, data, src, main, nyq, rows,
                                                       cols, ilog2i(cols));
    return 0;
  });
  if (s) return s;
  JLD_LAUNCH_CHECK("rfft_z_kernel");
  return JLD_OK;
}

template <typename T>
int launch_rfft_z(cudaStream_t st, const Plan3<T>& pl, const T* data, const void*,
                  cplx_t<T>* main, cplx_t<T>* nyq) {
  return launch_rfft_z_src<T, IdentitySrc>(st, pl, data, IdentitySrc(), main, nyq);
}

template <typename T, class Dst>
int launch_irfft_z_dst(cudaStream_t st, const Plan3<T>& pl, const cplx_t<T>* main,
                       const cplx_t<T>* nyq, T* out, Dst dst) {
  const LinePlan<T>& lp = pl.pz;
  int cols = tile_cols(lp.n, lp.E, sizeof(cplx_t<T>));
  int nthr = cols * lp.n / lp.E;
  int64_t rows = (int64_t)pl.nx * pl.ny;
  unsigned grid = (unsigned)((rows + cols - 1) / cols);
  size_t smem = (size_t)lp.n * (cols + 1) * sizeof(cplx_t<T>);
  int s = with_sched(lp, [&](auto sc) {
    constexpr int S = decltype(sc)::value;
    int e = ensure_smem(irfft_z_kernel<T, S, Dst>, smem);
    if (e) return e;
    irfft_z_kernel<T, S, Dst><<<grid, nthr, smem, st>>>(lp, pl.twr, main, nyq, out, dst, rows,
                                                        cols, ilog2i(cols));
    return 0;
  });
  if (s) return s;
  JLD_LAUNCH_CHECK("irfft_z_kernel");
  return JLD_OK;
}

template <typename T>
int launch_irfft_z(cudaStream_t st, const Plan3<T>& pl, const cplx_t<T>* main,
                   const cplx_t<T>* nyq, T* out) {
  return launch_irfft_z_dst<T, RowStoreDst>(st, pl, main, nyq, out, RowStoreDst());
}

template <typename T>
int launch_line_pass(cudaStream_t st, const LinePlan<T>& lp, LineJob<T> j0, LineJob<T> j1,
                     int sgn) {
  int cols = tile_cols(lp.n, lp.E, sizeof(cplx_t<T>));
  int nthr = cols * lp.n / lp.E;
  j0.tiles = (j0.ncol + cols - 1) / cols;
  j1.tiles = (j1.ncol + cols - 1) / cols;
  int64_t grid = j0.tiles + j1.tiles;
  if (grid == 0) return JLD_OK;
  size_t smem = (size_t)lp.n * (cols + 1) * sizeof(cplx_t<T>);
  int s = with_sched(lp, [&](auto sc) {
    constexpr int S = decltype(sc)::value;
    int e = ensure_smem(line_pass_kernel<T, S>, smem);
    if (e) return e;
    line_pass_kernel<T, S><<<(unsigned)grid, nthr, smem, st>>>(lp, j0, j1, cols, ilog2i(cols), sgn);
    return 0;
  });
  if (s) return s;
  JLD_LAUNCH_CHECK("line_pass_kernel");
  return JLD_OK;
}

// y pass on the internal layout, in place: main lines run along y with
// stride h, columns are (x, kz); nyq lines are contiguous rows of length ny.
template <typename T>
int launch_y_pass(cudaStream_t st, const Plan3<T>& pl, cplx_t<T>* main, cplx_t<T>* nyq, int sgn) {
  const int64_t h = pl.h, ny = pl.ny, nx = pl.nx;
  LineJob<T> jm, jn;
  jm.src = main; jm.dst = main;
  jm.es_in = jm.es_out = h;
  jm.cdiv_in = jm.cdiv_out = h;
  jm.cmul_in = jm.cmul_out = ny * h;
  jm.ncol = nx * h;
  jn.src = nyq; jn.dst = nyq;
  jn.es_in = jn.es_out = 1;
  jn.cdiv_in = jn.cdiv_out = 1;
  jn.cmul_in = jn.cmul_out = ny;
  jn.ncol = nx;
  return launch_line_pass<T>(st, pl.py, jm, jn, sgn);
}

// x pass over the internal layout (lines along x).
template <typename T>
LineJob<T> job_x_internal(const Plan3<T>& pl, cplx_t<T>* base, bool is_nyq) {
  const int64_t h = pl.h, ny = pl.ny;
  LineJob<T> j;
  j.src = base; j.dst = base;
  j.es_in = j.es_out = is_nyq ? ny : ny * h;
  j.ncol = is_nyq ? ny : ny * h;
  return j;
}

// Redirects a job's output to the caller layout (nx, ny, h+1).
template <typename T>
void set_job_out_ref(LineJob<T>& j, const Plan3<T>& pl, bool is_nyq, cplx_t<T>* out_c,
                     T* re, T* im) {
  const int64_t h = pl.h, ny = pl.ny;
  j.dst = out_c; j.dst_re = re; j.dst_im = im;
  j.es_out = ny * (h + 1);
  if (is_nyq) { j.cdiv_out = 1; j.cmul_out = h + 1; j.coff_out = h; }
  else { j.cdiv_out = h; j.cmul_out = h + 1; j.coff_out = 0; }
}

// Redirects a job's input to the caller layout (nx, ny, h+1).
template <typename T>
void set_job_in_ref(LineJob<T>& j, const Plan3<T>& pl, bool is_nyq, const cplx_t<T>* in_c,
                    const T* re, const T* im) {
  const int64_t h = pl.h, ny = pl.ny;
  j.src = in_c; j.src_re = re; j.src_im = im;
  j.es_in = ny * (h + 1);
  if (is_nyq) { j.cdiv_in = 1; j.cmul_in = h + 1; j.coff_in = h; }
  else { j.cdiv_in = h; j.cmul_in = h + 1; j.coff_in = 0; }
}

}  // namespace jld
