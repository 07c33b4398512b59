// 3-D real FFT pair on sm_103a: pencil passes over a split-Nyquist internal
// half-spectrum, each pass a shared-memory Stockham transform (fft_core.cuh).
//
// Replaces the FFTW-MPI slab transforms of the reference:
//   buildplan/buildplanf  lib/parfft.h:33-76   -> get_plan3 / jld_buildplan_*
//   pfft/pfftf + split    lib/parfft.h:78-94,111-125, lib/cpu.cc:169-200
//   pifft/pifftf + depad  lib/parfft.h:96-109,127-138, lib/cpu.cc:202-245
// Conventions (FFTW's): forward r2c is unnormalised with sign -1 over all
// three axes, keeping kz in [0, nz/2]; the inverse c2r is unnormalised with
// sign +1, done as complex inverses along x and y followed by a c2r along z
// that ignores the imaginary parts of kz = 0 and kz = nz/2.
//
// Forward (r2c):  z pass  real rows -> internal (even/odd packing: a length
//                 nz real row is one length nz/2 complex FFT plus a split)
//                 y pass  in place on the internal layout
//                 x pass  internal -> caller layout (nx, ny, nz/2+1)
// Inverse (c2r):  x pass  caller layout -> internal, y pass in place,
//                 z pass  internal -> real rows.

#include <map>
#include <mutex>
#include <tuple>
#include <vector>
#include <cmath>
#include <type_traits>

#include "fft_core.cuh"
#include "fft_passes.cuh"
#include "pipe_host.cuh"

namespace jld {

// ---------------------------------------------------------------------------
// Schedules.

static int lcm_int(int a, int b) {
  int x = a, y = b;
  while (y) { int t = x % y; x = y; y = t; }
  return a / x * b;
}

// Picks the radix sequence and elements-per-thread E for length n.
// Powers of two use radix 16 (then 8/4/2), E = min(16, n).  Mixed lengths
// use radices 4/2, 3 and 5 with E = lcm of the radices (at most 30).
static bool make_line_schedule(int n, int* E, int* nst, int* radix) {
  if (n < 1) return false;
  int a = 0, b = 0, c = 0, m = n;
  while (m % 2 == 0) { m /= 2; ++a; }
  while (m % 3 == 0) { m /= 3; ++b; }
  while (m % 5 == 0) { m /= 5; ++c; }
  if (m != 1) return false;
  int k = 0;
  if (b == 0 && c == 0) {
    while (a >= 4) { radix[k++] = 16; a -= 4; }
    if (a == 3) radix[k++] = 8;
    else if (a == 2) radix[k++] = 4;
    else if (a == 1) radix[k++] = 2;
  } else {
    if (c == 0) {
      while (a >= 2) { radix[k++] = 4; a -= 2; }
      if (a == 1) radix[k++] = 2;
    } else {
      while (a >= 1) { radix[k++] = 2; a -= 1; }
    }
    while (b-- > 0) radix[k++] = 3;
    while (c-- > 0) radix[k++] = 5;
  }
  if (k > kMaxStages) return false;
  int e = 1;
  for (int s = 0; s < k; ++s) e = lcm_int(e, radix[s]);
  *E = e;
  *nst = k;
  return true;
}

int tile_cols(int n, int E, size_t elem_bytes) {
  int cols = 16;
  while (cols > 1 && (int64_t)cols * n / E > 512) cols >>= 1;
  while (cols > 1 && (size_t)n * (cols + 1) * elem_bytes > 200 * 1024) cols >>= 1;
  // Small transforms: widen the tile so a CTA has a useful number of threads.
  while (cols < 64 && (int64_t)(cols * 2) * n / E <= 256 &&
         (size_t)n * (cols * 2 + 1) * elem_bytes <= 48 * 1024)
    cols <<= 1;
  return cols;
}

// ---------------------------------------------------------------------------
// Plan cache: one entry per (device, dtype, nx, ny, nz), never freed.

struct PlanEntry {
  int E[3], nst[3], radix[3][kMaxStages];
  void* dev = nullptr;  // twiddle tables
  size_t off[4];        // element offsets of tables x, y, z, r2c split
};

static std::mutex g_plan_mu;
static std::map<std::tuple<int, int, int, int, int>, PlanEntry> g_plans;

template <typename T>
static void fill_twiddles(std::vector<cplx_t<T>>& v, size_t off, int n, int count) {
  // exp(-2 pi i m / n) in FP64, reduced to the first octant-free form
  // cos(2 pi m/n), -sin(2 pi m/n) with m taken mod n.
  const double two_pi = 6.283185307179586476925286766559;
  for (int m = 0; m < count; ++m) {
    long mm = m % n;
    double ang = two_pi * (double)mm / (double)n;
    v[off + m].x = (T)std::cos(ang);
    v[off + m].y = (T)(-std::sin(ang));
  }
}

template <typename T>
int get_plan3(int nx, int ny, int nz, bool build, Plan3<T>* out) {
  if (nx < 1 || ny < 1 || nz < 2 || (nz & 1))
    return set_error(JLD_ERR_UNSUPPORTED, "FFT: mesh (%d,%d,%d) unsupported (need nz even >= 2)",
                     nx, ny, nz);
  int dev = 0;
  JLD_CUDA_TRY(cudaGetDevice(&dev));
  const int h = nz / 2;
  auto key = std::make_tuple(dev, (int)sizeof(T), nx, ny, nz);
  std::lock_guard<std::mutex> lock(g_plan_mu);
  auto it = g_plans.find(key);
  if (it == g_plans.end()) {
    if (!build)
      return set_error(JLD_ERR_NOPLAN,
                       "FFT plan for (%d,%d,%d) missing; call jld_buildplan before stream capture",
                       nx, ny, nz);
    PlanEntry e;
    const int lens[3] = {nx, ny, h};
    for (int a = 0; a < 3; ++a)
      if (!make_line_schedule(lens[a], &e.E[a], &e.nst[a], e.radix[a]))
        return set_error(JLD_ERR_UNSUPPORTED,
                         "FFT: length %d does not factor into 2, 3 and 5", lens[a]);
    e.off[0] = 0;
    e.off[1] = e.off[0] + nx;
    e.off[2] = e.off[1] + ny;
    e.off[3] = e.off[2] + h;
    size_t total = e.off[3] + h + 1;
    std::vector<cplx_t<T>> host(total);
    fill_twiddles<T>(host, e.off[0], nx, nx);
    fill_twiddles<T>(host, e.off[1], ny, ny);
    fill_twiddles<T>(host, e.off[2], h, h);
    fill_twiddles<T>(host, e.off[3], nz, h + 1);
    JLD_CUDA_TRY(cudaMalloc(&e.dev, total * sizeof(cplx_t<T>)));
    JLD_CUDA_TRY(cudaMemcpy(e.dev, host.data(), total * sizeof(cplx_t<T>),
                            cudaMemcpyHostToDevice));
    it = g_plans.emplace(key, e).first;
  }
  const PlanEntry& e = it->second;
  const cplx_t<T>* base = (const cplx_t<T>*)e.dev;
  out->nx = nx; out->ny = ny; out->nz = nz; out->h = h;
  LinePlan<T>* lp[3] = {&out->px, &out->py, &out->pz};
  const int lens[3] = {nx, ny, h};
  for (int a = 0; a < 3; ++a) {
    lp[a]->n = lens[a];
    lp[a]->E = e.E[a];
    lp[a]->nst = e.nst[a];
    for (int s = 0; s < kMaxStages; ++s) lp[a]->radix[s] = s < e.nst[a] ? e.radix[a][s] : 0;
    lp[a]->tw = base + e.off[a];
  }
  out->twr = base + e.off[3];
  return JLD_OK;
}

template int get_plan3<float>(int, int, int, bool, Plan3<float>*);
template int get_plan3<double>(int, int, int, bool, Plan3<double>*);

// Returns the plan for an FFT call: built on demand unless the stream is
// being captured into a CUDA graph (plan building allocates and copies).
template <typename T>
static int plan_for_call(cudaStream_t st, int nx, int ny, int nz, Plan3<T>* pl) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  JLD_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
  return get_plan3<T>(nx, ny, nz, cs == cudaStreamCaptureStatusNone, pl);
}

// ---------------------------------------------------------------------------
// Full transforms.

// Complex buffers (and the real input of r2c / output of c2r, which the
// passes access as pairs) must be aligned to one complex element.
template <typename T>
static bool cplx_aligned(const void* p) {
  return ((uintptr_t)p % sizeof(cplx_t<T>)) == 0;
}

template <typename T>
static int fft_args_check(int nx, int ny, int nz, const void* ws, size_t ws_bytes,
                          const char* who) {
  if (nx < 1 || ny < 1 || nz < 2)
    return set_error(JLD_ERR_ARG, "%s: mesh sizes must be positive (nz >= 2)", who);
  if (nz & 1) return set_error(JLD_ERR_UNSUPPORTED, "%s: nz must be even", who);
  size_t need = (size_t)nx * ny * (nz / 2 + 1) * sizeof(cplx_t<T>);
  if (!ws || ws_bytes < need)
    return set_error(JLD_ERR_WORKSPACE, "%s: workspace of %zu bytes needed, got %zu", who,
                     need, ws ? ws_bytes : (size_t)0);
  return JLD_OK;
}

// ---------------------------------------------------------------------------
// Pipelined single-precision transforms for power-of-two meshes
// (16 <= nx, ny, nz/2 <= 2048): the z pass and the y pass run on the
// TMA / bulk-copy staged kernels of the fused step, the x pass of the r2c
// writes the caller's layout straight from its last FFT stage.  The nyq
// plane (kz = nz/2) keeps the generic line kernel.  The c2r reads the
// caller's layout with the generic x pass (its rows of nz/2+1 complex values
// are not 16-byte aligned for a tensor copy) and pipelines y and z.
//
// A copy that never arrives makes a pipelined pass stop after a bounded wait
// and set the library's pass error word (jld_fft_error_word).
static __device__ int g_fft_pipe_err;
static std::mutex g_err_mu;
static int* g_err_ptr[64];

static int fft_err_word(int** out) {
  int dev = 0;
  JLD_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(JLD_ERR_UNSUPPORTED, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_err_mu);
  if (!g_err_ptr[dev]) JLD_CUDA_TRY(cudaGetSymbolAddress((void**)&g_err_ptr[dev], g_fft_pipe_err));
  *out = g_err_ptr[dev];
  return JLD_OK;
}

static bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// Error-path check of the bounded waits: an mbarrier armed for 16 bytes of
// a copy that is never issued, so its phase cannot complete.  The CTA polls
// it with the same bounded wait as the pipelined passes, gives up after
// `polls` tries, records kWaitSelftestCode in `word` and returns.  Nothing is
// in flight, so giving up touches no memory but the word.
constexpr int kWaitSelftestCode = 99;
__global__ void __launch_bounds__(32) wait_selftest_kernel(int polls, int* word) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar, 16);
  __syncthreads();
  const bool done = mbar_wait_bounded(&bar, 0, polls);
  if (!__syncthreads_or(done) && threadIdx.x == 0) atomicExch(word, kWaitSelftestCode);
}

static int wait_selftest(cudaStream_t st, int polls, int* word) {
  if (polls < 1 || polls > kWaitLimit)
    return set_error(JLD_ERR_ARG, "jld_wait_selftest: polls must be in [1, %d]", kWaitLimit);
  if (!word) {
    int s = fft_err_word(&word);
    if (s) return s;
  }
  wait_selftest_kernel<<<1, 32, 0, st>>>(polls, word);
  JLD_LAUNCH_CHECK("wait_selftest_kernel");
  return JLD_OK;
}

struct FftPipe {
  bool ok = false;
  PipeGeom py, px;
  ZPipeGeom z;
};

static FftPipe fft_pipe_geom(int nx, int ny, int nz, bool c2r) {
  FftPipe f;
  const int h = nz / 2;
  const int64_t rows = (int64_t)nx * ny;
  f.py = pipe_geom(nx, ny, h, 1, 0);
  f.px = pipe_geom(nx, ny, h, 0, 0);
  f.z = c2r ? zpipe_geom(rows, h, 1, (size_t)(h + 1) * 8) : zpipe_geom(rows, h, 1, (size_t)h * 8, 110 * 1024, kZr2cThreads);
  f.ok = f.py.ok && f.px.ok && f.z.ok && (c2r || f.px.ok);
  return f;
}

// y FFT of the internal layout in place: pipelined main block + nyq rows.
static int pipe_y_pass(cudaStream_t st, const Plan3<float>& pl, const FftPipe& fp, float2* main, int sgn,
                       int* err) {
  const int nx = pl.nx, ny = pl.ny, h = pl.h;
  CUtensorMap m;
  int s = make_main_map(&m, main, nx, ny, h, 1, fp.py.g.cols, ny);
  if (s) return s;
  s = with_p2(ny, [&](auto sch) {
    using Sch = decltype(sch);
    auto kern = sgn < 0 ? spass_kernel<Sch, 1, -1> : spass_kernel<Sch, 1, 1>;
    int r = ensure_smem(kern, fp.py.smem);
    if (r) return r;
    kern<<<fp.py.grid, fp.py.nthr, fp.py.smem, st>>>(m, main, fp.py.g, pl.py.tw, err, nullptr);
    return 0;
  });
  if (s) return s;
  JLD_LAUNCH_CHECK("spass_kernel");
  LineJob<float> jn, none;
  float2* nq = main + (size_t)nx * ny * h;
  jn.src = nq; jn.dst = nq;
  jn.es_in = jn.es_out = 1;
  jn.cdiv_in = jn.cdiv_out = 1;
  jn.cmul_in = jn.cmul_out = ny;
  jn.ncol = nx;
  return launch_line_pass<float>(st, pl.py, jn, none, sgn);
}

static int rfft3_pipe(cudaStream_t st, const Plan3<float>& pl, const FftPipe& fp, const float* data,
                      float2* out_c, float* out_re, float* out_im, float2* main) {
  const int nx = pl.nx, ny = pl.ny, h = pl.h;
  int* err = nullptr;
  int s = fft_err_word(&err);
  if (s) return s;
  s = with_p2(h, [&](auto sch) {
    using Sch = decltype(sch);
    auto kern = zr2c_pipe_kernel<Sch, SrcIdentity>;
    unsigned gz = 0;
    int r = ensure_smem(kern, fp.z.smem);
    if (!r) r = persistent_grid(kern, fp.z.nthr, fp.z.smem, fp.z.zt.ntiles, &gz);
    if (r) return r;
    kern<<<gz, fp.z.nthr, fp.z.smem, st>>>(data, SrcIdentity{}, fp.z.zt, pl.twr, main, pl.pz.tw, err, nullptr);
    return 0;
  });
  if (s) return s;
  JLD_LAUNCH_CHECK("zr2c_pipe_kernel");
  if ((s = pipe_y_pass(st, pl, fp, main, -1, err))) return s;
  CUtensorMap m;
  if ((s = make_main_map(&m, main, nx, ny, h, 0, fp.px.g.cols, nx))) return s;
  s = with_p2(nx, [&](auto sch) {
    using Sch = decltype(sch);
    auto kern = xref_pipe_kernel<Sch, -1>;
    int r = ensure_smem(kern, fp.px.smem);
    if (r) return r;
    kern<<<fp.px.grid, fp.px.nthr, fp.px.smem, st>>>(m, out_c, out_re, out_im, fp.px.g, pl.px.tw, err);
    return 0;
  });
  if (s) return s;
  JLD_LAUNCH_CHECK("xref_pipe_kernel");
  LineJob<float> jn = job_x_internal<float>(pl, main + (size_t)nx * ny * h, true), none;
  set_job_out_ref<float>(jn, pl, true, out_c, out_re, out_im);
  return launch_line_pass<float>(st, pl.px, jn, none, -1);
}

static int irfft3_pipe(cudaStream_t st, const Plan3<float>& pl, const FftPipe& fp, const float2* in_c,
                       const float* in_re, const float* in_im, float* out, float2* main) {
  const int nx = pl.nx, ny = pl.ny, h = pl.h;
  int* err = nullptr;
  int s = fft_err_word(&err);
  if (s) return s;
  float2* nyq = main + (size_t)nx * ny * h;
  LineJob<float> jm = job_x_internal<float>(pl, main, false);
  LineJob<float> jn = job_x_internal<float>(pl, nyq, true);
  set_job_in_ref<float>(jm, pl, false, in_c, in_re, in_im);
  set_job_in_ref<float>(jn, pl, true, in_c, in_re, in_im);
  if ((s = launch_line_pass<float>(st, pl.px, jm, jn, +1))) return s;
  if ((s = pipe_y_pass(st, pl, fp, main, +1, err))) return s;
  s = with_p2(h, [&](auto sch) {
    using Sch = decltype(sch);
    auto kern = zc2r_pipe_kernel<Sch>;
    unsigned gz = 0;
    int r = ensure_smem(kern, fp.z.smem);
    if (!r) r = persistent_grid(kern, fp.z.nthr, fp.z.smem, fp.z.zt.ntiles, &gz);
    if (r) return r;
    kern<<<gz, fp.z.nthr, fp.z.smem, st>>>(main, fp.z.zt, pl.twr, out, pl.pz.tw, err, nullptr);
    return 0;
  });
  if (s) return s;
  JLD_LAUNCH_CHECK("zc2r_pipe_kernel");
  return JLD_OK;
}

// r2c: data (nx,ny,nz) real -> out in caller layout (interleaved, or split
// when out_c == nullptr).
template <typename T>
static int rfft3(cudaStream_t st, const T* data, int nx, int ny, int nz, cplx_t<T>* out_c,
                 T* out_re, T* out_im, void* ws, size_t ws_bytes, const char* who) {
  int s = fft_args_check<T>(nx, ny, nz, ws, ws_bytes, who);
  if (s) return s;
  if (!data || (!out_c && (!out_re || !out_im)))
    return set_error(JLD_ERR_ARG, "%s: NULL data or output", who);
  if (!cplx_aligned<T>(data) || !cplx_aligned<T>(ws) || (out_c && !cplx_aligned<T>(out_c)))
    return set_error(JLD_ERR_ARG, "%s: data, workspace and complex output must be %zu-byte aligned", who,
                     sizeof(cplx_t<T>));
  Plan3<T> pl;
  if ((s = plan_for_call<T>(st, nx, ny, nz, &pl))) return s;
  const int h = pl.h;
  cplx_t<T>* main = (cplx_t<T>*)ws;
  cplx_t<T>* nyq = main + (size_t)nx * ny * h;
  if constexpr (std::is_same<T, float>::value) {
    // bulk and tensor copies need 16-byte aligned sources and staging
    const bool aligned = al16(data) && al16(ws) && ((uintptr_t)out_c % 8 == 0);
    const FftPipe fp = fft_pipe_geom(nx, ny, nz, false);
    if (fp.ok && aligned) return rfft3_pipe(st, pl, fp, data, out_c, out_re, out_im, main);
  }
  if ((s = launch_rfft_z<T>(st, pl, data, nullptr, main, nyq))) return s;
  if ((s = launch_y_pass<T>(st, pl, main, nyq, -1))) return s;
  // x pass: internal -> caller layout (row length h+1)
  LineJob<T> jm = job_x_internal<T>(pl, main, false);
  LineJob<T> jn = job_x_internal<T>(pl, nyq, true);
  set_job_out_ref<T>(jm, pl, false, out_c, out_re, out_im);
  set_job_out_ref<T>(jn, pl, true, out_c, out_re, out_im);
  return launch_line_pass<T>(st, pl.px, jm, jn, -1);
}

template <typename T>
static int irfft3(cudaStream_t st, const cplx_t<T>* in_c, const T* in_re, const T* in_im,
                  int nx, int ny, int nz, T* out, void* ws, size_t ws_bytes, const char* who) {
  int s = fft_args_check<T>(nx, ny, nz, ws, ws_bytes, who);
  if (s) return s;
  if (!out || (!in_c && (!in_re || !in_im)))
    return set_error(JLD_ERR_ARG, "%s: NULL input or output", who);
  if (!cplx_aligned<T>(out) || !cplx_aligned<T>(ws) || (in_c && !cplx_aligned<T>(in_c)))
    return set_error(JLD_ERR_ARG, "%s: output, workspace and complex input must be %zu-byte aligned", who,
                     sizeof(cplx_t<T>));
  Plan3<T> pl;
  if ((s = plan_for_call<T>(st, nx, ny, nz, &pl))) return s;
  const int h = pl.h;
  cplx_t<T>* main = (cplx_t<T>*)ws;
  cplx_t<T>* nyq = main + (size_t)nx * ny * h;
  if constexpr (std::is_same<T, float>::value) {
    const bool aligned = al16(ws) && al16(out);
    const FftPipe fp = fft_pipe_geom(nx, ny, nz, true);
    if (fp.ok && aligned) return irfft3_pipe(st, pl, fp, in_c, in_re, in_im, out, main);
  }
  LineJob<T> jm = job_x_internal<T>(pl, main, false);
  LineJob<T> jn = job_x_internal<T>(pl, nyq, true);
  set_job_in_ref<T>(jm, pl, false, in_c, in_re, in_im);
  set_job_in_ref<T>(jn, pl, true, in_c, in_re, in_im);
  if ((s = launch_line_pass<T>(st, pl.px, jm, jn, +1))) return s;
  if ((s = launch_y_pass<T>(st, pl, main, nyq, +1))) return s;
  return launch_irfft_z<T>(st, pl, main, nyq, out);
}

// ---------------------------------------------------------------------------
// Allocation-free r2c (jld_pfft_c_static_f32).
//
// For callers that cannot allocate device memory themselves -- code running
// inside a host framework that owns every allocation, or code running where
// allocation is forbidden (for example between the setup and the launch of a
// captured sequence) -- this variant keeps its scratch and its twiddle tables
// in file-scope device arrays instead of a caller workspace and the plan
// cache.  Limits: the internal half spectrum (nx * ny * (nz/2 + 1) complex
// floats) must fit in kStaticScratchBytes = 72 MiB (256^3 fits), and each of
// nx, ny, nz must be at most 4096.  The arrays are part of the library image,
// so every GPU that loads libjld holds them until the process exits.
//
// Host code must not pass the arrays' names to a kernel: on the host they are
// stand-ins, not device addresses.  The first call on each device resolves
// their device addresses with cudaGetSymbolAddress (with that device
// current); make that first call before any stream capture.  Every call
// shares both arrays and rewrites both -- the twiddle table for its own
// shape, the scratch by its passes (it needs no clearing: each pass writes
// all of it before it is read) -- so calls that overlap on the GPU (on two
// streams, or on one device from two threads) race on the twiddles as well
// as on the scratch.
static constexpr size_t kStaticScratchBytes = (size_t)72 << 20;
static constexpr int kStaticMaxLen = 4096;
static constexpr int kStaticTwLen = 2 * kStaticMaxLen + kStaticMaxLen / 2 + kStaticMaxLen / 2 + 1;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];
static __device__ __align__(256) float2 g_static_tw[kStaticTwLen];

struct StaticDev {
  bool ready = false;
  void* scratch = nullptr;
  float2* tw = nullptr;
};
static std::mutex g_static_mu;
static StaticDev g_static_dev[64];

// Resolves the device addresses of the file-scope arrays once per device.
static int static_setup(StaticDev* out) {
  int dev = 0;
  JLD_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(JLD_ERR_UNSUPPORTED, "device index %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_static_mu);
  StaticDev& s = g_static_dev[dev];
  if (!s.ready) {
    JLD_CUDA_TRY(cudaGetSymbolAddress(&s.scratch, g_static_scratch));
    JLD_CUDA_TRY(cudaGetSymbolAddress((void**)&s.tw, g_static_tw));
    s.ready = true;
  }
  *out = s;
  return JLD_OK;
}

// tw[m] = exp(-2 pi i (m mod n) / n) in FP64, rounded to float.
__global__ void static_twiddles_kernel(float2* tw, int n, int count) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < count; m += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)(m % n) / (double)n, &s, &c);
    tw[m] = make_float2((float)c, (float)(-s));
  }
}

static int pfft_static_impl(cudaStream_t st, const float* data, int nx, int ny, int nz, float2* out_c) {
  const char* who = "jld_pfft_c_static_f32";
  if (!data || !out_c) return set_error(JLD_ERR_ARG, "%s: NULL data or output", who);
  if (!cplx_aligned<float>(data) || !cplx_aligned<float>(out_c))
    return set_error(JLD_ERR_ARG, "%s: data and output must be 8-byte aligned", who);
  if (nx < 1 || ny < 1 || nz < 2) return set_error(JLD_ERR_ARG, "%s: mesh sizes must be positive (nz >= 2)", who);
  if (nz & 1) return set_error(JLD_ERR_UNSUPPORTED, "%s: nz must be even", who);
  if (nx > kStaticMaxLen || ny > kStaticMaxLen || nz > kStaticMaxLen)
    return set_error(JLD_ERR_UNSUPPORTED, "%s: each mesh size must be at most %d", who, kStaticMaxLen);
  const int h = nz / 2;
  const size_t need = (size_t)nx * ny * (h + 1) * sizeof(float2);
  if (need > kStaticScratchBytes)
    return set_error(JLD_ERR_WORKSPACE,
                     "%s: mesh (%d,%d,%d) needs %zu bytes of scratch, more than the fixed %zu bytes", who, nx,
                     ny, nz, need, kStaticScratchBytes);
  Plan3<float> pl;
  pl.nx = nx; pl.ny = ny; pl.nz = nz; pl.h = h;
  LinePlan<float>* lp[3] = {&pl.px, &pl.py, &pl.pz};
  const int lens[3] = {nx, ny, h};
  for (int a = 0; a < 3; ++a) {
    lp[a]->n = lens[a];
    if (!make_line_schedule(lens[a], &lp[a]->E, &lp[a]->nst, lp[a]->radix))
      return set_error(JLD_ERR_UNSUPPORTED, "%s: length %d does not factor into 2, 3 and 5", who, lens[a]);
    for (int s = lp[a]->nst; s < kMaxStages; ++s) lp[a]->radix[s] = 0;
  }
  StaticDev sd;
  int s = static_setup(&sd);
  if (s) return s;
  float2* tw = sd.tw;
  pl.px.tw = tw;
  pl.py.tw = tw + nx;
  pl.pz.tw = tw + nx + ny;
  pl.twr = tw + nx + ny + h;
  const int tl[4] = {nx, ny, h, nz}, tc[4] = {nx, ny, h, h + 1};
  size_t off = 0;
  for (int i = 0; i < 4; ++i) {
    static_twiddles_kernel<<<(tc[i] + 255) / 256, 256, 0, st>>>(tw + off, tl[i], tc[i]);
    off += tc[i];
  }
  JLD_LAUNCH_CHECK("static_twiddles_kernel");
  float2* main = (float2*)sd.scratch;
  float2* nyq = main + (size_t)nx * ny * h;
  if ((s = launch_rfft_z<float>(st, pl, data, nullptr, main, nyq))) return s;
  if ((s = launch_y_pass<float>(st, pl, main, nyq, -1))) return s;
  LineJob<float> jm = job_x_internal<float>(pl, main, false);
  LineJob<float> jn = job_x_internal<float>(pl, nyq, true);
  set_job_out_ref<float>(jm, pl, false, out_c, nullptr, nullptr);
  set_job_out_ref<float>(jn, pl, true, out_c, nullptr, nullptr);
  return launch_line_pass<float>(st, pl.px, jm, jn, -1);
}

}  // namespace jld

using namespace jld;
#define ST(s) reinterpret_cast<cudaStream_t>(s)

extern "C" {

int jld_buildplan_f32(int32_t nx, int32_t ny, int32_t nz, int32_t local_out[2]) {
  clear_error();
  Plan3<float> pl;
  int s = get_plan3<float>(nx, ny, nz, true, &pl);
  if (s) return s;
  if (local_out) { local_out[0] = nx; local_out[1] = 0; }
  return JLD_OK;
}
int jld_buildplan_f64(int32_t nx, int32_t ny, int32_t nz, int32_t local_out[2]) {
  clear_error();
  Plan3<double> pl;
  int s = get_plan3<double>(nx, ny, nz, true, &pl);
  if (s) return s;
  if (local_out) { local_out[0] = nx; local_out[1] = 0; }
  return JLD_OK;
}
size_t jld_fft_workspace_f32(int32_t nx, int32_t ny, int32_t nz) {
  if (nx < 1 || ny < 1 || nz < 2) return 0;
  return (size_t)nx * ny * (nz / 2 + 1) * sizeof(float2);
}
size_t jld_fft_workspace_f64(int32_t nx, int32_t ny, int32_t nz) {
  if (nx < 1 || ny < 1 || nz < 2) return 0;
  return (size_t)nx * ny * (nz / 2 + 1) * sizeof(double2);
}

int jld_pfft_f32(jld_stream_t s, const float* data, int32_t nx, int32_t ny, int32_t nz,
                 float* re, float* im, void* ws, size_t wsb) {
  clear_error();
  return rfft3<float>(ST(s), data, nx, ny, nz, nullptr, re, im, ws, wsb, "jld_pfft_f32");
}
int jld_pfft_f64(jld_stream_t s, const double* data, int32_t nx, int32_t ny, int32_t nz,
                 double* re, double* im, void* ws, size_t wsb) {
  clear_error();
  return rfft3<double>(ST(s), data, nx, ny, nz, nullptr, re, im, ws, wsb, "jld_pfft_f64");
}
int jld_pfft_c_f32(jld_stream_t s, const float* data, int32_t nx, int32_t ny, int32_t nz,
                   void* out, void* ws, size_t wsb) {
  clear_error();
  return rfft3<float>(ST(s), data, nx, ny, nz, (float2*)out, nullptr, nullptr, ws, wsb,
                      "jld_pfft_c_f32");
}
int jld_pfft_c_f64(jld_stream_t s, const double* data, int32_t nx, int32_t ny, int32_t nz,
                   void* out, void* ws, size_t wsb) {
  clear_error();
  return rfft3<double>(ST(s), data, nx, ny, nz, (double2*)out, nullptr, nullptr, ws, wsb,
                       "jld_pfft_c_f64");
}
int jld_pifft_f32(jld_stream_t s, const float* re, const float* im, int32_t nx, int32_t ny,
                  int32_t nz, float* out, void* ws, size_t wsb) {
  clear_error();
  return irfft3<float>(ST(s), nullptr, re, im, nx, ny, nz, out, ws, wsb, "jld_pifft_f32");
}
int jld_pifft_f64(jld_stream_t s, const double* re, const double* im, int32_t nx, int32_t ny,
                  int32_t nz, double* out, void* ws, size_t wsb) {
  clear_error();
  return irfft3<double>(ST(s), nullptr, re, im, nx, ny, nz, out, ws, wsb, "jld_pifft_f64");
}
int jld_pifft_c_f32(jld_stream_t s, const void* in, int32_t nx, int32_t ny, int32_t nz,
                    float* out, void* ws, size_t wsb) {
  clear_error();
  return irfft3<float>(ST(s), (const float2*)in, nullptr, nullptr, nx, ny, nz, out, ws, wsb,
                       "jld_pifft_c_f32");
}
int jld_pifft_c_f64(jld_stream_t s, const void* in, int32_t nx, int32_t ny, int32_t nz,
                    double* out, void* ws, size_t wsb) {
  clear_error();
  return irfft3<double>(ST(s), (const double2*)in, nullptr, nullptr, nx, ny, nz, out, ws, wsb,
                        "jld_pifft_c_f64");
}

int jld_pfft_c_static_f32(jld_stream_t s, const float* data, int32_t nx, int32_t ny, int32_t nz,
                          void* out) {
  clear_error();
  return pfft_static_impl(ST(s), data, nx, ny, nz, (float2*)out);
}

JLD_API int jld_wait_selftest(jld_stream_t s, int32_t polls, int32_t* word) {
  clear_error();
  return wait_selftest(ST(s), polls, (int*)word);
}

JLD_API int jld_fft_pipe_status(int32_t* value, int32_t reset) {
  clear_error();
  if (!value) return set_error(JLD_ERR_ARG, "jld_fft_pipe_status: NULL argument");
  int* p = nullptr;
  int s = fft_err_word(&p);
  if (s) return s;
  JLD_CUDA_TRY(cudaDeviceSynchronize());
  JLD_CUDA_TRY(cudaMemcpy(value, p, sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (reset) JLD_CUDA_TRY(cudaMemset(p, 0, sizeof(int32_t)));
  return JLD_OK;
}

}  // extern "C"
