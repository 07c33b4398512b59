// Host orchestration and C ABI of the fused LDL forward + adjoint step
// (kernels in ldl_kernels.cuh).  One call runs the whole step on one stream:
// ~9 launches per layer forward, ~9 per layer adjoint and 6 for the final
// map, all stream-ordered and free of host synchronisation, so the step can
// be captured into a CUDA graph once plans and tables exist
// (jld_ldl_prepare_f32).

#include <algorithm>

#include "bins.cuh"
#include "ldl_kernels.cuh"
#include "ldl_pipe.cuh"
#include "nvtx.cuh"
#include "hi_kernels.cuh"
#include "pipe_host.cuh"
#include "zpipe.cuh"

namespace jld {

struct LdlLayout {
  int64_t N, C, H;
  int nstep;
  size_t off_pos, off_xb, off_xb2, off_rho, off_S, off_g4, off_w[5], off_gb4, off_rb, off_part,
      off_npix, off_err, off_tick, off_xs0, off_keys, off_perm, off_tiles, off_g4x, off_s2, off_smu, off_dep,
      off_ctd, total;
  int nticks, nptick;
  TileGeom tg;
  int64_t part_doubles;
};

static size_t al(size_t v) { return (v + 255) & ~(size_t)255; }
static constexpr int kMaxCellBlocks = 8192;
// Option bits of the fused step (jld_ldl_step_f32).
constexpr int kOptWarpPaint = 1;   // warp-aggregated paint atomics
constexpr int kOptGeneric = 2;     // generic (non-pipelined) FFT passes
constexpr int kOptBinned = 4;      // per-step binning, tile-privatized scatters
constexpr int kOptRecompute = 8;   // one force-mesh slot, recomputed in the adjoint
// Schedule choices (same results, different speed; the batch autotuner
// picks them per box shape):
constexpr int kOptXRadix16 = 16;   // x passes on radix-16 schedules where radix-8 ones fit
constexpr int kOptColsShift = 5;   // 2 bits: narrowest pipelined tile, 0 auto, 1/2/3 = 4/8/16 columns
// 2 bits: binning tile edge, 0/1/2 = 16/8/20 cells (the adjoint's three
// float windows of (t + 3)^3 cells must fit in shared memory: 146 KB at 20)
constexpr int kOptBinShift = 7;
constexpr int kOptAll = 511;

static int opt_min_cols(int options) {
  const int c = (options >> kOptColsShift) & 3;
  return c ? 2 << c : 0;
}
static int opt_tile_cells(int options) {
  const int c = (options >> kOptBinShift) & 3;
  return c == 1 ? 8 : c == 2 ? 20 : 16;
}

// Force-mesh slots: the adjoint reads layer l's force mesh for l >= 1 only
// (the first layer's input positions need no cotangent), so nstep - 1 slots
// hold every mesh it needs; with kOptRecompute one slot, and the adjoint
// recomputes layers 1 .. nstep-2 from their stored density.
static int g4_slots(int nstep, int options) {
  return (options & kOptRecompute) ? 1 : std::max(1, nstep - 1);
}

// Workspace layout.  Everything up to the error word is independent of the
// options, then the binning buffers (kOptBinned), then the extra force-mesh
// slots.
static LdlLayout ldl_layout(int nx, int ny, int nz, int64_t N, int nstep, int options, bool hi = false) {
  LdlLayout L;
  const int64_t h = nz / 2;
  L.N = N; L.nstep = nstep;
  L.C = (int64_t)nx * ny * nz;
  L.H = (int64_t)nx * ny * (h + 1);
  L.part_doubles = std::max<int64_t>({4 * ((int64_t)ny * (h + 1) + ny), (int64_t)nx * ny + 64,
                                      4 * (int64_t)kMaxCellBlocks});
  size_t o = 0;
  L.off_pos = o; o += al(sizeof(float) * 3 * N * nstep);       // X_1 .. X_nstep
  L.off_xb = o; o += al(sizeof(float) * 3 * N);                // cotangent of X (ping)
  L.off_xb2 = o; o += al(sizeof(float) * 3 * N);               // (pong)
  L.off_rho = o; o += al(sizeof(float) * L.C * (nstep + 1));   // unit-mass paint per layer + final
  L.off_S = o; o += al(sizeof(float2) * L.H * nstep);          // FFT of the source per layer
  L.off_g4 = o; o += al(sizeof(float4) * L.C);                 // force mesh, slot 0
  for (int i = 0; i < 5; ++i) { L.off_w[i] = o; o += al(sizeof(float2) * L.H); }
  L.off_gb4 = o; o += al(sizeof(float4) * L.C);                // 3-channel cotangent mesh
  L.off_rb = o; o += al(sizeof(float) * L.C);                  // density cotangent
  L.off_part = o; o += al(sizeof(double) * L.part_doubles);    // per-block FP64 partials
  L.off_npix = o; o += al(sizeof(double) * 2);                 // 1 / Npixel
  L.off_err = o; o += al(sizeof(int) * 4);                     // pipelined-pass error word
  // tile counters of the pipelined passes (next_tile), one per launch, then
  // the particle kernels' batch counters (WarpBatches), kTicksPerLaunch per
  // launch
  L.nticks = 64 + 24 * nstep;
  L.nptick = 3 * nstep + 2;
  L.off_tick = o; o += al(sizeof(int) * (L.nticks + (size_t)L.nptick * kTicksPerLaunch));
  // particle binning: tile-ordered X_0, tile keys, order, tile counts/starts/fill
  L.tg = make_tile_geom(nx, ny, nz, opt_tile_cells(options), 1);
  L.off_xs0 = L.off_keys = L.off_perm = L.off_tiles = 0;
  if (options & kOptBinned) {
    L.off_xs0 = o; o += al(sizeof(float) * 3 * N);
    L.off_keys = o; o += al(sizeof(int) * N);
    L.off_perm = o; o += al(sizeof(int) * N);
    L.off_tiles = o; o += al(sizeof(int) * (3 * (size_t)L.tg.ntiles() + 1));
  }
  L.off_g4x = o; o += al(sizeof(float4) * L.C * (g4_slots(nstep, options) - 1));  // slots 1 ..
  // HI kind: star-map spectrum per layer, pfft(star map), dep1, its cotangent
  L.off_s2 = L.off_smu = L.off_dep = L.off_ctd = 0;
  if (hi) {
    L.off_s2 = o; o += al(sizeof(float2) * L.H * nstep);
    L.off_smu = o; o += al(sizeof(float2) * L.H);
    L.off_dep = o; o += al(sizeof(float) * L.C);
    L.off_ctd = o; o += al(sizeof(float) * L.C);
  }
  L.total = o;
  return L;
}

struct StepArgs {
  cudaStream_t st;
  const float* pos0; int64_t N;
  int nx, ny, nz; float box[3];
  int nstep, kind, L1, mode, paint_method;
  bool use_pipe;         // TMA-pipelined strided passes where the mesh qualifies
  bool binned;           // particles binned into tiles; tile-privatized scatters
  int options;           // option bits (layout)
  const float* params;   // device: npot*nstep (+3 for kind 0, +12 for kind 2)
  int npot;              // parameters per layer: 5, or 10 for the HI kind
  const float* starmap;  // HI kind: the star map (C floats), else nullptr
  const float* target; const float* mask;
  float n, index;        // loss smoothing exponent (0: none), map exponent (1: none)
  const float* field2;   // map factor or nullptr
  const float* maskvalid;  // validation mask or nullptr
  bool lossv_slot;       // out holds the validation loss after the gradient
  char* ws;
  double* out;           // device: [loss, grads... (, validation loss)]
};

struct SpecGeom {
  SpecPass sp;
  int64_t tiles;
  int nthr;
  size_t smem1;  // one tile
};

static SpecGeom spec_geom(const LinePlan<float>& lp, int nx, int ny, int h, int ax, int ntiles_smem) {
  SpecGeom g;
  g.sp.nx = nx; g.sp.ny = ny; g.sp.h = h;
  int cols = tile_cols(lp.n, lp.E, sizeof(float2));
  while (cols > 1 && (size_t)lp.n * (cols + 1) * sizeof(float2) * ntiles_smem > 200 * 1024) cols >>= 1;
  g.sp.cols = cols;
  g.sp.cshift = ilog2i(cols);
  const int64_t main_cols = ax == 0 ? (int64_t)ny * h : (int64_t)nx * h;
  const int64_t nyq_cols = ax == 0 ? ny : nx;
  g.sp.tiles_main = (main_cols + cols - 1) / cols;
  g.tiles = g.sp.tiles_main + (nyq_cols + cols - 1) / cols;
  g.nthr = cols * lp.n / lp.E;
  g.smem1 = (size_t)lp.n * (cols + 1) * sizeof(float2);
  return g;
}

// Sums per-block partial slots into out[out_off + j], j < nvals.
static void launch_finish(cudaStream_t st, const double* part, int nblocks, int stride, int nvals,
                          double* out, int out_off, const double* scale) {
  finish_kernel<<<nvals, 256, 0, st>>>(part, nblocks, stride, nvals, out, out_off, scale, 0);
}

static int ldl_step(const StepArgs& a) {
  const ScopedRange step_range("jld_ldl_step");
  const int nx = a.nx, ny = a.ny, nz = a.nz, h = nz / 2;
  const bool hi = a.kind == 2;
  const LdlLayout L = ldl_layout(nx, ny, nz, a.N, a.nstep, a.options, hi);
  const bool recompute = (a.options & kOptRecompute) != 0;
  const int npot = a.npot;
  cudaStream_t st = a.st;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  JLD_CUDA_TRY(cudaStreamIsCapturing(st, &cs));
  const bool may_build = cs == cudaStreamCaptureStatusNone;
  Plan3<float> pl;
  int s = get_plan3<float>(nx, ny, nz, may_build, &pl);
  if (s) return s;
  KTables kt;
  if ((s = get_ktables(nx, ny, nz, a.box, may_build, &kt))) return s;
  const Grid3 g = make_grid(nx, ny, nz);
  BoxGeom bg;
  const int nm[3] = {nx, ny, nz};
  for (int i = 0; i < 3; ++i) {
    bg.box[i] = a.box[i];
    bg.cell[i] = a.box[i] / (float)nm[i];
    bg.dw[i] = (float)nm[i] / a.box[i];
  }
  const float fact = (float)((double)L.C / (double)a.N);
  const float scale = (float)(1.0 / (double)L.C);
  char* ws = a.ws;
  float* Xs = (float*)(ws + L.off_pos);
  float* Xb = (float*)(ws + L.off_xb);
  float* Xb2 = (float*)(ws + L.off_xb2);
  float* rho = (float*)(ws + L.off_rho);
  float2* Sbuf = (float2*)(ws + L.off_S);
  float4* g4 = (float4*)(ws + L.off_g4);
  float4* g4x = (float4*)(ws + L.off_g4x);
  // force-mesh slot of layer l (g4_slots)
  auto g4_of = [&](int l) -> float4* {
    const int sl = (recompute || l == 0) ? 0 : l - 1;
    return sl == 0 ? g4 : g4x + (size_t)L.C * (sl - 1);
  };
  float2* W[5];
  for (int i = 0; i < 5; ++i) W[i] = (float2*)(ws + L.off_w[i]);
  float4* gb4 = (float4*)(ws + L.off_gb4);
  float* rb = (float*)(ws + L.off_rb);
  double* part = (double*)(ws + L.off_part);
  double* npix = (double*)(ws + L.off_npix);
  const int64_t nyq_off = (int64_t)nx * ny * h;
  const int pblock = 256;
  float* Xs0 = (float*)(ws + L.off_xs0);
  const float* X0 = a.binned ? Xs0 : a.pos0;
  auto Xl = [&](int l) -> const float* { return l == 0 ? X0 : Xs + (size_t)3 * a.N * (l - 1); };
  const TileGeom& tg = L.tg;
  int* tcounts = (int*)(ws + L.off_tiles);
  int* tstarts = tcounts + tg.ntiles();
  int* tfill = tstarts + tg.ntiles() + 1;
  const float3 boxv = make_float3(bg.box[0], bg.box[1], bg.box[2]);
  const float3 cellv = make_float3(bg.cell[0], bg.cell[1], bg.cell[2]);
  const float3 dwv = make_float3(bg.dw[0], bg.dw[1], bg.dw[2]);
  const size_t win1 = sizeof(float) * tg.wcells(), win3 = 3 * win1;
  const unsigned tgrid = (unsigned)std::min<int64_t>(tg.ntiles(), (int64_t)sm_count() * 8);
  // zeroed work counters, one set per persistent launch: a tile counter per
  // pipelined pass (next_tile), kTicksPerLaunch batch counters per particle
  // kernel (WarpBatches); nullptr past the last set (static order)
  int* ticks = (int*)(ws + L.off_tick);
  JLD_CUDA_TRY(cudaMemsetAsync(ticks, 0, sizeof(int) * (L.nticks + (size_t)L.nptick * kTicksPerLaunch), st));
  int nticks_used = 0, npticks_used = 0;
  auto tick = [&]() -> int* { return nticks_used < L.nticks ? ticks + nticks_used++ : nullptr; };
  auto ptick = [&]() -> int* {
    return npticks_used < L.nptick ? ticks + L.nticks + (size_t)kTicksPerLaunch * npticks_used++ : nullptr;
  };
  // Unit-mass paint of layer positions X into out (zeroed here).
  auto paint_into = [&](const float* X, float* out) -> int {
    if (!a.binned) return paint_unit_f32(st, X, a.N, nx, ny, nz, a.box, a.paint_method, out, ptick());
    JLD_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(float) * L.C, st));
    int e = ensure_smem(tiled_paint_kernel, win1);
    if (e) return e;
    tiled_paint_kernel<<<tgrid, 256, win1, st>>>(X, tstarts, tg, boxv, cellv, g, out);
    JLD_LAUNCH_CHECK("tiled_paint_kernel");
    return JLD_OK;
  };
  // Bin X_0 into tiles (counting sort); every layer then runs in tile order.
  if (a.binned) {
    JLD_CUDA_TRY(cudaMemsetAsync(tcounts, 0, sizeof(int) * tg.ntiles(), st));
    int* keys = (int*)(ws + L.off_keys);
    int* perm = (int*)(ws + L.off_perm);
    bin_count_kernel<<<resident_grid(bin_count_kernel, a.N, pblock), pblock, 0, st>>>(a.pos0, a.N, boxv, cellv, g, tg, keys, tcounts);
    JLD_LAUNCH_CHECK("bin_count_kernel");
    bin_scan_kernel<<<1, 1024, 0, st>>>(tcounts, tg.ntiles(), tstarts, tfill);
    JLD_LAUNCH_CHECK("bin_scan_kernel");
    bin_scatter_kernel<<<resident_grid(bin_scatter_kernel, a.N, pblock), pblock, 0, st>>>(a.pos0, a.N, keys, tfill, Xs0, perm);
    JLD_LAUNCH_CHECK("bin_scatter_kernel");
  }
  const int cblock = 256;
  const unsigned cgrid = (unsigned)std::min<int64_t>(kMaxCellBlocks, grid_for(L.C, cblock));
  const int64_t rows = (int64_t)nx * ny;

  const SpecGeom gx = spec_geom(pl.px, nx, ny, h, 0, 2);
  const SpecGeom gy = spec_geom(pl.py, nx, ny, h, 1, 2);
  int zcols = tile_cols(pl.pz.n, pl.pz.E, sizeof(float2));
  while (zcols > 1 && (size_t)pl.pz.n * (zcols + 1) * sizeof(float2) * 3 > 200 * 1024) zcols >>= 1;
  const int nthr_z = zcols * pl.pz.n / pl.pz.E;
  const unsigned zgrid = (unsigned)((rows + zcols - 1) / zcols);
  const size_t smz = (size_t)pl.pz.n * (zcols + 1) * sizeof(float2);
  if (gx.tiles * 4 > L.part_doubles || (int64_t)zgrid > L.part_doubles)
    return set_error(JLD_ERR_UNSUPPORTED, "mesh too large for the reduction buffer");

  // 1 / Npixel in FP64 (model.py:386-390), then 1 / Npixel of the
  // validation mask (model.py:458-463)
  for (int v = 0; v < 2; ++v) {
    const float* m = v ? a.maskvalid : a.mask;
    if (m) {
      mask_count_kernel<<<cgrid, cblock, 0, st>>>(m, L.C, part);
      JLD_LAUNCH_CHECK("mask_count_kernel");
      finish_kernel<<<1, 256, 0, st>>>(part, (int)cgrid, 1, 1, npix, v, nullptr, 1);
      JLD_LAUNCH_CHECK("finish_kernel");
    } else if (v == 0) {
      set_scalar_kernel<<<1, 1, 0, st>>>(npix, 1.0 / (double)L.C);
      JLD_LAUNCH_CHECK("set_scalar_kernel");
    }
  }

  // ---------------- pipelined (TMA-staged) strided passes, when the mesh qualifies
  int* err = (int*)(ws + L.off_err);
  JLD_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int) * 4, st));
  const int mc = opt_min_cols(a.options);
  const PipeGeom py0 = pipe_geom(nx, ny, h, 1, 0, 16, 128, mc), py1 = pipe_geom(nx, ny, h, 1, 1, 16, 128, mc);
  const PipeGeom px16 = pipe_geom(nx, ny, h, 0, 1, 16, 128, mc);
  // x passes: radix-8 schedules at <= 64 registers (twice the warps per SM)
  // where the tile fits, else the radix-16 ones
  const PipeGeom px8 = (a.options & kOptXRadix16) ? PipeGeom() : pipe_geom(nx, ny, h, 0, 1, 8, 64, mc);
  const PipeGeom& px1 = px8.ok ? px8 : px16;
  auto with_x = [&](auto&& body) { return px8.ok ? with_p2_8(nx, body) : with_p2(nx, body); };
  const bool pipe = a.use_pipe && py0.ok && py1.ok && px1.ok;
  ZPipeGeom zr2c, zc2r3, zadj, zr2c3;
  if (a.use_pipe) {
    zr2c = zpipe_geom(rows, h, 1, (size_t)h * 8, 110 * 1024, kZr2cThreads);
    // ~100 registers per thread: 192 / 128-thread CTAs keep 3-5 resident per SM
    zc2r3 = zpipe_geom(rows, h, 3, (size_t)3 * (h + 1) * 8, 110 * 1024, kZc2r3Threads);
    zadj = zpipe_geom(rows, h, 1, (size_t)(h + 1) * 8, 110 * 1024, kZadjThreads);
    zr2c3 = zpipe_geom(rows, h, 3, (size_t)2 * h * 16, 110 * 1024, kZr2c3Threads);
  }
  // the generic kernels then only cover the nyq plane
  SpecPass gxn = gx.sp, gyn = gy.sp;
  gxn.tiles_main = 0;
  gyn.tiles_main = 0;
  const unsigned gxn_tiles = (unsigned)((ny + gx.sp.cols - 1) / gx.sp.cols);
  const unsigned gyn_tiles = (unsigned)((nx + gy.sp.cols - 1) / gy.sp.cols);
  auto ymap = [&](CUtensorMap* m, const float2* B, const PipeGeom& p) {
    return make_main_map(m, B, nx, ny, h, 1, p.g.cols, ny);
  };
  auto xmap = [&](CUtensorMap* m, const float2* B, const PipeGeom& p) {
    return make_main_map(m, B, nx, ny, h, 0, p.g.cols, nx);
  };
  // y FFT in place on buffer B (main + nyq).
  auto ypass = [&](float2* B, int sgn) -> int {
    if (!pipe) return launch_y_pass<float>(st, pl, B, B + nyq_off, sgn);
    CUtensorMap m;
    int e = ymap(&m, B, py0);
    if (e) return e;
    e = with_p2(ny, [&](auto sch) {
      using Sch = decltype(sch);
      auto kern = sgn < 0 ? spass_kernel<Sch, 1, -1> : spass_kernel<Sch, 1, 1>;
      int r = ensure_smem(kern, py0.smem);
      if (r) return r;
      kern<<<py0.grid, py0.nthr, py0.smem, st>>>(m, B, py0.g, pl.py.tw, err, tick());
      return 0;
    });
    if (e) return e;
    JLD_LAUNCH_CHECK("spass_kernel");
    LineJob<float> jn, none;
    float2* nq = B + nyq_off;
    jn.src = nq; jn.dst = nq;
    jn.es_in = jn.es_out = 1;
    jn.cdiv_in = jn.cdiv_out = 1;
    jn.cmul_in = jn.cmul_out = ny;
    jn.ncol = nx;
    return launch_line_pass<float>(st, pl.py, jn, none, sgn);
  };

  // x FFT in place on buffer B (main + nyq), for the HI kind's star-map
  // spectrum and its cotangent.
  const PipeGeom pxs = pipe_geom(nx, ny, h, 0, 0, 16, 128, mc);
  auto xpass = [&](float2* B, int sgn) -> int {
    LineJob<float> jm = job_x_internal<float>(pl, B, false), jn = job_x_internal<float>(pl, B + nyq_off, true),
                   none;
    if (!(pipe && pxs.ok)) return launch_line_pass<float>(st, pl.px, jm, jn, sgn);
    CUtensorMap m;
    int e = xmap(&m, B, pxs);
    if (e) return e;
    e = with_p2(nx, [&](auto sch) {
      using Sch = decltype(sch);
      auto kern = sgn < 0 ? spass_kernel<Sch, 0, -1> : spass_kernel<Sch, 0, 1>;
      int r = ensure_smem(kern, pxs.smem);
      if (r) return r;
      kern<<<pxs.grid, pxs.nthr, pxs.smem, st>>>(m, B, pxs.g, pl.px.tw, err, tick());
      return 0;
    });
    if (e) return e;
    JLD_LAUNCH_CHECK("spass_kernel");
    return launch_line_pass<float>(st, pl.px, jn, none, sgn);
  };
  auto al16p = [](const void* q) { return ((uintptr_t)q & 15u) == 0; };

  // HI kind, layer l: S2 = FFT(sm^g2) in the internal layout (model.py:228).
  auto star_spectrum = [&](int l, float2* S2) -> int {
    const StarPow sp{a.params + npot * l};
    int s2 = JLD_OK;
    if (zr2c.ok && al16p(a.starmap)) {
      s2 = with_p2(h, [&](auto sch) {
        using Sch = decltype(sch);
        auto kern = zr2c_pipe_kernel<Sch, StarPow>;
        unsigned gz = 0;
        int r = ensure_smem(kern, zr2c.smem);
        if (!r) r = persistent_grid(kern, zr2c.nthr, zr2c.smem, zr2c.zt.ntiles, &gz);
        if (r) return r;
        kern<<<gz, zr2c.nthr, zr2c.smem, st>>>(a.starmap, sp, zr2c.zt, pl.twr, S2, pl.pz.tw, err, tick());
        return 0;
      });
      if (s2) return s2;
      JLD_LAUNCH_CHECK("zr2c_pipe_kernel");
    } else if ((s2 = launch_rfft_z_src<float, StarPow>(st, pl, a.starmap, sp, S2, S2 + nyq_off))) {
      return s2;
    }
    if ((s2 = ypass(S2, -1))) return s2;
    return xpass(S2, -1);
  };

  // HI kind, adjoint of layer l's star-map term from W (the cotangent
  // spectrum of the potential): d a2, d kh2, d kl2, d nu2, then V2 =
  // 1e-3 a2 G2 W / Nc back to real space (W[4]) and d g2.
  const ZPipeGeom zc2r1 = a.use_pipe ? zpipe_geom(rows, h, 1, (size_t)(h + 1) * 8) : ZPipeGeom();
  auto star_adjoint = [&](int l, const float* prm, float2* Wc, const float2* S2) -> int {
    const unsigned g5 = (unsigned)std::min<int64_t>(
        std::min<int64_t>(kMaxCellBlocks, L.part_doubles / 4), resident_grid(hi_src2_kernel, L.H, cblock));
    hi_src2_kernel<<<g5, cblock, 0, st>>>(Wc, S2, nx, ny, nz, kt, prm, a.mode, scale, part);
    JLD_LAUNCH_CHECK("hi_src2_kernel");
    launch_finish(st, part, (int)g5, 4, 1, a.out, 1 + npot * l + 5, nullptr);
    launch_finish(st, part + 1, (int)g5, 4, 3, a.out, 1 + npot * l + 7, nullptr);
    int s2 = xpass(Wc, +1);
    if (!s2) s2 = ypass(Wc, +1);
    if (s2) return s2;
    float* cts = (float*)W[4];
    if (zc2r1.ok) {
      s2 = with_p2(h, [&](auto sch) {
        using Sch = decltype(sch);
        auto kern = zc2r_pipe_kernel<Sch>;
        unsigned gz = 0;
        int r = ensure_smem(kern, zc2r1.smem);
        if (!r) r = persistent_grid(kern, zc2r1.nthr, zc2r1.smem, zc2r1.zt.ntiles, &gz);
        if (r) return r;
        kern<<<gz, zc2r1.nthr, zc2r1.smem, st>>>(Wc, zc2r1.zt, pl.twr, cts, pl.pz.tw, err, tick());
        return 0;
      });
      if (s2) return s2;
      JLD_LAUNCH_CHECK("zc2r_pipe_kernel");
    } else if ((s2 = launch_irfft_z<float>(st, pl, Wc, Wc + nyq_off, cts))) {
      return s2;
    }
    const unsigned g6 = (unsigned)std::min<int64_t>(kMaxCellBlocks, resident_grid(star_reduce_kernel, L.C, cblock));
    star_reduce_kernel<<<g6, cblock, 0, st>>>(cts, a.starmap, prm, L.C, part);
    JLD_LAUNCH_CHECK("star_reduce_kernel");
    launch_finish(st, part, (int)g6, 1, 1, a.out, 1 + npot * l + 6, nullptr);
    return JLD_OK;
  };

  // Force mesh of layer l from its stored unit-mass density: source map and
  // r2c along z, y FFT, x FFT (S_l) with the filter and gradient factors,
  // inverse y of three channels, inverse z into the float4 mesh g4_l.
  auto force_mesh = [&](int l, float4* g4_l) -> int {
    int s = JLD_OK;
    const float* prm = a.params + npot * l;
    float* rho_l = rho + (size_t)L.C * l;
    float2* S_l = Sbuf + (size_t)L.H * l;
    SourcePow src{prm, fact};
    const float2* S2_l = hi ? (float2*)(ws + L.off_s2) + (size_t)L.H * l : nullptr;
    if (zr2c.ok) {
      s = with_p2(h, [&](auto sch) {
        using Sch = decltype(sch);
        auto kern = zr2c_pipe_kernel<Sch, SourcePow>;
        unsigned gz = 0;
        int r = ensure_smem(kern, zr2c.smem);
        if (!r) r = persistent_grid(kern, zr2c.nthr, zr2c.smem, zr2c.zt.ntiles, &gz);
        if (r) return r;
        kern<<<gz, zr2c.nthr, zr2c.smem, st>>>(rho_l, src, zr2c.zt, pl.twr, W[0], pl.pz.tw, err, tick());
        return 0;
      });
      if (s) return s;
      JLD_LAUNCH_CHECK("zr2c_pipe_kernel");
    } else if ((s = launch_rfft_z_src<float, SourcePow>(st, pl, rho_l, src, W[0], W[0] + nyq_off))) {
      return s;
    }
    if ((s = ypass(W[0], -1))) return s;
    if (pipe) {
      CUtensorMap mA;
      if ((s = xmap(&mA, W[0], px1))) return s;
      s = with_x([&](auto sch) {
        using Sch = decltype(sch);
        auto kern = hi ? xfilt_pipe_kernel<Sch, true> : xfilt_pipe_kernel<Sch, false>;
        int r = ensure_smem(kern, px1.smem);
        if (r) return r;
        kern<<<px1.grid, px1.nthr, px1.smem, st>>>(mA, px1.g, kt, prm, a.kind, scale, S_l, W[1],
                                                                    W[2], pl.px.tw, err, S2_l, tick());
        return 0;
      });
      if (s) return s;
      JLD_LAUNCH_CHECK("xfilt_pipe_kernel");
    }
    s = with_sched(pl.px, [&](auto sc) {
      constexpr int SC = decltype(sc)::value;
      int e = ensure_smem(xfilt_kernel<SC>, 2 * gx.smem1);
      if (e) return e;
      xfilt_kernel<SC><<<pipe ? gxn_tiles : (unsigned)gx.tiles, gx.nthr, 2 * gx.smem1, st>>>(
          pl.px, pipe ? gxn : gx.sp, kt, prm, a.kind, scale, W[0], S_l, W[1], W[2], S2_l);
      return 0;
    });
    if (s) return s;
    JLD_LAUNCH_CHECK("xfilt_kernel");
    if (pipe) {
      CUtensorMap m0, m1;
      if ((s = ymap(&m0, W[1], py0)) || (s = ymap(&m1, W[2], py0))) return s;
      s = with_p2(ny, [&](auto sch) {
        using Sch = decltype(sch);
        int r = ensure_smem(yinv3_pipe_kernel<Sch>, py0.smem);
        if (r) return r;
        yinv3_pipe_kernel<Sch><<<py0.grid, py0.nthr, py0.smem, st>>>(m0, m1, py0.g, kt, W[3], W[0], W[4],
                                                                    pl.py.tw, err, tick());
        return 0;
      });
      if (s) return s;
      JLD_LAUNCH_CHECK("yinv3_pipe_kernel");
    }
    s = with_sched(pl.py, [&](auto sc) {
      constexpr int SC = decltype(sc)::value;
      int e = ensure_smem(yinv3_kernel<SC>, gy.smem1);
      if (e) return e;
      yinv3_kernel<SC><<<pipe ? gyn_tiles : (unsigned)gy.tiles, gy.nthr, gy.smem1, st>>>(
          pl.py, pipe ? gyn : gy.sp, kt, W[1], W[2], W[3], W[0], W[4]);
      return 0;
    });
    if (s) return s;
    JLD_LAUNCH_CHECK("yinv3_kernel");
    if (zc2r3.ok) {
      s = with_p2(h, [&](auto sch) {
        using Sch = decltype(sch);
        auto kern = zc2r3_pipe_kernel<Sch>;
        unsigned gz = 0;
        int r = ensure_smem(kern, zc2r3.smem);
        if (!r) r = persistent_grid(kern, zc2r3.nthr, zc2r3.smem, zc2r3.zt.ntiles, &gz);
        if (r) return r;
        kern<<<gz, zc2r3.nthr, zc2r3.smem, st>>>(W[3], W[0], W[4], zc2r3.zt, pl.twr, g4_l, pl.pz.tw, err, tick());
        return 0;
      });
    } else {
      s = with_sched(pl.pz, [&](auto sc) {
        constexpr int SC = decltype(sc)::value;
        int e = ensure_smem(zinv3_kernel<SC>, 3 * smz);
        if (e) return e;
        zinv3_kernel<SC><<<zgrid, nthr_z, 3 * smz, st>>>(pl.pz, pl.twr, W[3], W[0], W[4], nyq_off, g4_l, rows,
                                                         zcols, ilog2i(zcols));
        return 0;
      });
    }
    if (s) return s;
    JLD_LAUNCH_CHECK("zinv3_kernel");
    return JLD_OK;
  };

  // Outside the binned path the adjoint of layer l folds in the paint
  // adjoint of layer l+1 (no separate gather kernels, no cotangent round
  // trip).  Folding the paint of X_{l+1} into the update kernel was measured
  // slower (4.46 ms against 2.0 + 2.15 ms at 512^3): the fused kernel holds
  // more registers and runs fewer warps for the same load latency.
  const bool fuse_adj = !a.binned;

  // ---------------- forward layers (density of layer l+1 painted after its update)
  if ((s = paint_into(Xl(0), rho))) return s;
  for (int l = 0; l < a.nstep; ++l) {
    const ScopedRange layer_range("jld forward layer %d", l);
    float4* g4_l = g4_of(l);
    if (hi && (s = star_spectrum(l, (float2*)(ws + L.off_s2) + (size_t)L.H * l))) return s;
    if ((s = force_mesh(l, g4_l))) return s;
    update_kernel<<<resident_grid(update_kernel, a.N, pblock), pblock, 0, st>>>(Xl(l), a.N, bg, g, g4_l,
                                                                              Xs + (size_t)3 * a.N * l, ptick());
    JLD_LAUNCH_CHECK("update_kernel");
    if ((s = paint_into(Xl(l + 1), rho + (size_t)L.C * (l + 1)))) return s;  // the final map for l = nstep-1
  }

  // ---------------- final map, loss and its cotangent
  float* rho_f = rho + (size_t)L.C * a.nstep;
  {
    const ScopedRange map_range("jld final map and loss");
    const LossFields lf{rho_f, a.target, a.mask, a.field2, a.maskvalid};
    const float* fprm = a.params + npot * a.nstep;
    const int nparam = npot * a.nstep + (a.kind == 0 ? 3 : (a.kind == 2 ? kHiFinalParams : 0));
    const int64_t max_blocks = std::min<int64_t>(kMaxCellBlocks, L.part_doubles / 5);
    // validation loss: reduced only with a validation mask, else 0
    double* lossv_out = a.lossv_slot ? a.out + 1 + nparam : nullptr;
    if (lossv_out && !a.maskvalid) JLD_CUDA_TRY(cudaMemsetAsync(lossv_out, 0, sizeof(double), st));
    if (hi) {
      // dep1 = c2r(r2c(sm) Fk) (model.py:329-331), the map and loss, then
      // d(khi, kli, nui, xi) from r2c(dL/d dep1)
      const size_t wbytes = al(sizeof(float2) * L.H);
      float2* smu = (float2*)(ws + L.off_smu);
      float* dep = (float*)(ws + L.off_dep);
      float* ctd = (float*)(ws + L.off_ctd);
      if ((s = jld_pfft_c_f32((jld_stream_t)st, a.starmap, nx, ny, nz, smu, W[1], wbytes))) return s;
      hi_dep_filter_kernel<<<resident_grid(hi_dep_filter_kernel, L.H, cblock), cblock, 0, st>>>(
          W[0], smu, nx, ny, nz, kt, fprm, scale);
      JLD_LAUNCH_CHECK("hi_dep_filter_kernel");
      if ((s = jld_pifft_c_f32((jld_stream_t)st, W[0], nx, ny, nz, dep, W[1], wbytes))) return s;
      const unsigned g7 = (unsigned)std::min<int64_t>(std::min<int64_t>(kMaxCellBlocks, L.part_doubles / 9),
                                                      resident_grid(hi_loss_kernel, L.C, cblock));
      hi_loss_kernel<<<g7, cblock, 0, st>>>(rho_f, a.starmap, dep, a.target, a.mask, L.C, fact, fprm, a.L1, npix,
                                            rb, ctd, part);
      JLD_LAUNCH_CHECK("hi_loss_kernel");
      const int o = 1 + npot * a.nstep;
      launch_finish(st, part, (int)g7, 9, 1, a.out, 0, npix);
      launch_finish(st, part + 1, (int)g7, 9, 3, a.out, o, nullptr);       // mu, w, b
      launch_finish(st, part + 4, (int)g7, 9, 1, a.out, o + 3, nullptr);   // beta1
      launch_finish(st, part + 5, (int)g7, 9, 2, a.out, o + 7, nullptr);   // beta2, gamma3
      launch_finish(st, part + 7, (int)g7, 9, 2, a.out, o + 10, nullptr);  // eta, zs
      if ((s = jld_pfft_c_f32((jld_stream_t)st, ctd, nx, ny, nz, W[0], W[1], wbytes))) return s;
      const unsigned g8 = (unsigned)std::min<int64_t>(std::min<int64_t>(kMaxCellBlocks, L.part_doubles / 4),
                                                      resident_grid(hi_filter_grad_kernel, L.H, cblock));
      hi_filter_grad_kernel<<<g8, cblock, 0, st>>>(W[0], smu, nx, ny, nz, kt, fprm, a.mode, scale, part);
      JLD_LAUNCH_CHECK("hi_filter_grad_kernel");
      launch_finish(st, part, (int)g8, 4, 3, a.out, o + 4, nullptr);      // khi, kli, nui
      launch_finish(st, part + 3, (int)g8, 4, 1, a.out, o + 9, nullptr);  // xi
    } else if (a.n > 0.f) {
      // diff -> c2r(r2c(diff) K) -> loss -> the same smoothing on its
      // cotangent (a real, even Fourier multiplier is its own adjoint)
      const size_t wbytes = al(sizeof(float2) * L.H);
      auto smooth = [&](float* f) -> int {
        int r = jld_pfft_c_f32((jld_stream_t)st, f, nx, ny, nz, W[0], W[1], wbytes);
        if (r) return r;
        smooth_spec_kernel<<<resident_grid(smooth_spec_kernel, L.H, cblock), cblock, 0, st>>>(
            W[0], nx, ny, h + 1, kt, a.n, scale);
        JLD_LAUNCH_CHECK("smooth_spec_kernel");
        return jld_pifft_c_f32((jld_stream_t)st, W[0], nx, ny, nz, f, W[1], wbytes);
      };
      const unsigned g1 = (unsigned)std::min<int64_t>(max_blocks, resident_grid(smooth_map_kernel, L.C, cblock));
      smooth_map_kernel<<<g1, cblock, 0, st>>>(lf, L.C, fact, fprm, a.kind, a.index, rb);
      JLD_LAUNCH_CHECK("smooth_map_kernel");
      if ((s = smooth(rb))) return s;
      const unsigned g2 = (unsigned)std::min<int64_t>(max_blocks, resident_grid(smooth_loss_kernel, L.C, cblock));
      smooth_loss_kernel<<<g2, cblock, 0, st>>>(lf, L.C, a.L1, npix, rb, part);
      JLD_LAUNCH_CHECK("smooth_loss_kernel");
      launch_finish(st, part, (int)g2, 2, 1, a.out, 0, npix);
      if (lossv_out && a.maskvalid) launch_finish(st, part + 1, (int)g2, 2, 1, a.out, 1 + nparam, npix + 1);
      if ((s = smooth(rb))) return s;
      const unsigned g3 = (unsigned)std::min<int64_t>(max_blocks, resident_grid(smooth_adj_kernel, L.C, cblock));
      smooth_adj_kernel<<<g3, cblock, 0, st>>>(lf, L.C, fact, fprm, a.kind, a.index, rb, part);
      JLD_LAUNCH_CHECK("smooth_adj_kernel");
      if (a.kind == 0) launch_finish(st, part, (int)g3, 3, 3, a.out, 1 + 5 * a.nstep, nullptr);
    } else {
      auto al16 = [](const void* q) { return ((uintptr_t)q & 15u) == 0; };
      const int vec4 = L.C % 4 == 0 && al16(rho_f) && al16(a.target) && al16(rb) && (!a.mask || al16(a.mask)) &&
                       (!a.field2 || al16(a.field2)) && (!a.maskvalid || al16(a.maskvalid));
      const unsigned lgrid = (unsigned)std::min<int64_t>(
          max_blocks, resident_grid(loss_kernel, vec4 ? L.C / 4 : L.C, cblock));
      loss_kernel<<<lgrid, cblock, 0, st>>>(lf, L.C, fact, fprm, a.kind, a.L1, a.index, npix, rb, part, vec4);
      JLD_LAUNCH_CHECK("loss_kernel");
      launch_finish(st, part, (int)lgrid, 5, 1, a.out, 0, npix);
      if (a.kind == 0) launch_finish(st, part + 1, (int)lgrid, 5, 3, a.out, 1 + 5 * a.nstep, nullptr);
      if (lossv_out && a.maskvalid) launch_finish(st, part + 4, (int)lgrid, 5, 1, a.out, 1 + nparam, npix + 1);
    }
  }
  if (!fuse_adj) {
    gather_vjp_kernel<<<resident_grid(gather_vjp_kernel, a.N, pblock), pblock, 0, st>>>(Xl(a.nstep), a.N, bg, g, rb, Xb, 0);
    JLD_LAUNCH_CHECK("gather_vjp_kernel");
  }

  // ---------------- adjoint layers
  for (int l = a.nstep - 1; l >= 0; --l) {
    const ScopedRange layer_range("jld adjoint layer %d", l);
    const float* prm = a.params + npot * l;
    float* rho_l = rho + (size_t)L.C * l;
    float2* S_l = Sbuf + (size_t)L.H * l;
    float2* S2_l = hi ? (float2*)(ws + L.off_s2) + (size_t)L.H * l : nullptr;
    float4* g4_l = g4_of(l);
    // the last layer's mesh is still in its slot; layer 0's is not read
    if (recompute && l > 0 && l < a.nstep - 1 && (s = force_mesh(l, g4_l))) return s;
    JLD_CUDA_TRY(cudaMemsetAsync(gb4, 0, sizeof(float4) * L.C, st));
    if (a.binned) {
      if ((s = ensure_smem(tiled_bwd_kernel<true>, win3)) || (s = ensure_smem(tiled_bwd_kernel<false>, win3)))
        return s;
      if (l > 0)
        tiled_bwd_kernel<true><<<tgrid, 256, win3, st>>>(Xl(l), Xb, tstarts, tg, boxv, cellv, dwv, g, g4_l, gb4,
                                                         Xb2);
      else
        tiled_bwd_kernel<false><<<tgrid, 256, win3, st>>>(Xl(l), Xb, tstarts, tg, boxv, cellv, dwv, g, g4_l, gb4,
                                                          Xb2);
      JLD_LAUNCH_CHECK("tiled_bwd_kernel");
    } else {
      // cotangent of X_{l+1}: the previous layer's output plus the paint
      // adjoint of rho_{l+1} (rb holds it: the loss's for the last layer);
      // the first layer's input positions are data: scatter only
      const float* Xbp = (l == a.nstep - 1) ? nullptr : Xb;
      if (l > 0)
        bwd_fused_kernel<true><<<resident_grid(bwd_fused_kernel<true>, a.N, pblock), pblock, 0, st>>>(
            Xl(l + 1), rb, Xbp, Xl(l), a.N, bg, g, g4_l, gb4, Xb2, ptick());
      else
        bwd_fused_kernel<false><<<resident_grid(bwd_fused_kernel<false>, a.N, pblock), pblock, 0, st>>>(
            Xl(l + 1), rb, Xbp, Xl(l), a.N, bg, g, g4_l, gb4, Xb2, ptick());
      JLD_LAUNCH_CHECK("bwd_fused_kernel");
    }
    if (zr2c3.ok) {
      s = with_p2(h, [&](auto sch) {
        using Sch = decltype(sch);
        auto kern = zr2c3_pipe_kernel<Sch>;
        unsigned gz = 0;
        int r = ensure_smem(kern, zr2c3.smem);
        if (!r) r = persistent_grid(kern, zr2c3.nthr, zr2c3.smem, zr2c3.zt.ntiles, &gz);
        if (r) return r;
        kern<<<gz, zr2c3.nthr, zr2c3.smem, st>>>(gb4, zr2c3.zt, pl.twr, kt.cz, W[0], W[1], W[2], pl.pz.tw, err, tick());
        return 0;
      });
    } else {
      s = with_sched(pl.pz, [&](auto sc) {
        constexpr int SC = decltype(sc)::value;
        int e = ensure_smem(zfwd3_kernel<SC>, 3 * smz);
        if (e) return e;
        zfwd3_kernel<SC><<<zgrid, nthr_z, 3 * smz, st>>>(pl.pz, pl.twr, kt.cz, gb4, W[0], W[1], W[2], nyq_off,
                                                         rows, zcols, ilog2i(zcols));
        return 0;
      });
    }
    if (s) return s;
    JLD_LAUNCH_CHECK("zfwd3_kernel");
    if (pipe) {
      CUtensorMap m0, m1, m2;
      if ((s = ymap(&m0, W[0], py1)) || (s = ymap(&m1, W[1], py1)) || (s = ymap(&m2, W[2], py1))) return s;
      s = with_p2(ny, [&](auto sch) {
        using Sch = decltype(sch);
        int r = ensure_smem(yfwd_comb_pipe_kernel<Sch>, py1.smem);
        if (r) return r;
        yfwd_comb_pipe_kernel<Sch><<<py1.grid, py1.nthr, py1.smem, st>>>(m0, m1, m2, py1.g, kt, W[0], W[3],
                                                                        pl.py.tw, err, tick());
        return 0;
      });
      if (s) return s;
      JLD_LAUNCH_CHECK("yfwd_comb_pipe_kernel");
    }
    s = with_sched(pl.py, [&](auto sc) {
      constexpr int SC = decltype(sc)::value;
      int e = ensure_smem(yfwd_comb_kernel<SC>, 2 * gy.smem1);
      if (e) return e;
      yfwd_comb_kernel<SC><<<pipe ? gyn_tiles : (unsigned)gy.tiles, gy.nthr, 2 * gy.smem1, st>>>(
          pl.py, pipe ? gyn : gy.sp, kt, W[0], W[1], W[2], W[3]);
      return 0;
    });
    if (s) return s;
    JLD_LAUNCH_CHECK("yfwd_comb_kernel");
    // x adjoint: partial sums of the pipelined kernel first, the nyq plane's after them
    int nparts_x = 0;
    if (pipe) {
      CUtensorMap m0, m1, m2;
      if ((s = xmap(&m0, W[0], px1)) || (s = xmap(&m1, W[3], px1)) || (s = xmap(&m2, S_l, px1))) return s;
      s = with_x([&](auto sch) {
        using Sch = decltype(sch);
        auto kern = hi ? xbwd_pipe_kernel<Sch, true> : xbwd_pipe_kernel<Sch, false>;
        int r = ensure_smem(kern, px1.smem);
        if (r) return r;
        kern<<<px1.grid, px1.nthr, px1.smem, st>>>(m0, m1, m2, px1.g, kt, prm, a.kind, a.mode,
                                                                   scale, W[1], part, pl.px.tw, err,
                                                                   hi ? W[2] : nullptr, tick());
        return 0;
      });
      if (s) return s;
      JLD_LAUNCH_CHECK("xbwd_pipe_kernel");
      nparts_x = px1.grid;
    }
    const unsigned xb_grid = pipe ? gxn_tiles : (unsigned)gx.tiles;
    s = with_sched(pl.px, [&](auto sc) {
      constexpr int SC = decltype(sc)::value;
      int e = ensure_smem(xbwd_kernel<SC>, 2 * gx.smem1);
      if (e) return e;
      xbwd_kernel<SC><<<xb_grid, gx.nthr, 2 * gx.smem1, st>>>(pl.px, pipe ? gxn : gx.sp, kt, prm, a.kind, a.mode,
                                                               scale, W[0], W[3], S_l, W[1],
                                                               part + (size_t)4 * nparts_x, hi ? W[2] : nullptr);
      return 0;
    });
    if (s) return s;
    JLD_LAUNCH_CHECK("xbwd_kernel");
    nparts_x += (int)xb_grid;
    // d alpha -> out[1+5l], d kh, d kl, d nu -> out[1+5l+2 .. 4]
    launch_finish(st, part, nparts_x, 4, 1, a.out, 1 + npot * l, nullptr);
    launch_finish(st, part + 1, nparts_x, 4, 3, a.out, 1 + npot * l + 2, nullptr);
    if (hi && (s = star_adjoint(l, prm, W[2], S2_l))) return s;
    if ((s = ypass(W[1], +1))) return s;
    unsigned adj_blocks = zgrid;
    if (zadj.ok) {
      s = with_p2(h, [&](auto sch) {
        using Sch = decltype(sch);
        auto kern = zc2r_adj_pipe_kernel<Sch>;
        int r = ensure_smem(kern, zadj.smem);
        if (!r) r = persistent_grid(kern, zadj.nthr, zadj.smem, zadj.zt.ntiles, &adj_blocks);
        if (r) return r;
        kern<<<adj_blocks, zadj.nthr, zadj.smem, st>>>(W[1], zadj.zt, pl.twr, rho_l, prm, fact,
                                                       l > 0 ? rb : nullptr, part, pl.pz.tw, err, tick());
        return 0;
      });
    } else {
      s = with_sched(pl.pz, [&](auto sc) {
        constexpr int SC = decltype(sc)::value;
        int e = ensure_smem(zinv_adj_kernel<SC>, smz);
        if (e) return e;
        zinv_adj_kernel<SC><<<zgrid, nthr_z, smz, st>>>(pl.pz, pl.twr, W[1], nyq_off, rho_l, prm, fact,
                                                        l > 0 ? rb : nullptr, part, rows, zcols, ilog2i(zcols));
        return 0;
      });
    }
    if (s) return s;
    JLD_LAUNCH_CHECK("zinv_adj_kernel");
    launch_finish(st, part, (int)adj_blocks, 1, 1, a.out, 1 + npot * l + 1, nullptr);
    if (l > 0 && !fuse_adj) {
      gather_vjp_kernel<<<resident_grid(gather_vjp_kernel, a.N, pblock), pblock, 0, st>>>(Xl(l), a.N, bg, g, rb, Xb2, 1);
      JLD_LAUNCH_CHECK("gather_vjp_kernel");
    }
    std::swap(Xb, Xb2);
  }
  return JLD_OK;
}

static int check_step_args(int nx, int ny, int nz, int64_t nparts, int nstep, const float* box,
                           const char* who) {
  if (nx < 1 || ny < 1 || nz < 2 || (nz & 1))
    return set_error(JLD_ERR_UNSUPPORTED, "%s: mesh (%d,%d,%d) unsupported (nz must be even)", who, nx, ny, nz);
  if (nparts < 1) return set_error(JLD_ERR_ARG, "%s: need at least one particle", who);
  if (nstep < 1 || nstep > 64) return set_error(JLD_ERR_ARG, "%s: nstep must be in 1..64", who);
  if (!box || !(box[0] > 0 && box[1] > 0 && box[2] > 0))
    return set_error(JLD_ERR_ARG, "%s: box sizes must be positive", who);
  if ((int64_t)nx * ny * nz > ((int64_t)1 << 31))
    return set_error(JLD_ERR_UNSUPPORTED, "%s: mesh too large", who);
  return JLD_OK;
}

}  // namespace jld

using namespace jld;

extern "C" {

JLD_API size_t jld_ldl_workspace_f32(int32_t nx, int32_t ny, int32_t nz, int64_t nparts, int32_t nstep) {
  if (nx < 1 || ny < 1 || nz < 2 || nparts < 1 || nstep < 1) return 0;
  return ldl_layout(nx, ny, nz, nparts, nstep, kOptBinned).total;
}

JLD_API size_t jld_ldl_workspace_opt_f32(int32_t nx, int32_t ny, int32_t nz, int64_t nparts, int32_t nstep,
                                         int32_t options) {
  if (nx < 1 || ny < 1 || nz < 2 || nparts < 1 || nstep < 1 || (options & ~kOptAll)) return 0;
  return ldl_layout(nx, ny, nz, nparts, nstep, options).total;
}

JLD_API int jld_ldl_prepare_f32(int32_t nx, int32_t ny, int32_t nz, const float box[3]) {
  clear_error();
  int s = check_step_args(nx, ny, nz, 1, 1, box, "jld_ldl_prepare_f32");
  if (s) return s;
  Plan3<float> pl;
  if ((s = get_plan3<float>(nx, ny, nz, true, &pl))) return s;
  KTables kt;
  return get_ktables(nx, ny, nz, box, true, &kt);
}

static int step_entry(jld_stream_t stream, const float* pos, int64_t nparts, int32_t nx, int32_t ny, int32_t nz,
                      const float box[3], int32_t nstep, int32_t kind, int32_t L1, int32_t grad_mode,
                      int32_t options, const float* params, const float* target, const float* mask,
                      const jld_ldl_loss_ext* ext, const float* starmap, void* ws, size_t ws_bytes, double* out,
                      const char* who) {
  int s = check_step_args(nx, ny, nz, nparts, nstep, box, who);
  if (s) return s;
  const bool hi = kind == 2;
  if (kind != 0 && kind != 1 && !hi) return set_error(JLD_ERR_ARG, "%s: kind must be 0 (sm) or 1 (dm)", who);
  if (hi && !starmap) return set_error(JLD_ERR_ARG, "%s: star map required", who);
  if (L1 != 0 && L1 != 1) return set_error(JLD_ERR_ARG, "%s: L1 must be 0 or 1", who);
  if (grad_mode != 0 && grad_mode != 1)
    return set_error(JLD_ERR_ARG, "%s: grad_mode must be 0 (reference) or 1 (true)", who);
  if ((options & ~kOptAll) || ((options >> kOptBinShift) & 3) == 3)
    return set_error(JLD_ERR_ARG, "%s: unknown option bits 0x%x", who, options);
  if ((options & kOptBinned) && nparts > INT32_MAX)
    return set_error(JLD_ERR_UNSUPPORTED, "%s: binning needs fewer than 2^31 particles", who);
  const int paint_method = (options & kOptWarpPaint) ? 1 : 0;
  if (!pos || !params || !target || !out) return set_error(JLD_ERR_ARG, "%s: NULL pointer", who);
  size_t need = ldl_layout(nx, ny, nz, nparts, nstep, options, hi).total;
  if (!ws || ws_bytes < need)
    return set_error(JLD_ERR_WORKSPACE, "%s: workspace of %zu bytes needed, got %zu", who, need,
                     ws ? ws_bytes : (size_t)0);
  // tensor and bulk copies from workspace buffers need 16-byte alignment;
  // the layout keeps every buffer at a multiple of 256 bytes from ws
  if ((uintptr_t)ws & 255u) return set_error(JLD_ERR_ARG, "%s: workspace must be 256-byte aligned", who);
  StepArgs a;
  a.st = reinterpret_cast<cudaStream_t>(stream);
  a.pos0 = pos; a.N = nparts;
  a.nx = nx; a.ny = ny; a.nz = nz;
  for (int i = 0; i < 3; ++i) a.box[i] = box[i];
  a.nstep = nstep; a.kind = kind; a.L1 = L1; a.mode = grad_mode; a.paint_method = paint_method;
  a.use_pipe = (options & kOptGeneric) == 0;
  a.binned = (options & kOptBinned) != 0;
  a.options = options;
  a.params = params; a.target = target; a.mask = mask;
  a.npot = hi ? kHiLayerParams : 5;
  a.starmap = hi ? starmap : nullptr;
  a.n = ext ? ext->n : 0.f;
  a.index = ext ? ext->index : 1.f;
  a.field2 = ext ? ext->field2 : nullptr;
  a.maskvalid = ext ? ext->maskvalid : nullptr;
  a.lossv_slot = ext != nullptr;
  if (!(a.n >= 0.f) || !std::isfinite(a.index))
    return set_error(JLD_ERR_ARG, "%s: n must be >= 0 and index finite", who);
  a.ws = (char*)ws; a.out = out;
  return ldl_step(a);
}

JLD_API int jld_ldl_step_f32(jld_stream_t stream, const float* pos, int64_t nparts, int32_t nx, int32_t ny,
                             int32_t nz, const float box[3], int32_t nstep, int32_t kind, int32_t L1,
                             int32_t grad_mode, int32_t options, const float* params,
                             const float* target, const float* mask, void* ws, size_t ws_bytes,
                             double* out) {
  clear_error();
  return step_entry(stream, pos, nparts, nx, ny, nz, box, nstep, kind, L1, grad_mode, options, params, target,
                    mask, nullptr, nullptr, ws, ws_bytes, out, "jld_ldl_step_f32");
}

JLD_API int jld_ldl_step_ext_f32(jld_stream_t stream, const float* pos, int64_t nparts, int32_t nx, int32_t ny,
                                 int32_t nz, const float box[3], int32_t nstep, int32_t kind, int32_t L1,
                                 int32_t grad_mode, int32_t options, const float* params,
                                 const float* target, const float* mask, const jld_ldl_loss_ext* ext, void* ws,
                                 size_t ws_bytes, double* out) {
  clear_error();
  const char* who = "jld_ldl_step_ext_f32";
  if (!ext) return set_error(JLD_ERR_ARG, "%s: ext is NULL", who);
  return step_entry(stream, pos, nparts, nx, ny, nz, box, nstep, kind, L1, grad_mode, options, params, target,
                    mask, ext, nullptr, ws, ws_bytes, out, who);
}

JLD_API size_t jld_ldl_workspace_hi_f32(int32_t nx, int32_t ny, int32_t nz, int64_t nparts, int32_t nstep,
                                        int32_t options) {
  if (nx < 1 || ny < 1 || nz < 2 || nparts < 1 || nstep < 1 || (options & ~kOptAll)) return 0;
  return ldl_layout(nx, ny, nz, nparts, nstep, options, true).total;
}

JLD_API int jld_ldl_step_hi_f32(jld_stream_t stream, const float* pos, int64_t nparts, int32_t nx, int32_t ny,
                                int32_t nz, const float box[3], int32_t nstep, int32_t L1, int32_t grad_mode,
                                int32_t options, const float* params, const float* target, const float* mask,
                                const float* starmap, void* ws, size_t ws_bytes, double* out) {
  clear_error();
  return step_entry(stream, pos, nparts, nx, ny, nz, box, nstep, 2, L1, grad_mode, options, params, target, mask,
                    nullptr, starmap, ws, ws_bytes, out, "jld_ldl_step_hi_f32");
}

JLD_API int jld_ldl_error_word_f32(const void* ws, int32_t nx, int32_t ny, int32_t nz, int64_t nparts,
                                   int32_t nstep, const int** out) {
  clear_error();
  if (!ws || !out || nstep < 1 || nparts < 1) return set_error(JLD_ERR_ARG, "jld_ldl_error_word_f32: bad arguments");
  LdlLayout L = ldl_layout(nx, ny, nz, nparts, nstep, 0);  // base offsets do not depend on options
  *out = (const int*)((const char*)ws + L.off_err);
  return JLD_OK;
}

JLD_API int jld_ldl_order_f32(const void* ws, int32_t nx, int32_t ny, int32_t nz, int64_t nparts,
                              int32_t nstep, const int** out) {
  clear_error();
  if (!ws || !out || nstep < 1 || nparts < 1) return set_error(JLD_ERR_ARG, "jld_ldl_order_f32: bad arguments");
  LdlLayout L = ldl_layout(nx, ny, nz, nparts, nstep, kOptBinned);
  *out = (const int*)((const char*)ws + L.off_perm);
  return JLD_OK;
}

JLD_API int jld_ldl_positions_f32(const void* ws, int32_t nx, int32_t ny, int32_t nz, int64_t nparts,
                                  int32_t nstep, int32_t layer, const float** out) {
  clear_error();
  if (!ws || !out || layer < 1 || layer > nstep)
    return set_error(JLD_ERR_ARG, "jld_ldl_positions_f32: bad arguments");
  LdlLayout L = ldl_layout(nx, ny, nz, nparts, nstep, 0);
  *out = (const float*)((const char*)ws + L.off_pos) + (size_t)3 * nparts * (layer - 1);
  return JLD_OK;
}

}  // extern "C"
