// Host-side helpers of the pipelined passes: TMA descriptors over the main
// block of the internal half spectrum and the geometry (tile shape, threads,
// shared memory, persistent grid) of the strided and row passes.
#pragma once

#include <cstdlib>

#include <algorithm>
#include <mutex>

#include <cudaTypedefs.h>

#include "pipe_passes.cuh"
#include "zpipe_core.cuh"

namespace jld {

// ---------------------------------------------------------------------------
// TMA descriptors for the pipelined passes.

inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

// Tensor map over the main block main[nx][ny][h] (complex, viewed as float
// pairs) with a box of `cols` columns by min(lines, 256) lines.
inline int make_main_map(CUtensorMap* m, const float2* main, int nx, int ny, int h, int ax, int cols,
                         int lines) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return set_error(JLD_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const cuuint32_t boxl = (cuuint32_t)std::min(lines, 256);
  CUresult r;
  if (ax == 1) {
    cuuint64_t dims[3] = {(cuuint64_t)2 * h, (cuuint64_t)ny, (cuuint64_t)nx};
    cuuint64_t strides[2] = {(cuuint64_t)h * 8, (cuuint64_t)ny * h * 8};
    cuuint32_t box[3] = {(cuuint32_t)(2 * cols), boxl, 1};
    cuuint32_t es[3] = {1, 1, 1};
    r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)main, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  } else {
    cuuint64_t dims[2] = {(cuuint64_t)2 * ny * h, (cuuint64_t)nx};
    cuuint64_t strides[1] = {(cuuint64_t)ny * h * 8};
    cuuint32_t box[2] = {(cuuint32_t)(2 * cols), boxl};
    cuuint32_t es[2] = {1, 1};
    r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)main, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  }
  if (r != CUDA_SUCCESS) return set_error(JLD_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return JLD_OK;
}

// Geometry of a pipelined strided pass over the main block, or ok = false
// when the mesh does not qualify (line length not a power of two in
// [16, 2048], or h not a multiple of the tile width).
struct PipeGeom {
  bool ok = false;
  SGeom g;
  int nthr = 0;
  int grid = 0;
  size_t smem = 0;
};

// E = values per thread per line of the schedule (16: P2For, 8: P2For8);
// regs = registers per thread the kernel is built for.
inline PipeGeom pipe_geom(int nx, int ny, int h, int ax, int nacc, int E = 16, int regs = 128, int min_cols_req = 0) {
  PipeGeom p;
  const int lines = ax == 1 ? ny : nx;
  if (lines < 16 || lines > 2048 || h < 2 || (h & 1)) return p;
  if (lines & (lines - 1)) {
    // 3 x 2^k: only the P2For family has such schedules; lines of at most
    // 256 keep a tile one TMA box high
    int psh = 0;
    if (E != 16 || lines > 256 || !p2_shape(lines, &E, &psh)) return p;
  }
  // Widest tile (<= 16 columns, <= 512 threads, cols dividing h) whose CTA
  // leaves room for a second one on the SM (a CTA waits at barriers between
  // FFT stages; a second CTA keeps the SM busy meanwhile), else the widest
  // that fits alone.
  auto smem_of = [&](int c) { return (size_t)lines * c * 8 * (2 + nacc) + 64; };
  auto fits = [&](int c, size_t cap) { return c * lines / E <= 512 && h % c == 0 && smem_of(c) <= cap; };
  // The narrowest tile taken at two CTAs per SM before a wider one at one
  // CTA per SM: a tile reads `cols` consecutive complex values (8 * cols
  // bytes) of each of its lines, every line in another part of the spectrum
  // (4 MiB apart for the x pass at 1024^3).  At 1024 lines 64-byte pieces
  // at one CTA per SM beat 32-byte pieces at two: the 1024^3 r2c took
  // 8.58 instead of 12.28 ms; 512^3 and 256^3 (which get 8 or 16 columns at
  // two CTAs anyway) did not change.  min_cols_req (4, 8 or 16; the fused
  // step's tuning option) or else JLD_PIPE_MIN_COLS = 4, 8 or 16 overrides
  // the choice (results are the same).
  static const int min_cols_env = [] {
    const char* e = getenv("JLD_PIPE_MIN_COLS");
    const int v = e ? atoi(e) : 0;
    return (v == 4 || v == 8 || v == 16) ? v : 0;
  }();
  const int min_cols = min_cols_req ? min_cols_req : min_cols_env ? min_cols_env : (lines >= 1024 ? 8 : 4);
  int cols = 16;
  while (cols >= min_cols && !fits(cols, 112 * 1024)) cols >>= 1;
  if (cols < min_cols) {
    cols = 16;
    while (cols >= 4 && !fits(cols, 226 * 1024)) cols >>= 1;
  }
  if (cols < 4) return p;
  SGeom& g = p.g;
  g.nx = nx; g.ny = ny; g.h = h;
  g.cols = cols;
  g.cshift = ilog2i(cols);
  g.lines = lines;
  g.ntiles = (int)(((int64_t)(ax == 1 ? nx : ny) * h) / cols);
  g.es = ax == 1 ? h : (int64_t)ny * h;
  p.nthr = cols * lines / E;
  p.smem = smem_of(cols);
  // resident CTAs per SM: shared memory, registers and threads
  const int per_sm = std::max(1, std::min({(int)((227 * 1024) / (p.smem + 1024)), 65536 / (p.nthr * regs),
                                           2048 / p.nthr, 32}));
  p.grid = (int)std::min<int64_t>(g.ntiles, (int64_t)per_sm * sm_count());
  p.ok = true;
  return p;
}

// Geometry of a pipelined z pass over `nin` meshes (tiles of R whole rows of
// each), or ok = false when h has no pipelined schedule (2^k in [16, 2048],
// 48, 96, 192) or no even
// R divides the row count within 512 threads and ~110 KB of shared memory
// (two CTAs per SM).
struct ZPipeGeom {
  bool ok = false;
  ZTile zt;
  int nthr = 0;
  size_t smem = 0;
};

// slot_row = staging bytes per row of the tile (all meshes), cap = shared
// memory limit.
// max_thr caps the CTA size for kernels whose register count would
// otherwise leave one CTA per SM (smaller tiles, more resident CTAs).
inline ZPipeGeom zpipe_geom(int64_t rows, int h, int nin, size_t slot_row, size_t cap = 110 * 1024,
                            int max_thr = 512) {
  ZPipeGeom z;
  int E = 0, psh = 0;
  if (h < 16 || h > 2048 || !p2_shape(h, &E, &psh)) return z;
  const int ldw = h + (h >> psh);  // ZShape<P2For<h>>::LDW
  for (int R = 32; R >= 2; R >>= 1) {
    const int lines = nin * R;
    const int64_t thr = (int64_t)lines * h / E;
    const size_t smem = (size_t)R * slot_row + (size_t)lines * ldw * 8 + 16;
    if (thr > max_thr || rows % R || smem > cap) continue;
    if (thr < 32) return z;
    z.ok = true;
    z.zt.R = R;
    z.zt.ntiles = (int)(rows / R);
    z.zt.rows = rows;
    z.zt.nyq_off = rows * h;
    z.nthr = (int)thr;
    z.smem = smem;
    return z;
  }
  return z;
}

// Persistent grid of a pipelined kernel: every SM full, never more CTAs
// than tiles.
template <class K>
inline int persistent_grid(K kern, int nthr, size_t smem, int ntiles, unsigned* grid) {
  int per_sm = 0;
  JLD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nthr, smem));
  if (per_sm < 1) return set_error(JLD_ERR_CUDA, "pipelined z pass does not fit on an SM");
  *grid = (unsigned)std::min<int64_t>(ntiles, (int64_t)per_sm * sm_count());
  return JLD_OK;
}

}  // namespace jld
