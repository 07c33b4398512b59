/*
 * ORACLE — test infrastructure only.  CPU restatement of the reference's
 * single-rank cloud-in-cell loops, used by tests/, the smoke check and the
 * CPU-baseline leg of bench.py to check results against.  Nothing in the
 * product links or calls this file.
 *
 * Parity status: pinned.  The reference's own CIC loops (lib/parops_fast.h)
 * are compiled from its source with a world-size-one MPI stand-in
 * (oracle/ref_stub/mpi.h, oracle/build.py: build_ref) and
 * tests/test_ref_pin.py requires this restatement's outputs to equal theirs
 * bit for bit.
 *
 * Restated functions (world size one: every particle is local, edges are
 * [0, N) on each axis, the decomposition keeps input order):
 *   orc_box_to_mesh   jaxpops_bind.py:163-164   (pos % BoxSize) / (BoxSize/Nmesh)
 *   orc_cell_keys     lib/parops_fast.h:91-93   int(pos) % Nmesh per axis
 *   orc_paint         lib/parops_fast.h:354-411 (lpaint) + 527 (zeroing)
 *   orc_readout       lib/parops_fast.h:414-481 (lreadout, vjpdim)
 *   orc_paint3d       lib/parops_fast.h:616-676 (lpaint3D) + 720-721
 *   orc_readout3d     lib/parops_fast.h:730-821 (lreadout3D, vjp)
 * The arithmetic follows the reference's expression order; build with
 * -ffp-contract=off so no multiply-add is fused (x86-64 builds of the
 * reference have no FMA).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_DEFINE(T, SFX)                                                      \
  /* jnp.remainder: fmod, plus the divisor when signs differ and r != 0 */     \
  static T orc_rem_##SFX(T x, T m) {                                            \
    T r = (T)fmod(x, m);                                                        \
    if (r != (T)0 && ((r < (T)0) != (m < (T)0))) r = r + m;                      \
    return r;                                                                   \
  }                                                                             \
  void orc_box_to_mesh_##SFX(const T* pos, int64_t n, const T* box,            \
                             const int64_t* nmesh, T* out) {                    \
    T cell[3];                                                                  \
    for (int a = 0; a < 3; ++a) cell[a] = box[a] / (T)nmesh[a];                 \
    for (int64_t p = 0; p < n; ++p)                                             \
      for (int a = 0; a < 3; ++a)                                               \
        out[3 * p + a] = orc_rem_##SFX(pos[3 * p + a], box[a]) / cell[a];       \
  }                                                                             \
  void orc_cell_keys_##SFX(const T* pos, int64_t n, const int64_t* nmesh,       \
                           int64_t* keys) {                                     \
    for (int64_t p = 0; p < n; ++p) {                                           \
      int i = (int)pos[3 * p] % (int)nmesh[0];                                  \
      int j = (int)pos[3 * p + 1] % (int)nmesh[1];                              \
      int k = (int)pos[3 * p + 2] % (int)nmesh[2];                              \
      keys[p] = ((int64_t)i * nmesh[1] + j) * nmesh[2] + k;                     \
    }                                                                           \
  }                                                                             \
  /* Per-particle CIC setup shared by the loops below. */                       \
  typedef struct {                                                              \
    int i, j, k, ip1, jp1, kp1;                                                 \
    int inx, iny, inz, inpx, inpy, inpz;                                        \
    T d[3];                                                                     \
  } orc_cic_##SFX;                                                              \
  static void orc_setup_##SFX(const T* q, const int64_t* nm, orc_cic_##SFX* c) { \
    int sz[3] = {(int)nm[0], (int)nm[1], (int)nm[2]};                           \
    int i = (int)q[0], j = (int)q[1], k = (int)q[2];                            \
    c->d[0] = q[0] - (T)i;                                                      \
    c->d[1] = q[1] - (T)j;                                                      \
    c->d[2] = q[2] - (T)k;                                                      \
    int ip1 = (i + 1) % sz[0], jp1 = (j + 1) % sz[1], kp1 = (k + 1) % sz[2];    \
    c->inx = (unsigned)i < (unsigned)sz[0];                                     \
    c->iny = (unsigned)j < (unsigned)sz[1];                                     \
    c->inz = (unsigned)k < (unsigned)sz[2];                                     \
    c->inpx = (unsigned)ip1 < (unsigned)sz[0];                                  \
    c->inpy = (unsigned)jp1 < (unsigned)sz[1];                                  \
    c->inpz = (unsigned)kp1 < (unsigned)sz[2];                                  \
    c->i = abs(i % sz[0]); c->j = abs(j % sz[1]); c->k = abs(k % sz[2]);        \
    c->ip1 = abs(ip1 % sz[0]); c->jp1 = abs(jp1 % sz[1]);                       \
    c->kp1 = abs(kp1 % sz[2]);                                                  \
  }                                                                             \
  static void orc_paint_into_##SFX(const T* pos, int64_t n, const T* mass,      \
                                   int mstride, int64_t moff, const int64_t* nm, \
                                   T* f) {                                      \
    int64_t sy = nm[2], sx = nm[1] * nm[2];                                     \
    for (int64_t p = 0; p < n; ++p) {                                           \
      orc_cic_##SFX c;                                                          \
      orc_setup_##SFX(pos + 3 * p, nm, &c);                                     \
      T dx = c.d[0], dy = c.d[1], dz = c.d[2];                                  \
      T tx = 1 - dx, ty = 1 - dy, tz = 1 - dz;                                  \
      T m = mass[mstride * p + moff];                                           \
      f[c.i * sx + c.j * sy + c.k] += tx * ty * tz * m * c.inx * c.iny * c.inz; \
      f[c.ip1 * sx + c.j * sy + c.k] += dx * ty * tz * m * c.inpx * c.iny * c.inz; \
      f[c.i * sx + c.jp1 * sy + c.k] += tx * dy * tz * m * c.inx * c.inpy * c.inz; \
      f[c.i * sx + c.j * sy + c.kp1] += tx * ty * dz * m * c.inx * c.iny * c.inpz; \
      f[c.ip1 * sx + c.jp1 * sy + c.k] += dx * dy * tz * m * c.inpx * c.inpy * c.inz; \
      f[c.ip1 * sx + c.j * sy + c.kp1] += dx * ty * dz * m * c.inpx * c.iny * c.inpz; \
      f[c.i * sx + c.jp1 * sy + c.kp1] += tx * dy * dz * m * c.inx * c.inpy * c.inpz; \
      f[c.ip1 * sx + c.jp1 * sy + c.kp1] += dx * dy * dz * m * c.inpx * c.inpy * c.inpz; \
    }                                                                           \
  }                                                                             \
  void orc_paint_##SFX(const T* pos, int64_t n, const T* mass,                  \
                       const int64_t* nm, T* field) {                           \
    memset(field, 0, sizeof(T) * (size_t)(nm[0] * nm[1] * nm[2]));              \
    orc_paint_into_##SFX(pos, n, mass, 1, 0, nm, field);                        \
  }                                                                             \
  void orc_paint3d_##SFX(const T* pos, int64_t n, const T* mass,                \
                         const int64_t* nm, T* field) {                         \
    /* lpaint3D loops d inside the particle loop; each channel is an */         \
    /* independent accumulation so the per-channel order is the same. */        \
    int64_t C = nm[0] * nm[1] * nm[2];                                          \
    memset(field, 0, sizeof(T) * (size_t)(3 * C));                              \
    for (int d = 0; d < 3; ++d)                                                 \
      orc_paint_into_##SFX(pos, n, mass, 3, d, nm, field + d * C);              \
  }                                                                             \
  static T orc_gather_##SFX(const orc_cic_##SFX* c, const T* ds, const T* ts,   \
                            const T* f, int64_t sx, int64_t sy) {               \
    return ts[0] * ts[1] * ts[2] * f[c->i * sx + c->j * sy + c->k] * c->inx * c->iny * c->inz + \
           ds[0] * ts[1] * ts[2] * f[c->ip1 * sx + c->j * sy + c->k] * c->inpx * c->iny * c->inz + \
           ts[0] * ds[1] * ts[2] * f[c->i * sx + c->jp1 * sy + c->k] * c->inx * c->inpy * c->inz + \
           ts[0] * ts[1] * ds[2] * f[c->i * sx + c->j * sy + c->kp1] * c->inx * c->iny * c->inpz + \
           ds[0] * ds[1] * ts[2] * f[c->ip1 * sx + c->jp1 * sy + c->k] * c->inpx * c->inpy * c->inz + \
           ds[0] * ts[1] * ds[2] * f[c->ip1 * sx + c->j * sy + c->kp1] * c->inpx * c->iny * c->inpz + \
           ts[0] * ds[1] * ds[2] * f[c->i * sx + c->jp1 * sy + c->kp1] * c->inx * c->inpy * c->inpz + \
           ds[0] * ds[1] * ds[2] * f[c->ip1 * sx + c->jp1 * sy + c->kp1] * c->inpx * c->inpy * c->inpz; \
  }                                                                             \
  void orc_readout_##SFX(const T* pos, int64_t n, const T* field,               \
                         const int64_t* nm, const T* box, int vjpdim, T* out) { \
    int64_t sy = nm[2], sx = nm[1] * nm[2];                                     \
    for (int64_t p = 0; p < n; ++p) {                                           \
      orc_cic_##SFX c;                                                          \
      orc_setup_##SFX(pos + 3 * p, nm, &c);                                     \
      T ds[3] = {c.d[0], c.d[1], c.d[2]};                                       \
      T ts[3] = {1 - ds[0], 1 - ds[1], 1 - ds[2]};                              \
      if (vjpdim >= 0) {                                                        \
        ds[vjpdim] = (T)nm[vjpdim] / box[vjpdim];                               \
        ts[vjpdim] = -ds[vjpdim];                                               \
      }                                                                         \
      out[p] = orc_gather_##SFX(&c, ds, ts, field, sx, sy);                     \
    }                                                                           \
  }                                                                             \
  void orc_readout3d_##SFX(const T* pos, int64_t n, const T* field,             \
                           const int64_t* nm, const T* box, int vjp, T* out) {  \
    int64_t sy = nm[2], sx = nm[1] * nm[2], C = nm[0] * nm[1] * nm[2];          \
    T dg[3], tg[3];                                                             \
    for (int a = 0; a < 3; ++a) { dg[a] = (T)nm[a] / box[a]; tg[a] = -dg[a]; }  \
    for (int64_t p = 0; p < n; ++p) {                                           \
      orc_cic_##SFX c;                                                          \
      orc_setup_##SFX(pos + 3 * p, nm, &c);                                     \
      for (int d = 0; d < 3; ++d) {                                             \
        T ds[3] = {c.d[0], c.d[1], c.d[2]};                                     \
        T ts[3] = {1 - ds[0], 1 - ds[1], 1 - ds[2]};                            \
        const T* f = field + (vjp ? 0 : d * C);                                 \
        if (vjp) { ds[d] = dg[d]; ts[d] = tg[d]; }                              \
        out[3 * p + d] = orc_gather_##SFX(&c, ds, ts, f, sx, sy);               \
      }                                                                         \
    }                                                                           \
  }

ORC_DEFINE(float, f32)
ORC_DEFINE(double, f64)
