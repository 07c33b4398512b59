// Snapshot-map ingestion on sm_103a: the per-particle part of makemap
// (JERALD/snaputils.py:253-406).  One elementwise pass turns a chunk of
// snapshot particles into paint inputs:
//   positions  pos / unit (snaputils.py:379, float32 division), then the
//              periodic wrap pos % BoxSize (snaputils.py:380), which NumPy
//              evaluates in float64 against the float64 BoxSize and rounds
//              back to float32;
//   weights    the map kind's weight from the particle fields
//              (snaputils.py:360-376) with NumPy 2's promotion: a float32
//              array times a float64 coefficient is float64, a product of
//              two float32 arrays stays float32; rounded once to float32 for
//              the paint.
// The chunk is then painted without clearing the map (jld_ppaint_box_acc_f32)
// so that a snapshot streams through the GPU chunk by chunk.

#include "common.cuh"

namespace jld {

// Map kinds (snaputils.py:288-318) and their weights, with
// c1 = 4.0475e-7 h^2 / a^3 XH / prod(BoxSize) * prod(Nmesh), c2 = 323.06014:
//   0 dm       none (painted with the scalar mass prod(Nmesh) / Ntotal)
//   1 Mstar    Masses
//   2 ne       c1 Masses Xe
//   3 nT       c1 Masses Xe c2 u / (1 + 3 XH + 4 XH Xe)
//   4 nHI      c1 Masses NHI
//   5 neVz     c1 Masses Xe vz sqrt(a)
//   6 MstarVz  Masses vz sqrt(a)
//   7 XHI      NHI
struct SnapFields {
  const float* mass;  // Masses
  const float* xe;    // ElectronAbundance
  const float* u;     // InternalEnergy
  const float* nhi;   // NeutralHydrogenAbundance
  const float* vz;    // vz of particle p at vz[vstride * p]
  int64_t vstride;
};

__device__ __forceinline__ double wrap_box(double x, double L) {
  double r = fmod(x, L);
  if (r != 0.0 && ((r < 0.0) != (L < 0.0))) r += L;
  return r;
}

__global__ void __launch_bounds__(256)
snap_prep_kernel(const float* __restrict__ pos, int64_t n, float unit, double bx, double by, double bz,
                 int kind, SnapFields f, double c1, double c2, double XH, double sqa,
                 float* __restrict__ pos_out, float* __restrict__ w) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    const double L[3] = {bx, by, bz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float x = __fdiv_rn(__ldg(pos + 3 * p + a), unit);
      pos_out[3 * p + a] = (float)wrap_box((double)x, L[a]);
    }
    if (kind == 0) continue;
    double v = 0.0;
    switch (kind) {
      case 1: v = (double)__ldg(f.mass + p); break;
      case 2: v = c1 * (double)__ldg(f.mass + p) * (double)__ldg(f.xe + p); break;
      case 3: {
        // (1 + 3 * XH + 4 * XH * Xe) with XH a Python float and Xe a float32
        // array is a float32 array under NumPy 2 promotion: the Python-float
        // constants 1 + 3 XH and 4 XH are rounded to float32 once, the
        // product and the sum are float32 operations.  The numerator has a
        // float64 coefficient, so the quotient is float64.
        const float xef = __ldg(f.xe + p);
        const float den = __fadd_rn((float)(1.0 + 3.0 * XH), __fmul_rn((float)(4.0 * XH), xef));
        v = c1 * (double)__ldg(f.mass + p) * (double)xef * c2 * (double)__ldg(f.u + p) / (double)den;
        break;
      }
      case 4: v = c1 * (double)__ldg(f.mass + p) * (double)__ldg(f.nhi + p); break;
      case 5:
        v = c1 * (double)__ldg(f.mass + p) * (double)__ldg(f.xe + p) * (double)__ldg(f.vz + f.vstride * p) * sqa;
        break;
      // Masses * Velocities is a float32 product (both arrays float32)
      case 6: v = (double)__fmul_rn(__ldg(f.mass + p), __ldg(f.vz + f.vstride * p)) * sqa; break;
      default: v = (double)__ldg(f.nhi + p); break;
    }
    w[p] = (float)v;
  }
}

}  // namespace jld

using namespace jld;

extern "C" {

int jld_snap_prep_f32(jld_stream_t s, const float* pos, int64_t n, float unit, const double box[3], int32_t kind,
                      const float* masses, const float* xe, const float* u, const float* nhi,
                      const float* vz, int64_t vstride, double c1, double c2, double XH, double sqrt_a,
                      float* pos_out, float* weights) {
  clear_error();
  const char* who = "jld_snap_prep_f32";
  if (n < 0) return set_error(JLD_ERR_ARG, "%s: n < 0", who);
  if (!box || !(box[0] > 0 && box[1] > 0 && box[2] > 0))
    return set_error(JLD_ERR_ARG, "%s: box sizes must be positive", who);
  if (!(unit > 0)) return set_error(JLD_ERR_ARG, "%s: unit must be positive", who);
  if (kind < 0 || kind > 7) return set_error(JLD_ERR_ARG, "%s: kind must be in 0..7", who);
  if (n == 0) return JLD_OK;
  if (!pos || !pos_out) return set_error(JLD_ERR_ARG, "%s: positions are NULL", who);
  const bool need_m = kind >= 1 && kind <= 6, need_xe = kind == 2 || kind == 3 || kind == 5;
  const bool need_u = kind == 3, need_nhi = kind == 4 || kind == 7, need_v = kind == 5 || kind == 6;
  if ((need_m && !masses) || (need_xe && !xe) || (need_u && !u) || (need_nhi && !nhi) || (need_v && !vz))
    return set_error(JLD_ERR_ARG, "%s: a field that map kind %d needs is NULL", who, kind);
  if (need_v && vstride < 1) return set_error(JLD_ERR_ARG, "%s: vz stride must be >= 1", who);
  if (kind != 0 && !weights) return set_error(JLD_ERR_ARG, "%s: weights is NULL", who);
  SnapFields f{masses, xe, u, nhi, vz, vstride};
  cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
  snap_prep_kernel<<<resident_grid(snap_prep_kernel, n, 256), 256, 0, st>>>(
      pos, n, unit, box[0], box[1], box[2], kind, f, c1, c2, XH, sqrt_a, pos_out, weights);
  JLD_LAUNCH_CHECK(who);
  return JLD_OK;
}

}  // extern "C"
