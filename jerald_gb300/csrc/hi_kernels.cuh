// Kernels of the fused step's "HI" kind (model.py:213-247 layers,
// model.py:313-336 final map).  With a star map sm (an input mesh):
//   layer l (10 parameters a1, g1, kh1, kl1, nu1, a2, g2, kh2, kl2, nu2):
//     potk = 1e-3 (a1 G1(k) S1 + a2 G2(k) S2) / Nc,
//     S1 = pfft((fact rho + 1e-8)^g1), S2 = pfft(sm^g2),
//     G1 = -exp(-k^2/kl1^2 - kh1^2/k^2) k^nu1, G2 = +exp(-k^2/kl2^2 - kh2^2/k^2) k^nu2;
//   final map (12 parameters mu, w, b, beta1, khi, kli, nui, beta2, gamma3,
//   xi, eta, zs):
//     dep1 = pifft(pfft(sm) Fk / Nc),  Fk = exp(-k/kli - khi/k) k^nui + xi,
//     D = ReLU(beta1 dep1 + eta) + beta2 sm^gamma3,
//     F = ReLU(w ReLU(fact rho + zs)^mu - D + b).
// The S1 half of a layer is the "sm" machinery of the step (the x filter
// adds the S2 term); the kernels here are the S2 half and the final map:
//   StarPow            source map sm^g2 on the rows of the z r2c
//   hi_src2_kernel     adjoint over the whole spectrum: d(a2, kh2, kl2, nu2)
//                      from W (the cotangent spectrum of potk) and S2, and
//                      V2 = 1e-3 a2 G2 W / Nc for the g2 adjoint
//   star_reduce_kernel d g2 = sum ct_s2 sm^g2 ln sm after V2's inverse
//   hi_dep_filter_kernel  Y = pfft(sm) Fk / Nc on the caller's half spectrum
//   hi_loss_kernel     map, loss and the cell-sum gradients; the density
//                      cotangent and the cotangent of dep1
//   hi_filter_grad_kernel d(khi, kli, nui, xi) from pfft(ct_dep1) and pfft(sm)
// The gradient conventions follow the sm kind: mode 0 applies the
// reference's VJP rules (a1 and a2 without the half-spectrum multiplicity),
// mode 1 the exact adjoint.  sm^e is taken as 0 where sm <= 0, and so are
// its derivatives (the star map is zero in most cells).
#pragma once

#include "ldl_kernels.cuh"

namespace jld {

constexpr int kHiLayerParams = 10;
constexpr int kHiFinalParams = 12;

// sm^g2 (g2 = params[6] of the layer); 0 where sm <= 0.
struct StarPow {
  const float* params;
  __device__ __forceinline__ float operator()(float v, int64_t) const {
    return v > 0.f ? pow_pos(v, __ldg(params + 6)) : 0.f;
  }
};

// Spectral index (kx, ky, kz) of element e of the internal split layout:
// main[x][y][kz] (kz < h), then nyq[x][y] (kz = h).
__device__ __forceinline__ void spec_index(int64_t e, int ny, int h, int64_t nmain, int* ix, int* iy, int* kz) {
  if (e < nmain) {
    *kz = (int)(e % h);
    const int64_t r = e / h;
    *iy = (int)(r % ny);
    *ix = (int)(r / ny);
  } else {
    const int64_t r = e - nmain;
    *kz = h;
    *iy = (int)(r % ny);
    *ix = (int)(r / ny);
  }
}

// Half-spectrum weights of the gradient conventions (as xbwd_kernel):
// m_alpha for a spectrum amplitude, m_green for a real Fourier multiplier.
__device__ __forceinline__ void spec_weights(int kz, int h, int ny, int nz, int mode, float* m_alpha,
                                             float* m_green) {
  const float mk = (kz == 0 || (kz == h && (nz & 1) == 0)) ? 1.f : 2.f;
  *m_alpha = mode == 1 ? mk : 1.f;
  *m_green = mode == 1 ? mk : ((kz >= 1 && kz < ny / 2) ? 2.f : 1.f);
}

// Partials per block: [d a2, d kh2, d kl2, d nu2].  W -> V2 in place.
__global__ void __launch_bounds__(256)
hi_src2_kernel(float2* __restrict__ W, const float2* __restrict__ S2, int nx, int ny, int nz, KTables kt,
               const float* __restrict__ params, int mode, float scale, double* __restrict__ partials) {
  const int h = nz / 2;
  const int64_t nmain = (int64_t)nx * ny * h, ntot = nmain + (int64_t)nx * ny;
  const float a2 = __ldg(params + 5), kh2 = __ldg(params + 7), kl2 = __ldg(params + 8), nu2 = __ldg(params + 9);
  const float a1f = 1e-3f * scale, vm = 1e-3f * a2 * scale;
  KahanF acc[4];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ntot; e += (int64_t)gridDim.x * blockDim.x) {
    int ix, iy, kz;
    spec_index(e, ny, h, nmain, &ix, &iy, &kz);
    // G2 = +exp(...) k^nu2: the sm-kind Green's function with the sign flipped
    const Green gr = green_fn(__ldg(kt.kx + ix), __ldg(kt.ky + iy), __ldg(kt.kz + kz), 0, kh2, kl2, nu2);
    const float g2 = -gr.g;
    const float2 w = W[e], s = __ldg(S2 + e);
    const float reWS = w.x * s.x + w.y * s.y;
    float m_alpha, m_green;
    spec_weights(kz, h, ny, nz, mode, &m_alpha, &m_green);
    acc[0].add(m_alpha * a1f * g2 * reWS);
    const float qg = m_green * 1e-3f * a2 * scale * reWS;
    acc[1].add(qg * -gr.dkh);
    acc[2].add(qg * -gr.dkl);
    acc[3].add(qg * -gr.dnu);
    const float m = vm * g2;
    W[e] = make_float2(w.x * m, w.y * m);
  }
  block_reduce_kahan<4>(acc, partials, 4);
}

// d g2 = sum ct_s2 sm^g2 ln(sm) over cells with sm > 0; one partial per block.
__global__ void __launch_bounds__(256)
star_reduce_kernel(const float* __restrict__ cts, const float* __restrict__ sm, const float* __restrict__ params,
                   int64_t C, double* __restrict__ partials) {
  const float g2 = __ldg(params + 6);
  KahanF acc[1];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < C; e += (int64_t)gridDim.x * blockDim.x) {
    const float v = __ldg(sm + e);
    if (v > 0.f) {
      float lb;
      const float s = pow_pos(v, g2, &lb);
      acc[0].add(__ldg(cts + e) * s * lb);
    }
  }
  block_reduce_kahan<1>(acc, partials, 1);
}

// The depletion filter Fk = exp(-k/kli - khi/k) k^nui + xi and its
// derivatives (the dm-kind Green's function with the sign flipped).
struct DepFilter {
  float f, dkhi, dkli, dnui;
};
__device__ __forceinline__ DepFilter dep_filter(float kx, float ky, float kz, float khi, float kli, float nui,
                                                float xi) {
  const Green gr = green_fn(kx, ky, kz, 1, khi, kli, nui);
  DepFilter d;
  d.f = -gr.g + xi;
  d.dkhi = -gr.dkh;
  d.dkli = -gr.dkl;
  d.dnui = -gr.dnu;
  return d;
}

// Y = SMu Fk scale on the caller's half-spectrum layout (nx, ny, h+1).
__global__ void __launch_bounds__(256)
hi_dep_filter_kernel(float2* __restrict__ Y, const float2* __restrict__ SMu, int nx, int ny, int nz, KTables kt,
                     const float* __restrict__ fparams, float scale) {
  const int h1 = nz / 2 + 1;
  const int64_t ntot = (int64_t)nx * ny * h1;
  const float khi = __ldg(fparams + 4), kli = __ldg(fparams + 5), nui = __ldg(fparams + 6),
              xi = __ldg(fparams + 9);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ntot; e += (int64_t)gridDim.x * blockDim.x) {
    const int kz = (int)(e % h1);
    const int64_t r = e / h1;
    const int iy = (int)(r % ny), ix = (int)(r / ny);
    const DepFilter d = dep_filter(__ldg(kt.kx + ix), __ldg(kt.ky + iy), __ldg(kt.kz + kz), khi, kli, nui, xi);
    const float m = d.f * scale;
    const float2 s = __ldg(SMu + e);
    Y[e] = make_float2(s.x * m, s.y * m);
  }
}

// Partials per block: [d khi, d kli, d nui, d xi] from C = pfft(ct_dep1)
// and SMu = pfft(sm) (caller layout).
__global__ void __launch_bounds__(256)
hi_filter_grad_kernel(const float2* __restrict__ Cspec, const float2* __restrict__ SMu, int nx, int ny, int nz,
                      KTables kt, const float* __restrict__ fparams, int mode, float scale,
                      double* __restrict__ partials) {
  const int h = nz / 2, h1 = h + 1;
  const int64_t ntot = (int64_t)nx * ny * h1;
  const float khi = __ldg(fparams + 4), kli = __ldg(fparams + 5), nui = __ldg(fparams + 6),
              xi = __ldg(fparams + 9);
  KahanF acc[4];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ntot; e += (int64_t)gridDim.x * blockDim.x) {
    const int kz = (int)(e % h1);
    const int64_t r = e / h1;
    const int iy = (int)(r % ny), ix = (int)(r / ny);
    const DepFilter d = dep_filter(__ldg(kt.kx + ix), __ldg(kt.ky + iy), __ldg(kt.kz + kz), khi, kli, nui, xi);
    const float2 c = __ldg(Cspec + e), s = __ldg(SMu + e);
    float m_alpha, m_green;
    spec_weights(kz, h, ny, nz, mode, &m_alpha, &m_green);
    const float q = m_green * scale * (c.x * s.x + c.y * s.y);
    acc[0].add(q * d.dkhi);
    acc[1].add(q * d.dkli);
    acc[2].add(q * d.dnui);
    acc[3].add(q);
  }
  block_reduce_kahan<4>(acc, partials, 4);
}

// ReLU of model.py:55-57 and its derivative (1 above the floor, else 0).
__device__ __forceinline__ float relu_floor(float x) { return x > 1e-12f ? x : 1e-12f; }

// Final map, loss and cotangents.  Partials per block: [loss, d mu, d w,
// d b, d beta1, d beta2, d gamma3, d eta, d zs].  rb = fact * dL/d(rho);
// ctd = dL/d(dep1).
__global__ void __launch_bounds__(256)
hi_loss_kernel(const float* __restrict__ rho_paint, const float* __restrict__ sm, const float* __restrict__ dep1,
               const float* __restrict__ target, const float* __restrict__ mask, int64_t C, float fact,
               const float* __restrict__ fparams, int L1, const double* __restrict__ inv_npix,
               float* __restrict__ rb, float* __restrict__ ctd, double* __restrict__ partials) {
  const float mu = __ldg(fparams + 0), w = __ldg(fparams + 1), b = __ldg(fparams + 2), beta1 = __ldg(fparams + 3),
              beta2 = __ldg(fparams + 7), gamma3 = __ldg(fparams + 8), eta = __ldg(fparams + 10),
              zs = __ldg(fparams + 11);
  const float inpx = (float)(*inv_npix);
  KahanF acc[9];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < C; e += (int64_t)gridDim.x * blockDim.x) {
    const float a0 = __fadd_rn(__fmul_rn(__ldg(rho_paint + e), fact), zs);
    const float A = relu_floor(a0);
    float lnA;
    const float Am = pow_pos(A, mu, &lnA);
    const float smv = __ldg(sm + e);
    float lns = 0.f, s3 = 0.f;
    if (smv > 0.f) s3 = pow_pos(smv, gamma3, &lns);
    const float d1 = __ldg(dep1 + e);
    const float v = __fadd_rn(__fmul_rn(beta1, d1), eta);
    const float D = __fadd_rn(relu_floor(v), __fmul_rn(beta2, s3));
    const float u = __fadd_rn(__fsub_rn(__fmul_rn(w, Am), D), b);
    const float F = relu_floor(u);
    const float m = mask ? __ldg(mask + e) : 1.f;
    const float diff = F - __ldg(target + e);
    const float ad = fabsf(diff) * m;
    acc[0].add(L1 ? ad : ad * ad);
    const float sg = diff >= 0.f ? 1.f : -1.f;
    const float ctF = (L1 ? sg * m : 2.f * fabsf(diff) * m * m * sg) * inpx;
    const float ctu = u > 1e-12f ? ctF : 0.f;
    acc[1].add(ctu * w * Am * lnA);
    acc[2].add(ctu * Am);
    acc[3].add(ctu);
    // A^(mu-1) = A^mu / A (A >= 1e-12)
    const float ctA = a0 > 1e-12f ? ctu * w * mu * (Am / A) : 0.f;
    acc[8].add(ctA);
    rb[e] = ctA * fact;
    const float ctD = -ctu;
    acc[5].add(ctD * s3);
    acc[6].add(ctD * beta2 * s3 * lns);
    const float ctv = v > 1e-12f ? ctD : 0.f;
    acc[7].add(ctv);
    acc[4].add(ctv * d1);
    ctd[e] = ctv * beta1;
  }
  block_reduce_kahan<9>(acc, partials, 9);
}

}  // namespace jld
