// Shared-memory pencil FFT engine (sm_103a, FP32 or FP64 data).
//
// A CTA holds `ncols` lines of length n in shared memory, laid out
// sm[j * ld + c] (line element j, column c, ld = ncols + 1 so that both a row
// of columns and a column of elements map to distinct banks).  The lines are
// transformed with a self-sorting (Stockham) mixed-radix decimation-in-time
// schedule: stage s with radix R reads the R values b + r*(n/R) of butterfly
// b, twiddles them by w_{pR}^{r*(b mod p)} (p = product of the earlier
// radices), applies a radix-R DFT and writes them to (b - b mod p)*R +
// b mod p + r*p.  The output comes out in natural order, so no bit reversal is
// needed.  Every thread owns E/R butterflies of every stage (E elements),
// loads them all, synchronises, and stores, so one buffer suffices.
//
// Twiddles come from per-length tables tw[m] = exp(-2*pi*i*m/n) generated on
// the host in FP64 (see fft.cu); the inverse transform conjugates them.
#pragma once

#include "common.cuh"

namespace jld {

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };
template <typename T> using cplx_t = typename Cplx<T>::type;

template <typename C> __device__ __forceinline__ C cmake(decltype(C::x) a, decltype(C::x) b) { C r; r.x = a; r.y = b; return r; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmake<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmake<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return cmake<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __device__ __forceinline__ C cconj(C a) { return cmake<C>(a.x, -a.y); }
template <typename C, typename S> __device__ __forceinline__ C cscale(C a, S s) { return cmake<C>(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse): sgn = -1 forward, +1 inverse
template <typename C> __device__ __forceinline__ C cmul_i(C a, int sgn) {
  return sgn < 0 ? cmake<C>(a.y, -a.x) : cmake<C>(-a.y, a.x);
}

// One 1-D transform schedule, passed by value to kernels.
constexpr int kMaxStages = 16;
template <typename T>
struct LinePlan {
  int n;                     // length
  int E;                     // elements per thread per column
  int nst;                   // number of stages
  int radix[kMaxStages];     // radix of each stage
  const cplx_t<T>* tw;       // n twiddles exp(-2 pi i m / n)
};

// ---------------------------------------------------------------------------
// Radix-R DFTs on registers: y[m] = sum_r u[r] exp(sgn * 2 pi i r m / R).

template <typename C>
__device__ __forceinline__ void dft2(C& a, C& b) {
  C t = a; a = cadd(t, b); b = csub(t, b);
}

template <typename C>
__device__ __forceinline__ void dft4(C& u0, C& u1, C& u2, C& u3, int sgn) {
  C t0 = cadd(u0, u2), t1 = csub(u0, u2);
  C t2 = cadd(u1, u3), t3 = cmul_i(csub(u1, u3), sgn);
  u0 = cadd(t0, t2); u2 = csub(t0, t2);
  u1 = cadd(t1, t3); u3 = csub(t1, t3);
}

template <typename C>
__device__ __forceinline__ void dft8(C* u, int sgn) {
  using S = decltype(C::x);
  const S h = (S)0.70710678118654752440;  // sqrt(1/2)
  C e0 = u[0], e1 = u[2], e2 = u[4], e3 = u[6];
  C o0 = u[1], o1 = u[3], o2 = u[5], o3 = u[7];
  dft4(e0, e1, e2, e3, sgn);
  dft4(o0, o1, o2, o3, sgn);
  // o1 *= w8^1, o2 *= w8^2, o3 *= w8^3 with w8 = exp(sgn*i*pi/4)
  S sg = (S)sgn;
  o1 = cmake<C>(h * (o1.x - sg * o1.y), h * (o1.y + sg * o1.x));
  o2 = cmul_i(o2, sgn);
  o3 = cmake<C>(h * (-o3.x - sg * o3.y), h * (-o3.y + sg * o3.x));
  u[0] = cadd(e0, o0); u[4] = csub(e0, o0);
  u[1] = cadd(e1, o1); u[5] = csub(e1, o1);
  u[2] = cadd(e2, o2); u[6] = csub(e2, o2);
  u[3] = cadd(e3, o3); u[7] = csub(e3, o3);
}

template <typename C>
__device__ __forceinline__ void dft16(C* u, int sgn) {
  using S = decltype(C::x);
  C e[8], o[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) { e[r] = u[2 * r]; o[r] = u[2 * r + 1]; }
  dft8(e, sgn);
  dft8(o, sgn);
  // w16^m = cos(2 pi m/16) + sgn*i*sin(2 pi m/16)
  const S c[8] = {(S)1.0, (S)0.92387953251128675613, (S)0.70710678118654752440,
                  (S)0.38268343236508977173, (S)0.0, (S)-0.38268343236508977173,
                  (S)-0.70710678118654752440, (S)-0.92387953251128675613};
  const S s[8] = {(S)0.0, (S)0.38268343236508977173, (S)0.70710678118654752440,
                  (S)0.92387953251128675613, (S)1.0, (S)0.92387953251128675613,
                  (S)0.70710678118654752440, (S)0.38268343236508977173};
  S sg = (S)sgn;
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    C w = cmake<C>(c[m], sg * s[m]);
    C t = (m == 0) ? o[m] : cmul(o[m], w);
    u[m] = cadd(e[m], t);
    u[m + 8] = csub(e[m], t);
  }
}

template <typename C>
__device__ __forceinline__ void dft3(C* u, int sgn) {
  using S = decltype(C::x);
  const S s3 = (S)0.86602540378443864676;  // sqrt(3)/2
  C t = cadd(u[1], u[2]);
  C m = csub(u[0], cscale(t, (S)0.5));
  C d = csub(u[1], u[2]);
  // i*sgn*s3*d
  C id = cmake<C>(-(S)sgn * s3 * d.y, (S)sgn * s3 * d.x);
  u[0] = cadd(u[0], t);
  u[1] = cadd(m, id);
  u[2] = csub(m, id);
}

template <typename C>
__device__ __forceinline__ void dft5(C* u, int sgn) {
  using S = decltype(C::x);
  const S c1 = (S)0.30901699437494742410;   // cos(2pi/5)
  const S c2 = (S)-0.80901699437494742410;  // cos(4pi/5)
  const S s1 = (S)0.95105651629515357212;   // sin(2pi/5)
  const S s2 = (S)0.58778525229247312917;   // sin(4pi/5)
  C a1 = cadd(u[1], u[4]), a2 = cadd(u[2], u[3]);
  C b1 = csub(u[1], u[4]), b2 = csub(u[2], u[3]);
  C r1 = cadd(u[0], cadd(cscale(a1, c1), cscale(a2, c2)));
  C r2 = cadd(u[0], cadd(cscale(a1, c2), cscale(a2, c1)));
  C q1 = cadd(cscale(b1, s1), cscale(b2, s2));   // multiplies sgn*i
  C q2 = csub(cscale(b1, s2), cscale(b2, s1));
  S sg = (S)sgn;
  C iq1 = cmake<C>(-sg * q1.y, sg * q1.x);
  C iq2 = cmake<C>(-sg * q2.y, sg * q2.x);
  u[0] = cadd(u[0], cadd(a1, a2));
  u[1] = cadd(r1, iq1);
  u[4] = csub(r1, iq1);
  u[2] = cadd(r2, iq2);
  u[3] = csub(r2, iq2);
}

template <int R, typename C>
__device__ __forceinline__ void dftR(C* u, int sgn) {
  if constexpr (R == 2) dft2(u[0], u[1]);
  else if constexpr (R == 3) dft3(u, sgn);
  else if constexpr (R == 4) dft4(u[0], u[1], u[2], u[3], sgn);
  else if constexpr (R == 5) dft5(u, sgn);
  else if constexpr (R == 8) dft8(u, sgn);
  else if constexpr (R == 16) dft16(u, sgn);
}

// ---------------------------------------------------------------------------
// One Stockham stage over all columns of the shared-memory tile.
// Column-fastest thread mapping: id -> c = id & cmask, b = id >> cshift.
template <typename T, int EMAX, int R>
__device__ __forceinline__ void fft_stage(cplx_t<T>* sm, int ld, int n, int p, int E,
                                          int cshift, const cplx_t<T>* __restrict__ tw,
                                          int sgn, int tid, int nthr) {
  using C = cplx_t<T>;
  constexpr int QMAX = EMAX / R;
  const int nq = E / R;
  const int Tn = n / R;
  const int tws = n / (p * R);
  const int cmask = (1 << cshift) - 1;
  C u[QMAX > 0 ? QMAX : 1][R];
#pragma unroll
  for (int q = 0; q < QMAX; ++q) {
    if (q < nq) {
      int id = tid + q * nthr;
      int c = id & cmask, b = id >> cshift;
#pragma unroll
      for (int r = 0; r < R; ++r) u[q][r] = sm[(b + r * Tn) * ld + c];
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < QMAX; ++q) {
    if (q < nq) {
      int id = tid + q * nthr;
      int c = id & cmask, b = id >> cshift;
      int k = b % p;
      if (k != 0) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          C w = __ldg(tw + r * k * tws);
          if (sgn > 0) w.y = -w.y;
          u[q][r] = cmul(u[q][r], w);
        }
      }
      dftR<R>(u[q], sgn);
      int j = (b - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) sm[(j + r * p) * ld + c] = u[q][r];
    }
  }
  __syncthreads();
}

// Out-of-line copy of a stage for the mixed-radix schedules, so that each
// radix keeps its own register allocation.
template <typename T, int R>
__device__ __noinline__ void fft_stage_gen(cplx_t<T>* sm, int ld, int n, int p, int E,
                                           int cshift, const cplx_t<T>* __restrict__ tw,
                                           int sgn, int tid, int nthr) {
  fft_stage<T, 30, R>(sm, ld, n, p, E, cshift, tw, sgn, tid, nthr);
}

// Schedule classes (compile-time):
//   kSchedGen  mixed radix 2/3/4/5/8 stages chosen at run time, E <= 30;
//   kSchedP2   powers of two >= 16: radix-16 stages then one tail stage of
//              radix RT (1 = no tail), E = 16.
constexpr int kSchedGen = 0;
template <int RT> struct SchedP2 { static constexpr int tail = RT; };

// Transforms all columns of the tile in place.  sgn = -1 forward, +1 inverse.
// Requires nthr == ncols * n / E and ncols == 1 << cshift.
// SCHED: 0 = mixed radix; 1, 2, 4, 8 = power of two with that tail radix.
template <typename T, int SCHED>
__device__ __forceinline__ void fft_tile(cplx_t<T>* sm, int ld, const LinePlan<T>& pl,
                                         int cshift, int sgn, int tid, int nthr) {
  if constexpr (SCHED == kSchedGen) {
    int p = 1;
    for (int s = 0; s < pl.nst; ++s) {
      int R = pl.radix[s];
      switch (R) {
        case 2: fft_stage_gen<T, 2>(sm, ld, pl.n, p, pl.E, cshift, pl.tw, sgn, tid, nthr); break;
        case 3: fft_stage_gen<T, 3>(sm, ld, pl.n, p, pl.E, cshift, pl.tw, sgn, tid, nthr); break;
        case 4: fft_stage_gen<T, 4>(sm, ld, pl.n, p, pl.E, cshift, pl.tw, sgn, tid, nthr); break;
        case 5: fft_stage_gen<T, 5>(sm, ld, pl.n, p, pl.E, cshift, pl.tw, sgn, tid, nthr); break;
        default: fft_stage_gen<T, 8>(sm, ld, pl.n, p, pl.E, cshift, pl.tw, sgn, tid, nthr); break;
      }
      p *= R;
    }
  } else {
    int p = 1;
    const int n16 = pl.nst - (SCHED > 1 ? 1 : 0);
    for (int s = 0; s < n16; ++s) {
      fft_stage<T, 16, 16>(sm, ld, pl.n, p, 16, cshift, pl.tw, sgn, tid, nthr);
      p *= 16;
    }
    if constexpr (SCHED > 1)
      fft_stage<T, 16, SCHED>(sm, ld, pl.n, p, 16, cshift, pl.tw, sgn, tid, nthr);
  }
}

// Schedule class of a line plan (host and device).
template <typename T>
__host__ __device__ inline int sched_of(const LinePlan<T>& pl) {
  if (pl.E != 16) return kSchedGen;
  for (int s = 0; s + 1 < pl.nst; ++s)
    if (pl.radix[s] != 16) return kSchedGen;
  int last = pl.nst > 0 ? pl.radix[pl.nst - 1] : 16;
  return last == 16 ? 1 : last;
}

// ---------------------------------------------------------------------------
// Host-side plan description for a 3-D real transform of (nx, ny, nz).
// The internal half-spectrum layout used between passes is "split Nyquist":
//   main[x][y][kz] for kz in [0, nz/2)   (row length h = nz/2)
//   nyq [x][y]     for kz = nz/2
// which keeps every main row a whole number of 16-column tiles.
template <typename T>
struct Plan3 {
  int nx, ny, nz, h;
  LinePlan<T> px, py, pz;     // lengths nx, ny, h
  const cplx_t<T>* twr;       // h+1 entries exp(-2 pi i k / nz), r2c split
};

// Returns the cached plan for (nx, ny, nz) on the current device, building
// it if needed (build == true).  Returns an error status otherwise.
template <typename T>
int get_plan3(int nx, int ny, int nz, bool build, Plan3<T>* out);

// Chooses the CTA column count for length n with E elements per thread.
int tile_cols(int n, int E, size_t elem_bytes);

}  // namespace jld
