// passes.cuh -- the fused line passes of one Strang step.
//
// A reference step (src/strang_splitting.jl:86-90) is
//   half(t+dt/2, dt/2) ; FFT ; * exp(-i dt D(k)) ; iFFT ; half(t+dt, dt/2)
// with the real-space half step of src/kernels.jl:37-54.  Here a 2D step is two
// passes over HBM, each reading and writing the field once:
//   row pass    : [iFFT_x] [half A] [save] [half B] [FFT_x]   (lines along x)
//   column pass : FFT_y  * table(k)  iFFT_y                    (tiles of CC columns)
// Between steps the state stays x-transformed, so the trailing half of step k and
// the leading half of step k+1 share one row pass.  In 1D a line is the whole
// field, so one resident kernel runs many steps without touching HBM.
//
// Three precisions share the code: double (native FP64), float (FP32) and DWR
// (double-word FP64 on the FP32 pipes, dw.cuh).
#pragma once
#include "fft.cuh"
#include "kernels.h"
#include "philox.cuh"
#include "tma.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <climits>

namespace gpe {

__host__ __device__ constexpr int cmin(int a, int b) { return a < b ? a : b; }
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int pow2floor(int v) { return v <= 1 ? 1 : 2 * pow2floor(v / 2); }

// Tiling of a line of 2^LOGN points for precision Real and M components.  V selects an
// alternative tiling where one exists (FP32, one component: V=1 holds 8 points a thread
// in the row pass and 16 in the column pass instead of 16 and 8); the ensemble
// autotuner picks V per grid size.
template <typename Real, int M, int LOGN, int V = 0>
struct LineCfg {
  using C = typename CT<Real>::T;
  static constexpr int N = 1 << LOGN;
  // points per thread: column pass (E) and row pass (ER, which also carries the
  // pointwise half steps and so keeps fewer points live).  FP32 column passes use 8 so
  // two CTAs share an SM and one's loads overlap the other's FFTs.
  static constexpr bool ALT = V == 1 && sizeof(C) == 8 && M == 1;
  // V=2: fine tiling for fields too small to fill the GPU (4 points a thread in both
  // passes: twice the threads of the default at the price of more radix-4 stages)
  static constexpr bool FINE = V == 2;
// one-component 16-byte lines: 8 points a thread in both passes (1024^2 Kerr, 16 copies:
// 1.141 ms per step against 1.174 ms with 16 / 16, 1.154 with 8 / 16, 1.156 with 16 / 8)
#ifndef GPE_E_W16_M1
#define GPE_E_W16_M1 8
#endif
#ifndef GPE_ER_W16_M1
#define GPE_ER_W16_M1 8
#endif
  static constexpr int EMAX = FINE ? 4 : ALT ? 16 : ((sizeof(C) == 16 && M == 2) || sizeof(C) == 8 ? 8 : GPE_E_W16_M1);
  static constexpr int E = cmin(EMAX, N / 2);
  static constexpr int T = N / E;  // threads per line, column pass
#ifndef GPE_ER_F32
#define GPE_ER_F32 8
#endif
  static constexpr int ERMAX = FINE ? 4 : ALT ? 8 : ((M == 2) ? (sizeof(C) == 8 ? GPE_ER_F32 : 8) : (sizeof(C) == 16 ? GPE_ER_W16_M1 : 16));
  static constexpr int ER = cmin(ERMAX, N / 2);
  static constexpr int TR = N / ER;  // threads per line, row pass
#ifndef GPE_ROWT_W16
#define GPE_ROWT_W16 256
#endif
  static constexpr int ROWT = sizeof(C) == 16 ? GPE_ROWT_W16 : 256;
  static constexpr int L = TR >= ROWT ? 1 : ROWT / TR;  // lines per row-pass block
  static constexpr int CCMAX = 128 / (int)sizeof(C);  // columns per tile: one 128-byte row
#ifndef GPE_COL_TPB_M2
#define GPE_COL_TPB_M2 512
#endif
  // 16-byte two-component column tiles: 256 threads (4 columns), two CTAs per SM
  // (polariton 512^2 double-word: 0.796 ms against 0.825 ms with one CTA of 512)
#ifndef GPE_COL_TPB_W16_M2
#define GPE_COL_TPB_W16_M2 256
#endif
  static constexpr int TPB = (M == 2) ? (sizeof(C) == 16 ? GPE_COL_TPB_W16_M2 : GPE_COL_TPB_M2) : 1024;
  static constexpr int SMEM_LIMIT = 200 * 1024;
  // FP32 lines of two components transform jointly (each component its own exchange)
  static constexpr bool JOINT = sizeof(C) == 8 && M == 2;
  static constexpr int NPAD = sizeof(C) == 8 ? N + N / 8 : N;  // rows of a column exchange (ColLayout)
  static constexpr int CC = cmax(1, cmin(cmin(CCMAX, cmax(1, TPB / T)),
                                         pow2floor(SMEM_LIMIT / (NPAD * (int)sizeof(C) * (JOINT ? M : 1)))));
  static constexpr int ROW_THREADS = L * TR;
#ifndef GPE_ROW_MIN_BLOCKS
#define GPE_ROW_MIN_BLOCKS 2
#endif
#ifndef GPE_ROW_MIN_BLOCKS_F32
#define GPE_ROW_MIN_BLOCKS_F32 3
#endif
  // blocks of more than 256 threads (lines of 4096 points) keep 128 registers a thread
  static constexpr int ROW_MINB = L * TR > 256 ? 1 : (sizeof(C) == 8 ? GPE_ROW_MIN_BLOCKS_F32 : GPE_ROW_MIN_BLOCKS);
#ifndef GPE_COL_MINB_F32
#define GPE_COL_MINB_F32 2
#endif
#ifndef GPE_COL_MINB_W16_M2
#define GPE_COL_MINB_W16_M2 2
#endif
  static constexpr int COL_MINB_WANT = sizeof(C) == 8 ? GPE_COL_MINB_F32 : (M == 2 ? GPE_COL_MINB_W16_M2 : 1);
  static constexpr int COL_THREADS = CC * T;
  static constexpr int COL_MINB = COL_THREADS * COL_MINB_WANT <= 2048 ? COL_MINB_WANT : 1;
  static constexpr size_t ROW_SMEM = (size_t)L * N * sizeof(C);
  static constexpr size_t ROW_KERNEL_SMEM = JOINT ? (size_t)M * L * N * sizeof(C) : ROW_SMEM;
  static constexpr size_t COL_SMEM = (size_t)(JOINT ? M : 1) * CC * NPAD * sizeof(C);
};

// ------------------------------------------------------------------ scalar helpers
template <typename Real> __device__ __forceinline__ void sc(Real x, Real* s, Real* c);
// FP64 sin/cos of the nonlinear phase.  FP64 runs at 1/64 of the FP32 rate on GB300, so
// small angles (the usual case: |dt/2 * G| << 1) use the Taylor series through x^9 / x^10
// for |x| < 1/8 (the first dropped terms below 3e-17 relative and 3e-20): 12 FP64
// operations, a fraction of the general routine, which handles the rest.  The interval is
// picked from the high word of x on the integer pipe.  One polynomial, not a ladder of
// shorter ones: the compiler evaluates the rungs of a ladder both and selects.
template <> __device__ __forceinline__ void sc<double>(double x, double* s, double* c) {
  if ((__double2hiint(x) & 0x7fffffff) < 0x3fc00000) {  // |x| < 1/8
    const double x2 = x * x;
    *c = fma(x2, fma(x2, fma(x2, fma(x2, fma(x2, -1.0 / 3628800, 1.0 / 40320), -1.0 / 720), 1.0 / 24), -0.5), 1.0);
    *s = x * fma(x2, fma(x2, fma(x2, fma(x2, 1.0 / 362880, -1.0 / 5040), 1.0 / 120), -1.0 / 6), 1.0);
  } else {
    sincos(x, s, c);
  }
}
// FP32: small angles (|x| <= 1/8, truncation below x^9/9! < 1e-14) by the Taylor series,
// a dozen FMAs instead of the general routine's range reduction.
template <> __device__ __forceinline__ void sc<float>(float x, float* s, float* c) {
  if (fabsf(x) <= 0.125f) {
    const float x2 = x * x;
    *c = 1.0f + x2 * (-0.5f + x2 * (1.0f / 24 + x2 * (-1.0f / 720 + x2 * (1.0f / 40320))));
    *s = x * (1.0f + x2 * (-1.0f / 6 + x2 * (1.0f / 120 + x2 * (-1.0f / 5040))));
  } else {
    sincosf(x, s, c);
  }
}
// FP32 sin x and cos x - 1.  The nonlinear phase factor is applied to FP32 fields as
// u + (E - 1) u with E - 1 = (cos - 1) - i sin formed without the leading 1: rounded near
// 1, cos carries an error of up to 3e-8 that depends smoothly on x, so it does not average
// out over a smooth field, and |E|^2 - 1 of that size would bias the norm every half step.
__device__ __forceinline__ void sc_m1(float x, float* s, float* cm1) {
  if (fabsf(x) <= 0.125f) {
    const float x2 = x * x;
    *cm1 = x2 * (-0.5f + x2 * (1.0f / 24 + x2 * (-1.0f / 720 + x2 * (1.0f / 40320))));
    *s = x * (1.0f + x2 * (-1.0f / 6 + x2 * (1.0f / 120 + x2 * (-1.0f / 5040))));
  } else {
    float c;
    sincosf(x, s, &c);
    *cm1 = c - 1.0f;
  }
}
__device__ __forceinline__ double rexp(double x) { return exp(x); }
__device__ __forceinline__ float rexp(float x) { return expf(x); }

// Double-word sin/cos.  |x| <= 1/8: cos = 1 - x^2/2 + x^4/24 + tail, sin = x (1 - x^2/6 +
// x^4/120 + tail) with the double-word leading terms and the tails (below 6e-9 and
// 8e-10) summed in FP32, which keeps the result within a few units of 2^-48 (for
// |x| <= 2^-6 the x^4 terms join the FP32 tails).  Larger angles go through the FP64
// routine.
__device__ __forceinline__ void dw_sincos(dw x, dw& s, dw& c) {
  if (fabsf(x.h) <= 0.125f) {
    const dw x2 = dw_mul(x, x);
    const float t = x2.h;
    const float t3 = t * t * t;
    const float tc = t3 * (-1.0f / 720 + t * (1.0f / 40320 + t * (-1.0f / 3628800 + t * (1.0f / 479001600))));
    const float ts = t3 * (-1.0f / 5040 + t * (1.0f / 362880 + t * (-1.0f / 39916800 + t * (1.0f / 6227020800.0f))));
    if (t <= 0x1p-12f) {
      // |x| <= 2^-6: x^4/24 <= 2.5e-9 and x^4/120 <= 5e-10, so FP32 carries them (and
      // the tails) to well inside 2^-48 absolute; only 1 - x^2/2 and 1 - x^2/6 need
      // double-word sums
      c = dw_add(dw_add({1.0f, 0.0f}, {-0.5f * x2.h, -0.5f * x2.l}), {t * t * (1.0f / 24) + tc, 0.0f});
      dw ss = dw_add({1.0f, 0.0f}, dw_neg(dw_mul(x2, {dwh(1.0 / 6), dwl(1.0 / 6)})));
      ss = dw_add(ss, {t * t * (1.0f / 120) + ts, 0.0f});
      s = dw_mul(x, ss);
      return;
    }
    const dw q = dw_mul(x2, x2);
    // every partial sum stays within [0.99, 1] (x^2 <= 1/64): no cancellation, so the
    // sloppy double-word sum keeps its relative bound
    dw cc = dw_add({1.0f, 0.0f}, {-0.5f * x2.h, -0.5f * x2.l});
    cc = dw_add(cc, dw_mul(q, {dwh(1.0 / 24), dwl(1.0 / 24)}));
    c = dw_add(cc, {tc, 0.0f});
    dw ss = dw_add({1.0f, 0.0f}, dw_neg(dw_mul(x2, {dwh(1.0 / 6), dwl(1.0 / 6)})));
    ss = dw_add(ss, dw_mul(q, {dwh(1.0 / 120), dwl(1.0 / 120)}));
    ss = dw_add(ss, {ts, 0.0f});
    s = dw_mul(x, ss);
  } else {
    double sd, cd;
    sincos(dw_to_double(x), &sd, &cd);
    s = dw_from(sd);
    c = dw_from(cd);
  }
}

// Typed views of the coefficient block.
template <typename Real> struct Coef;
template <> struct Coef<double> {
  __device__ static __forceinline__ double g(const PassArgs& a, int j, int l, int r) { return a.g[j][l][r]; }
  __device__ static __forceinline__ double c(const PassArgs& a, int j, int r) { return a.c[j][r]; }
  __device__ static __forceinline__ double nf(const PassArgs& a, int j, int r) { return a.nfac[j][r]; }
  __device__ static __forceinline__ double dth(const PassArgs& a) { return 0.5 * a.dt; }
};
template <> struct Coef<float> {
  __device__ static __forceinline__ float g(const PassArgs& a, int j, int l, int r) { return a.gf[j][l][r]; }
  __device__ static __forceinline__ float c(const PassArgs& a, int j, int r) { return a.cf[j][r]; }
  __device__ static __forceinline__ float nf(const PassArgs& a, int j, int r) { return a.nfacf[j][r]; }
  __device__ static __forceinline__ float dth(const PassArgs& a) { return a.dthf; }
};

// real profile value at p (pump or noise profile), stored as Real / Real / dw
template <typename Real> struct Prof;
template <> struct Prof<double> {
  __device__ static __forceinline__ double2 cplx(const void* base, int64_t p) { return make_double2(__ldg((const double*)base + p), 0.0); }
};
template <> struct Prof<float> {
  __device__ static __forceinline__ float2 cplx(const void* base, int64_t p) { return make_float2(__ldg((const float*)base + p), 0.0f); }
};
template <> struct Prof<DWR> {
  __device__ static __forceinline__ dwc cplx(const void* base, int64_t p) {
    const float2 v = __ldg((const float2*)base + p);
    dwc z; z.xh = v.x; z.xl = v.y; z.yh = 0.0f; z.yl = 0.0f;
    return z;
  }
};

// coef * profile for a pump term: a real profile (the usual case) scales the complex
// coefficient, two real multiplies instead of a complex product
__device__ __forceinline__ float rpart(const float2& z) { return z.x; }
__device__ __forceinline__ double rpart(const double2& z) { return z.x; }
__device__ __forceinline__ dw rpart(const dwc& z) { return re(z); }
template <typename C> __device__ __forceinline__ C pump_mul(const C& coef, const C& prof, int cplx) {
  return cplx ? cmul(coef, prof) : cscale(coef, rpart(prof));
}
// u + coef * prof.  FP64: one complex multiply-add whatever the profile (a real profile is
// loaded with a zero imaginary part), four FMAs; choosing between the real and complex
// forms at run time makes the compiler evaluate both and select.
template <typename C> __device__ __forceinline__ C pump_add(const C& u, const C& coef, const C& prof, int cplx) {
  return cadd(u, pump_mul(coef, prof, cplx));
}
__device__ __forceinline__ double2 pump_add(const double2& u, const double2& coef, const double2& prof, int) {
  double2 r;
  r.x = fma(coef.x, prof.x, fma(-coef.y, prof.y, u.x));
  r.y = fma(coef.y, prof.x, fma(coef.x, prof.y, u.y));
  return r;
}

// complex normal deviate in the pass precision
template <typename Real> struct Xi;
template <> struct Xi<double> {
  __device__ static __forceinline__ double2 get(uint32_t w0, uint32_t w1) { return box_muller_f64(w0, w1); }
};
template <> struct Xi<float> {
  __device__ static __forceinline__ float2 get(uint32_t w0, uint32_t w1) { return box_muller_f32(w0, w1); }
};
template <> struct Xi<DWR> {
  __device__ static __forceinline__ dwc get(uint32_t w0, uint32_t w1) {
    const double2 v = box_muller_f64(w0, w1);
    return mk(dw_from(v.x), dw_from(v.y));
  }
};

template <typename C> __device__ __forceinline__ C czero() {
  C z;
  memset(&z, 0, sizeof z);
  return z;
}
// 1 + 0i in the pass precision
__device__ __forceinline__ float2 cunit_(float2*) { return make_float2(1.0f, 0.0f); }
__device__ __forceinline__ double2 cunit_(double2*) { return make_double2(1.0, 0.0); }
__device__ __forceinline__ dwc cunit_(dwc*) { return mk(dw{1.0f, 0.0f}, dw{0.0f, 0.0f}); }
template <typename C> __device__ __forceinline__ C cunit() { return cunit_((C*)nullptr); }

// Phase tables (k-space exp(-i dt D)/P, real-space exp(-i dt/2 V)) keep FP64 accuracy in
// every precision: FP64 passes read double2, double-word and FP32 passes read hi/lo float
// pairs (t = hi + lo, 16 bytes, the double-word layout).  FP32 passes apply such a table
// entry to an FP32 value with FMA corrections, so the product is the FP32 rounding of the
// product with the FP64 entry (within a few units of the last place, unbiased) -- as the
// reference's ComplexF32 path, where the ComplexF64 table promotes the product to FP64
// before it is stored in FP32 (src/misc.jl:16, src/kernels.jl:44-53).  A table rounded
// to FP32 instead would carry a fixed error per entry that every step repeats.
template <typename Real> struct TabT { using T = dwc; };
template <> struct TabT<double> { using T = double2; };
__device__ __forceinline__ double2 tmul(const double2& t, const double2& v) { return cmul(t, v); }
__device__ __forceinline__ dwc tmul(const dwc& t, const dwc& v) { return cmul(t, v); }
__device__ __forceinline__ float2 tmul(const dwc& t, const float2& v) { return cmul_hl(v, t); }

// whether half_step applies component j's two pump terms as one (no E multiplies it)
__device__ __forceinline__ bool pump_merged(const PassArgs& a, int j) {
  return !a.nl_on[j] && a.vkind == TAB_NONE;
}

// Pump coefficients (dt/4) a(t_h) and (dt/4) a(t_{h+1}) for half step h.  merge: a
// component that neither G nor V touches takes both pump terms in one product,
// (u + pn F) + px F = u + (pn + px) F, so px carries the sum (formed once here, not per
// point) and half_step applies it alone (the matrix family's half step applies pn and px
// on either side of its exponential and does not merge).
template <typename Real, int M>
__device__ __forceinline__ void load_pump(const PassArgs& a, int64_t h, typename CT<Real>::T (&pn)[M],
                                          typename CT<Real>::T (&px)[M], bool merge = false) {
  using C = typename CT<Real>::T;
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if (a.pprof[j] && h >= 0) {
      const int64_t n = a.pcoef_n[j];
      const C* pc = (const C*)a.pcoef[j];
      pn[j] = n == 1 ? ldgc(pc) : ldgc(pc + (h < n ? h : n - 1));
      px[j] = n == 1 ? pn[j] : ldgc(pc + (h + 1 < n ? h + 1 : n - 1));
      if (merge && pump_merged(a, j)) px[j] = cadd(pn[j], px[j]);
    } else {
      pn[j] = czero<C>();
      px[j] = pn[j];
    }
  }
}

// xi for half step h at point p of trajectory b (Philox or replayed).  Philox blocks:
// with two components the point's own block, words (0,1) and (2,3); with one component
// the points x and x + n0/2 of a row share the block of the lower one (words (0,1) for
// it, (2,3) for the upper one), so no draw is wasted.
template <typename Real, int M>
__device__ __forceinline__ void draw_xi(const PassArgs& a, int64_t p, int64_t b, int64_t h,
                                        typename CT<Real>::T (&xi)[M]) {
  using C = typename CT<Real>::T;
  if (a.noise == NOISE_PHILOX) {
    if constexpr (M == 1) {
      const int64_t hx = a.n0 >> 1;
      const bool up = (p & (a.n0 - 1)) >= hx;
      const uint4 r = Philox4x32::gen(noise_counter(up ? p - hx : p, b + a.traj0, h), a.seed_lo, a.seed_hi);
      xi[0] = Xi<Real>::get(up ? r.z : r.x, up ? r.w : r.y);
    } else {
      const uint4 r = Philox4x32::gen(noise_counter(p, b + a.traj0, h), a.seed_lo, a.seed_hi);
      xi[0] = Xi<Real>::get(r.x, r.y);
      xi[M - 1] = Xi<Real>::get(r.z, r.w);
    }
  } else {
    const C* xb = (const C*)a.xi;
#pragma unroll
    for (int j = 0; j < M; ++j) xi[j] = xb[((h - a.xi_h0) * M + j) * a.B * a.P + b * a.P + p];
  }
}

// exp(-i delta G) for a 2x2 complex matrix G (row-major g[4] as (re, im)), FP64:
// e^{tr/2} [cosh(s) I + sinh(s)/s (A - tr/2 I)], A = -i delta G, s^2 = ((a-d)/2)^2 + bc,
// with the series 1 + s^2/6 + s^4/120 for sinh(s)/s when |s| < 1e-3.
struct cd2 {
  double x, y;
};
__device__ __forceinline__ cd2 cdmul(cd2 a, cd2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cd2 cdadd(cd2 a, cd2 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cd2 cdsub(cd2 a, cd2 b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cd2 cdsqrt(cd2 z) {
  const double r = hypot(z.x, z.y);
  if (r == 0.0) return {0.0, 0.0};
  const double t = sqrt(0.5 * (r + fabs(z.x)));
  return z.x >= 0.0 ? cd2{t, z.y / (2.0 * t)} : cd2{fabs(z.y) / (2.0 * t), copysign(t, z.y)};
}
__device__ inline void expm2_dev(const cd2 (&G)[4], double delta, cd2 (&E)[4]) {
  cd2 A[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) A[q] = {delta * G[q].y, -delta * G[q].x};  // -i delta G
  const cd2 ht = {0.5 * (A[0].x + A[3].x), 0.5 * (A[0].y + A[3].y)};
  const cd2 hd = {0.5 * (A[0].x - A[3].x), 0.5 * (A[0].y - A[3].y)};
  const cd2 s = cdsqrt(cdadd(cdmul(hd, hd), cdmul(A[1], A[2])));
  double sh_, ch_, sn, cs;
  sincos(s.y, &sn, &cs);
  sh_ = sinh(s.x);
  ch_ = cosh(s.x);
  const cd2 chs = {ch_ * cs, sh_ * sn};
  cd2 shs;
  if (hypot(s.x, s.y) < 1e-3) {
    const cd2 s2 = cdmul(s, s);
    const cd2 s4 = cdmul(s2, s2);
    shs = {1.0 + s2.x / 6.0 + s4.x / 120.0, s2.y / 6.0 + s4.y / 120.0};
  } else {
    const cd2 sinhs = {sh_ * cs, ch_ * sn};
    const double den = s.x * s.x + s.y * s.y;
    shs = {(sinhs.x * s.x + sinhs.y * s.y) / den, (sinhs.y * s.x - sinhs.x * s.y) / den};
  }
  double es, ec;
  sincos(ht.y, &es, &ec);
  const double em = exp(ht.x);
  const cd2 e = {em * ec, em * es};
  E[0] = cdmul(e, cdadd(chs, cdmul(shs, cdsub(A[0], ht))));
  E[3] = cdmul(e, cdadd(chs, cdmul(shs, cdsub(A[3], ht))));
  E[1] = cdmul(e, cdmul(shs, A[1]));
  E[2] = cdmul(e, cdmul(shs, A[2]));
}

template <typename C> __device__ __forceinline__ cd2 to_cd2(const C& v) { return {(double)v.x, (double)v.y}; }
template <> __device__ __forceinline__ cd2 to_cd2<dwc>(const dwc& v) { return {dw_to_double(re(v)), dw_to_double(im(v))}; }
template <typename C> __device__ __forceinline__ C from_cd2(cd2 v) { C r; r.x = v.x; r.y = v.y; return r; }
template <> __device__ __forceinline__ dwc from_cd2<dwc>(cd2 v) { return mk(dw_from(v.x), dw_from(v.y)); }

// E = exp(-i delta G(u)) V at one point for the matrix family, V the potential table entry
// (scalar or 2x2; none when vkind is neither), evaluated in FP64 for every pass precision.
template <typename Real>
__device__ __forceinline__ void matrix_phase(const typename CT<Real>::T (&u)[2], const PassArgs& a, int64_t p,
                                             typename CT<Real>::T (&Em)[4]) {
  using C = typename CT<Real>::T;
  const cd2 v0 = to_cd2(u[0]), v1 = to_cd2(u[1]);
  const double d0 = v0.x * v0.x + v0.y * v0.y, d1 = v1.x * v1.x + v1.y * v1.y;
  cd2 G[4], E[4];
#pragma unroll
  for (int ab = 0; ab < 4; ++ab) {
    const double* g = a.nlm + 4 * ab;
    const double* c = a.nlm + 16 + 2 * ab;
    G[ab] = {__ldg(c) + __ldg(g) * d0 + __ldg(g + 2) * d1, __ldg(c + 1) + __ldg(g + 1) * d0 + __ldg(g + 3) * d1};
  }
  expm2_dev(G, 0.5 * a.dt, E);
  using TT = typename TabT<Real>::T;
  if (a.vkind == TAB_SCALAR) {
    const cd2 v = to_cd2(ldgc((const TT*)a.vtab + p));
#pragma unroll
    for (int q = 0; q < 4; ++q) E[q] = cdmul(E[q], v);
  } else if (a.vkind == TAB_MATRIX) {
    cd2 V[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) V[q] = to_cd2(ldgc((const TT*)a.vtab + (int64_t)q * a.P + p));
    const cd2 r0 = cdadd(cdmul(E[0], V[0]), cdmul(E[1], V[2]));
    const cd2 r1 = cdadd(cdmul(E[0], V[1]), cdmul(E[1], V[3]));
    const cd2 r2 = cdadd(cdmul(E[2], V[0]), cdmul(E[3], V[2]));
    const cd2 r3 = cdadd(cdmul(E[2], V[1]), cdmul(E[3], V[3]));
    E[0] = r0;
    E[1] = r1;
    E[2] = r2;
    E[3] = r3;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) Em[q] = from_cd2<C>(E[q]);
}

//   u <- cis(-delta G(u)) V (u + delta/2 F_now) + delta/2 F_next - i sqrt(delta) eta xi
// G is evaluated on u before the pump is added (src/kernels.jl:40,44).
// pn/px: pump coefficients (dt/4)a(t_h), (dt/4)a(t_{h+1}).
template <typename Real, int M>
__device__ __forceinline__ void half_step(typename CT<Real>::T (&u)[M], const PassArgs& a,
                                          int64_t p, int64_t b, int64_t h,
                                          const typename CT<Real>::T (&pn)[M],
                                          const typename CT<Real>::T (&px)[M],
                                          const typename CT<Real>::T* xi_pre = nullptr) {
  using C = typename CT<Real>::T;
  C E[M];
  bool hasE[M];
  if constexpr (std::is_same<Real, DWR>::value) {
    dw dens[M];
#pragma unroll
    for (int l = 0; l < M; ++l)
      dens[l] = ((a.dens_mask >> l) & 1) ? dot2<+1>(re(u[l]), re(u[l]), im(u[l]), im(u[l])) : dw{0.0f, 0.0f};
    const dw dth = {a.dthf, a.dthl};
#pragma unroll
    for (int j = 0; j < M; ++j) {
      hasE[j] = a.nl_on[j] != 0;
      if (hasE[j]) {
        // sum of the nonzero terms, starting from the first one when c_j is zero (the
        // usual case) rather than adding it to zero
        dw gr = {a.cf[j][0], a.cl[j][0]};
        bool empty = a.cf[j][0] == 0.0f && a.cl[j][0] == 0.0f;
#pragma unroll
        for (int l = 0; l < M; ++l)
          if (a.gf[j][l][0] != 0.0f || a.gl[j][l][0] != 0.0f) {
            const dw term = dw_mul({a.gf[j][l][0], a.gl[j][l][0]}, dens[l]);
            if (empty) gr = term;
            else gr = dw_add_acc(gr, term);
            empty = false;
          }
        dw s, c;
        dw_sincos(dw_mul(dth, gr), s, c);
        if (a.nl_imag[j]) {
          dw gi = {a.cf[j][1], a.cl[j][1]};
#pragma unroll
          for (int l = 0; l < M; ++l)
            if (a.gf[j][l][1] != 0.0f || a.gl[j][l][1] != 0.0f)
              gi = dw_add_acc(gi, dw_mul({a.gf[j][l][1], a.gl[j][l][1]}, dens[l]));
          const dw mag = dw_from(exp(dw_to_double(dw_mul(dth, gi))));
          s = dw_mul(s, mag);
          c = dw_mul(c, mag);
        }
        E[j] = mk(c, dw_neg(s));
      }
    }
  } else {
    using K = Coef<Real>;
    [[maybe_unused]] const Real dth = K::dth(a);
    // only the densities some active G_j uses, and only the nonzero coefficients (uniform
    // branches on host-made bit masks, so no FP64 compare; adding a zero term would not
    // change the sum): the polariton's G_2 = g |u_2|^2 costs one density and one product
    // instead of two of each
    Real dens[M];
#pragma unroll
    for (int l = 0; l < M; ++l) dens[l] = ((a.dens_mask >> l) & 1) ? u[l].x * u[l].x + u[l].y * u[l].y : (Real)0;
#pragma unroll
    for (int j = 0; j < M; ++j) {
      hasE[j] = a.nl_on[j] != 0;
      if (hasE[j]) {
        if constexpr (std::is_same<Real, double>::value) {
          // the phase dt/2 G from the dt/2-scaled coefficients, one FMA a nonzero term
          double pr = ((a.c_nz >> (j * 2)) & 1) ? a.cd[j][0] : 0.0;
          double pi = ((a.c_nz >> (j * 2 + 1)) & 1) ? a.cd[j][1] : 0.0;
#pragma unroll
          for (int l = 0; l < M; ++l) {
            if ((a.g_nz >> (j * 4 + l * 2)) & 1) pr = fma(a.gd[j][l][0], dens[l], pr);
            if ((a.g_nz >> (j * 4 + l * 2 + 1)) & 1) pi = fma(a.gd[j][l][1], dens[l], pi);
          }
          double s, c;
          sc<double>(pr, &s, &c);
          if (a.nl_imag[j]) {
            const double mag = exp(pi);
            E[j].x = mag * c;
            E[j].y = -mag * s;
          } else {
            E[j].x = c;
            E[j].y = -s;
          }
          continue;
        }
        Real gr = K::c(a, j, 0), gi = K::c(a, j, 1);
#pragma unroll
        for (int l = 0; l < M; ++l) {
          if ((a.g_nz >> (j * 4 + l * 2)) & 1) gr += K::g(a, j, l, 0) * dens[l];
          if ((a.g_nz >> (j * 4 + l * 2 + 1)) & 1) gi += K::g(a, j, l, 1) * dens[l];
        }
        if constexpr (std::is_same<Real, float>::value) {
          // E - 1 (see sc_m1): mag cos - 1 = (mag - 1) + mag (cos - 1)
          float s, cm1;
          sc_m1(dth * gr, &s, &cm1);
          if (a.nl_imag[j]) {
            const float em1 = expm1f(dth * gi), mag = 1.0f + em1;
            E[j].x = __fmaf_rn(mag, cm1, em1);
            E[j].y = -mag * s;
          } else {
            E[j].x = cm1;
            E[j].y = -s;
          }
        } else {
          Real s, c;
          sc<Real>(dth * gr, &s, &c);
          if (a.nl_imag[j]) {
            const Real mag = rexp(dth * gi);
            E[j].x = mag * c;
            E[j].y = -mag * s;
          } else {  // a real G: no magnitude factor to multiply in
            E[j].x = c;
            E[j].y = -s;
          }
        }
      }
    }
  }
  // real-space table.  FP64 and double-word passes fold it into E (E = cis(-delta G) V,
  // the reference's order); FP32 passes apply it as its own FMA-corrected product after
  // cis(-delta G), so it keeps its FP64 accuracy (an FP32 E V would round it)
  using TT = typename TabT<Real>::T;
  constexpr bool SEPV = std::is_same<Real, float>::value;
  TT vt[SEPV ? M : 1];
  const bool hasV = SEPV && (a.vkind == TAB_SCALAR || a.vkind == TAB_DIAG);
  if (a.vkind == TAB_SCALAR || a.vkind == TAB_DIAG) {
#pragma unroll
    for (int j = 0; j < M; ++j) {
      const TT v = ldgc((const TT*)a.vtab + (a.vkind == TAB_DIAG ? (int64_t)j * a.P : 0) + p);
      if constexpr (SEPV) {
        vt[j] = v;
      } else {
        E[j] = hasE[j] ? cmul(E[j], v) : v;
        hasE[j] = true;
      }
    }
  }
  C prof[M];
  // a component that neither G nor V touches takes both pump terms in one product:
  // (u + pn F) + px F = u + (pn + px) F
  bool pm[M];
#pragma unroll
  for (int j = 0; j < M; ++j) pm[j] = pump_merged(a, j);  // = !hasE[j] && vkind != MATRIX
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if (a.pprof[j]) {
      prof[j] = ((a.pump_uniform >> j) & 1) ? cunit<C>()
                : a.pprof_cplx ? ldgc((const C*)a.pprof[j] + p) : Prof<Real>::cplx(a.pprof[j], p);
      if (!pm[j]) u[j] = pump_add(u[j], pn[j], prof[j], a.pprof_cplx);
    }
  }
  if (a.vkind == TAB_MATRIX && M == 2) {
    // matrix potential with no nonlinearity: mat-vec with the per-point 2x2 table
    const TT* mt = (const TT*)a.vtab;
    const TT t00 = ldgc(mt + p), t01 = ldgc(mt + a.P + p);
    const TT t10 = ldgc(mt + 2 * a.P + p), t11 = ldgc(mt + 3 * a.P + p);
    const C y0 = cadd(tmul(t00, u[0]), tmul(t01, u[M - 1]));
    const C y1 = cadd(tmul(t10, u[0]), tmul(t11, u[M - 1]));
    u[0] = y0;
    u[M - 1] = y1;
  } else {
#pragma unroll
    for (int j = 0; j < M; ++j) {
      if constexpr (SEPV) {
        if (hasE[j]) {
          // u + (E - 1) u with the whole increment formed first and added once: added in
          // two roundings, the small (cos - 1) u part is dropped whenever it is below half
          // a unit of the partly rotated value, and the rotation then grows the norm
          // (+1.7e-9 a half step on the Kerr sweep; added once, the growth is at rounding
          // level)
          const C v = u[j];
          const float dx = __fmaf_rn(E[j].x, v.x, -__fmul_rn(E[j].y, v.y));
          const float dy = __fmaf_rn(E[j].x, v.y, __fmul_rn(E[j].y, v.x));
          u[j].x = __fadd_rn(v.x, dx);
          u[j].y = __fadd_rn(v.y, dy);
        }
        if (hasV) u[j] = tmul(vt[j], u[j]);
      } else {
        if (hasE[j]) u[j] = cmul(E[j], u[j]);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < M; ++j)
    if (a.pprof[j]) u[j] = pump_add(u[j], px[j], prof[j], a.pprof_cplx);  // px: pn + px when merged
  if (a.noise != NOISE_OFF) {
    C xi[M];
    if (xi_pre) {
#pragma unroll
      for (int j = 0; j < M; ++j) xi[j] = xi_pre[j];
    } else {
      draw_xi<Real, M>(a, p, b, h, xi);
    }
#pragma unroll
    for (int j = 0; j < M; ++j) {
      C nf;
      if constexpr (std::is_same<Real, DWR>::value) {
        nf = mk({a.nfacf[j][0], a.nfacl[j][0]}, {a.nfacf[j][1], a.nfacl[j][1]});
        if (a.etaprof[j]) {
          const float2 e = __ldg((const float2*)a.etaprof[j] + p);
          nf = cscale(nf, dw{e.x, e.y});
        }
      } else {
        nf.x = Coef<Real>::nf(a, j, 0);
        nf.y = Coef<Real>::nf(a, j, 1);
        if (a.etaprof[j]) nf = cscale(nf, __ldg((const Real*)a.etaprof[j] + p));
      }
      u[j] = cadd(u[j], cmul(nf, xi[j]));
    }
  }
}

// k-space multiply of the M values at table index kp (src/strang_splitting.jl:73-74)
template <typename Real, int M>
__device__ __forceinline__ void kmul(typename CT<Real>::T (&v)[M], const PassArgs& a, int64_t kp) {
  using C = typename CT<Real>::T;
  using TT = typename TabT<Real>::T;
  const TT* kt = (const TT*)a.ktab;
  if (a.kkind == TAB_SCALAR) {
    const TT k = ldgc(kt + kp);
#pragma unroll
    for (int m = 0; m < M; ++m) v[m] = tmul(k, v[m]);
  } else if (a.kkind == TAB_DIAG) {
#pragma unroll
    for (int m = 0; m < M; ++m) v[m] = tmul(ldgc(kt + (int64_t)m * a.P + kp), v[m]);
  } else if (a.kkind == TAB_MATRIX) {
    if constexpr (M == 2) {
      const TT t00 = ldgc(kt + kp), t01 = ldgc(kt + a.P + kp);
      const TT t10 = ldgc(kt + 2 * a.P + kp), t11 = ldgc(kt + 3 * a.P + kp);
      if constexpr (std::is_same<Real, double>::value) {
        // each output as one chain of a product and three FMAs (16 FP64 operations for the
        // mat-vec instead of 20 as two complex products and a sum)
        const double2 x0 = v[0], x1 = v[1];
        v[0].x = t00.x * x0.x - t00.y * x0.y + t01.x * x1.x - t01.y * x1.y;
        v[0].y = t00.x * x0.y + t00.y * x0.x + t01.x * x1.y + t01.y * x1.x;
        v[1].x = t10.x * x0.x - t10.y * x0.y + t11.x * x1.x - t11.y * x1.y;
        v[1].y = t10.x * x0.y + t10.y * x0.x + t11.x * x1.y + t11.y * x1.x;
      } else {
        const C y0 = cadd(tmul(t00, v[0]), tmul(t01, v[1]));
        const C y1 = cadd(tmul(t10, v[0]), tmul(t11, v[1]));
        v[0] = y0;
        v[1] = y1;
      }
    } else {
      v[0] = tmul(ldgc(kt + kp), v[0]);
    }
  }
}

// Saved states are written in the caller's precision: a double-word state is rounded
// to FP64 (double2) on the way out.
template <typename Real>
__device__ __forceinline__ void store_save(void* base, int64_t idx, const typename CT<Real>::T& v) {
  if constexpr (std::is_same<Real, DWR>::value) {
    ((double2*)base)[idx] = make_double2(dw_to_double(re(v)), dw_to_double(im(v)));
  } else {
    ((typename CT<Real>::T*)base)[idx] = v;
  }
}

// Swap real and imaginary parts in place.  With s(z) = i conj(z), s o FFT o s equals
// conj o FFT o conj, the inverse transform: each kernel holds a single forward FFT
// instance, and the inverse costs register moves, no floating-point instruction (a
// negation under the run-time direction test could take an FP64 pipe slot).
template <typename C, int E>
__device__ __forceinline__ void swap_all(C (&x)[E]) {
#pragma unroll
  for (int i = 0; i < E; ++i) {
    if constexpr (std::is_same<C, dwc>::value) {
      const float h = x[i].xh, l = x[i].xl;
      x[i].xh = x[i].yh;
      x[i].xl = x[i].yl;
      x[i].yh = h;
      x[i].yl = l;
    } else {
      const auto r = x[i].x;
      x[i].x = x[i].y;
      x[i].y = r;
    }
  }
}

// Transform every component's line in place: forward (unnormalised) or inverse (the
// 1/P is folded into the k-space table).  One FFT instance serves all components and
// both directions: component 1 is swapped into the slot of component 0 and back.
// FXG > 0: FP64 lines may take the block floating point transform (fx_line; runtime switch
// fx), the threads of a line being spread with stride FXG (1 for row lines, the column
// count for column tiles); the Q62 twiddles follow the N FP64 ones in the table.
template <typename C, int N, int E, int M, class Lay, bool JOINT = false, int FXG = 0>
__device__ __forceinline__ void fft_components(C (&x)[M][E], bool inverse, int t, const Lay& lay,
                                               const typename TwT<C>::T* __restrict__ tw, int cstride = 0, bool renorm = true,
                                               bool fx = false) {
  if constexpr (JOINT) {
    // all components in one pass (FP32: the twiddle loads and barriers are shared)
    if (inverse) {
#pragma unroll
      for (int m = 0; m < M; ++m) swap_all(x[m]);
    }
    fft_line_joint<C, N, E, -1, M>(x, t, lay, cstride, tw);
    if (inverse) {
#pragma unroll
      for (int m = 0; m < M; ++m) swap_all(x[m]);
    }
  } else {
#pragma unroll 1
    for (int m = 0; m < M; ++m) {
      if (inverse) swap_all(x[0]);
      if constexpr (std::is_same<C, double2>::value && FXG > 0 && N > E) {
        if (fx) {
          using LF = typename Lay::template rebind<fxc>;
          fx_line<N, E, FXG>(x[0], t, LF{reinterpret_cast<fxc*>(lay.base)}, reinterpret_cast<const fxw*>(tw + N));
        } else {
          fft_line<C, N, E, -1>(x[0], t, lay, tw, renorm);
        }
      } else {
        fft_line<C, N, E, -1>(x[0], t, lay, tw, renorm);
      }
      if (inverse) swap_all(x[0]);
      if constexpr (M == 2) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
          const C tmp = x[0][i];
          x[0][i] = x[1][i];
          x[1][i] = tmp;
        }
      }
    }
  }
}

// ------------------------------------------------------------------ lean FP64 half steps
// The generic half step decides its families (potential, pump, noise, which components G
// touches) at run time.  Short conditional blocks are compiled to predicated code that
// issues whether or not it applies, so on the two-component polariton the row pass issued
// about 81 FP64 operations a point for two half steps that need 42 (ncu), on an FP64 pipe
// that runs at 1/64 of the FP32 rate.  The common families therefore get a half step whose
// families are template parameters -- GM: components with a (real) nonlinearity, DM: the
// densities it reads, PM: components with a real, non-uniform pump profile; no potential,
// no noise -- chosen by the host (PassArgs::lean).  Its arithmetic is the generic half
// step's operation for operation (src/kernels.jl:37-54): G on u, u + dt/4 a(t_h) p, the
// phase cis(-dt/2 G) (sc<double>), + dt/4 a(t_{h+1}) p; components without G take both
// pump terms as one (coefficients summed by load_pump).
// sin/cos of the phase with the Taylor series as short as the angle allows: |x| < 2^-10
// through x^4 / x^5 (the first dropped terms below 2e-21, relative for sin), |x| < 2^-6
// through x^6 / x^7 (below 9e-20), else sc<double>: 6, 8 or 12 FP64 operations.  Each
// point takes its own tier, so results do not depend on which points share a warp; a warp
// whose points agree runs that tier alone (warp votes), a mixed warp runs every tier its
// points need.
__device__ __forceinline__ void sc_tier0(double x, double* s, double* c) {
  const double x2 = x * x;
  *c = fma(x2, fma(x2, 1.0 / 24, -0.5), 1.0);
  *s = x * fma(x2, fma(x2, 1.0 / 120, -1.0 / 6), 1.0);
}
__device__ __forceinline__ void sc_tier1(double x, double* s, double* c) {
  const double x2 = x * x;
  *c = fma(x2, fma(x2, fma(x2, -1.0 / 720, 1.0 / 24), -0.5), 1.0);
  *s = x * fma(x2, fma(x2, fma(x2, -1.0 / 5040, 1.0 / 120), -1.0 / 6), 1.0);
}
__device__ __forceinline__ void sc_lean(double x, double* s, double* c) {
  const int hx = __double2hiint(x) & 0x7fffffff;
  const int tier = hx < 0x3f500000 ? 0 : hx < 0x3f900000 ? 1 : 2;
  const unsigned w = __activemask();
  if (__all_sync(w, tier == 0)) {
    sc_tier0(x, s, c);
  } else if (__all_sync(w, tier == 1)) {
    sc_tier1(x, s, c);
  } else {
    sc<double>(x, s, c);
    if (tier == 1) sc_tier1(x, s, c);
    if (tier == 0) sc_tier0(x, s, c);
  }
}

template <int M, int GM, int DM, int PM>
__device__ __forceinline__ void half_step_lean(double2 (&u)[M], const PassArgs& a, int64_t p,
                                               const double2 (&pn)[M], const double2 (&px)[M]) {
  double dens[M], prof[M];
#pragma unroll
  for (int l = 0; l < M; ++l) dens[l] = ((DM >> l) & 1) ? u[l].x * u[l].x + u[l].y * u[l].y : 0.0;
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if ((PM >> j) & 1) {
      prof[j] = __ldg((const double*)a.pprof[j] + p);
      if ((GM >> j) & 1) {
        u[j].x = fma(pn[j].x, prof[j], u[j].x);
        u[j].y = fma(pn[j].y, prof[j], u[j].y);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if ((GM >> j) & 1) {
      double pr = a.cd[j][0];
#pragma unroll
      for (int l = 0; l < M; ++l)
        if ((DM >> l) & 1) pr = fma(a.gd[j][l][0], dens[l], pr);
      double s, c;
      sc_lean(pr, &s, &c);
      double2 E;
      E.x = c;
      E.y = -s;
      u[j] = cmul(E, u[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if ((PM >> j) & 1) {
      u[j].x = fma(px[j].x, prof[j], u[j].x);
      u[j].y = fma(px[j].y, prof[j], u[j].y);
    }
  }
}

// Double-word form of half_step_lean, operation for operation the generic double-word half
// step (the same coefficient sums, dw_sincos, products and sums).
template <int M, int GM, int DM, int PM>
__device__ __forceinline__ void half_step_lean(dwc (&u)[M], const PassArgs& a, int64_t p,
                                               const dwc (&pn)[M], const dwc (&px)[M]) {
  dw dens[M], prof[M];
#pragma unroll
  for (int l = 0; l < M; ++l)
    dens[l] = ((DM >> l) & 1) ? dot2<+1>(re(u[l]), re(u[l]), im(u[l]), im(u[l])) : dw{0.0f, 0.0f};
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if ((PM >> j) & 1) {
      const float2 v = __ldg((const float2*)a.pprof[j] + p);
      prof[j] = dw{v.x, v.y};
      if ((GM >> j) & 1) u[j] = cadd(u[j], cscale(pn[j], prof[j]));
    }
  }
  const dw dth = {a.dthf, a.dthl};
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if ((GM >> j) & 1) {
      dw gr = {a.cf[j][0], a.cl[j][0]};
      bool empty = a.cf[j][0] == 0.0f && a.cl[j][0] == 0.0f;
#pragma unroll
      for (int l = 0; l < M; ++l)
        if (((DM >> l) & 1) && (a.gf[j][l][0] != 0.0f || a.gl[j][l][0] != 0.0f)) {
          const dw term = dw_mul({a.gf[j][l][0], a.gl[j][l][0]}, dens[l]);
          gr = empty ? term : dw_add_acc(gr, term);
          empty = false;
        }
      dw s, c;
      dw_sincos(dw_mul(dth, gr), s, c);
      u[j] = cmul(mk(c, dw_neg(s)), u[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < M; ++j)
    if ((PM >> j) & 1) u[j] = cadd(u[j], cscale(px[j], prof[j]));
}

template <int M, int E, int GM, int DM, int PM, typename C>
__device__ __forceinline__ void lean_points(C (&x)[M][E], const PassArgs& a, int64_t p0, int T,
                                            const C (&pn)[M], const C (&px)[M]) {
  // U points a trip, their chains independent (the phase routine's general branch is long,
  // so the loop is not unrolled further; double-word half steps, several hundred
  // instructions, one a trip); the arrays rotate by U
  constexpr int U = E % 2 == 0 && !std::is_same<C, dwc>::value ? 2 : 1;
#pragma unroll 1
  for (int i = 0; i < E; i += U) {
    C v[U][M];
#pragma unroll
    for (int u = 0; u < U; ++u) {
#pragma unroll
      for (int m = 0; m < M; ++m) v[u][m] = x[m][u];
      half_step_lean<M, GM, DM, PM>(v[u], a, p0 + (int64_t)T * (i + u), pn, px);
    }
#pragma unroll
    for (int m = 0; m < M; ++m) {
#pragma unroll
      for (int q = 0; q + U < E; ++q) x[m][q] = x[m][q + U];
#pragma unroll
      for (int u = 0; u < U; ++u) x[m][E - U + u] = v[u][m];
    }
  }
}

// FP32 form of half_step_lean, operation for operation the generic FP32 half step: the
// phase from the FP32 coefficients, E - 1 by sc_m1, the rotation's whole increment formed
// before it is added (see half_step).
template <int M, int GM, int DM, int PM>
__device__ __forceinline__ void half_step_lean(float2 (&u)[M], const PassArgs& a, int64_t p,
                                               const float2 (&pn)[M], const float2 (&px)[M]) {
  float dens[M], prof[M];
#pragma unroll
  for (int l = 0; l < M; ++l) dens[l] = ((DM >> l) & 1) ? u[l].x * u[l].x + u[l].y * u[l].y : 0.0f;
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if ((PM >> j) & 1) {
      prof[j] = __ldg((const float*)a.pprof[j] + p);
      if ((GM >> j) & 1) u[j] = cadd(u[j], cscale(pn[j], prof[j]));
    }
  }
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if ((GM >> j) & 1) {
      float gr = a.cf[j][0];
#pragma unroll
      for (int l = 0; l < M; ++l)
        if ((DM >> l) & 1) gr += a.gf[j][l][0] * dens[l];
      float s, cm1;
      sc_m1(a.dthf * gr, &s, &cm1);
      const float2 v = u[j];
      const float dx = __fmaf_rn(cm1, v.x, -__fmul_rn(-s, v.y));
      const float dy = __fmaf_rn(cm1, v.y, __fmul_rn(-s, v.x));
      u[j].x = __fadd_rn(v.x, dx);
      u[j].y = __fadd_rn(v.y, dy);
    }
  }
#pragma unroll
  for (int j = 0; j < M; ++j)
    if ((PM >> j) & 1) u[j] = cadd(u[j], cscale(px[j], prof[j]));
}

// the lean half step of kind a.lean on the E points a thread holds; false if there is none
template <int M, int E, typename C>
__device__ __forceinline__ bool lean_dispatch(C (&x)[M][E], const PassArgs& a, int64_t p0, int T,
                                              const C (&pn)[M], const C (&px)[M]) {
  if constexpr (M == 1) {
    if (a.lean == LEAN_M1_G) { lean_points<1, E, 1, 1, 0>(x, a, p0, T, pn, px); return true; }
    if (a.lean == LEAN_M1_GP) { lean_points<1, E, 1, 1, 1>(x, a, p0, T, pn, px); return true; }
  } else {
    if (a.lean == LEAN_M2_G1P0) { lean_points<2, E, 2, 2, 1>(x, a, p0, T, pn, px); return true; }
    if (a.lean == LEAN_M2_GG) { lean_points<2, E, 3, 3, 0>(x, a, p0, T, pn, px); return true; }
  }
  return false;
}

// Half step h on the E points a thread holds (points p0 + T*i).  The point loop is not
// unrolled, so the kernel holds one copy of the half step (the double-word step is
// several hundred instructions; eight unrolled copies overflow the instruction cache).
// Registers cannot be indexed at run time, so each trip works on x[.][0] and rotates
// the arrays by one; after E trips they are back in order.
template <typename Real, int M, int E>
__device__ __forceinline__ void half_points(typename CT<Real>::T (&x)[M][E], const PassArgs& a, int64_t p0, int T,
                                            int64_t b, int64_t h) {
  using C = typename CT<Real>::T;
  C pn[M], px[M];
  load_pump<Real, M>(a, h, pn, px, true);
  if (a.lean != LEAN_OFF && lean_dispatch<M, E>(x, a, p0, T, pn, px)) return;
// FP32 points per trip of the half-step loop: 2 measured fastest on the 512^2 polariton
// row pass (0.61 ms against 0.68 ms with all 8 unrolled, whose code spills out of the
// instruction cache, and 0.64 ms with 1)
#ifndef GPE_F32_HALF_UNROLL
#define GPE_F32_HALF_UNROLL 2
#endif
// 16-byte precisions (double-word, FP64): several hundred instructions a half step, one
// point a trip unless set otherwise
#ifndef GPE_W16_HALF_UNROLL
#define GPE_W16_HALF_UNROLL 1
#endif
  constexpr int UQ = sizeof(C) <= 8 ? GPE_F32_HALF_UNROLL : GPE_W16_HALF_UNROLL;
  constexpr int U = UQ < E ? UQ : E;
  if constexpr (sizeof(C) <= 8 && U == E) {
    // FP32: the half step is short, so unrolled copies fit the instruction cache and
    // interleave the independent points
#pragma unroll
    for (int i = 0; i < E; ++i) {
      C v[M];
#pragma unroll
      for (int m = 0; m < M; ++m) v[m] = x[m][i];
      half_step<Real, M>(v, a, p0 + (int64_t)T * i, b, h, pn, px);
#pragma unroll
      for (int m = 0; m < M; ++m) x[m][i] = v[m];
    }
  } else if constexpr (sizeof(C) <= 8 && M == 1) {
    // FP32, one component: a trip takes the points x and x + n0/2 (slots i and i + E/2),
    // which share one Philox block; both halves of the array rotate by one a trip
    constexpr int H = E / 2;
#pragma unroll 1
    for (int i = 0; i < H; ++i) {
      C v0[1] = {x[0][0]}, v1[1] = {x[0][H]};
      const int64_t pa = p0 + (int64_t)T * i, pb = pa + (int64_t)T * H;
      C xa[1], xb[1];
      const bool pre = a.noise == NOISE_PHILOX;
      if (pre) {
        const uint4 r = Philox4x32::gen(noise_counter(pa, b + a.traj0, h), a.seed_lo, a.seed_hi);
        xa[0] = Xi<Real>::get(r.x, r.y);
        xb[0] = Xi<Real>::get(r.z, r.w);
      }
      half_step<Real, 1>(v0, a, pa, b, h, pn, px, pre ? xa : nullptr);
      half_step<Real, 1>(v1, a, pb, b, h, pn, px, pre ? xb : nullptr);
#pragma unroll
      for (int q = 0; q + 1 < H; ++q) {
        x[0][q] = x[0][q + 1];
        x[0][H + q] = x[0][H + q + 1];
      }
      x[0][H - 1] = v0[0];
      x[0][E - 1] = v1[0];
    }
  } else {
    // U points a trip: U copies of the half step, the arrays rotated by U a trip
#pragma unroll 1
    for (int i0 = 0; i0 < E; i0 += U) {
      C v[U][M];
#pragma unroll
      for (int u = 0; u < U; ++u) {
#pragma unroll
        for (int m = 0; m < M; ++m) v[u][m] = x[m][u];
        half_step<Real, M>(v[u], a, p0 + (int64_t)T * (i0 + u), b, h, pn, px);
      }
#pragma unroll
      for (int m = 0; m < M; ++m) {
#pragma unroll
        for (int q = 0; q + U < E; ++q) x[m][q] = x[m][q + U];
#pragma unroll
        for (int u = 0; u < U; ++u) x[m][E - U + u] = v[u][m];
      }
    }
  }
}

// ------------------------------------------------------------------ row pass
template <typename Real, int LOGN, int M, int V = 0>
__global__ void __launch_bounds__(LineCfg<Real, M, LOGN, V>::ROW_THREADS, LineCfg<Real, M, LOGN, V>::ROW_MINB)
row_kernel(const PassArgs a, const int64_t nlines, const int lb) {
  // lb lines per block (Cfg::L, or fewer when there are too few lines to fill the SMs)
  using Cfg = LineCfg<Real, M, LOGN, V>;
  using C = typename CT<Real>::T;
  constexpr int N = Cfg::N, E = Cfg::ER, T = Cfg::TR;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int t = threadIdx.x % T, l = threadIdx.x / T;
  int64_t line = (int64_t)blockIdx.x * lb + l;
  const bool active = line < nlines;
  if (!active) line = nlines - 1;  // idle lines of the last block compute a copy, store nothing
  const RowLayout<C> lay{sm + l * N};
  const auto* tw = (const typename TwT<C>::T*)a.tw;
  const int64_t lpb = a.P / N;
  const int64_t b = line / lpb;
  const int64_t p0 = (line - b * lpb) * N + t;
  const int64_t g0 = b * a.P + p0;
  C x[M][E];
#pragma unroll
  for (int m = 0; m < M; ++m)
#pragma unroll
    for (int i = 0; i < E; ++i) x[m][i] = ((const C*)a.u[m])[g0 + T * i];
  // Phases: 0 inverse FFT_x, 1 half step A (+ save), 2 half step B, 3 forward FFT_x.
  // The loop is not unrolled, so the kernel holds one FFT and one half-step instance:
  // a half step rounds identically whether it opens a run (entry pass) or sits
  // between two steps, and a checkpointed, resumed run reproduces an uninterrupted one
  // bit for bit.
#pragma unroll 1
  for (int ph = 0; ph < 4; ++ph) {
    if (ph == 0 || ph == 3) {
      if (ph == 0 ? a.do_ifft : a.do_fft)
        // the inverse transform's values go straight into the half steps' double-word
        // products and sums: no closing renormalisation, unless the pass ends without the
        // forward transform (then they may be stored as they are)
        fft_components<C, N, E, M, RowLayout<C>, Cfg::JOINT, 1>(x, ph == 0, t, lay, tw, lb * N, ph != 0 || !a.do_fft,
                                                                a.fx != 0);
      continue;
    }
    const int64_t hr = ph == 2 ? a.hB : a.hA;
    if (hr >= 0) half_points<Real, M, E>(x, a, p0, T, b, hr + (a.kbase ? 2 * *a.kbase : 0));
    if (ph == 1 && a.save[0] && active) {
#pragma unroll
      for (int m = 0; m < M; ++m)
#pragma unroll
        for (int i = 0; i < E; ++i) store_save<Real>(a.save[m], g0 + T * i, x[m][i]);
    }
  }
  if (active) {
#pragma unroll
    for (int m = 0; m < M; ++m)
#pragma unroll
      for (int i = 0; i < E; ++i) ((C*)a.u[m])[g0 + T * i] = x[m][i];
  }
}

// Row pass of FP64 fields whose line transforms run in block floating point (a.fx):
// the transforms occupy the integer pipes and the half steps the FP64 pipe, and when every
// line of a block is in the same phase one pipe idles while the other works.  So each block
// holds two groups of lines that step through the same work half a cycle apart.  The
// block's items (LG lines each) alternate between the groups; time is cut into slots
// closed by a block barrier, and in every slot one group runs half steps (FP64) while the
// other runs integer work -- the forward transform and store of its last item, then the
// load and inverse transform of its next:
//   slot:     0        1        2              3        4  ...
//   group 0:  iFFT(0)  half(0)  FFT(0) iFFT(2) half(2)  FFT(2) iFFT(4) ...
//   group 1:  -        iFFT(1)  half(1)        FFT(1) iFFT(3) half(3) ...
// The transforms' exchanges synchronise per line (named barriers).  Blocks are persistent
// (two a multiprocessor), block c taking items c, c + gridDim, ...  Every item goes through
// the same code as in row_kernel, so the results are bit-identical to it.
template <int LOGN, int M>
__global__ void __launch_bounds__(LineCfg<double, M, LOGN, 0>::ROW_THREADS, LineCfg<double, M, LOGN, 0>::ROW_MINB)
row_kernel_pipe(const PassArgs a, const int64_t nlines) {
  using Cfg = LineCfg<double, M, LOGN, 0>;
  using C = double2;
  constexpr int N = Cfg::N, E = Cfg::ER, T = Cfg::TR, L = Cfg::L, LG = L / 2;
  static_assert(T % 32 == 0 && L % 2 == 0, "groups of whole-warp lines");
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int t = threadIdx.x % T, l = threadIdx.x / T;
  const int grp = l / LG, lg = l % LG;
  using RL = RowLayout<C, T>;
  const RL lay{sm + l * N};
  const auto* tw = (const C*)a.tw;
  const int64_t lpb = a.P / N;
  const int64_t nitems = (nlines + LG - 1) / LG;
  const int G = gridDim.x;
  // items of group g: (2k + g) G + blockIdx.x for k < n[g]
  auto count = [&](int g) -> int {
    const int64_t first = (int64_t)g * G + blockIdx.x;
    return first < nitems ? (int)((nitems - 1 - first) / (2 * (int64_t)G)) + 1 : 0;
  };
  const int n0 = count(0), n1 = count(1), ng = grp ? n1 : n0;
  const int nslots = n0 > 0 ? 2 * (n0 > n1 ? n0 : n1) + 2 : 0;
  C x[M][E];
  int64_t p0 = 0, b = 0;
  bool active = false;
  auto locate = [&](int k) {
    int64_t line = ((int64_t)(2 * k + grp) * G + blockIdx.x) * LG + lg;
    active = line < nlines;
    if (!active) line = nlines - 1;  // idle lines compute a copy, store nothing
    b = line / lpb;
    p0 = (line - b * lpb) * N + t;
  };
  const int64_t hbase = a.kbase ? 2 * *a.kbase : 0;
  // one call site each for the transform and the half step (as in row_kernel): the inner
  // loops are not unrolled
#pragma unroll 1
  for (int s = 0; s < nslots; ++s) {
    const int ls = s - grp;
    const int k = ls >> 1;
    if (ls >= 0 && (ls & 1) == 0) {
      // integer slot: j = 0 finishes item k - 1 (forward transform, store), j = 1 starts
      // item k (load, inverse transform)
#pragma unroll 1
      for (int j = 0; j < 2; ++j) {
        const bool fin = j == 0;
        if (fin ? (k >= 1 && k - 1 < ng) : (k < ng)) {
          if (!fin) {
            locate(k);
#pragma unroll
            for (int m = 0; m < M; ++m)
#pragma unroll
              for (int i = 0; i < E; ++i) x[m][i] = ((const C*)a.u[m])[b * a.P + p0 + T * i];
          }
          if (fin ? a.do_fft : a.do_ifft)
            fft_components<C, N, E, M, RL, false, 1>(x, !fin, t, lay, tw, 0, fin || !a.do_fft, true);
          if (fin && active) {
#pragma unroll
            for (int m = 0; m < M; ++m)
#pragma unroll
              for (int i = 0; i < E; ++i) ((C*)a.u[m])[b * a.P + p0 + T * i] = x[m][i];
          }
        }
      }
    } else if (ls >= 0 && k < ng) {
      // FP64 slot: half step A, the save, half step B
#pragma unroll 1
      for (int j = 0; j < 2; ++j) {
        const int64_t hr = j ? a.hB : a.hA;
        if (hr >= 0) half_points<double, M, E>(x, a, p0, T, b, hr + hbase);
        if (j == 0 && a.save[0] && active) {
#pragma unroll
          for (int m = 0; m < M; ++m)
#pragma unroll
            for (int i = 0; i < E; ++i) store_save<double>(a.save[m], b * a.P + p0 + T * i, x[m][i]);
        }
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ column pass
// The work on one tile held in registers: FFT_y, the k-space table, iFFT_y (one FFT
// instance: the phase loop is not unrolled).  sp0: spatial index of this thread's first
// point, step: index distance between its points.
// v 2^-d rounded to the nearest (d > 0, at most 63) or exactly (d <= 0, the result below 2^63)
__device__ __forceinline__ long long fx_shift(long long v, int d) {
  if (d > 0) {
    d = min(d, 63);
    return (v + (1LL << (d - 1))) >> d;
  }
  return v << (-d);
}

// Column tile of FP64 lines with block floating point transforms and a k-space table
// (FFT_y, table, iFFT_y in one pass): the forward transforms' outputs stay in fixed point,
// the table is applied to them on the integer pipes from its Q62 copy (a.ktab_q, entries
// scaled by 2^-kexp so that no component exceeds 1; a.kq_exp = kexp - log2 P restores the
// scale), and the inverse transforms start from the products.  Two of the four conversions
// between FP64 and fixed point of every line, and the FP64 work of the table, drop out.
// Before the table the lines are shifted to a common exponent (the 2x2 table mixes the
// components) that puts the largest component below 2^56, so the mat-vec's sums stay below
// 2^58, the transforms' input bound.  Each product rounds to within a unit of 2^-56 of the
// larger line's largest component; FP64 rounds each to 2^-53 of its own value.  One
// transform instance serves the four transforms (runtime direction, components rotated
// through the registers of component 0, as fft_components does).
template <int N, int E, int M, int CC>
__device__ __forceinline__ void col_fx_ktab(double2 (&x)[M][E], const PassArgs& a, int t, double2* xbase,
                                            int64_t sp0, int64_t step) {
  using LF = ColLayout<fxc, CC>;
  using LM = LineMax<CC, N / E>;
  const LF lf{reinterpret_cast<fxc*>(xbase)};
  const fxw* twq = reinterpret_cast<const fxw*>((const double2*)a.tw + N);
  __shared__ int red_in[LM::RED], red_x[LM::RED];
  constexpr int TOPK = 56;
  // per component (slot 0 holds the one being transformed; the others rotate with it):
  // exponent (value = integer 2^e), bit length of the largest component, non-finite input
  int e[M], top[M];
  bool bad[M];
#pragma unroll
  for (int m = 0; m < M; ++m) { e[m] = 0; top[m] = 0; bad[m] = false; }
#pragma unroll 1
  for (int q = 0; q < 2 * M; ++q) {
    const bool inv = q >= M;
    if (q == M) {
      // components back in order: align, then the table
      const fxw* kq = (const fxw*)a.ktab_q;
      int d[M];
      if (a.kkind == TAB_MATRIX) {
        int ec = top[0];
#pragma unroll
        for (int m = 1; m < M; ++m) ec = max(ec, top[m]);
        ec -= TOPK;
#pragma unroll
        for (int m = 0; m < M; ++m) { d[m] = ec - e[m]; e[m] = ec; }
        const bool b = M == 2 ? (bad[0] || bad[M - 1]) : bad[0];
#pragma unroll
        for (int m = 0; m < M; ++m) bad[m] = b;
      } else {
#pragma unroll
        for (int m = 0; m < M; ++m) { d[m] = max(0, top[m] - e[m] - TOPK); e[m] += d[m]; }
      }
#pragma unroll
      for (int i = 0; i < E; ++i) {
        fxc v[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
          v[m].x = fx_shift(__double_as_longlong(x[m][i].x), d[m]);
          v[m].y = fx_shift(__double_as_longlong(x[m][i].y), d[m]);
        }
        const int64_t kp = sp0 + step * i;
        fxc y[M];
        if (a.kkind == TAB_MATRIX && M == 2) {
          const fxc p00 = twmul(v[0], ldgc(kq + kp)), p01 = twmul(v[M - 1], ldgc(kq + a.P + kp));
          const fxc p10 = twmul(v[0], ldgc(kq + 2 * a.P + kp)), p11 = twmul(v[M - 1], ldgc(kq + 3 * a.P + kp));
          y[0].x = p00.x + p01.x;
          y[0].y = p00.y + p01.y;
          y[M - 1].x = p10.x + p11.x;
          y[M - 1].y = p10.y + p11.y;
        } else {
#pragma unroll
          for (int m = 0; m < M; ++m) y[m] = twmul(v[m], ldgc(kq + (a.kkind == TAB_DIAG ? (int64_t)m * a.P : 0) + kp));
        }
#pragma unroll
        for (int m = 0; m < M; ++m) x[m][i] = make_double2(__longlong_as_double(y[m].x), __longlong_as_double(y[m].y));
      }
#pragma unroll
      for (int m = 0; m < M; ++m) e[m] += a.kq_exp;
    }
    fxc v[E];
    if (!inv) {
      // largest biased exponent of the line, conversion below 2^FX_TOP
      unsigned hm = 0;
#pragma unroll
      for (int i = 0; i < E; ++i) {
        hm = max(hm, (unsigned)__double2hiint(x[0][i].x) & 0x7fffffffu);
        hm = max(hm, (unsigned)__double2hiint(x[0][i].y) & 0x7fffffffu);
      }
      int em = LM::warp((int)(hm >> 20));
      LM::publish(em, red_in);
      if constexpr (LM::MULTI) lf.sync();
      em = LM::collect(em, red_in);
#pragma unroll
      for (int i = 0; i < E; ++i) {
        v[i].x = fx_from_double(x[0][i].x, em);
        v[i].y = fx_from_double(x[0][i].y, em);
      }
      e[0] = em - 1022 - FX_TOP;
      bad[0] = em == 0x7ff;
    } else {
      // the inverse transform as the forward one of the values with real and imaginary
      // parts swapped
#pragma unroll
      for (int i = 0; i < E; ++i) {
        v[i].x = __double_as_longlong(x[0][i].y);
        v[i].y = __double_as_longlong(x[0][i].x);
      }
    }
    int shsum = 0;
    fx_stages<N, E, 1, LF, LM>(v, t, lf, twq, red_x, shsum);
    e[0] += shsum;
    if (!inv) {
      // bit length of the line's largest component (from the high words, as the stages do)
      unsigned mag = 0;
#pragma unroll
      for (int i = 0; i < E; ++i) mag |= fx_mag(v[i]);
      const int lw = LM::warp(mag ? 64 - __clz((int)mag) : 32);
      LM::publish(lw, red_x);
      lf.sync();
      top[0] = e[0] + LM::collect(lw, red_x);
      lf.sync();  // red_x is written again by the next transform's first stage
#pragma unroll
      for (int i = 0; i < E; ++i) x[0][i] = make_double2(__longlong_as_double(v[i].x), __longlong_as_double(v[i].y));
    } else {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        x[0][i].x = bad[0] ? __longlong_as_double(0x7ff8000000000000LL) : fx_to_double(v[i].y, e[0]);
        x[0][i].y = bad[0] ? __longlong_as_double(0x7ff8000000000000LL) : fx_to_double(v[i].x, e[0]);
      }
    }
    if constexpr (M == 2) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const double2 tmp = x[0][i];
        x[0][i] = x[1][i];
        x[1][i] = tmp;
      }
      int ti = e[0]; e[0] = e[1]; e[1] = ti;
      ti = top[0]; top[0] = top[1]; top[1] = ti;
      const bool tb = bad[0]; bad[0] = bad[1]; bad[1] = tb;
    }
  }
}

template <typename Real, int LOGN, int M, int V>
__device__ __forceinline__ void col_tile_work(typename CT<Real>::T (&x)[M][LineCfg<Real, M, LOGN, V>::E],
                                              const PassArgs& a, int t,
                                              const ColLayout<typename CT<Real>::T, LineCfg<Real, M, LOGN, V>::CC>& lay,
                                              int64_t sp0, int64_t step) {
  using Cfg = LineCfg<Real, M, LOGN, V>;
  using C = typename CT<Real>::T;
  constexpr int N = Cfg::N, E = Cfg::E, CC = Cfg::CC;
  const auto* tw = (const typename TwT<C>::T*)a.tw;
  if constexpr (std::is_same<Real, double>::value && !Cfg::JOINT && N > E) {
    if (a.fx && a.ktab && a.ktab_q && a.col_fwd && a.col_inv) {
      col_fx_ktab<N, E, M, CC>(x, a, t, lay.base, sp0, step);
      return;
    }
  }
#pragma unroll 1
  for (int ph = 0; ph < 3; ++ph) {
    if (ph != 1) {
      if (ph == 0 ? a.col_fwd : a.col_inv)
        // the forward transform's values go straight into the table's complex products
        fft_components<C, N, E, M, ColLayout<C, CC>, Cfg::JOINT, CC>(x, ph == 2, t, lay, tw, CC * Cfg::NPAD,
                                                                     ph == 2 || !a.ktab, a.fx != 0);
      continue;
    }
    if (a.ktab) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        C v[M];
#pragma unroll
        for (int m = 0; m < M; ++m) v[m] = x[m][i];
        kmul<Real, M>(v, a, sp0 + step * i);
#pragma unroll
        for (int m = 0; m < M; ++m) x[m][i] = v[m];
      }
    }
  }
}

template <typename Real, int LOGN, int M, int V = 0>
__global__ void __launch_bounds__(LineCfg<Real, M, LOGN, V>::COL_THREADS, LineCfg<Real, M, LOGN, V>::COL_MINB)
col_kernel(const PassArgs a) {
  using Cfg = LineCfg<Real, M, LOGN, V>;
  using C = typename CT<Real>::T;
  constexpr int E = Cfg::E, T = Cfg::T, CC = Cfg::CC;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int c = threadIdx.x % CC, t = threadIdx.x / CC;
  int64_t tile = blockIdx.x;
  const int64_t ntx = a.n0 / CC;
  const int64_t xt = tile % ntx;
  tile /= ntx;
  const int64_t o = tile % a.nouter;
  const int64_t b = tile / a.nouter;
  const int64_t sp0 = o * a.ostride + xt * CC + c + (int64_t)t * a.ld;
  const int64_t g0 = b * a.P + sp0;
  const int64_t step = (int64_t)T * a.ld;
  const ColLayout<C, CC> lay{sm + c};
  C x[M][E];
#pragma unroll
  for (int m = 0; m < M; ++m)
#pragma unroll
    for (int i = 0; i < E; ++i) x[m][i] = ((const C*)a.u[m])[g0 + step * i];
  col_tile_work<Real, LOGN, M, V>(x, a, t, lay, sp0, step);
#pragma unroll
  for (int m = 0; m < M; ++m)
#pragma unroll
    for (int i = 0; i < E; ++i) ((C*)a.u[m])[g0 + step * i] = x[m][i];
}

// Shared-memory plan of the TMA column pass: the FFT exchange, then the staging buffer
// (1024-byte aligned) holding one tile of every component as TMA writes it (rows of CC
// points, dense), then the mbarrier.  SLACK covers the alignment of the dynamic base.
template <typename Real, int M, int LOGN>
struct ColTmaCfg {
  using Cfg = LineCfg<Real, M, LOGN, 0>;
  using C = typename CT<Real>::T;
  static constexpr int N = Cfg::N, CC = Cfg::CC;
  static constexpr int XF = CC * (int)sizeof(C) / 4;  // floats per tile row (box width)
  static constexpr int BOXR = N < 256 ? N : 256;      // rows per box
  static constexpr size_t EXCH = (Cfg::COL_SMEM + 1023) / 1024 * 1024;
  static constexpr size_t STAGE = (size_t)M * N * CC * sizeof(C);
  static constexpr size_t SLACK = 1024;
  static constexpr size_t SMEM = SLACK + EXCH + STAGE + 16;
  static constexpr bool OK = XF % 4 == 0 && SMEM <= 227 * 1024 && STAGE < (1u << 20);
};

// Persistent 2D column pass with TMA staging: CTA k takes tiles k, k + grid, ...; while
// it transforms one tile, the copy engine brings the next into the staging buffer.
// tm[m] maps component m as a 2D array of B*n1 rows of n0 points (counted in floats).
template <typename Real, int LOGN, int M>
__global__ void __launch_bounds__(LineCfg<Real, M, LOGN, 0>::COL_THREADS, LineCfg<Real, M, LOGN, 0>::COL_MINB)
col_kernel_tma(const PassArgs a, const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1) {
  using Cfg = LineCfg<Real, M, LOGN, 0>;
  using TC = ColTmaCfg<Real, M, LOGN>;
  using C = typename CT<Real>::T;
  constexpr int N = Cfg::N, E = Cfg::E, T = Cfg::T, CC = Cfg::CC;
  extern __shared__ __align__(16) unsigned char smraw[];
  unsigned char* base = smraw + ((1024u - (smem_addr(smraw) & 1023u)) & 1023u);
  C* sm = reinterpret_cast<C*>(base);
  C* stg = reinterpret_cast<C*>(base + TC::EXCH);
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + TC::EXCH + TC::STAGE);
  const int c = threadIdx.x % CC, t = threadIdx.x / CC;
  const int64_t ntx = a.n0 / CC;
  const int64_t ntiles = ntx * a.B;
  const int64_t step = (int64_t)T * a.ld;
  const ColLayout<C, CC> lay{sm + c};
  auto issue = [&](int64_t tile) {
    const int64_t xt = tile % ntx, b = tile / ntx;
    mbar_arrive_expect_tx(bar, (uint32_t)TC::STAGE);
#pragma unroll
    for (int m = 0; m < M; ++m)
#pragma unroll
      for (int j = 0; j < N / TC::BOXR; ++j)
        tma_load_2d(stg + ((size_t)m * N + (size_t)j * TC::BOXR) * CC, m == 0 ? &tm0 : &tm1, (int32_t)(xt * TC::XF),
                    (int32_t)(b * a.n1 + j * TC::BOXR), bar);
  };
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_init_fence();
  }
  __syncthreads();
  int64_t tile = blockIdx.x;
  if (threadIdx.x == 0 && tile < ntiles) issue(tile);
  uint32_t parity = 0;
  for (; tile < ntiles; tile += gridDim.x) {
    const bool got = mbar_wait(bar, parity, kWaitLimitNs);
    if (__syncthreads_or(!got)) {
      // the tile never arrived: report, and leave only once the copy engine is done
      // with this CTA's shared memory (again a bounded wait)
      if (threadIdx.x == 0 && a.status) atomicExch(a.status, 1);
      if (threadIdx.x == 0) mbar_wait(bar, parity, kWaitLimitNs);
      __syncthreads();
      return;
    }
    parity ^= 1u;
    C x[M][E];
#pragma unroll
    for (int m = 0; m < M; ++m)
#pragma unroll
      for (int i = 0; i < E; ++i) x[m][i] = stg[((size_t)m * N + t + T * i) * CC + c];
    // staging consumed: the copy engine's writes of the next tile are ordered after these
    // reads only through the proxy fence (a barrier alone orders ordinary accesses)
    fence_proxy_async_smem();
    __syncthreads();
    const int64_t nxt = tile + gridDim.x;
    if (nxt < ntiles && threadIdx.x == 0) issue(nxt);
    const int64_t xt = tile % ntx, b = tile / ntx;
    const int64_t sp0 = xt * CC + c + (int64_t)t * a.ld;
    const int64_t g0 = b * a.P + sp0;
    col_tile_work<Real, LOGN, M, 0>(x, a, t, lay, sp0, step);
#pragma unroll
    for (int m = 0; m < M; ++m)
#pragma unroll
      for (int i = 0; i < E; ++i) ((C*)a.u[m])[g0 + step * i] = x[m][i];
  }
}

// ------------------------------------------------------------------ 1D resident
// nlines = B trajectories of one line each; runs a.nsteps full steps in registers.
// Both half steps of a step share one half_step instance (a non-unrolled loop), like
// the row pass.
template <typename Real, int LOGN, int M>
__global__ void __launch_bounds__(LineCfg<Real, M, LOGN>::ROW_THREADS)
line1d_kernel(const PassArgs a, const int64_t nlines) {
  using Cfg = LineCfg<Real, M, LOGN>;
  using C = typename CT<Real>::T;
  constexpr int N = Cfg::N, E = Cfg::ER, T = Cfg::TR, L = Cfg::L;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int t = threadIdx.x % T, l = threadIdx.x / T;
  int64_t line = (int64_t)blockIdx.x * L + l;
  const bool active = line < nlines;
  if (!active) line = nlines - 1;
  const RowLayout<C> lay{sm + l * N};
  const auto* tw = (const typename TwT<C>::T*)a.tw;
  const int64_t b = line;
  const int64_t g0 = b * a.P + t;
  C x[M][E];
#pragma unroll
  for (int m = 0; m < M; ++m)
#pragma unroll
    for (int i = 0; i < E; ++i) x[m][i] = ((const C*)a.u[m])[g0 + T * i];
  const int64_t step0 = a.step0 + (a.kbase ? *a.kbase : 0);
  for (int64_t s = 0; s < a.nsteps; ++s) {
    const int64_t k = step0 + s;
    // phases: 0 half step 2k, 1 forward FFT, 2 k-space table, 3 inverse FFT,
    // 4 half step 2k+1 (one FFT and one half-step instance)
#pragma unroll 1
    for (int ph = 0; ph < 5; ++ph) {
      if (ph == 1 || ph == 3) {
        if (a.ktab) fft_components<C, N, E, M, RowLayout<C>, false, 1>(x, ph == 3, t, lay, tw, 0, true, a.fx != 0);
      } else if (ph == 2) {
        if (a.ktab) {
#pragma unroll
          for (int i = 0; i < E; ++i) {
            C v[M];
#pragma unroll
            for (int m = 0; m < M; ++m) v[m] = x[m][i];
            kmul<Real, M>(v, a, t + T * i);
#pragma unroll
            for (int m = 0; m < M; ++m) x[m][i] = v[m];
          }
        }
      } else {
        half_points<Real, M, E>(x, a, t, T, b, 2 * k + (ph == 4 ? 1 : 0));
      }
    }
    if (a.save_every > 0 && ((s + 1) % a.save_every) == 0 && active) {
      const int64_t slot = (s + 1) / a.save_every - 1;
#pragma unroll
      for (int m = 0; m < M; ++m)
#pragma unroll
        for (int i = 0; i < E; ++i) store_save<Real>(a.save[m], slot * a.save_stride + g0 + T * i, x[m][i]);
    }
  }
  if (active) {
#pragma unroll
    for (int m = 0; m < M; ++m)
#pragma unroll
      for (int i = 0; i < E; ++i) ((C*)a.u[m])[g0 + T * i] = x[m][i];
  }
}

template <typename K>
static inline int set_smem(K k, size_t bytes);

// ------------------------------------------------------------------ resident plane
// A whole 2D trajectory (M planes of N x N points) lives in shared memory for all
// nsteps steps; one CTA per trajectory.  Each step is one column round-set
// (FFT_y * table * iFFT_y) and one row round-set ([iFFT_x] [half A] [save] [half B]
// [FFT_x]), the same operations, code and order as the HBM column and row passes, so
// the result equals theirs.  A line's FFT exchanges run in place in the line's own
// shared-memory slots (its points are in registers meanwhile).
template <typename Real, int M, int LOGN>
struct PlaneCfg {
  using C = typename CT<Real>::T;
  static constexpr int N = 1 << LOGN;
  static constexpr int E = cmin(sizeof(C) == 16 ? 8 : 8, N / 2);
  static constexpr int T = N / E;            // threads per line
  static constexpr int NT = cmin(512, N * T);  // threads per CTA
  static constexpr int LPR = NT / T;         // lines per round
  static constexpr int ROUNDS = N / LPR;
  static constexpr size_t SMEM = (size_t)M * N * N * sizeof(C);
  static constexpr bool FITS = SMEM <= 200 * 1024;
};

template <int STRIDE, typename C>
struct StridedLayout {  // point n of a column at n * STRIDE
  template <typename D> using rebind = StridedLayout<STRIDE, D>;
  C* base;
  __device__ __forceinline__ static void sync() { __syncthreads(); }
  template <int NS, int R>
  __device__ __forceinline__ int addr(int idx) const { return idx * STRIDE; }
};

template <typename Real, int LOGN, int M>
__global__ void __launch_bounds__(PlaneCfg<Real, M, LOGN>::NT)
plane_kernel(const PassArgs a) {
  using Cfg = PlaneCfg<Real, M, LOGN>;
  using C = typename CT<Real>::T;
  constexpr int N = Cfg::N, E = Cfg::E, T = Cfg::T, NT = Cfg::NT, LPR = Cfg::LPR, ROUNDS = Cfg::ROUNDS;
  constexpr int P = N * N;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* f = reinterpret_cast<C*>(smraw);  // f[m * P + p]
  const int64_t b = blockIdx.x;
  const int tid = threadIdx.x;
  const auto* twx = (const typename TwT<C>::T*)a.tw;
  const auto* twy = (const typename TwT<C>::T*)a.tw2;
  for (int m = 0; m < M; ++m)
    for (int p = tid; p < P; p += NT) f[m * P + p] = ((const C*)a.u[m])[b * P + p];
  __syncthreads();
  const int t = tid % T, lr = tid / T;       // row rounds: line lr of the round
  const int cc = tid % LPR, ct = tid / LPR;  // column rounds: column cc, thread ct
  const int64_t step0 = a.step0 + (a.kbase ? *a.kbase : 0);
  for (int64_t s = 0; s <= a.nsteps; ++s) {
    const int64_t k = step0 + s;
    // ---- column round-set (absent before the first step)
    if (s > 0 && a.ktab) {
#pragma unroll 1
      for (int r = 0; r < ROUNDS; ++r) {
        const int c = r * LPR + cc;
        const StridedLayout<N, C> lay{f + c};
        C x[M][E];
#pragma unroll
        for (int m = 0; m < M; ++m)
#pragma unroll
          for (int i = 0; i < E; ++i) x[m][i] = f[m * P + (ct + T * i) * N + c];
        __syncthreads();  // the column's slots become FFT exchange space
        fft_components<C, N, E, M, StridedLayout<N, C>, false, LPR>(x, false, ct, lay, twy, 0, true, a.fx != 0);
#pragma unroll 1
        for (int i = 0; i < E; ++i) {
          C v[M];
#pragma unroll
          for (int m = 0; m < M; ++m) v[m] = x[m][0];
          kmul<Real, M>(v, a, (int64_t)(ct + T * i) * N + c);
#pragma unroll
          for (int m = 0; m < M; ++m) {
#pragma unroll
            for (int q = 0; q + 1 < E; ++q) x[m][q] = x[m][q + 1];
            x[m][E - 1] = v[m];
          }
        }
        fft_components<C, N, E, M, StridedLayout<N, C>, false, LPR>(x, true, ct, lay, twy, 0, true, a.fx != 0);
        __syncthreads();
#pragma unroll
        for (int m = 0; m < M; ++m)
#pragma unroll
          for (int i = 0; i < E; ++i) f[m * P + (ct + T * i) * N + c] = x[m][i];
        __syncthreads();
      }
    }
    // ---- row round-set: end of step k-1 (s > 0) and start of step k (s < nsteps)
    const bool first = (s == 0), last = (s == a.nsteps);
    const bool save = !first && a.save_every > 0 && (s % a.save_every) == 0;
#pragma unroll 1
    for (int r = 0; r < ROUNDS; ++r) {
      const int y = r * LPR + lr;
      const RowLayout<C> lay{f + y * N};
      C x[M][E];
#pragma unroll
      for (int m = 0; m < M; ++m)
#pragma unroll
        for (int i = 0; i < E; ++i) x[m][i] = f[m * P + y * N + t + T * i];
      __syncthreads();  // the line's slots become FFT exchange space
      if (!first && a.ktab) fft_components<C, N, E, M, RowLayout<C>, false, 1>(x, true, t, lay, twx, 0, true, a.fx != 0);
      if (!first) half_points<Real, M, E>(x, a, y * N + t, T, b, 2 * k - 1);
      if (save) {
        const int64_t slot = s / a.save_every - 1;
#pragma unroll
        for (int m = 0; m < M; ++m)
#pragma unroll
          for (int i = 0; i < E; ++i) store_save<Real>(a.save[m], slot * a.save_stride + b * P + y * N + t + T * i, x[m][i]);
      }
      if (!last) half_points<Real, M, E>(x, a, y * N + t, T, b, 2 * k);
      if (!last && a.ktab) fft_components<C, N, E, M, RowLayout<C>, false, 1>(x, false, t, lay, twx, 0, true, a.fx != 0);
      __syncthreads();
#pragma unroll
      for (int m = 0; m < M; ++m)
#pragma unroll
        for (int i = 0; i < E; ++i) f[m * P + y * N + t + T * i] = x[m][i];
      __syncthreads();
    }
  }
  for (int m = 0; m < M; ++m)
    for (int p = tid; p < P; p += NT) ((C*)a.u[m])[b * P + p] = f[m * P + p];
}

template <typename Real, int M, int LOGN>
int launch_plane_n(const PassArgs& a, cudaStream_t s) {
  using Cfg = PlaneCfg<Real, M, LOGN>;
  if constexpr (!Cfg::FITS) {
    return (int)cudaErrorInvalidValue;
  } else {
    auto k = plane_kernel<Real, LOGN, M>;
    int e = set_smem(k, Cfg::SMEM);
    if (e) return e;
    k<<<(unsigned)a.B, Cfg::NT, Cfg::SMEM, s>>>(a);
    return (int)cudaGetLastError();
  }
}

// ------------------------------------------------------------------ no dispersion
// Without a dispersion the step is pointwise: one thread per point runs all steps.
template <typename Real, int M>
__global__ void __launch_bounds__(256) nl_only_kernel(const PassArgs a) {
  using C = typename CT<Real>::T;
  const int64_t total = a.P * a.B;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = q / a.P, p = q - b * a.P;
    C v[M];
#pragma unroll
    for (int m = 0; m < M; ++m) v[m] = ((const C*)a.u[m])[q];
    const int64_t step0 = a.step0 + (a.kbase ? *a.kbase : 0);
    for (int64_t s = 0; s < a.nsteps; ++s) {
#pragma unroll 1
      for (int half = 0; half < 2; ++half) {
        const int64_t h = 2 * (step0 + s) + half;
        C pn[M], px[M];
        load_pump<Real, M>(a, h, pn, px, true);
        half_step<Real, M>(v, a, p, b, h, pn, px);
      }
      if (a.save_every > 0 && ((s + 1) % a.save_every) == 0) {
        const int64_t slot = (s + 1) / a.save_every - 1;
#pragma unroll
        for (int m = 0; m < M; ++m) store_save<Real>(a.save[m], slot * a.save_stride + q, v[m]);
      }
    }
#pragma unroll
    for (int m = 0; m < M; ++m) ((C*)a.u[m])[q] = v[m];
  }
}

// Half step h of the matrix family (SMatrix G, src/kernels.jl:23-25,36-50):
//   u <- exp(-i delta G(u)) V (u + delta/2 F_now) + delta/2 F_next - i sqrt(delta) eta xi
template <typename Real>
__device__ __forceinline__ void matrix_half_step(typename CT<Real>::T (&u)[2], const PassArgs& a, int64_t p,
                                                 int64_t b, int64_t h) {
  using C = typename CT<Real>::T;
  C pn[2], px[2];
  load_pump<Real, 2>(a, h, pn, px);
  C Em[4];
  matrix_phase<Real>(u, a, p, Em);
  C prof[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    if (a.pprof[j]) {
      prof[j] = ((a.pump_uniform >> j) & 1) ? cunit<C>()
                : a.pprof_cplx ? ldgc((const C*)a.pprof[j] + p) : Prof<Real>::cplx(a.pprof[j], p);
      u[j] = pump_add(u[j], pn[j], prof[j], a.pprof_cplx);
    }
  }
  const C y0 = cadd(cmul(Em[0], u[0]), cmul(Em[1], u[1]));
  const C y1 = cadd(cmul(Em[2], u[0]), cmul(Em[3], u[1]));
  u[0] = y0;
  u[1] = y1;
#pragma unroll
  for (int j = 0; j < 2; ++j)
    if (a.pprof[j]) u[j] = pump_add(u[j], px[j], prof[j], a.pprof_cplx);
  if (a.noise != NOISE_OFF) {
    C xi[2];
    draw_xi<Real, 2>(a, p, b, h, xi);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      C nf;
      if constexpr (std::is_same<Real, DWR>::value) {
        nf = mk({a.nfacf[j][0], a.nfacl[j][0]}, {a.nfacf[j][1], a.nfacl[j][1]});
        if (a.etaprof[j]) {
          const float2 e = __ldg((const float2*)a.etaprof[j] + p);
          nf = cscale(nf, dw{e.x, e.y});
        }
      } else {
        nf.x = Coef<Real>::nf(a, j, 0);
        nf.y = Coef<Real>::nf(a, j, 1);
        if (a.etaprof[j]) nf = cscale(nf, __ldg((const Real*)a.etaprof[j] + p));
      }
      u[j] = cadd(u[j], cmul(nf, xi[j]));
    }
  }
}

// Pointwise pass of the matrix family.  nsteps > 0: whole steps of a problem without a
// k-space table (saves every save_every steps, like nl_only_kernel); otherwise the real-
// space part of a row-pass program between two FFT-only passes: [half hA] [save] [half hB].
template <typename Real>
__global__ void __launch_bounds__(256) mat_kernel(const PassArgs a) {
  using C = typename CT<Real>::T;
  const int64_t total = a.P * a.B;
  const int64_t kb = a.kbase ? *a.kbase : 0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = q / a.P, p = q - b * a.P;
    C v[2] = {((const C*)a.u[0])[q], ((const C*)a.u[1])[q]};
    if (a.nsteps > 0) {
      for (int64_t s = 0; s < a.nsteps; ++s) {
#pragma unroll 1
        for (int half = 0; half < 2; ++half) matrix_half_step<Real>(v, a, p, b, 2 * (a.step0 + kb + s) + half);
        if (a.save_every > 0 && ((s + 1) % a.save_every) == 0) {
          const int64_t slot = (s + 1) / a.save_every - 1;
#pragma unroll
          for (int m = 0; m < 2; ++m) store_save<Real>(a.save[m], slot * a.save_stride + q, v[m]);
        }
      }
    } else {
#pragma unroll 1
      for (int ph = 0; ph < 2; ++ph) {
        const int64_t hr = ph ? a.hB : a.hA;
        if (hr >= 0) matrix_half_step<Real>(v, a, p, b, hr + 2 * kb);
        if (ph == 0 && a.save[0]) {
#pragma unroll
          for (int m = 0; m < 2; ++m) store_save<Real>(a.save[m], q, v[m]);
        }
      }
    }
#pragma unroll
    for (int m = 0; m < 2; ++m) ((C*)a.u[m])[q] = v[m];
  }
}

// ------------------------------------------------------------------ FP64 norm
template <typename C> __device__ __forceinline__ double abs2d(const C& v) {
  return (double)v.x * (double)v.x + (double)v.y * (double)v.y;
}
template <> __device__ __forceinline__ double abs2d<dwc>(const dwc& v) {
  const double x = dw_to_double(re(v)), y = dw_to_double(im(v));
  return x * x + y * y;
}

template <typename Real, int M>
__global__ void __launch_bounds__(256) norm_kernel(const PassArgs a, double* out) {
  using C = typename CT<Real>::T;
  __shared__ double red[M][8];
  const int64_t total = a.P * a.B;
  double acc[M];
#pragma unroll
  for (int m = 0; m < M; ++m) acc[m] = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int m = 0; m < M; ++m) acc[m] += abs2d(((const C*)a.u[m])[q]);
  }
#pragma unroll
  for (int m = 0; m < M; ++m) {
    double v = acc[m];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[m][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int m = 0; m < M; ++m) {
      double v = (threadIdx.x < (blockDim.x >> 5)) ? red[m][threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0) atomicAdd(out + m, v);
    }
  }
}

// ------------------------------------------------------------------ launchers
template <typename K>
static inline int set_smem(K k, size_t bytes) {
  if (bytes > 48 * 1024) return (int)cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return 0;
}

template <typename Real, int M, int LOGN, int V = 0>
int launch_row_n(const PassArgs& a, int64_t nlines, cudaStream_t s) {
  using Cfg = LineCfg<Real, M, LOGN, V>;
  if constexpr (std::is_same<Real, double>::value && M == 1 && V == 0 && Cfg::TR % 32 == 0 && Cfg::L % 2 == 0) {
    // block floating point transforms: the pipelined pass when every block gets at least
    // four items a group.  One-component lines only: on the two-component polariton (512^2,
    // 64 copies) it took 1.79 ms against 1.60 ms for row_kernel (each phase then has half
    // the warps of a block to hide the FP64 pipe's latency), on one-component 1024^2 lines
    // (16 copies) it gained 7 % of the step.
    const int64_t blocks = 2 * (int64_t)(a.nsm > 0 ? a.nsm : 152);
    const int64_t nitems = (nlines + Cfg::L / 2 - 1) / (Cfg::L / 2);
    if (a.fx && nitems >= 8 * blocks) {
      auto kp = row_kernel_pipe<LOGN, M>;
      int e = set_smem(kp, Cfg::ROW_KERNEL_SMEM);
      if (e) return e;
      kp<<<(unsigned)blocks, Cfg::ROW_THREADS, Cfg::ROW_KERNEL_SMEM, s>>>(a, nlines);
      return (int)cudaGetLastError();
    }
  }
  auto k = row_kernel<Real, LOGN, M, V>;
  int e = set_smem(k, Cfg::ROW_KERNEL_SMEM);
  if (e) return e;
  // fewer lines per block when the default tiling would not give every SM two blocks
  // (e.g. one 512^2 field: 128 blocks of 4 lines, 512 blocks of one line)
  int lb = Cfg::L;
  const int64_t want = 2 * (int64_t)(a.nsm > 0 ? a.nsm : 152);
  while (lb > 1 && (nlines + lb - 1) / lb < want) lb /= 2;
  const int64_t blocks = (nlines + lb - 1) / lb;
  const size_t smem = Cfg::ROW_KERNEL_SMEM / Cfg::L * lb;
  k<<<(unsigned)blocks, lb * Cfg::TR, smem, s>>>(a, nlines, lb);
  return (int)cudaGetLastError();
}
// cuTensorMapEncodeTiled from the driver, looked up once through the runtime (no link
// against libcuda); null when the driver does not provide it
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// Tensor map of one component for the TMA column pass: rows of `row_floats` floats,
// `rows` rows, box of box_x floats by box_y rows, no swizzle.
inline bool encode_rows_map(CUtensorMap* tm, const void* base, uint64_t row_floats, uint64_t rows, uint32_t box_x,
                            uint32_t box_y) {
  auto enc = tensor_map_encoder();
  if (!enc || ((uintptr_t)base & 15) || (row_floats * 4) % 16) return false;
  const cuuint64_t dims[2] = {row_floats, rows};
  const cuuint64_t strides[1] = {row_floats * 4};
  const cuuint32_t box[2] = {box_x, box_y};
  const cuuint32_t es[2] = {1, 1};
  return enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// TMA column pass for a 2D field (lines along y of length N = n1, stride n0); returns
// -1 when this shape does not take it (the caller then launches col_kernel)
template <typename Real, int M, int LOGN>
int launch_col_tma_n(const PassArgs& a, cudaStream_t s) {
  using Cfg = LineCfg<Real, M, LOGN, 0>;
  using TC = ColTmaCfg<Real, M, LOGN>;
  using C = typename CT<Real>::T;
  if constexpr (!TC::OK) {
    return -1;
  } else {
    if (a.nouter != 1 || a.ld != a.n0 || a.n1 != Cfg::N || a.n0 % Cfg::CC || a.B * (int64_t)a.n1 > INT32_MAX) return -1;
    // measured on GB300 (ms per column pass, plain -> TMA): one component 0.139 -> 0.135
    // (256^2 x 341, FP32), 0.107 -> 0.104 (512^2 x 16, double-word), 0.193 -> 0.191 (512^2
    // x 64, FP32); two components 0.796 -> 0.817 (512^2 x 64, double-word), 0.412 -> 0.479
    // (512^2 x 128, FP32, one CTA per SM instead of two); 1024-point FP32 lines 0.214 -> 0.221
    if (a.col_tma == 2 && (M != 1 || Cfg::N > 512)) return -1;
    CUtensorMap tm[2];
    const uint64_t row_floats = (uint64_t)a.n0 * sizeof(C) / 4;
    for (int m = 0; m < M; ++m)
      if (!encode_rows_map(&tm[m], a.u[m], row_floats, (uint64_t)a.B * a.n1, TC::XF, TC::BOXR)) return -1;
    if (M == 1) tm[1] = tm[0];
    auto k = col_kernel_tma<Real, LOGN, M>;
    int e = set_smem(k, TC::SMEM);
    if (e) return e;
    // resident CTAs per SM, queried once per instantiation (the kernel's registers and
    // shared memory decide it, not the field)
    static std::atomic<int> per_sm_cache{0};
    int per_sm = per_sm_cache.load(std::memory_order_relaxed);
    if (per_sm == 0) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, Cfg::COL_THREADS, TC::SMEM) != cudaSuccess ||
          per_sm < 1)
        per_sm = 1;
      per_sm_cache.store(per_sm, std::memory_order_relaxed);
    }
    const int64_t ntiles = (int64_t)(a.n0 / Cfg::CC) * a.B;
    const int64_t grid = std::min<int64_t>(ntiles, (int64_t)per_sm * (a.nsm > 0 ? a.nsm : 152));
    k<<<(unsigned)grid, Cfg::COL_THREADS, TC::SMEM, s>>>(a, tm[0], tm[1]);
    return (int)cudaGetLastError();
  }
}

template <typename Real, int M, int LOGN, int V = 0>
int launch_col_n(const PassArgs& a, cudaStream_t s) {
  using Cfg = LineCfg<Real, M, LOGN, V>;
  if (a.n0 % Cfg::CC) return (int)cudaErrorInvalidValue;
  if constexpr (V == 0) {
    if (a.col_tma) {
      const int r = launch_col_tma_n<Real, M, LOGN>(a, s);
      if (r >= 0) return r;
    }
  }
  auto k = col_kernel<Real, LOGN, M, V>;
  int e = set_smem(k, Cfg::COL_SMEM);
  if (e) return e;
  const int64_t blocks = (int64_t)(a.n0 / Cfg::CC) * a.nouter * a.B;
  k<<<(unsigned)blocks, Cfg::COL_THREADS, Cfg::COL_SMEM, s>>>(a);
  return (int)cudaGetLastError();
}
template <typename Real, int M, int LOGN>
int launch_line1d_n(const PassArgs& a, cudaStream_t s) {
  using Cfg = LineCfg<Real, M, LOGN>;
  auto k = line1d_kernel<Real, LOGN, M>;
  int e = set_smem(k, Cfg::ROW_SMEM);
  if (e) return e;
  const int64_t blocks = (a.B + Cfg::L - 1) / Cfg::L;
  k<<<(unsigned)blocks, Cfg::ROW_THREADS, Cfg::ROW_SMEM, s>>>(a, a.B);
  return (int)cudaGetLastError();
}

#define GPE_LOGN_SWITCH(FN, ...)                \
  switch (logn) {                               \
    case 4: return FN<Real, M, 4>(__VA_ARGS__);   \
    case 5: return FN<Real, M, 5>(__VA_ARGS__);   \
    case 6: return FN<Real, M, 6>(__VA_ARGS__);   \
    case 7: return FN<Real, M, 7>(__VA_ARGS__);   \
    case 8: return FN<Real, M, 8>(__VA_ARGS__);   \
    case 9: return FN<Real, M, 9>(__VA_ARGS__);   \
    case 10: return FN<Real, M, 10>(__VA_ARGS__); \
    case 11: return FN<Real, M, 11>(__VA_ARGS__); \
    case 12: return FN<Real, M, 12>(__VA_ARGS__); \
    default: return (int)cudaErrorInvalidValue;   \
  }

#define GPE_LOGN_SWITCH_V(FN, ...)                  \
  switch (logn) {                                   \
    case 4: return FN<Real, M, 4, V>(__VA_ARGS__);    \
    case 5: return FN<Real, M, 5, V>(__VA_ARGS__);    \
    case 6: return FN<Real, M, 6, V>(__VA_ARGS__);    \
    case 7: return FN<Real, M, 7, V>(__VA_ARGS__);    \
    case 8: return FN<Real, M, 8, V>(__VA_ARGS__);    \
    case 9: return FN<Real, M, 9, V>(__VA_ARGS__);    \
    case 10: return FN<Real, M, 10, V>(__VA_ARGS__);  \
    case 11: return FN<Real, M, 11, V>(__VA_ARGS__);  \
    case 12: return FN<Real, M, 12, V>(__VA_ARGS__);  \
    default: return (int)cudaErrorInvalidValue;     \
  }

template <typename Real, int M, int V = 0>
int launch_row_t(int logn, const PassArgs& a, int64_t nlines, cudaStream_t s) {
  GPE_LOGN_SWITCH_V(launch_row_n, a, nlines, s)
}
template <typename Real, int M, int V = 0>
int launch_col_t(int logn, const PassArgs& a, cudaStream_t s) {
  GPE_LOGN_SWITCH_V(launch_col_n, a, s)
}
template <typename Real, int M>
int launch_line1d_t(int logn, const PassArgs& a, cudaStream_t s) {
  GPE_LOGN_SWITCH(launch_line1d_n, a, s)
}
template <typename Real, int M>
int launch_plane_t(int logn, const PassArgs& a, cudaStream_t s) {
  switch (logn) {
    case 4: return launch_plane_n<Real, M, 4>(a, s);
    case 5: return launch_plane_n<Real, M, 5>(a, s);
    case 6: return launch_plane_n<Real, M, 6>(a, s);
    case 7: return launch_plane_n<Real, M, 7>(a, s);
    default: return (int)cudaErrorInvalidValue;
  }
}
// whether a 2^logn x 2^logn field of M components fits the resident kernel
template <typename Real, int M>
bool plane_fits_t(int logn) {
  switch (logn) {
    case 4: return PlaneCfg<Real, M, 4>::FITS;
    case 5: return PlaneCfg<Real, M, 5>::FITS;
    case 6: return PlaneCfg<Real, M, 6>::FITS;
    case 7: return PlaneCfg<Real, M, 7>::FITS;
    default: return false;
  }
}
template <typename Real, int M>
int launch_nl_only_t(const PassArgs& a, cudaStream_t s) {
  const int64_t total = a.P * a.B;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  nl_only_kernel<Real, M><<<(unsigned)blocks, 256, 0, s>>>(a);
  return (int)cudaGetLastError();
}
template <typename Real>
int launch_mat_t(const PassArgs& a, cudaStream_t s) {
  const int64_t total = a.P * a.B;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  mat_kernel<Real><<<(unsigned)blocks, 256, 0, s>>>(a);
  return (int)cudaGetLastError();
}
template <typename Real, int M>
int launch_norm_t(const PassArgs& a, double* out, cudaStream_t s) {
  const int64_t total = a.P * a.B;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  norm_kernel<Real, M><<<(unsigned)blocks, 256, 0, s>>>(a, out);
  return (int)cudaGetLastError();
}

#define GPE_INSTANTIATE_ROW(REAL, MM) \
  template int launch_row_t<REAL, MM, 0>(int, const PassArgs&, int64_t, cudaStream_t);
#define GPE_INSTANTIATE_COL(REAL, MM) \
  template int launch_col_t<REAL, MM, 0>(int, const PassArgs&, cudaStream_t);
#define GPE_INSTANTIATE_ROW_V(REAL, MM, VV) \
  template int launch_row_t<REAL, MM, VV>(int, const PassArgs&, int64_t, cudaStream_t);
#define GPE_INSTANTIATE_COL_V(REAL, MM, VV) \
  template int launch_col_t<REAL, MM, VV>(int, const PassArgs&, cudaStream_t);
#define GPE_INSTANTIATE_PLANE(REAL, MM)                                      \
  template int launch_plane_t<REAL, MM>(int, const PassArgs&, cudaStream_t);  \
  template bool plane_fits_t<REAL, MM>(int);
#define GPE_INSTANTIATE_MAT(REAL) template int launch_mat_t<REAL>(const PassArgs&, cudaStream_t);
#define GPE_INSTANTIATE_OTHER(REAL, MM)                                           \
  template int launch_line1d_t<REAL, MM>(int, const PassArgs&, cudaStream_t);    \
  template int launch_nl_only_t<REAL, MM>(const PassArgs&, cudaStream_t);        \
  template int launch_norm_t<REAL, MM>(const PassArgs&, double*, cudaStream_t);

}  // namespace gpe
