// fft.cuh -- shared-memory Stockham line FFTs for sm_103a.
//
// The reference transforms each component with an FFTW / cuFFT plan over the
// spatial dims (src/misc.jl:53-64): an unnormalised forward transform, and an
// inverse scaled by 1/P.  Here a line of N = 2^LOGN points is transformed by
// T = N/E threads that each hold E points in registers.  Thread t always holds
// the points t + T*i (i < E) before and after every stage, so global loads and
// stores of a line are fully coalesced and the output is in natural order
// (Stockham autosort: no bit-reversal pass).  A stage of radix R (R | E) does
// E/R radix-R DFTs in registers; between stages the points are exchanged once
// through shared memory.  With R = E = 16 a 1024-point line takes 3 stages and
// 2 exchanges.
//
// Stage s (span NS = product of the earlier radices, radix R), butterfly j:
//   inputs  x[j + r*N/R], r < R
//   twiddle x_r *= w_N^{(j mod NS) * r * N/(NS*R)}
//   outputs y[(j/NS)*NS*R + (j mod NS) + r*NS] = DFT_R(x)_r
// (the self-sorting Stockham formulation of Van Loan, "Computational Frameworks
// for the Fast Fourier Transform", SIAM 1992, sec. 1.7).  In the last stage the
// output index equals the input slot, so no exchange follows it.
//
// Twiddles come from a per-length FP64-built table w_N^k = exp(-2 pi i k / N);
// the inverse uses its conjugate.  The in-register radix-R DFTs use the constants
// cos(2 pi k / 16).  FP32 passes hold both as FP32 hi/lo pairs and apply them with FMA
// corrections (cmul_hl), so no rounded constant biases every transform the same way.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "dw.cuh"

namespace gpe {

// Precision tags: double (native FP64), float (FP32) and DWR (double-word FP64 on the
// FP32 pipes, see dw.cuh).  CT<R>::T is the complex storage type.
struct DWR {};
template <typename Real> struct CT;
template <> struct CT<double> { using T = double2; };
template <> struct CT<float> { using T = float2; };
template <> struct CT<DWR> { using T = dwc; };

// read-only cached loads of complex table entries
__device__ __forceinline__ double2 ldgc(const double2* p) { return __ldg(p); }
__device__ __forceinline__ float2 ldgc(const float2* p) { return __ldg(p); }
__device__ __forceinline__ dwc ldgc(const dwc* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  dwc z;
  z.xh = v.x; z.xl = v.y; z.yh = v.z; z.yl = v.w;
  return z;
}

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {
  C r;
  r.x = a.x * b.x + a.y * b.y;
  r.y = a.y * b.x - a.x * b.y;
  return r;
}
template <typename C, typename R> __device__ __forceinline__ C cscale(C a, R s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }

// FP32 value times an FP64-accurate constant held as hi/lo float pairs (w = (xh + xl) +
// i (yh + yl)), with FMA corrections: the FP32 rounding of the product with the exact
// constant (within a few units of the last place, unbiased), where a plain FP32 constant
// would carry a fixed rounding error into every product with it.
__device__ __forceinline__ float2 cmul_hl(float2 v, dwc w) {
  float2 r;
  r.x = __fmaf_rn(v.x, w.xh, __fmaf_rn(-v.y, w.yh, __fmaf_rn(v.x, w.xl, -(v.y * w.yl))));
  r.y = __fmaf_rn(v.x, w.yh, __fmaf_rn(v.y, w.xh, __fmaf_rn(v.x, w.yl, v.y * w.xl)));
  return r;
}
// v * conj(w)
__device__ __forceinline__ float2 cmulc_hl(float2 v, dwc w) {
  float2 r;
  r.x = __fmaf_rn(v.x, w.xh, __fmaf_rn(v.y, w.yh, __fmaf_rn(v.x, w.xl, v.y * w.yl)));
  r.y = __fmaf_rn(v.y, w.xh, __fmaf_rn(-v.x, w.yh, __fmaf_rn(v.y, w.xl, -(v.x * w.yl))));
  return r;
}

// Twiddle tables: the complex type of the pass for FP64 and double-word passes, hi/lo
// float pairs (16 bytes an entry) for FP32 passes.
template <typename C> struct TwT { using T = C; };
template <> struct TwT<float2> { using T = dwc; };
template <typename C> __device__ __forceinline__ C twmul(C v, C w) { return cmul(v, w); }
template <typename C> __device__ __forceinline__ C twmulc(C v, C w) { return cmulc(v, w); }
__device__ __forceinline__ float2 twmul(float2 v, dwc w) { return cmul_hl(v, w); }
__device__ __forceinline__ float2 twmulc(float2 v, dwc w) { return cmulc_hl(v, w); }
template <typename C> __device__ __forceinline__ C cmake(double x, double y) { C r; r.x = x; r.y = y; return r; }

// cos(2 pi k / 16), k in [0, 16): exact constants of the regular 16-gon.
__host__ __device__ constexpr double cos16(int k) {
  k &= 15;
  return k == 0 ? 1.0
       : k == 1 || k == 15 ? 0.92387953251128675613
       : k == 2 || k == 14 ? 0.70710678118654752440
       : k == 3 || k == 13 ? 0.38268343236508977173
       : k == 4 || k == 12 ? 0.0
       : k == 5 || k == 11 ? -0.38268343236508977173
       : k == 6 || k == 10 ? -0.70710678118654752440
       : k == 7 || k == 9 ? -0.92387953251128675613
       : -1.0;
}
__host__ __device__ constexpr double sin16(int k) { return cos16(k - 4); }

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }
__host__ __device__ constexpr int bitrev(int v, int bits) {
  int r = 0;
  for (int i = 0; i < bits; ++i) r |= ((v >> i) & 1) << (bits - 1 - i);
  return r;
}

// d * w_n^i with w_n = exp(DIR * 2 pi i / n), n in {2,4,8,16}
template <int DIR, int n, int i, typename C>
__device__ __forceinline__ C twc(C d) {
  constexpr int k = (i * 16 / n) & 15;
  if constexpr (std::is_same<C, dwc>::value) {
    if constexpr (k == 0) {
      return d;
    } else if constexpr (k == 4) {  // w = DIR * i: (x, y) -> (-DIR y, DIR x)
      dwc r;
      r.xh = -DIR * d.yh; r.xl = -DIR * d.yl; r.yh = DIR * d.xh; r.yl = DIR * d.xl;
      return r;
    } else if constexpr (k == 8) {
      dwc r;
      r.xh = -d.xh; r.xl = -d.xl; r.yh = -d.yh; r.yl = -d.yl;
      return r;
    } else if constexpr (k == 12) {
      dwc r;
      r.xh = DIR * d.yh; r.xl = DIR * d.yl; r.yh = -DIR * d.xh; r.yl = -DIR * d.xl;
      return r;
    } else {
      dwc w;
      w.xh = dwh(cos16(k)); w.xl = dwl(cos16(k));
      w.yh = dwh(DIR * sin16(k)); w.yl = dwl(DIR * sin16(k));
      return cmul(d, w);
    }
  } else {
    if constexpr (k == 0) {
      return d;
    } else if constexpr (k == 4) {  // w = DIR * i
      C r; r.x = -DIR * d.y; r.y = DIR * d.x; return r;
    } else if constexpr (k == 8) {
      C r; r.x = -d.x; r.y = -d.y; return r;
    } else if constexpr (k == 12) {  // w = -DIR * i
      C r; r.x = DIR * d.y; r.y = -DIR * d.x; return r;
    } else if constexpr (std::is_same<C, float2>::value) {
      // FP32: the constant as an FP32 hi/lo pair with FMA corrections, so the product is
      // the FP32 rounding of d times the exact constant.  Plain FP32 constants are each
      // rounded once and |c + i s| misses 1 by a fixed amount (-3.4e-8 for cos = sin =
      // 1/sqrt 2), which every transform of every step repeats: a systematic drift of the
      // norm that grows linearly in time.
      constexpr float ch = dwh(cos16(k)), cl = dwl(cos16(k));
      constexpr float sh = dwh(DIR * sin16(k)), sl = dwl(DIR * sin16(k));
      float2 r;
      r.x = __fmaf_rn(d.x, ch, __fmaf_rn(-d.y, sh, __fmaf_rn(d.x, cl, -(d.y * sl))));
      r.y = __fmaf_rn(d.x, sh, __fmaf_rn(d.y, ch, __fmaf_rn(d.x, sl, d.y * cl)));
      return r;
    } else {
      using R = decltype(d.x);
      const R c = (R)cos16(k), s = (R)(DIR * sin16(k));
      C r; r.x = d.x * c - d.y * s; r.y = d.x * s + d.y * c; return r;
    }
  }
}

// Butterfly sums.  Double-word sums renormalise every result (dw_add closes with a
// FastTwoSum), so every value a butterfly passes on is a normalised pair: deferring that
// renormalisation to the end of the line transform saved 13 % of the double-word step
// but doubled its distance to FP64 on a collapsing Kerr packet (2048^2, 1000 steps:
// 1.5e-10 instead of 5.6e-11), which the 1e-10 parity bar does not allow.
template <typename C> __device__ __forceinline__ C badd(C a, C b) { return cadd(a, b); }
template <typename C> __device__ __forceinline__ C bsub(C a, C b) { return csub(a, b); }
template <typename C> __device__ __forceinline__ C bfinish(C a) { return a; }

// Radix-2 decimation-in-frequency layer of half-size H over an array of R points.
template <int R, int DIR, int H, int B, int I, typename C>
__device__ __forceinline__ void dif_bfly(C (&v)[R]) {
  C a = v[B + I], c = v[B + I + H];
  v[B + I] = badd(a, c);
  v[B + I + H] = twc<DIR, 2 * H, I>(bsub(a, c));
}
template <int R, int DIR, int H, int B, int I, typename C>
__device__ __forceinline__ void dif_row(C (&v)[R]) {
  if constexpr (I < H) {
    dif_bfly<R, DIR, H, B, I>(v);
    dif_row<R, DIR, H, B, I + 1>(v);
  }
}
template <int R, int DIR, int H, int B, typename C>
__device__ __forceinline__ void dif_blocks(C (&v)[R]) {
  if constexpr (B < R) {
    dif_row<R, DIR, H, B, 0>(v);
    dif_blocks<R, DIR, H, B + 2 * H>(v);
  }
}
template <int R, int DIR, int H, typename C>
__device__ __forceinline__ void dif_layers(C (&v)[R]) {
  if constexpr (H >= 1) {
    dif_blocks<R, DIR, H, 0>(v);
    dif_layers<R, DIR, H / 2>(v);
  }
}

// bit-reversed register order -> natural order
template <int R, typename C>
__device__ __forceinline__ void unscramble(C (&v)[R]) {
  C tmp[R];
#pragma unroll
  for (int k = 0; k < R; ++k) tmp[k] = v[bitrev(k, ilog2(R))];
#pragma unroll
  for (int k = 0; k < R; ++k) v[k] = tmp[k];
}

// In-register DFT of R points (R in {1,2,4,8,16}), natural order in and out.
template <int R, int DIR, typename C>
__device__ __forceinline__ void dft_regs(C (&v)[R]) {
  if constexpr (R > 1) {
    dif_layers<R, DIR, R / 2>(v);
    unscramble<R>(v);
  }
}

// FP64: the first decimation-in-frequency layer of a twiddled radix-R stage with the
// twiddle products taken into FMAs.  For the pair (I, I + H), a = x_I w_I and c = x_{I+H}
// w_{I+H}: a + c is one chain of two FMAs per part on top of a, and a - c = 2a - (a + c)
// one more FMA per part: 10 FP64 operations a pair instead of 12 (a complex product, a sum
// and a difference), 6 instead of 8 for I = 0 whose twiddle is 1.  The difference carries
// the sum's rounding, an error bounded by the pair's norm as an FFT butterfly's is.
template <int R, int DIR, int H, int I>
__device__ __forceinline__ void fused_first_layer(double2 (&v)[R], const double2 (&w)[R]) {
  if constexpr (I < H) {
    const double2 a = I == 0 ? v[0] : cmul(v[I], w[I]);
    const double2 c = v[I + H], wc = w[I + H];
    double2 sum, dif;
    sum.x = fma(c.x, wc.x, fma(-c.y, wc.y, a.x));
    sum.y = fma(c.x, wc.y, fma(c.y, wc.x, a.y));
    dif.x = fma(2.0, a.x, -sum.x);
    dif.y = fma(2.0, a.y, -sum.y);
    v[I] = sum;
    v[I + H] = twc<DIR, 2 * H, I>(dif);
    fused_first_layer<R, DIR, H, I + 1>(v, w);
  }
}

// ---------------------------------------------------------------- layouts
// Row layout: each line owns N consecutive shared-memory slots.  The exchange
// after a stage (NS, R) XOR-swizzles the slot within each 128-byte row with a key
// taken from the row number, chosen so that both the scattered stage writes and
// the strided reads of the next stage are free of bank conflicts.
template <typename C>
struct RowLayout {
  C* base;
  static constexpr int S = 128 / (int)sizeof(C);  // complex slots per 128-byte row
  static constexpr int LOGS = ilog2(S);
  template <int NS, int R>
  __device__ __forceinline__ int addr(int idx) const {
    constexpr int LOGR = ilog2(R);
    constexpr int A = (NS == 1) ? (LOGR > LOGS ? LOGR - LOGS : 0) : 0;
    constexpr int B = (NS > 1 && NS < S) ? (LOGS > LOGR ? LOGS - LOGR : 0) : 0;
    const int row = idx >> LOGS;
    return idx ^ (((row >> A) << B) & (S - 1));
  }
};

// Column layout: CC lines (columns) interleaved, point n of column c at n*CC + c; for
// 8-byte elements with one padding row after every 8 rows, (n + n/8)*CC + c.  The reads
// of a stage and the writes of the later stages touch consecutive rows; the first stage
// writes rows 8t + r for neighbouring threads t, which the padding spreads over both
// halves of the bank space (without it, 8-byte elements hit the same 16 banks four
// times over; 16-byte elements fill all 32 banks either way).
template <typename C, int CC>
struct ColLayout {
  static constexpr bool PAD = sizeof(C) == 8;
  C* base;  // already offset by the column index
  template <int NS, int R>
  __device__ __forceinline__ int addr(int idx) const { return (PAD ? idx + (idx >> 3) : idx) * CC; }
};

// One Stockham stage.  x: this thread's E points; t: thread index in the line.
template <typename C, int N, int E, int R, int NS, int DIR, bool LAST, class Lay>
__device__ __forceinline__ void fft_stage(C (&x)[E], int t, const Lay& lay, const typename TwT<C>::T* __restrict__ tw) {
  constexpr int T = N / E, Q = E / R;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = x[q + r * Q];
    const int j = t + q * T;
    if constexpr (std::is_same<C, double2>::value && NS > 1 && DIR < 0 && R > 1) {
      // FP64 forward stage: twiddles fused into the first butterfly layer
      const int k = j & (NS - 1);
      constexpr int TS = N / (NS * R);
      double2 w[R];
      w[0] = make_double2(1.0, 0.0);
#pragma unroll
      for (int r = 1; r < R; ++r) w[r] = ldgc(tw + k * r * TS);
      fused_first_layer<R, DIR, R / 2, 0>(v, w);
      dif_layers<R, DIR, R / 4>(v);
      unscramble<R>(v);
    } else {
      if constexpr (NS > 1) {
        const int k = j & (NS - 1);
        constexpr int TS = N / (NS * R);
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const auto w = ldgc(tw + k * r * TS);
          v[r] = (DIR < 0) ? twmul(v[r], w) : twmulc(v[r], w);
        }
      }
      dft_regs<R, DIR>(v);
    }
    if constexpr (LAST) {
#pragma unroll
      for (int r = 0; r < R; ++r) x[q + r * Q] = v[r];
    } else {
      const int jb = (j / NS) * NS * R + (j & (NS - 1));
#pragma unroll
      for (int r = 0; r < R; ++r) lay.base[lay.template addr<NS, R>(jb + r * NS)] = v[r];
    }
  }
}

template <typename C, int N, int E, int DIR, int NS, class Lay>
__device__ __forceinline__ void fft_stages(C (&x)[E], int t, const Lay& lay, const typename TwT<C>::T* __restrict__ tw) {
  constexpr int REM = N / NS;
  constexpr int R = REM >= E ? E : REM;
  constexpr bool LAST = (NS * R == N);
  constexpr int T = N / E;
  fft_stage<C, N, E, R, NS, DIR, LAST>(x, t, lay, tw);
  if constexpr (!LAST) {
    __syncthreads();
#pragma unroll
    for (int i = 0; i < E; ++i) x[i] = lay.base[lay.template addr<NS, R>(t + T * i)];
    __syncthreads();
    fft_stages<C, N, E, DIR, NS * R>(x, t, lay, tw);
  }
}

// Transform one line held as x[i] = point t + T*i.  DIR = -1 forward (unnormalised),
// DIR = +1 inverse (unnormalised; the 1/P factor is folded into the k-space table).
// Every thread of the block must call this the same number of times.  renorm: apply
// bfinish to the outputs (a no-op for every precision now that double-word butterflies
// renormalise as they go).
template <typename C, int N, int E, int DIR, class Lay>
__device__ __forceinline__ void fft_line(C (&x)[E], int t, const Lay& lay, const typename TwT<C>::T* __restrict__ tw,
                                         bool renorm = true) {
  fft_stages<C, N, E, DIR, 1>(x, t, lay, tw);
  if (renorm) {
#pragma unroll
    for (int i = 0; i < E; ++i) x[i] = bfinish(x[i]);
  }
}

// Joint transform of the M lines (components) a thread holds: each twiddle is loaded
// once for all components, and one pair of barriers per stage serves all of them.
// Component m exchanges through lay.base + m * cstride.
template <typename C, int N, int E, int R, int NS, int DIR, bool LAST, int M, class Lay>
__device__ __forceinline__ void fft_stage_joint(C (&x)[M][E], int t, const Lay& lay, int cstride,
                                                const typename TwT<C>::T* __restrict__ tw) {
  constexpr int T = N / E, Q = E / R;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    C v[M][R];
#pragma unroll
    for (int m = 0; m < M; ++m)
#pragma unroll
      for (int r = 0; r < R; ++r) v[m][r] = x[m][q + r * Q];
    const int j = t + q * T;
    if constexpr (NS > 1) {
      const int k = j & (NS - 1);
      constexpr int TS = N / (NS * R);
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const auto w = ldgc(tw + k * r * TS);
#pragma unroll
        for (int m = 0; m < M; ++m) v[m][r] = (DIR < 0) ? twmul(v[m][r], w) : twmulc(v[m][r], w);
      }
    }
#pragma unroll
    for (int m = 0; m < M; ++m) dft_regs<R, DIR>(v[m]);
    if constexpr (LAST) {
#pragma unroll
      for (int m = 0; m < M; ++m)
#pragma unroll
        for (int r = 0; r < R; ++r) x[m][q + r * Q] = v[m][r];
    } else {
      const int jb = (j / NS) * NS * R + (j & (NS - 1));
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int ad = lay.template addr<NS, R>(jb + r * NS);
#pragma unroll
        for (int m = 0; m < M; ++m) lay.base[m * cstride + ad] = v[m][r];
      }
    }
  }
}

template <typename C, int N, int E, int DIR, int NS, int M, class Lay>
__device__ __forceinline__ void fft_stages_joint(C (&x)[M][E], int t, const Lay& lay, int cstride,
                                                 const typename TwT<C>::T* __restrict__ tw) {
  constexpr int REM = N / NS;
  constexpr int R = REM >= E ? E : REM;
  constexpr bool LAST = (NS * R == N);
  constexpr int T = N / E;
  fft_stage_joint<C, N, E, R, NS, DIR, LAST, M>(x, t, lay, cstride, tw);
  if constexpr (!LAST) {
    __syncthreads();
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int ad = lay.template addr<NS, R>(t + T * i);
#pragma unroll
      for (int m = 0; m < M; ++m) x[m][i] = lay.base[m * cstride + ad];
    }
    __syncthreads();
    fft_stages_joint<C, N, E, DIR, NS * R, M>(x, t, lay, cstride, tw);
  }
}

template <typename C, int N, int E, int DIR, int M, class Lay>
__device__ __forceinline__ void fft_line_joint(C (&x)[M][E], int t, const Lay& lay, int cstride,
                                               const typename TwT<C>::T* __restrict__ tw) {
  fft_stages_joint<C, N, E, DIR, 1, M>(x, t, lay, cstride, tw);
#pragma unroll
  for (int m = 0; m < M; ++m)
#pragma unroll
    for (int i = 0; i < E; ++i) x[m][i] = bfinish(x[m][i]);
}

}  // namespace gpe
