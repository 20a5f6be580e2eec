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

// ---------------------------------------------------------------- block floating point
// FP64 lines can be transformed on the integer pipes: GB300 runs two FP64 operations a
// clock per SM, but 64-bit integer adds at 32 and 32x32->64 multiply-adds fast enough
// for a complex product in Q62 fixed point at 2.7x the FP64 rate (both measured on the
// GB300).  A line is held as 64-bit integers with one exponent for the whole line
// (block floating point, the scheme of Oppenheim & Weinstein, "Effects of finite
// register length in digital filtering and the fast Fourier transform", Proc. IEEE
// 60(8), 1972): the input is scaled so that its largest component is just below 2^58,
// each radix-8 stage grows the largest component by at most 8 sqrt(2) (below 2^62), and
// at each exchange every value of the line is shifted right by the bits its largest
// component grew beyond 2^58 (rounded), so every stage again starts below 2^58.  Sums are
// exact; each product with a twiddle or an internal constant rounds to within one unit
// (2^-58 of the line's largest component), where an FP64 transform rounds every sum and
// product to 2^-53 of its own value.
struct __align__(16) fxc { long long x, y; };
// Q62 constant c + i s, each as hi * 2^32 + lo with lo signed (so that products of its
// halves are signed 32 x 32 -> 64 multiply-adds)
struct __align__(16) fxw { int ch, cl, sh, sl; };
template <> struct TwT<fxc> { using T = fxw; };
__device__ __forceinline__ fxw ldgc(const fxw* p) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(p));
  fxw w;
  w.ch = v.x; w.cl = v.y; w.sh = v.z; w.sl = v.w;
  return w;
}

// v << 2 (|v| < 2^61) as h * 2^32 + l, l signed
__device__ __forceinline__ void fx_split(long long v, int& h, int& l) {
  const long long s = v << 2;
  l = (int)(unsigned)s;
  h = (int)((s - (long long)l) >> 32);
}
// v * (c + i s) for Q62 c, s and components |v| < 2^60: (4v)(c + i s) / 2^64 from the
// 32-bit halves.  The middle partial products (with a rounding half unit) are summed
// first and shifted down, the low-by-low ones (below 1/8 unit) are dropped: the result is
// within 0.9 units of the exact product and unbiased.
__device__ __forceinline__ fxc fx_cmul(fxc v, int ch, int cl, int sh, int sl) {
  int rh, rl, ih, il;
  fx_split(v.x, rh, rl);
  fx_split(v.y, ih, il);
  long long tr = (long long)rh * cl + (1LL << 31);
  tr = (long long)rl * ch + tr;
  tr = (long long)(-ih) * sl + tr;
  tr = (long long)il * (-sh) + tr;  // il may be -2^31; |sh| <= 2^30
  long long ti = (long long)rh * sl + (1LL << 31);
  ti = (long long)rl * sh + ti;
  ti = (long long)ih * cl + ti;
  ti = (long long)il * ch + ti;
  fxc r;
  r.x = (long long)rh * ch + ((long long)(-ih) * sh + (tr >> 32));
  r.y = (long long)rh * sh + ((long long)ih * ch + (ti >> 32));
  return r;
}
__device__ __forceinline__ fxc twmul(fxc v, fxw w) { return fx_cmul(v, w.ch, w.cl, w.sh, w.sl); }
// the table's lo halves are never -2^31 (see the table builder), so -s splits as (-sh, -sl)
__device__ __forceinline__ fxc twmulc(fxc v, fxw w) { return fx_cmul(v, w.ch, w.cl, -w.sh, -w.sl); }

// Q62 of cos(2 pi k / 16), exactly rounded
__host__ __device__ constexpr long long q62_cos16(int k) {
  k &= 15;
  return k == 0 ? 4611686018427387904LL
       : k == 1 || k == 15 ? 4260642322793532497LL
       : k == 2 || k == 14 ? 3260954456333195553LL
       : k == 3 || k == 13 ? 1764815834521887442LL
       : k == 4 || k == 12 ? 0LL
       : k == 5 || k == 11 ? -1764815834521887442LL
       : k == 6 || k == 10 ? -3260954456333195553LL
       : k == 7 || k == 9 ? -4260642322793532497LL
       : -4611686018427387904LL;
}
__host__ __device__ constexpr int q62_lo(long long v) { return (int)(unsigned)(unsigned long long)v; }
__host__ __device__ constexpr int q62_hi(long long v) { return (int)((v - (long long)q62_lo(v)) >> 32); }

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
  if constexpr (std::is_same<C, fxc>::value) {
    if constexpr (k == 0) {
      return d;
    } else if constexpr (k == 4) {  // w = DIR * i
      fxc r; r.x = DIR < 0 ? d.y : -d.y; r.y = DIR < 0 ? -d.x : d.x; return r;
    } else if constexpr (k == 8) {
      fxc r; r.x = -d.x; r.y = -d.y; return r;
    } else if constexpr (k == 12) {  // w = -DIR * i
      fxc r; r.x = DIR < 0 ? -d.y : d.y; r.y = DIR < 0 ? d.x : -d.x; return r;
    } else {
      constexpr long long c = q62_cos16(k), s = DIR * q62_cos16(k - 4);
      return fx_cmul(d, q62_hi(c), q62_lo(c), q62_hi(s), q62_lo(s));
    }
  } else if constexpr (std::is_same<C, dwc>::value) {
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
//
// TL > 0: each line is held by TL threads of its own (whole warps, or a part of one warp),
// and the exchange barriers cover only the line (a named barrier of the line's warps, or
// the warp), so lines of one block can be at different points of their work.  TL = 0:
// block-wide barriers.
template <typename C, int TL = 0>
struct RowLayout {
  template <typename D> using rebind = RowLayout<D, TL>;
  C* base;
  __device__ __forceinline__ static void sync() {
    if constexpr (TL == 0) {
      __syncthreads();
    } else if constexpr (TL <= 32) {
      __syncwarp(blockDim.x >= 32 ? 0xffffffffu : (1u << blockDim.x) - 1u);
    } else {
      static_assert(TL % 32 == 0, "a line must be whole warps");
      // barrier 1 + line index, as immediates so that a block reserves only the ones it
      // uses; row blocks hold at most 256 threads, so at most NL lines
      constexpr int NL = TL >= 256 ? 1 : 256 / TL;
      const int l = threadIdx.x / TL;
      if (NL == 1 || l == 0) asm volatile("bar.sync 1, %0;" ::"n"(TL) : "memory");
      else if (NL == 2 || l == 1) asm volatile("bar.sync 2, %0;" ::"n"(TL) : "memory");
      else if (l == 2) asm volatile("bar.sync 3, %0;" ::"n"(TL) : "memory");
      else if (NL == 4 || l == 3) asm volatile("bar.sync 4, %0;" ::"n"(TL) : "memory");
      else if (l == 4) asm volatile("bar.sync 5, %0;" ::"n"(TL) : "memory");
      else if (l == 5) asm volatile("bar.sync 6, %0;" ::"n"(TL) : "memory");
      else if (l == 6) asm volatile("bar.sync 7, %0;" ::"n"(TL) : "memory");
      else asm volatile("bar.sync 8, %0;" ::"n"(TL) : "memory");
    }
  }
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
  template <typename D> using rebind = ColLayout<D, CC>;
  static constexpr bool PAD = sizeof(C) == 8;
  C* base;  // already offset by the column index
  __device__ __forceinline__ static void sync() { __syncthreads(); }
  template <int NS, int R>
  __device__ __forceinline__ int addr(int idx) const { return (PAD ? idx + (idx >> 3) : idx) * CC; }
};

// One Stockham stage.  x: this thread's E points; t: thread index in the line.
// Block floating point: the high word of |v| (one's complement for negative v) for the
// bit length of a line's largest component.  Lines are scaled so that their largest
// component exceeds 2^53, so the high words decide it.
__device__ __forceinline__ unsigned fx_mag(fxc v) {
  const int hx = (int)(v.x >> 32), hy = (int)(v.y >> 32);
  return (unsigned)(hx ^ (hx >> 31)) | (unsigned)(hy ^ (hy >> 31));
}

template <typename C, int N, int E, int R, int NS, int DIR, bool LAST, class Lay>
__device__ __forceinline__ void fft_stage(C (&x)[E], int t, const Lay& lay, const typename TwT<C>::T* __restrict__ tw,
                                          unsigned* mag = nullptr) {
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
      if constexpr (std::is_same<C, fxc>::value) {
#pragma unroll
        for (int r = 0; r < R; ++r) *mag |= fx_mag(v[r]);
      }
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
    lay.sync();
#pragma unroll
    for (int i = 0; i < E; ++i) x[i] = lay.base[lay.template addr<NS, R>(t + T * i)];
    lay.sync();
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
    lay.sync();
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int ad = lay.template addr<NS, R>(t + T * i);
#pragma unroll
      for (int m = 0; m < M; ++m) x[m][i] = lay.base[m * cstride + ad];
    }
    lay.sync();
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


// ---------------------------------------------------------------- block floating point lines
constexpr int FX_TOP = 58;  // a stage's input components stay below 2^FX_TOP

// Maximum over the threads of a line.  The threads of a line are those with equal
// threadIdx.x % G and equal threadIdx.x / (G * T): row lines (G = 1) are T consecutive
// threads, the G columns of a column tile interleave.  Lines inside one warp reduce with
// shuffles.  Wider lines publish one value a warp and column (G < 32), or one a thread
// (G >= 32, where a warp holds one thread of each of 32 lines), in red and read their
// line's values back after the caller's barrier.  Blocks narrower than a warp (a few
// short lines) shuffle under the mask of the threads they have.
template <int G, int T>
struct LineMax {
  static constexpr int W = G * T;
  static constexpr bool MULTI = W > 32;
  static constexpr int RED = G < 32 ? 32 * G : W;  // slots of red
  __device__ __forceinline__ static int warp(int v) {
    const unsigned mask = blockDim.x >= 32 ? 0xffffffffu : (1u << blockDim.x) - 1u;
#pragma unroll
    for (int off = G; off < (W < 32 ? W : 32); off *= 2) v = max(v, __shfl_xor_sync(mask, v, off));
    return v;
  }
  __device__ __forceinline__ static void publish(int v, int* red) {
    if constexpr (MULTI) {
      if constexpr (G < 32) {
        const int lane = threadIdx.x & 31;
        if (lane < G) red[(threadIdx.x >> 5) * G + lane] = v;
      } else {
        red[threadIdx.x % W] = v;
      }
    }
  }
  __device__ __forceinline__ static int collect(int v, const int* red) {
    if constexpr (MULTI) {
      const int c = threadIdx.x % G;
      if constexpr (G < 32) {
        const int w0 = (int)(threadIdx.x / W) * (W / 32);
        int r = red[w0 * G + c];
#pragma unroll
        for (int w = 1; w < W / 32; ++w) r = max(r, red[(w0 + w) * G + c]);
        return r;
      } else {
        int r = red[c];
#pragma unroll
        for (int j = 1; j < T; ++j) r = max(r, red[c + G * j]);
        return r;
      }
    } else {
      return v;
    }
  }
};

// round(v * 2^(FX_TOP + 1022 - emax)) for a component v of a line whose largest biased
// exponent is emax (so |v| < 2^(emax - 1022) maps below 2^FX_TOP); zero and subnormals
// (below 2^-1022) give 0.  Integer operations only.
__device__ __forceinline__ long long fx_from_double(double v, int emax) {
  const long long b = __double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  // the significand with its leading bit, times 2^6 (below 2^59); zero and subnormals: 0
  const unsigned long long m6 = e ? ((b & 0xfffffffffffffULL) | 0x10000000000000ULL) << 6 : 0ull;
  // v 2^(FX_TOP + 1022 - emax) = m 2^(5 - s) = m6 2^-(s + 1), s = emax - e >= 0: shift right by
  // s, then by one more with the rounding half unit (exact for s <= 5; branch-free)
  static_assert(FX_TOP == 58, "the shifts below place the top at 2^58");
  const int s = min(emax - e, 63);
  const long long r = (long long)(((m6 >> s) + 1) >> 1);
  return b < 0 ? -r : r;
}
// r * 2^eb rounded to the nearest double (ties away from zero), integer operations only;
// results below the normal range are flushed to zero
__device__ __forceinline__ double fx_to_double(long long r, int eb) {
  const unsigned long long a = r < 0 ? 0ull - (unsigned long long)r : (unsigned long long)r;
  const int lz = __clzll((long long)a);
  const unsigned long long n = a << (lz & 63);
  const unsigned long long mant = ((n >> 10) + 1) >> 1;  // 53 bits, 2^53 when rounding carries
  // a = mant 2^(11 - lz): biased exponent 1086 - lz + eb; mant's leading bit adds one
  const int E = 1086 - lz + eb;
  unsigned long long bits = ((unsigned long long)(E - 1) << 52) + mant;
  if (a == 0 || E <= 0) bits = 0;
  if (E >= 2047) bits = 0x7ff0000000000000ull;
  return __longlong_as_double((long long)(bits | ((unsigned long long)r & 0x8000000000000000ull)));
}

// Stockham stages on block floating point values: after every stage but the last the
// line's largest component (bit length from the high words of what each thread wrote) is
// reduced over the line across the exchange barrier, and the values read back are shifted
// right by its excess over FX_TOP, rounded; shsum collects the shifts.
template <int N, int E, int NS, class Lay, class LM>
__device__ __forceinline__ void fx_stages(fxc (&x)[E], int t, const Lay& lay, const fxw* __restrict__ tw, int* red,
                                          int& shsum) {
  static_assert(E <= 8, "radix-16 stages would exceed the 63-bit headroom");
  constexpr int REM = N / NS;
  constexpr int R = REM >= E ? E : REM;
  constexpr bool LAST = (NS * R == N);
  constexpr int T = N / E;
  unsigned mag = 0;
  fft_stage<fxc, N, E, R, NS, -1, LAST>(x, t, lay, tw, &mag);
  if constexpr (!LAST) {
    const int lw = LM::warp(mag ? 64 - __clz((int)mag) : 32);
    LM::publish(lw, red);
    lay.sync();
#pragma unroll
    for (int i = 0; i < E; ++i) x[i] = lay.base[lay.template addr<NS, R>(t + T * i)];
    const int sh = max(0, LM::collect(lw, red) - FX_TOP);
    if (sh > 0) {
      const long long half = 1LL << (sh - 1);
#pragma unroll
      for (int i = 0; i < E; ++i) {
        x[i].x = (x[i].x + half) >> sh;
        x[i].y = (x[i].y + half) >> sh;
      }
    }
    shsum += sh;
    lay.sync();
    fx_stages<N, E, NS * R, Lay, LM>(x, t, lay, tw, red, shsum);
  }
}

// Forward (unnormalised) transform of one line of FP64 values in block floating point;
// lay: the line's exchange space viewed as fxc, tw: the Q62 twiddle table.  A line holding
// an infinity or NaN comes out as NaN.  Every thread of the block calls this the same number
// of times (it holds barriers); N > E.
template <int N, int E, int G, class Lay>
__device__ __forceinline__ void fx_line(double2 (&x)[E], int t, const Lay& lay, const fxw* __restrict__ tw) {
  static_assert(N > E, "one-stage lines have no exchange to reduce across");
  using LM = LineMax<G, N / E>;
  __shared__ int red_in[LM::RED], red_x[LM::RED];
  // largest biased exponent of the line (from the high words, integer compares)
  unsigned hm = 0;
#pragma unroll
  for (int i = 0; i < E; ++i) {
    hm = max(hm, (unsigned)__double2hiint(x[i].x) & 0x7fffffffu);
    hm = max(hm, (unsigned)__double2hiint(x[i].y) & 0x7fffffffu);
  }
  int em = LM::warp((int)(hm >> 20));
  LM::publish(em, red_in);
  if constexpr (LM::MULTI) lay.sync();
  em = LM::collect(em, red_in);
  fxc v[E];
#pragma unroll
  for (int i = 0; i < E; ++i) {
    v[i].x = fx_from_double(x[i].x, em);
    v[i].y = fx_from_double(x[i].y, em);
  }
  int shsum = 0;
  fx_stages<N, E, 1, Lay, LM>(v, t, lay, tw, red_x, shsum);
  const int eb = em - 1022 - FX_TOP + shsum;
  const bool bad = em == 0x7ff;
#pragma unroll
  for (int i = 0; i < E; ++i) {
    x[i].x = bad ? __longlong_as_double(0x7ff8000000000000LL) : fx_to_double(v[i].x, eb);
    x[i].y = bad ? __longlong_as_double(0x7ff8000000000000LL) : fx_to_double(v[i].y, eb);
  }
}

}  // namespace gpe
