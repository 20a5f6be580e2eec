// dw.cuh -- double-word ("float-float") arithmetic: FP64-class accuracy on the FP32 pipes.
//
// GB300 issues FP32 FMAs 62x faster than FP64 ones (measured: 74.7 vs 1.20 TFLOP/s), so
// the FP64 (GPE_C128) solver keeps its state as pairs of floats x = hi + lo with
// |lo| <= ulp(hi)/2, 48 significant bits (unit roundoff 2^-48 ~ 3.6e-15), and does its
// FFTs, table products and half steps with error-free transformations:
//   TwoSum (Knuth, TAOCP vol. 2, 4.2.2), FastTwoSum (Dekker 1971), TwoProd with FMA,
// combined as in Joldes, Muller, Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", ACM TOMS 44(2), 2017 (Alg. 5, 6, 9, 10).
// Every primitive uses the _rn intrinsics, which the compiler never contracts into an
// FMA or reassociates, so each transformation stays exact.
//
// A complex double-word number is stored as 16 bytes {re.hi, re.lo, im.hi, im.lo}: the
// same HBM and shared-memory footprint as a double2.
#pragma once
#include <cuda_runtime.h>

namespace gpe {

struct dw {
  float h, l;
};
struct __align__(16) dwc {
  float xh, xl, yh, yl;  // re = xh + xl, im = yh + yl
};

__device__ __forceinline__ dw two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ dw fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dw two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

// x + y, "sloppy" form (Joldes et al. Alg. 5): error <= 2^-47 (|x| + |y|); the FFT
// butterflies need only this normwise bound.
__device__ __forceinline__ dw dw_add(dw x, dw y) {
  const dw s = two_sum(x.h, y.h);
  const float v = __fadd_rn(x.l, y.l);
  const float w = __fadd_rn(s.l, v);
  return fast_two_sum(s.h, w);
}
__device__ __forceinline__ dw dw_neg(dw x) { return {-x.h, -x.l}; }
__device__ __forceinline__ dw dw_sub(dw x, dw y) { return dw_add(x, dw_neg(y)); }
// x + y with relative error <= 3u^2 even under cancellation (Alg. 6)
__device__ __forceinline__ dw dw_add_acc(dw x, dw y) {
  const dw s = two_sum(x.h, y.h);
  const dw t = two_sum(x.l, y.l);
  const float c = __fadd_rn(s.l, t.h);
  const dw v = fast_two_sum(s.h, c);
  const float w = __fadd_rn(t.l, v.l);
  return fast_two_sum(v.h, w);
}
// x * y (Alg. 10 form): relative error <= 7u^2
__device__ __forceinline__ dw dw_mul(dw x, dw y) {
  const float ch = __fmul_rn(x.h, y.h);
  const float cl1 = __fmaf_rn(x.h, y.h, -ch);
  const float tl = __fmul_rn(x.h, y.l);
  const float cl2 = __fmaf_rn(x.l, y.h, tl);
  const float cl3 = __fadd_rn(cl1, cl2);
  return fast_two_sum(ch, cl3);
}
// x * f for a float f (Alg. 9)
__device__ __forceinline__ dw dw_mulf(dw x, float f) {
  const float ch = __fmul_rn(x.h, f);
  const float cl1 = __fmaf_rn(x.h, f, -ch);
  const float cl3 = __fmaf_rn(x.l, f, cl1);
  return fast_two_sum(ch, cl3);
}
__device__ __forceinline__ dw dw_from(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ double dw_to_double(dw x) { return (double)x.h + (double)x.l; }

__device__ __forceinline__ dw re(const dwc& z) { return {z.xh, z.xl}; }
__device__ __forceinline__ dw im(const dwc& z) { return {z.yh, z.yl}; }
__device__ __forceinline__ dwc mk(dw r, dw i) { dwc z; z.xh = r.h; z.xl = r.l; z.yh = i.h; z.yl = i.l; return z; }

__device__ __forceinline__ dwc cadd(dwc a, dwc b) { return mk(dw_add(re(a), re(b)), dw_add(im(a), im(b))); }
__device__ __forceinline__ dwc csub(dwc a, dwc b) { return mk(dw_sub(re(a), re(b)), dw_sub(im(a), im(b))); }

// p*q - r*s (or + when SIGN = +1) for double-word p, q, r, s, rounded once: the two
// high products and their exact errors, the four first-order cross terms and two
// TwoSums.  Terms of order lo*lo (2^-48 relative) are dropped.  The closing sum is a full
// TwoSum: when the high products cancel, |hs.h| may be smaller than the error term e,
// which a FastTwoSum would not renormalise exactly.
template <int SIGN>
__device__ __forceinline__ dw dot2(dw p, dw q, dw r, dw s) {
  const float a = __fmul_rn(p.h, q.h);
  const float ea = __fmaf_rn(p.h, q.h, -a);
  const float b0 = __fmul_rn(r.h, s.h);
  const float eb = __fmaf_rn(r.h, s.h, -b0);
  const float b = SIGN > 0 ? b0 : -b0;
  const dw hs = two_sum(a, b);
  float cross = __fmul_rn(r.h, s.l);
  cross = __fmaf_rn(r.l, s.h, cross);
  cross = SIGN > 0 ? cross : -cross;
  cross = __fmaf_rn(p.h, q.l, cross);
  cross = __fmaf_rn(p.l, q.h, cross);
  const float e = __fadd_rn(__fadd_rn(hs.l, SIGN > 0 ? __fadd_rn(ea, eb) : __fsub_rn(ea, eb)), cross);
  return two_sum(hs.h, e);
}
__device__ __forceinline__ dwc cmul(dwc a, dwc b) {
  return mk(dot2<-1>(re(a), re(b), im(a), im(b)), dot2<+1>(re(a), im(b), im(a), re(b)));
}
// a * conj(b)
__device__ __forceinline__ dwc cmulc(dwc a, dwc b) {
  return mk(dot2<+1>(re(a), re(b), im(a), im(b)), dot2<-1>(im(a), re(b), re(a), im(b)));
}
__device__ __forceinline__ dwc cscale(dwc a, dw s) { return mk(dw_mul(re(a), s), dw_mul(im(a), s)); }

// constant double -> (hi, lo) at compile time
__host__ __device__ constexpr float dwh(double v) { return (float)v; }
__host__ __device__ constexpr float dwl(double v) { return (float)(v - (double)(float)v); }

}  // namespace gpe
