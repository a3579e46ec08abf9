// Double-float helpers shared by the kernels that move FP64 work to the
// FP32 pipes.
#pragma once

#include <cuda_runtime.h>

namespace tbsla_gpu {

// Double-float arithmetic: a value is the unevaluated sum h + l of two
// floats (about 46 significant bits; Dekker 1971, TwoSum after Knuth).  The
// batched PageRank and the DENSE GEMV with FP32 / BF16 values use it: their
// FP64 multiply-adds held GB300's narrow FP64 pipe 80-97% busy, and FP32 runs
// 64 times faster.  Every step is a round-to-nearest intrinsic, so nothing is
// contracted or reassociated.
struct DF {
  float h, l;
};
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  DF s = two_sum(a.h, b.h);
  const DF t = two_sum(a.l, b.l);
  s = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
  return fast_two_sum(s.h, __fadd_rn(s.l, t.l));
}
// a + b for double-float values of the same sign: one two_sum of the high
// parts, the low parts added to its error, then renormalised (the "sloppy"
// double-word addition of Dekker 1971; Joldes, Muller & Popescu 2017,
// Algorithm 5).  Without cancellation its relative error stays within a few
// units of 2^-48, and in any case its absolute error within a few units of
// 2^-48 (|a| + |b|); operands that may cancel take df_add.
__device__ __forceinline__ DF df_add_same_sign(DF a, DF b) {
  const DF s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float pr = __fmul_rn(a.h, b.h);
  const float e = __fmaf_rn(a.l, b.h, __fmaf_rn(a.h, b.l, __fmaf_rn(a.h, b.h, -pr)));
  return fast_two_sum(pr, e);
}
// One term of a compensated dot product (Ogita, Rump and Oishi 2005,
// Dot2): sum s plus error c gathers a (xh + xl), with the product's and the
// sum's rounding errors carried exactly into c; the row's value is s + c.
__device__ __forceinline__ void dot2_step(float& s, float& c, float a, DF x) {
  const float pr = __fmul_rn(a, x.h);
  const float e1 = __fmaf_rn(a, x.h, -pr);
  const DF t = two_sum(s, pr);
  s = t.h;
  c = __fmaf_rn(a, x.l, __fadd_rn(c, __fadd_rn(e1, t.l)));
}
__device__ __forceinline__ DF df_neg(DF a) { return {-a.h, -a.l}; }
__device__ __forceinline__ DF df_of(double d) {
  const float h = __double2float_rn(d);
  return {h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double df_val(DF a) { return (double)a.h + (double)a.l; }

}  // namespace tbsla_gpu
