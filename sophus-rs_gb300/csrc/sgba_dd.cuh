// sgba_dd.cuh -- float-float ("double-float", 48-bit significand) arithmetic
// on the FP32 pipes.
//
// GB300 issues FP32 FMAs at 128 per clock per SM but FP64 at about 2, so the
// FP64-class sums this solver needs (Hessian, Schur complement, costs) are
// carried as unevaluated pairs hi + lo of floats.  The building blocks are the
// error-free transformations of Knuth (TwoSum), Dekker (FastTwoSum) and the
// FMA-based TwoProduct, combined as in Hida, Li and Bailey's double-double
// library ("Algorithms for quad-double precision floating point arithmetic",
// ARITH 2001) but on float components.  Explicit _rn intrinsics keep the
// compiler from contracting or reassociating the transformations.
#pragma once

#include <cuda_runtime.h>

struct dd {
  float hi;
  float lo;
};

__host__ __device__ __forceinline__ dd dd_make(float hi, float lo) {
  dd r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// Knuth TwoSum: s + e == a + b exactly.
__device__ __forceinline__ dd dd_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dd_make(s, e);
}

// Dekker FastTwoSum, valid when |a| >= |b| (or a == 0).
__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return dd_make(s, e);
}

// TwoProduct with FMA: p + e == a * b exactly.
__device__ __forceinline__ dd dd_two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return dd_make(p, e);
}

__device__ __forceinline__ dd dd_neg(dd a) { return dd_make(-a.hi, -a.lo); }

// a + b, both double-float (accurate variant: TwoSum on both components).
__device__ __forceinline__ dd dd_add(dd a, dd b) {
  dd s = dd_two_sum(a.hi, b.hi);
  dd t = dd_two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = dd_fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return dd_fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }

// a + b, b a float.
__device__ __forceinline__ dd dd_add_f(dd a, float b) {
  dd s = dd_two_sum(a.hi, b);
  s.lo = __fadd_rn(s.lo, a.lo);
  return dd_fast_two_sum(s.hi, s.lo);
}

// a * b
__device__ __forceinline__ dd dd_mul(dd a, dd b) {
  dd p = dd_two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
  p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
  return dd_fast_two_sum(p.hi, p.lo);
}

// a * b, b a float
__device__ __forceinline__ dd dd_mul_f(dd a, float b) {
  dd p = dd_two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return dd_fast_two_sum(p.hi, p.lo);
}

// c + a * b
__device__ __forceinline__ dd dd_fma(dd a, dd b, dd c) { return dd_add(c, dd_mul(a, b)); }

// a / b: long division with two float quotient digits and a correction
// (Hida-Li-Bailey "accurate" division restated for float components).
__device__ __forceinline__ dd dd_div(dd a, dd b) {
  float q1 = __fdiv_rn(a.hi, b.hi);
  dd r = dd_sub(a, dd_mul_f(b, q1));
  float q2 = __fdiv_rn(r.hi, b.hi);
  r = dd_sub(r, dd_mul_f(b, q2));
  float q3 = __fdiv_rn(r.hi, b.hi);
  dd q = dd_fast_two_sum(q1, q2);
  return dd_add_f(q, q3);
}

// sqrt(a) for a >= 0: one Newton correction of the float root, with the
// residual a - s*s formed exactly (Karp-Markstein style).
__device__ __forceinline__ dd dd_sqrt(dd a) {
  if (a.hi <= 0.0f) return dd_make(0.0f, 0.0f);
  float s = __fsqrt_rn(a.hi);
  dd s2 = dd_two_prod(s, s);
  dd e = dd_sub(a, s2);
  float corr = __fdiv_rn(e.hi, __fmul_rn(2.0f, s));
  return dd_fast_two_sum(s, corr);
}

__device__ __forceinline__ dd dd_from_double(double x) {
  float hi = __double2float_rn(x);
  float lo = __double2float_rn(x - static_cast<double>(hi));
  return dd_make(hi, lo);
}

__device__ __forceinline__ double dd_to_double(dd a) {
  return static_cast<double>(a.hi) + static_cast<double>(a.lo);
}

__device__ __forceinline__ dd dd_from_float(float x) { return dd_make(x, 0.0f); }

// Warp-level sum of a double-float (butterfly; every lane gets the total).
__device__ __forceinline__ dd dd_warp_sum(dd v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    dd o;
    o.hi = __shfl_xor_sync(0xffffffffu, v.hi, off);
    o.lo = __shfl_xor_sync(0xffffffffu, v.lo, off);
    v = dd_add(v, o);
  }
  return v;
}
