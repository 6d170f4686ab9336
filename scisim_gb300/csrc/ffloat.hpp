// ffloat.hpp -- float-float arithmetic: a value held as a pair of floats hi + lo (|lo| at most
// half an ulp of hi, 48 significant bits), with error-free sums and products (Knuth's two-sum,
// the FMA two-product) as in Dekker's double-length arithmetic (1971) and the double-double
// arithmetic of Hida, Li and Bailey, restated for pairs of floats.  The FP64-precision Gauss-Seidel
// sweeps for discs run in it on GB300's FP32 pipe.  Host and device code: on the device every
// operation is a round-to-nearest intrinsic (no contraction); on the host the same operations
// compile to IEEE single-precision arithmetic and fmaf (built without contraction), so that a host
// test can check the pairs' accuracy on any inputs.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define SG_FF_FN __host__ __device__ __forceinline__
#else
#define SG_FF_FN inline
#endif

namespace sg {

struct FF {
  float hi, lo;
};

SG_FF_FN float ff_fadd(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}

SG_FF_FN float ff_fsub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}

SG_FF_FN float ff_fmul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

SG_FF_FN float ff_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}

SG_FF_FN float ff_to_float(double x) {
#ifdef __CUDA_ARCH__
  return __double2float_rn(x);
#else
  return (float)x;
#endif
}

SG_FF_FN FF ff_make(float hi, float lo) {
  FF r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// x to 48 bits: the nearest float, then the nearest float to the (exact) remainder.
SG_FF_FN FF ff_split(double x) {
  const float h = ff_to_float(x);
  return ff_make(h, ff_to_float(x - (double)h));
}

// hi + lo exactly (the two floats' significands span at most 49 bits).
SG_FF_FN double ff_value(FF a) { return (double)a.hi + (double)a.lo; }

SG_FF_FN FF ff_two_sum(float a, float b) {
  const float s = ff_fadd(a, b);
  const float bb = ff_fsub(s, a);
  return ff_make(s, ff_fadd(ff_fsub(a, ff_fsub(s, bb)), ff_fsub(b, bb)));
}

SG_FF_FN FF ff_quick_two_sum(float a, float b) {
  const float s = ff_fadd(a, b);
  return ff_make(s, ff_fsub(b, ff_fsub(s, a)));
}

SG_FF_FN FF ff_neg(FF a) { return ff_make(-a.hi, -a.lo); }

SG_FF_FN FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  return ff_quick_two_sum(s.hi, ff_fadd(s.lo, ff_fadd(a.lo, b.lo)));
}

SG_FF_FN FF ff_sub(FF a, FF b) { return ff_add(a, ff_neg(b)); }

SG_FF_FN FF ff_add_f(FF a, float b) {
  const FF s = ff_two_sum(a.hi, b);
  return ff_quick_two_sum(s.hi, ff_fadd(s.lo, a.lo));
}

SG_FF_FN FF ff_mul(FF a, FF b) {
  const float p = ff_fmul(a.hi, b.hi);
  float e = ff_fma(a.hi, b.hi, -p);
  e = ff_fma(a.hi, b.lo, e);
  e = ff_fma(a.lo, b.hi, e);
  return ff_quick_two_sum(p, e);
}

}  // namespace sg
