// gw_dfloat.h -- double-float numbers: a value held as the unevaluated sum of
// two FP32 numbers, hi + lo with |lo| <= ulp(hi) / 2, about 48 significant
// bits.  The engine's GW_DF64 precision stores every dial coefficient, the
// parameter values and the base weights this way and evaluates the dials and
// the per-event weight product on the FP32 pipe, whose rate on GB300 is many
// times the FP64 pipe's; the bin sums, the sums of squared weights and the
// likelihood stay in FP64.
//
// The arithmetic is the error-free-transformation method of Dekker ("A
// floating-point technique for extending the available precision", Numer.
// Math. 18, 1971) and Knuth (TAOCP vol. 2, 4.2.2: the two-sum), in the
// "double-double" arrangement of Hida, Li and Bailey ("Algorithms for
// quad-double precision floating point arithmetic", ARITH-15, 2001) applied
// to FP32 words, with the fused multiply-add forming the exact product error:
//   two_sum(a, b)      = (s, e), s = fl(a + b), a + b = s + e exactly;
//   fast_two_sum(a, b) = the same when |a| >= |b| (three operations);
//   a * b              = p + e with p = fl(a * b), e = fma(a, b, -p).
// A sum adds the low words together and carries the high words' exact
// rounding error (the "sloppy" sum of the double-double literature): its
// error is a few units of 2^-48 of the larger operand, which is what the
// reweighting needs (every value is a bounded combination of stored
// coefficients of similar size); a product carries a relative error of a few
// units of 2^-48 (about 1e-14); a quotient is formed from three corrected
// partial quotients.  Scaling by a power of two is exact (df_scale).
#pragma once
#include <cmath>

#ifndef GW_HD
#ifdef __CUDACC__
#define GW_HD __host__ __device__ __forceinline__
#else
#define GW_HD inline
#endif
#endif

namespace gw {

struct alignas(8) dfloat {
  float hi, lo;
  dfloat() = default;
  GW_HD constexpr dfloat(float h, float l) : hi(h), lo(l) {}
  GW_HD explicit constexpr dfloat(int i) : hi((float)i), lo(0.0f) {}  // exact for |i| < 2^24
  GW_HD explicit constexpr dfloat(float f) : hi(f), lo(0.0f) {}
  // Nearest double-float of a double: hi = the nearest float, lo = the
  // nearest float of the remainder (beyond the FP32 range: hi = +-inf, lo = 0).
  GW_HD explicit dfloat(double d) : hi(0.0f), lo(0.0f) {
    if (d > 3.4028234663852886e38) {
      hi = HUGE_VALF;
    } else if (d < -3.4028234663852886e38) {
      hi = -HUGE_VALF;
    } else {
      hi = (float)d;
      lo = (float)(d - (double)hi);
    }
  }
  GW_HD explicit operator double() const { return (double)hi + (double)lo; }
  // Truncation toward zero of hi + lo.
  GW_HD explicit operator int() const {
    int i = (int)hi;
    if ((float)i == hi) {
      if (hi > 0.0f && lo < 0.0f) --i;
      else if (hi < 0.0f && lo > 0.0f) ++i;
    }
    return i;
  }
};

#ifdef __CUDACC__
__device__ __forceinline__ dfloat df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return dfloat(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ dfloat df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dfloat(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ dfloat operator-(dfloat a) { return dfloat(-a.hi, -a.lo); }

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  const dfloat s = df_two_sum(a.hi, b.hi);
  return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return a + (-b); }

__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
// Exact product with a power of two.
__device__ __forceinline__ dfloat df_scale(dfloat a, float pow2) { return dfloat(a.hi * pow2, a.lo * pow2); }
// Product with a single float (its low word zero).
__device__ __forceinline__ dfloat df_mul_f(dfloat a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return df_fast_two_sum(p, e);
}

// Quotient: three partial quotients, each from the remainder of the ones
// before it, summed exactly (Hida, Li and Bailey's accurate division).
__device__ __forceinline__ dfloat df_div(dfloat a, dfloat b) {
  const float rb = __frcp_rn(b.hi);
  const float q1 = __fmul_rn(a.hi, rb);
  dfloat r = a - df_mul_f(b, q1);
  const float q2 = __fmul_rn(r.hi, rb);
  r = r - df_mul_f(b, q2);
  const float q3 = __fmul_rn(r.hi, rb);
  const dfloat q = df_fast_two_sum(q1, q2);
  return q + dfloat(q3);
}

__device__ __forceinline__ dfloat& operator+=(dfloat& a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat& operator-=(dfloat& a, dfloat b) { return a = a - b; }
__device__ __forceinline__ dfloat& operator*=(dfloat& a, dfloat b) { return a = a * b; }

__device__ __forceinline__ bool operator<(dfloat a, dfloat b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dfloat a, dfloat b) { return b < a; }
__device__ __forceinline__ bool operator<=(dfloat a, dfloat b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dfloat a, dfloat b) { return !(a < b); }
__device__ __forceinline__ bool operator==(dfloat a, dfloat b) { return a.hi == b.hi && a.lo == b.lo; }
#endif

}  // namespace gw
