// gt_dfloat.cuh -- double-float arithmetic: FP64-accurate element math on
// the FP32 pipes.
//
// On GB300 the FP64 units run at about 1/58 of the FP32 rate, so a kernel
// whose arithmetic is FP64 (the P1 element kernel: ~75 FP64 operations per
// cell) is FP64-pipe bound.  A double-float number is an unevaluated sum
// hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2: 48 significant bits.
// Its operations are built from the error-free transformations of the
// published literature -- Knuth's two-sum (TAOCP vol. 2, 4.2.2), Dekker's
// fast two-sum (|a| >= |b|; Dekker 1971) and the FMA-based two-product
// (the product's rounding error is fma(a, b, -a*b)) -- so each double-float
// operation costs 3-20 FP32 instructions and carries a relative error of a
// few units of 2^-48.  Conversions from and to FP64 are done with integer
// instructions on the bit patterns (no FP64 instruction).
//
// Every addition and multiplication below is an explicit round-to-nearest
// intrinsic (__fadd_rn, __fmul_rn, __fsub_rn, __fmaf_rn): the compiler must
// neither contract a product into a following addition nor reassociate,
// or the error terms would be lost.
#pragma once

#include <cstdint>

namespace gt {

struct alignas(8) dfl {
  float hi, lo;
};

// s + e == a + b exactly (Knuth)
__device__ __forceinline__ dfl df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// s + e == a + b exactly when |a| >= |b| or a == 0 (Dekker)
__device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

// x + y with both error terms carried (the accurate double-float sum)
__device__ __forceinline__ dfl df_add(dfl x, dfl y) {
  const dfl s = df_two_sum(x.hi, y.hi);
  const dfl t = df_two_sum(x.lo, y.lo);
  const dfl u = df_fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return df_fast_two_sum(u.hi, __fadd_rn(u.lo, t.lo));
}

// x + y with one two-sum of the high parts and the low parts added in FP32
// (Dekker's / Bailey's "sloppy" sum: absolute error about 2^-47 of the
// larger operand, not of the result -- enough for sums whose terms are all
// of the size of the result, such as a matrix entry over its cells)
__device__ __forceinline__ dfl df_add_sloppy(dfl x, dfl y) {
  const dfl s = df_two_sum(x.hi, y.hi);
  return df_fast_two_sum(s.hi, __fadd_rn(__fadd_rn(x.lo, y.lo), s.lo));
}

__device__ __forceinline__ dfl df_neg(dfl x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ dfl df_sub(dfl x, dfl y) { return df_add(x, df_neg(y)); }
__device__ __forceinline__ dfl df_abs(dfl x) { return x.hi < 0.0f ? df_neg(x) : x; }

// x * y: the rounding error of hi*hi from the FMA, plus the two cross terms
// (added in one commutative order, so df_mul(x, y) == df_mul(y, x) bitwise:
// the difference of two equal products is exactly zero, as in FP64)
__device__ __forceinline__ dfl df_mul(dfl x, dfl y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fadd_rn(e, __fadd_rn(__fmul_rn(x.hi, y.lo), __fmul_rn(x.lo, y.hi)));
  return df_fast_two_sum(p, e);
}

// a*b - c*d
__device__ __forceinline__ dfl df_mul_sub(dfl a, dfl b, dfl c, dfl d) { return df_sub(df_mul(a, b), df_mul(c, d)); }

// x . y of two 3-vectors, summed left to right
__device__ __forceinline__ dfl df_dot3(const dfl* x, const dfl* y) {
  return df_add(df_add(df_mul(x[0], y[0]), df_mul(x[1], y[1])), df_mul(x[2], y[2]));
}

// 1 / x by Newton's iteration r <- r + r (1 - x r) from the FP32 reciprocal
// (each step doubles the correct bits: 24 -> 48)
__device__ __forceinline__ dfl df_recip(dfl x) {
  dfl r = {__frcp_rn(x.hi), 0.0f};
  const dfl one = {1.0f, 0.0f};
#pragma unroll
  for (int it = 0; it < 2; it++) r = df_add(r, df_mul(r, df_sub(one, df_mul(x, r))));
  return r;
}

// The rare cases of the two conversions below, in FP64 arithmetic.  Out of
// line on purpose: inlined, the compiler may if-convert them into the common
// path, and their FP64 instructions would then issue (predicated off) for
// every value converted.
static __device__ __noinline__ dfl df_from_double_rare(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}

static __device__ __noinline__ double df_to_double_rare(float hi, float lo) { return (double)hi + (double)lo; }

// The same operations with the sloppy sum (df_add_sloppy): absolute error
// about 2^-47 of the operands rather than of the result -- for formulas
// whose accuracy is measured against their largest terms (an element
// matrix against its largest entry), at about half the instructions of the
// accurate sum
__device__ __forceinline__ dfl df_sub_s(dfl x, dfl y) { return df_add_sloppy(x, df_neg(y)); }
__device__ __forceinline__ dfl df_mul_sub_s(dfl a, dfl b, dfl c, dfl d) { return df_sub_s(df_mul(a, b), df_mul(c, d)); }
__device__ __forceinline__ dfl df_dot3_s(const dfl* x, const dfl* y) {
  return df_add_sloppy(df_add_sloppy(df_mul(x[0], y[0]), df_mul(x[1], y[1])), df_mul(x[2], y[2]));
}
__device__ __forceinline__ dfl df_recip_s(dfl x) {
  dfl r = {__frcp_rn(x.hi), 0.0f};
  const dfl one = {1.0f, 0.0f};
#pragma unroll
  for (int it = 0; it < 2; it++) r = df_add_sloppy(r, df_mul(r, df_sub_s(one, df_mul(x, r))));
  return r;
}

// FP64 -> double-float with integer instructions: hi takes the top 24
// significand bits of x (exact), lo the remaining 29 bits rounded to FP32.
// Zeros stay integer too; other values outside |x| in [2^-74, 2^127) take
// the FP64 conversion instead.  (Conversions between FP64 and FP32 run on
// GB300's FP64 pipe, measured slower than a DFMA: ~0.74 lanes per clock per
// SM, so the common cases here use none.)
__device__ __forceinline__ dfl df_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if ((b << 1) == 0) return {__uint_as_float((unsigned)(b >> 32) & 0x80000000u), 0.0f};  // +-0
  const int e = (int)((b >> 52) & 0x7ff);
  if (e < 949 || e > 1149) return df_from_double_rare(x);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const float hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
  // remainder: (b & (2^29 - 1)) * 2^(e - 1075); the scale is a normal FP32 power of two
  const float rem = __uint2float_rn((unsigned)(b & 0x1fffffffu));
  const float scale = __uint_as_float((unsigned)(e - 948) << 23);
  const float lo = __fmul_rn(rem, scale);
  return {hi, sign ? -lo : lo};
}

// double-float -> FP64 with integer instructions: hi and lo aligned in one
// 64-bit signed significand, summed exactly, normalised to 53 bits
// (truncating at most one bit: the result is within 1 ulp of hi + lo)
__device__ __forceinline__ double df_to_double(dfl v) {
  const unsigned hb = __float_as_uint(v.hi), lb = __float_as_uint(v.lo);
  if ((hb << 1) == 0 && (lb << 1) == 0) return __longlong_as_double((long long)(hb >> 31) << 63);  // +-0
  const int eh = (int)((hb >> 23) & 0xff), el = (int)((lb >> 23) & 0xff);
  if (eh == 0 || eh == 255 || (el == 0 && (lb & 0x7fffffffu) != 0))
    return df_to_double_rare(v.hi, v.lo);  // zero, subnormal or non-finite parts: FP64 arithmetic
  // hi = mh * 2^(eh - 150), unit of the sum: 2^(eh - 179)
  long long H = (long long)((hb & 0x7fffffu) | 0x800000u) << 29;
  if (hb >> 31) H = -H;
  long long L = 0;
  if (el != 0) {
    const long long ml = (long long)((lb & 0x7fffffu) | 0x800000u);
    const int sh = el - eh + 29;  // lo's significand shifted into the unit of the sum
    if (sh >= 0) L = ml << sh;
    else if (sh > -40) L = ml >> (-sh);
    if (lb >> 31) L = -L;
  }
  long long S = H + L;
  if (S == 0) return 0.0;
  const unsigned long long neg = S < 0 ? 1ull : 0ull;
  unsigned long long m = (unsigned long long)(S < 0 ? -S : S);
  const int lz = __clzll((long long)m);
  const int shift = 11 - lz;  // brings the leading 1 to bit 52
  if (shift > 0) m >>= shift;
  else m <<= -shift;
  const long long E = (long long)eh + shift + 896;
  return __longlong_as_double((long long)((neg << 63) | ((unsigned long long)E << 52) | (m & 0xfffffffffffffull)));
}

}  // namespace gt
