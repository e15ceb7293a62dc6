// Double-float arithmetic: a value is an unevaluated sum hi + lo of two FP32
// numbers (about 48 significant bits), computed on the FP32 pipe.  GB300
// retires FP64 at 1/64 of its FP32 rate, so the mixed-precision path runs
// its FFT-based vertical transforms in this format where FP32 is too coarse
// (the mean-exchange corrector maps the state itself through them).
//
// The operations are the classical error-free transformations: TwoSum
// (Knuth, TAOCP vol. 2, 4.2.2), Fast2Sum (Dekker 1971) and the FMA-based
// exact product (a*b - fl(a*b) = fma(a, b, -fl(a*b))); addition is the
// "sloppy" double-float sum of Dekker's scheme, whose error is bounded
// relative to |a| + |b| (about 2^-47), which is the norm-wise accuracy FFT
// butterflies need.  Every operation is written with the _rn intrinsics so
// that the compiler neither contracts a product into a later sum nor
// reorders the compensated steps.  The exponent range is FP32's: values
// below about 2^-103 lose their low word (the transforms' operands are
// relative to column norms far above that).
#pragma once
#include <cstdint>

#include "common.cuh"

namespace nhqg {

// the overloads below must not hide the built-in ones inside this namespace
using ::fma;
using ::__shfl_xor_sync;
using ::__shfl_up_sync;
using ::__shfl_down_sync;

struct __align__(8) dfl {
  float hi, lo;
  dfl() = default;
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  // from a double (constants and host tables): nearest float, then the
  // rounded remainder
  __host__ __device__ dfl(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

// 16-byte aligned like double2, so that a complex value moves in one
// 128-bit shared-memory access
struct __align__(16) cdfl {
  dfl x, y;
};

__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }

__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  const float h = __fadd_rn(s, e);
  return dfl(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }

__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const float h = __fadd_rn(p, e);
  return dfl(h, __fsub_rn(e, __fsub_rn(h, p)));
}

// a * b + c with one normalisation
__device__ __forceinline__ dfl fma(dfl a, dfl b, dfl c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float pe = __fmaf_rn(a.hi, b.hi, -p);
  pe = __fmaf_rn(a.hi, b.lo, pe);
  pe = __fmaf_rn(a.lo, b.hi, pe);
  const float s = __fadd_rn(p, c.hi);
  const float bb = __fsub_rn(s, p);
  float e = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(c.hi, bb));
  e = __fadd_rn(e, __fadd_rn(pe, c.lo));
  const float h = __fadd_rn(s, e);
  return dfl(h, __fsub_rn(e, __fsub_rn(h, s)));
}

__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { return a = a - b; }
__device__ __forceinline__ dfl& operator*=(dfl& a, dfl b) { return a = a * b; }

__device__ __forceinline__ dfl __shfl_xor_sync(unsigned mask, dfl v, int o, int width = 32) {
  return dfl(__shfl_xor_sync(mask, v.hi, o, width), __shfl_xor_sync(mask, v.lo, o, width));
}
__device__ __forceinline__ dfl __shfl_up_sync(unsigned mask, dfl v, unsigned d, int width = 32) {
  return dfl(__shfl_up_sync(mask, v.hi, d, width), __shfl_up_sync(mask, v.lo, d, width));
}
__device__ __forceinline__ dfl __shfl_down_sync(unsigned mask, dfl v, unsigned d, int width = 32) {
  return dfl(__shfl_down_sync(mask, v.hi, d, width), __shfl_down_sync(mask, v.lo, d, width));
}

// FP64 -> double-float in integer arithmetic (no FP64 operation): the high
// word is the significand truncated to 24 bits, the low word the remaining 29
// bits rounded to 24 and scaled by the exponent (relative error below
// 2^-46.7 for magnitudes above 2^-103; smaller magnitudes keep the high word
// only, and below 2^-126 flush to zero).  Back to FP64: both words widened
// exactly in integer arithmetic, then one FP64 addition (an integer assembly
// of the sum itself, with 64-bit shifts, rounding and renormalisation,
// measured slower on GB300).
__device__ __forceinline__ dfl df_from_double(double v) {
  const uint64_t b = static_cast<uint64_t>(__double_as_longlong(v));
  const uint32_t hw = static_cast<uint32_t>(b >> 32);
  const int eb = static_cast<int>((hw >> 20) & 0x7FFu);  // biased FP64 exponent
  const int e = eb - 1023 + 127;
  const uint32_t sgn = hw & 0x80000000u;
  if (e <= 0) return dfl(0.f, 0.f);
  const uint32_t m = ((hw & 0xFFFFFu) << 3) | static_cast<uint32_t>((b >> 29) & 7u);
  const float hi = __uint_as_float(sgn | (static_cast<uint32_t>(e) << 23) | m);
  // remainder: the low 29 significand bits times 2^(eb-1075) = 2^-29 2^(eb-1046)
  const uint32_t rbits = static_cast<uint32_t>(b & 0x1FFFFFFFu);
  const int er = eb - 1046 + 127;
  float lo = 0.f;
  if (er > 0)
    lo = __fmul_rn(__fmul_rn(__uint2float_rn(rbits), __uint_as_float(static_cast<uint32_t>(127 - 29) << 23)),
                   __uint_as_float(static_cast<uint32_t>(er) << 23));
  return dfl(hi, sgn ? -lo : lo);
}
// float -> double by rebiasing the exponent in integer arithmetic (exact;
// zero and magnitudes below 2^-126 give 0)
__device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint32_t hw = e ? (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3) : 0u;
  const uint32_t lw = e ? (u << 29) : 0u;
  return __hiloint2double(static_cast<int>(hw), static_cast<int>(lw));
}
__device__ __forceinline__ double df_to_double(dfl a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }

__device__ __forceinline__ cdfl cdf_from(double2 v) { return cdfl{df_from_double(v.x), df_from_double(v.y)}; }
__device__ __forceinline__ double2 cdf_to(cdfl v) { return make_double2(df_to_double(v.x), df_to_double(v.y)); }

}  // namespace nhqg
