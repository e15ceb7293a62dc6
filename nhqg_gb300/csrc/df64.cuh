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
// relative to |a| + |b| (below 2^-46), which is the norm-wise accuracy FFT
// butterflies need; products and fma stay within 2^-44 relative, the worst
// case being operands straight from the truncating FP64 split below (checked
// on the host by tests/df64_check.cu).  Every operation is written with the _rn intrinsics so
// that the compiler neither contracts a product into a later sum nor
// reorders the compensated steps.  The exponent range is FP32's: values
// below about 2^-103 lose their low word (the transforms' operands are
// relative to column norms far above that).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

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

// FP32 primitives, correctly rounded and never contracted or reordered: the
// _rn intrinsics on the device; plain IEEE operations on the host (the
// host-side accuracy check, compiled without FP contraction).
__host__ __device__ __forceinline__ float df_add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
__host__ __device__ __forceinline__ float df_sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
__host__ __device__ __forceinline__ float df_mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ __forceinline__ float df_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

__host__ __device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }

__host__ __device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const float s = df_add(a.hi, b.hi);
  const float bb = df_sub(s, a.hi);
  float e = df_add(df_sub(a.hi, df_sub(s, bb)), df_sub(b.hi, bb));
  e = df_add(e, df_add(a.lo, b.lo));
  const float h = df_add(s, e);
  return dfl(h, df_sub(e, df_sub(h, s)));
}
__host__ __device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }

__host__ __device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = df_mul(a.hi, b.hi);
  float e = df_fma(a.hi, b.hi, -p);
  e = df_fma(a.hi, b.lo, e);
  e = df_fma(a.lo, b.hi, e);
  const float h = df_add(p, e);
  return dfl(h, df_sub(e, df_sub(h, p)));
}

// a * b + c with one normalisation
__host__ __device__ __forceinline__ dfl fma(dfl a, dfl b, dfl c) {
  const float p = df_mul(a.hi, b.hi);
  float pe = df_fma(a.hi, b.hi, -p);
  pe = df_fma(a.hi, b.lo, pe);
  pe = df_fma(a.lo, b.hi, pe);
  const float s = df_add(p, c.hi);
  const float bb = df_sub(s, p);
  float e = df_add(df_sub(p, df_sub(s, bb)), df_sub(c.hi, bb));
  e = df_add(e, df_add(pe, c.lo));
  const float h = df_add(s, e);
  return dfl(h, df_sub(e, df_sub(h, s)));
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
__host__ __device__ __forceinline__ uint64_t df_bits64(double v) {
#ifdef __CUDA_ARCH__
  return static_cast<uint64_t>(__double_as_longlong(v));
#else
  uint64_t b;
  std::memcpy(&b, &v, 8);
  return b;
#endif
}
__host__ __device__ __forceinline__ float df_asf(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
__host__ __device__ __forceinline__ uint32_t df_asu(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
__host__ __device__ __forceinline__ float df_u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint2float_rn(u);
#else
  return static_cast<float>(u);
#endif
}
__host__ __device__ __forceinline__ double df_hilo(uint32_t hw, uint32_t lw) {
#ifdef __CUDA_ARCH__
  return __hiloint2double(static_cast<int>(hw), static_cast<int>(lw));
#else
  const uint64_t b = (static_cast<uint64_t>(hw) << 32) | lw;
  double d;
  std::memcpy(&d, &b, 8);
  return d;
#endif
}

__host__ __device__ __forceinline__ dfl df_from_double(double v) {
  const uint64_t b = df_bits64(v);
  const uint32_t hw = static_cast<uint32_t>(b >> 32);
  const int eb = static_cast<int>((hw >> 20) & 0x7FFu);  // biased FP64 exponent
  const int e = eb - 1023 + 127;
  const uint32_t sgn = hw & 0x80000000u;
  if (e <= 0) return dfl(0.f, 0.f);
  const uint32_t m = ((hw & 0xFFFFFu) << 3) | static_cast<uint32_t>((b >> 29) & 7u);
  const float hi = df_asf(sgn | (static_cast<uint32_t>(e) << 23) | m);
  // remainder: the low 29 significand bits times 2^(eb-1075) = 2^-29 2^(eb-1046)
  const uint32_t rbits = static_cast<uint32_t>(b & 0x1FFFFFFFu);
  const int er = eb - 1046 + 127;
  float lo = 0.f;
  if (er > 0)
    lo = df_mul(df_mul(df_u2f(rbits), df_asf(static_cast<uint32_t>(127 - 29) << 23)),
                df_asf(static_cast<uint32_t>(er) << 23));
  return dfl(hi, sgn ? -lo : lo);
}
// float -> double by rebiasing the exponent in integer arithmetic (exact;
// zero and magnitudes below 2^-126 give 0)
__host__ __device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t u = df_asu(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint32_t hw = e ? (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3) : 0u;
  const uint32_t lw = e ? (u << 29) : 0u;
  return df_hilo(hw, lw);
}
__host__ __device__ __forceinline__ double df_to_double(dfl a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }

__device__ __forceinline__ cdfl cdf_from(double2 v) { return cdfl{df_from_double(v.x), df_from_double(v.y)}; }
__device__ __forceinline__ double2 cdf_to(cdfl v) { return make_double2(df_to_double(v.x), df_to_double(v.y)); }

}  // namespace nhqg
