// Double-float arithmetic: a value is an unevaluated sum hi + lo of two
// float32 numbers (about 46 significant bits), computed with the error-free
// transformations of Knuth (TwoSum), Dekker (Fast2Sum) and the FMA product
// residual.  On GB300 a float64 warp instruction occupies the float64 pipe
// for about 64 cycles of a scheduler, a float32 instruction for one, so a
// double-float update v - l a (about 12 float32 instructions) is several
// times cheaper than one float64 FMA.
//
// Normalised pairs have hi = fl32(hi + lo); the accumulators of df_fms_acc
// may be unnormalised (any s + t) until df_norm.  Every operation is written
// with round-to-nearest intrinsics so that the compiler cannot contract or
// reorder the steps the transformations rely on.  Compiles as host C++ too
// (g++ -ffp-contract=off) for the CPU checks of these operations.
#pragma once

#ifdef __CUDACC__
#define SV_DF __host__ __device__ __forceinline__
#else
#include <cmath>
#define SV_DF inline
#endif

namespace sv {

struct alignas(8) dfv {
  float hi, lo;
};

SV_DF float df_addf(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
SV_DF float df_subf(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
SV_DF float df_mulf(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
SV_DF float df_fmaf(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
SV_DF float df_rcpf(float a) {
#ifdef __CUDA_ARCH__
  return __frcp_rn(a);
#else
  return 1.0f / a;
#endif
}
SV_DF float df_sqrtf(float a) {
#ifdef __CUDA_ARCH__
  return __fsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}

// s + e = a + b exactly (Knuth's TwoSum, no condition on a and b)
SV_DF void two_sum(float a, float b, float& s, float& e) {
  s = df_addf(a, b);
  const float bb = df_subf(s, a);
  e = df_addf(df_subf(a, df_subf(s, bb)), df_subf(b, bb));
}

// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker's Fast2Sum)
SV_DF void fast_two_sum(float a, float b, float& s, float& e) {
  s = df_addf(a, b);
  e = df_subf(b, df_subf(s, a));
}

SV_DF dfv df_make(float hi, float lo) {
  dfv r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// normalised pair of an accumulator s + t
SV_DF dfv df_norm(float s, float t) {
  dfv r;
  two_sum(s, t, r.hi, r.lo);
  return r;
}

// (s, t) <- (s, t) - l a: the product's rounding residual by FMA, the cross
// terms hi*lo (lo*lo, below 2^-46 of the product, left out), the leading
// subtraction by TwoSum; the small parts gather in t.
SV_DF void df_fms_acc(float& s, float& t, dfv l, dfv a) {
  const float p = df_mulf(l.hi, a.hi);
  float q = df_fmaf(l.hi, a.hi, -p);
  q = df_fmaf(l.hi, a.lo, q);
  q = df_fmaf(l.lo, a.hi, q);
  float s2, e;
  two_sum(s, -p, s2, e);
  s = s2;
  t = df_addf(t, df_subf(e, q));
}

// normalised v - l a
SV_DF dfv df_fms(dfv v, dfv l, dfv a) {
  float s = v.hi, t = v.lo;
  df_fms_acc(s, t, l, a);
  return df_norm(s, t);
}

// normalised a b
SV_DF dfv df_mul(dfv a, dfv b) {
  const float p = df_mulf(a.hi, b.hi);
  float q = df_fmaf(a.hi, b.hi, -p);
  q = df_fmaf(a.hi, b.lo, q);
  q = df_fmaf(a.lo, b.hi, q);
  dfv r;
  fast_two_sum(p, q, r.hi, r.lo);
  return r;
}

// normalised a + b
SV_DF dfv df_add(dfv a, dfv b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  return df_norm(s, df_addf(e, df_addf(a.lo, b.lo)));
}

// 1 / d for normalised d != 0: the float32 reciprocal y and one Newton
// correction y (1 - d y), whose residual 1 - d_hi y is exact in float32;
// relative error about 2^-46
SV_DF dfv df_rcp(dfv d) {
  const float y = df_rcpf(d.hi);
  float r = df_fmaf(-d.hi, y, 1.0f);
  r = df_fmaf(-d.lo, y, r);
  dfv out;
  fast_two_sum(y, df_mulf(y, r), out.hi, out.lo);
  return out;
}

// sqrt(a) for normalised a > 0: the float32 root y and one Newton correction
// (a - y^2) / (2 y), whose residual a_hi - y^2 is exact in float32
SV_DF dfv df_sqrt(dfv a) {
  const float y = df_sqrtf(a.hi);
  float r = df_fmaf(-y, y, a.hi);
  r = df_addf(r, a.lo);
  dfv out;
  fast_two_sum(y, df_mulf(r, df_mulf(0.5f, df_rcpf(y))), out.hi, out.lo);
  return out;
}

// s2 (1 - D) for s2 > 0 and 0 <= D <= 1 (a covariance entry from its
// correlation deficit): s2 D <= s2, so the leading subtraction is a Fast2Sum
SV_DF dfv df_scaled_deficit(dfv s2, float D) {
  const float p = df_mulf(s2.hi, D);
  float q = df_fmaf(s2.hi, D, -p);
  q = df_fmaf(s2.lo, D, q);
  float s, e;
  fast_two_sum(s2.hi, -p, s, e);
  return df_norm(s, df_addf(e, df_subf(s2.lo, q)));
}

// the float64 value of a pair, and the nearest pair of a float64 value
// (float64 instructions: for per-block values, not inner loops)
SV_DF double df_to_double(dfv v) { return (double)v.hi + (double)v.lo; }
SV_DF dfv df_from_double(double x) {
  const float hi = (float)x;
  return df_make(hi, (float)(x - (double)hi));
}

}  // namespace sv
