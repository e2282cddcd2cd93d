// Float32 parts shared by the two split-precision block kernels
// (sv_loglik_split64.cu: float64 factorisation and solves, the split form;
// sv_loglik_split.cu: double-float factorisation and solves): the closed-form
// Matern terms and correlation deficits in float32, the float32 right-hand
// sides dSigma_l a, the packed column layout of the block factor, bit-pattern
// order tests, and float32 <-> float64 conversions on the integer pipe.
#pragma once
#include "sv_loglik.cuh"

namespace sv {

__device__ __forceinline__ void matern_closed_f32(int code, float r, float& M, float& g) {
  if (code == 0) {
    if (r > 0.0f) {
      const float e = expf(-r);
      M = e;
      g = -e / r;
    } else {
      M = 1.0f;
      g = 0.0f;
    }
  } else if (code == 1) {
    const float c = 1.7320508075688772f * r;
    const float e = expf(-c);
    M = (1.0f + c) * e;
    g = -3.0f * e;
  } else {
    const float c = 2.23606797749979f * r;
    const float e = expf(-c);
    M = (1.0f + c + c * c * (1.0f / 3.0f)) * e;
    g = -(5.0f / 3.0f) * (1.0f + c) * e;
  }
}

// Correlation deficit D = 1 - M(r) with small relative error for every r
// (for nearby points M is close to 1 and 1 - M would lose all of float32's
// digits):  nu = 0.5: -expm1(-r);  for c = sqrt(2 nu) r <= 2,
// nu = 1.5: e^-c c^2 P(c) with P(c) = sum_{k >= 2} c^(k-2) / k!,
// nu = 2.5: e^-c c^2 (P(c) - 1/3)   (1 - M = e^-c (c^2/6 + sum_{k>=3} c^k/k!)),
// P by Horner's rule in c with the constants 1/k!, k = 3 .. 14 (positive
// terms, no cancellation; the terms beyond k = 14 are below 1e-8 of P at
// c = 2).  Measured against 40-digit values on c in [1e-4, 2]: at most 4 ulp,
// 0.8 ulp on average, as the exponential-tail sum it replaces.
__device__ __forceinline__ float matern_deficit_f32(int code, float r) {
  if (code == 0) return -expm1f(-r);
  const float c = (code == 1 ? 1.7320508075688772f : 2.23606797749979f) * r;
  if (c > 2.0f) {
    float M, g;
    matern_closed_f32(code, r, M, g);
    return 1.0f - M;
  }
  constexpr float kInvFact[12] = {1.1470745597729725e-11f, 1.6059043836821613e-10f,
                                  2.08767569878681e-09f,   2.505210838544172e-08f,
                                  2.755731922398589e-07f,  2.7557319223985893e-06f,
                                  2.48015873015873e-05f,   0.0001984126984126984f,
                                  0.001388888888888889f,   0.008333333333333333f,
                                  0.041666666666666664f,   0.16666666666666666f};  // 1/14! .. 1/3!
  float P = kInvFact[0];
#pragma unroll
  for (int t = 1; t < 12; ++t) P = fmaf(P, c, kInvFact[t]);
  P = fmaf(P, c, code == 1 ? 0.5f : 0.16666666666666666f);
  return (expf(-c) * (c * c)) * P;
}

// Rows i of the float32 right-hand sides dSigma_l a for l = 1..d:
//   R(1 + l, i) = -s2 sum_{j != i} g_ij a_j (u_il - u_jl)^2,
// one pass over the neighbours j with row i's coordinates, the squared
// differences and the d sums in registers (DR >= d, zero padded); the same
// roundings in the same order as a pass per l.  store(1 + l, value) writes
// the value into column 1 + l of the caller's right-hand sides.
template <int DR, typename Store>
__device__ __forceinline__ void split_dsig_row(int i, int K, int d, int code, float s2f,
                                               const float* u, const float* a32, Store store) {
  float ui[DR], S[DR];
#pragma unroll
  for (int l = 0; l < DR; ++l) {
    ui[l] = l < d ? u[l * 32 + i] : 0.0f;
    S[l] = 0.0f;
  }
  for (int j = 0; j < K; ++j) {
    if (j == i) continue;  // g_ii a_i (u_i - u_i)^2 adds exactly nothing
    float sq[DR];
    float r2 = 0.0f;
#pragma unroll
    for (int l = 0; l < DR; ++l)
      if (l < d) {
        const float df = ui[l] - u[l * 32 + j];
        r2 = fmaf(df, df, r2);
        sq[l] = df * df;
      }
    float M, g;
    matern_closed_f32(code, sqrtf(r2), M, g);
    const float c = g * a32[j];
#pragma unroll
    for (int l = 0; l < DR; ++l)
      if (l < d) S[l] = fmaf(c, sq[l], S[l]);
  }
#pragma unroll
  for (int l = 0; l < DR; ++l)
    if (l < d) store(1 + l, -s2f * S[l]);
}

// The same for d > 12: row i's g_ij a_j for all j in registers, then one
// pass per coordinate.
template <typename Store>
__device__ __forceinline__ void split_dsig_row_wide(int i, int K, int d, int code, float s2f,
                                                    const float* u, const float* a32, Store store) {
  float cj[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    float c = 0.0f;
    if (j < K && j != i) {
      float r2 = 0.0f;
      for (int l = 0; l < d; ++l) {
        const float df = u[l * 32 + i] - u[l * 32 + j];
        r2 = fmaf(df, df, r2);
      }
      float M, g;
      matern_closed_f32(code, sqrtf(r2), M, g);
      c = g * a32[j];
    }
    cj[j] = c;
  }
  for (int l = 0; l < d; ++l) {
    const float uil = u[l * 32 + i];
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      if (j < K) {
        const float df = uil - u[l * 32 + j];
        s = fmaf(cj[j], df * df, s);
      }
    }
    store(1 + l, -s2f * s);
  }
}

// L is stored packed by columns with capacity kc (the launch's largest K):
// entry (i, j), i >= j, at cstart(j) + i - j.  Column walks (scaling,
// trailing updates, forward solves) then touch consecutive words, free of
// bank conflicts.  Once factored, the diagonal holds the pivots' reciprocals.
__device__ __forceinline__ int cstart(int j, int kc) { return j * kc - (j * (j - 1)) / 2; }
__device__ __forceinline__ int cm(int i, int j, int kc) { return cstart(j, kc) + (i - j); }

}  // namespace sv
