// Float32 parts shared by the two split-precision block kernels
// (sv_loglik_split64.cu: float64 factorisation and solves, the split form;
// sv_loglik_split.cu: double-float factorisation and solves): the float32
// right-hand sides dSigma_l a and the packed column layout of the block
// factor.  The float32 Matern terms and deficits are in sv_matern.cuh.
#pragma once
#include "sv_loglik.cuh"

namespace sv {

// Rows i of the float32 right-hand sides dSigma_l a for l = 1..d:
//   R(1 + l, i) = -s2 sum_{j != i} g_ij a_j (u_il - u_jl)^2,
// one pass over the neighbours j with row i's coordinates, the squared
// differences and the d sums in registers (DR >= d, zero padded); the same
// roundings in the same order as a pass per l.  store(1 + l, value) writes
// the value into column 1 + l of the caller's right-hand sides.  An
// estimated nu (mf.dtab set) also takes its row in the same pass:
//   R(1 + d, i) = s2 nu sum_{j != i} dM/dnu_ij a_j   (_matern_general.py:177).
template <int DR, bool EST, typename Store>
__device__ __forceinline__ void split_dsig_row_t(int i, int K, int d, const MaternF32& mf, float s2f,
                                                 const float* u, const float* a32, Store store) {
  float ui[DR], S[DR];
#pragma unroll
  for (int l = 0; l < DR; ++l) {
    ui[l] = l < d ? u[l * 32 + i] : 0.0f;
    S[l] = 0.0f;
  }
  float Snu = 0.0f;
  for (int j = 0; j < K; ++j) {
    if (j == i) continue;  // g_ii a_i (u_i - u_i)^2 and dM/dnu_ii add exactly nothing
    float sq[DR];
    float r2 = 0.0f;
#pragma unroll
    for (int l = 0; l < DR; ++l)
      if (l < d) {
        const float df = ui[l] - u[l * 32 + j];
        r2 = fmaf(df, df, r2);
        sq[l] = df * df;
      }
    const float r = sqrtf(r2);
    const float c = matern_g_f32(mf, r) * a32[j];
    if (EST) Snu = fmaf(matern_dnu_f32(mf, r), a32[j], Snu);
#pragma unroll
    for (int l = 0; l < DR; ++l)
      if (l < d) S[l] = fmaf(c, sq[l], S[l]);
  }
#pragma unroll
  for (int l = 0; l < DR; ++l)
    if (l < d) store(1 + l, -s2f * S[l]);
  if (EST) store(1 + d, s2f * mf.nuf * Snu);
}

// the pass above, the estimated-nu row taken when mf.dtab is set (one test
// per row, outside the loop over the neighbours)
template <int DR, typename Store>
__device__ __forceinline__ void split_dsig_row(int i, int K, int d, const MaternF32& mf, float s2f,
                                               const float* u, const float* a32, Store store) {
  if (mf.dtab)
    split_dsig_row_t<DR, true>(i, K, d, mf, s2f, u, a32, store);
  else
    split_dsig_row_t<DR, false>(i, K, d, mf, s2f, u, a32, store);
}

// The same for d > 12: row i's g_ij a_j for all j in registers, then one
// pass per coordinate.
template <bool EST, typename Store>
__device__ __forceinline__ void split_dsig_row_wide_t(int i, int K, int d, const MaternF32& mf, float s2f,
                                                      const float* u, const float* a32, Store store) {
  float cj[32];
  float Snu = 0.0f;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    float c = 0.0f;
    if (j < K && j != i) {
      float r2 = 0.0f;
      for (int l = 0; l < d; ++l) {
        const float df = u[l * 32 + i] - u[l * 32 + j];
        r2 = fmaf(df, df, r2);
      }
      const float r = sqrtf(r2);
      c = matern_g_f32(mf, r) * a32[j];
      if (EST) Snu = fmaf(matern_dnu_f32(mf, r), a32[j], Snu);
    }
    cj[j] = c;
  }
  if (EST) store(1 + d, s2f * mf.nuf * Snu);
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

template <typename Store>
__device__ __forceinline__ void split_dsig_row_wide(int i, int K, int d, const MaternF32& mf, float s2f,
                                                    const float* u, const float* a32, Store store) {
  if (mf.dtab)
    split_dsig_row_wide_t<true>(i, K, d, mf, s2f, u, a32, store);
  else
    split_dsig_row_wide_t<false>(i, K, d, mf, s2f, u, a32, store);
}

// L is stored packed by columns with capacity kc (the launch's largest K):
// entry (i, j), i >= j, at cstart(j) + i - j.  Column walks (scaling,
// trailing updates, forward solves) then touch consecutive words, free of
// bank conflicts.  Once factored, the diagonal holds the pivots' reciprocals.
__device__ __forceinline__ int cstart(int j, int kc) { return j * kc - (j * (j - 1)) / 2; }
__device__ __forceinline__ int cm(int i, int j, int kc) { return cstart(j, kc) + (i - j); }

}  // namespace sv
