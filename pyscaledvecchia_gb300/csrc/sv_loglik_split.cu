// Split-precision block kernel of the Vecchia likelihood / score / Fisher
// evaluation (blocks with K = k+1 <= 32, closed-form nu).
//
// Same per-block record as the float64 kernels (likelihood.py:111-144 of the
// reference), computed with float64 only where conditioning needs it:
//   float32 : centred scaled coordinates, distances, the correlation
//             deficit 1 - M (accurate for close pairs) and g, the
//             products dSigma_l a (K^2 d), the Fisher / score Gram products;
//   float64 : the diagonal s2(1+tau) (+ jitter), the Cholesky factorisation,
//             a = L^-T e_K, the forward solves W = L^-1 [dSigma a], L^-1 y,
//             L^-1 Z, log L_KK and everything reduced afterwards.
// On GB300 a float64 instruction costs 1/66 of the FP32 rate and a masked
// lane costs as much as an active one, so a block is owned by a team of G
// lanes and a warp holds 32/G blocks: the serial part of each factorisation
// step is shared by 32/G blocks.  The factorisation is LDL^T (unit lower L,
// D = diag(d_k)), which needs one reciprocal per step (an FP32 seed and one
// float64 Newton step) and no square roots; the Cholesky factor is
// C = L D^(1/2), so a = C^-T e_K = L^-T e_K / sqrt(d_K), W = D^(-1/2) L^-1 V
// (unit forward solves, the D^(-1/2) weights applied in the float32 Gram)
// and L_KK = sqrt(d_K) (one float64 square root per block).
//
// Warp-uniform outer loops (up to the warp's largest K) with team-local
// predication keep every __syncwarp reached by all lanes when the blocks of a
// warp differ in size.
#include "sv_loglik.cuh"

namespace sv {

constexpr int kSplitMaxThreads = 512;
// independent elements per lane per round of the factorisation update and the
// multi-column forward solve (instruction-level parallelism per lane)
constexpr int kSplitU = 4;
// columns per factorisation step (panel width) and trailing elements per
// round of a step (kSplitW FMAs each): measured at C2, widths 2, 3, 4, 6, 8
// took 9.31, 9.18, 9.05, 9.11, 9.16 ms
constexpr int kSplitW = 4;
// steps per pass of the forward solves
constexpr int kSplitWF = 4;
constexpr int kSplitU2 = 1;

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

// Exponential-series tail E_m(c) = sum_{k >= m} c^k / k! for 0 <= c <= 2
// (nested Horner form, positive terms only: no cancellation).  Terms up to
// k = 16: the rest is below 2e-10 of E_2 and E_3 at c = 2, far under float32
// rounding.
__device__ __forceinline__ float exp_tail(float c, int m) {
  float t = 1.0f;
#pragma unroll
  for (int k = 16; k > 0; --k)
    if (k > m) t = fmaf(t, c * (1.0f / (float)k), 1.0f);
  float p = 1.0f, f = 1.0f;
  for (int k = 1; k <= m; ++k) {
    p *= c;
    f *= (float)k;
  }
  return t * (p / f);
}

// Correlation deficit D = 1 - M(r) with small relative error for every r
// (for nearby points M is close to 1 and 1 - M would lose all of float32's
// digits):  nu = 0.5: -expm1(-r);  nu = 1.5: e^-c E_2(c);
// nu = 2.5: e^-c (c^2/6 + E_3(c)), c = sqrt(2 nu) r.
__device__ __forceinline__ float matern_deficit_f32(int code, float r) {
  if (code == 0) return -expm1f(-r);
  const float c = (code == 1 ? 1.7320508075688772f : 2.23606797749979f) * r;
  if (c > 2.0f) {
    float M, g;
    matern_closed_f32(code, r, M, g);
    return 1.0f - M;
  }
  const float e = expf(-c);
  if (code == 1) return e * exp_tail(c, 2);
  return e * fmaf(c * c, 1.0f / 6.0f, exp_tail(c, 3));
}

// Order tests on the bit patterns of positive doubles (integer pipe, not the
// slow float64 pipe): for x, y >= 0, x < y <=> bits(x) < bits(y).
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
constexpr long long kBitsTiny = 0x39B4484BFEEBC2A0LL;  // 1e-30
constexpr long long kBitsHuge = 0x46293E5939A08CEALL;  // 1e30
constexpr long long kBitsInf = 0x7FF0000000000000LL;

// float64 reciprocal of a pivot from the float32 reciprocal refined by one
// Newton step y <- y + y (1 - d y): relative error about 2^-44, far below the
// float32 assembly error of the split form; a chain of two float64 FMAs.
__device__ __forceinline__ double pivot_rcp(double dkk) {
  const long long bd = dbits(dkk);
  if (bd > kBitsTiny && bd < kBitsHuge) {
    const double y = (double)(1.0f / (float)dkk);
    return fma(y, fma(-dkk, y, 1.0), y);
  }
  return 1.0 / dkk;
}

// Rows i of the float32 right-hand sides dSigma_l a for l = 1..d:
//   R(1 + l, i) = -s2 sum_{j != i} g_ij a_j (u_il - u_jl)^2,
// one pass over the neighbours j with row i's coordinates, the squared
// differences and the d sums in registers (DR >= d, zero padded); the same
// roundings in the same order as a pass per l.
template <int DR>
__device__ __forceinline__ void split_dsig_row(int i, int K, int d, int code, float s2f,
                                               const float* u, const float* a32, double* R) {
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
    if (l < d) R[(1 + l) * 33 + i] = (double)(-s2f * S[l]);
}

// pivot kk of the team's factorisation: LAPACK's criterion (a pivot that is
// not > 0, i.e. negative, zero or NaN, fails: flag[0]), the conditioning
// test against rho_min (flag[1]) and the reciprocal
__device__ __forceinline__ void split_pivot(double dkk, int kk, long long rho_bits, double* invd,
                                            volatile int* flag) {
  const long long bd = dbits(dkk);
  if (bd <= 0 || bd >= kBitsInf) {
    flag[0] = 1;
  } else {
    if (bd < rho_bits) flag[1] = 1;
    invd[kk] = pivot_rcp(dkk);
  }
}

// L is stored packed by columns with capacity 32: entry (i, j), i >= j, at
// cstart(j) + i - j.  Column walks (scaling, trailing updates, forward
// solves) then touch consecutive words, free of bank conflicts.
__device__ __forceinline__ int cstart(int j) { return j * 32 - (j * (j - 1)) / 2; }
__device__ __forceinline__ int cm(int i, int j) { return cstart(j) + (i - j); }

// Entries (h, j < h) and (K-1-h, j < K-1-h) of Sigma below the diagonal,
// s2 (1 - D(r_ij)), and both diagonal entries dj; u is [d][32] (row i at
// column i), the current row's coordinates are held in registers (DR >= d,
// 0: read from shared memory).  The same value per entry as any other
// traversal.
template <int DR>
__device__ __forceinline__ void split_sigma_rows(int h, int K, int d, int code, double s2, double dj,
                                                 const float* u, double* Lp) {
  const int ib = K - 1 - h;            // >= h
  const int na = ib == h ? 0 : h;      // entries of row h when it is a row of its own
  constexpr int W = DR > 0 ? DR : 1;
  float ur[W];
  int i = na > 0 ? h : ib;
  if constexpr (DR > 0) {
#pragma unroll
    for (int l = 0; l < DR; ++l) ur[l] = l < d ? u[l * 32 + i] : 0.0f;
  }
  for (int s = 0; s < na + ib; ++s) {
    if (s == na && na > 0) {
      i = ib;
      if constexpr (DR > 0) {
#pragma unroll
        for (int l = 0; l < DR; ++l) ur[l] = l < d ? u[l * 32 + i] : 0.0f;
      }
    }
    const int j = s < na ? s : s - na;
    float r2 = 0.0f;
    if constexpr (DR > 0) {
#pragma unroll
      for (int l = 0; l < DR; ++l)
        if (l < d) {
          const float df = ur[l] - u[l * 32 + j];
          r2 = fmaf(df, df, r2);
        }
    } else {
      for (int l = 0; l < d; ++l) {
        const float df = u[l * 32 + i] - u[l * 32 + j];
        r2 = fmaf(df, df, r2);
      }
    }
    Lp[cm(i, j)] = fma(-s2, (double)matern_deficit_f32(code, sqrtf(r2)), s2);
  }
  Lp[cm(h, h)] = dj;
  if (ib != h) Lp[cm(ib, ib)] = dj;
}

template <int G>
__global__ void __launch_bounds__(kSplitMaxThreads, 1) k_block_split(LikArgs A, int wpc) {
  extern __shared__ double smem[];
  constexpr int NB = 32 / G;
  const unsigned full = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tm = lane / G, tl = lane - (lane / G) * G;
  const int dmax = A.dmax;
  // at least kSplitW - 1 R columns: R's first columns and a are the
  // factorisation's scratch
  const int nrs = A.NRmax > kSplitW - 1 ? A.NRmax : kSplitW - 1;
  const int64_t slot = split_slot_doubles(dmax, nrs);
  double* Lp = smem + (int64_t)(warp * NB + tm) * slot;
  double* R = Lp + 528;  // NR columns, stride 33
  double* a = R + 33 * nrs;
  double* invd = a + 32;
  float* a32 = (float*)(invd + 32);
  float* u = a32 + 32;
  int* idx = (int*)(u + 32 * dmax);
  volatile int* tflag = idx + 32;
  double* acc = R;            // column 0 of R is scratch during the a solve
  // unscaled columns of a factorisation step: R's first columns, then a
  double* accs[kSplitW];
#pragma unroll
  for (int p = 0; p < kSplitW; ++p) accs[p] = p < kSplitW - 1 ? R + 33 * p : a;
  float* R32 = (float*)Lp;    // float32 copy of R once L is no longer needed

  const int64_t nb = A.b1 - A.b0;
  const int64_t stride = (int64_t)gridDim.x * wpc * NB;
  for (int64_t base = ((int64_t)blockIdx.x * wpc + warp) * NB; base < nb; base += stride) {
    const int64_t tix = base + tm;
    bool active = tix < nb;
    const int64_t b = active ? launch_block(A, A.b0 + tix) : 0;
    if (active && A.probs[block_problem(A, b)].skip) active = false;
    if (active && A.fixup) active = A.chunk_max[A.chunk[b]] > A.level[b];
    const int K = active ? A.kb[b] + 1 : 0;
    const int Kw = __reduce_max_sync(full, K);
    if (Kw == 0) continue;
    const int k = K - 1;
    // this team's problem
    const int pid = active ? block_problem(A, b) : 0;
    const ProbInfo& PI = A.probs[pid];
    const int d = PI.d, q = PI.q, P = PI.P, NR = P + 1 + q;
    const double s2 = PI.s2, tau = PI.tau;
    const float s2f = (float)s2;
    const int code = PI.closed;
    const double diag = s2 * (1.0 + tau);
    const double* Y = A.y + PI.y_off;
    const double* Zm = A.Z + PI.z_off;
    const float2* XH = A.xhl + PI.x_off;
    int32_t* info = A.info + 4 * pid;

    // ---- gather: neighbours first, self last; coordinates centred on self
    if (active)
      for (int i = tl; i < K; i += G) idx[i] = (i < k) ? A.nbr[b * A.ldnbr + i] : A.rowb[b];
    __syncwarp();
    if (active) {
      // centred scaled coordinates from the (hi, lo) float32 pairs: the
      // difference keeps ~24 bits relative to itself, however close the points
      const float2* xs = XH + (int64_t)idx[k] * d;
      for (int t = tl; t < K * d; t += G) {
        const int i = t / d, l = t - (t / d) * d;
        const float2 v = XH[(int64_t)idx[i] * d + l];
        const float2 w = xs[l];
        u[l * 32 + i] = (v.x - w.x) + (v.y - w.y);
      }
      if (A.need_grad)
        for (int i = tl; i < K; i += G) {
          R[P * 33 + i] = Y[idx[i]];
          for (int c = 0; c < q; ++c) R[(P + 1 + c) * 33 + i] = Zm[(int64_t)idx[i] * q + c];
        }
    }
    __syncwarp();

    // ---- Sigma (float32 deficit, float64 entries) and Cholesky with the
    //      jitter ladder of _covariance.py:235-252
    int lv = (active && A.fixup) ? A.chunk_max[A.chunk[b]] : 0;
    bool done = !active, failed = false;
    double jit = 0.0;
    long long rho_bits = 0;
    while (__any_sync(full, !done)) {
      const bool need = !done;
      if (need) {
        jit = (lv > 0) ? jitter_pow10(lv) * diag : 0.0;  // 10^p * mean(diag)
        rho_bits = dbits(A.rho_min * (diag + jit));
        // lane h takes rows h and K-1-h (K-1 entries below the diagonal
        // between them); s2 (1 - D): the deficit carries the information of
        // close pairs
        for (int h = tl; 2 * h < K; h += G) {
          if (d <= 4)
            split_sigma_rows<4>(h, K, d, code, s2, diag + jit, u, Lp);
          else if (d <= 8)
            split_sigma_rows<8>(h, K, d, code, s2, diag + jit, u, Lp);
          else if (d <= 12)
            split_sigma_rows<12>(h, K, d, code, s2, diag + jit, u, Lp);
          else
            split_sigma_rows<0>(h, K, d, code, s2, diag + jit, u, Lp);
        }
        if (tl == 0) {
          tflag[0] = 0;  // a pivot failed
          tflag[1] = 0;  // a pivot ratio L_kk^2 / Sigma_kk fell below rho_min
        }
      }
      __syncwarp();
      if (need && tl == 0) split_pivot(Lp[cm(0, 0)], 0, rho_bits, invd, tflag);
      __syncwarp();
      // right-looking LDL^T, kSplitW columns (a panel) per step, warp-uniform
      // loop.  Panel column c = kk + p takes the steps kk .. c-1 in order (its
      // pivot follows at once), then is scaled by 1/d_c, its unscaled values
      // in accs[p]; every trailing element (j >= kk + kSplitW) then takes all
      // kSplitW updates in one visit, fma(-l(i,s) a(j,s), .) for s = kk, kk+1,
      // ...: the same roundings in the same order as single steps.  The lane
      // that updates (kk+W, kk+W) takes that pivot's reciprocal (look-ahead).
      // A failed pivot stops the attempt (it is redone with jitter).
      auto colp = [&](int c) { return Lp + cstart(c) - c; };  // colp(c)[i] = L(i, c)
      for (int kk = 0; kk < Kw; kk += kSplitW) {
        bool go = need && kk < K && tflag[0] == 0;
#pragma unroll
        for (int p = 0; p < kSplitW; ++p) {
          const int c = kk + p;
          if (p > 0) {
            if (go && c < K) {
              double* colc = colp(c);
              for (int i = c + tl; i < K; i += G) {
                double v = colc[i];
#pragma unroll
                for (int s2 = 0; s2 < p; ++s2) v = fma(-colp(kk + s2)[i], accs[s2][c], v);
                colc[i] = v;
                accs[p][i] = v;
                if (i == c) split_pivot(v, c, rho_bits, invd, tflag);
              }
            }
            __syncwarp();
            go = go && tflag[0] == 0;
          }
          if (go && c < K) {
            double* colc = colp(c);
            const double inv = invd[c];
            for (int i = c + 1 + tl; i < K; i += G) {
              const double v = p == 0 ? colc[i] : accs[p][i];
              if (p == 0) accs[0][i] = v;
              colc[i] = v * inv;
            }
          }
          __syncwarp();
        }
        if (go) {
          const int j0 = kk + kSplitW;
          const int m = K - j0;
          const int cnt = m > 0 ? m * (m + 1) / 2 : 0;
          if (tl < cnt) {
            int j = j0, rem = tl;
            while (rem >= K - j) {
              rem -= K - j;
              ++j;
            }
            for (int t = tl; t < cnt; t += kSplitU2 * G) {
              int jj[kSplitU2], ii[kSplitU2];
#pragma unroll
              for (int u4 = 0; u4 < kSplitU2; ++u4) {
                jj[u4] = j;
                ii[u4] = j + rem;
                rem += G;
                while (j < K && rem >= K - j) {
                  rem -= K - j;
                  ++j;
                }
              }
              double nv[kSplitU2];
#pragma unroll
              for (int u4 = 0; u4 < kSplitU2; ++u4)
                if (t + u4 * G < cnt) nv[u4] = Lp[cm(ii[u4], jj[u4])];
#pragma unroll
              for (int s2 = 0; s2 < kSplitW; ++s2) {
                const double* cs = colp(kk + s2);
#pragma unroll
                for (int u4 = 0; u4 < kSplitU2; ++u4)
                  if (t + u4 * G < cnt) nv[u4] = fma(-cs[ii[u4]], accs[s2][jj[u4]], nv[u4]);
              }
#pragma unroll
              for (int u4 = 0; u4 < kSplitU2; ++u4)
                if (t + u4 * G < cnt) {
                  Lp[cm(ii[u4], jj[u4])] = nv[u4];
                  if (ii[u4] == j0 && jj[u4] == j0) split_pivot(nv[u4], j0, rho_bits, invd, tflag);
                }
            }
          }
        }
        __syncwarp();
      }
      if (need) {
        if (tflag[0] == 0) {
          done = true;
        } else if (++lv > 9) {
          done = true;
          failed = true;
        }
      }
      __syncwarp();
    }

    double* rec = A.cache + b * (int64_t)A.CS;
    if (failed) {
      // not positive definite even with jitter after float32 assembly: the
      // float64 pass decides (and reports a failure if it fails as well)
      if (tl == 0) {
        A.level[b] = 0;
        A.redo[b] = 1;
        atomicAdd(info + SV_INFO_AUX, 1);
      }
      for (int f = tl; f < A.CS; f += G) rec[f] = 0.0;
    } else if (active && tl == 0) {
      A.level[b] = (int8_t)lv;
      if (lv > 0) {
        atomicMax(info + SV_INFO_JITTER, lv);
        A.flags[0] = 1;
      }
      // ill-conditioned blocks lose too much to float32 assembly: redo in float64
      const bool again = tflag[1] != 0;
      A.redo[b] = again ? 1 : 0;
      if (again) atomicAdd(info + SV_INFO_AUX, 1);
    }
    const bool ok = active && !failed;

    // ---- a = C^-T e_K = L^-T e_K / sqrt(d_K)  (float64, unit back substitution)
    double lKK = 0.0, sK = 0.0;  // L_KK = sqrt(d_K) and its reciprocal
    if (ok) {
      lKK = sqrt(Lp[cm(k, k)]);
      sK = 1.0 / lKK;
      if (tl == 0) rec[0] = lKK;  // L_KK; the log is taken in the reduction
      for (int i = tl; i < K; i += G) acc[i] = (i == k) ? 1.0 : 0.0;
    }
    __syncwarp();
    for (int i = Kw - 1; i >= 0; --i) {
      if (ok && i < K) {
        const double ai = acc[i];
        for (int j = tl; j < i; j += G) acc[j] -= Lp[cm(i, j)] * ai;
      }
      __syncwarp();
    }
    if (ok)
      for (int i = tl; i < K; i += G) {
        const double ai = acc[i] * sK;
        a[i] = ai;
        a32[i] = (float)ai;
      }
    __syncwarp();

    // ---- GLS parts (float64 team sums)
    {
      double vy = 0.0;
      if (ok)
        for (int i = tl; i < K; i += G) vy += a[i] * Y[idx[i]];
      for (int o = G / 2; o > 0; o >>= 1) vy += __shfl_xor_sync(full, vy, o);
      if (ok && tl == 0) rec[1] = vy;
      // teams of one warp may belong to problems with different q: the
      // shuffles run to the warp's largest q
      const int qw = __reduce_max_sync(full, active ? q : 0);
      for (int c = 0; c < qw; ++c) {
        double vz = 0.0;
        if (ok && c < q)
          for (int i = tl; i < K; i += G) vz += a[i] * Zm[(int64_t)idx[i] * q + c];
        for (int o = G / 2; o > 0; o >>= 1) vz += __shfl_xor_sync(full, vz, o);
        if (ok && c < q && tl == 0) rec[2 + c] = vz;
      }
    }
    if (!A.need_grad) {
      __syncwarp();
      if (ok && tl == 0) {
        rec[2 + q] = rec[1];
        for (int c = 0; c < q; ++c) rec[3 + q + c] = rec[2 + c];
      }
      __syncwarp();
      continue;
    }
    __syncwarp();

    // ---- right-hand sides dSigma_p a
    if (ok) {
      // p = 0: Sigma (un-jittered) a = L_KK e_K - jit a
      for (int i = tl; i < K; i += G) R[i] = ((i == k) ? lKK : 0.0) - jit * a[i];
      // p = 1..d (float32): -s2 sum_j g_ij a_j (u_il - u_jl)^2
      if (d <= 12) {
        for (int i = tl; i < K; i += G) {
          if (d <= 4)
            split_dsig_row<4>(i, K, d, code, s2f, u, a32, R);
          else if (d <= 8)
            split_dsig_row<8>(i, K, d, code, s2f, u, a32, R);
          else
            split_dsig_row<12>(i, K, d, code, s2f, u, a32, R);
        }
      } else
      for (int i = tl; i < K; i += G) {
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
          R[(1 + l) * 33 + i] = (double)(-s2f * s);
        }
      }
      // nugget row: dSigma_tau = s2 tau I
      for (int i = tl; i < K; i += G) R[(P - 1) * 33 + i] = s2 * tau * a[i];
    }
    __syncwarp();

    // ---- forward solves (float64) with the unit factor: L^-1 [dSigma a, y, Z];
    // W = D^(-1/2) L^-1 dSigma a.  Without jitter Sigma a = L_KK e_K, whose
    // solution is sqrt(d_K) e_K, so that column is left out of the solve.
    const int c0 = (jit == 0.0) ? 1 : 0;
    // columns c0 + tl, c0 + tl + G, ... per lane, with no warp
    // synchronisation between steps; kSplitWF steps per pass: the panel's
    // own rows are finished in order, then every later row takes the
    // panel's updates in one visit (each element sees the steps in order)
    if (ok)
      for (int c = c0 + tl; c < NR; c += G) {
        double* col = R + c * 33;
        for (int i = 0; i < K - 1; i += kSplitWF) {
          const int ns = min(kSplitWF, K - 1 - i);  // steps i .. i+ns-1
          double r[kSplitWF];
#pragma unroll
          for (int s2 = 0; s2 < kSplitWF; ++s2)
            if (s2 < ns) {
              double v = col[i + s2];
#pragma unroll
              for (int t2 = 0; t2 < s2; ++t2) v = fma(-Lp[cm(i + s2, i + t2)], r[t2], v);
              r[s2] = v;
              col[i + s2] = v;
            }
          for (int j = i + ns; j < K; ++j) {
            double v = col[j];
#pragma unroll
            for (int t2 = 0; t2 < kSplitWF; ++t2)
              if (t2 < ns) v = fma(-Lp[cm(j, i + t2)], r[t2], v);
            col[j] = v;
          }
        }
      }
    __syncwarp();
    if (ok) {
      if (c0 == 1)
        for (int i = tl; i < K; i += G) R[i] = (i == k) ? lKK : 0.0;
      // a32 is free now: it takes the float32 weights d_j^(-1/2)
      for (int j = tl; j < K; j += G) a32[j] = sqrtf((float)invd[j]);
    }
    __syncwarp();

    // ---- record: z parts, w_K (float64), Gram products (float32) of the
    //      D^(-1/2)-weighted solutions
    if (ok) {
      for (int e = tl; e < NR * 33; e += G) {
        const int c = e / 33, j = e - (e / 33) * 33;
        R32[e] = (j < K) ? (float)R[c * 33 + j] * a32[j] : 0.0f;
      }
    }
    __syncwarp();
    if (ok) {
      double* wK = rec + 3 + 2 * q;
      double* wzy = wK + P;
      double* wzZ = wzy + P;
      double* F = wzZ + P * q;
      for (int c = tl; c < 1 + q; c += G) rec[2 + q + c] = R[(P + c) * 33 + k] * sK;
      for (int p = tl; p < P; p += G) wK[p] = R[p * 33 + k] * sK;
      const int nf = P * (P + 1) / 2;
      const int ntot = nf + P * (1 + q);
      for (int t = tl; t < ntot; t += G) {
        int c1, c2;
        if (t < nf) {
          tri_index(t, c1, c2);
        } else {
          const int s3 = t - nf;
          c1 = s3 / (1 + q);
          c2 = P + (s3 - c1 * (1 + q));
        }
        const float* r1 = R32 + c1 * 33;
        const float* r2 = R32 + c2 * 33;
        float sacc = 0.0f;
        for (int i = 0; i < K; ++i) sacc = fmaf(r1[i], r2[i], sacc);
        if (t < nf) {
          F[t] = 0.5 * (2.0 * (double)sacc - (R[c1 * 33 + k] * sK) * (R[c2 * 33 + k] * sK));
        } else {
          const int s3 = t - nf;
          const int p = s3 / (1 + q);
          const int cc = s3 - p * (1 + q);
          if (cc == 0)
            wzy[p] = (double)sacc;
          else
            wzZ[p * q + (cc - 1)] = (double)sacc;
        }
      }
    }
    __syncwarp();
  }
}

// (hi, lo) float32 pairs of x / lambda: hi = fl32(v), lo = fl32(v - hi);
// grid row = problem
__global__ void k_split_prep(const double* X, const ProbInfo* probs, float2* xhl) {
  const ProbInfo& PI = probs[blockIdx.y];
  if (PI.skip) return;
  const int d = PI.d;
  const int64_t tot = PI.n * d;
  const double* Xp = X + PI.x_off;
  float2* out = xhl + PI.x_off;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int l = (int)(e % d);
    const double v = Xp[e] * PI.invlam[l];
    const float hi = (float)v;
    out[e] = make_float2(hi, (float)(v - (double)hi));
  }
}

int launch_split_prep(const LikArgs& A, int64_t nx, cudaStream_t st) {
  if (nx == 0) return SV_OK;
  int64_t gx = (nx / A.nprob + 255) / 256;
  if (gx > 4LL * sv_num_sms()) gx = 4LL * sv_num_sms();
  if (gx < 1) gx = 1;
  k_split_prep<<<dim3((unsigned)gx, (unsigned)A.nprob), 256, 0, st>>>(A.X, A.probs, A.xhl);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

int launch_block_split(const LikArgs& A, int lanes, cudaStream_t st) {
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t per_warp =
      sizeof(double) * (size_t)split_slot_doubles(A.dmax, A.NRmax > kSplitW - 1 ? A.NRmax : kSplitW - 1) *
      (32 / lanes);
  int wpc = kSplitMaxThreads / 32;
  while (wpc > 1 && wpc * per_warp > (size_t)maxsm) --wpc;
  const size_t smem = wpc * per_warp;
  if (smem > (size_t)maxsm) return SV_EINVAL;
  const int64_t nb = A.b1 - A.b0;
  const int64_t per_cta = (int64_t)wpc * (32 / lanes);
  int64_t grid = (nb + per_cta - 1) / per_cta;
  const int nsm = sv_num_sms();
  if (grid > 64LL * nsm) grid = 64LL * nsm;
  if (grid < 1) grid = 1;
  switch (lanes) {
#define SV_SPLIT_CASE(GV)                                                                          \
  case GV:                                                                                         \
    SV_CUDA_TRY(cudaFuncSetAttribute(k_block_split<GV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)smem));                                                  \
    k_block_split<GV><<<(unsigned)grid, 32 * wpc, smem, st>>>(A, wpc);                            \
    break;
    SV_SPLIT_CASE(4)
    SV_SPLIT_CASE(8)
    SV_SPLIT_CASE(16)
    SV_SPLIT_CASE(32)
#undef SV_SPLIT_CASE
    default:
      return SV_EINVAL;
  }
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

}  // namespace sv
