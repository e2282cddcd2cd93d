// Split-precision block kernel of the Vecchia likelihood / score / Fisher
// evaluation (blocks with K = k+1 <= 32; a closed-form nu or the float32
// Matern table of a fixed nu).
//
// Same per-block record as the float64 kernels (likelihood.py:111-144 of the
// reference), computed with float64 precision only where conditioning needs
// it:
//   float32      : centred scaled coordinates, distances, the correlation
//                  deficit 1 - M (accurate for close pairs) and g, the
//                  products dSigma_l a (K^2 d), the Fisher / score Gram
//                  products;
//   double-float : (pairs of float32, about 46 bits; sv_df64.cuh) the entries
//                  s2 (1 - D) and the diagonal s2 (1 + tau) (+ jitter), the
//                  LDL^T factorisation, a = L^-T e_K, the forward solves
//                  W = L^-1 [dSigma a], L^-1 y, L^-1 Z and the GLS sums;
//   float64      : the record and everything reduced afterwards.
// On GB300 a float64 instruction occupies the float64 pipe for about 64
// scheduler cycles, a float32 instruction for one: a double-float update
// v - l a takes about 12 float32 instructions, several times less than the
// float64 FMA it replaces, with errors (2^-46 relative) far below the float32
// assembly's.  A block is owned by a team of G lanes and a warp holds 32/G
// blocks.  The factorisation is LDL^T (unit lower L, D = diag(d_k)), which
// needs one reciprocal per step and no square roots; the Cholesky factor is
// C = L D^(1/2), so a = C^-T e_K = L^-T e_K / sqrt(d_K), W = D^(-1/2) L^-1 V
// (unit forward solves, the D^(-1/2) weights applied in the float32 Gram)
// and L_KK = sqrt(d_K).  Blocks whose smallest pivot ratio d_k / Sigma_kk
// falls below rho_min (ill-conditioned: the float32 assembly would cost too
// much), that do not factor even with jitter, or whose scale or data leave
// float32's exponent range are left to the float64 pass.
//
// Warp-uniform outer loops (up to the warp's largest K) with team-local
// predication keep every __syncwarp reached by all lanes when the blocks of a
// warp differ in size.
#include "sv_df64.cuh"
#include "sv_split.cuh"

namespace sv {

// 12 warps per CTA (shared memory holds 24 teams at d = 10, m = 30): bounds
// of 384 threads let the kernel use 144 registers without spills instead of
// 128 (measured at n = 200k, d = 10, m = 30: 5.71 against 5.80 ms);
// likelihood-only launches, whose smaller team slots would hold more warps,
// are held to 12 as well
constexpr int kSplitMaxThreads = 384;
// Panel widths, measured at n = 200k, d = 10, m = 30 (ms per evaluation):
// columns per factorisation step (kSplitW) and steps per forward-solve pass
// (kSplitWF) 4/4 6.71, 6/4 6.54, 4/8 6.54, 6/8 6.42, 8/8 6.38; two later rows
// per iteration of a forward-solve pass (kSplitJU, independent double-float
// chains) 8/8 6.29, 8/12 6.27, 6/6 6.32; two trailing elements per lane per
// factorisation round (kSplitU2) 7.24 against 6.71 (6.11 against 5.71 with
// 144 registers).  With the 384-thread bounds: kSplitW/kSplitWF/kSplitJU
// 8/8/2 5.71, 8/16/2 5.61, 8/16/4 5.68, 8/24/2 6.07, 8/32/2 6.02, 12/8/2 5.70,
// 16/8/2 6.16.
constexpr int kSplitW = 8;
constexpr int kSplitWF = 16;
constexpr int kSplitJU = 2;
constexpr int kSplitU2 = 1;

// a pivot of the team's factorisation: LAPACK's criterion (a pivot that is
// not > 0, i.e. negative, zero or NaN, fails: flag[0]), the conditioning
// test against rho_min (flag[1]; rho_bits = bits of the float32 threshold)
// and the reciprocal, which takes the pivot's place on L's diagonal.  A
// normalised pair has the sign of its hi part.
__device__ __forceinline__ void split_pivot(dfv dkk, dfv* diag, int rho_bits, volatile int* flag) {
  const int bd = __float_as_int(dkk.hi);
  if (bd <= 0 || bd >= kFBitsInf) {
    flag[0] = 1;
  } else {
    if (bd < rho_bits) flag[1] = 1;
    *diag = df_rcp(dkk);
  }
}

// Entries (h, j < h) and (K-1-h, j < K-1-h) of Sigma below the diagonal,
// s2 (1 - D(r_ij)), and both diagonal entries dj; u is [d][32] (row i at
// column i), the current row's coordinates are held in registers (DR >= d,
// 0: read from shared memory).  The same value per entry as any other
// traversal.
template <int DR>
__device__ __forceinline__ void split_sigma_rows(int h, int K, int d, const MaternF32& mf, dfv s2, dfv dj,
                                                 const float* u, dfv* Lp, int kc) {
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
    Lp[cm(i, j, kc)] = df_scaled_deficit(s2, matern_deficit_f32(mf, sqrtf(r2)));
  }
  Lp[cm(h, h, kc)] = dj;
  if (ib != h) Lp[cm(ib, ib, kc)] = dj;
}

template <int G>
__global__ void __launch_bounds__(kSplitMaxThreads, 1) k_block_split_df(LikArgs A, int wpc) {
  extern __shared__ double smem[];
  constexpr int NB = 32 / G;
  if (!pass_has_work(A)) return;
  const unsigned full = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tm = lane / G, tl = lane - (lane / G) * G;
  const unsigned tmask = (G == 32 ? full : ((1u << G) - 1u)) << (tm * G);
  const int dmax = A.dmax;
  // at least kSplitW - 1 R columns: R's first columns and a are the
  // factorisation's scratch
  const int nrs = A.NRmax > kSplitW - 1 ? A.NRmax : kSplitW - 1;
  const int kc = A.kcap;
  const int64_t slot = split_slot_doubles(dmax, nrs, kc);
  dfv* Lp = (dfv*)(smem + (int64_t)(warp * NB + tm) * slot);
  dfv* R = Lp + split_lp_cap(kc, nrs);  // NR columns, stride 33
  dfv* a = R + 33 * nrs;
  float* a32 = (float*)(a + 32);
  auto cm = [kc](int i, int j) { return sv::cm(i, j, kc); };
  float* u = a32 + 32;
  int* idx = (int*)(u + 32 * dmax);
  volatile int* tflag = idx + 32;
  dfv* acc = R;               // column 0 of R is scratch during the a solve
  // unscaled columns of a factorisation step: R's first columns, then a
  dfv* accs[kSplitW];
#pragma unroll
  for (int p = 0; p < kSplitW; ++p) accs[p] = p < kSplitW - 1 ? R + 33 * p : a;
  float* R32 = (float*)Lp;    // float32 copy of R once L is no longer needed
  double* wkd = (double*)a;   // float64 last rows of the solutions, for the record
  const dfv dzero = df_make(0.0f, 0.0f);
  const float rhof = (float)A.rho_min;

  const int64_t nb = A.b1 - A.b0;
  const int64_t stride = (int64_t)gridDim.x * wpc * NB;
  for (int64_t base = ((int64_t)blockIdx.x * wpc + warp) * NB; base < nb; base += stride) {
    const int64_t tix = base + tm;
    bool active = tix < nb;
    const int64_t b = active ? launch_block(A, A.b0 + tix) : 0;
    if (active && A.probs[block_problem(A, b)].skip) active = false;
    if (active && A.fixup) active = chunk_level(A, b) > A.level[b];
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
    const MaternF32 mf = PI.mf32;
    const double diag = s2 * (1.0 + tau);
    const dfv s2d = df_make(PI.s2_hi, PI.s2_lo);
    const double* Y = A.y + PI.y_off;
    const double* Zm = A.Z + PI.z_off;
    const float2* XH = A.xhl + PI.x_off;
    int32_t* info = A.info + 4 * pid;
    // scale inside [1e-30, 1e30] and data below 1e30 in magnitude keep every
    // pair inside float32's exponent range; other blocks, and the blocks of a
    // problem whose nu has no float32 form here, go to the float64 pass
    bool range_ok = mf.code >= 0 && dbits(diag) > kBitsTiny && dbits(diag) < kBitsHuge;

    // ---- gather: neighbours first, self last; coordinates centred on self
    if (active)
      for (int i = tl; i < K; i += G) idx[i] = (i < k) ? A.nbr[b * A.ldnbr + i] : A.rowb[b];
    __syncwarp();
    bool data_ok = true;
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
      // y and Z enter R after the factorisation, whose scratch columns
      // may cover theirs (measured: no faster when loaded here where they
      // do not); here only their range is checked
      for (int i = tl; i < K; i += G) {
        data_ok = data_ok && in_f32_range(Y[idx[i]]);
        for (int c = 0; c < q; ++c) data_ok = data_ok && in_f32_range(Zm[(int64_t)idx[i] * q + c]);
      }
    }
    range_ok = range_ok && (__ballot_sync(full, !data_ok) & tmask) == 0;
    __syncwarp();

    // ---- Sigma (float32 deficit, double-float entries) and LDL^T with the
    //      jitter ladder of _covariance.py:235-252
    int lv = (active && A.fixup) ? chunk_level(A, b) : 0;
    bool done = !active || !range_ok, failed = active && !range_ok;
    double jit = 0.0;
    int rho_bits = 0;
    while (__any_sync(full, !done)) {
      const bool need = !done;
      if (need) {
        jit = (lv > 0) ? jitter_pow10(lv) * diag : 0.0;  // 10^p * mean(diag)
        dfv dj;
        if (lv > 0) {
          rho_bits = __float_as_int((float)(A.rho_min * (diag + jit)));
          dj = df_from_double(diag + jit);
        } else {
          rho_bits = __float_as_int(rhof * PI.dg_hi);
          dj = df_make(PI.dg_hi, PI.dg_lo);
        }
        // lane h takes rows h and K-1-h (K-1 entries below the diagonal
        // between them); s2 (1 - D): the deficit carries the information of
        // close pairs
        for (int h = tl; 2 * h < K; h += G) {
          if (d <= 4)
            split_sigma_rows<4>(h, K, d, mf, s2d, dj, u, Lp, kc);
          else if (d <= 8)
            split_sigma_rows<8>(h, K, d, mf, s2d, dj, u, Lp, kc);
          else if (d <= 12)
            split_sigma_rows<12>(h, K, d, mf, s2d, dj, u, Lp, kc);
          else
            split_sigma_rows<0>(h, K, d, mf, s2d, dj, u, Lp, kc);
        }
        if (tl == 0) {
          tflag[0] = 0;  // a pivot failed
          tflag[1] = 0;  // a pivot ratio L_kk^2 / Sigma_kk fell below rho_min
        }
      }
      __syncwarp();
      if (need && tl == 0) split_pivot(Lp[0], Lp, rho_bits, tflag);
      __syncwarp();
      // right-looking LDL^T, kSplitW columns (a panel) per step, warp-uniform
      // loop.  Panel column c = kk + p takes the steps kk .. c-1 in order (its
      // pivot follows at once), then is scaled by 1/d_c, its unscaled values
      // in accs[p]; every trailing element (j >= kk + kSplitW) then takes all
      // kSplitW updates in one visit, l(i,s) a(j,s) for s = kk, kk+1, ... in
      // order, kept as an unnormalised double-float accumulator (normalised
      // where it becomes a multiplier, a pivot or a square root).  The
      // lane that updates (kk+W, kk+W) takes that pivot's reciprocal
      // (look-ahead).  A failed pivot stops the attempt (it is redone with
      // jitter).
      auto colp = [&](int c) { return Lp + cstart(c, kc) - c; };  // colp(c)[i] = L(i, c)
      for (int kk = 0; kk < Kw; kk += kSplitW) {
        bool go = need && kk < K && tflag[0] == 0;
#pragma unroll
        for (int p = 0; p < kSplitW; ++p) {
          const int c = kk + p;
          if (p > 0) {
            if (go && c < K) {
              dfv* colc = colp(c);
              for (int i = c + tl; i < K; i += G) {
                const dfv v0 = colc[i];
                float s = v0.hi, t = v0.lo;
#pragma unroll
                for (int s2 = 0; s2 < p; ++s2) df_fms_acc(s, t, colp(kk + s2)[i], accs[s2][c]);
                const dfv v = df_norm(s, t);
                colc[i] = v;
                accs[p][i] = v;
                if (i == c) split_pivot(v, colc + c, rho_bits, tflag);
              }
            }
            __syncwarp();
            go = go && tflag[0] == 0;
          }
          if (go && c < K) {
            dfv* colc = colp(c);
            const dfv inv = colc[c];
            for (int i = c + 1 + tl; i < K; i += G) {
              const dfv v = p == 0 ? df_norm(colc[i].hi, colc[i].lo) : accs[p][i];
              if (p == 0) accs[0][i] = v;
              colc[i] = df_mul(v, inv);
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
              float sv[kSplitU2], tv[kSplitU2];
#pragma unroll
              for (int u4 = 0; u4 < kSplitU2; ++u4)
                if (t + u4 * G < cnt) {
                  const dfv v0 = Lp[cm(ii[u4], jj[u4])];
                  sv[u4] = v0.hi;
                  tv[u4] = v0.lo;
                }
#pragma unroll
              for (int s2 = 0; s2 < kSplitW; ++s2) {
                const dfv* cs = colp(kk + s2);
#pragma unroll
                for (int u4 = 0; u4 < kSplitU2; ++u4)
                  if (t + u4 * G < cnt) df_fms_acc(sv[u4], tv[u4], cs[ii[u4]], accs[s2][jj[u4]]);
              }
#pragma unroll
              for (int u4 = 0; u4 < kSplitU2; ++u4)
                if (t + u4 * G < cnt) {
                  Lp[cm(ii[u4], jj[u4])] = df_make(sv[u4], tv[u4]);
                  if (ii[u4] == j0 && jj[u4] == j0)
                    split_pivot(df_norm(sv[u4], tv[u4]), Lp + cm(j0, j0), rho_bits, tflag);
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
      // not positive definite even with jitter after float32 assembly, or
      // outside float32's range: the float64 pass decides (and reports a
      // failure if it fails as well)
      if (tl == 0) {
        A.level[b] = 0;
        A.redo[b] = 1;
        A.flags[1] = 1;
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
      if (again) {
        A.flags[1] = 1;
        atomicAdd(info + SV_INFO_AUX, 1);
      }
    }
    const bool ok = active && !failed;

    // y and the first Z column at this lane's first two rows, loaded now so
    // that their latency passes during the a solve
    double ypre[2] = {0.0, 0.0}, zpre[2] = {0.0, 0.0};
    if (ok)
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int i = tl + u * G;
        if (i < K) {
          ypre[u] = Y[idx[i]];
          if (q > 0) zpre[u] = Zm[(int64_t)idx[i] * q];
        }
      }

    // ---- a = C^-T e_K = L^-T e_K / sqrt(d_K)  (unit back substitution)
    dfv lKKd = dzero, sKd = dzero;  // L_KK = sqrt(d_K) and its reciprocal
    if (ok) {
      sKd = df_sqrt(Lp[cm(k, k)]);  // the diagonal holds 1 / d_K
      lKKd = df_rcp(sKd);
      if (tl == 0) rec[0] = df_to_double(lKKd);  // L_KK; the log is taken in the reduction
      for (int i = tl; i < K; i += G) acc[i] = (i == k) ? df_make(1.0f, 0.0f) : dzero;
    }
    __syncwarp();
    for (int i = Kw - 1; i >= 0; --i) {
      if (ok && i < K) {
        const dfv ai = acc[i];
        for (int j = tl; j < i; j += G) acc[j] = df_fms(acc[j], Lp[cm(i, j)], ai);
      }
      __syncwarp();
    }
    if (ok)
      for (int i = tl; i < K; i += G) {
        const dfv ai = df_mul(acc[i], sKd);
        a[i] = ai;
        a32[i] = ai.hi;
      }
    __syncwarp();

    // ---- GLS parts a'y, a'Z (double-float team sums of unnormalised pairs);
    //      y and Z also take their columns of R for the forward solves
    {
      const int qw = __reduce_max_sync(full, active ? q : 0);
      // teams of one warp may belong to problems with different q: the
      // shuffles run to the warp's largest q
      for (int c = 0; c <= qw; ++c) {
        float s = 0.0f, t = 0.0f;
        if (ok && c <= q)
          for (int i = tl, u = 0; i < K; i += G, ++u) {
            double x;
            if (c <= 1 && u < 2)
              x = c == 0 ? (u == 0 ? ypre[0] : ypre[1]) : (u == 0 ? zpre[0] : zpre[1]);
            else
              x = c == 0 ? Y[idx[i]] : Zm[(int64_t)idx[i] * q + (c - 1)];
            const dfv v = df_from_double(x);
            if (A.need_grad) R[(P + c) * 33 + i] = v;
            df_fms_acc(s, t, a[i], df_make(-v.hi, -v.lo));
          }
        for (int o = G / 2; o > 0; o >>= 1) {
          const float so = __shfl_xor_sync(full, s, o), to = __shfl_xor_sync(full, t, o);
          float s3, e;
          two_sum(s, so, s3, e);
          s = s3;
          t = df_addf(t, df_addf(to, e));
        }
        if (ok && c <= q && tl == 0) rec[1 + c] = (double)s + (double)t;
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
      const dfv jitd = df_from_double(jit);
      for (int i = tl; i < K; i += G) {
        const dfv e = (i == k) ? lKKd : dzero;
        R[i] = jit == 0.0 ? e : df_fms(e, jitd, a[i]);
      }
      // p = 1..d (float32): -s2 sum_j g_ij a_j (u_il - u_jl)^2
      for (int i = tl; i < K; i += G) {
        auto store = [&](int c, float v) { R[c * 33 + i] = df_make(v, 0.0f); };
        if (d <= 4)
          split_dsig_row<4>(i, K, d, mf, s2f, u, a32, store);
        else if (d <= 8)
          split_dsig_row<8>(i, K, d, mf, s2f, u, a32, store);
        else if (d <= 12)
          split_dsig_row<12>(i, K, d, mf, s2f, u, a32, store);
        else
          split_dsig_row_wide(i, K, d, mf, s2f, u, a32, store);
      }
      // nugget row: dSigma_tau = s2 tau I
      const dfv s2taud = df_make(PI.s2t_hi, PI.s2t_lo);
      for (int i = tl; i < K; i += G) R[(P - 1) * 33 + i] = df_mul(s2taud, a[i]);
    }
    __syncwarp();

    // ---- forward solves (double-float) with the unit factor:
    // L^-1 [dSigma a, y, Z]; W = D^(-1/2) L^-1 dSigma a.  Without jitter
    // Sigma a = L_KK e_K, whose solution is sqrt(d_K) e_K, so that column is
    // left out of the solve.
    const int c0 = (jit == 0.0) ? 1 : 0;
    // columns c0 + tl, c0 + tl + G, ... per lane, with no warp
    // synchronisation between steps; kSplitWF steps per pass: the panel's
    // own rows are finished in order (and normalised), then every later row
    // takes the panel's updates in one visit, stored as an unnormalised
    // accumulator until its own step
    if (ok)
      for (int c = c0 + tl; c < NR; c += G) {
        dfv* col = R + c * 33;
        for (int i = 0; i < K - 1; i += kSplitWF) {
          const int ns = min(kSplitWF, K - 1 - i);  // steps i .. i+ns-1
          dfv r[kSplitWF];
#pragma unroll
          for (int s2 = 0; s2 < kSplitWF; ++s2)
            if (s2 < ns) {
              const dfv v0 = col[i + s2];
              float s = v0.hi, t = v0.lo;
#pragma unroll
              for (int t2 = 0; t2 < s2; ++t2) df_fms_acc(s, t, Lp[cm(i + s2, i + t2)], r[t2]);
              r[s2] = df_norm(s, t);
              col[i + s2] = r[s2];
            }
#pragma unroll kSplitJU
          for (int j = i + ns; j < K; ++j) {
            const dfv v0 = col[j];
            float s = v0.hi, t = v0.lo;
#pragma unroll
            for (int t2 = 0; t2 < kSplitWF; ++t2)
              if (t2 < ns) df_fms_acc(s, t, Lp[cm(j, i + t2)], r[t2]);
            col[j] = df_make(s, t);
          }
        }
        col[K - 1] = df_norm(col[K - 1].hi, col[K - 1].lo);
      }
    __syncwarp();
    if (ok) {
      if (c0 == 1)
        for (int i = tl; i < K; i += G) R[i] = (i == k) ? lKKd : dzero;
      // a32 is free now: it takes the float32 weights d_j^(-1/2)
      for (int j = tl; j < K; j += G) a32[j] = sqrtf(Lp[cm(j, j)].hi);
      // a is free: the last rows of the solutions times 1 / L_KK, in float64
      for (int c = tl; c < NR; c += G)
        wkd[c] = df_to_double(df_mul((c == 0 && c0 == 1) ? lKKd : R[c * 33 + k], sKd));
    }
    __syncwarp();

    // ---- record: z parts, w_K (float64), Gram products (float32) of the
    //      D^(-1/2)-weighted solutions
    if (ok) {
      for (int e = tl; e < NR * 33; e += G) {
        const int c = e / 33, j = e - (e / 33) * 33;
        R32[e] = (j < K) ? R[c * 33 + j].hi * a32[j] : 0.0f;
      }
    }
    __syncwarp();
    if (ok) {
      double* wK = rec + 3 + 2 * q;
      double* wzy = wK + P;
      double* wzZ = wzy + P;
      double* F = wzZ + P * q;
      for (int c = tl; c < 1 + q; c += G) rec[2 + q + c] = wkd[P + c];
      for (int p = tl; p < P; p += G) wK[p] = wkd[p];
      // Gram products G(c1, c2) = sum_i R32(i, c1) R32(i, c2) for c2 < P and
      // c2 <= c1 < NR (the Fisher triangle, then the y and Z columns), by 2x2
      // tiles: columns (c2, c2 + 1) for even c2, rows (c1, c1 + 1) for
      // c1 = c2, c2 + 2, ...; a lane takes one tile at a time, one shared-
      // memory load per FMA.  Each entry is the same sum in the same order as
      // alone; tile entries above the diagonal or outside the set are dropped.
      auto tiles_of = [&](int u) { return (NR - 2 * u + 1) / 2; };
      const int npair = (P + 1) / 2;
      int ntile = 0;
      for (int u = 0; u < npair; ++u) ntile += tiles_of(u);
      auto put = [&](int c1, int c2, float g) {
        if (c1 >= NR || c2 >= P || c1 < c2) return;
        if (c1 < P) {
          F[tri_off(c1, c2)] = fma(-0.5 * wkd[c1], wkd[c2], (double)g);
        } else if (c1 == P) {
          wzy[c2] = (double)g;
        } else {
          wzZ[c2 * q + (c1 - P - 1)] = (double)g;
        }
      };
      for (int t = tl; t < ntile; t += G) {
        int u = 0, rem = t;
        while (rem >= tiles_of(u)) {
          rem -= tiles_of(u);
          ++u;
        }
        const int c2 = 2 * u, c1 = 2 * u + 2 * rem;
        const float* xa = R32 + c1 * 33;
        const float* xb = R32 + min(c1 + 1, NR - 1) * 33;
        const float* ya = R32 + c2 * 33;
        const float* yb = R32 + min(c2 + 1, NR - 1) * 33;
        float g00 = 0.0f, g01 = 0.0f, g10 = 0.0f, g11 = 0.0f;
        for (int i = 0; i < K; ++i) {
          const float a0 = xa[i], a1 = xb[i], b0 = ya[i], b1 = yb[i];
          g00 = fmaf(a0, b0, g00);
          g01 = fmaf(a0, b1, g01);
          g10 = fmaf(a1, b0, g10);
          g11 = fmaf(a1, b1, g11);
        }
        put(c1, c2, g00);
        put(c1, c2 + 1, g01);
        put(c1 + 1, c2, g10);
        put(c1 + 1, c2 + 1, g11);
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

int launch_block_split_df(const LikArgs& A, int lanes, cudaStream_t st) {
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t per_warp =
      sizeof(double) * (size_t)split_slot_doubles(A.dmax, A.NRmax > kSplitW - 1 ? A.NRmax : kSplitW - 1, A.kcap) *
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
    SV_CUDA_TRY(cudaFuncSetAttribute(k_block_split_df<GV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)smem));                                                  \
    k_block_split_df<GV><<<(unsigned)grid, 32 * wpc, smem, st>>>(A, wpc);                            \
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
