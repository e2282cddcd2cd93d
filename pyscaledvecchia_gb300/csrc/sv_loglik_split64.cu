// The split-precision block kernel of the Vecchia likelihood / score /
// Fisher evaluation (blocks with K = k+1 <= 32; a closed-form nu or the
// float32 Matern table of a fixed nu): float32 assembly, float64
// factorisation.
//
// Same per-block record as the float64 kernels (likelihood.py:111-144 of the
// reference), with the precision of each step chosen by what conditioning
// needs:
//   float32 : centred scaled coordinates, distances, the correlation deficit
//             1 - M (accurate for close pairs) and g, the products dSigma_l a
//             (K^2 d) and the Fisher / score Gram products (trace
//             contractions), float32 accumulation;
//   float64 : the entries s2 (1 - D) and the diagonal s2 (1 + tau)
//             (+ jitter), the LDL^T factorisation (_batch_chol,
//             _covariance.py:235-252), a = L^-T e_K (_backsolve_LT,
//             likelihood.py:125-127), the forward solves W = L^-1 [dSigma a],
//             L^-1 y, L^-1 Z (_forward_solve, likelihood.py:139, 154), the
//             log-determinant term L_KK, the GLS sums, the record and every
//             reduction after it.
// A fixed nugget of 1e-8 drives block condition numbers toward 1e10, which is
// why the factorisation and solves stay in float64; blocks whose smallest
// pivot ratio d_k / Sigma_kk falls below rho_min (so ill-conditioned that
// the float32 assembly error would show), that do not factor even with
// jitter, or whose scale or data leave float32's exponent range, are
// re-evaluated by the all-float64 kernel.
//
// GB300 runs float64 at 1/64 of the float32 rate, and a float64 warp
// instruction costs the same with one active lane as with 32.  The kernel is
// laid out so that its float64 instructions carry as many lanes as possible:
//   * a block is owned by a team of G lanes and a warp holds 32/G blocks, so
//     every serial step (a pivot, a back-substitution step) is one
//     instruction for 32/G blocks at once;
//   * float32 <-> float64 conversions are bit manipulations on the integer
//     pipe, order and sign tests compare bit patterns;
//   * the factorisation is LDL^T (unit lower L, D = diag(d_k)): one
//     reciprocal per pivot (a float32 seed and a third-order correction in
//     three float64 FMAs), no square roots; the Cholesky factor is C = L D^(1/2), so
//     a = C^-T e_K = L^-T e_K / sqrt(d_K), W = D^(-1/2) L^-1 V (unit forward
//     solves, the D^(-1/2) weights applied in the float32 Gram) and
//     L_KK = sqrt(d_K);
//   * right-looking panels of kS64W columns: every trailing element takes the
//     panel's updates in one visit; the forward solves give each lane whole
//     columns with no synchronisation between steps.
//
// Warp-uniform outer loops (up to the warp's largest K) with team-local
// predication keep every __syncwarp reached by all lanes when the blocks of a
// warp differ in size.
#include "sv_split.cuh"

namespace sv {

constexpr int kS64MaxThreads = 384;
constexpr int kS64W = 8;    // columns per factorisation panel
constexpr int kS64WF = 16;  // steps per forward-solve pass
constexpr int kS64JU = 2;   // later rows per iteration of a forward-solve pass

// a pivot of the team's factorisation: LAPACK's criterion (a pivot that is
// not > 0, i.e. negative, zero or NaN, fails: flag[0]), the conditioning
// test against rho_min (flag[1]; rho_bits = bits of rho_min Sigma_kk) and the
// reciprocal, which takes the pivot's place on L's diagonal.
__device__ __forceinline__ void split64_pivot(double dkk, double* diag, long long rho_bits,
                                              volatile int* flag) {
  const long long bd = dbits(dkk);
  if (bd <= 0 || bd >= kBitsInf) {
    flag[0] = 1;
  } else {
    if (bd < rho_bits) flag[1] = 1;
    *diag = pivot_rcp64(dkk);
  }
}

// Entries (h, j < h) and (K-1-h, j < K-1-h) of Sigma below the diagonal,
// s2 (1 - D(r_ij)) as one float64 FMA of the float32 deficit, and both
// diagonal entries dj; u is [d][32] (row i at column i), the current row's
// coordinates are held in registers (DR >= d, 0: read from shared memory).
template <int DR>
__device__ __forceinline__ void split64_sigma_rows(int h, int K, int d, const MaternF32& mf, double s2,
                                                   double dj, const float* u, double* Lp, int kc) {
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
    Lp[cm(i, j, kc)] = fma(-s2, f2d_int(matern_deficit_f32(mf, sqrtf(r2))), s2);
  }
  Lp[cm(h, h, kc)] = dj;
  if (ib != h) Lp[cm(ib, ib, kc)] = dj;
}

template <int G>
__global__ void __launch_bounds__(kS64MaxThreads, 1) k_block_split64(LikArgs A, int wpc) {
  extern __shared__ double smem[];
  constexpr int NB = 32 / G;
  if (!pass_has_work(A)) return;
  const unsigned full = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tm = lane / G, tl = lane - (lane / G) * G;
  const unsigned tmask = (G == 32 ? full : ((1u << G) - 1u)) << (tm * G);
  const int dmax = A.dmax;
  // at least kS64W - 1 R columns: R's first columns and a are the
  // factorisation's scratch
  const int nrs = A.NRmax > kS64W - 1 ? A.NRmax : kS64W - 1;
  const int kc = A.kcap;
  const int64_t slot = split_slot_doubles(dmax, nrs, kc);
  double* Lp = smem + (int64_t)(warp * NB + tm) * slot;
  double* R = Lp + split_lp_cap(kc, nrs);  // NR columns, stride 33
  double* a = R + 33 * nrs;
  float* a32 = (float*)(a + 32);
  auto cm = [kc](int i, int j) { return sv::cm(i, j, kc); };
  float* u = a32 + 32;
  int* idx = (int*)(u + 32 * dmax);
  volatile int* tflag = idx + 32;
  double* acc = R;  // column 0 of R is scratch during the a solve
  // unscaled columns of a factorisation panel: R's first columns, then a
  double* accs[kS64W];
#pragma unroll
  for (int p = 0; p < kS64W; ++p) accs[p] = p < kS64W - 1 ? R + 33 * p : a;
  float* R32 = (float*)Lp;  // float32 copy of R once L is no longer needed
  double* wkd = a;          // last rows of the solutions times 1 / L_KK

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
    const double s2 = PI.s2;
    const float s2f = d2f_int(s2);
    const MaternF32 mf = PI.mf32;
    const double diag = PI.dg;
    const double* Y = A.y + PI.y_off;
    const double* Zm = A.Z + PI.z_off;
    const float2* XH = A.xhl + PI.x_off;
    int32_t* info = A.info + 4 * pid;
    // scale inside [1e-30, 1e30] and data below 1e30 in magnitude keep every
    // float32 quantity inside float32's exponent range; other blocks, and
    // the blocks of a problem whose nu has no float32 form here, go to the
    // float64 pass
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
      for (int i = tl; i < K; i += G) {
        data_ok = data_ok && in_f32_range(Y[idx[i]]);
        for (int c = 0; c < q; ++c) data_ok = data_ok && in_f32_range(Zm[(int64_t)idx[i] * q + c]);
      }
    }
    range_ok = range_ok && (__ballot_sync(full, !data_ok) & tmask) == 0;
    __syncwarp();

    // ---- Sigma (float32 deficit, float64 entries) and LDL^T with the
    //      jitter ladder of _covariance.py:235-252
    int lv = (active && A.fixup) ? chunk_level(A, b) : 0;
    bool done = !active || !range_ok, failed = active && !range_ok;
    double jit = 0.0;
    long long rho_bits = 0;
    while (__any_sync(full, !done)) {
      const bool need = !done;
      if (need) {
        jit = (lv > 0) ? jitter_pow10(lv) * diag : 0.0;  // 10^p * mean(diag)
        const double dj = (lv > 0) ? diag + jit : diag;
        rho_bits = dbits(A.rho_min * dj);
        // lane h takes rows h and K-1-h (K-1 entries below the diagonal
        // between them)
        for (int h = tl; 2 * h < K; h += G) {
          if (d <= 4)
            split64_sigma_rows<4>(h, K, d, mf, s2, dj, u, Lp, kc);
          else if (d <= 8)
            split64_sigma_rows<8>(h, K, d, mf, s2, dj, u, Lp, kc);
          else if (d <= 12)
            split64_sigma_rows<12>(h, K, d, mf, s2, dj, u, Lp, kc);
          else
            split64_sigma_rows<0>(h, K, d, mf, s2, dj, u, Lp, kc);
        }
        if (tl == 0) {
          tflag[0] = 0;  // a pivot failed
          tflag[1] = 0;  // a pivot ratio d_k / Sigma_kk fell below rho_min
        }
      }
      __syncwarp();
      if (need && tl == 0) split64_pivot(Lp[0], Lp, rho_bits, tflag);
      __syncwarp();
      // right-looking LDL^T, kS64W columns (a panel) per step, warp-uniform
      // loop.  Panel column c = kk + p takes the steps kk .. c-1 in order (its
      // pivot follows at once), then is scaled by 1/d_c, its unscaled values
      // in accs[p]; every trailing element (j >= kk + kS64W) then takes all
      // kS64W updates in one visit, a(i,j) - l(i,s) a(j,s) for s = kk, kk+1,
      // ... in order.  The lane that updates (kk+W, kk+W) takes that pivot's
      // reciprocal at once (look-ahead).  A failed pivot stops the attempt
      // (it is redone with jitter).
      auto colp = [&](int c) { return Lp + cstart(c, kc) - c; };  // colp(c)[i] = L(i, c)
      for (int kk = 0; kk < Kw; kk += kS64W) {
        bool go = need && kk < K && tflag[0] == 0;
#pragma unroll
        for (int p = 0; p < kS64W; ++p) {
          const int c = kk + p;
          if (p > 0) {
            if (go && c < K) {
              double* colc = colp(c);
              for (int i = c + tl; i < K; i += G) {
                double v = colc[i];
#pragma unroll
                for (int s2i = 0; s2i < p; ++s2i) v = fma(-colp(kk + s2i)[i], accs[s2i][c], v);
                colc[i] = v;
                accs[p][i] = v;
                if (i == c) split64_pivot(v, colc + c, rho_bits, tflag);
              }
            }
            __syncwarp();
            go = go && tflag[0] == 0;
          }
          if (go && c < K) {
            double* colc = colp(c);
            const double inv = colc[c];
            for (int i = c + 1 + tl; i < K; i += G) {
              const double v = p == 0 ? colc[i] : accs[p][i];
              if (p == 0) accs[0][i] = v;
              colc[i] = v * inv;
            }
          }
          __syncwarp();
        }
        if (go) {
          const int j0 = kk + kS64W;
          const int m = K - j0;
          const int cnt = m > 0 ? m * (m + 1) / 2 : 0;
          if (tl < cnt) {
            int j = j0, rem = tl;
            while (rem >= K - j) {
              rem -= K - j;
              ++j;
            }
            for (int t = tl; t < cnt; t += G) {
              const int jj = j, ii = j + rem;
              rem += G;
              while (j < K && rem >= K - j) {
                rem -= K - j;
                ++j;
              }
              double v = Lp[cm(ii, jj)];
#pragma unroll
              for (int s2i = 0; s2i < kS64W; ++s2i) v = fma(-colp(kk + s2i)[ii], accs[s2i][jj], v);
              Lp[cm(ii, jj)] = v;
              if (ii == j0 && jj == j0) split64_pivot(v, Lp + cm(j0, j0), rho_bits, tflag);
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
      for (int uu = 0; uu < 2; ++uu) {
        const int i = tl + uu * G;
        if (i < K) {
          ypre[uu] = Y[idx[i]];
          if (q > 0) zpre[uu] = Zm[(int64_t)idx[i] * q];
        }
      }

    // ---- a = C^-T e_K = L^-T e_K / sqrt(d_K)  (unit back substitution)
    double lKK = 0.0, sK = 0.0;  // L_KK = sqrt(d_K) and its reciprocal
    if (ok) {
      sK = sqrt(Lp[cm(k, k)]);  // the diagonal holds 1 / d_K
      lKK = pivot_rcp64(sK);
      if (tl == 0) rec[0] = lKK;  // L_KK; the log is taken in the reduction
      for (int i = tl; i < K; i += G) acc[i] = (i == k) ? 1.0 : 0.0;
    }
    __syncwarp();
    for (int i = Kw - 1; i >= 0; --i) {
      if (ok && i < K) {
        const double ai = acc[i];
        for (int j = tl; j < i; j += G) acc[j] = fma(-Lp[cm(i, j)], ai, acc[j]);
      }
      __syncwarp();
    }
    if (ok)
      for (int i = tl; i < K; i += G) {
        const double ai = acc[i] * sK;
        a[i] = ai;
        a32[i] = d2f_int(ai);
      }
    __syncwarp();

    // ---- GLS parts a'y, a'Z (float64 team sums); y and Z also take their
    //      columns of R for the forward solves
    {
      const int qw = __reduce_max_sync(full, active ? q : 0);
      // teams of one warp may belong to problems with different q: the
      // shuffles run to the warp's largest q
      for (int c = 0; c <= qw; ++c) {
        double s = 0.0;
        if (ok && c <= q)
          for (int i = tl, uu = 0; i < K; i += G, ++uu) {
            double x;
            if (c <= 1 && uu < 2)
              x = c == 0 ? (uu == 0 ? ypre[0] : ypre[1]) : (uu == 0 ? zpre[0] : zpre[1]);
            else
              x = c == 0 ? Y[idx[i]] : Zm[(int64_t)idx[i] * q + (c - 1)];
            if (A.need_grad) R[(P + c) * 33 + i] = x;
            s = fma(a[i], x, s);
          }
        for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(full, s, o);
        if (ok && c <= q && tl == 0) rec[1 + c] = s;
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
      for (int i = tl; i < K; i += G) {
        const double e = (i == k) ? lKK : 0.0;
        R[i] = lv == 0 ? e : fma(-jit, a[i], e);
      }
      // p = 1..d (float32): -s2 sum_j g_ij a_j (u_il - u_jl)^2
      for (int i = tl; i < K; i += G) {
        auto store = [&](int c, float v) { R[c * 33 + i] = f2d_int(v); };
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
      for (int i = tl; i < K; i += G) R[(P - 1) * 33 + i] = PI.s2t * a[i];
    }
    __syncwarp();

    // ---- forward solves with the unit factor: L^-1 [dSigma a, y, Z];
    // W = D^(-1/2) L^-1 dSigma a.  Without jitter Sigma a = L_KK e_K, whose
    // solution is sqrt(d_K) e_K, so that column is left out of the solve.
    const int c0 = lv == 0 ? 1 : 0;
    // columns c0 + tl, c0 + tl + G, ... per lane, with no warp
    // synchronisation between steps; kS64WF steps per pass: the pass's own
    // rows are finished in order, then every later row takes the pass's
    // updates in one visit
    if (ok)
      for (int c = c0 + tl; c < NR; c += G) {
        double* col = R + c * 33;
        for (int i = 0; i < K - 1; i += kS64WF) {
          const int ns = min(kS64WF, K - 1 - i);  // steps i .. i+ns-1
          double r[kS64WF];
#pragma unroll
          for (int s2i = 0; s2i < kS64WF; ++s2i)
            if (s2i < ns) {
              double v = col[i + s2i];
#pragma unroll
              for (int t2 = 0; t2 < s2i; ++t2) v = fma(-Lp[cm(i + s2i, i + t2)], r[t2], v);
              r[s2i] = v;
              col[i + s2i] = v;
            }
#pragma unroll kS64JU
          for (int j = i + ns; j < K; ++j) {
            double v = col[j];
#pragma unroll
            for (int t2 = 0; t2 < kS64WF; ++t2)
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
      for (int j = tl; j < K; j += G) a32[j] = sqrtf(d2f_int(Lp[cm(j, j)]));
      // a is free: the last rows of the solutions times 1 / L_KK
      for (int c = tl; c < NR; c += G) wkd[c] = ((c == 0 && c0 == 1) ? lKK : R[c * 33 + k]) * sK;
    }
    __syncwarp();

    // ---- record: z parts, w_K (float64), Gram products (float32) of the
    //      D^(-1/2)-weighted solutions
    if (ok) {
      for (int e = tl; e < NR * 33; e += G) {
        const int c = e / 33, j = e - (e / 33) * 33;
        R32[e] = (j < K) ? d2f_int(R[c * 33 + j]) * a32[j] : 0.0f;
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
      // memory load per FMA.  Tile entries above the diagonal or outside the
      // set are dropped.
      auto tiles_of = [&](int t) { return (NR - 2 * t + 1) / 2; };
      const int npair = (P + 1) / 2;
      int ntile = 0;
      for (int t = 0; t < npair; ++t) ntile += tiles_of(t);
      auto put = [&](int c1, int c2, float g) {
        if (c1 >= NR || c2 >= P || c1 < c2) return;
        if (c1 < P) {
          F[tri_off(c1, c2)] = fma(-0.5 * wkd[c1], wkd[c2], f2d_int(g));
        } else if (c1 == P) {
          wzy[c2] = f2d_int(g);
        } else {
          wzZ[c2 * q + (c1 - P - 1)] = f2d_int(g);
        }
      };
      for (int t = tl; t < ntile; t += G) {
        int pu = 0, rem = t;
        while (rem >= tiles_of(pu)) {
          rem -= tiles_of(pu);
          ++pu;
        }
        const int c2 = 2 * pu, c1 = 2 * pu + 2 * rem;
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

int launch_block_split(const LikArgs& A, int lanes, cudaStream_t st) {
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t per_warp =
      sizeof(double) * (size_t)split_slot_doubles(A.dmax, A.NRmax > kS64W - 1 ? A.NRmax : kS64W - 1, A.kcap) *
      (32 / lanes);
  int wpc = kS64MaxThreads / 32;
  while (wpc > 1 && wpc * per_warp > (size_t)maxsm) --wpc;
  const size_t smem = wpc * per_warp;
  if (smem > (size_t)maxsm) return SV_EINVAL;
  const int64_t nb = A.b1 - A.b0;
  const int64_t per_cta = (int64_t)wpc * (32 / lanes);
  int64_t need = (nb + per_cta - 1) / per_cta;
  const int nsm = sv_num_sms();
  // persistent grid: the CTAs that fit on the SMs at once, each warp taking
  // blocks in a grid-stride loop (warps drift apart, so the phases with
  // little float64 work of some warps overlap the float64 work of others;
  // no per-CTA tail)
  auto grid_for = [&](const void* fn) -> int64_t {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * wpc, smem) != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    int64_t g = need < (int64_t)per_sm * nsm ? need : (int64_t)per_sm * nsm;
    return g < 1 ? 1 : g;
  };
  switch (lanes) {
#define SV_S64_CASE(GV)                                                                              \
  case GV: {                                                                                         \
    SV_CUDA_TRY(cudaFuncSetAttribute(k_block_split64<GV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)smem));                                                    \
    const int64_t grid = grid_for((const void*)k_block_split64<GV>);                               \
    k_block_split64<GV><<<(unsigned)grid, 32 * wpc, smem, st>>>(A, wpc);                            \
    break;                                                                                           \
  }
    SV_S64_CASE(4)
    SV_S64_CASE(8)
    SV_S64_CASE(16)
    SV_S64_CASE(32)
#undef SV_S64_CASE
    default:
      return SV_EINVAL;
  }
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

}  // namespace sv
