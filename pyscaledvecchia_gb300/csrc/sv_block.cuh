// Team-level building blocks of the Vecchia block kernels.
//
// A "team" of T threads owns one conditioning block at a time: T = 32 is one
// warp (blocks of size K <= 32), T = blockDim.x is a whole CTA (K > 32).  All
// of a team's data lives in shared memory; work inside a step is spread over
// the team's lanes with a strided loop, steps are separated by team barriers.
//
// Storage of a K x K symmetric/lower matrix is the packed lower triangle,
// row-major: entry (i, j), i >= j, at i(i+1)/2 + j.
#pragma once
#include "sv_common.cuh"
#include "sv_matern.cuh"

namespace sv {

template <int T>
struct Team {
  // T == 16: one half of a warp (two blocks per warp, each half with its own
  // control flow); T == 32: one warp; T > 32: the whole CTA (T == blockDim.x)
  __device__ __forceinline__ static int lane() {
    return T == 16 ? (threadIdx.x & 15) : T == 32 ? (threadIdx.x & 31) : threadIdx.x;
  }
  __device__ __forceinline__ static unsigned mask() {
    return T == 16 ? (0xFFFFu << (threadIdx.x & 16)) : 0xffffffffu;
  }
  __device__ __forceinline__ static void sync() {
    if (T == 16)
      __syncwarp(mask());
    else if (T == 32)
      __syncwarp();
    else
      __syncthreads();
  }
};

// Matern evaluation mode of a block
struct MaternMode {
  int closed;          // 0/1/2 for nu = 0.5/1.5/2.5, -1 = general (Bessel)
  int estimate_nu;     // also dM/dnu by central difference
  double nu;           // smoothness
  double log_coef;     // (1-nu) ln2 - lgamma(nu)
  double nu_p, nu_m;   // nu +- h
  double lc_p, lc_m;   // log_coef at nu +- h
  double inv2h;        // 1 / (2h)
  const double* tab;   // general nu: the table of M and g (or null)
  int tab_elo;         // its first octave
  double s2n;          // sqrt(2 nu)
  // estimated nu with tables: those of nu + h and nu - h
  const double* tab_p;
  const double* tab_m;
  int elo_p, elo_m;
  double s2n_p, s2n_m;
};

__device__ __forceinline__ void matern_eval(const MaternMode& mm, double r, double& M, double& g,
                                            double& dMnu, bool want_g) {
  if (mm.closed >= 0) {
    matern_closed(mm.closed, r, M, g);
    dMnu = 0.0;
    return;
  }
  if (mm.tab) {
    matern_table_Mg(mm.tab, mm.tab_elo, mm.s2n, mm.nu, mm.log_coef, r, M, g, want_g);
    dMnu = 0.0;
    if (mm.estimate_nu) {
      // _matern_general.py:170-176 (central difference in nu), M at nu +- h
      // from their tables
      double Mp, Mm, gx;
      matern_table_Mg(mm.tab_p, mm.elo_p, mm.s2n_p, mm.nu_p, mm.lc_p, r, Mp, gx, false);
      matern_table_Mg(mm.tab_m, mm.elo_m, mm.s2n_m, mm.nu_m, mm.lc_m, r, Mm, gx, false);
      dMnu = (Mp - Mm) * mm.inv2h;
    }
    return;
  }
  if (want_g) {
    matern_general_Mg(r, mm.nu, mm.log_coef, M, g);
  } else {
    M = matern_general_M(r, mm.nu, mm.log_coef);
    g = 0.0;
  }
  if (mm.estimate_nu) {
    // _matern_general.py:170-176 (central difference in nu)
    const double Mp = matern_general_M(r, mm.nu_p, mm.lc_p);
    const double Mm = matern_general_M(r, mm.nu_m, mm.lc_m);
    dMnu = (Mp - Mm) * mm.inv2h;
  } else {
    dMnu = 0.0;
  }
}

// Assemble the packed lower triangle of Sigma (+ jitter on the diagonal) for
// a block whose scaled coordinates u (K x d, row-major) are in shared memory.
//   nug[i]  : nugget multiplier of entry i (1 observation, 0 noise-free)
//   Gp, Dp  : optional packed -s2*g and s2*nu*dM/dnu (derivative factors)
template <int T>
__device__ void assemble_sigma(int K, int d, const double* u, const double* nugmask, double s2,
                               double tau, double jit, const MaternMode& mm, double* Lp,
                               double* Gp, double* Dp) {
  const int lane = Team<T>::lane();
  const int npair = K * (K + 1) / 2;
  // g at r = 0 (the diagonal): the closed forms' -3 (nu = 1.5) and -5/3
  // (nu = 2.5); 0 for nu = 0.5 and the general form (r below its floor)
  const double g0 = mm.closed == 1 ? -3.0 : mm.closed == 2 ? -(5.0 / 3.0) : 0.0;
  for (int t = lane; t < npair; t += T) {
    int i, j;
    tri_index(t, i, j);
    double M, g, dMnu;
    if (i == j) {
      // r = 0: M = 1 and dM/dnu = 0, the values the routines below return
      // there, without their square root and exponential
      M = 1.0;
      g = g0;
      dMnu = 0.0;
    } else {
      const double* ui = u + i * d;
      const double* uj = u + j * d;
      double s = 0.0;
      for (int l = 0; l < d; ++l) {
        const double df = ui[l] - uj[l];
        s += df * df;
      }
      const double r = sqrt(s);
      matern_eval(mm, r, M, g, dMnu, Gp != nullptr);
    }
    double nug = 0.0;
    if (i == j) nug = tau * (nugmask ? nugmask[i] : 1.0);
    double v = s2 * (M + nug);
    if (i == j) v += jit;
    Lp[t] = v;
    if (Gp) Gp[t] = -s2 * g;
    if (Dp) Dp[t] = s2 * mm.nu * dMnu;
  }
}

// In-place right-looking Cholesky of the packed lower triangle.  Pivots
// follow LAPACK dpotrf: a pivot that is not > 0 (or NaN) fails.  On success
// invd[k] = 1/L_kk.  Returns true on success (team-uniform).
template <int T>
__device__ bool cholesky_packed(int K, double* Lp, double* invd, volatile int* flag) {
  const int lane = Team<T>::lane();
  for (int k = 0; k < K; ++k) {
    const int kk = tri_off(k, k);
    if (lane == 0) {
      const double dkk = Lp[kk];
      if (!(dkk > 0.0)) {
        *flag = 1;
      } else {
        const double lkk = sqrt(dkk);
        Lp[kk] = lkk;
        invd[k] = 1.0 / lkk;
      }
    }
    Team<T>::sync();
    if (*flag) return false;
    const double inv = invd[k];
    for (int i = k + 1 + lane; i < K; i += T) Lp[tri_off(i, k)] *= inv;
    Team<T>::sync();
    const int m = K - k - 1;
    const int cnt = m * (m + 1) / 2;
    for (int t = lane; t < cnt; t += T) {
      int ii, jj;
      tri_index(t, ii, jj);
      const int i = k + 1 + ii, j = k + 1 + jj;
      Lp[tri_off(i, j)] -= Lp[tri_off(i, k)] * Lp[tri_off(j, k)];
    }
    Team<T>::sync();
  }
  return true;
}

// float64 reciprocal of a pivot inside [1e-30, 1e30]: the float32
// reciprocal y of the rounded pivot (relative error e = 1 - d y, |e| below
// ~2^-23) corrected by the third-order step y (1 + e + e^2), whose
// truncation error y e^3 (~2^-69) lies far below float64 rounding: three
// float64 FMAs (e exact to float64 rounding by the FMA, e + e^2, y + y t),
// the result within an ulp of 1/d.  Pivots outside that range take the
// float64 division.
__device__ __forceinline__ double pivot_rcp64(double d) {
  const long long b = dbits(d);
  if (b > kBitsTiny && b < kBitsHuge) {
    const double y = f2d_int(__frcp_rn(d2f_int(d)));
    const double e = fma(-d, y, 1.0);
    return fma(y, fma(e, e, e), y);
  }
  return 1.0 / d;
}

// LAPACK dpotrf's pivot criterion (a pivot that is not > 0 fails: negative,
// zero or NaN) as a test of the bit pattern on the integer pipe
__device__ __forceinline__ bool pivot_positive(double d) {
  const long long b = dbits(d);
  return b > 0 && b < kBitsInf;
}

// LDL^T of the packed lower triangle in place (unit L below the diagonal,
// D = diag(d_k) on it): one reciprocal per step instead of a square root and
// a division.  Fails as the Cholesky does (LAPACK dpotrf: a pivot that is not
// > 0, d_k = L_kk^2).  acc is K doubles of scratch.  With rb (the bit
// patterns of per-row thresholds), a pivot below its row's threshold stops
// the factorisation too (*flag = 2: too ill-conditioned for the entries'
// precision).
template <int T>
__device__ bool ldlt_packed(int K, double* Lp, double* invd, double* acc, volatile int* flag,
                            const long long* rb = nullptr) {
  const int lane = Team<T>::lane();
  for (int k = 0; k < K; ++k) {
    if (lane == 0) {
      const double dkk = Lp[tri_off(k, k)];
      if (!pivot_positive(dkk))
        *flag = 1;
      else if (rb && dbits(dkk) < rb[k])
        *flag = 2;
      else
        invd[k] = pivot_rcp64(dkk);
    }
    Team<T>::sync();
    if (*flag) return false;
    const double inv = invd[k];
    for (int i = k + 1 + lane; i < K; i += T) {
      const double v = Lp[tri_off(i, k)];
      acc[i] = v;
      Lp[tri_off(i, k)] = v * inv;
    }
    Team<T>::sync();
    const int m = K - k - 1;
    const int cnt = m * (m + 1) / 2;
    for (int t = lane; t < cnt; t += T) {
      int ii, jj;
      tri_index(t, ii, jj);
      const int i = k + 1 + ii, j = k + 1 + jj;
      Lp[tri_off(i, j)] -= Lp[tri_off(i, k)] * acc[j];  // a_ij -= l_ik d_k l_jk
    }
    Team<T>::sync();
  }
  return true;
}

// The same LDL^T by panels of W columns: the panel's columns are factored
// one by one (pivot, scaling, updates of the panel's later columns), then
// every element right of the panel takes the panel's W updates in one visit,
// a_ij - l_is (d_s l_js) for s = kk, kk+1, ... in order, so every element
// sees the same operations in the same order as in ldlt_packed (the results
// are bitwise equal).  One load and one store of a_ij per panel instead of
// per column, and three barriers per column only over the panel's W columns.
// accs: W columns of ldacc doubles holding the panel's unscaled columns
// d_s l_js (accs column 0 doubles as ldlt_packed's acc).
template <int T, int W>
__device__ bool ldlt_blocked(int K, double* Lp, double* invd, double* accs, int ldacc,
                             volatile int* flag, const long long* rb = nullptr) {
  const int lane = Team<T>::lane();
  for (int kk = 0; kk < K; kk += W) {
    const int ke = kk + W < K ? kk + W : K;
    for (int c = kk; c < ke; ++c) {
      if (lane == 0) {
        const double dcc = Lp[tri_off(c, c)];
        if (!pivot_positive(dcc))
          *flag = 1;
        else if (rb && dbits(dcc) < rb[c])
          *flag = 2;
        else
          invd[c] = pivot_rcp64(dcc);
      }
      Team<T>::sync();
      if (*flag) return false;
      const double inv = invd[c];
      double* ac = accs + (c - kk) * ldacc;
      for (int i = c + 1 + lane; i < K; i += T) {
        const double v = Lp[tri_off(i, c)];
        ac[i] = v;
        Lp[tri_off(i, c)] = v * inv;
      }
      Team<T>::sync();
      // the panel's later columns j in (c, ke), rows i >= j
      const int np = ke - c - 1;
      if (np > 0) {
        const int cnt = (K - c - 1) * np;
        for (int t = lane; t < cnt; t += T) {
          const int i = c + 1 + t / np, j = c + 1 + t % np;
          if (j <= i) Lp[tri_off(i, j)] -= Lp[tri_off(i, c)] * ac[j];
        }
        Team<T>::sync();
      }
    }
    // everything right of the panel: rows and columns >= ke
    const int m = K - ke;
    const int cnt = m * (m + 1) / 2;
    const int w = ke - kk;
    for (int t = lane; t < cnt; t += T) {
      int ii, jj;
      tri_index(t, ii, jj);
      const int i = ke + ii, j = ke + jj;
      const double* li = Lp + tri_off(i, kk);
      double v = Lp[tri_off(i, j)];
      if (w == W) {
#pragma unroll
        for (int p = 0; p < W; ++p) v -= li[p] * accs[p * ldacc + j];
      } else {
        for (int p = 0; p < w; ++p) v -= li[p] * accs[p * ldacc + j];
      }
      Lp[tri_off(i, j)] = v;
    }
    Team<T>::sync();
  }
  return true;
}

// u = L^-T e_K for a unit lower L (packed); u_K = 1.
template <int T>
__device__ void backsolve_unit_eK(int K, const double* Lp, double* u, double* acc) {
  const int lane = Team<T>::lane();
  for (int i = lane; i < K; i += T) acc[i] = (i == K - 1) ? 1.0 : 0.0;
  Team<T>::sync();
  for (int i = K - 1; i >= 0; --i) {
    const double ui = acc[i];
    for (int j = lane; j < i; j += T) acc[j] -= Lp[tri_off(i, j)] * ui;
    if (lane == 0) u[i] = ui;
    Team<T>::sync();
  }
}

// a = L^-T e_K (the block's column of the sparse inverse Cholesky factor).
// acc is K doubles of scratch.
template <int T>
__device__ void backsolve_eK(int K, const double* Lp, const double* invd, double* a, double* acc) {
  const int lane = Team<T>::lane();
  for (int i = lane; i < K; i += T) acc[i] = (i == K - 1) ? 1.0 : 0.0;
  Team<T>::sync();
  for (int i = K - 1; i >= 0; --i) {
    // a_i = acc_i / L_ii, then acc_j -= L_ij a_i for j < i
    const double ai = acc[i] * invd[i];
    for (int j = lane; j < i; j += T) acc[j] -= Lp[tri_off(i, j)] * ai;
    if (lane == 0) a[i] = ai;
    Team<T>::sync();
  }
}

// Forward solve L W = R for NR right-hand sides stored column-major with
// leading dimension ldr (R[c*ldr + i]), in place.
template <int T>
__device__ void forward_solve_multi(int K, const double* Lp, const double* invd, double* R, int NR,
                                    int ldr) {
  const int lane = Team<T>::lane();
  for (int i = 0; i < K; ++i) {
    for (int c = lane; c < NR; c += T) R[c * ldr + i] *= invd[i];
    Team<T>::sync();
    const int m = K - i - 1;
    const int cnt = m * NR;
    for (int t = lane; t < cnt; t += T) {
      const int c = t / m;
      const int j = i + 1 + (t - c * m);
      R[c * ldr + j] -= Lp[tri_off(j, i)] * R[c * ldr + i];
    }
    Team<T>::sync();
  }
}

// Forward solve L W = R with a unit lower L (packed, diagonal ignored) for
// NR right-hand sides stored column-major with leading dimension ldr, in place.
template <int T>
__device__ void forward_solve_unit_multi(int K, const double* Lp, double* R, int NR, int ldr) {
  const int lane = Team<T>::lane();
  for (int i = 0; i < K - 1; ++i) {
    const int m = K - i - 1;
    const int cnt = m * NR;
    for (int t = lane; t < cnt; t += T) {
      const int c = t / m;
      const int j = i + 1 + (t - c * m);
      R[c * ldr + j] -= Lp[tri_off(j, i)] * R[c * ldr + i];
    }
    Team<T>::sync();
  }
}

// Team-wide sum of a per-lane value (result valid in every lane).  A
// 16-lane team's tree is the 32-lane tree without its first step, which for
// a block of at most 16 points adds the zeros of lanes 16..31.
template <int T>
__device__ double team_sum(double v, double* red) {
  if (T == 16) {
    for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(Team<16>::mask(), v, o, 16);
    return v;
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (T == 32) return v;
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int k = 0; k < T / 32; ++k) s += red[k];
  __syncthreads();
  return s;
}

}  // namespace sv
