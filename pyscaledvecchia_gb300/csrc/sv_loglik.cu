// Profile Vecchia log-likelihood, score and Fisher information on the GPU.
//
// Follows likelihood.py:66-175 (vecchia_profile_loglik) of the reference:
//   pass 1 (per block, likelihood.py:111-144): Sigma and dSigma factors
//     (_covariance.py:111-147 / _matern_general.py:134-179), Cholesky with
//     jitter retry (_covariance.py:235-252), a = L^-T e_K, the GLS parts
//     a.y, a.Z, W = L^-1 (dSigma a) and the block's Fisher contribution;
//   beta = solve(XtX + 1e-12 I, Zty)  (likelihood.py:146);
//   pass 2 (likelihood.py:149-162): z = L^-1 (y - Z beta), ll and score.
// Pass 2 needs only the K-th entry of z and the products W z, which are
// linear in beta; pass 1 therefore stores, per block, (L^-1 y)_K, (L^-1 Z)_K,
// W (L^-1 y) and W (L^-1 Z) instead of L and W, so pass 2 is a light
// reduction over that per-block record.
//
// An evaluation covers a batch of independent problems (one for
// sv_vecchia_loglik): every block carries its problem index, so one launch of
// the block kernel processes the blocks of all problems.
//
// Kernels: k_prob_params (theta -> per-problem parameters), k_block_warp (one
// warp per block, K <= 32), k_block_cta (one CTA per block, K > 32),
// k_chunk_max / fix-up pass (reference chunk-wide jitter), k_reduce1 /
// k_final1 (GLS + Fisher sums, beta), k_reduce2 / k_final2 (ll, score,
// variance penalty).  Reductions are in a fixed order, so results are bitwise
// reproducible run to run.  Only kernels and memsets are enqueued, so a
// batched evaluation can be captured in a CUDA graph.
#include <stdio.h>

#include <algorithm>
#include <atomic>

#include "sv_loglik.cuh"

namespace sv {

// the central difference step of an estimated nu (_matern_general.py:135, nu_fd_h)
constexpr double kNuFdH = 1e-3;

// the smoothness of problem D at theta th (fixed, or estimated: exp of its
// entry of theta)
__device__ __forceinline__ double problem_nu(const sv_prob_desc& D, const double* th) {
  return D.estimate_nu ? exp(th[1 + D.d]) : D.nu;
}

// whether problem D interpolates its Matern from tables at smoothness nu: a
// fixed nu without a closed form, at most 10, whose floor octave the table
// reaches; an estimated nu whose nu - h and nu + h are in that range
__device__ __forceinline__ bool uses_matern_table(const sv_prob_desc& D, double nu) {
  return D.estimate_nu ? mtab_est_ok(nu, kNuFdH) : mtab_ok(nu);
}

// theta -> per-problem parameters (sigma^2, tau, nu, 1/lambda)
__global__ void k_prob_params(const sv_prob_desc* descs, const double* theta, int tstride,
                              int nprob, ProbInfo* out, const double* mtabs, int ftabs) {
  const int p = blockIdx.x;
  if (p >= nprob) return;
  const sv_prob_desc& D = descs[p];
  ProbInfo& I = out[p];
  const double* th = theta + (int64_t)p * tstride;
  const int d = D.d;
  if (threadIdx.x == 0) {
    I.n = D.n;
    I.x_off = D.x_off;
    I.y_off = D.y_off;
    I.z_off = D.z_off;
    I.blk_off = D.blk_off;
    I.nblk = D.nblk;
    I.d = d;
    I.q = D.q;
    I.estimate_nu = D.estimate_nu;
    I.skip = D.skip;
    I.P = d + 2 + (D.estimate_nu ? 1 : 0);
    I.nu_fixed = D.nu;
    I.var_penalty = D.var_penalty;
    I.log_var_target = D.log_var_target;
    I.s2 = exp(th[0]);
    double nu = D.nu;
    if (D.estimate_nu) {
      nu = exp(th[1 + d]);
      I.tau = exp(th[2 + d]);
    } else {
      I.tau = exp(th[1 + d]);
    }
    {
      const double dg = I.s2 * (1.0 + I.tau), s2t = I.s2 * I.tau;
      I.dg = dg;
      I.s2t = s2t;
      I.s2_hi = (float)I.s2;
      I.s2_lo = (float)(I.s2 - (double)I.s2_hi);
      I.dg_hi = (float)dg;
      I.dg_lo = (float)(dg - (double)I.dg_hi);
      I.s2t_hi = (float)s2t;
      I.s2t_lo = (float)(s2t - (double)I.s2t_hi);
    }
    MaternMode mm;
    mm.closed = D.estimate_nu ? -1 : matern_closed_code(D.nu);
    I.closed = mm.closed;
    mm.estimate_nu = D.estimate_nu;
    mm.nu = nu;
    mm.log_coef = (mm.closed < 0) ? matern_log_coef(nu) : 0.0;
    const double h = kNuFdH;
    mm.nu_p = nu + h;
    mm.nu_m = nu - h;
    mm.lc_p = D.estimate_nu ? matern_log_coef(mm.nu_p) : 0.0;
    mm.lc_m = D.estimate_nu ? matern_log_coef(mm.nu_m) : 0.0;
    mm.inv2h = 1.0 / (2.0 * h);
    // general nu: M and g from the tables built for this call (an estimated
    // nu also M at nu +- h)
    mm.tab = (mtabs && uses_matern_table(D, nu)) ? mtabs + (size_t)p * kMtabSlotDoubles : nullptr;
    mm.tab_elo = mm.tab ? mtab_elo(nu) : 0;
    mm.s2n = sqrt(2.0 * nu);
    const bool est_tab = mm.tab && D.estimate_nu;
    mm.tab_p = est_tab ? mm.tab + kMtabOffP : nullptr;
    mm.tab_m = est_tab ? mm.tab + kMtabOffM : nullptr;
    mm.elo_p = est_tab ? mtab_elo(mm.nu_p) : 0;
    mm.elo_m = est_tab ? mtab_elo(mm.nu_m) : 0;
    mm.s2n_p = sqrt(2.0 * mm.nu_p);
    mm.s2n_m = sqrt(2.0 * mm.nu_m);
    I.mm = mm;
    // split kernels: a closed form, the float32 tables, or none
    MaternF32 mf;
    mf.code = mm.closed;
    mf.elo = mm.tab_elo;
    mf.esw = ftab_switch(nu);
    mf.s2n = (float)mm.s2n;
    mf.tab = nullptr;
    mf.dtab = nullptr;
    mf.nuf = (float)nu;
    if (mf.code < 0 && mm.tab && ftabs && (D.estimate_nu ? ftab_est_ok(nu, h) : ftab_ok(nu))) {
      mf.code = 3;
      mf.tab = (const float4*)(mm.tab + kFtabOff);
      if (D.estimate_nu) mf.dtab = (const float4*)(mm.tab + kDtabOff);
    }
    I.mf32 = mf;
  }
  for (int l = threadIdx.x; l < d; l += blockDim.x) I.invlam[l] = exp(-th[1 + l]);
}

// the Matern tables of the problems that use them (kMtabMaxDoubles each, in
// problem p's slot: nu, and for an estimated nu also nu + h and nu - h):
// CTA (interval, p, table) of kMtabN threads takes the node values e^c M(c),
// e^c G(c) at the interval's Chebyshev points, then their Chebyshev
// coefficients ([16 of M, 16 of G] per interval)
__global__ void k_matern_tables(const sv_prob_desc* descs, const double* theta, int tstride,
                                double* tabs) {
  __shared__ double fm[kMtabN], fg[kMtabN];
  const sv_prob_desc& D = descs[blockIdx.y];
  const double nu0 = problem_nu(D, theta + (int64_t)blockIdx.y * tstride);
  if (!uses_matern_table(D, nu0)) return;
  const int z = blockIdx.z;  // 0: nu, 1: nu + h, 2: nu - h
  if (z > 0 && !D.estimate_nu) return;
  const double nu = z == 0 ? nu0 : z == 1 ? nu0 + kNuFdH : nu0 - kNuFdH;
  if ((int)blockIdx.x >= mtab_intervals(mtab_elo(nu))) return;
  double* tab = tabs + (size_t)blockIdx.y * kMtabSlotDoubles + (z == 0 ? 0 : z == 1 ? kMtabOffP : kMtabOffM);
  mtab_build_interval(nu, blockIdx.x, fm, fg, tab);
}

// the float32 tables of the split kernels (after the float64 tables in each
// problem's slot): CTA (interval, p) of kFtabN threads takes the node values
// F (the deficit D below 2^esw, e^c M above) and e^c G, for an estimated nu
// also those of dM/dnu, then their Chebyshev coefficients rounded to float32
// ([8 of F, 8 of Q] per interval; [8 of dM/dnu] per interval after them)
__global__ void k_matern_ftabs(const sv_prob_desc* descs, const double* theta, int tstride,
                               double* tabs) {
  __shared__ double ff[kFtabN], fq[kFtabN], fd[kFtabN];
  const sv_prob_desc& D = descs[blockIdx.y];
  const double nu = problem_nu(D, theta + (int64_t)blockIdx.y * tstride);
  if (!uses_matern_table(D, nu) || !(D.estimate_nu ? ftab_est_ok(nu, kNuFdH) : ftab_ok(nu))) return;
  const int elo = mtab_elo(nu), esw = ftab_switch(nu);
  const int iv = blockIdx.x, j = threadIdx.x;
  if (iv >= ftab_intervals(elo)) return;
  ftab_node(nu, elo, esw, iv, j, ff[j], fq[j]);
  if (D.estimate_nu) fd[j] = ftab_dnu_node(nu, kNuFdH, elo, esw, iv, j);
  __syncthreads();
  double* slot = tabs + (size_t)blockIdx.y * kMtabSlotDoubles;
  float* ft = (float*)(slot + kFtabOff);
  ft[(size_t)iv * 2 * kFtabN + j] = ftab_coef(ff, j);
  ft[(size_t)iv * 2 * kFtabN + kFtabN + j] = ftab_coef(fq, j);
  if (D.estimate_nu) ((float*)(slot + kDtabOff))[(size_t)iv * kFtabN + j] = ftab_coef(fd, j);
}

// the problem table of a one-problem evaluation, passed by value
__global__ void k_put_desc(sv_prob_desc pd, sv_prob_desc* out) { *out = pd; }

// info words of every problem: status 0, first failing block -1, jitter 0, aux 0
__global__ void k_info_init(int32_t* info, int nprob) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nprob; p += gridDim.x * blockDim.x) {
    info[4 * p + 0] = 0;
    info[4 * p + 1] = -1;
    info[4 * p + 2] = 0;
    info[4 * p + 3] = 0;
  }
}

// shared-memory footprint (doubles) of one team with block capacity kt
__host__ __device__ inline int64_t team_smem_doubles(int kt, int d, int NR, int need_grad,
                                                     int estimate_nu) {
  const int64_t tri = (int64_t)kt * (kt + 1) / 2;
  int64_t s = (int64_t)kt * d;  // u
  s += tri;                     // Lp
  if (need_grad) s += tri;      // Gp
  if (estimate_nu) s += tri;    // Dp
  s += (int64_t)NR * kt;        // R
  s += 3 * (int64_t)kt;         // a, invd, acc
  s += (kt + 1) / 2 + 1;        // idx (int32) + flag
  s += 40;                      // reduction scratch
  return s;
}

// dSigma_l a for l = 1..d (_covariance.py:142-146), one warp per block, lane i
// owning row i:  S_il = sum_{j != i} g_ij a_j (u_il - u_jl)^2.  Every unordered
// pair is visited once: in round r lane i takes the pair (i, i + r mod K),
// adds its own term and hands the squared differences to lane i + r by a
// shuffle, which adds g_ij a_i times them (rounds 1 .. K/2; for even K the
// pairs of round K/2 are met from both ends, each lane adding its own term).
// Half the float64 work of a pass per (row, coordinate) over all partners;
// the sums are those of the same terms in another (fixed) order.
template <int DR, int T>
__device__ __forceinline__ void dsig_pairs_warp(int K, int d, const double* u, const double* Gp,
                                                const double* a, double* R, int ldr, int lane) {
  // T = 32: the whole warp, K <= 32; T = 16: one half of the warp, K <= 16
  // (shuffles within the half)
  const unsigned full = Team<T>::mask();
  const bool own = lane < K;
  double ui[DR], S[DR];
#pragma unroll
  for (int l = 0; l < DR; ++l) {
    ui[l] = (own && l < d) ? u[lane * d + l] : 0.0;
    S[l] = 0.0;
  }
  auto g = [&](int i, int j) { return i >= j ? Gp[tri_off(i, j)] : Gp[tri_off(j, i)]; };
  for (int r = 1; r <= K / 2; ++r) {
    int j = lane + r;
    if (j >= K) j -= K;
    int src = lane - r;
    if (src < 0) src += K;
    const bool both = !((K & 1) == 0 && r == K / 2);
    double cij = 0.0, cji = 0.0;
    if (own) {
      cij = g(lane, j) * a[j];
      cji = g(lane, src) * a[src];
    }
    double sq[DR];
#pragma unroll
    for (int l = 0; l < DR; ++l) {
      sq[l] = 0.0;
      if (own && l < d) {
        const double df = ui[l] - u[j * d + l];
        sq[l] = df * df;
        S[l] = fma(cij, sq[l], S[l]);
      }
    }
    if (both) {
#pragma unroll
      for (int l = 0; l < DR; ++l)
        if (l < d) {
          const double rv = __shfl_sync(full, sq[l], src & (T - 1), T);
          if (own) S[l] = fma(cji, rv, S[l]);
        }
    }
  }
#pragma unroll
  for (int l = 0; l < DR; ++l)
    if (own && l < d) R[(1 + l) * ldr + lane] = S[l];
}

// One block, processed by a team (float64 throughout).  Writes the block's record.
// kt is the block capacity of the team's slot (its shared-memory layout).
template <int T>
__device__ void block_pass1(const LikArgs& A, int64_t b, double* sm, int kt) {
  const int lane = Team<T>::lane();
  const int p = block_problem(A, b);
  const ProbInfo& PI = A.probs[p];
  const int d = PI.d, q = PI.q, P = PI.P, NR = A.need_grad ? (P + 1 + q) : 0;
  const int dmax = A.dmax;
  const int k = A.kb[b];
  const int K = k + 1;
  const int64_t tri = (int64_t)kt * (kt + 1) / 2;
  double* u = sm;
  double* Lp = u + (int64_t)kt * dmax;
  double* Gp = A.need_grad ? Lp + tri : nullptr;
  double* Dp = (A.any_estimate_nu && PI.estimate_nu) ? (Lp + tri * (A.need_grad ? 2 : 1)) : nullptr;
  double* R = Lp + tri * (1 + (A.need_grad ? 1 : 0) + (A.any_estimate_nu ? 1 : 0));
  double* a = R + (int64_t)A.NRmax * kt;
  double* invd = a + kt;
  double* acc = invd + kt;
  int* idx = (int*)(acc + kt);
  volatile int* flag = idx + kt;
  double* red = (double*)(acc + kt + (kt + 1) / 2 + 1);
  const double* X = A.X + PI.x_off;
  const double* Y = A.y + PI.y_off;
  const double* Zm = A.Z + PI.z_off;
  int32_t* info = A.info + 4 * p;

  // ---- gather: neighbours first, self last (likelihood.py:113)
  for (int i = lane; i < K; i += T) idx[i] = (i < k) ? A.nbr[b * A.ldnbr + i] : A.rowb[b];
  Team<T>::sync();
  for (int t = lane; t < K * d; t += T) {
    const int i = t / d, l = t - (t / d) * d;
    u[i * d + l] = X[(int64_t)idx[i] * d + l] * PI.invlam[l];
  }
  Team<T>::sync();

  // ---- Sigma, Cholesky, jitter retry (_covariance.py:235-252)
  const double s2 = PI.s2, tau = PI.tau;
  int lv = 0;
  if (A.fixup) {
    lv = chunk_level(A, b);
  } else if (A.redo_mode) {
    lv = A.level[b];
  }
  bool ok = false;
  for (; lv <= 9; ++lv) {
    // scale = mean(diag Sigma): every diagonal entry is s2 * (1 + tau)
    double jit = 0.0;
    if (lv > 0) {
      double sc = 0.0;
      for (int i = 0; i < K; ++i) sc += s2 * (1.0 + tau);
      sc /= (double)K;
      jit = jitter_pow10(lv) * sc;
    }
    if (lane == 0) *flag = 0;
    assemble_sigma<T>(K, d, u, nullptr, s2, tau, jit, PI.mm, Lp, Gp, Dp);
    Team<T>::sync();
    // LDL^T (one three-FMA reciprocal per pivot on one lane, where a
    // Cholesky pivot takes a square root and a division); the Cholesky
    // factor is L D^(1/2), with the same failure criterion (dpotrf: a pivot
    // that is not > 0)
    ok = ldlt_packed<T>(K, Lp, invd, acc, flag);
    Team<T>::sync();
    if (ok) break;
  }
  double* rec = A.cache + b * (int64_t)A.CS;
  if (!ok) {
    if (lane == 0) {
      set_error(info + SV_INFO_STATUS, SV_ECHOL);
      atomicCAS(info + SV_INFO_BLOCK, -1, (int)(b - PI.blk_off));
    }
    if (lane == 0) A.level[b] = 10;
    for (int f = lane; f < A.CS; f += T) rec[f] = 0.0;
    return;
  }
  if (lane == 0) {
    A.level[b] = (int8_t)lv;
    if (lv > 0) {
      atomicMax(info + SV_INFO_JITTER, lv);
      A.flags[0] = 1;
    }
  }
  double jit_used = 0.0;
  if (lv > 0) {
    double sc = 0.0;
    for (int i = 0; i < K; ++i) sc += s2 * (1.0 + tau);
    jit_used = jitter_pow10(lv) * (sc / (double)K);
  }

  // ---- a = C^-T e_K = L^-T e_K / sqrt(d_K)  (likelihood.py:125-127);
  //      L_KK = sqrt(d_K)
  backsolve_unit_eK<T>(K, Lp, a, acc);
  const double lKK = sqrt(Lp[tri_off(K - 1, K - 1)]);
  const double sK = sqrt(invd[K - 1]);
  for (int i = lane; i < K; i += T) a[i] *= sK;
  Team<T>::sync();

  // ---- GLS parts a.y, a.Z (likelihood.py:129-134)
  {
    double vy = 0.0;
    for (int i = lane; i < K; i += T) vy += a[i] * Y[idx[i]];
    vy = team_sum<T>(vy, red);
    if (lane == 0) {
      rec[0] = lKK;  // L_KK; the log is taken in the reduction
      rec[1] = vy;
    }
    for (int c = 0; c < q; ++c) {
      double vz = 0.0;
      for (int i = lane; i < K; i += T) vz += a[i] * Zm[(int64_t)idx[i] * q + c];
      vz = team_sum<T>(vz, red);
      if (lane == 0) rec[2 + c] = vz;
    }
  }
  if (!A.need_grad) {
    Team<T>::sync();
    if (lane == 0) {
      rec[2 + q] = rec[1];
      for (int c = 0; c < q; ++c) rec[3 + q + c] = rec[2 + c];
    }
    return;
  }

  // ---- right-hand sides dSigma_p a (likelihood.py:138), then y and Z
  // R columns: p = 0..P-1 (dSigma rows), P: y, P+1..P+q: Z
  const int ldr = kt;
  // p = 0: dSigma_0 = Sigma (un-jittered) = C C^T - jit I, so Sigma a = L_KK e_K - jit a
  for (int i = lane; i < K; i += T) R[i] = ((i == K - 1) ? lKK : 0.0) - jit_used * a[i];
  // p = 1..d: (dSigma_l a)_i = sum_j G_ij (u_il - u_jl)^2 a_j   (_covariance.py:142-146)
  bool dsig_done = false;
  if constexpr (T == 32 || T == 16) {
    if (K <= T && d <= 12) {
      if (d <= 4)
        dsig_pairs_warp<4, T>(K, d, u, Gp, a, R, ldr, lane);
      else if (d <= 8)
        dsig_pairs_warp<8, T>(K, d, u, Gp, a, R, ldr, lane);
      else
        dsig_pairs_warp<12, T>(K, d, u, Gp, a, R, ldr, lane);
      dsig_done = true;
    }
  }
  if (!dsig_done)
  for (int t = lane; t < K * d; t += T) {
    const int i = t / d, l = t - (t / d) * d;
    const double uil = u[i * d + l];
    double s = 0.0;
    for (int j = 0; j < K; ++j) {
      const double df = uil - u[j * d + l];
      const double g = (i >= j) ? Gp[tri_off(i, j)] : Gp[tri_off(j, i)];
      s += g * (df * df) * a[j];
    }
    R[(1 + l) * ldr + i] = s;
  }
  int pr = 1 + d;
  if (PI.estimate_nu) {
    for (int i = lane; i < K; i += T) {
      double s = 0.0;
      for (int j = 0; j < K; ++j) s += ((i >= j) ? Dp[tri_off(i, j)] : Dp[tri_off(j, i)]) * a[j];
      R[pr * ldr + i] = s;
    }
    ++pr;
  }
  // nugget row: dSigma_tau = s2 * tau * I
  for (int i = lane; i < K; i += T) R[pr * ldr + i] = s2 * tau * a[i];
  for (int i = lane; i < K; i += T) {
    R[P * ldr + i] = Y[idx[i]];
    for (int c = 0; c < q; ++c) R[(P + 1 + c) * ldr + i] = Zm[(int64_t)idx[i] * q + c];
  }
  Team<T>::sync();

  // ---- W = C^-1 [dSigma a], z parts = C^-1 [y, Z]  (likelihood.py:139, 154):
  //      unit forward solves, then row i times d_i^(-1/2)
  forward_solve_unit_multi<T>(K, Lp, R, NR, ldr);
  for (int i = lane; i < K; i += T) invd[i] = sqrt(invd[i]);
  Team<T>::sync();
  for (int t = lane; t < K * NR; t += T) {
    const int c = t / K, i = t - c * K;
    R[c * ldr + i] *= invd[i];
  }
  Team<T>::sync();

  // ---- record: zK parts, wK, W.zy, W.zZ, Fisher (likelihood.py:140-142)
  double* wK = rec + 3 + 2 * q;
  double* wzy = wK + P;
  double* wzZ = wzy + P;
  double* F = wzZ + P * q;
  for (int c = lane; c < 1 + q; c += T) rec[2 + q + c] = R[(P + c) * ldr + K - 1];
  for (int pp = lane; pp < P; pp += T) wK[pp] = R[pp * ldr + K - 1];
  // Gram entries among the first P columns (Fisher) and with the y/Z columns
  const int nf = P * (P + 1) / 2;
  const int ntot = nf + P * (1 + q);
  for (int t = lane; t < ntot; t += T) {
    int c1, c2;
    if (t < nf) {
      int i2, j2;
      tri_index(t, i2, j2);  // i2 >= j2
      c1 = i2;
      c2 = j2;
    } else {
      const int s = t - nf;
      c1 = s / (1 + q);
      c2 = P + (s - c1 * (1 + q));
    }
    const double* r1 = R + c1 * ldr;
    const double* r2 = R + c2 * ldr;
    double s = 0.0;
    for (int i = 0; i < K; ++i) s += r1[i] * r2[i];
    if (t < nf) {
      // fish += 0.5 (2 W W^T - wK wK^T)
      F[t] = 0.5 * (2.0 * s - r1[K - 1] * r2[K - 1]);
    } else {
      const int s3 = t - nf;
      const int pp = s3 / (1 + q);
      const int cc = s3 - pp * (1 + q);
      if (cc == 0)
        wzy[pp] = s;
      else
        wzZ[pp * q + (cc - 1)] = s;
    }
  }
}

// which blocks a launch of the block kernels processes
__device__ __forceinline__ bool block_selected(const LikArgs& A, int64_t b, int kcap) {
  if (A.redo_mode) return A.redo[b] != 0;
  if (A.fixup) return chunk_level(A, b) > A.level[b];
  return A.kb[b] + 1 <= kcap;
}

// Blocks of 17 to 32 points, one per warp (blocks of up to 16 points are
// k_block_half's).
__global__ void k_block_warp(LikArgs A) {
  extern __shared__ double smem[];
  if (!pass_has_work(A)) return;
  const int64_t per_team = team_smem_doubles(32, A.dmax, A.NRmax, A.need_grad, A.any_estimate_nu);
  const int w = threadIdx.x >> 5;
  double* sm = smem + w * per_team;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t = A.b0 + (int64_t)blockIdx.x * (blockDim.x >> 5) + w; t < A.b1; t += nw) {
    const int64_t b = launch_block(A, t);
    if (A.probs[block_problem(A, b)].skip) continue;
    if (!block_selected(A, b, 32)) {
      if (!A.redo_mode && !A.fixup && (threadIdx.x & 31) == 0)
        set_error(A.info + 4 * block_problem(A, b) + SV_INFO_STATUS, SV_EINVAL);
      continue;
    }
    if (A.kb[b] + 1 <= 16) continue;
    block_pass1<32>(A, b, sm, 32);
    __syncwarp();
  }
}

// Blocks of up to 16 points, two per warp: each half of the warp takes its
// own list entry (16-lane teams with slots of capacity 16, their own control
// flow).  A block's arithmetic does not depend on the team width (every
// step's per-element order is fixed by the block), so the results are those
// of a whole warp on the block.
__global__ void k_block_half(LikArgs A) {
  extern __shared__ double smem[];
  if (!pass_has_work(A)) return;
  const int64_t per_half = team_smem_doubles(16, A.dmax, A.NRmax, A.need_grad, A.any_estimate_nu);
  const int h = threadIdx.x >> 4;  // half-warp index in the CTA
  double* sm = smem + h * per_half;
  const int64_t nh = (int64_t)gridDim.x * (blockDim.x >> 4);
  for (int64_t t = A.b0 + (int64_t)blockIdx.x * (blockDim.x >> 4) + h; t < A.b1; t += nh) {
    const int64_t b = launch_block(A, t);
    if (A.probs[block_problem(A, b)].skip) continue;
    // larger blocks are k_block_warp's (which reports sizes beyond 32); the
    // fix-up and re-evaluation passes select by chunk and flag, not by size
    if (A.kb[b] + 1 > 16 || !block_selected(A, b, 16)) continue;
    block_pass1<16>(A, b, sm, 16);
    __syncwarp(Team<16>::mask());
  }
}

__global__ void k_block_cta(LikArgs A) {
  extern __shared__ double smem[];
  if (!pass_has_work(A)) return;
  for (int64_t t = A.b0 + blockIdx.x; t < A.b1; t += gridDim.x) {
    const int64_t b = launch_block(A, t);
    if (A.probs[block_problem(A, b)].skip) continue;
    if (!block_selected(A, b, A.kt)) {
      if (!A.redo_mode && !A.fixup && threadIdx.x == 0)
        set_error(A.info + 4 * block_problem(A, b) + SV_INFO_STATUS, SV_EINVAL);
      continue;
    }
    block_pass1<128>(A, b, smem, A.kt);
    __syncthreads();
  }
}

// chunk-wide jitter: chunk_max[c] = max level over the chunk's blocks.  A
// chunk id outside [0, nblk) is the caller's error: it is skipped and its
// problem's status set to SV_EINVAL (chunk ids are read only when some block
// needed jitter)
__global__ void k_chunk_max(const int32_t* flags, const int32_t* chunk, const int8_t* level,
                            int64_t nblk, int64_t bb0, int64_t bb1, int32_t* chunk_max,
                            const int32_t* bprob, int32_t* info) {
  if (flags[0] == 0) return;
  for (int64_t b = bb0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < bb1;
       b += (int64_t)gridDim.x * blockDim.x) {
    const int c = chunk[b];
    if (c < 0 || c >= nblk) {
      set_error(info + 4 * (bprob ? bprob[b] : 0) + SV_INFO_STATUS, SV_EINVAL);
      continue;
    }
    const int lv = level[b];
    if (lv > 0 && lv <= 9) atomicMax(chunk_max + c, lv);
  }
}

// flags[0] = 1 when any chunk of the (exchanged) chunk table needs jitter:
// the fix-up pass of a shard must run when another shard's block raised the
// level of a chunk this shard shares
__global__ void k_any_jitter(const int32_t* chunk_max, int64_t nchunk, int32_t* flags) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nchunk;
       c += (int64_t)gridDim.x * blockDim.x)
    if (chunk_max[c] > 0) flags[0] = 1;
}

// ---------------------------------------------------------------------------
// reductions (grid row = problem, R.parts partitions of its blocks)
// ---------------------------------------------------------------------------
struct RedArgs {
  const double* cache;
  const ProbInfo* probs;
  int CS, need_grad, nfmax, qmax, Pmax;
  int parts;      // partitions of every problem's blocks
  int pbeg;       // the partitions this launch reduces: pbeg + blockIdx.x (< parts)
  double* part1;  // [nprob][parts][nfmax]
  double* part2;  // [nprob][parts][Pmax + 1]
  double* beta;   // [nprob][qmax + 1]
  double* sums;   // [nprob][nfmax]
  const double* theta;
  int tstride;
  double* out;
  int ostride;
};

// pass-1 fields of a problem: logdet, Zty[q], XtX[q*q], F[P(P+1)/2]
__host__ __device__ inline int nfield1(int q, int P, int need_grad) {
  return 1 + q + q * q + (need_grad ? P * (P + 1) / 2 : 0);
}

// Pass-1 sums of one partition: warp w takes the partition's blocks
// w, w + nwarp, ..., its lanes the fields; each (warp, field) accumulator in
// shared memory has one owner, and the warps' rows are added in a fixed order.
// partitions of a problem's blocks: a function of its own block count only,
// so a problem's sums are the same alone and in any batch
__host__ __device__ inline int red_parts_n(int64_t nblk) {
  int64_t parts = (nblk + 1023) / 1024;
  if (parts < 8) parts = 8;
  if (parts > 4096) parts = 4096;
  return (int)parts;
}

__global__ void k_reduce1(RedArgs R) {
  extern __shared__ double racc[];  // [nwarp][nfmax]
  const int p = blockIdx.y;
  const ProbInfo& PI = R.probs[p];
  if (PI.skip) return;
  const int q = PI.q, P = PI.P;
  const int nf = nfield1(q, P, R.need_grad);
  const int nwarp = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int parts = red_parts_n(PI.nblk);
  const int part = R.pbeg + (int)blockIdx.x;
  if (part >= parts) return;
  const int64_t per = (PI.nblk + parts - 1) / parts;
  const int64_t b0 = PI.blk_off + part * per;
  const int64_t b1 = min(PI.blk_off + PI.nblk, b0 + per);
  double* acc = racc + (int64_t)w * R.nfmax;
  const int foff = 3 + 2 * q + P * (2 + q);
  // the (warp, field) sums, one owner lane each: fields lane + 32 r < 128 in
  // registers a[r], the rest (large d) in shared memory
  constexpr int kFr = 4;
  double a[kFr];
#pragma unroll
  for (int r = 0; r < kFr; ++r) a[r] = 0.0;
  for (int f = lane + 32 * kFr; f < nf; f += 32) acc[f] = 0.0;
  auto field = [&](const double* c, int f, double lgj) -> double {
    if (f == 0) return lgj;
    if (f < 1 + q) return c[2 + (f - 1)] * c[1];
    if (f < 1 + q + q * q) {
      const int e = f - 1 - q;
      const int i = e / q, jj = e - (e / q) * q;
      return c[2 + i] * c[2 + jj];
    }
    return c[foff + (f - 1 - q - q * q)];
  };
  for (int64_t base = b0 + w; base < b1; base += 32 * (int64_t)nwarp) {
    // log L_KK of the warp's next 32 blocks, one per lane (a float64 warp
    // instruction costs the same with one lane as with 32)
    const int64_t bl = base + (int64_t)lane * nwarp;
    const double lg = bl < b1 ? log(R.cache[bl * R.CS]) : 0.0;
    const int nj = (int)min((int64_t)32, (b1 - base + nwarp - 1) / nwarp);
    // kRb blocks' register fields are loaded before they are added (in
    // block order, so the sums are those of one block at a time)
    constexpr int kRb = 4;
    for (int j0 = 0; j0 < nj; j0 += kRb) {
      double v[kRb][kFr];
#pragma unroll
      for (int u = 0; u < kRb; ++u) {
        const int j = j0 + u < nj ? j0 + u : nj - 1;
        const double lgj = __shfl_sync(0xffffffffu, lg, j);
        const double* c = R.cache + (base + (int64_t)j * nwarp) * R.CS;
#pragma unroll
        for (int r = 0; r < kFr; ++r) {
          const int f = lane + 32 * r;
          v[u][r] = f < nf ? field(c, f, lgj) : 0.0;
        }
      }
#pragma unroll
      for (int u = 0; u < kRb; ++u) {
        if (j0 + u >= nj) break;
#pragma unroll
        for (int r = 0; r < kFr; ++r)
          if (lane + 32 * r < nf) a[r] += v[u][r];
        const int j = j0 + u;
        const double lgj = __shfl_sync(0xffffffffu, lg, j);
        const double* c = R.cache + (base + (int64_t)j * nwarp) * R.CS;
        for (int f = lane + 32 * kFr; f < nf; f += 32) acc[f] += field(c, f, lgj);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < kFr; ++r)
    if (lane + 32 * r < nf) acc[lane + 32 * r] = a[r];
  __syncthreads();
  double* partv = R.part1 + ((int64_t)p * R.parts + part) * R.nfmax;
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nwarp; ++k) s += racc[(int64_t)k * R.nfmax + f];
    partv[f] = s;
  }
}

__global__ void k_final1(RedArgs R) {
  const int p = blockIdx.x;
  const ProbInfo& PI = R.probs[p];
  if (PI.skip) return;
  const int q = PI.q, P = PI.P;
  const int nf = nfield1(q, P, R.need_grad);
  double* sums = R.sums + (int64_t)p * R.nfmax;
  const int parts = red_parts_n(PI.nblk);
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    double s = 0.0;
    const double* src = R.part1 + (int64_t)p * R.parts * R.nfmax + f;
#pragma unroll 8
    for (int c = 0; c < parts; ++c) s += src[(int64_t)c * R.nfmax];
    sums[f] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // beta = solve(XtX + 1e-12 I, Zty): Gaussian elimination, partial pivoting
    double* beta = R.beta + (int64_t)p * (R.qmax + 1);
    double M[kMaxQ][kMaxQ + 1];
    for (int i = 0; i < q; ++i) {
      for (int j = 0; j < q; ++j) M[i][j] = sums[1 + q + i * q + j] + (i == j ? 1e-12 : 0.0);
      M[i][q] = sums[1 + i];
    }
    for (int c = 0; c < q; ++c) {
      int piv = c;
      for (int r = c + 1; r < q; ++r)
        if (fabs(M[r][c]) > fabs(M[piv][c])) piv = r;
      if (piv != c)
        for (int j = 0; j <= q; ++j) {
          const double t = M[c][j];
          M[c][j] = M[piv][j];
          M[piv][j] = t;
        }
      for (int r = c + 1; r < q; ++r) {
        const double f = M[r][c] / M[c][c];
        for (int j = c; j <= q; ++j) M[r][j] -= f * M[c][j];
      }
    }
    for (int c = q - 1; c >= 0; --c) {
      double s = M[c][q];
      for (int j = c + 1; j < q; ++j) s -= M[c][j] * beta[j];
      beta[c] = s / M[c][c];
    }
  }
}

__global__ void k_reduce2(RedArgs R) {
  __shared__ double sbeta[kMaxQ];
  __shared__ double red[kRedThreads / 32][kMaxP + 1];
  const int p = blockIdx.y;
  const ProbInfo& PI = R.probs[p];
  if (PI.skip) return;
  const int q = PI.q, P = PI.P, np = R.need_grad ? P : 0;
  for (int i = threadIdx.x; i < q; i += blockDim.x) sbeta[i] = R.beta[(int64_t)p * (R.qmax + 1) + i];
  __syncthreads();
  const int parts = red_parts_n(PI.nblk);
  const int part = R.pbeg + (int)blockIdx.x;
  if (part >= parts) return;
  const int64_t per = (PI.nblk + parts - 1) / parts;
  const int64_t b0 = PI.blk_off + part * per;
  const int64_t b1 = min(PI.blk_off + PI.nblk, b0 + per);
  double acc[kMaxP + 1];
  for (int i = 0; i <= np; ++i) acc[i] = 0.0;
  for (int64_t b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
    const double* c = R.cache + b * R.CS;
    double zK = c[2 + q];
    for (int i = 0; i < q; ++i) zK -= c[3 + q + i] * sbeta[i];
    acc[0] -= 0.5 * (2.0 * log(c[0]) + zK * zK);
    if (R.need_grad) {
      const double* wK = c + 3 + 2 * q;
      const double* wzy = wK + P;
      const double* wzZ = wzy + P;
      for (int pp = 0; pp < P; ++pp) {
        double wz = wzy[pp];
        for (int i = 0; i < q; ++i) wz -= wzZ[pp * q + i] * sbeta[i];
        acc[1 + pp] -= 0.5 * (wK[pp] * (1.0 + zK * zK) - 2.0 * zK * wz);
      }
    }
  }
  // fixed-order block reduction
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  for (int i = 0; i <= np; ++i) {
    double v = acc[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (ln == 0) red[w][i] = v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= np; i += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k][i];
    R.part2[((int64_t)p * R.parts + part) * (R.Pmax + 1) + i] = s;
  }
}

__global__ void k_final2(RedArgs R) {
  const int p = blockIdx.x;
  const ProbInfo& PI = R.probs[p];
  if (PI.skip) return;
  const int P = PI.P, q = PI.q, np = R.need_grad ? P : 0;
  __shared__ double tot[kMaxP + 1];
  const int parts = red_parts_n(PI.nblk);
  for (int i = threadIdx.x; i <= np; i += blockDim.x) {
    double s = 0.0;
    const double* src = R.part2 + (int64_t)p * R.parts * (R.Pmax + 1) + i;
#pragma unroll 8
    for (int c = 0; c < parts; ++c) s += src[(int64_t)c * (R.Pmax + 1)];
    tot[i] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double* out = R.out + (int64_t)p * R.ostride;
    const double* sums = R.sums + (int64_t)p * R.nfmax;
    const double* th = R.theta + (int64_t)p * R.tstride;
    // ll = -n/2 log(2pi) - sum_b (log L_KK + z_K^2 / 2)  (likelihood.py:149-156)
    double ll = -0.5 * (double)PI.n * 1.8378770664093453 + tot[0];
    double g0 = np ? tot[1] : 0.0;
    double f00_add = 0.0;
    if (PI.var_penalty > 0.0) {  // likelihood.py:165-171
      double excess = th[0] - PI.log_var_target;
      if (excess < 0.0) excess = 0.0;
      ll -= 0.5 * PI.var_penalty * excess * excess;
      g0 -= PI.var_penalty * excess;
      if (excess > 0.0) f00_add = PI.var_penalty;
    }
    out[0] = ll;
    if (np) {
      out[1] = g0;
      for (int pp = 1; pp < P; ++pp) out[1 + pp] = tot[1 + pp];
      // Fisher: sums hold the packed lower triangle
      double* fish = out + 1 + P;
      const int foff = 1 + q + q * q;
      for (int i = 0; i < P; ++i)
        for (int j = 0; j <= i; ++j) {
          const double v = sums[foff + i * (i + 1) / 2 + j];
          fish[i * P + j] = v;
          fish[j * P + i] = v;
        }
      fish[0] += f00_add;
    } else {
      for (int i = 0; i < P + P * P; ++i) out[1 + i] = 0.0;
    }
    double* bo = out + 1 + P + P * P;
    for (int i = 0; i < q; ++i) bo[i] = R.beta[(int64_t)p * (R.qmax + 1) + i];
  }
}

}  // namespace sv

// ---------------------------------------------------------------------------
// evaluation driver shared by the single-problem and batched entry points
// ---------------------------------------------------------------------------
using namespace sv;

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

namespace {

struct EvalShape {
  int64_t nprob, nblk, nx, nblk_max;
  int dmax, qmax, Pmax, kmax, need_grad, any_est, precision;
  int tabs;  // a Matern table per problem (problems of fixed general nu fill theirs)
};

// reduction grid rows: the partitions of the largest problem
int red_parts(const EvalShape& S) { return red_parts_n(S.nblk_max); }

struct WsLayout {
  size_t desc, probs, cache, level, redo, chunk_max, flags, part1, part2, beta, sums, xhl, mtab, total;
  int CS, nfmax;
};

WsLayout ws_layout(const EvalShape& S) {
  WsLayout L;
  const int P = S.Pmax, q = S.qmax;
  L.CS = record_stride(q, P, S.need_grad);
  L.nfmax = nfield1(q, P, S.need_grad);
  const size_t nb = (size_t)(S.nblk > 0 ? S.nblk : 1);
  size_t off = 0;
  L.desc = off;
  off = align256(off + sizeof(sv_prob_desc));
  L.probs = off;
  off = align256(off + sizeof(ProbInfo) * (size_t)S.nprob);
  L.cache = off;
  off = align256(off + sizeof(double) * (size_t)L.CS * nb);
  L.level = off;
  off = align256(off + nb);
  L.redo = off;
  off = align256(off + nb);
  L.chunk_max = off;
  off = align256(off + sizeof(int32_t) * nb);
  L.flags = off;
  off = align256(off + 4 * sizeof(int32_t));
  L.part1 = off;
  off = align256(off + sizeof(double) * (size_t)S.nprob * red_parts(S) * L.nfmax);
  L.part2 = off;
  off = align256(off + sizeof(double) * (size_t)S.nprob * red_parts(S) * (P + 1));
  L.beta = off;
  off = align256(off + sizeof(double) * (size_t)S.nprob * (q + 1));
  L.sums = off;
  off = align256(off + sizeof(double) * (size_t)S.nprob * L.nfmax);
  L.xhl = off;
  if (S.precision == 1 || S.precision == 2) off = align256(off + sizeof(float) * 2 * (size_t)S.nx);
  L.mtab = off;
  if (S.tabs) off = align256(off + sizeof(double) * (size_t)kMtabSlotDoubles * (size_t)S.nprob);
  L.total = off;
  return L;
}

// opt-in shared memory per block of the current device, read once per
// device (devices may differ; calls may come from several host threads)
constexpr int kMaxDevices = 64;
std::atomic<int> g_max_smem_optin[kMaxDevices];
int max_smem_optin() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
  }
  int v = g_max_smem_optin[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    g_max_smem_optin[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

struct EvalCall {
  EvalShape S;
  const sv_prob_desc* probs;  // device
  const double* theta;        // device, nprob x tstride
  int tstride;
  const double *X, *y, *Z;
  const int32_t *rowb, *kb, *nbr, *chunk, *bprob, *wlist, *clist;
  int64_t nwarp, ncta;  // list lengths (lists nullptr: ranges [0,nwarp), [nwarp,nwarp+ncta))
  int ldnbr, chunked, team_lanes;
  double rho_min;
  double* out;
  int ostride;
  int32_t* info;
  char* ws;
};

// launch of a block kernel whose CTAs are teams of `tw` threads: as many
// teams per CTA as shared memory and the kernel's registers allow (the
// float64 pipe needs every resident warp it can get to cover its latency),
// a persistent grid of the CTAs that fit on the SMs at once
template <typename Kern>
int launch_team_kernel(Kern kern, LikArgs A, int kt, int tw, int max_teams, cudaStream_t st) {
  const int nsm = sv_num_sms();
  const size_t team = sizeof(double) * team_smem_doubles(kt, A.dmax, A.NRmax, A.need_grad, A.any_estimate_nu);
  cudaFuncAttributes fa;
  SV_CUDA_TRY(cudaFuncGetAttributes(&fa, kern));
  int tpc = max_teams;
  while (tpc > 1 && (tpc * team > (size_t)max_smem_optin() || tpc * tw > fa.maxThreadsPerBlock)) --tpc;
  const size_t smem = tpc * team;
  if (smem > (size_t)max_smem_optin()) return SV_EINVAL;
  SV_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tw * tpc, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  int64_t grid = (A.b1 - A.b0 + tpc - 1) / tpc;
  if (grid > (int64_t)per_sm * nsm) grid = (int64_t)per_sm * nsm;
  if (grid < 1) grid = 1;
  kern<<<(int)grid, tw * tpc, smem, st>>>(A);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

int launch_warp_kernel(LikArgs A, cudaStream_t st) {
  int rc = launch_team_kernel(k_block_half, A, 16, 16, 32, st);
  if (rc != SV_OK) return rc;
  return launch_team_kernel(k_block_warp, A, 32, 32, 16, st);
}

int launch_cta_kernel(LikArgs A, cudaStream_t st) {
  const int nsm = sv_num_sms();
  const size_t smem = sizeof(double) * team_smem_doubles(A.kt, A.dmax, A.NRmax, A.need_grad, A.any_estimate_nu);
  if (smem > (size_t)max_smem_optin()) return SV_EINVAL;
  SV_CUDA_TRY(cudaFuncSetAttribute(k_block_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = A.b1 - A.b0;
  if (grid > 8LL * nsm) grid = 8LL * nsm;
  if (grid < 1) grid = 1;
  k_block_cta<<<(int)grid, 128, smem, st>>>(A);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

// One stage of a sharded one-problem evaluation (sv_vecchia_loglik_stage):
// the shard is reduction partitions [pb, pe); the exchanged tables live in
// caller buffers.
struct ShardStage {
  int stage;           // 1 .. 4
  int pb, pe;          // the shard's partitions
  int32_t* chunk_max;  // [nblk] chunk levels (stage 1 writes the shard's, stage 2 reads all)
  double* part1;       // [parts][nfield1]
  double* part2;       // [parts][P + 1]
};

// Enqueues one evaluation (sh == nullptr), or one stage of a sharded one.
// Only kernels and memsets: capturable in a graph.
int run_eval(const EvalCall& C, cudaStream_t st, const ShardStage* sh = nullptr) {
  const EvalShape& S = C.S;
  WsLayout W = ws_layout(S);
  char* ws = C.ws;
  ProbInfo* probs = (ProbInfo*)(ws + W.probs);
  const int stage = sh ? sh->stage : 0;  // 0: the whole evaluation

  LikArgs A;
  A.X = C.X;
  A.y = C.y;
  A.Z = C.Z;
  A.rowb = C.rowb;
  A.kb = C.kb;
  A.nbr = C.nbr;
  A.chunk = C.chunk;
  A.bprob = C.bprob;
  A.list = nullptr;
  A.probs = probs;
  A.cache = (double*)(ws + W.cache);
  A.level = (int8_t*)(ws + W.level);
  A.redo = (int8_t*)(ws + W.redo);
  A.chunk_max = sh ? sh->chunk_max : (int32_t*)(ws + W.chunk_max);
  A.flags = (int32_t*)(ws + W.flags);
  A.info = C.info;
  A.b0 = 0;
  A.b1 = 0;
  A.nprob = (int)S.nprob;
  A.ldnbr = C.ldnbr;
  A.CS = W.CS;
  A.kt = 32;
  A.dmax = S.dmax;
  A.NRmax = S.need_grad ? (S.Pmax + 1 + S.qmax) : 0;
  A.need_grad = S.need_grad;
  A.any_estimate_nu = S.any_est;
  A.fixup = 0;
  A.nchunk = S.nblk;
  A.redo_mode = 0;
  A.rho_min = C.rho_min > 0.0 ? C.rho_min : 1e-4;
  A.xhl = (float2*)(ws + W.xhl);
  A.kcap = S.kmax + 1 < 32 ? (S.kmax + 1 > 0 ? S.kmax + 1 : 1) : 32;

  // the blocks of this call: all, or those of the shard's partitions
  const int parts = red_parts(S);
  int64_t blo = 0, bhi = S.nblk;
  if (sh) {
    const int64_t per = (S.nblk + parts - 1) / parts;
    blo = std::min<int64_t>((int64_t)sh->pb * per, S.nblk);
    bhi = std::min<int64_t>((int64_t)sh->pe * per, S.nblk);
  }

  // split forms (1: float64 factorisation, 2: double-float factorisation):
  // at most 32 right-hand sides (P + 1 + q); anything else runs the float64
  // kernels.  The blocks of a problem whose nu (fixed, or estimated at this
  // theta) has neither a closed form nor the float32 tables go from the
  // split kernels to the float64 pass
  const bool split = (S.precision == 1 || S.precision == 2) && A.NRmax <= 32;
  // 16 lanes per block is the fastest team width measured for every K from 6
  // to 31 (d = 3 and 10); 8 and 32 trail by up to 37 % and 12 %
  const int lanes = C.team_lanes > 0 ? C.team_lanes : 16;
  if (split && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32) return SV_EINVAL;

  // list ranges: the warp-kernel blocks are [0, nwarp) (or wlist), the CTA
  // blocks the rest; a shard (one problem, no lists) takes its part of each
  auto warp_pass = [&](LikArgs B) -> int {
    B.kt = 32;
    B.list = C.wlist;
    B.b0 = sh ? std::min<int64_t>(blo, C.nwarp) : 0;
    B.b1 = sh ? std::min<int64_t>(bhi, C.nwarp) : C.nwarp;
    if (B.b1 <= B.b0) return SV_OK;
    if (split && !B.redo_mode)
      return S.precision == 1 ? launch_block_split(B, lanes, st) : launch_block_split_df(B, lanes, st);
    return launch_warp_kernel(B, st);
  };
  auto cta_pass = [&](LikArgs B) -> int {
    B.kt = S.kmax + 1;
    B.list = C.clist;
    B.b0 = C.clist ? 0 : C.nwarp;
    B.b1 = C.clist ? C.ncta : C.nwarp + C.ncta;
    if (sh) {
      B.b0 = std::max<int64_t>(blo, C.nwarp);
      B.b1 = std::min<int64_t>(bhi, C.nwarp + C.ncta);
    }
    if (B.b1 <= B.b0) return SV_OK;
    return launch_cta_kernel(B, st);
  };

  int rc;
  if (stage == 0 || stage == 1) {
    k_info_init<<<(int)((S.nprob + 255) / 256), 256, 0, st>>>(C.info, (int)S.nprob);
    SV_CUDA_TRY(cudaGetLastError());
    SV_CUDA_TRY(cudaMemsetAsync(A.flags, 0, 4 * sizeof(int32_t), st));
    if (C.chunked)
      SV_CUDA_TRY(cudaMemsetAsync(A.chunk_max, 0, sizeof(int32_t) * (S.nblk > 0 ? S.nblk : 1), st));
    double* mtabs = nullptr;
    if (S.tabs) {
      // the Matern tables of the problems of fixed general nu
      mtabs = (double*)(ws + W.mtab);
      k_matern_tables<<<dim3(2 * (kMtabEhi - kMtabEloMin), (unsigned)S.nprob, S.any_est ? 3 : 1), kMtabN, 0,
                        st>>>(C.probs, C.theta, C.tstride, mtabs);
      SV_CUDA_TRY(cudaGetLastError());
      if (split) {
        k_matern_ftabs<<<dim3(kFtabIntervals, (unsigned)S.nprob), kFtabN, 0, st>>>(C.probs, C.theta, C.tstride,
                                                                                 mtabs);
        SV_CUDA_TRY(cudaGetLastError());
      }
    }
    k_prob_params<<<(int)S.nprob, 64, 0, st>>>(C.probs, C.theta, C.tstride, (int)S.nprob, probs, mtabs,
                                               split ? 1 : 0);
    SV_CUDA_TRY(cudaGetLastError());
    if (split && C.nwarp > 0) {
      rc = launch_split_prep(A, S.nx, st);
      if (rc != SV_OK) return rc;
    }
    if ((rc = warp_pass(A)) != SV_OK) return rc;
    if ((rc = cta_pass(A)) != SV_OK) return rc;
    // the largest jitter level of every chunk (of this call's blocks)
    if (C.chunked && bhi > blo) {
      int64_t g = (bhi - blo + 255) / 256;
      if (g > 4096) g = 4096;
      k_chunk_max<<<(int)g, 256, 0, st>>>(A.flags, C.chunk, A.level, S.nblk, blo, bhi, A.chunk_max,
                                           C.bprob, C.info);
      SV_CUDA_TRY(cudaGetLastError());
    }
  }
  if (stage == 0 || stage == 2) {
    // reference chunk-wide jitter: redo blocks whose chunk needed a larger level
    if (C.chunked && bhi > blo) {
      if (sh) {
        const int64_t g = std::min<int64_t>((S.nblk + 255) / 256, 4096);
        k_any_jitter<<<(int)(g > 0 ? g : 1), 256, 0, st>>>(A.chunk_max, S.nblk, A.flags);
        SV_CUDA_TRY(cudaGetLastError());
      }
      LikArgs B = A;
      B.fixup = 1;
      if ((rc = warp_pass(B)) != SV_OK) return rc;
      if ((rc = cta_pass(B)) != SV_OK) return rc;
    }
    // split form: float64 re-evaluation of the blocks it flagged as ill-conditioned
    if (split && C.nwarp > 0) {
      LikArgs B = A;
      B.redo_mode = 1;
      if ((rc = warp_pass(B)) != SV_OK) return rc;
    }
  }

  RedArgs R;
  R.cache = A.cache;
  R.probs = probs;
  R.CS = W.CS;
  R.need_grad = S.need_grad;
  R.nfmax = W.nfmax;
  R.qmax = S.qmax;
  R.Pmax = S.Pmax;
  R.part1 = sh ? sh->part1 : (double*)(ws + W.part1);
  R.part2 = sh ? sh->part2 : (double*)(ws + W.part2);
  R.beta = (double*)(ws + W.beta);
  R.sums = (double*)(ws + W.sums);
  R.theta = C.theta;
  R.tstride = C.tstride;
  R.out = C.out;
  R.ostride = C.ostride;
  R.parts = parts;
  R.pbeg = sh ? sh->pb : 0;
  const int npart = sh ? sh->pe - sh->pb : parts;
  const dim3 rgrid((unsigned)(npart > 0 ? npart : 1), (unsigned)S.nprob);
  if (stage == 0 || stage == 2) {
    int rwarps = kRedThreads / 32;
    while (rwarps > 1 && sizeof(double) * (size_t)rwarps * W.nfmax > (size_t)max_smem_optin()) --rwarps;
    const size_t rsmem = sizeof(double) * (size_t)rwarps * W.nfmax;
    if (rsmem > (size_t)max_smem_optin()) return SV_EINVAL;
    if (npart > 0) {
      SV_CUDA_TRY(cudaFuncSetAttribute(k_reduce1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem));
      k_reduce1<<<rgrid, 32 * rwarps, rsmem, st>>>(R);
      SV_CUDA_TRY(cudaGetLastError());
    }
  }
  if (stage == 0 || stage == 3) {
    k_final1<<<(unsigned)S.nprob, kRedThreads, 0, st>>>(R);
    SV_CUDA_TRY(cudaGetLastError());
    if (npart > 0) {
      k_reduce2<<<rgrid, kRedThreads, 0, st>>>(R);
      SV_CUDA_TRY(cudaGetLastError());
    }
  }
  if (stage == 0 || stage == 4) {
    k_final2<<<(unsigned)S.nprob, 64, 0, st>>>(R);
    SV_CUDA_TRY(cudaGetLastError());
  }
  return SV_OK;
}

EvalShape single_shape(const sv_loglik_desc* D) {
  EvalShape S;
  S.nprob = 1;
  S.nblk = D->nblk;
  S.nblk_max = D->nblk;
  S.nx = D->n * D->d;
  S.dmax = D->d;
  S.qmax = D->q;
  S.Pmax = D->d + 2 + (D->estimate_nu ? 1 : 0);
  S.kmax = D->kmax;
  S.need_grad = D->need_grad;
  S.any_est = D->estimate_nu;
  // the split forms assemble in float32 the closed forms (nu 0.5, 1.5, 2.5)
  // and a fixed nu of the float32 table; another fixed nu runs the float64
  // kernels (an estimated nu is decided on the device at each theta)
  const bool f32 = D->estimate_nu || matern_closed_code(D->nu) >= 0 || ftab_ok(D->nu);
  S.precision = f32 ? D->precision : 0;
  // a fixed nu without a closed form, or an estimated nu: its Matern is
  // interpolated from tables (built if the evaluation's nu is in their range)
  S.tabs = (D->estimate_nu || mtab_ok(D->nu)) ? 1 : 0;
  return S;
}

EvalShape batch_shape(const sv_batch_desc* B) {
  EvalShape S;
  S.nprob = B->nprob;
  S.nblk = B->nblk;
  S.nblk_max = B->nblk_max > 0 ? B->nblk_max : B->nblk;
  S.nx = B->nx;
  S.dmax = B->dmax;
  S.qmax = B->qmax;
  S.Pmax = B->dmax + 2 + (B->any_estimate_nu ? 1 : 0);
  S.kmax = B->kmax;
  S.need_grad = B->need_grad;
  S.any_est = B->any_estimate_nu;
  S.precision = B->precision;
  S.tabs = B->general_nu ? 1 : 0;
  return S;
}

}  // namespace

extern "C" size_t sv_loglik_workspace_bytes(const sv_loglik_desc* D) {
  if (!D) return 0;
  return ws_layout(single_shape(D)).total;
}

namespace {

// Checks of a one-problem call and its EvalCall (the problem table is written
// into the workspace by a one-thread kernel that takes it by value).
int single_call(const sv_loglik_desc* D, const double* theta, const double* X, const double* y,
                const double* Z, const int32_t* rowb, const int32_t* kb, const int32_t* nbr,
                const int32_t* chunk, double* out, int32_t* info, void* workspace,
                size_t workspace_bytes, cudaStream_t st, EvalCall& C) {
  if (!D || !theta || !X || !y || !rowb || !kb || !out || !info) return SV_EINVAL;
  if (D->d < 1 || D->d > kMaxD || D->q < 0 || D->q > kMaxQ || D->nblk < 0 || D->n < 0)
    return SV_EINVAL;
  if (D->q > 0 && !Z) return SV_EINVAL;
  if (D->nblk_warp < 0 || D->nblk_warp > D->nblk) return SV_EINVAL;
  if (D->kmax > 0 && (!nbr || D->ldnbr < D->kmax)) return SV_EINVAL;
  if (D->chunked && !chunk) return SV_EINVAL;
  if (!D->estimate_nu && !(D->nu > 0.0)) return SV_EINVAL;
  if (D->precision < 0 || D->precision > 2) return SV_EINVAL;
  const EvalShape S = single_shape(D);
  WsLayout W = ws_layout(S);
  if (!workspace || workspace_bytes < W.total) return SV_ENOSPC;
  char* ws = (char*)workspace;
  sv_prob_desc pd;
  pd.n = D->n;
  pd.x_off = 0;
  pd.y_off = 0;
  pd.z_off = 0;
  pd.blk_off = 0;
  pd.nblk = D->nblk;
  pd.d = D->d;
  pd.q = D->q;
  pd.estimate_nu = D->estimate_nu;
  pd.skip = 0;
  pd.nu = D->nu;
  pd.var_penalty = D->var_penalty;
  pd.log_var_target = D->log_var_target;
  // written by a one-thread kernel that takes the descriptor by value (no
  // copy from host memory on the stream)
  k_put_desc<<<1, 1, 0, st>>>(pd, (sv_prob_desc*)(ws + W.desc));
  SV_CUDA_TRY(cudaGetLastError());
  C.S = S;
  C.probs = (const sv_prob_desc*)(ws + W.desc);
  C.theta = theta;
  C.tstride = S.Pmax;
  C.X = X;
  C.y = y;
  C.Z = Z;
  C.rowb = rowb;
  C.kb = kb;
  C.nbr = nbr;
  C.chunk = chunk;
  C.bprob = nullptr;
  C.wlist = nullptr;
  C.clist = nullptr;
  C.nwarp = D->nblk_warp;
  C.ncta = D->nblk - D->nblk_warp;
  C.ldnbr = D->ldnbr;
  C.chunked = D->chunked;
  C.team_lanes = D->team_lanes;
  C.rho_min = D->split_rho_min;
  C.out = out;
  C.ostride = 1 + S.Pmax + S.Pmax * S.Pmax + S.qmax;
  C.info = info;
  C.ws = ws;
  return SV_OK;
}

}  // namespace

extern "C" int sv_vecchia_loglik(const sv_loglik_desc* D, const double* theta, const double* X,
                                 const double* y, const double* Z, const int32_t* rowb,
                                 const int32_t* kb, const int32_t* nbr, const int32_t* chunk,
                                 double* out, int32_t* info, void* workspace,
                                 size_t workspace_bytes, sv_stream_t stream) {
  cudaStream_t st = (cudaStream_t)stream;
  EvalCall C;
  const int rc = single_call(D, theta, X, y, Z, rowb, kb, nbr, chunk, out, info, workspace,
                             workspace_bytes, st, C);
  if (rc != SV_OK) return rc;
  return run_eval(C, st);
}

extern "C" int sv_loglik_shard_sizes(const sv_loglik_desc* D, int32_t* parts, int32_t* part1_len,
                                     int32_t* part2_len) {
  if (!D || !parts || !part1_len || !part2_len || D->nblk < 0 || D->d < 1 || D->d > kMaxD ||
      D->q < 0 || D->q > kMaxQ)
    return SV_EINVAL;
  const EvalShape S = single_shape(D);
  *parts = red_parts(S);
  *part1_len = nfield1(S.qmax, S.Pmax, S.need_grad);
  *part2_len = S.Pmax + 1;
  return SV_OK;
}

extern "C" int sv_vecchia_loglik_stage(const sv_loglik_desc* D, int32_t stage, int32_t part_begin,
                                       int32_t part_end, const double* theta, const double* X,
                                       const double* y, const double* Z, const int32_t* rowb,
                                       const int32_t* kb, const int32_t* nbr, const int32_t* chunk,
                                       int32_t* chunk_max, double* part1, double* part2,
                                       double* out, int32_t* info, void* workspace,
                                       size_t workspace_bytes, sv_stream_t stream) {
  if (!D || stage < 1 || stage > 4) return SV_EINVAL;
  int32_t parts = 0, l1 = 0, l2 = 0;
  if (sv_loglik_shard_sizes(D, &parts, &l1, &l2) != SV_OK) return SV_EINVAL;
  if (part_begin < 0 || part_end < part_begin || part_end > parts) return SV_EINVAL;
  if (!part1 || !part2 || (D->chunked && !chunk_max)) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  EvalCall C;
  const int rc = single_call(D, theta, X, y, Z, rowb, kb, nbr, chunk, out, info, workspace,
                             workspace_bytes, st, C);
  if (rc != SV_OK) return rc;
  ShardStage sh;
  sh.stage = stage;
  sh.pb = part_begin;
  sh.pe = part_end;
  sh.chunk_max = chunk_max;
  sh.part1 = part1;
  sh.part2 = part2;
  return run_eval(C, st, &sh);
}

extern "C" size_t sv_loglik_batched_workspace_bytes(const sv_batch_desc* B) {
  if (!B) return 0;
  return ws_layout(batch_shape(B)).total;
}

extern "C" int sv_vecchia_loglik_batched(const sv_batch_desc* B, const sv_prob_desc* probs,
                                         const double* theta, const double* X, const double* y,
                                         const double* Z, const int32_t* rowb, const int32_t* kb,
                                         const int32_t* nbr, const int32_t* bprob,
                                         const int32_t* wlist, const int32_t* clist,
                                         const int32_t* chunk, double* out, int32_t* info,
                                         void* workspace, size_t workspace_bytes,
                                         sv_stream_t stream) {
  if (!B || !probs || !theta || !X || !y || !rowb || !kb || !bprob || !out || !info)
    return SV_EINVAL;
  if (B->nprob < 1 || B->nblk < 0 || B->dmax < 1 || B->dmax > kMaxD || B->qmax < 0 ||
      B->qmax > kMaxQ || B->nwarp < 0 || B->ncta < 0 || B->nwarp + B->ncta != B->nblk)
    return SV_EINVAL;
  if (B->qmax > 0 && !Z) return SV_EINVAL;
  if (B->kmax > 0 && (!nbr || B->ldnbr < B->kmax)) return SV_EINVAL;
  if ((B->nwarp > 0 && !wlist) || (B->ncta > 0 && !clist)) return SV_EINVAL;
  if (B->chunked && !chunk) return SV_EINVAL;
  if (B->precision < 0 || B->precision > 2) return SV_EINVAL;
  const int Pmax = B->dmax + 2 + (B->any_estimate_nu ? 1 : 0);
  if (B->theta_stride < Pmax || B->out_stride < 1 + Pmax + Pmax * Pmax + B->qmax) return SV_EINVAL;
  const EvalShape S = batch_shape(B);
  WsLayout W = ws_layout(S);
  if (!workspace || workspace_bytes < W.total) return SV_ENOSPC;
  EvalCall C;
  C.S = S;
  C.probs = probs;
  C.theta = theta;
  C.tstride = B->theta_stride;
  C.X = X;
  C.y = y;
  C.Z = Z;
  C.rowb = rowb;
  C.kb = kb;
  C.nbr = nbr;
  C.chunk = chunk;
  C.bprob = bprob;
  C.wlist = wlist;
  C.clist = clist;
  C.nwarp = B->nwarp;
  C.ncta = B->ncta;
  C.ldnbr = B->ldnbr;
  C.chunked = B->chunked;
  C.team_lanes = B->team_lanes;
  C.rho_min = B->split_rho_min;
  C.out = out;
  C.ostride = B->out_stride;
  C.info = info;
  C.ws = (char*)workspace;
  return run_eval(C, (cudaStream_t)stream);
}
