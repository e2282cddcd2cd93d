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
// Kernels: k_block_warp (one warp per block, K <= 32), k_block_cta (one CTA
// per block, K > 32), k_chunk_max / fixup (reference chunk-wide jitter),
// k_reduce1 / k_final1 (GLS + Fisher sums, beta), k_reduce2 / k_final2
// (ll, score, variance penalty).  Reductions are in a fixed order, so results
// are bitwise reproducible run to run.
#include <stdio.h>

#include "sv_loglik.cuh"

namespace sv {

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

// One block, processed by a team.  Writes the block's record to the cache.
template <int T>
__device__ void block_pass1(const LikArgs& A, const PrmSmem* prm, int64_t b, double* sm) {
  const int lane = Team<T>::lane();
  const int d = A.d, q = A.q, P = A.P, NR = A.NR, kt = A.kt;
  const int k = A.kb[b];
  const int K = k + 1;
  const int64_t tri = (int64_t)kt * (kt + 1) / 2;
  double* u = sm;
  double* Lp = u + (int64_t)kt * d;
  double* Gp = A.need_grad ? Lp + tri : nullptr;
  double* Dp = A.estimate_nu ? (Lp + tri * (A.need_grad ? 2 : 1)) : nullptr;
  double* R = Lp + tri * (1 + (A.need_grad ? 1 : 0) + (A.estimate_nu ? 1 : 0));
  double* a = R + (int64_t)NR * kt;
  double* invd = a + kt;
  double* acc = invd + kt;
  int* idx = (int*)(acc + kt);
  volatile int* flag = idx + kt;
  double* red = (double*)(acc + kt + (kt + 1) / 2 + 1);

  // ---- gather: neighbours first, self last (likelihood.py:113)
  for (int i = lane; i < K; i += T) idx[i] = (i < k) ? A.nbr[b * A.ldnbr + i] : A.rowb[b];
  Team<T>::sync();
  for (int t = lane; t < K * d; t += T) {
    const int i = t / d, l = t - (t / d) * d;
    u[i * d + l] = A.X[(int64_t)idx[i] * d + l] * prm->invlam[l];
  }
  Team<T>::sync();

  // ---- Sigma, Cholesky, jitter retry (_covariance.py:235-252)
  const double s2 = prm->s2, tau = prm->tau;
  int lv = 0;
  if (A.fixup) {
    lv = A.chunk_max[A.chunk[b]];
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
    assemble_sigma<T>(K, d, u, nullptr, s2, tau, jit, prm->mm, Lp, Gp, Dp);
    Team<T>::sync();
    ok = cholesky_packed<T>(K, Lp, invd, flag);
    Team<T>::sync();
    if (ok) break;
  }
  double* rec = A.cache + b * (int64_t)A.CS;
  if (!ok) {
    if (lane == 0) {
      set_error(A.info + SV_INFO_STATUS, SV_ECHOL);
      atomicCAS(A.info + SV_INFO_BLOCK, -1, (int)b);
    }
    if (lane == 0) A.level[b] = 10;
    for (int f = lane; f < A.CS; f += T) rec[f] = 0.0;
    return;
  }
  if (lane == 0) {
    A.level[b] = (int8_t)lv;
    if (lv > 0) {
      atomicMax(A.info + SV_INFO_JITTER, lv);
      A.flags[0] = 1;
    }
  }
  double jit_used = 0.0;
  if (lv > 0) {
    double sc = 0.0;
    for (int i = 0; i < K; ++i) sc += s2 * (1.0 + tau);
    jit_used = jitter_pow10(lv) * (sc / (double)K);
  }

  // ---- a = L^-T e_K  (likelihood.py:125-127)
  backsolve_eK<T>(K, Lp, invd, a, acc);
  Team<T>::sync();

  // ---- GLS parts a.y, a.Z (likelihood.py:129-134)
  {
    double vy = 0.0;
    for (int i = lane; i < K; i += T) vy += a[i] * A.y[idx[i]];
    vy = team_sum<T>(vy, red);
    if (lane == 0) {
      rec[0] = Lp[tri_off(K - 1, K - 1)];  // L_KK; the log is taken in the reduction
      rec[1] = vy;
    }
    for (int c = 0; c < q; ++c) {
      double vz = 0.0;
      for (int i = lane; i < K; i += T) vz += a[i] * A.Z[(int64_t)idx[i] * q + c];
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
  // p = 0: dSigma_0 = Sigma (un-jittered) = L L^T - jit I, so Sigma a = L_KK e_K - jit a
  for (int i = lane; i < K; i += T)
    R[i] = ((i == K - 1) ? Lp[tri_off(K - 1, K - 1)] : 0.0) - jit_used * a[i];
  // p = 1..d: (dSigma_l a)_i = sum_j G_ij (u_il - u_jl)^2 a_j   (_covariance.py:142-146)
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
  int p = 1 + d;
  if (A.estimate_nu) {
    for (int i = lane; i < K; i += T) {
      double s = 0.0;
      for (int j = 0; j < K; ++j) s += ((i >= j) ? Dp[tri_off(i, j)] : Dp[tri_off(j, i)]) * a[j];
      R[p * ldr + i] = s;
    }
    ++p;
  }
  // nugget row: dSigma_tau = s2 * tau * I
  for (int i = lane; i < K; i += T) R[p * ldr + i] = s2 * tau * a[i];
  for (int i = lane; i < K; i += T) {
    R[P * ldr + i] = A.y[idx[i]];
    for (int c = 0; c < q; ++c) R[(P + 1 + c) * ldr + i] = A.Z[(int64_t)idx[i] * q + c];
  }
  Team<T>::sync();

  // ---- W = L^-1 [dSigma a], z parts = L^-1 [y, Z]  (likelihood.py:139, 154)
  forward_solve_multi<T>(K, Lp, invd, R, NR, ldr);

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

__global__ void k_block_warp(LikArgs A) {
  extern __shared__ double smem[];
  PrmSmem* prm = (PrmSmem*)smem;
  load_params(A, prm);
  const int64_t per_team = team_smem_doubles(32, A.d, A.NR, A.need_grad, A.estimate_nu);
  const int w = threadIdx.x >> 5;
  double* sm = smem + (sizeof(PrmSmem) + 7) / 8 + w * per_team;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t b = A.b0 + (int64_t)blockIdx.x * (blockDim.x >> 5) + w; b < A.b1; b += nw) {
    if (A.redo_mode) {
      if (!A.redo[b]) continue;
    } else if (A.fixup) {
      if (A.chunk_max[A.chunk[b]] <= A.level[b]) continue;
    } else if (A.kb[b] + 1 > 32) {
      if ((threadIdx.x & 31) == 0) set_error(A.info + SV_INFO_STATUS, SV_EINVAL);
      continue;
    }
    block_pass1<32>(A, prm, b, sm);
    __syncwarp();
  }
}

__global__ void k_block_cta(LikArgs A) {
  extern __shared__ double smem[];
  PrmSmem* prm = (PrmSmem*)smem;
  load_params(A, prm);
  double* sm = smem + (sizeof(PrmSmem) + 7) / 8;
  for (int64_t b = A.b0 + blockIdx.x; b < A.b1; b += gridDim.x) {
    if (A.fixup) {
      if (A.chunk_max[A.chunk[b]] <= A.level[b]) continue;
    } else if (A.kb[b] + 1 > A.kt) {
      if (threadIdx.x == 0) set_error(A.info + SV_INFO_STATUS, SV_EINVAL);
      continue;
    }
    block_pass1<128>(A, prm, b, sm);
    __syncthreads();
  }
}

// chunk-wide jitter: chunk_max[c] = max level over the chunk's blocks
__global__ void k_chunk_max(const int32_t* flags, const int32_t* chunk, const int8_t* level,
                            int64_t nblk, int32_t* chunk_max) {
  if (flags[0] == 0) return;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nblk;
       b += (int64_t)gridDim.x * blockDim.x) {
    const int lv = level[b];
    if (lv > 0 && lv <= 9) atomicMax(chunk_max + chunk[b], lv);
  }
}

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
struct RedArgs {
  const double* cache;
  int64_t nblk;
  int CS, q, P, need_grad;
  double* part1;  // [nctas][nfield1]
  double* part2;  // [nctas][1 + P]
  double* beta;   // [q]
  double* sums;   // [nfield1] final pass-1 sums
  const double* theta;
  double var_penalty, log_var_target;
  int64_t n;
  double* out;
  int32_t* info;
};

// pass-1 fields: logdet, Zty[q], XtX[q*q], F[P(P+1)/2]
__host__ __device__ inline int nfield1(int q, int P, int need_grad) {
  return 1 + q + q * q + (need_grad ? P * (P + 1) / 2 : 0);
}

__global__ void k_reduce1(RedArgs R) {
  const int nf = nfield1(R.q, R.P, R.need_grad);
  const int64_t per = (R.nblk + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = blockIdx.x * per;
  const int64_t b1 = min(R.nblk, b0 + per);
  const int q = R.q;
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    double s = 0.0;
    if (f == 0) {
      for (int64_t b = b0; b < b1; ++b) s += log(R.cache[b * R.CS]);
    } else if (f < 1 + q) {
      const int i = f - 1;
      for (int64_t b = b0; b < b1; ++b) s += R.cache[b * R.CS + 2 + i] * R.cache[b * R.CS + 1];
    } else if (f < 1 + q + q * q) {
      const int e = f - 1 - q;
      const int i = e / q, j = e - (e / q) * q;
      for (int64_t b = b0; b < b1; ++b)
        s += R.cache[b * R.CS + 2 + i] * R.cache[b * R.CS + 2 + j];
    } else {
      const int e = f - 1 - q - q * q;
      const int off = 3 + 2 * q + R.P * (2 + q) + e;
      for (int64_t b = b0; b < b1; ++b) s += R.cache[b * R.CS + off];
    }
    R.part1[blockIdx.x * (int64_t)nf + f] = s;
  }
}

__global__ void k_final1(RedArgs R, int nparts) {
  const int nf = nfield1(R.q, R.P, R.need_grad);
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nparts; ++c) s += R.part1[c * (int64_t)nf + f];
    R.sums[f] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // beta = solve(XtX + 1e-12 I, Zty): Gaussian elimination, partial pivoting
    const int q = R.q;
    double M[kMaxQ][kMaxQ + 1];
    for (int i = 0; i < q; ++i) {
      for (int j = 0; j < q; ++j) M[i][j] = R.sums[1 + q + i * q + j] + (i == j ? 1e-12 : 0.0);
      M[i][q] = R.sums[1 + i];
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
      for (int j = c + 1; j < q; ++j) s -= M[c][j] * R.beta[j];
      R.beta[c] = s / M[c][c];
    }
  }
}

__global__ void k_reduce2(RedArgs R) {
  __shared__ double sbeta[kMaxQ];
  __shared__ double red[kRedThreads / 32][kMaxP + 1];
  const int q = R.q, P = R.P, np = R.need_grad ? P : 0;
  for (int i = threadIdx.x; i < q; i += blockDim.x) sbeta[i] = R.beta[i];
  __syncthreads();
  const int64_t per = (R.nblk + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = blockIdx.x * per;
  const int64_t b1 = min(R.nblk, b0 + per);
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
      for (int p = 0; p < P; ++p) {
        double wz = wzy[p];
        for (int i = 0; i < q; ++i) wz -= wzZ[p * q + i] * sbeta[i];
        acc[1 + p] -= 0.5 * (wK[p] * (1.0 + zK * zK) - 2.0 * zK * wz);
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
    R.part2[blockIdx.x * (int64_t)(1 + np) + i] = s;
  }
}

__global__ void k_final2(RedArgs R, int nparts) {
  const int P = R.P, q = R.q, np = R.need_grad ? P : 0;
  const int nf = nfield1(q, P, R.need_grad);
  __shared__ double tot[kMaxP + 1];
  for (int i = threadIdx.x; i <= np; i += blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nparts; ++c) s += R.part2[c * (int64_t)(1 + np) + i];
    tot[i] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // ll = -n/2 log(2pi) - sum_b (log L_KK + z_K^2 / 2)  (likelihood.py:149-156)
    double ll = -0.5 * (double)R.n * 1.8378770664093453 + tot[0];
    double g0 = np ? tot[1] : 0.0;
    double f00_add = 0.0;
    if (R.var_penalty > 0.0) {  // likelihood.py:165-171
      double excess = R.theta[0] - R.log_var_target;
      if (excess < 0.0) excess = 0.0;
      ll -= 0.5 * R.var_penalty * excess * excess;
      g0 -= R.var_penalty * excess;
      if (excess > 0.0) f00_add = R.var_penalty;
    }
    R.out[0] = ll;
    if (np) {
      R.out[1] = g0;
      for (int p = 1; p < P; ++p) R.out[1 + p] = tot[1 + p];
    }
    (void)f00_add;
    if (np) {
      // Fisher: sums hold the packed lower triangle
      double* fish = R.out + 1 + P;
      const int foff = 1 + q + q * q;
      for (int i = 0; i < P; ++i)
        for (int j = 0; j <= i; ++j) {
          const double v = R.sums[foff + i * (i + 1) / 2 + j];
          fish[i * P + j] = v;
          fish[j * P + i] = v;
        }
      fish[0] += f00_add;
    }
    if (!np)
      for (int i = 0; i < P + P * P; ++i) R.out[1 + i] = 0.0;
    double* bo = R.out + 1 + P + P * P;
    for (int i = 0; i < q; ++i) bo[i] = R.beta[i];
  }
  (void)nf;
}

}  // namespace sv

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace sv;

static int nred_ctas(int64_t nblk) {
  int64_t c = (nblk + 1023) / 1024;
  if (c < 1) c = 1;
  if (c > 4 * (int64_t)sv_num_sms()) c = 4 * (int64_t)sv_num_sms();
  return (int)c;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct WsLayout {
  size_t cache, level, redo, chunk_max, flags, part1, part2, beta, sums, xhl, total;
};

static WsLayout ws_layout(const sv_loglik_desc* D) {
  const int P = D->d + 2 + (D->estimate_nu ? 1 : 0);
  const int q = D->q;
  const int CS = 3 + 2 * q + (D->need_grad ? (2 * P + P * q + P * (P + 1) / 2) : 0);
  const int nr = nred_ctas(D->nblk);
  WsLayout L;
  size_t off = 0;
  L.cache = off;
  off = align256(off + sizeof(double) * (size_t)CS * (size_t)(D->nblk > 0 ? D->nblk : 1));
  L.level = off;
  off = align256(off + (size_t)(D->nblk > 0 ? D->nblk : 1));
  L.redo = off;
  off = align256(off + (size_t)(D->nblk > 0 ? D->nblk : 1));
  L.chunk_max = off;
  off = align256(off + sizeof(int32_t) * (size_t)(D->nblk > 0 ? D->nblk : 1));
  L.flags = off;
  off = align256(off + 4 * sizeof(int32_t));
  L.part1 = off;
  off = align256(off + sizeof(double) * (size_t)nr * nfield1(q, P, D->need_grad));
  L.part2 = off;
  off = align256(off + sizeof(double) * (size_t)nr * (P + 1));
  L.beta = off;
  off = align256(off + sizeof(double) * (kMaxQ + 1));
  L.sums = off;
  off = align256(off + sizeof(double) * (size_t)nfield1(q, P, D->need_grad));
  L.xhl = off;
  if (D->precision == 1) off = align256(off + sizeof(float) * 2 * (size_t)D->n * (size_t)D->d);
  L.total = off;
  return L;
}

extern "C" size_t sv_loglik_workspace_bytes(const sv_loglik_desc* D) {
  if (!D) return 0;
  return ws_layout(D).total;
}

static int g_max_smem_optin = -1;
static int max_smem_optin() {
  if (g_max_smem_optin < 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    g_max_smem_optin = v;
  }
  return g_max_smem_optin;
}

extern "C" int sv_vecchia_loglik(const sv_loglik_desc* D, const double* theta, const double* X,
                                 const double* y, const double* Z, const int32_t* rowb,
                                 const int32_t* kb, const int32_t* nbr, const int32_t* chunk,
                                 double* out, int32_t* info, void* workspace,
                                 size_t workspace_bytes, sv_stream_t stream) {
  if (!D || !theta || !X || !y || !rowb || !kb || !out || !info) return SV_EINVAL;
  if (D->d < 1 || D->d > kMaxD || D->q < 0 || D->q > kMaxQ || D->nblk < 0 || D->n < 0)
    return SV_EINVAL;
  if (D->q > 0 && !Z) return SV_EINVAL;
  if (D->nblk_warp < 0 || D->nblk_warp > D->nblk) return SV_EINVAL;
  if (D->kmax > 0 && (!nbr || D->ldnbr < D->kmax)) return SV_EINVAL;
  if (D->chunked && !chunk) return SV_EINVAL;
  const int closed = matern_closed_code(D->nu);
  if (!D->estimate_nu && !(D->nu > 0.0)) return SV_EINVAL;
  if (D->precision != 0 && D->precision != 1) return SV_EINVAL;
  WsLayout W = ws_layout(D);
  if (!workspace || workspace_bytes < W.total) return SV_ENOSPC;
  cudaStream_t st = (cudaStream_t)stream;
  char* ws = (char*)workspace;

  LikArgs A;
  A.X = X;
  A.y = y;
  A.Z = Z;
  A.rowb = rowb;
  A.kb = kb;
  A.nbr = nbr;
  A.chunk = chunk;
  A.theta = theta;
  A.cache = (double*)(ws + W.cache);
  A.level = (int8_t*)(ws + W.level);
  A.chunk_max = (int32_t*)(ws + W.chunk_max);
  A.flags = (int32_t*)(ws + W.flags);
  A.info = info;
  A.n = D->n;
  A.d = D->d;
  A.q = D->q;
  A.ldnbr = D->ldnbr;
  A.P = D->d + 2 + (D->estimate_nu ? 1 : 0);
  A.NR = D->need_grad ? (A.P + 1 + A.q) : 0;
  A.CS = 3 + 2 * A.q + (D->need_grad ? (2 * A.P + A.P * A.q + A.P * (A.P + 1) / 2) : 0);
  A.need_grad = D->need_grad;
  A.estimate_nu = D->estimate_nu;
  A.closed = closed;
  A.nu_fixed = D->nu;
  A.nu_fd_h = 1e-3;  // _matern_general.py:135 (nu_fd_h)
  A.fixup = 0;
  A.redo = (int8_t*)(ws + W.redo);
  A.rho_min = D->split_rho_min > 0.0 ? D->split_rho_min : 1e-4;
  A.redo_mode = 0;
  A.xhl = (float2*)(ws + W.xhl);

  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  SV_CUDA_TRY(cudaMemsetAsync(A.flags, 0, 4 * sizeof(int32_t), st));
  if (D->chunked) SV_CUDA_TRY(cudaMemsetAsync(A.chunk_max, 0, sizeof(int32_t) * D->nblk, st));

  const int nsm = sv_num_sms();
  const size_t prm_bytes = (sizeof(PrmSmem) + 7) / 8 * 8;
  // warp-sized blocks [0, nblk_warp): float64 warp kernel or split kernel
  // split form: closed-form nu and at most 32 right-hand sides (d + q <= 29);
  // anything else runs the float64 kernels
  const bool split = D->precision == 1 && !D->estimate_nu && closed >= 0 && A.NR <= 32;
  const int lanes = D->team_lanes > 0 ? D->team_lanes : 8;
  if (split && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32) return SV_EINVAL;
  if (D->nblk_warp > 0) {
    A.kt = 32;
    A.b0 = 0;
    A.b1 = D->nblk_warp;
    if (split) {
      int rc = launch_split_prep(A, st);
      if (rc != SV_OK) return rc;
      rc = launch_block_split(A, lanes, st);
      if (rc != SV_OK) return rc;
    } else {
      const size_t team = sizeof(double) * team_smem_doubles(32, A.d, A.NR, A.need_grad, A.estimate_nu);
      int wpc = 8;
      while (wpc > 1 && prm_bytes + wpc * team > (size_t)max_smem_optin()) --wpc;
      const size_t smem = prm_bytes + wpc * team;
      if (smem > (size_t)max_smem_optin()) return SV_EINVAL;
      SV_CUDA_TRY(cudaFuncSetAttribute(k_block_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      int64_t grid = (D->nblk_warp + wpc - 1) / wpc;
      if (grid > 64LL * nsm) grid = 64LL * nsm;
      k_block_warp<<<(int)grid, 32 * wpc, smem, st>>>(A);
      SV_CUDA_TRY(cudaGetLastError());
    }
  }
  // CTA kernel: blocks [nblk_warp, nblk)
  size_t cta_smem = 0;
  if (D->nblk > D->nblk_warp) {
    A.kt = D->kmax + 1;
    A.b0 = D->nblk_warp;
    A.b1 = D->nblk;
    cta_smem = prm_bytes + sizeof(double) * team_smem_doubles(A.kt, A.d, A.NR, A.need_grad, A.estimate_nu);
    if (cta_smem > (size_t)max_smem_optin()) return SV_EINVAL;
    SV_CUDA_TRY(cudaFuncSetAttribute(k_block_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cta_smem));
    int64_t grid = D->nblk - D->nblk_warp;
    if (grid > 8LL * nsm) grid = 8LL * nsm;
    k_block_cta<<<(int)grid, 128, cta_smem, st>>>(A);
    SV_CUDA_TRY(cudaGetLastError());
  }
  // reference chunk-wide jitter: redo blocks whose chunk needed a larger level
  if (D->chunked && D->nblk > 0) {
    k_chunk_max<<<(int)((D->nblk + 255) / 256 > 4096 ? 4096 : (D->nblk + 255) / 256), 256, 0, st>>>(
        A.flags, chunk, A.level, D->nblk, A.chunk_max);
    SV_CUDA_TRY(cudaGetLastError());
    A.fixup = 1;
    if (D->nblk_warp > 0) {
      A.kt = 32;
      A.b0 = 0;
      A.b1 = D->nblk_warp;
      if (split) {
        const int rc = launch_block_split(A, lanes, st);
        if (rc != SV_OK) return rc;
      } else {
        const size_t team = sizeof(double) * team_smem_doubles(32, A.d, A.NR, A.need_grad, A.estimate_nu);
        int wpc = 8;
        while (wpc > 1 && prm_bytes + wpc * team > (size_t)max_smem_optin()) --wpc;
        k_block_warp<<<(int)((D->nblk_warp + wpc - 1) / wpc > 64LL * nsm ? 64LL * nsm : (D->nblk_warp + wpc - 1) / wpc),
                       32 * wpc, prm_bytes + wpc * team, st>>>(A);
        SV_CUDA_TRY(cudaGetLastError());
      }
    }
    if (D->nblk > D->nblk_warp) {
      A.kt = D->kmax + 1;
      A.b0 = D->nblk_warp;
      A.b1 = D->nblk;
      int64_t grid = D->nblk - D->nblk_warp;
      if (grid > 8LL * nsm) grid = 8LL * nsm;
      k_block_cta<<<(int)grid, 128, cta_smem, st>>>(A);
      SV_CUDA_TRY(cudaGetLastError());
    }
  }

  // split form: float64 re-evaluation of the blocks it flagged as ill-conditioned
  if (split && D->nblk_warp > 0) {
    A.fixup = 0;
    A.redo_mode = 1;
    A.kt = 32;
    A.b0 = 0;
    A.b1 = D->nblk_warp;
    const size_t team = sizeof(double) * team_smem_doubles(32, A.d, A.NR, A.need_grad, A.estimate_nu);
    int wpc = 8;
    while (wpc > 1 && prm_bytes + wpc * team > (size_t)max_smem_optin()) --wpc;
    const size_t smem = prm_bytes + wpc * team;
    if (smem > (size_t)max_smem_optin()) return SV_EINVAL;
    SV_CUDA_TRY(cudaFuncSetAttribute(k_block_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int64_t grid = (D->nblk_warp + wpc - 1) / wpc;
    if (grid > 64LL * nsm) grid = 64LL * nsm;
    k_block_warp<<<(int)grid, 32 * wpc, smem, st>>>(A);
    SV_CUDA_TRY(cudaGetLastError());
  }

  RedArgs R;
  R.cache = A.cache;
  R.nblk = D->nblk;
  R.CS = A.CS;
  R.q = A.q;
  R.P = A.P;
  R.need_grad = A.need_grad;
  R.part1 = (double*)(ws + W.part1);
  R.part2 = (double*)(ws + W.part2);
  R.beta = (double*)(ws + W.beta);
  R.sums = (double*)(ws + W.sums);
  R.theta = theta;
  R.var_penalty = D->var_penalty;
  R.log_var_target = D->log_var_target;
  R.n = D->n;
  R.out = out;
  R.info = info;
  const int nr = nred_ctas(D->nblk);
  k_reduce1<<<nr, kRedThreads, 0, st>>>(R);
  SV_CUDA_TRY(cudaGetLastError());
  k_final1<<<1, kRedThreads, 0, st>>>(R, nr);
  SV_CUDA_TRY(cudaGetLastError());
  k_reduce2<<<nr, kRedThreads, 0, st>>>(R);
  SV_CUDA_TRY(cudaGetLastError());
  k_final2<<<1, 64, 0, st>>>(R, nr);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}
