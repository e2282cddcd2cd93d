// Prediction blocks and the sparse triangular solve of the joint predictive
// distribution.
//
//   k_pred_*      : gp.py:257-276 (_predict_scaled) and gp.py:329-348
//                   (_joint_factor): per target, the block [neighbours, target]
//                   with a noise-free target (nugget only on observation rows),
//                   Cholesky with jitter retry, a = L^-T e_K; marginal mean
//                   -a[:k].r / a_K and variance 1 / a_K^2, or the column a of
//                   the sparse inverse Cholesky factor U.
//                   Split form (closed-form nu): the entries below the
//                   diagonal from coordinates centred on the target, held as
//                   float32 (hi, lo) pairs, and the float32 correlation
//                   deficit, one float64 FMA each; the diagonal,
//                   the LDL^T and every solve in float64.  A block with a
//                   pivot ratio d_k / Sigma_kk below rho_min, or that does not
//                   factor, is redone in float64 from the start.
//   k_joint_solve : U_pp^T x = rhs (gp.py:380-401, scipy spsolve_triangular),
//                   one CTA per row (its threads split the right-hand sides),
//                   rows claimed in order, bounded waits on the rows it
//                   depends on.
#include "sv_block.cuh"

namespace sv {

struct PredArgs {
  const double* theta;  // [log s2, log lam_1..d, log tau]
  const double* Xall;
  const int32_t* tgt;
  const int32_t* nbr;
  const double* resid;
  double* mean;
  double* var;
  double* acol;
  double* rhs;
  int32_t* info;
  int64_t nobs, nblk;
  int d, k, ldnbr, kt;
  int closed;
  int target_nugget;
  int split;       // 1: float32 assembly (closed-form nu only)
  double rho_min;  // split: smallest pivot ratio d_k / Sigma_kk kept
  double nu;
  const double* tab;    // general nu: its Matern table (or null: K_nu per entry)
  const float4* ftab;   // general nu, split: the table's float32 part (or null)
};

struct PredPrm {
  double s2, tau;
  MaternMode mm;
  MaternF32 mf;  // the split form's float32 Matern: a closed form or the table
  double invlam[64];
};

__device__ void pred_params(const PredArgs& A, PredPrm* prm) {
  if (threadIdx.x == 0) {
    prm->s2 = exp(A.theta[0]);
    prm->tau = exp(A.theta[1 + A.d]);
    MaternMode mm;
    mm.closed = A.closed;
    mm.estimate_nu = 0;
    mm.nu = A.nu;
    mm.log_coef = A.closed < 0 ? matern_log_coef(A.nu) : 0.0;
    mm.nu_p = mm.nu_m = mm.lc_p = mm.lc_m = 0.0;
    mm.inv2h = 0.0;
    mm.tab = A.closed < 0 ? A.tab : nullptr;
    mm.tab_elo = mm.tab ? mtab_elo(A.nu) : 0;
    mm.s2n = sqrt(2.0 * A.nu);
    mm.tab_p = mm.tab_m = nullptr;
    mm.elo_p = mm.elo_m = 0;
    mm.s2n_p = mm.s2n_m = 0.0;
    prm->mm = mm;
    MaternF32 mf;
    mf.code = A.closed >= 0 ? A.closed : (A.ftab ? 3 : -1);
    mf.elo = A.ftab ? mtab_elo(A.nu) : 0;
    mf.esw = ftab_switch(A.nu);
    mf.s2n = (float)sqrt(2.0 * A.nu);
    mf.tab = A.closed >= 0 ? nullptr : A.ftab;
    mf.dtab = nullptr;
    mf.nuf = (float)A.nu;
    prm->mf = mf;
  }
  for (int l = threadIdx.x; l < A.d; l += blockDim.x) prm->invlam[l] = exp(-A.theta[1 + l]);
  __syncthreads();
}

// columns per panel of the blocked LDL^T
constexpr int kPredW = 8;

__host__ __device__ inline int64_t pred_team_doubles(int kt, int d) {
  return (int64_t)kt * d + (int64_t)kt * (kt + 1) / 2 + (4 + kPredW) * (int64_t)kt + (kt + 1) / 2 +
         1 + 40;
}

// |x| below 2^60: d <= 64 squared float32 differences of such coordinates
// stay finite
constexpr long long kBitsCoordMax = 0x43B0000000000000LL;

// The split form's attempt at a block: coordinates centred on the target
// (scaled differences formed in float64, kept as float32 (hi, lo) pairs), the entries
// below the diagonal s2 (1 - D(r_ij)) with D the float32 correlation deficit
// (accurate for close pairs), the diagonal s2 (1 + tau mask_i) in float64,
// then the LDL^T with the pivot-ratio guard (thresholds rho_min Sigma_kk in
// rb).  Returns false when the block must be redone in float64: a coordinate
// out of range, a pivot that is not > 0 or below its threshold.
template <int T>
__device__ bool pred_split_factor(const PredArgs& A, const PredPrm* prm, int K, double* u,
                                  double* Lp, double* invd, double* acc, const double* mask,
                                  long long* rb, const int* idx, volatile int* flag) {
  const int lane = Team<T>::lane();
  const int d = A.d;
  float2* u2 = (float2*)u;
  const double* xt = A.Xall + (int64_t)idx[K - 1] * d;
  if (lane == 0) flag[1] = 0;
  Team<T>::sync();
  bool in_range = true;
  for (int t = lane; t < K * d; t += T) {
    const int i = t / d, l = t - (t / d) * d;
    const double v = (A.Xall[(int64_t)idx[i] * d + l] - xt[l]) * prm->invlam[l];
    in_range = in_range && (dbits(v) & 0x7FFFFFFFFFFFFFFFLL) < kBitsCoordMax;
    const float hi = d2f_int(v);
    u2[t] = make_float2(hi, d2f_int(v - f2d_int(hi)));
  }
  if (!in_range) flag[1] = 1;
  const double s2 = prm->s2, tau = prm->tau;
  for (int i = lane; i < K; i += T) rb[i] = dbits(A.rho_min * (s2 * (1.0 + tau * mask[i])));
  Team<T>::sync();
  if (flag[1]) return false;
  const MaternF32 mf = prm->mf;
  const int npair = K * (K + 1) / 2;
  for (int t = lane; t < npair; t += T) {
    int i, j;
    tri_index(t, i, j);
    double v;
    if (i == j) {
      v = s2 * (1.0 + tau * mask[i]);
    } else {
      const float2* ui = u2 + i * d;
      const float2* uj = u2 + j * d;
      float r2 = 0.0f;
      for (int l = 0; l < d; ++l) {
        // (hi_i - hi_j) + (lo_i - lo_j): the difference to about one float32
        // rounding of itself, however far the pair lies from the target
        const float2 a = ui[l], c = uj[l];
        const float df = (a.x - c.x) + (a.y - c.y);
        r2 = fmaf(df, df, r2);
      }
      v = fma(-s2, f2d_int(matern_deficit_f32(mf, sqrtf(r2))), s2);
    }
    Lp[t] = v;
  }
  if (lane == 0) *flag = 0;
  Team<T>::sync();
  const bool ok = ldlt_blocked<T, kPredW>(K, Lp, invd, acc, A.kt, flag, rb);
  Team<T>::sync();
  return ok;
}

template <int T>
__device__ void pred_block(const PredArgs& A, const PredPrm* prm, int64_t b, double* sm) {
  const int lane = Team<T>::lane();
  const int d = A.d, kcap = A.k, kt = A.kt;
  double* u = sm;
  double* Lp = u + (int64_t)kt * d;
  double* a = Lp + (int64_t)kt * (kt + 1) / 2;
  double* invd = a + kt;
  double* acc = invd + kt;                 // kPredW columns of kt
  double* mask = acc + kPredW * kt;
  double* rv = mask + kt;
  int* idx = (int*)(rv + kt);
  volatile int* flag = idx + kt;
  double* red = (double*)(rv + kt + (kt + 1) / 2 + 1);

  // neighbours are packed at the front of the row; -1 marks absent entries
  // (rows with fewer than k predecessors)
  if (lane == 0) {
    int kb = 0;
    while (kb < kcap && A.nbr[b * A.ldnbr + kb] >= 0) ++kb;
    *flag = kb;
  }
  Team<T>::sync();
  const int k = *flag;
  const int K = k + 1;
  Team<T>::sync();
  for (int i = lane; i < K; i += T) {
    const int ix = (i < k) ? A.nbr[b * A.ldnbr + i] : A.tgt[b];
    idx[i] = ix;
    // gp.py:263-265, 336-339: nugget on observations only, target noise-free
    // (a prior draw keeps the nugget on every row, target included)
    mask[i] = ((i < k && ix < A.nobs) || (i == k && A.target_nugget)) ? 1.0 : 0.0;
    rv[i] = (A.resid && i < k && ix < A.nobs) ? A.resid[ix] : 0.0;
  }
  Team<T>::sync();
  const double s2 = prm->s2, tau = prm->tau;
  bool ok = false;
  if (A.split) ok = pred_split_factor<T>(A, prm, K, u, Lp, invd, acc, mask, (long long*)a, idx, flag);
  if (!ok) {
    if (A.split && lane == 0) atomicAdd(A.info + SV_INFO_AUX, 1);
    for (int t = lane; t < K * d; t += T) {
      const int i = t / d, l = t - (t / d) * d;
      u[i * d + l] = A.Xall[(int64_t)idx[i] * d + l] * prm->invlam[l];
    }
    Team<T>::sync();
  }
  for (int lv = 0; lv <= 9 && !ok; ++lv) {
    double jit = 0.0;
    if (lv > 0) {
      // 10^p * mean(diag Sigma)   (_covariance.py:245-249)
      double sc = 0.0;
      for (int i = 0; i < K; ++i) sc += s2 * (1.0 + tau * mask[i]);
      const double p10[10] = {0.0, 1e-12, 1e-11, 1e-10, 1e-9, 1e-8, 1e-7, 1e-6, 1e-5, 1e-4};
      jit = p10[lv] * (sc / (double)K);
    }
    if (lane == 0) *flag = 0;
    assemble_sigma<T>(K, d, u, mask, s2, tau, jit, prm->mm, Lp, nullptr, nullptr);
    Team<T>::sync();
    ok = ldlt_blocked<T, kPredW>(K, Lp, invd, acc, kt, flag);
    Team<T>::sync();
    if (ok) {
      if (lv > 0 && lane == 0) atomicMax(A.info + SV_INFO_JITTER, lv);
      break;
    }
  }
  if (!ok) {
    if (lane == 0) {
      set_error(A.info + SV_INFO_STATUS, SV_ECHOL);
      atomicCAS(A.info + SV_INFO_BLOCK, -1, (int)b);
    }
    return;
  }
  // Sigma = L D L^T = C C^T with C = L D^(1/2): a = C^-T e_K = u / sqrt(d_K),
  // u = L^-T e_K (u_K = 1), so mean = -a[:k].r / a_K = -u[:k].r and
  // var = 1 / a_K^2 = d_K; only the U column needs the square root
  backsolve_unit_eK<T>(K, Lp, a, acc);
  Team<T>::sync();
  double s = 0.0;
  for (int i = lane; i < k; i += T) s += a[i] * rv[i];
  s = team_sum<T>(s, red);
  const double dK = Lp[tri_off(K - 1, K - 1)];
  const double sK = 1.0 / sqrt(dK);
  if (lane == 0) {
    if (A.mean) A.mean[b] = -s;
    if (A.var) A.var[b] = dK;
    if (A.rhs) A.rhs[b] = -s * sK;
  }
  if (A.acol) {
    // column of U laid out as [neighbour slots 0..kcap-1, target]; absent
    // neighbour slots hold 0
    const int Kc = kcap + 1;
    for (int i = lane; i < Kc; i += T)
      A.acol[b * (int64_t)Kc + i] = (i < k) ? a[i] * sK : (i == kcap ? sK : 0.0);
  }
}

__global__ void k_pred_warp(PredArgs A) {
  extern __shared__ double smem[];
  PredPrm* prm = (PredPrm*)smem;
  pred_params(A, prm);
  const int64_t per = pred_team_doubles(32, A.d);
  const int w = threadIdx.x >> 5;
  double* sm = smem + (sizeof(PredPrm) + 7) / 8 + w * per;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + w; b < A.nblk; b += nw) {
    pred_block<32>(A, prm, b, sm);
    __syncwarp();
  }
}

// threads of the CTA that owns one large prediction block: two CTAs of a
// 141-point block fill an SM's shared memory, so 12 warps each keep 24 warps
// resident to cover the float64 and shared-memory latency (measured at 50,000
// blocks of 141: 256 threads 58.9 ms, 384 57.8 ms, 512 86 ms, where the
// registers allow one CTA per SM)
constexpr int kPredCta = 384;

__global__ void __launch_bounds__(kPredCta) k_pred_cta(PredArgs A) {
  extern __shared__ double smem[];
  PredPrm* prm = (PredPrm*)smem;
  pred_params(A, prm);
  double* sm = smem + (sizeof(PredPrm) + 7) / 8;
  for (int64_t b = blockIdx.x; b < A.nblk; b += gridDim.x) {
    pred_block<kPredCta>(A, prm, b, sm);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// sparse triangular solve  U_pp^T X = R
// ---------------------------------------------------------------------------
struct JsArgs {
  int64_t npred, nobs;
  int k, ldnbr, nrhs;
  const int32_t* nbr;
  const double* acol;
  const double* R;
  double* X;
  int* ready;
  unsigned* counter;
  unsigned* progress;    // rows published so far
  int32_t* info;
  unsigned spin_limit;   // polls without progress anywhere before a wait gives up
  int skip_ready_row0;   // test aid: row 0 never publishes, its dependants' waits run out
};

// One CTA per row at a time, rows claimed in order by an atomic counter (a
// row depends only on rows claimed before it, so every awaited row is held
// by a running CTA).  The row's earlier-prediction neighbours and their
// coefficients go to shared memory, one thread waits per dependency, then
// the threads split the right-hand sides; each right-hand side is the same
// sum in the same order as a one-thread solve.  A wait gives up when neither
// its row nor any other row has been published for spin_limit polls (a
// stall, not a long dependency chain: a row's time grows with nrhs).
__global__ void k_joint_solve(JsArgs A) {
  extern __shared__ double js_sm[];
  double* s_a = js_sm;                              // [k] coefficients
  int* s_p = (int*)(js_sm + (A.k > 0 ? A.k : 1));   // [k] earlier rows
  __shared__ long long s_c;
  __shared__ int s_np;
  const int K = A.k + 1;
  while (true) {
    if (threadIdx.x == 0) s_c = (long long)atomicAdd(A.counter, 1u);
    __syncthreads();
    const int64_t c = s_c;
    if (c >= A.npred) break;
    const double* ac = A.acol + c * (int64_t)K;
    if (threadIdx.x == 0) {
      int np = 0;
      for (int i = 0; i < A.k; ++i) {
        const int64_t ix = A.nbr[c * (int64_t)A.ldnbr + i];
        if (ix < 0 || ix < A.nobs) continue;  // absent slot or observation
        s_p[np] = (int)(ix - A.nobs);         // an earlier prediction row
        s_a[np] = ac[i];
        ++np;
      }
      s_np = np;
    }
    __syncthreads();
    const int np = s_np;
    for (int j = threadIdx.x; j < np; j += blockDim.x) {
      const int p = s_p[j];
      unsigned it = 0, seen = ld_acquire_u32(A.progress);
      while (ld_acquire_s32(A.ready + p) == 0) {
        if (++it > A.spin_limit) {
          const unsigned now = ld_acquire_u32(A.progress);
          if (now != seen) {
            seen = now;
            it = 0;
            continue;
          }
          set_error(A.info + SV_INFO_STATUS, SV_ETIMEOUT);
          atomicCAS(A.info + SV_INFO_BLOCK, -1, (int)c);
          break;
        }
      }
    }
    __syncthreads();
    const double aK = ac[K - 1];
    for (int r = threadIdx.x; r < A.nrhs; r += blockDim.x) {
      double v = A.R[c * (int64_t)A.nrhs + r];
#pragma unroll 4
      for (int j = 0; j < np; ++j) v -= s_a[j] * __ldcg(A.X + (int64_t)s_p[j] * A.nrhs + r);
      A.X[c * (int64_t)A.nrhs + r] = v / aK;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0 && !(A.skip_ready_row0 && c == 0)) {
      st_release_s32(A.ready + c, 1);
      atomicAdd(A.progress, 1u);
    }
  }
}

// ---------------------------------------------------------------------------
// diag((U_pp U_pp^T)^-1): rows of S = U_pp^-T against identity columns
// ---------------------------------------------------------------------------
struct JvArgs {
  int64_t npred, nobs, row0;  // panel: identity columns row0 .. row0 + w - 1
  int k, ldnbr, w;
  const int32_t* nbr;
  const double* acol;
  double* S;        // rows row0 .. npred-1 of the panel, row stride w
  double* var;      // += the panel's sum of squares of each row
  int* ready;
  unsigned* counter;
  unsigned* progress;
  int32_t* info;
  unsigned spin_limit;
};

// Row c of S = U_pp^-T restricted to the panel's columns: the recurrence of
// k_joint_solve with the identity as right-hand side, S_cr = (delta(c, row0
// + r) - sum_j a_j S_{p_j r}) / a_K.  S is lower triangular, so rows before
// row0 are zero in the panel (never formed, their dependencies skipped) and
// row c is zero beyond column c - row0 (never formed; a dependency p is read
// only where r <= p - row0).  The row's sum of squares is added to var[c].
__global__ void k_joint_inv_rows(JvArgs A) {
  extern __shared__ double jv_sm[];
  double* s_a = jv_sm;
  int* s_p = (int*)(jv_sm + (A.k > 0 ? A.k : 1));
  __shared__ long long s_c;
  __shared__ int s_np;
  __shared__ double s_red[32];
  const int K = A.k + 1;
  while (true) {
    if (threadIdx.x == 0) s_c = A.row0 + (long long)atomicAdd(A.counter, 1u);
    __syncthreads();
    const int64_t c = s_c;
    if (c >= A.npred) break;
    const double* ac = A.acol + c * (int64_t)K;
    if (threadIdx.x == 0) {
      int np = 0;
      for (int i = 0; i < A.k; ++i) {
        const int64_t ix = A.nbr[c * (int64_t)A.ldnbr + i];
        if (ix < 0 || ix < A.nobs || ix - A.nobs < A.row0) continue;  // zero in this panel
        s_p[np] = (int)(ix - A.nobs);
        s_a[np] = ac[i];
        ++np;
      }
      s_np = np;
    }
    __syncthreads();
    const int np = s_np;
    for (int j = threadIdx.x; j < np; j += blockDim.x) {
      const int p = s_p[j];
      unsigned it = 0, seen = ld_acquire_u32(A.progress);
      while (ld_acquire_s32(A.ready + p) == 0) {
        if (++it > A.spin_limit) {
          const unsigned now = ld_acquire_u32(A.progress);
          if (now != seen) {
            seen = now;
            it = 0;
            continue;
          }
          set_error(A.info + SV_INFO_STATUS, SV_ETIMEOUT);
          atomicCAS(A.info + SV_INFO_BLOCK, -1, (int)c);
          break;
        }
      }
    }
    __syncthreads();
    const double aK = ac[K - 1];
    const int64_t own = c - A.row0;
    const int64_t lim = own < A.w - 1 ? own : A.w - 1;
    double sq = 0.0;
    for (int64_t r = threadIdx.x; r <= lim; r += blockDim.x) {
      double v = (r == own) ? 1.0 : 0.0;
      for (int j = 0; j < np; ++j) {
        const int64_t pr = s_p[j] - A.row0;
        if (r <= pr) v -= s_a[j] * __ldcg(A.S + pr * A.w + r);
      }
      v = v / aK;
      A.S[own * A.w + r] = v;
      sq = fma(v, v, sq);
    }
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = sq;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w];
      A.var[c] += t;
      st_release_s32(A.ready + c, 1);
      atomicAdd(A.progress, 1u);
    }
  }
}

}  // namespace sv

using namespace sv;

extern "C" int sv_predict_blocks(const sv_pred_desc* D, const double* theta, const double* Xall,
                                 const int32_t* tgt, const int32_t* nbr, const double* resid,
                                 double* mean, double* var, double* acol, double* rhs, int32_t* info,
                                 sv_stream_t stream) {
  if (!D || !theta || !Xall || !tgt || !info) return SV_EINVAL;
  if (D->d < 1 || D->d > 64 || D->k < 0 || D->nblk < 0 || (D->k > 0 && (!nbr || D->ldnbr < D->k)))
    return SV_EINVAL;
  if (!(D->nu > 0.0)) return SV_EINVAL;
  const int closed = matern_closed_code(D->nu);
  if (!D->general && closed < 0) return SV_EINVAL;
  if (D->matern_table && (!D->general || !mtab_ok(D->nu))) return SV_EINVAL;
  if (D->nobs > 0 && !resid && (mean || rhs)) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  if (D->nblk == 0) return SV_OK;
  PredArgs A;
  A.theta = theta;
  A.Xall = Xall;
  A.tgt = tgt;
  A.nbr = nbr;
  A.resid = resid;
  A.mean = mean;
  A.var = var;
  A.acol = acol;
  A.rhs = rhs;
  A.info = info;
  A.nobs = D->nobs;
  A.nblk = D->nblk;
  A.d = D->d;
  A.k = D->k;
  A.ldnbr = D->ldnbr;
  A.closed = D->general ? -1 : closed;
  A.target_nugget = D->target_nugget;
  A.nu = D->nu;
  A.tab = D->matern_table;
  // the float32 part of the table (built where the nu has one)
  A.ftab = (D->matern_table && ftab_ok(D->nu)) ? (const float4*)(D->matern_table + kMtabMaxDoubles) : nullptr;
  if (D->precision < 0 || D->precision > 1) return SV_EINVAL;
  A.split = (D->precision == 1 && (A.closed >= 0 || A.ftab)) ? 1 : 0;
  A.rho_min = D->split_rho_min > 0.0 ? D->split_rho_min : 1e-4;
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t prm = (sizeof(PredPrm) + 7) / 8 * 8;
  const int nsm = sv_num_sms();
  if (D->k + 1 <= 32) {
    A.kt = 32;
    const size_t team = sizeof(double) * pred_team_doubles(32, D->d);
    int wpc = 8;
    while (wpc > 1 && prm + wpc * team > (size_t)maxsm) --wpc;
    const size_t smem = prm + wpc * team;
    if (smem > (size_t)maxsm) return SV_EINVAL;
    SV_CUDA_TRY(cudaFuncSetAttribute(k_pred_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int64_t grid = (D->nblk + wpc - 1) / wpc;
    if (grid > 64LL * nsm) grid = 64LL * nsm;
    k_pred_warp<<<(unsigned)grid, 32 * wpc, smem, st>>>(A);
  } else {
    A.kt = D->k + 1;
    const size_t smem = prm + sizeof(double) * pred_team_doubles(A.kt, D->d);
    if (smem > (size_t)maxsm) return SV_EINVAL;
    SV_CUDA_TRY(cudaFuncSetAttribute(k_pred_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int64_t grid = D->nblk;
    if (grid > 16LL * nsm) grid = 16LL * nsm;
    k_pred_cta<<<(unsigned)grid, kPredCta, smem, st>>>(A);
  }
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" size_t sv_joint_solve_workspace_bytes(int64_t npred) {
  return 256 + ((sizeof(int) * (size_t)(npred > 0 ? npred : 1) + 255) & ~(size_t)255);
}

static int joint_solve(int64_t npred, int64_t nobs, int32_t k, int32_t ldnbr, const int32_t* nbr,
                       const double* acol, const double* R, int32_t nrhs, double* X, int32_t* info,
                       void* workspace, size_t workspace_bytes, int32_t flags, sv_stream_t stream) {
  if (npred < 0 || nobs < 0 || k < 0 || k > 4096 || nrhs < 1 || !info || flags < 0 || flags > 1)
    return SV_EINVAL;
  if (npred > 0 && (!acol || !R || !X || (k > 0 && (!nbr || ldnbr < k)))) return SV_EINVAL;
  if (npred > 0x7fffffffLL) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  if (npred == 0) return SV_OK;
  if (!workspace || workspace_bytes < sv_joint_solve_workspace_bytes(npred)) return SV_ENOSPC;
  unsigned* counter = (unsigned*)workspace;
  unsigned* progress = counter + 1;
  int* ready = (int*)((char*)workspace + 256);
  SV_CUDA_TRY(cudaMemsetAsync(workspace, 0, sv_joint_solve_workspace_bytes(npred), st));
  JsArgs A;
  A.npred = npred;
  A.nobs = nobs;
  A.k = k;
  A.ldnbr = ldnbr;
  A.nrhs = nrhs;
  A.nbr = nbr;
  A.acol = acol;
  A.R = R;
  A.X = X;
  A.ready = ready;
  A.counter = counter;
  A.progress = progress;
  A.info = info;
  A.skip_ready_row0 = flags & 1;
  A.spin_limit = (flags & 1) ? SV_SPIN_LIMIT_TEST : SV_SPIN_LIMIT;
  const int nsm = sv_num_sms();
  // threads per row: the right-hand sides, rounded to whole warps, at most 256
  int tpb = ((nrhs + 31) / 32) * 32;
  if (tpb > 256) tpb = 256;
  const size_t smem = (size_t)(k > 0 ? k : 1) * (sizeof(double) + sizeof(int)) + 8;
  int per_sm = 0;
  SV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_joint_solve, tpb, smem));
  if (per_sm < 1) return SV_EINVAL;
  int64_t grid = (int64_t)per_sm * nsm;
  if (grid > npred) grid = npred;
  k_joint_solve<<<(unsigned)grid, tpb, smem, st>>>(A);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" int sv_joint_solve(int64_t npred, int64_t nobs, int32_t k, int32_t ldnbr,
                              const int32_t* nbr, const double* acol, const double* R, int32_t nrhs,
                              double* X, int32_t* info, void* workspace, size_t workspace_bytes,
                              sv_stream_t stream) {
  return joint_solve(npred, nobs, k, ldnbr, nbr, acol, R, nrhs, X, info, workspace, workspace_bytes,
                     0, stream);
}

extern "C" int sv_joint_solve_flags(int64_t npred, int64_t nobs, int32_t k, int32_t ldnbr,
                                    const int32_t* nbr, const double* acol, const double* R,
                                    int32_t nrhs, double* X, int32_t* info, void* workspace,
                                    size_t workspace_bytes, int32_t flags, sv_stream_t stream) {
  return joint_solve(npred, nobs, k, ldnbr, nbr, acol, R, nrhs, X, info, workspace, workspace_bytes,
                     flags, stream);
}

extern "C" int sv_joint_var_diag(int64_t npred, int64_t nobs, int32_t k, int32_t ldnbr,
                                 const int32_t* nbr, const double* acol, double* var, int32_t* info,
                                 void* workspace, size_t workspace_bytes, double* panel,
                                 size_t panel_bytes, sv_stream_t stream) {
  if (npred < 0 || nobs < 0 || k < 0 || k > 4096 || !info) return SV_EINVAL;
  if (npred > 0 && (!acol || !var || !panel || (k > 0 && (!nbr || ldnbr < k)))) return SV_EINVAL;
  if (npred > 0x7fffffffLL) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  if (npred == 0) return SV_OK;
  if (!workspace || workspace_bytes < sv_joint_solve_workspace_bytes(npred)) return SV_ENOSPC;
  const int64_t pd = (int64_t)(panel_bytes / sizeof(double));
  if (pd < npred) return SV_ENOSPC;  // one column of all rows at least
  SV_CUDA_TRY(cudaMemsetAsync(var, 0, sizeof(double) * (size_t)npred, st));
  JvArgs A;
  A.npred = npred;
  A.nobs = nobs;
  A.k = k;
  A.ldnbr = ldnbr;
  A.nbr = nbr;
  A.acol = acol;
  A.S = panel;
  A.var = var;
  A.counter = (unsigned*)workspace;
  A.progress = A.counter + 1;
  A.ready = (int*)((char*)workspace + 256);
  A.info = info;
  A.spin_limit = SV_SPIN_LIMIT;
  const int nsm = sv_num_sms();
  const size_t smem = (size_t)(k > 0 ? k : 1) * (sizeof(double) + sizeof(int)) + 8;
  for (int64_t c0 = 0; c0 < npred;) {
    // the widest panel whose rows c0 .. npred-1 fit
    const int64_t rows = npred - c0;
    int64_t w = pd / rows;
    if (w > rows) w = rows;
    if (w > 0x7fffffffLL) w = 0x7fffffffLL;
    A.row0 = c0;
    A.w = (int)w;
    SV_CUDA_TRY(cudaMemsetAsync(workspace, 0, sv_joint_solve_workspace_bytes(npred), st));
    int tpb = (int)(((w + 31) / 32) * 32);
    if (tpb > 256) tpb = 256;
    int per_sm = 0;
    SV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_joint_inv_rows, tpb, smem));
    if (per_sm < 1) return SV_EINVAL;
    int64_t grid = (int64_t)per_sm * nsm;
    if (grid > rows) grid = rows;
    k_joint_inv_rows<<<(unsigned)grid, tpb, smem, st>>>(A);
    SV_CUDA_TRY(cudaGetLastError());
    c0 += w;
  }
  return SV_OK;
}
