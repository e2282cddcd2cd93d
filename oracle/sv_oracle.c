/*
 * sv_oracle.c -- CPU restatement of the scaled Vecchia hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA path is
 * checked against, and the CPU port that the benchmark times beside it.  The
 * product (pyscaledvecchia_gb300) never links, loads or calls it.
 *
 * Every routine restates the algorithm of the reference implementation
 * (jdtuck/pyscaledvecchia, src/scaled_vecchia/...) in plain C, in double
 * precision, compiled with -ffp-contract=off so that sums and products are
 * IEEE-sequential (no fused multiply-add):
 *
 *   or_maximin          ordering.py:27-59 (_maximin_core), :62-73
 *   or_ordered_nn       ordering.py:76-116 (exact brute force; the reference
 *                       mixes cKDTree and cdist, whose neighbour SETS this
 *                       reproduces; ties are broken by the smaller index)
 *   or_knn_query        gp.py:253-255 (cKDTree.query of the m nearest)
 *   or_vecchia_loglik   likelihood.py:66-175 with the block kernels of
 *                       _covariance.py:111-147 (Sigma, dSigma/dlog theta),
 *                       _batch_chol :235-252 (per-block jitter), the solves
 *                       _forward_solve/_backsolve_LT :205-232
 *   or_block_records    the per-block first pass of or_vecchia_loglik
 *   or_predict_blocks   gp.py:242-277 (_predict_scaled: marginal mean/var)
 *
 * Closed-form Matern smoothness only (nu in {0.5, 1.5, 2.5}); the Bessel path
 * is restated in oracle.py with scipy.special.kv.
 *
 * Blocks are processed independently (OpenMP over blocks, as the reference's
 * Numba prange), and per-block results are summed in block order afterwards,
 * so the result does not depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SQRT3 1.7320508075688772
#define SQRT5 2.23606797749979

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_num_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

/* ------------------------------------------------------------------------ */
/* maximin ordering: ordering.py:27-59                                       */
/* ------------------------------------------------------------------------ */
void or_maximin(const double* X, int64_t n, int d, int64_t first, int64_t* order) {
  double* dist = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  order[0] = first;
  for (int64_t i = 0; i < n; i++) {
    double s = 0.0;
    for (int l = 0; l < d; l++) {
      double diff = X[i * d + l] - X[first * d + l];
      s += diff * diff;
    }
    dist[i] = sqrt(s);
  }
  dist[first] = -1.0;
  for (int64_t t = 1; t < n; t++) {
    int64_t j = 0;
    double best = -1.0;
    for (int64_t i = 0; i < n; i++) {
      if (dist[i] > best) { best = dist[i]; j = i; }
    }
    order[t] = j;
    const double* xj = X + j * d;
    for (int64_t i = 0; i < n; i++) {
      if (dist[i] < 0.0) continue;
      double s = 0.0;
      const double* xi = X + i * d;
      for (int l = 0; l < d; l++) {
        double diff = xi[l] - xj[l];
        s += diff * diff;
      }
      double dj = sqrt(s);
      if (dj < dist[i]) dist[i] = dj;
    }
    dist[j] = -1.0;
  }
  free(dist);
}

/* ------------------------------------------------------------------------ */
/* exact k nearest by (squared distance, index)                              */
/* ------------------------------------------------------------------------ */
static double sqdist(const double* a, const double* b, int d) {
  double s = 0.0;
  for (int l = 0; l < d; l++) {
    double diff = a[l] - b[l];
    s += diff * diff;
  }
  return s;
}

/* insert (dd, jj) into the ascending list (ds, js) of length cnt <= k. */
static int topk_insert(double* ds, int64_t* js, int cnt, int k, double dd, int64_t jj) {
  if (cnt == k) {
    double dl = ds[k - 1];
    int64_t jl = js[k - 1];
    if (!(dd < dl || (dd == dl && jj < jl))) return cnt;
    cnt--;
  }
  int p = cnt;
  while (p > 0 && (ds[p - 1] > dd || (ds[p - 1] == dd && js[p - 1] > jj))) {
    ds[p] = ds[p - 1];
    js[p] = js[p - 1];
    p--;
  }
  ds[p] = dd;
  js[p] = jj;
  return cnt + 1;
}

/* ordering.py:76-116: row i conditions on the min(i, m) nearest of rows < i.
 * nn is (n, m+1) int64: column 0 = i, then neighbours nearest first, -1 pad.
 * Rows 1 .. start-1 are left with only their self column (as the reference). */
void or_ordered_nn(const double* X, int64_t n, int d, int m, int64_t start, int64_t* nn) {
  for (int64_t i = 0; i < n; i++) {
    nn[i * (m + 1)] = i;
    for (int c = 1; c <= m; c++) nn[i * (m + 1) + c] = -1;
  }
  int64_t r0 = start > 1 ? start : 1;
#pragma omp parallel
  {
    double* ds = (double*)malloc(sizeof(double) * (size_t)(m + 1));
    int64_t* js = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m + 1));
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = r0; i < n; i++) {
      int k = (int)(i < m ? i : m);
      int cnt = 0;
      for (int64_t j = 0; j < i; j++) {
        double dd = sqdist(X + i * d, X + j * d, d);
        cnt = topk_insert(ds, js, cnt, k, dd, j);
      }
      for (int c = 0; c < cnt; c++) nn[i * (m + 1) + 1 + c] = js[c];
    }
    free(ds);
    free(js);
  }
}

/* gp.py:253-255: the k nearest reference rows of every query row (sorted). */
void or_knn_query(const double* Xref, int64_t nref, const double* Xq, int64_t nq, int d,
                  int k, int64_t* nb) {
#pragma omp parallel
  {
    double* ds = (double*)malloc(sizeof(double) * (size_t)(k + 1));
    int64_t* js = (int64_t*)malloc(sizeof(int64_t) * (size_t)(k + 1));
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = 0; i < nq; i++) {
      int cnt = 0;
      for (int64_t j = 0; j < nref; j++) {
        double dd = sqdist(Xq + i * d, Xref + j * d, d);
        cnt = topk_insert(ds, js, cnt, k, dd, j);
      }
      for (int c = 0; c < k; c++) nb[i * k + c] = c < cnt ? js[c] : -1;
    }
    free(ds);
    free(js);
  }
}

/* ------------------------------------------------------------------------ */
/* block kernels: _covariance.py:86-147                                      */
/* ------------------------------------------------------------------------ */
static void matern_Mg(double r, double nu, double* M, double* g) {
  if (nu == 0.5) {
    if (r > 0.0) { *M = exp(-r); *g = -exp(-r) / r; }
    else { *M = 1.0; *g = 0.0; }
  } else if (nu == 1.5) {
    double c = SQRT3 * r;
    *M = (1.0 + c) * exp(-c);
    *g = -3.0 * exp(-c);
  } else {
    double c = SQRT5 * r;
    *M = (1.0 + c + c * c / 3.0) * exp(-c);
    *g = -(5.0 / 3.0) * (1.0 + c) * exp(-c);
  }
}

/* Sigma (K,K) and, if dS != NULL, dS (P,K,K) with P = d+2, rows
 * [sigma^2, lambda_1..d, tau]  (_covariance.py:111-147). */
static void block_cov(const double* Xb, int K, int d, const double* ranges, double variance,
                      double nugget, double nu, const double* mask, double* S, double* dS) {
  int P = d + 2;
  for (int i = 0; i < K; i++) {
    for (int j = 0; j < K; j++) {
      double s = 0.0;
      for (int l = 0; l < d; l++) {
        double diff = (Xb[i * d + l] - Xb[j * d + l]) / ranges[l];
        s += diff * diff;
      }
      double r = sqrt(s), M, g;
      matern_Mg(r, nu, &M, &g);
      double nug = (i == j) ? nugget * (mask ? mask[i] : 1.0) : 0.0;
      S[i * K + j] = variance * (M + nug);
      if (dS) {
        dS[(0 * K + i) * K + j] = S[i * K + j];
        for (int l = 0; l < d; l++) {
          double diffl = (Xb[i * d + l] - Xb[j * d + l]) / ranges[l];
          dS[((1 + l) * K + i) * K + j] = -variance * g * diffl * diffl;
        }
        dS[((P - 1) * K + i) * K + j] = variance * nug;
      }
    }
  }
}

/* unblocked lower Cholesky in place (LAPACK dpotf2 criterion: a pivot that is
 * not > 0 fails).  Returns 0 on success. */
static int chol_lower(double* A, int K) {
  for (int j = 0; j < K; j++) {
    double ajj = A[j * K + j];
    for (int k = 0; k < j; k++) ajj -= A[j * K + k] * A[j * K + k];
    if (!(ajj > 0.0)) return j + 1;
    ajj = sqrt(ajj);
    A[j * K + j] = ajj;
    for (int i = j + 1; i < K; i++) {
      double s = A[i * K + j];
      for (int k = 0; k < j; k++) s -= A[i * K + k] * A[j * K + k];
      A[i * K + j] = s / ajj;
    }
  }
  for (int i = 0; i < K; i++)
    for (int j = i + 1; j < K; j++) A[i * K + j] = 0.0;
  return 0;
}

/* _batch_chol (_covariance.py:235-252) for one block: plain, then jitter
 * 10^p * mean(diag) for p = -12..-4.  Returns the level used: 0 = none,
 * 1..9 = p=-12..-4, -1 = failed.  If force_level > 0 that level is used
 * directly (reference chunk semantics: a whole chunk shares one level). */
static int chol_jitter(const double* S, double* L, int K, int force_level) {
  double scale = 0.0;
  for (int i = 0; i < K; i++) scale += S[i * K + i];
  scale /= K;
  int lv0 = force_level > 0 ? force_level : 0;
  for (int lv = lv0; lv <= 9; lv++) {
    memcpy(L, S, sizeof(double) * (size_t)K * K);
    if (lv > 0) {
      double jit = pow(10.0, (double)(lv - 13)) * scale;
      for (int i = 0; i < K; i++) L[i * K + i] += jit;
    }
    if (chol_lower(L, K) == 0) return lv;
  }
  return -1;
}

/* L x = b in place (b has nrhs columns stored as b[i*nrhs + r]) */
static void fwd_solve(const double* L, int K, double* b, int nrhs) {
  for (int r = 0; r < nrhs; r++)
    for (int i = 0; i < K; i++) {
      double acc = b[i * nrhs + r];
      for (int j = 0; j < i; j++) acc -= L[i * K + j] * b[j * nrhs + r];
      b[i * nrhs + r] = acc / L[i * K + i];
    }
}

/* L^T x = e_K  (the column a of likelihood.py:125-127) */
static void back_solve_eK(const double* L, int K, double* a) {
  for (int i = K - 1; i >= 0; i--) {
    double acc = (i == K - 1) ? 1.0 : 0.0;
    for (int j = i + 1; j < K; j++) acc -= L[j * K + i] * a[j];
    a[i] = acc / L[i * K + i];
  }
}

/* Per-block quantities (everything the two passes of likelihood.py need):
 *   out[0]            log L_KK
 *   out[1]            yt   = a . y_blk
 *   out[2 .. 2+q)     Zt   = a . Z_blk
 *   out[2+q]          zK (y part)  = (L^-1 y)_K
 *   out[3+q .. 3+2q)  zK (Z parts) = (L^-1 Z)_K
 *   then (if grad)    wK (P), wzy (P), wzZ (P*q), F (P*P, full)
 */
static int block_stride(int q, int P, int need_grad) {
  return 3 + 2 * q + (need_grad ? (2 * P + P * q + P * P) : 0);
}

typedef struct {
  const double* X; const double* y; const double* Z;
  int64_t n; int d; int q;
  const int64_t* rowb; const int32_t* kb; const int64_t* nbr; int ldnbr;
  double variance, nugget, nu; const double* ranges;
  int need_grad;
} lik_args;

static int eval_block(const lik_args* A, int64_t b, int force_level, double* out, int* level_out) {
  int d = A->d, q = A->q, P = d + 2;
  int k = A->kb[b], K = k + 1;
  double* Xb = (double*)malloc(sizeof(double) * (size_t)K * d);
  double* S = (double*)malloc(sizeof(double) * (size_t)K * K);
  double* L = (double*)malloc(sizeof(double) * (size_t)K * K);
  double* dS = A->need_grad ? (double*)malloc(sizeof(double) * (size_t)P * K * K) : NULL;
  double* a = (double*)malloc(sizeof(double) * (size_t)K);
  int nr = A->need_grad ? (P + 1 + q) : 0;
  double* R = nr ? (double*)malloc(sizeof(double) * (size_t)K * nr) : NULL;
  int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)K);
  for (int i = 0; i < k; i++) idx[i] = A->nbr[b * A->ldnbr + i];
  idx[k] = A->rowb[b];
  for (int i = 0; i < K; i++)
    for (int l = 0; l < d; l++) Xb[i * d + l] = A->X[idx[i] * d + l];
  block_cov(Xb, K, d, A->ranges, A->variance, A->nugget, A->nu, NULL, S, dS);
  int lv = chol_jitter(S, L, K, force_level);
  *level_out = lv;
  if (lv < 0) { free(Xb); free(S); free(L); free(dS); free(a); free(R); free(idx); return -1; }
  back_solve_eK(L, K, a);
  out[0] = log(L[(K - 1) * K + (K - 1)]);
  double yt = 0.0;
  for (int i = 0; i < K; i++) yt += a[i] * A->y[idx[i]];
  out[1] = yt;
  for (int c = 0; c < q; c++) {
    double s = 0.0;
    for (int i = 0; i < K; i++) s += a[i] * A->Z[idx[i] * q + c];
    out[2 + c] = s;
  }
  if (!A->need_grad) {
    /* zK from the forward solve of y and Z (likelihood.py:153-156) */
    double* v = (double*)malloc(sizeof(double) * (size_t)K * (1 + q));
    for (int i = 0; i < K; i++) {
      v[i * (1 + q)] = A->y[idx[i]];
      for (int c = 0; c < q; c++) v[i * (1 + q) + 1 + c] = A->Z[idx[i] * q + c];
    }
    fwd_solve(L, K, v, 1 + q);
    out[2 + q] = v[(K - 1) * (1 + q)];
    for (int c = 0; c < q; c++) out[3 + q + c] = v[(K - 1) * (1 + q) + 1 + c];
    free(v);
  } else {
    /* rhs = dS . a  (likelihood.py:138), then y and Z columns */
    for (int p = 0; p < P; p++)
      for (int i = 0; i < K; i++) {
        double s = 0.0;
        for (int j = 0; j < K; j++) s += dS[(p * K + i) * K + j] * a[j];
        R[i * nr + p] = s;
      }
    for (int i = 0; i < K; i++) {
      R[i * nr + P] = A->y[idx[i]];
      for (int c = 0; c < q; c++) R[i * nr + P + 1 + c] = A->Z[idx[i] * q + c];
    }
    fwd_solve(L, K, R, nr);
    out[2 + q] = R[(K - 1) * nr + P];
    for (int c = 0; c < q; c++) out[3 + q + c] = R[(K - 1) * nr + P + 1 + c];
    double* wK = out + 3 + 2 * q;
    double* wzy = wK + P;
    double* wzZ = wzy + P;
    double* F = wzZ + P * q;
    for (int p = 0; p < P; p++) {
      wK[p] = R[(K - 1) * nr + p];
      double s = 0.0;
      for (int i = 0; i < K; i++) s += R[i * nr + p] * R[i * nr + P];
      wzy[p] = s;
      for (int c = 0; c < q; c++) {
        double t = 0.0;
        for (int i = 0; i < K; i++) t += R[i * nr + p] * R[i * nr + P + 1 + c];
        wzZ[p * q + c] = t;
      }
    }
    /* fish += 0.5 (2 W W^T - wK wK^T)  (likelihood.py:141-142) */
    for (int p = 0; p < P; p++)
      for (int s2 = 0; s2 < P; s2++) {
        double t = 0.0;
        for (int i = 0; i < K; i++) t += R[i * nr + p] * R[i * nr + s2];
        F[p * P + s2] = 0.5 * (2.0 * t - wK[p] * wK[s2]);
      }
  }
  free(Xb); free(S); free(L); free(dS); free(a); free(R); free(idx);
  return 0;
}

/*
 * likelihood.py:66-175 for fixed closed-form nu.
 *   blocks: block b has self row rowb[b], kb[b] neighbours nbr[b*ldnbr + i].
 *   chunk_id (optional, may be NULL): blocks with the same id share a jitter
 *   level, as the reference's chunked _batch_chol does; NULL = per block.
 *   out: [ll, grad(P), fish(P*P), beta(q)]  (grad/fish only if need_grad)
 * Returns 0, or -1 when a block fails even with jitter (LinAlgError).
 */
int or_vecchia_loglik(const double* theta, const double* X, const double* y, const double* Z,
                      int64_t n, int d, int q, const int64_t* rowb, const int32_t* kb,
                      const int64_t* nbr, int ldnbr, int64_t nblk, const int64_t* chunk_id,
                      double nu, int need_grad, double var_penalty, double log_var_target,
                      double* out) {
  int P = d + 2;
  double ranges[256];
  if (d > 256) return -2;
  for (int l = 0; l < d; l++) ranges[l] = exp(theta[1 + l]);
  lik_args A = {X, y, Z, n, d, q, rowb, kb, nbr, ldnbr, exp(theta[0]), exp(theta[1 + d]), nu,
                ranges, need_grad};
  int cs = block_stride(q, P, need_grad);
  double* cache = (double*)malloc(sizeof(double) * (size_t)cs * (size_t)(nblk > 0 ? nblk : 1));
  int* level = (int*)malloc(sizeof(int) * (size_t)(nblk > 0 ? nblk : 1));
  int failed = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : failed)
  for (int64_t b = 0; b < nblk; b++) {
    if (eval_block(&A, b, 0, cache + b * cs, &level[b]) != 0) failed |= 1;
  }
  if (failed) { free(cache); free(level); return -1; }
  if (chunk_id) {
    /* chunk-wide jitter: every block of a chunk uses the chunk's largest level */
    int64_t b0 = 0;
    while (b0 < nblk) {
      int64_t b1 = b0;
      int mx = 0;
      while (b1 < nblk && chunk_id[b1] == chunk_id[b0]) { if (level[b1] > mx) mx = level[b1]; b1++; }
      if (mx > 0)
        for (int64_t b = b0; b < b1; b++)
          if (level[b] != mx) {
            int lv;
            if (eval_block(&A, b, mx, cache + b * cs, &lv) != 0) { free(cache); free(level); return -1; }
          }
      b0 = b1;
    }
  }
  /* GLS normal equations (likelihood.py:129-134, 146) */
  double XtX[64 * 64], Zty[64], beta[64];
  if (q > 64) { free(cache); free(level); return -2; }
  memset(XtX, 0, sizeof(XtX));
  memset(Zty, 0, sizeof(Zty));
  for (int64_t b = 0; b < nblk; b++) {
    const double* c = cache + b * cs;
    for (int i = 0; i < q; i++) {
      Zty[i] += c[2 + i] * c[1];
      for (int j = 0; j < q; j++) XtX[i * q + j] += c[2 + i] * c[2 + j];
    }
  }
  /* beta = solve(XtX + 1e-12 I, Zty) by Gaussian elimination, partial pivoting */
  if (q > 0) {
    double Mq[64 * 65];
    for (int i = 0; i < q; i++) {
      for (int j = 0; j < q; j++) Mq[i * (q + 1) + j] = XtX[i * q + j] + (i == j ? 1e-12 : 0.0);
      Mq[i * (q + 1) + q] = Zty[i];
    }
    for (int c = 0; c < q; c++) {
      int piv = c;
      for (int r = c + 1; r < q; r++)
        if (fabs(Mq[r * (q + 1) + c]) > fabs(Mq[piv * (q + 1) + c])) piv = r;
      if (piv != c)
        for (int j = 0; j <= q; j++) {
          double t = Mq[c * (q + 1) + j];
          Mq[c * (q + 1) + j] = Mq[piv * (q + 1) + j];
          Mq[piv * (q + 1) + j] = t;
        }
      for (int r = c + 1; r < q; r++) {
        double f = Mq[r * (q + 1) + c] / Mq[c * (q + 1) + c];
        for (int j = c; j <= q; j++) Mq[r * (q + 1) + j] -= f * Mq[c * (q + 1) + j];
      }
    }
    for (int c = q - 1; c >= 0; c--) {
      double s = Mq[c * (q + 1) + q];
      for (int j = c + 1; j < q; j++) s -= Mq[c * (q + 1) + j] * beta[j];
      beta[c] = s / Mq[c * (q + 1) + c];
    }
  }
  /* second pass over the cached quantities (likelihood.py:149-162) */
  double ll = -0.5 * (double)n * log(2.0 * M_PI);
  double grad[256];
  double* fish = out + 1 + P;
  memset(grad, 0, sizeof(grad));
  if (need_grad) memset(fish, 0, sizeof(double) * (size_t)P * P);
  for (int64_t b = 0; b < nblk; b++) {
    const double* c = cache + b * cs;
    double zK = c[2 + q];
    for (int i = 0; i < q; i++) zK -= c[3 + q + i] * beta[i];
    ll -= 0.5 * (2.0 * c[0] + zK * zK);
    if (!need_grad) continue;
    const double* wK = c + 3 + 2 * q;
    const double* wzy = wK + P;
    const double* wzZ = wzy + P;
    const double* F = wzZ + P * q;
    for (int p = 0; p < P; p++) {
      double wz = wzy[p];
      for (int i = 0; i < q; i++) wz -= wzZ[p * q + i] * beta[i];
      grad[p] -= 0.5 * (wK[p] * (1.0 + zK * zK) - 2.0 * zK * wz);
    }
    for (int t = 0; t < P * P; t++) fish[t] += F[t];
  }
  /* variance penalty (likelihood.py:165-171) */
  if (var_penalty > 0.0) {
    double excess = theta[0] - log_var_target;
    if (excess < 0.0) excess = 0.0;
    ll -= 0.5 * var_penalty * excess * excess;
    if (need_grad) {
      grad[0] -= var_penalty * excess;
      if (excess > 0.0) fish[0] += var_penalty;
    }
  }
  out[0] = ll;
  if (need_grad) {
    for (int p = 0; p < P; p++) out[1 + p] = grad[p];
    for (int i = 0; i < q; i++) out[1 + P + P * P + i] = beta[i];
  } else {
    for (int i = 0; i < q; i++) out[1 + i] = beta[i];
  }
  free(cache);
  free(level);
  return 0;
}

/*
 * Per-block records of blocks [b0, b1) (the first pass of or_vecchia_loglik,
 * likelihood.py:111-144): [log L_KK, a.y, a.Z(q), (L^-1 y)_K, (L^-1 Z)_K(q),
 * w_K(P), W (L^-1 y)(P), W (L^-1 Z)(P q), F(P P)] per block, the jitter search
 * starting at force_level[b - b0] (NULL: 0; the chunk-wide redo of
 * _covariance.py:235-252 passes the chunk's level), the level used in
 * level_out.  Returns the record length, or -1 when a block fails even with
 * jitter.
 */
int or_block_records(const double* theta, const double* X, const double* y, const double* Z,
                     int64_t n, int d, int q, const int64_t* rowb, const int32_t* kb,
                     const int64_t* nbr, int ldnbr, int64_t b0, int64_t b1,
                     const int32_t* force_level, double nu, int need_grad, double* records,
                     int32_t* level_out) {
  int P = d + 2;
  double ranges[256];
  if (d > 256) return -2;
  for (int l = 0; l < d; l++) ranges[l] = exp(theta[1 + l]);
  lik_args A = {X, y, Z, n, d, q, rowb, kb, nbr, ldnbr, exp(theta[0]), exp(theta[1 + d]), nu,
                ranges, need_grad};
  int cs = block_stride(q, P, need_grad);
  int failed = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : failed)
  for (int64_t b = b0; b < b1; b++) {
    int lv = 0;
    if (eval_block(&A, b, force_level ? force_level[b - b0] : 0, records + (b - b0) * cs, &lv) != 0)
      failed |= 1;
    level_out[b - b0] = lv;
  }
  return failed ? -1 : cs;
}

/*
 * gp.py:242-277 (_predict_scaled), one block per query:
 * block = [Xtr[nb[t, 0..m-1]], Xq[t]], nugget on the neighbours only,
 * mean = -a[:m].resid[nb] / a_K, var = 1 / a_K^2.
 */
int or_predict_blocks(const double* Xtr, const double* resid, const double* Xq, int64_t nq,
                      int d, int m, const int64_t* nb, const double* ranges, double variance,
                      double nugget, double nu, double* mean, double* var) {
  int K = m + 1, failed = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : failed)
  for (int64_t t = 0; t < nq; t++) {
    double* Xb = (double*)malloc(sizeof(double) * (size_t)K * d);
    double* S = (double*)malloc(sizeof(double) * (size_t)K * K);
    double* L = (double*)malloc(sizeof(double) * (size_t)K * K);
    double* a = (double*)malloc(sizeof(double) * (size_t)K);
    double* mask = (double*)malloc(sizeof(double) * (size_t)K);
    for (int i = 0; i < m; i++) {
      for (int l = 0; l < d; l++) Xb[i * d + l] = Xtr[nb[t * m + i] * d + l];
      mask[i] = 1.0;
    }
    for (int l = 0; l < d; l++) Xb[m * d + l] = Xq[t * d + l];
    mask[m] = 0.0;
    block_cov(Xb, K, d, ranges, variance, nugget, nu, mask, S, NULL);
    if (chol_jitter(S, L, K, 0) < 0) {
      failed |= 1;
    } else {
      back_solve_eK(L, K, a);
      double s = 0.0;
      for (int i = 0; i < m; i++) s += a[i] * resid[nb[t * m + i]];
      mean[t] = -s / a[m];
      var[t] = 1.0 / (a[m] * a[m]);
    }
    free(Xb); free(S); free(L); free(a); free(mask);
  }
  return failed ? -1 : 0;
}
