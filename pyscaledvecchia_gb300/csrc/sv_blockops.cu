// Block-level routines of _covariance.py exposed one by one: the covariance
// and derivative tensors of a batch of blocks (_block_cov / _block_cov_general),
// the batched Cholesky with the reference's batch-wide jitter retry
// (_batch_chol) and the batched triangular solves (_forward_solve,
// _backsolve_LT).  The fused likelihood and prediction kernels do not use
// these; they serve callers of the block-level interface.
#include "sv_common.cuh"
#include "sv_matern.cuh"

namespace sv {

struct CovArgs {
  const double* Xb;
  int64_t B;
  int K, d, P;
  double ranges[64];
  double variance, nugget, nu, log_coef, nu_p, nu_m, lc_p, lc_m, h;
  int closed, general, estimate_nu;
  const double* mask;
  double* S;
  double* dS;
};

// one thread per (b, i, j): _covariance.py:111-147 / _matern_general.py:134-179
__global__ void k_block_cov(CovArgs A) {
  const int64_t KK = (int64_t)A.K * A.K;
  const int64_t tot = A.B * KK;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / KK;
    const int r = (int)(e - b * KK);
    const int i = r / A.K, j = r - (r / A.K) * A.K;
    const double* xi = A.Xb + (b * A.K + i) * A.d;
    const double* xj = A.Xb + (b * A.K + j) * A.d;
    double s = 0.0;
    for (int l = 0; l < A.d; ++l) {
      const double df = (xi[l] - xj[l]) / A.ranges[l];
      s += df * df;
    }
    const double rr = sqrt(s);
    double M, g;
    if (A.general) {
      if (A.dS)
        matern_general_Mg(rr, A.nu, A.log_coef, M, g);
      else
        M = matern_general_M(rr, A.nu, A.log_coef), g = 0.0;
    } else {
      matern_closed(A.closed, rr, M, g);
    }
    const double nug = (i == j) ? A.nugget * (A.mask ? A.mask[b * A.K + i] : 1.0) : 0.0;
    const double sig = A.variance * (M + nug);
    A.S[e] = sig;
    if (!A.dS) continue;
    double* ds = A.dS + b * (int64_t)A.P * KK;
    ds[r] = sig;
    for (int l = 0; l < A.d; ++l) {
      const double dl = (xi[l] - xj[l]) / A.ranges[l];
      ds[(1 + l) * KK + r] = -A.variance * g * dl * dl;
    }
    int p = 1 + A.d;
    if (A.estimate_nu) {
      const double Mp = matern_general_M(rr, A.nu_p, A.lc_p);
      const double Mm = matern_general_M(rr, A.nu_m, A.lc_m);
      ds[p * KK + r] = A.variance * A.nu * ((Mp - Mm) / (2.0 * A.h));
      ++p;
    }
    ds[p * KK + r] = A.variance * nug;
  }
}

// one CTA per block: Cholesky of Sigma + 10^p mean(diag) I with the given
// level (forced >= 0) or the smallest level that succeeds (forced < 0).
__global__ void k_chol_batch(const double* S, int64_t B, int K, double* L, int8_t* level,
                             const int32_t* forced) {
  extern __shared__ double A[];  // K*K
  __shared__ int fail;
  __shared__ double scale;
  const double p10[10] = {0.0, 1e-12, 1e-11, 1e-10, 1e-9, 1e-8, 1e-7, 1e-6, 1e-5, 1e-4};
  for (int64_t b = blockIdx.x; b < B; b += gridDim.x) {
    const double* Sb = S + b * (int64_t)K * K;
    int lv0 = 0;
    if (forced) {
      lv0 = *forced;
      if (lv0 <= 0 || lv0 > 9 || level[b] == lv0) continue;  // nothing to redo
    }
    if (threadIdx.x == 0) {
      double sc = 0.0;
      for (int i = 0; i < K; ++i) sc += Sb[i * K + i];
      scale = sc / (double)K;
    }
    __syncthreads();
    int lv = lv0;
    for (; lv <= 9; ++lv) {
      for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
        const int i = e / K, j = e - (e / K) * K;
        A[e] = Sb[e] + ((i == j && lv > 0) ? p10[lv] * scale : 0.0);
      }
      if (threadIdx.x == 0) fail = 0;
      __syncthreads();
      for (int k = 0; k < K; ++k) {
        if (threadIdx.x == 0) {
          const double dkk = A[k * K + k];
          if (!(dkk > 0.0))
            fail = 1;
          else
            A[k * K + k] = sqrt(dkk);
        }
        __syncthreads();
        if (fail) break;
        const double lkk = A[k * K + k];
        for (int i = k + 1 + threadIdx.x; i < K; i += blockDim.x) A[i * K + k] /= lkk;
        __syncthreads();
        const int m = K - k - 1;
        for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
          const int i = k + 1 + t / m, j = k + 1 + t % m;
          if (j <= i) A[i * K + j] -= A[i * K + k] * A[j * K + k];
        }
        __syncthreads();
      }
      __syncthreads();
      if (!fail) break;
      __syncthreads();
      if (forced) {
        lv = 10;  // the forced level itself failed
        break;
      }
    }
    double* Lb = L + b * (int64_t)K * K;
    for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
      const int i = e / K, j = e - (e / K) * K;
      Lb[e] = (j <= i) ? A[e] : 0.0;
    }
    if (threadIdx.x == 0) level[b] = (int8_t)(lv > 9 ? 10 : lv);
    __syncthreads();
  }
}

__global__ void k_level_max(const int8_t* level, int64_t B, int32_t* out) {
  int m = 0;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < B;
       b += (int64_t)gridDim.x * blockDim.x)
    m = max(m, (int)level[b]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void k_chol_status(const int32_t* lvmax, int32_t* info) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const int m = *lvmax;
    info[SV_INFO_JITTER] = m > 9 ? 9 : m;
    if (m > 9) info[SV_INFO_STATUS] = SV_ECHOL;
  }
}

// one thread per (block, rhs column): _covariance.py:205-218 / :220-232
__global__ void k_trsm(const double* L, const double* Bm, int64_t nb, int K, int nrhs, double* X,
                       int transposed) {
  const int64_t tot = nb * nrhs;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nrhs;
    const int r = (int)(e - b * nrhs);
    const double* Lb = L + b * (int64_t)K * K;
    const double* Bb = Bm + b * (int64_t)K * nrhs;
    double* Xb = X + b * (int64_t)K * nrhs;
    if (!transposed) {
      for (int i = 0; i < K; ++i) {
        double acc = Bb[i * nrhs + r];
        for (int j = 0; j < i; ++j) acc -= Lb[i * K + j] * Xb[j * nrhs + r];
        Xb[i * nrhs + r] = acc / Lb[i * K + i];
      }
    } else {
      for (int i = K - 1; i >= 0; --i) {
        double acc = Bb[i * nrhs + r];
        for (int j = i + 1; j < K; ++j) acc -= Lb[j * K + i] * Xb[j * nrhs + r];
        Xb[i * nrhs + r] = acc / Lb[i * K + i];
      }
    }
  }
}

}  // namespace sv

using namespace sv;

extern "C" int sv_block_cov(const double* Xb, int64_t B, int32_t K, int32_t d,
                            const double* ranges_host, double variance, double nugget, double nu,
                            int32_t general, int32_t estimate_nu, double nu_fd_h,
                            const double* nug_mask, double* Sigma, double* dS, sv_stream_t stream) {
  if (B < 0 || K < 1 || d < 1 || d > 64 || !ranges_host || !(nu > 0.0)) return SV_EINVAL;
  if (B > 0 && (!Xb || !Sigma)) return SV_EINVAL;
  const int closed = matern_closed_code(nu);
  if (!general && closed < 0) return SV_EINVAL;
  if (estimate_nu && !general) return SV_EINVAL;
  if (B == 0) return SV_OK;
  CovArgs A;
  A.Xb = Xb;
  A.B = B;
  A.K = K;
  A.d = d;
  A.P = d + 2 + (estimate_nu ? 1 : 0);
  for (int l = 0; l < d; ++l) A.ranges[l] = ranges_host[l];
  A.variance = variance;
  A.nugget = nugget;
  A.nu = nu;
  A.closed = closed;
  A.general = general;
  A.estimate_nu = estimate_nu;
  A.log_coef = general ? matern_log_coef(nu) : 0.0;
  A.h = nu_fd_h;
  A.nu_p = nu + nu_fd_h;
  A.nu_m = nu - nu_fd_h;
  A.lc_p = estimate_nu ? matern_log_coef(A.nu_p) : 0.0;
  A.lc_m = estimate_nu ? matern_log_coef(A.nu_m) : 0.0;
  A.mask = nug_mask;
  A.S = Sigma;
  A.dS = dS;
  const int64_t tot = B * (int64_t)K * K;
  int64_t grid = (tot + 255) / 256;
  if (grid > 32LL * sv_num_sms()) grid = 32LL * sv_num_sms();
  k_block_cov<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(A);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" size_t sv_batch_chol_workspace_bytes(int64_t B) {
  return 256 + (((size_t)(B > 0 ? B : 1) + 255) & ~(size_t)255);
}

extern "C" int sv_batch_chol(const double* Sigma, int64_t B, int32_t K, double* L, int32_t* info,
                             void* workspace, size_t workspace_bytes, sv_stream_t stream) {
  if (B < 0 || K < 1 || !info || (B > 0 && (!Sigma || !L))) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  if (B == 0) return SV_OK;
  if (!workspace || workspace_bytes < sv_batch_chol_workspace_bytes(B)) return SV_ENOSPC;
  const size_t smem = sizeof(double) * (size_t)K * K;
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > (size_t)maxsm) return SV_EINVAL;
  int32_t* lvmax = (int32_t*)workspace;
  int8_t* level = (int8_t*)workspace + 256;
  SV_CUDA_TRY(cudaMemsetAsync(lvmax, 0, sizeof(int32_t), st));
  SV_CUDA_TRY(cudaFuncSetAttribute(k_chol_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = B;
  if (grid > 16LL * sv_num_sms()) grid = 16LL * sv_num_sms();
  const int threads = K >= 64 ? 256 : 64;
  // 1) smallest level per block  2) batch maximum  3) redo the others at it
  k_chol_batch<<<(unsigned)grid, threads, smem, st>>>(Sigma, B, K, L, level, nullptr);
  int64_t g2 = (B + 255) / 256;
  if (g2 > 4LL * sv_num_sms()) g2 = 4LL * sv_num_sms();
  k_level_max<<<(unsigned)g2, 256, 0, st>>>(level, B, lvmax);
  k_chol_batch<<<(unsigned)grid, threads, smem, st>>>(Sigma, B, K, L, level, lvmax);
  k_chol_status<<<1, 32, 0, st>>>(lvmax, info);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" int sv_forward_solve(const double* L, const double* Bm, int64_t b, int32_t K,
                                int32_t nrhs, double* Xout, sv_stream_t stream) {
  if (b < 0 || K < 1 || nrhs < 1 || (b > 0 && (!L || !Bm || !Xout))) return SV_EINVAL;
  if (b == 0) return SV_OK;
  const int64_t tot = b * nrhs;
  int64_t grid = (tot + 127) / 128;
  if (grid > 32LL * sv_num_sms()) grid = 32LL * sv_num_sms();
  k_trsm<<<(unsigned)grid, 128, 0, (cudaStream_t)stream>>>(L, Bm, b, K, nrhs, Xout, 0);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" int sv_backsolve_LT(const double* L, const double* Bm, int64_t b, int32_t K,
                               int32_t nrhs, double* Xout, sv_stream_t stream) {
  if (b < 0 || K < 1 || nrhs < 1 || (b > 0 && (!L || !Bm || !Xout))) return SV_EINVAL;
  if (b == 0) return SV_OK;
  const int64_t tot = b * nrhs;
  int64_t grid = (tot + 127) / 128;
  if (grid > 32LL * sv_num_sms()) grid = 32LL * sv_num_sms();
  k_trsm<<<(unsigned)grid, 128, 0, (cudaStream_t)stream>>>(L, Bm, b, K, nrhs, Xout, 1);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}
