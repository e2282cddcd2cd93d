// Shared definitions of the likelihood kernels (float64 plain form in
// sv_loglik.cu, split-precision form in sv_loglik_split.cu).
#pragma once
#include "sv_block.cuh"

namespace sv {

constexpr int kMaxD = 64;         // input dimensions supported by the block kernels
constexpr int kMaxQ = 16;         // trend columns
constexpr int kRedThreads = 256;  // reduction CTA size
constexpr int kMaxP = kMaxD + 3;

struct LikArgs {
  const double* X;
  const double* y;
  const double* Z;
  const int32_t* rowb;
  const int32_t* kb;
  const int32_t* nbr;
  const int32_t* chunk;
  const double* theta;
  double* cache;
  int8_t* level;
  int32_t* chunk_max;
  int32_t* flags;  // [0] = any block used jitter
  int32_t* info;
  int64_t n, b0, b1;
  int d, q, ldnbr, P, NR, CS, kt;  // kt = team block capacity (32 or kmax+1)
  int need_grad, estimate_nu, closed;
  double nu_fixed, nu_fd_h;
  int fixup;
  // split form: blocks whose smallest pivot ratio L_kk^2 / Sigma_kk falls
  // below rho_min are flagged in redo[] and re-evaluated in float64
  int8_t* redo;
  double rho_min;
  int redo_mode;  // float64 kernel: only blocks with redo[b] != 0
  // split form: scaled coordinates x / lambda as float32 (hi, lo) pairs
  float2* xhl;
};

// 10^p for jitter level lv = p + 13, p = -12..-4 (_covariance.py:247-249)
__device__ __forceinline__ double jitter_pow10(int lv) {
  switch (lv) {
    case 1: return 1e-12;
    case 2: return 1e-11;
    case 3: return 1e-10;
    case 4: return 1e-9;
    case 5: return 1e-8;
    case 6: return 1e-7;
    case 7: return 1e-6;
    case 8: return 1e-5;
    default: return 1e-4;
  }
}

// per-CTA parameter block in shared memory
struct PrmSmem {
  double s2, tau;
  MaternMode mm;
  double invlam[kMaxD];
};

__device__ inline void load_params(const LikArgs& A, PrmSmem* prm) {
  if (threadIdx.x == 0) {
    const int d = A.d;
    prm->s2 = exp(A.theta[0]);
    double nu = A.nu_fixed;
    if (A.estimate_nu) {
      nu = exp(A.theta[1 + d]);
      prm->tau = exp(A.theta[2 + d]);
    } else {
      prm->tau = exp(A.theta[1 + d]);
    }
    MaternMode mm;
    mm.closed = A.estimate_nu ? -1 : A.closed;
    mm.estimate_nu = A.estimate_nu;
    mm.nu = nu;
    mm.log_coef = (mm.closed < 0) ? matern_log_coef(nu) : 0.0;
    mm.nu_p = nu + A.nu_fd_h;
    mm.nu_m = nu - A.nu_fd_h;
    mm.lc_p = A.estimate_nu ? matern_log_coef(mm.nu_p) : 0.0;
    mm.lc_m = A.estimate_nu ? matern_log_coef(mm.nu_m) : 0.0;
    mm.inv2h = 1.0 / (2.0 * A.nu_fd_h);
    prm->mm = mm;
  }
  for (int l = threadIdx.x; l < A.d; l += blockDim.x) prm->invlam[l] = exp(-A.theta[1 + l]);
  __syncthreads();
}


// block record layout (doubles): [L_KK, a.y, a.Z(q), (L^-1 y)_K, (L^-1 Z)_K(q),
// w_K(P), W(L^-1 y)(P), W(L^-1 Z)(P q), F(P(P+1)/2) packed lower]
__host__ __device__ inline int record_stride(int q, int P, int need_grad) {
  return 3 + 2 * q + (need_grad ? (2 * P + P * q + P * (P + 1) / 2) : 0);
}

// split-precision kernel: per-block shared-memory slot (doubles), K <= 32:
// L packed by columns (528) | R (NR columns, stride 33) | a, invd (64) |
// a as float32 (16) | coordinates float32 (16 d) | indices + flags (18);
// the stride is kept = 8 (mod 16) doubles so that two 8-lane teams in a
// half-warp fall on disjoint banks
__host__ __device__ inline int split_slot_doubles(int d, int NR) {
  int s = 528 + 33 * NR + 64 + 16 + 16 * d + 18;
  s += ((8 - s % 16) + 16) % 16;
  return s;
}

// launches the split-precision kernel over blocks [A.b0, A.b1) (all K <= 32,
// closed-form nu); lanes = block team width (4, 8, 16 or 32)
int launch_block_split(const LikArgs& A, int lanes, cudaStream_t st);

// split form: fills A.xhl (n * d float2) from X and theta
int launch_split_prep(const LikArgs& A, cudaStream_t st);

}  // namespace sv
