// Shared definitions of the likelihood kernels (float64 plain form in
// sv_loglik.cu, split-precision form in sv_loglik_split.cu).
//
// Every evaluation is a batch of independent problems (one problem for
// sv_vecchia_loglik, many for sv_vecchia_loglik_batched).  Each problem has
// its own inputs (offsets into concatenated X, y, Z), its own contiguous run
// of conditioning blocks and its own parameter vector; a per-block problem
// index lets one launch process the blocks of all problems together.
#pragma once
#include "sv_block.cuh"

namespace sv {

constexpr int kMaxD = 64;         // input dimensions supported by the block kernels
constexpr int kMaxQ = 16;         // trend columns
constexpr int kRedThreads = 256;  // reduction CTA size
constexpr int kMaxP = kMaxD + 3;

// Per-problem data in device memory: the layout from sv_prob_desc and the
// parameters derived from theta (filled by k_prob_params every evaluation).
struct ProbInfo {
  int64_t n, x_off, y_off, z_off, blk_off, nblk;
  int32_t d, q, P, estimate_nu, closed, skip;
  double nu_fixed, var_penalty, log_var_target;
  double s2, tau;
  double dg, s2t;  // s2 (1 + tau) and s2 tau
  // double-float split form: s2, s2 (1 + tau) and s2 tau as float32 (hi, lo) pairs
  float s2_hi, s2_lo, dg_hi, dg_lo, s2t_hi, s2t_lo;
  MaternMode mm;
  MaternF32 mf32;  // the split kernels' float32 Matern (code -1: the float64 pass)
  double invlam[kMaxD];
};

struct LikArgs {
  const double* X;
  const double* y;
  const double* Z;
  const int32_t* rowb;
  const int32_t* kb;
  const int32_t* nbr;
  const int32_t* chunk;
  const int32_t* bprob;   // problem of each block (nullptr: all problem 0)
  const int32_t* list;    // blocks this launch processes (nullptr: [b0, b1))
  const ProbInfo* probs;
  double* cache;          // per-block records, stride CS
  int8_t* level;
  int8_t* redo;
  int32_t* chunk_max;
  int32_t* flags;         // [0] = any block used jitter, [1] = any block flagged for redo
  int32_t* info;          // 4 words per problem
  int64_t b0, b1;         // list range (indices into list, or block ids)
  int nprob, ldnbr, CS, kt, dmax, NRmax;  // kt = team block capacity (32 or kmax+1)
  int need_grad, any_estimate_nu;
  int fixup;              // only blocks whose chunk needs a larger jitter level
  int64_t nchunk;         // length of chunk_max: chunk ids lie in [0, nchunk)
  int redo_mode;          // float64 kernel: only blocks flagged by the split kernel
  double rho_min;
  float2* xhl;            // split form: x / lambda as float32 (hi, lo) pairs
  int kcap;               // split form: largest K of the launch (<= 32)
};

// The chunk fix-up pass has work only when some block used jitter
// (flags[0]); the float64 re-evaluation only when the split kernel flagged a
// block (flags[1]).  Both flags are cleared at the start of an evaluation.
__device__ __forceinline__ bool pass_has_work(const LikArgs& A) {
  if (A.fixup && A.flags[0] == 0) return false;
  if (A.redo_mode && A.flags[1] == 0) return false;
  return true;
}

// the jitter level the chunk of block b needs (chunk-wide jitter fix-up);
// a chunk id outside [0, nchunk) has none (k_chunk_max reports it)
__device__ __forceinline__ int chunk_level(const LikArgs& A, int64_t b) {
  const int c = A.chunk[b];
  return (c >= 0 && c < A.nchunk) ? A.chunk_max[c] : 0;
}

// block id of the t-th entry handled by a launch
__device__ __forceinline__ int64_t launch_block(const LikArgs& A, int64_t t) {
  return A.list ? (int64_t)A.list[t] : t;
}
__device__ __forceinline__ int block_problem(const LikArgs& A, int64_t b) {
  return A.bprob ? A.bprob[b] : 0;
}

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
// split kernel: L's packed capacity for blocks of up to kc points (the
// launch's largest K), at least the float32 copy of R that reuses it
__host__ __device__ inline int split_lp_cap(int kc, int NR) {
  const int tri = kc * (kc + 1) / 2, r32 = (33 * NR + 1) / 2;
  const int c = tri > r32 ? tri : r32;
  return c + (c & 1);
}

// split kernel team slot (8-byte words): L (packed, pivot reciprocals on
// the diagonal), R (NR columns of 33), a, a32, u (d x 32 floats), idx, flags
__host__ __device__ inline int split_slot_doubles(int d, int NR, int kc) {
  int s = split_lp_cap(kc, NR) + 33 * NR + 32 + 16 + 16 * d + 18;
  s += ((8 - s % 16) + 16) % 16;
  return s;
}

// launch the split-precision kernels over list entries [A.b0, A.b1) (all
// K <= 32; a closed-form nu or the float32 table of a fixed nu, the blocks
// of other problems go to the float64 pass); lanes = block team width (4, 8,
// 16 or 32).
// launch_block_split: float64 factorisation and solves (the split form);
// launch_block_split_df: double-float factorisation and solves
int launch_block_split(const LikArgs& A, int lanes, cudaStream_t st);
int launch_block_split_df(const LikArgs& A, int lanes, cudaStream_t st);

// split form: fills A.xhl (X's n * d entries as float2) for every problem
int launch_split_prep(const LikArgs& A, int64_t nx, cudaStream_t st);

}  // namespace sv
