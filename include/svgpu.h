/*
 * svgpu.h -- C ABI of libsvgpu.so, the sm_103a (GB300) implementation of the
 * scaled Vecchia hot path (Katzfuss, Guinness & Lawrence 2020/22).
 *
 * Every entry point is a plain C function over caller-owned DEVICE buffers
 * (pointers + sizes; sv_pack_blocks also takes host arrays where the device
 * reads host memory), stream-ordered on `stream` (NULL = legacy default
 * stream).  Nothing here allocates device memory: each call that needs
 * scratch memory takes a caller-provided workspace whose size is returned by
 * the matching *_workspace_bytes query.  Errors detected on the device (a
 * failed block Cholesky, a wait that ran out of its iteration limit) are
 * written to a caller-provided device `info` word array and become visible
 * once the stream is synchronised; launch/argument errors are returned
 * directly.  No C++ exception crosses this boundary.
 *
 * Each declaration names the reference function (jdtuck/pyscaledvecchia,
 * paths relative to src/scaled_vecchia/) whose behaviour it reproduces.
 */
#ifndef SVGPU_H
#define SVGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* sv_stream_t; /* identical to cudaStream_t */

/* status codes (returned, and in info[0]) */
#define SV_OK 0
#define SV_EINVAL 1   /* bad argument / unsupported size -> ValueError */
#define SV_ECHOL 2    /* block Cholesky failed even with jitter -> LinAlgError */
#define SV_ETIMEOUT 3 /* a bounded device wait ran out -> RuntimeError */
#define SV_ECUDA 4    /* CUDA runtime error (see sv_last_cuda_error) */
#define SV_ENOSPC 5   /* workspace too small */

/* layout of the device `info` array used by the calls below (int32[4]) */
#define SV_INFO_STATUS 0     /* SV_* status of the device work */
#define SV_INFO_BLOCK 1      /* first failing block / row, or -1 */
#define SV_INFO_JITTER 2     /* largest jitter level used (0 = none, 1..9 = 1e-12..1e-4) */
#define SV_INFO_AUX 3        /* split form: blocks re-evaluated in float64 */

/* version of this interface: sv_abi_version() returns it; bumped whenever a
 * signature or a structure layout changes */
#define SV_ABI_VERSION 4

const char* sv_status_string(int status);
int sv_abi_version(void);
/* last cudaError_t recorded by a call that returned SV_ECUDA */
int sv_last_cuda_error(void);

/* ---------------------------------------------------------------------- */
/* Ordering (ordering.py)                                                  */
/* ---------------------------------------------------------------------- */

/* Exact maximin ordering: replaces ordering.py:27-59 (_maximin_core; the
 * caller supplies `first` as ordering.py:72 computes it).  X is (n, d)
 * row-major float64; order receives n int64 indices.  Bit-exact: IEEE
 * sequential squared distances without FMA, correctly rounded sqrt, strict
 * '>' argmax with the smallest index winning ties, strict '<' updates. */
size_t sv_maximin_workspace_bytes(int64_t n, int32_t d);
int sv_maximin_order(const double* X, int64_t n, int32_t d, int64_t first, int64_t* order,
                     int32_t* info, void* workspace, size_t workspace_bytes, sv_stream_t stream);
/* The same with test aids that give the same order by other routes: bit 0
 * ranks every pivot choice by exact roots, bit 1 takes pivots by the tie
 * pass only, bit 2 runs the grid form even when one cluster would hold X,
 * bit 4 runs the tree form (not with bit 2).  Bit 3 (with bit 2) tests the
 * grid barrier's bounded wait: one CTA does not arrive at the first barrier
 * and every wait is limited to 4096 polls, so all waits run out, every CTA
 * returns and info[0] = SV_ETIMEOUT.  The workspace of a call with flags is
 * sv_maximin_workspace_bytes_flags(n, d, flags) bytes. */
int sv_maximin_order_flags(const double* X, int64_t n, int32_t d, int64_t first, int64_t* order,
                           int32_t* info, void* workspace, size_t workspace_bytes, int32_t flags,
                           sv_stream_t stream);
size_t sv_maximin_workspace_bytes_flags(int64_t n, int32_t d, int32_t flags);
/* largest n sv_maximin_order accepts (int32 row indices): rows beyond the
 * shared memory of all SMs (sv_maximin_grid_max_rows) take the tree form,
 * whose workspace grows with n (about 260 bytes per row at d = 10) */
int64_t sv_maximin_max_rows(int32_t d);
/* largest n the grid form holds for dimension d (rows in the shared memory
 * of all SMs) */
int64_t sv_maximin_grid_max_rows(int32_t d);

/* Ordered nearest neighbours: replaces ordering.py:76-116 (find_ordered_nn).
 * nn is (n, m+1) int64: column 0 = row index, columns 1..min(i,m) the nearest
 * rows j < i (nearest first, ties to the smaller index), -1 padding; rows
 * 1..start-1 keep only their self column, as in the reference. */
size_t sv_ordered_knn_workspace_bytes(int64_t n, int32_t d);
int sv_ordered_knn(const double* X, int64_t n, int32_t d, int32_t m, int64_t start, int64_t* nn,
                   int32_t* info, void* workspace, size_t workspace_bytes, sv_stream_t stream);

/* k nearest reference rows of every query row, sorted nearest first:
 * replaces gp.py:253-255 (cKDTree(X_tr / lambda).query(X_star / lambda, k=m)).
 * nb is (nq, k) int64. */
size_t sv_knn_query_workspace_bytes(int64_t nref, int64_t nq, int32_t d);
int sv_knn_query(const double* Xref, int64_t nref, const double* Xq, int64_t nq, int32_t d,
                 int32_t k, int64_t* nb, int32_t* info, void* workspace, size_t workspace_bytes,
                 sv_stream_t stream);

/* Batched rebuild of many problems' Vecchia structure: gp.py:182-191 (the
 * fit's `rebuild`: Xs = X_e / ranges, maximin_order(Xs), find_ordered_nn of
 * Xs[order], _nn_groups, X_e/y_e/Z_e[order]) for every listed problem in one
 * call.  No counterpart in the reference, which rebuilds one fit at a time;
 * the per-problem results are the reference's own (bit-exact ordering and
 * neighbour sets).  Problem p reads rows from Xe/ye/Ze at its *e_off offsets
 * and writes the reordered rows to X/y/Z at x_off/y_off/z_off, its maximin
 * order (indices into its own rows) to order at its running row offset
 * (problems in call order; order may be NULL), and row i's min(i, m)
 * neighbours, nearest first, to nbr[(blk_off + i) * ldnbr ..], -1 padded.
 * probs and ranges (nprob x dmax: exp(log lambda) as the caller computed it)
 * are HOST arrays; the library stages them into the workspace.  A problem
 * must fit one thread-block cluster: n <= sv_maximin_cluster_max_rows(d).
 * info is device int32[4 * nprob]. */
typedef struct sv_reorder_prob {
  int64_t n;
  int64_t xe_off, ye_off, ze_off;  /* source rows (any order)                */
  int64_t x_off, y_off, z_off;     /* destination rows (maximin order)       */
  int64_t blk_off;                 /* likelihood block of row 0              */
  int64_t first;                   /* first row of the ordering (ordering.py:72) */
  int32_t d, q, m;
  int32_t flags;                   /* test aids, same orders by other routes: bit 0
                                      ranks every maximin pivot choice by exact
                                      roots, bit 1 takes one pivot per pass by a
                                      full scan */
} sv_reorder_prob;

typedef struct sv_reorder_desc {
  int64_t nprob;
  int32_t dmax;   /* row stride of ranges                                   */
  int32_t ldnbr;  /* row stride of nbr (>= every m)                          */
} sv_reorder_desc;

int64_t sv_maximin_cluster_max_rows(int32_t d);
size_t sv_reorder_batched_workspace_bytes(const sv_reorder_desc* desc, const sv_reorder_prob* probs);
int sv_reorder_batched(const sv_reorder_desc* desc, const sv_reorder_prob* probs,
                       const double* ranges, const double* Xe, const double* ye, const double* Ze,
                       double* X, double* y, double* Z, int32_t* nbr, int64_t* order,
                       int32_t* info, void* workspace, size_t workspace_bytes,
                       sv_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Likelihood (likelihood.py)                                              */
/* ---------------------------------------------------------------------- */

typedef struct sv_loglik_desc {
  int64_t n;            /* rows of X, y, Z (Vecchia order)                      */
  int64_t nblk;         /* conditioning blocks                                  */
  int64_t nblk_warp;    /* leading blocks with k+1 <= 32 (warp kernel);        */
                        /* the rest (k+1 > 32) go to the CTA kernel            */
  int32_t d;            /* input dimension                                      */
  int32_t q;            /* trend columns (0 = none)                             */
  int32_t ldnbr;        /* row stride of nbr                                    */
  int32_t kmax;         /* largest conditioning-set size k                      */
  int32_t need_grad;    /* 1: score and Fisher information too                 */
  int32_t estimate_nu;  /* 1: theta = [log s2, log lam.., log nu, log tau]     */
  int32_t chunked;      /* 1: chunk[] gives the jitter-sharing chunk of a block */
  int32_t precision;    /* 0 = float64 throughout; 1 = split: float32         */
                        /*   distances, Matern assembly, dSigma.a and Gram     */
                        /*   products, float64 LDL^T, solves, log-determinant  */
                        /*   and sums; 2 = split with a double-float (float32  */
                        /*   pair) factorisation and solves.  The split forms  */
                        /*   take k+1 <= 32 blocks of a closed-form nu or of   */
                        /*   a general nu with float32 tables (0 < nu <= 8,    */
                        /*   at least 1e-3 from an integer; an estimated nu    */
                        /*   at theta, with nu +- 1e-3 too); other blocks run  */
                        /*   in float64                                        */
  int32_t team_lanes;   /* split forms: lanes per block (4, 8, 16, 32; 0 = 16) */
  double split_rho_min; /* split forms: blocks whose smallest pivot ratio     */
                        /*   L_kk^2 / Sigma_kk is below this (0 = 1e-4) are    */
                        /*   re-evaluated in float64; info[SV_INFO_AUX] counts */
  double nu;            /* fixed smoothness (estimate_nu = 0)                   */
  double var_penalty;   /* likelihood.py:165-171                                */
  double log_var_target;
} sv_loglik_desc;

/* Profile Vecchia log-likelihood, score and Fisher information with GLS
 * profiling of the trend: replaces likelihood.py:66-175
 * (vecchia_profile_loglik), including _block_cov / _block_cov_general,
 * _batch_chol, _backsolve_LT and _forward_solve on its path.
 *   theta : device float64[P], P = d+2 (+1 if estimate_nu)
 *   block b: self row rowb[b], neighbours nbr[b*ldnbr + 0..kb[b]-1]
 *   chunk : device int32[nblk] chunk ids in [0, nblk) (desc->chunked) or
 *           NULL; an id outside that range sets info[SV_INFO_STATUS] to
 *           SV_EINVAL when the chunk table is read (some block needed jitter)
 *   out   : device float64[1 + P + P*P + q] = ll, grad, fish (row-major), beta
 *   info  : device int32[4] (SV_INFO_*) */
/* The block table of sv_vecchia_loglik from the groups of _nn_groups
 * (ordering.py:119-127), packed on the device: group g's rows (int64, count
 * of them) with k neighbour rows each (int64, count x k row-major) become
 * blocks out_off .. out_off+count-1: rowb = row, kb = k, nbr = the
 * neighbours then -1 up to ldnbr.  An index outside [0, n) sets *bad (device
 * int32, cleared first) and is written as 0.  rows and nb are device memory,
 * or ordinary host memory when sv_device_reads_host_memory reports 1 (the
 * caller keeps it alive until the stream has passed the packing). */
typedef struct sv_pack_group {
  const int64_t* rows;
  const int64_t* nb;
  int64_t count, out_off;
  int32_t k, pad;
} sv_pack_group;
int sv_pack_blocks(const sv_pack_group* groups, int32_t ngroups, int64_t n, int32_t ldnbr,
                   int32_t* rowb, int32_t* kb, int32_t* nbr, int32_t* bad, sv_stream_t stream);

/* Jitter-sharing chunk of every block (the chunks of _covariance.py:255-259
 * that likelihood.py:114 factorises together): block r of a group, at
 * out_off + r in the block table, gets chunk base + r / step, where step is
 * _chunks' row count and base the chunks of the groups before it. */
typedef struct sv_chunk_group {
  int64_t count, out_off;
  int32_t base, step;
} sv_chunk_group;
int sv_chunk_ids(const sv_chunk_group* groups, int32_t ngroups, int32_t* ids, sv_stream_t stream);

size_t sv_loglik_workspace_bytes(const sv_loglik_desc* desc);
int sv_vecchia_loglik(const sv_loglik_desc* desc, const double* theta, const double* X,
                      const double* y, const double* Z, const int32_t* rowb, const int32_t* kb,
                      const int32_t* nbr, const int32_t* chunk, double* out, int32_t* info,
                      void* workspace, size_t workspace_bytes, sv_stream_t stream);

/* Sharded form of sv_vecchia_loglik: one problem's blocks split across
 * several GPUs (one process each; no counterpart in the reference, which
 * evaluates on one host; the arithmetic is likelihood.py:66-175 unchanged).
 * The evaluation's reduction partitions (the `parts` of
 * sv_loglik_shard_sizes: contiguous runs of blocks, fixed by nblk) are
 * divided among the ranks: a rank owns partitions [part_begin, part_end)
 * and every rank holds the whole of X, y, Z and the block table.  Four
 * stages with three exchanges between them, each an element-wise
 * all-reduce over the ranks:
 *   stage 1: blocks of the rank's partitions; their chunks' jitter levels
 *            into chunk_max (int32[nblk], zeroed first)  -> all-reduce MAX
 *   stage 2: chunk-wide jitter fix-up of the rank's blocks from the exchanged
 *            chunk_max, split-form re-evaluation, pass-1 partial sums of its
 *            partitions into rows [part_begin, part_end) of part1
 *            (double[parts][part1_len]; the other rows must be 0)  -> SUM
 *   stage 3: XtX, Zty, Fisher and beta from all of part1; pass-2 partial sums
 *            of its partitions into part2 (double[parts][part2_len], other
 *            rows 0)                                            -> SUM
 *   stage 4: ll, score, Fisher and beta from all of part2 into out.
 * Each partition's partial sums are computed by the same kernels as in one
 * GPU's evaluation and the sums of the SUM exchanges add exact zeros, so
 * the result is bit for bit that of sv_vecchia_loglik.  The workspace must
 * persist from stage 1 to stage 4 of an evaluation; info is per rank
 * (combine the status words, e.g. by MAX). */
int sv_loglik_shard_sizes(const sv_loglik_desc* desc, int32_t* parts, int32_t* part1_len,
                          int32_t* part2_len);
int sv_vecchia_loglik_stage(const sv_loglik_desc* desc, int32_t stage, int32_t part_begin,
                            int32_t part_end, const double* theta, const double* X, const double* y,
                            const double* Z, const int32_t* rowb, const int32_t* kb,
                            const int32_t* nbr, const int32_t* chunk, int32_t* chunk_max,
                            double* part1, double* part2, double* out, int32_t* info,
                            void* workspace, size_t workspace_bytes, sv_stream_t stream);

/* Batched form: many independent problems evaluated by one set of launches
 * (batched fits of hundreds of problems; the reference fits problems one at
 * a time, so the per-problem arithmetic is likelihood.py:66-175 unchanged).  Problem p
 * has its own inputs (offsets into the concatenated X, y, Z), its own
 * contiguous run of blocks [blk_off, blk_off + nblk) with row indices local
 * to the problem, its own parameter vector theta[p * theta_stride ..] and its
 * own output out[p * out_stride ..] = ll, grad(P_p), fish(P_p * P_p), beta(q_p)
 * and info[4 p .. 4 p + 3].  bprob gives each block's problem; wlist / clist
 * list the blocks with k+1 <= 32 / k+1 > 32.  Only kernels and memsets are
 * enqueued, so the call can be captured in a CUDA graph and replayed with new
 * theta values. */
typedef struct sv_prob_desc {
  int64_t n;            /* rows of the problem                               */
  int64_t x_off;        /* offset (doubles) of its X (n x d, row-major)      */
  int64_t y_off;        /* offset (doubles) of its y                         */
  int64_t z_off;        /* offset (doubles) of its Z (n x q)                 */
  int64_t blk_off;      /* first block                                      */
  int64_t nblk;         /* number of blocks                                 */
  int32_t d, q;
  int32_t estimate_nu;
  int32_t skip;         /* nonzero: not evaluated by this call; its out and   */
                        /* info entries are left as they were               */
  double nu, var_penalty, log_var_target;
} sv_prob_desc;

typedef struct sv_batch_desc {
  int64_t nprob, nblk;  /* problems, blocks in all                          */
  int64_t nwarp, ncta;  /* lengths of wlist and clist (sum = nblk)          */
  int64_t nx;           /* doubles in X                                     */
  int32_t dmax, qmax, kmax, ldnbr;
  int32_t need_grad, any_estimate_nu, chunked, precision, team_lanes;
  int32_t theta_stride, out_stride;
  int32_t general_nu;   /* 1: some problem has a fixed nu outside {0.5, 1.5, */
                        /*    2.5} or an estimated nu; the workspace then    */
                        /*    holds Matern tables per problem (as the        */
                        /*    one-problem call builds for such a nu), so     */
                        /*    results match it bit for bit                   */
  double split_rho_min;
  int64_t nblk_max;     /* blocks of the largest problem (sizes the reductions) */
} sv_batch_desc;

size_t sv_loglik_batched_workspace_bytes(const sv_batch_desc* desc);
int sv_vecchia_loglik_batched(const sv_batch_desc* desc, const sv_prob_desc* probs,
                              const double* theta, const double* X, const double* y,
                              const double* Z, const int32_t* rowb, const int32_t* kb,
                              const int32_t* nbr, const int32_t* bprob, const int32_t* wlist,
                              const int32_t* clist, const int32_t* chunk, double* out,
                              int32_t* info, void* workspace, size_t workspace_bytes,
                              sv_stream_t stream);

/* No counterpart in the reference.  The same evaluation as sv_vecchia_loglik
 * for callers that cannot allocate device memory (an application whose fixed
 * memory pool owns the GPU, or a loop that must not call cudaMalloc, which
 * synchronises the device and can fail under memory pressure): inputs and
 * outputs as above, but the scratch comes from a file-scope static device
 * array of SV_NOALLOC_SCRATCH_BYTES held by every GPU that loads the library
 * until exit.  Returns SV_ENOSPC, launching nothing, when
 * sv_loglik_workspace_bytes(desc) exceeds it: at d = 10, m = 30, q = 1 with
 * score and Fisher, 34,995 blocks in float64 (precision 0) and 32,300 in the
 * split forms (precision 1 and 2, whose scratch also holds the float32
 * coordinate pairs).  The first call on a device looks up the array's address
 * (cudaGetSymbolAddress) and must come before any stream capture; later calls
 * enqueue only kernels (the problem descriptor passed by value, the status
 * words cleared by a kernel) and can be captured in a CUDA graph and
 * replayed.  All calls share the array: calls that overlap on the GPU race,
 * so serialise them. */
#define SV_NOALLOC_SCRATCH_BYTES (32u << 20)
int sv_vecchia_loglik_noalloc(const sv_loglik_desc* desc, const double* theta, const double* X,
                              const double* y, const double* Z, const int32_t* rowb,
                              const int32_t* kb, const int32_t* nbr, const int32_t* chunk,
                              double* out, int32_t* info, sv_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Learned warm start (set encoder)                                        */
/* ---------------------------------------------------------------------- */

/* No counterpart in the reference: a DeepSets encoder whose output replaces
 * the default starting point of Fisher scoring (gp.py:169-177); the fit
 * itself is unchanged.  Sets of S points (S a multiple of 128), 32 bfloat16
 * features per point (x_1..x_12 zero padded, y, and for the point's nearest
 * neighbour in the whole set its distance, the y difference and its square
 * and |dx_1|..|dx_12|; four zeros); cnt[b] valid points in set b.
 * Parameters: a flat float32 vector of
 * sv_encoder_param_count() entries, W1[128][32] b1[128] W2[128][128] b2[128]
 * W3[128][128] b3[128] W4[16][128] b4[16], and its bfloat16 copy
 * (sv_encoder_to_bf16); weights are read as bfloat16, biases as float32, all
 * sums accumulate in float32.  out is float32 [nset][16].  The backward also
 * takes target and weights [nset][16] (loss = sum w (out - target)^2) and
 * writes the loss (1 float) and the float32 gradient (param_count floats). */
int64_t sv_encoder_param_count(void);
size_t sv_encoder_workspace_bytes(int64_t nset, int32_t S, int32_t train);
int sv_encoder_pack(const double* features, int64_t n, uint16_t* x_bf16, sv_stream_t stream);
int sv_encoder_to_bf16(const float* params, uint16_t* params_bf16, int64_t n, sv_stream_t stream);
/* variant 0: per-point layers on tcgen05 (tensor memory accumulators);
 * variant 1: on mma.sync (the training path's forward).  A tcgen05 wait that
 * runs out leaves NaN outputs. */
int sv_encoder_forward(int64_t nset, int32_t S, const uint16_t* x, const int32_t* cnt,
                       const float* params, const uint16_t* params_bf16, float* out,
                       int32_t variant, void* workspace, size_t workspace_bytes,
                       sv_stream_t stream);
int sv_encoder_backward(int64_t nset, int32_t S, const uint16_t* x, const int32_t* cnt,
                        const float* params, const uint16_t* params_bf16, const float* target,
                        const float* weights, float* out, float* loss, float* grad,
                        void* workspace, size_t workspace_bytes, sv_stream_t stream);
/* Adam step (bias-corrected, decoupled weight decay added to the gradient)
 * on the float32 master parameters; refreshes the bfloat16 copy. */
int sv_encoder_adam(float* params, const float* grad, float* m, float* v, uint16_t* params_bf16,
                    int64_t n, float lr, float beta1, float beta2, float eps, int32_t step,
                    float weight_decay, sv_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Matern correlation (elementwise)                                        */
/* ---------------------------------------------------------------------- */

/* which = 0: M_nu(r); which = 1: g(r) = M_nu'(r)/r.
 * general = 0: closed forms, nu in {0.5,1.5,2.5}: _covariance.py:49-72.
 * general = 1: Bessel form 2^(1-nu)/Gamma(nu) c^nu K_nu(c), c = sqrt(2nu) r,
 *              r floored at 1e-7: _matern_general.py:87-116.
 * which = 2, 3, 4: the float32 forms the split kernels assemble with, at r
 * rounded to float32 (values of float32, returned as doubles): 2 the
 * correlation deficit D = 1 - M_nu(r), 3 g(r), 4 dM/dnu of an estimated nu
 * (the central difference (M_{nu+h} - M_{nu-h}) / 2h, h = 1e-3,
 * _matern_general.py:170-176); general = 0 the closed forms (which 2, 3),
 * general = 1 the float32 tables of a general nu (0 < nu <= 8 and at least
 * 1e-3 from an integer, for which = 4 nu +- h as well; else SV_EINVAL). */
int sv_matern_eval(const double* r, int64_t n, double nu, int32_t which, int32_t general,
                   double* out, sv_stream_t stream);

/* The Chebyshev tables of M and g of a fixed smoothness nu without a closed
 * form (0 < nu <= 10) that the likelihood builds for such a nu (16-term
 * series of e^c M(c) and e^c g(c) on half-octave intervals of
 * c = sqrt(2 nu) r; for nu <= 8 at least 1e-3 from an integer also the
 * float32 table of the deficit and g the split forms use), into device
 * float64[sv_matern_table_doubles()] (16-byte aligned), for
 * sv_pred_desc.matern_table.  SV_EINVAL for a nu without a table or a
 * smaller or misaligned buffer. */
int64_t sv_matern_table_doubles(void);
int sv_matern_table(double nu, double* table, int64_t table_doubles, sv_stream_t stream);

/* Modified Bessel function of the second kind K_nu(x) (device Temme/Steed
 * evaluation; stands in for scipy.special.kv on the _matern_general.py path). */
int sv_bessel_k(const double* x, int64_t n, double nu, double* out, sv_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Block-level routines (_covariance.py)                                   */
/* ---------------------------------------------------------------------- */

/* Sigma (B,K,K) and dSigma (B,P,K,K) of B blocks of K points:
 * replaces _covariance.py:150-198 (_block_cov) and _matern_general.py:134-179
 * (_block_cov_general).  Xb (B,K,d); ranges (d) host; nug_mask (B,K) or NULL.
 * dS may be NULL (derivs=False).  estimate_nu adds the log-nu row (FD h). */
int sv_block_cov(const double* Xb, int64_t B, int32_t K, int32_t d, const double* ranges_host,
                 double variance, double nugget, double nu, int32_t general, int32_t estimate_nu,
                 double nu_fd_h, const double* nug_mask, double* Sigma, double* dS,
                 sv_stream_t stream);

/* Batched lower Cholesky with the jitter retry of _covariance.py:235-252
 * (_batch_chol): if any block fails, all blocks are retried with
 * 10^p * mean(diag) for p = -12..-4 (the first p where every block succeeds).
 * info[SV_INFO_JITTER] = level used; info[0] = SV_ECHOL if all fail. */
size_t sv_batch_chol_workspace_bytes(int64_t B);
int sv_batch_chol(const double* Sigma, int64_t B, int32_t K, double* L, int32_t* info,
                  void* workspace, size_t workspace_bytes, sv_stream_t stream);

/* Batched triangular solves: replaces _covariance.py:205-218 (_forward_solve,
 * L X = B) and :220-232 (_backsolve_LT, L^T X = B).  L (b,K,K), B/X (b,K,nrhs). */
int sv_forward_solve(const double* L, const double* Bm, int64_t b, int32_t K, int32_t nrhs,
                     double* Xout, sv_stream_t stream);
int sv_backsolve_LT(const double* L, const double* Bm, int64_t b, int32_t K, int32_t nrhs,
                    double* Xout, sv_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Prediction (gp.py)                                                      */
/* ---------------------------------------------------------------------- */

typedef struct sv_pred_desc {
  int64_t nall;     /* rows of Xall                                    */
  int64_t nobs;     /* rows < nobs carry the nugget (observations)     */
  int64_t nblk;     /* prediction blocks                               */
  int32_t d;
  int32_t k;        /* neighbours per block (block size K = k+1)       */
  int32_t ldnbr;
  int32_t general;  /* 1: Bessel Matern                                */
  int32_t target_nugget; /* 1: the target row carries the nugget too     */
                         /*    (prior / unconditional draws)              */
  int32_t precision;     /* 0: float64; 1: split (closed-form nu, or a   */
                         /*    general nu whose matern_table holds a      */
                         /*    float32 part; float64 otherwise): entries  */
                         /*    below the diagonal from coordinates        */
                         /*    centred on the target as float32 (hi, lo)  */
                         /*    pairs and the float32 correlation deficit, */
                         /*    one float64 FMA each; diagonal, LDL^T and  */
                         /*    solves in float64                          */
  double nu;
  double split_rho_min;  /* split: a block whose smallest pivot ratio     */
                         /*    d_k / Sigma_kk falls below this (<= 0:     */
                         /*    1e-4), or that does not factor, is redone  */
                         /*    in float64; info[SV_INFO_AUX] counts them  */
  const double* matern_table; /* general = 1: the Matern table of nu from  */
                         /*    sv_matern_table (device memory), so that   */
                         /*    M and g are interpolated as the likelihood */
                         /*    interpolates them; NULL: K_nu per entry    */
} sv_pred_desc;

/* One prediction block per target row tgt[b] (noise-free unless
 * desc->target_nugget) with neighbours nbr[b*ldnbr + 0..k-1] (rows of Xall;
 * rows >= nobs are noise-free; a -1 ends a row with fewer neighbours):
 * replaces the per-chunk work of gp.py:257-276 (_predict_scaled) and
 * gp.py:329-348 (_joint_factor).
 *   theta : device float64[d+2] = [log s2, log lam_1..d, log tau]
 *   resid : device float64[nobs] residuals of the observations
 *   mean, var : device float64[nblk] (may be NULL)
 *             mean = -sum_{i<k, obs} a_i resid / a_K (marginal form when all
 *             neighbours are observations), var = 1 / a_K^2
 *   acol  : device float64[nblk * (k+1)] column a = L^-T e_K laid out as
 *           [neighbour slots 0..k-1, target], absent slots 0 (may be NULL)
 *   rhs   : device float64[nblk] = -sum_{obs i} a_i resid_i (may be NULL) */
int sv_predict_blocks(const sv_pred_desc* desc, const double* theta, const double* Xall,
                      const int32_t* tgt, const int32_t* nbr, const double* resid, double* mean,
                      double* var, double* acol, double* rhs, int32_t* info, sv_stream_t stream);

/* Sparse triangular solve U_pp^T X = R of gp.py:380-401 (scipy
 * spsolve_triangular), from the block columns of sv_predict_blocks.  With
 * nobs = 0 and the columns of an ordered Vecchia factor it also draws
 * unconditional Vecchia samples y = U^-T eps (no reference counterpart: the
 * reference only samples conditionally, gp.py:395-401):
 * row c: acol[c*(k+1)+k] x_c + sum_{i<k, nbr_ic >= nobs} acol[c*(k+1)+i] x_{nbr_ic - nobs} = R_c
 * (entries with nbr_ic < 0 are absent).
 * R and X are (npred, nrhs) row-major; rows are processed in order with
 * bounded waits on their predecessors (info[0] = SV_ETIMEOUT on expiry). */
size_t sv_joint_solve_workspace_bytes(int64_t npred);
int sv_joint_solve(int64_t npred, int64_t nobs, int32_t k, int32_t ldnbr, const int32_t* nbr,
                   const double* acol, const double* R, int32_t nrhs, double* X, int32_t* info,
                   void* workspace, size_t workspace_bytes, sv_stream_t stream);
/* The same with a test aid for the bounded waits: flags bit 0 keeps row 0
 * from publishing its result and limits every wait to 4096 polls, so the
 * waits of the rows that depend on row 0 run out (info[0] = SV_ETIMEOUT,
 * info[1] = the first such row); the kernel still finishes. */
int sv_joint_solve_flags(int64_t npred, int64_t nobs, int32_t k, int32_t ldnbr, const int32_t* nbr,
                         const double* acol, const double* R, int32_t nrhs, double* X,
                         int32_t* info, void* workspace, size_t workspace_bytes, int32_t flags,
                         sv_stream_t stream);

/* diag((U_pp U_pp^T)^-1), the marginal variances of the joint predictive
 * law N(mean, (U_pp U_pp^T)^-1) in the elimination ordering: replaces the
 * dense S = U_pp^-T of gp.py:391-393 (predict_joint(exact_var=True),
 * var = (S**2).sum(1)) without forming it.  Rows of S come from the
 * recurrence of sv_joint_solve against identity columns, in column panels:
 * a panel [c0, c0 + w) needs only rows >= c0 (S is lower triangular) and
 * row i only its columns <= i - c0; w is the widest panel whose rows
 * c0 .. npred-1 fit in `panel` ((npred - c0) w doubles; at least npred
 * doubles, else SV_ENOSPC).  npred * npred doubles do it in one launch.
 *   var       : device float64[npred]
 *   workspace : sv_joint_solve_workspace_bytes(npred) bytes
 *   panel     : device scratch of panel_bytes */
int sv_joint_var_diag(int64_t npred, int64_t nobs, int32_t k, int32_t ldnbr, const int32_t* nbr,
                      const double* acol, double* var, int32_t* info, void* workspace,
                      size_t workspace_bytes, double* panel, size_t panel_bytes,
                      sv_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Measurement                                                             */
/* ---------------------------------------------------------------------- */

/* No reference counterpart: *out = 1 when the current device reads ordinary
 * (pageable) host memory coherently through the host's page tables (a
 * Grace-Blackwell chip-to-chip link), else 0. */
int sv_device_reads_host_memory(int32_t* out);

/* No reference counterpart: a float64 FMA throughput probe (8 independent
 * chains of `iters` FMAs in each of sv_fp64_probe_threads() threads, one
 * double written per thread to out), used to state the float64 peak that the
 * block kernels are measured against. */
int64_t sv_fp64_probe_threads(void);
int sv_fp64_fma_probe(double* out, int32_t iters, sv_stream_t stream);

/* No reference counterpart: the same probe with float32 FMAs (one float per
 * thread, sv_fp64_probe_threads() threads), the FP32-pipe peak that the
 * split kernel's double-float arithmetic is measured against. */
int sv_fp32_fma_probe(float* out, int32_t iters, sv_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SVGPU_H */
