// Batched reorder of many independent problems: the rebuild step of the fit
// (gp.py:182-191) for every problem of a batched fit in one call.
//
// Per problem p with inputs X_e (n x d, subsample order), y_e, Z_e and
// ranges r (host values, so the division below sees numpy's exp bits):
//   Xs   = X_e / r                                (gp.py:184, IEEE division)
//   ord  = maximin order of Xs from row `first`   (ordering.py:27-73)
//   X, y, Z <- X_e[ord], y_e[ord], Z_e[ord]        (gp.py:189-191)
//   nbr  <- ordered kNN of Xs[ord], m neighbours   (ordering.py:76-116), written
//           straight into the likelihood's block columns: block blk_off + i
//           holds row i's min(i, m) neighbours, nearest first, -1 padded
//           (the _nn_groups layout, ordering.py:119-127, with row i = block i).
//
// Maximin runs one thread-block cluster per problem.  The cluster's CTAs
// split the problem's points; each keeps, in shared memory, the squared
// float64 distances, float32 skip thresholds, exact coordinates and float32
// coordinates centred on the first row.  Every decision is the reference's:
//  * screening: a rigorous float32 bound skips a point only when the
//    reference would not update it;
//  * update: the squared distance s_new is computed in IEEE sequential
//    float64 exactly as ordering.py:52-57 does before its square root; the
//    point is updated when s_new < s_stored (bit compare).  With a correctly
//    rounded, monotone sqrt this keeps fl(sqrt(s_stored)) equal to the
//    reference's stored distance at every step: the reference updates only
//    when fl(sqrt(s_new)) < fl(sqrt(s_stored)), which implies s_new <
//    s_stored; an update here that the reference skips has
//    fl(sqrt(s_new)) == fl(sqrt(s_stored)) and leaves the root unchanged.
//    No square root is taken on this path;
//  * argmax: many pivots per pass, each provably the reference's next choice
//    (the comment above k_maximin_cluster gives the argument); candidate
//    lists meet through distributed shared memory after one hardware cluster
//    barrier per pass (double-buffered by pass parity), so there is no
//    spin-wait at all.
// Problems are grouped by cluster size (1, 2, 4, 8 or 16 CTAs, the smallest
// whose shared memory holds the problem), one launch per group, largest
// problems first.
#include <cooperative_groups.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "sv_maximin_ops.cuh"
#include "sv_reorder.cuh"

namespace cg = cooperative_groups;

namespace sv {

constexpr int kMcThreads = 512;
constexpr int kMcWarps = kMcThreads / 32;
constexpr int kMcSlots = 32;  // candidate slots; slot 31 holds a pivot found by a full scan
// static shared memory of k_maximin_cluster (about 1.3 KB), rounded up: the
// capacity of a cluster is computed from what is left of 227 KB
constexpr int kMcStaticSmem = 4096;
constexpr int kMcMaxCluster = 16;
// work area: the warps' candidate lists (bits + index) or the pair distances
constexpr int kMcWorkBytes = ((kMcU * kMcU * 8 > kMcWarps * 32 * 12 ? kMcU * kMcU * 8 : kMcWarps * 32 * 12) + 15) & ~15;

struct RoProb {
  int64_t n, xe_off, ye_off, ze_off, x_off, y_off, z_off, blk_off, first;
  int64_t xs_off;   // doubles: this call's scaled rows (and their maximin-order copy)
  int64_t v_off;    // floats: centred float32 rows [n][DP]
  int64_t row_off;  // rows: order, B
  int32_t d, q, m, DP, C, flags;
};

// per-point shared memory of the pass maximin: dist f64, exact coordinates
// f64[d] (cluster form only), thr f32, B f32, float32 centred coordinates f32[d]
__host__ __device__ inline int64_t mc_point_bytes(int d, bool grid = false) {
  return 16 + (grid ? 4 : 12) * (int64_t)d;
}
// width of the pivot images held in registers (zero padded)
__host__ __device__ inline int mc_dv(int d) { return d <= 4 ? 4 : d <= 8 ? 8 : d <= 16 ? 16 : d <= 32 ? 32 : 64; }
// per-CTA shared memory before the points: candidate slots (exact and float32
// coordinates, squared bits, index, bound), the pivot images and the work area
__host__ __device__ inline int64_t mc_fixed_bytes(int d) {
  return (int64_t)kMcSlots * (12 * d + 16) + (int64_t)kMcSlots * 4 * mc_dv(d) + kMcWorkBytes;
}

__global__ void k_ro_info_init(int32_t* info, int nprob) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nprob; p += gridDim.x * blockDim.x) {
    info[4 * p + 0] = 0;
    info[4 * p + 1] = -1;
    info[4 * p + 2] = 0;
    info[4 * p + 3] = 0;
  }
}

// Xs = X_e / r; grid row = problem
__global__ void k_ro_scale(const RoProb* probs, const double* ranges, int dmax, const double* Xe,
                           double* Xs) {
  const RoProb& P = probs[blockIdx.y];
  const int d = P.d;
  const int64_t tot = P.n * d;
  const double* r = ranges + (int64_t)blockIdx.y * dmax;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x)
    Xs[P.xs_off + e] = __ddiv_rn(Xe[P.xe_off + e], r[e % d]);
}

// shared-memory layout of one CTA of the cluster maximin (identical in every
// CTA of a cluster, so remote reads use the same offsets)
struct McSmem {
  double* Ux;      // [32][d] exact coordinates of the candidate slots
  float* Uv;       // [32][d] their centred float32 images
  long long* Ub;   // [32] squared-distance bits at the start of the selection
  int* Ui;         // [32] row index
  float* UB;       // [32] float32 rounding bound of the image
  float* Pv;       // [32][DV] images of this pass's pivots, zero padded to DV
  double* pairS;   // [31][31] exact squared distances between candidates (work area)
  long long* wlb;  // [warps][32] candidate lists (work area)
  int* wli;
  double* dist;    // [Sc] squared distance to the ordered set; -1 once ordered
  const double* xs;  // [Sc][d] exact coordinates (shared memory, or the rows in global memory)
  float* thr;      // [Sc] float32 screening threshold
  float* Bp;       // [Sc] float32 rounding bound of the image
  float* v;        // [d][Sc] centred float32 images
};

// xg: the CTA's exact rows in global memory (grid form), or null to keep
// them in shared memory (cluster form)
__device__ __forceinline__ McSmem mc_layout(unsigned char* base, int d, int Sc, const double* xg) {
  McSmem L;
  L.Ux = (double*)base;
  L.Uv = (float*)(base + (size_t)kMcSlots * 8 * d);
  L.Ub = (long long*)(base + (size_t)kMcSlots * 12 * d);
  L.Ui = (int*)(L.Ub + kMcSlots);
  L.UB = (float*)(L.Ui + kMcSlots);
  L.Pv = (float*)(base + (size_t)kMcSlots * (12 * d + 16));
  unsigned char* work = (unsigned char*)(L.Pv + kMcSlots * mc_dv(d));
  L.pairS = (double*)work;
  L.wlb = (long long*)work;
  L.wli = (int*)(work + kMcWarps * 32 * 8);
  unsigned char* pts = work + kMcWorkBytes;
  L.dist = (double*)pts;
  L.xs = xg ? xg : L.dist + Sc;
  L.thr = (float*)(L.dist + Sc + (xg ? 0 : (size_t)Sc * d));
  L.Bp = L.thr + Sc;
  L.v = L.Bp + Sc;
  return L;
}

// exact squared distances (ordering.py:52-57) of the pivots in `mask`, in
// pivot order, lower point p's distance; its threshold follows
__device__ __forceinline__ void mc_exact(const McSmem& M, const int* Ps, int p, int d, unsigned mask) {
  const double* xp = M.xs + (size_t)p * d;
  double dp = M.dist[p];
  const long long b0 = __double_as_longlong(dp);
  do {
    const int t = __ffs(mask) - 1;
    mask &= mask - 1;
    const double sn = sqdist_exact(xp, M.Ux + Ps[t] * d, d);
    if (__double_as_longlong(sn) < __double_as_longlong(dp)) dp = sn;
  } while (mask);
  if (__double_as_longlong(dp) != b0) {
    M.dist[p] = dp;
    M.thr[p] = thr_sq(dp, M.Bp[p]);
  }
}

// float32 squared distance of a register image to pivot image t
template <int DV>
__device__ __forceinline__ float mc_s32(const float (&vp)[DV], const float4* pv) {
  float s32 = 0.0f;
#pragma unroll
  for (int q = 0; q < DV / 4; ++q) {
    const float4 f = pv[q];
    float df = __fsub_rn(vp[4 * q], f.x);
    s32 = __fmaf_rn(df, df, s32);
    df = __fsub_rn(vp[4 * q + 1], f.y);
    s32 = __fmaf_rn(df, df, s32);
    df = __fsub_rn(vp[4 * q + 2], f.z);
    s32 = __fmaf_rn(df, df, s32);
    df = __fsub_rn(vp[4 * q + 3], f.w);
    s32 = __fmaf_rn(df, df, s32);
  }
  return s32;
}

// queue of (point, pivot mask) for the exact distances, in the work area
constexpr int kMcQueue = kMcWorkBytes / 8;

// after the screen of point p: ordered if it is a pivot of this pass
// (ordering.py:58); else the pivots in `mask` go to the queue (processed by
// dense warps: a float64 warp instruction costs the same with one lane
// active as with 32), or are applied here when the queue is full
__device__ __forceinline__ void mc_screened(const McSmem& M, const int* Ps, int* qn, int p, int d,
                                            bool hit, unsigned mask) {
  if (hit) {
    M.dist[p] = -1.0;
    mask = 0;
  }
  const unsigned act = __activemask();
  const unsigned want = __ballot_sync(act, mask != 0);
  if (!want) return;
  const int leader = __ffs(want) - 1;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == leader) base = atomicAdd(qn, __popc(want));
  base = __shfl_sync(act, base, leader);
  if (mask) {
    const int slot = base + __popc(want & ((1u << lane) - 1));
    if (slot < kMcQueue) {
      int2* q = reinterpret_cast<int2*>(M.pairS);
      q[slot] = make_int2(p, (int)mask);
    } else {
      mc_exact(M, Ps, p, d, mask);
    }
  }
}

// This pass's pivots (table entries t < k: row Pi, bound PB, image Pv, slot
// Ps of the exact coordinates) applied to the CTA's points, then each
// thread's three largest keys.  For every point the float32 screen runs over
// all pivots first, with the threshold of the pass start (an upper bound of
// every later one, so a pivot it skips cannot update); the exact squared
// distances of the pivots left then update in pivot order, as the reference
// applies them (ordering.py:49-58).  DV: the image width held in registers
// (0: read from shared memory, any d); up to 16, two points share each
// read of a pivot image.
template <int DV>
__device__ __forceinline__ void mc_apply(const McSmem& M, const int* Pi, const float* PB,
                                         const int* Ps, int* qn, int k, int S, int Sc, int d,
                                         int p0, float growth, long long& b1, int& i1,
                                         long long& b2, int& i2, long long& b3, int& i3) {
  if constexpr (DV > 0 && DV <= 16) {
    const int T = blockDim.x;
    for (int p = threadIdx.x; p < S; p += 2 * T) {
      const int q = p + T;
      const bool liveA = __double_as_longlong(M.dist[p]) >= 0;
      const bool liveB = q < S && __double_as_longlong(M.dist[q]) >= 0;
      if (!liveA && !liveB) continue;  // ordered (ordering.py:50-51)
      const float thA = M.thr[p], thB = liveB ? M.thr[q] : 0.0f;
      float va[DV], vb[DV];
#pragma unroll
      for (int l = 0; l < DV; ++l) {
        va[l] = l < d ? M.v[(size_t)l * Sc + p] : 0.0f;
        vb[l] = l < d && liveB ? M.v[(size_t)l * Sc + q] : 0.0f;
      }
      unsigned mA = 0, mB = 0;
      bool hA = false, hB = false;
#pragma unroll 2
      for (int t = 0; t < k; ++t) {
        const float4* pv = reinterpret_cast<const float4*>(M.Pv + t * DV);
        const float sA = mc_s32<DV>(va, pv), sB = mc_s32<DV>(vb, pv);
        const int pi = Pi[t];
        const float pb = PB[t];
        hA = hA || pi == p0 + p;
        hB = hB || pi == p0 + q;
        if (mc_may_update(sA, thA, pb, growth)) mA |= 1u << t;
        if (mc_may_update(sB, thB, pb, growth)) mB |= 1u << t;
      }
      mc_screened(M, Ps, qn, p, d, hA, liveA ? mA : 0u);
      if (liveB) mc_screened(M, Ps, qn, q, d, hB, mB);
    }
  } else {
    constexpr int W = DV > 0 ? DV : 64;
    for (int p = threadIdx.x; p < S; p += blockDim.x) {
      if (__double_as_longlong(M.dist[p]) < 0) continue;  // ordered (ordering.py:50-51)
      const float th = M.thr[p];
      unsigned mask = 0;
      bool hit = false;
      if constexpr (DV > 0) {
        float vp[DV];
#pragma unroll
        for (int l = 0; l < DV; ++l) vp[l] = l < d ? M.v[(size_t)l * Sc + p] : 0.0f;
#pragma unroll 2
        for (int t = 0; t < k; ++t) {
          const float s32 = mc_s32<DV>(vp, reinterpret_cast<const float4*>(M.Pv + t * DV));
          hit = hit || Pi[t] == p0 + p;
          if (mc_may_update(s32, th, PB[t], growth)) mask |= 1u << t;
        }
      } else {
        for (int t = 0; t < k; ++t) {
          const float* pv = M.Pv + t * W;
          float s32 = 0.0f;
          for (int l = 0; l < d; ++l) {
            const float df = __fsub_rn(M.v[(size_t)l * Sc + p], pv[l]);
            s32 = __fmaf_rn(df, df, s32);
          }
          hit = hit || Pi[t] == p0 + p;
          if (mc_may_update(s32, th, PB[t], growth)) mask |= 1u << t;
        }
      }
      mc_screened(M, Ps, qn, p, d, hit, mask);
    }
  }
  __syncthreads();
  // the queued exact distances, densely
  const int nq = min(*qn, kMcQueue);
  const int2* q = reinterpret_cast<const int2*>(M.pairS);
  for (int e = threadIdx.x; e < nq; e += blockDim.x) {
    const int2 E = q[e];
    mc_exact(M, Ps, E.x, d, (unsigned)E.y);
  }
  __syncthreads();
  // each thread's three largest keys, its points in index order
  for (int p = threadIdx.x; p < S; p += blockDim.x) {
    const long long b = __double_as_longlong(M.dist[p]);
    if (b < 0 || b >= 0x7ff0000000000000LL) continue;  // ordered, or not finite
    mc_insert3(b, p0 + p, b1, i1, b2, i2, b3, i3);
  }
}

// One problem of the pass maximin.
struct McRun {
  const double* X;     // the problem's rows (scaled), n x d
  int64_t n;
  int64_t first;       // the first row of the order (ordering.py:72)
  int64_t* order;
  int32_t* info;       // the problem's 4 status words
  int32_t d, flags;
  // grid form: the iteration limit of a barrier wait, and a test aid: CTA 0
  // does not arrive at the first barrier, so every wait there runs out
  unsigned spin_limit;
  int32_t skip_first_arrival;
  // grid form: candidate lists of every CTA [2][G][32], their bounds [2][G],
  // and the monotone arrival counter of the grid barrier
  long long* gl_b;
  int* gl_i;
  long long* gl_Kb;
  int* gl_Ki;
  unsigned* arrive;
};

// Maximin in passes.  A pass applies a batch of pivots, in order, to every
// unordered point (the reference's update, ordering.py:49-58, once per
// pivot), then chooses the next batch:
//  * the 31 largest keys (squared bits, then index) of all CTAs form the
//    candidate set U, and R bounds the squared bits of every other point
//    (the 32nd key and every thread's third-largest key);
//  * the exact squared distances between candidates (float32-screened) give
//    each candidate's value after any pivots taken from U;
//  * repeatedly the largest surviving candidate is the reference's next
//    pivot (ordering.py:42-47: largest root, then smallest index) as long as
//    its squared bits exceed R by more than 4 ulps: distinct squares with
//    equal roots lie within 3 ulps, so every point outside U then has a
//    smaller root.  Candidates within 4 ulps of the largest are ranked by
//    their exact roots;
//  * if not even the first choice is certain (many near-equal distances, as
//    on a lattice), a tie pass takes the points whose root equals the largest
//    root, in index order.
// The CTAs' lists meet through a hardware cluster barrier and distributed
// shared memory (cluster form, kGrid false), or through global memory and a
// grid barrier with bounded waits (grid form: one CTA per SM of a
// cooperative launch, exact rows read from global memory).  flags bit 0
// ranks every choice by exact roots, bit 1 runs a tie pass every time; both
// give the same order (test aids).
template <bool kGrid>
__device__ __forceinline__ void mc_run(const McRun& Q, int C, int r) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int64_t n = Q.n;
  const int d = Q.d;
  const int DV = mc_dv(d);
  const double* X = Q.X;
  int64_t* order = Q.order;
  const int per = (int)((n + C - 1) / C);
  const int p0 = r * per;
  const int S = (int)max((int64_t)0, min(n, (int64_t)p0 + per) - p0);
  const int Sc = per;
  const McSmem M = mc_layout(smraw, d, Sc, kGrid ? X + (size_t)p0 * d : nullptr);
  __shared__ double cen[64];
  __shared__ long long cl_b[2][32], cl_Kb[2];
  __shared__ int cl_i[2][32], cl_Ki[2];
  __shared__ long long w_Kb[kMcWarps];
  __shared__ int w_Ki[kMcWarps];
  __shared__ int piv_slot[kMcSlots], P_i[kMcSlots], P_s[kMcSlots];
  __shared__ float P_B[kMcSlots], Uthr[kMcSlots];
  __shared__ int s_k, s_tie, s_err, s_Ki, s_qn, s_abort;
  __shared__ unsigned s_epoch;
  __shared__ long long s_Kb, s_top;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarp = blockDim.x >> 5;
  const float growth = mc_growth(d);
  const bool roots_always = (Q.flags & 1) != 0;
  const bool scan_always = (Q.flags & 2) != 0;

  // all CTAs of the problem: the hardware cluster barrier, or the grid
  // barrier (monotone arrival counter, bounded wait); false once a wait gave up
  auto all_sync = [&]() -> bool {
    if constexpr (kGrid) {
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        if (!(Q.skip_first_arrival && r == 0 && s_epoch == 0)) atomicAdd(Q.arrive, 1u);
        const unsigned target = (unsigned)C * ++s_epoch;
        unsigned it = 0;
        while (ld_acquire_u32(Q.arrive) < target) {
          if (++it > Q.spin_limit) {
            set_error(Q.info + SV_INFO_STATUS, SV_ETIMEOUT);
            s_abort = 1;
            break;
          }
        }
        __threadfence();
      }
      __syncthreads();
      return s_abort == 0;
    } else {
      if (C > 1)
        cg::this_cluster().sync();
      else
        __syncthreads();
      return true;
    }
  };
  // element l of row idx: exact coordinate and float32 image
  auto row_elem = [&](int idx, int l, double& x, float& vv) {
    if constexpr (kGrid) {
      x = X[(size_t)idx * d + l];
      vv = __double2float_rn(x - cen[l]);
    } else {
      const int owner = idx / per, loc = idx - owner * per;
      const double* xs = M.xs;
      const float* v = M.v;
      if (C > 1 && owner != r) {
        xs = cg::this_cluster().map_shared_rank(M.xs, owner);
        v = cg::this_cluster().map_shared_rank(M.v, owner);
      }
      x = xs[(size_t)loc * d + l];
      vv = v[(size_t)l * Sc + loc];
    }
  };
  // warp 0: the pivot table from slots piv_slot[0..kk)
  auto build_pivots = [&](int kk) {
    __syncwarp();
    for (int e = lane; e < kk * DV; e += 32) {
      const int t = e / DV, l = e - t * DV;
      M.Pv[e] = l < d ? M.Uv[piv_slot[t] * d + l] : 0.0f;
    }
    if (lane < kk) {
      const int u = piv_slot[lane];
      P_i[lane] = M.Ui[u];
      P_B[lane] = M.UB[u];
      P_s[lane] = u;
    }
    if (lane == 0) s_qn = 0;
    __syncwarp();
  };

  // centre: the first row (any shift serves the float32 screen)
  for (int l = threadIdx.x; l < d; l += blockDim.x) cen[l] = X[Q.first * d + l];
  if (threadIdx.x == 0) {
    s_abort = 0;
    s_epoch = 0;
  }
  __syncthreads();
  if constexpr (!kGrid)
    for (int e = threadIdx.x; e < S * d; e += blockDim.x) const_cast<double*>(M.xs)[e] = X[(size_t)p0 * d + e];
  for (int p = threadIdx.x; p < S; p += blockDim.x) {
    const double* xp = X + (size_t)(p0 + p) * d;
    double e2 = 0.0;
    for (int l = 0; l < d; ++l) {
      const double c = xp[l] - cen[l];
      M.v[(size_t)l * Sc + p] = __double2float_rn(c);
      e2 += c * c;
    }
    M.Bp[p] = __double2float_ru(1.01 * 0x1p-24 * sqrt(e2));
    M.dist[p] = __longlong_as_double(0x7ff0000000000000LL);  // +inf: the first pass is exact
    M.thr[p] = __int_as_float(0x7f800000);
  }
  // every CTA's rows are in place before the first remote read
  if (!all_sync()) return;
  // the first pivot: row `first` (ordering.py:38-39) in slot 31
  if (warp == 0) {
    const int idx = (int)Q.first;
    for (int l = lane; l < d; l += 32) row_elem(idx, l, M.Ux[kMcU * d + l], M.Uv[kMcU * d + l]);
    __syncwarp();
    if (lane == 0) {
      M.UB[kMcU] = mc_img_bound(M.Uv + kMcU * d, d);
      M.Ui[kMcU] = idx;
      piv_slot[0] = kMcU;
      s_k = 1;
      s_err = 0;
      s_tie = 0;
      if (r == 0) order[0] = Q.first;
    }
    build_pivots(1);
  }
  __syncthreads();

  // Candidate lists: from every thread's three largest keys (b1 > b2 > b3),
  // the 32 largest keys of all CTAs land in slots 0..31 (bits Ub, index Ui)
  // and (Kb, Ki) is the largest key that may belong to a point outside slots
  // 0..30: the 32nd key or a thread's third.  The same in every CTA.
  // False once a grid wait gave up.
  int par = 0;  // parity of the list buffers, flipped per collection
  auto collect = [&](long long b1, int i1, long long b2, int i2, long long b3, int i3,
                     long long& Kb, int& Ki) -> bool {
    mc_warp_sort2(b1, i1, b2, i2);
    mc_warp_merge(b1, i1, b2, i2);
    mc_warp_max(b3, i3);
    M.wlb[warp * 32 + lane] = b1;
    M.wli[warp * 32 + lane] = i1;
    if (lane == 0) {
      w_Kb[warp] = b3;
      w_Ki[warp] = i3;
    }
    __syncthreads();
    // a tree over the lists wlb[0..nwarp): warp w < s merges list w + s
    auto tree = [&]() {
      for (int s = nwarp >> 1; s >= 1; s >>= 1) {
        if (warp < s) {
          mc_warp_merge(b1, i1, M.wlb[(warp + s) * 32 + lane], M.wli[(warp + s) * 32 + lane]);
          if (s > 1) {
            M.wlb[warp * 32 + lane] = b1;
            M.wli[warp * 32 + lane] = i1;
          }
        }
        if (s > 1) __syncthreads();
      }
    };
    tree();
    long long kb = -1LL;
    int ki = kMcNone;
    if (warp == 0) {
      if (lane < nwarp) {
        kb = w_Kb[lane];
        ki = w_Ki[lane];
      }
      mc_warp_max(kb, ki);
    }
    if (C > 1) {
      // every CTA merges all lists (the same keys, so the same result
      // everywhere).  A buffer is rewritten two collections on, after the
      // next barrier, which no CTA passes before all have read it.
      if constexpr (kGrid) {
        if (warp == 0) {
          Q.gl_b[((size_t)par * C + r) * 32 + lane] = b1;
          Q.gl_i[((size_t)par * C + r) * 32 + lane] = i1;
          if (lane == 0) {
            Q.gl_Kb[par * C + r] = kb;
            Q.gl_Ki[par * C + r] = ki;
          }
        }
        if (!all_sync()) return false;
        // warp w merges the lists of CTAs w, w + nwarp, ... (next one in flight)
        b1 = -1LL;
        i1 = kMcNone;
        long long nb = -1LL;
        int ni = kMcNone;
        if (warp < C) {
          nb = __ldcg(Q.gl_b + ((size_t)par * C + warp) * 32 + lane);
          ni = __ldcg(Q.gl_i + ((size_t)par * C + warp) * 32 + lane);
        }
        for (int c = warp; c < C; c += nwarp) {
          const long long ob = nb;
          const int oi = ni;
          if (c + nwarp < C) {
            nb = __ldcg(Q.gl_b + ((size_t)par * C + c + nwarp) * 32 + lane);
            ni = __ldcg(Q.gl_i + ((size_t)par * C + c + nwarp) * 32 + lane);
          }
          mc_warp_merge(b1, i1, ob, oi);
        }
        if (warp == 0) {
          kb = -1LL;
          ki = kMcNone;
          for (int c = lane; c < C; c += 32) {
            const long long ob = __ldcg(Q.gl_Kb + par * C + c);
            const int oi = __ldcg(Q.gl_Ki + par * C + c);
            if (mc_greater(ob, oi, kb, ki)) {
              kb = ob;
              ki = oi;
            }
          }
          mc_warp_max(kb, ki);
        }
      } else {
        cg::cluster_group cluster = cg::this_cluster();
        if (warp == 0) {
          cl_b[par][lane] = b1;
          cl_i[par][lane] = i1;
          if (lane == 0) {
            cl_Kb[par] = kb;
            cl_Ki[par] = ki;
          }
        }
        cluster.sync();
        b1 = -1LL;
        i1 = kMcNone;
        if (warp < C) {
          // warp c brings the list of CTA c (one remote round trip for all)
          b1 = cluster.map_shared_rank(&cl_b[par][0], warp)[lane];
          i1 = cluster.map_shared_rank(&cl_i[par][0], warp)[lane];
        }
        if (warp == 0) {
          kb = -1LL;
          ki = kMcNone;
          if (lane < C) {
            kb = *cluster.map_shared_rank(&cl_Kb[par], lane);
            ki = *cluster.map_shared_rank(&cl_Ki[par], lane);
          }
          mc_warp_max(kb, ki);
        }
      }
      M.wlb[warp * 32 + lane] = b1;
      M.wli[warp * 32 + lane] = i1;
      __syncthreads();
      tree();
    }
    if (warp == 0) {
      const long long b32 = __shfl_sync(0xffffffffu, b1, 31);
      const int i32 = __shfl_sync(0xffffffffu, i1, 31);
      if (mc_greater(b32, i32, kb, ki)) {
        kb = b32;
        ki = i32;
      }
      M.Ub[lane] = b1;  // slot 31 is rewritten before any use
      M.Ui[lane] = i1;
      if (lane == 0) {
        s_Kb = kb;
        s_Ki = ki;
      }
    }
    __syncthreads();
    Kb = s_Kb;
    Ki = s_Ki;
    par ^= 1;
    return true;
  };
  // the candidates' rows, then their pairwise exact squared distances
  // (float32-screened: +inf where neither can lower the other; -1 where a
  // float32 upper bound already puts either below R once the other is a pivot)
  auto fetch_pairs = [&](double Rv) {
    for (int e = threadIdx.x; e < kMcU * d; e += blockDim.x) {
      const int u = e / d, l = e - u * d;
      if (M.Ub[u] >= 0) row_elem(M.Ui[u], l, M.Ux[u * d + l], M.Uv[u * d + l]);
    }
    __syncthreads();
    if (threadIdx.x < kMcU && M.Ub[threadIdx.x] >= 0) {
      const int u = threadIdx.x;
      const float B = mc_img_bound(M.Uv + u * d, d);
      M.UB[u] = B;
      Uthr[u] = thr_sq(__longlong_as_double(M.Ub[u]), B);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kMcU * kMcU; t += blockDim.x) {
      const int a = t / kMcU, b = t - a * kMcU;
      if (a >= b || M.Ub[a] < 0 || M.Ub[b] < 0) continue;
      float s32 = 0.0f;
      for (int l = 0; l < d; ++l) {
        const float df = __fsub_rn(M.Uv[a * d + l], M.Uv[b * d + l]);
        s32 = __fmaf_rn(df, df, s32);
      }
      double sp = __longlong_as_double(0x7ff0000000000000LL);  // cannot update
      if (mc_may_update(s32, Uthr[a], M.UB[b], growth) || mc_may_update(s32, Uthr[b], M.UB[a], growth)) {
        if (Rv >= 0.0 && (double)mc_sq_upper(s32, M.UB[a], M.UB[b], growth) < Rv)
          sp = -1.0;  // either, once the other is a pivot, falls below R: out of this pass
        else
          sp = sqdist_exact(M.Ux + a * d, M.Ux + b * d, d);  // (x_a - x_b)^2 = (x_b - x_a)^2
      }
      M.pairS[a * kMcU + b] = sp;
      M.pairS[b * kMcU + a] = sp;
    }
    __syncthreads();
  };

  int64_t nsel = 1;
  while (nsel < n) {
    // 1. apply the pivots to this CTA's points; keep each thread's three
    //    largest keys
    const int k = s_k;
    long long b1 = -1, b2 = -1, b3 = -1;
    int i1 = kMcNone, i2 = kMcNone, i3 = kMcNone;
    switch (DV) {
      case 4:
        mc_apply<4>(M, P_i, P_B, P_s, &s_qn, k, S, Sc, d, p0, growth, b1, i1, b2, i2, b3, i3);
        break;
      case 8:
        mc_apply<8>(M, P_i, P_B, P_s, &s_qn, k, S, Sc, d, p0, growth, b1, i1, b2, i2, b3, i3);
        break;
      case 16:
        mc_apply<16>(M, P_i, P_B, P_s, &s_qn, k, S, Sc, d, p0, growth, b1, i1, b2, i2, b3, i3);
        break;
      case 32:
        mc_apply<32>(M, P_i, P_B, P_s, &s_qn, k, S, Sc, d, p0, growth, b1, i1, b2, i2, b3, i3);
        break;
      default:
        mc_apply<0>(M, P_i, P_B, P_s, &s_qn, k, S, Sc, d, p0, growth, b1, i1, b2, i2, b3, i3);
    }
    // 2. candidates U = slots 0..30; R bounds every other point's bits
    long long R;
    int Ri;
    if (!collect(b1, i1, b2, i2, b3, i3, R, Ri)) return;  // a grid wait gave up
    fetch_pairs(R >= 0 ? __longlong_as_double(R) : -1.0);
    // 3. pivots from the candidates (warp 0, one candidate per lane)
    if (warp == 0) {
      long long sb = lane < kMcU ? M.Ub[lane] : -1LL;
      const int si = lane < kMcU ? M.Ui[lane] : kMcNone;
      bool alive = sb >= 0;
      const long long top = __shfl_sync(0xffffffffu, sb, 0);  // the largest square
      int kk = 0;
      if (!scan_always && !roots_always) {
        // the leading run of slots that are certain in list order: each is
        // above R + 4 ulps, more than 4 ulps above the next slot (no equal
        // root below it) and not lowered by a slot before it
        bool red = false;
        for (int i = 0; i < lane && i < kMcU; ++i)
          red = red || __double_as_longlong(M.pairS[lane * kMcU + i]) < sb;  // (knock-outs are < 0)
        const long long nb = __shfl_down_sync(0xffffffffu, sb, 1);
        const bool near = lane + 1 < kMcU && nb >= 0 && nb >= sb - 4;
        const bool bad = lane >= kMcU || !alive || red || near || !(R < 0 || sb > R + 4);
        const int m = (int)min((int64_t)(__ffs(__ballot_sync(0xffffffffu, bad)) - 1), n - nsel);
        if (m > 0) {
          if (lane < m) {
            piv_slot[lane] = lane;
            alive = false;
          }
          for (int i = 0; alive && i < m; ++i) {
            const long long sn = __double_as_longlong(M.pairS[lane * kMcU + i]);
            if (sn < 0)
              alive = false;  // below R: cannot be chosen in this pass
            else if (sn < sb)
              sb = sn;
          }
          kk = m;
        }
      }
      while (!scan_always && kk < kMcU && nsel + kk < n) {
        // the largest key among the survivors: high word, low word, index
        const unsigned hi = alive ? (unsigned)((unsigned long long)sb >> 32) + 1u : 0u;
        const unsigned mh = __reduce_max_sync(0xffffffffu, hi);
        if (mh == 0) break;  // none left
        const unsigned lo = alive && hi == mh ? (unsigned)sb : 0u;
        const unsigned ml = __reduce_max_sync(0xffffffffu, lo);
        const long long mb = ((long long)(mh - 1u) << 32) | (long long)ml;
        if (!(R < 0 || mb > R + 4)) break;  // not certain
        const bool is_max = alive && hi == mh && (unsigned)sb == ml;
        int mi = (int)__reduce_min_sync(0xffffffffu, is_max ? (unsigned)si : (unsigned)kMcNone);
        const unsigned nearm = __ballot_sync(0xffffffffu, alive && sb >= mb - 4 && si < mi);
        if (nearm || roots_always) {
          // equal roots: the smaller index (ordering.py:45 keeps the first maximum)
          long long rb = -1LL;
          int ri = kMcNone;
          if (alive && sb >= mb - 4) {
            rb = __double_as_longlong(__dsqrt_rn(__longlong_as_double(sb)));
            ri = si;
          }
          mc_warp_max(rb, ri);
          mi = ri;
        }
        const int ws = __ffs(__ballot_sync(0xffffffffu, alive && si == mi)) - 1;
        if (lane == 0) piv_slot[kk] = ws;
        if (lane == ws) alive = false;
        if (alive) {
          const long long sn = __double_as_longlong(M.pairS[lane * kMcU + ws]);
          if (sn < 0)
            alive = false;  // below R after this pivot: cannot be chosen in this pass
          else if (sn < sb)
            sb = sn;
        }
        ++kk;
      }
      build_pivots(kk);
      if (lane == 0) {
        s_k = kk;
        s_tie = kk == 0;
        s_top = top;
        if (r == 0)
          for (int t = 0; t < kk; ++t) order[nsel + t] = P_i[t];
      }
    }
    __syncthreads();
    if (s_tie) {
      // 4. tie pass: no choice was certain, so many squares lie within 4 ulps
      //    of the largest, top.  The largest root is fl(sqrt(top)); the points
      //    with that root, T, are the reference's next choices in index order
      //    (ordering.py:45) while they keep it.  Slots 0..30 take the 31
      //    smallest indices of T; any other member of T has an index >= the
      //    bound Ki.
      const long long top = s_top;
      if (top < 0) {
        // no finite candidate left (NaN inputs): report and stop
        if (threadIdx.x == 0) {
          s_err = 1;
          if (r == 0) {
            set_error(Q.info + SV_INFO_STATUS, SV_EINVAL);
            Q.info[SV_INFO_BLOCK] = (int)nsel;
          }
        }
      } else {
        const long long rmax = __double_as_longlong(__dsqrt_rn(__longlong_as_double(top)));
        b1 = b2 = b3 = -1;
        i1 = i2 = i3 = kMcNone;
        for (int p = threadIdx.x; p < S; p += blockDim.x) {
          const double dp = M.dist[p];
          const long long bits = __double_as_longlong(dp);
          if (bits < 0 || bits > top || bits < top - 4) continue;
          if (__double_as_longlong(__dsqrt_rn(dp)) != rmax) continue;
          // key: the smaller index first; the low 3 bits carry top - bits
          mc_insert3(((1LL << 40) - (p0 + p)) * 8 + (top - bits), p0 + p, b1, i1, b2, i2, b3, i3);
        }
        long long Kb;
        int Ki;
        if (!collect(b1, i1, b2, i2, b3, i3, Kb, Ki)) return;
        const int bound = Kb >= 0 ? Ki : kMcNone;
        // the slots' squares from their keys
        if (threadIdx.x < kMcU && M.Ub[threadIdx.x] >= 0) M.Ub[threadIdx.x] = top - (M.Ub[threadIdx.x] & 7);
        __syncthreads();
        fetch_pairs(-1.0);
        if (warp == 0) {
          long long sb = lane < kMcU ? M.Ub[lane] : -1LL;
          const int si = lane < kMcU ? M.Ui[lane] : kMcNone;
          bool alive = sb >= 0, tied = alive;
          int kk = 0;
          while (kk < kMcU && nsel + kk < n) {
            const int mi = (int)__reduce_min_sync(0xffffffffu, alive && tied ? (unsigned)si : (unsigned)kMcNone);
            if (mi == kMcNone || mi >= bound) break;
            const int ws = __ffs(__ballot_sync(0xffffffffu, alive && si == mi)) - 1;
            if (lane == 0) piv_slot[kk] = ws;
            if (lane == ws) alive = false;
            if (alive) {
              const double sn = M.pairS[lane * kMcU + ws];
              if (__double_as_longlong(sn) < sb) {
                sb = __double_as_longlong(sn);
                if (tied) tied = __double_as_longlong(__dsqrt_rn(sn)) == rmax;
              }
            }
            ++kk;
          }
          build_pivots(kk);
          if (lane == 0) {
            s_k = kk;
            if (r == 0)
              for (int t = 0; t < kk; ++t) order[nsel + t] = P_i[t];
          }
        }
      }
      __syncthreads();
    }
    if (s_err) break;  // the same value in every CTA
    nsel += s_k;
  }
  // keep this CTA's shared memory alive until every remote read is done
  if constexpr (!kGrid)
    if (C > 1) cg::this_cluster().sync();
}

__global__ void __launch_bounds__(kMcThreads, 1) k_maximin_cluster(const RoProb* probs,
                                                                   const int32_t* plist,
                                                                   const double* Xs, int64_t* ord,
                                                                   int32_t* info) {
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int pid = plist[blockIdx.x / C];
  const RoProb& P = probs[pid];
  McRun Q = {};
  Q.X = Xs + P.xs_off;
  Q.n = P.n;
  Q.first = P.first;
  Q.order = ord + P.row_off;
  Q.info = info + 4 * pid;
  Q.d = P.d;
  Q.flags = P.flags;
  mc_run<false>(Q, C, (int)cluster.block_rank());
}

// grid form: one problem over a cooperative grid (one CTA per SM)
__global__ void __launch_bounds__(kMcThreads, 1) k_maximin_grid(McRun Q) {
  mc_run<true>(Q, (int)gridDim.x, (int)blockIdx.x);
}



// X, y, Z <- rows of X_e, y_e, Z_e in maximin order; Xso <- Xs in that order;
// grid row = problem
__global__ void k_ro_permute(const RoProb* probs, const int64_t* ord, const double* Xe,
                             const double* ye, const double* Ze, const double* Xs, double* X,
                             double* y, double* Z, double* Xso, int64_t* order_out) {
  const RoProb& P = probs[blockIdx.y];
  const int d = P.d, q = P.q;
  const int64_t* o = ord + P.row_off;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t src = o[i];
    for (int l = 0; l < d; ++l) {
      X[P.x_off + i * d + l] = Xe[P.xe_off + src * d + l];
      Xso[P.xs_off + P.n * d + i * d + l] = Xs[P.xs_off + src * d + l];
    }
    y[P.y_off + i] = ye[P.ye_off + src];
    for (int c = 0; c < q; ++c) Z[P.z_off + i * q + c] = Ze[P.ze_off + src * q + c];
    if (order_out) order_out[P.row_off + i] = src;
  }
}

// centred float32 rows (zero padded to DP) and their rounding bound for the
// kNN screen, centre = row 0 of the ordered problem; grid row = problem
__global__ void k_ro_knn_prep(const RoProb* probs, const double* Xso, float* v, float* B) {
  const RoProb& P = probs[blockIdx.y];
  const int d = P.d, DP = P.DP;
  const double* X = Xso + P.xs_off + P.n * d;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double e2 = 0.0;
    for (int l = 0; l < DP; ++l) {
      float f = 0.0f;
      if (l < d) {
        const double c = X[i * d + l] - X[l];
        f = __double2float_rn(c);
        e2 += c * c;
      }
      v[P.v_off + i * DP + l] = f;
    }
    B[P.row_off + i] = __double2float_ru(1.01 * 0x1p-24 * sqrt(e2));
  }
}

static size_t ro_align(size_t x) { return (x + 255) & ~(size_t)255; }

static int ro_max_smem() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

static int launch_maximin_cluster(int C, size_t smem, unsigned nclusters, const RoProb* probs,
                                  const int32_t* plist, const double* Xs, int64_t* ord,
                                  int32_t* info, cudaStream_t st);

// largest cluster the device can schedule with a full shared-memory budget
// per CTA (16 needs the non-portable cluster size; else 8)
static int g_mc_max_cluster = 0;
static int mc_max_cluster() {
  if (g_mc_max_cluster) return g_mc_max_cluster;
  int C = 8;
  if (cudaFuncSetAttribute(k_maximin_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
      cudaSuccess) {
    const int smem = ro_max_smem() - kMcStaticSmem;
    cudaFuncSetAttribute(k_maximin_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kMcMaxCluster);
    cfg.blockDim = dim3(kMcThreads);
    cfg.dynamicSmemBytes = (size_t)smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kMcMaxCluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclus = 0;
    if (cudaOccupancyMaxActiveClusters(&nclus, (void*)k_maximin_cluster, &cfg) == cudaSuccess && nclus > 0)
      C = kMcMaxCluster;
  }
  cudaGetLastError();  // a refused query leaves no error behind
  g_mc_max_cluster = C;
  return C;
}

// cluster size for n rows of dimension d: 1, 2, 4, 8 (or 16), or 0 when none fits
static int mc_cluster_size(int64_t n, int d, int maxsm) {
  const int64_t budget = (int64_t)maxsm - kMcStaticSmem - mc_fixed_bytes(d);
  const int cmax = mc_max_cluster();
  for (int C = 1; C <= cmax; C *= 2) {
    const int64_t per = (n + C - 1) / C;
    if (per * mc_point_bytes(d) <= budget) return C;
  }
  return 0;
}

struct RoPlan {
  std::vector<RoProb> probs;
  std::vector<KnnBatchProb> kprobs;
  std::vector<int32_t> plist[5];   // problems per cluster size 1, 2, 4, 8, 16
  size_t smem[5] = {0, 0, 0, 0, 0};
  std::vector<int2> tiles[8];      // kNN tiles per padded dimension
  int DPs[8] = {4, 8, 12, 16, 24, 32, 48, 64};
  int kcap[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int trows[8] = {128, 128, 128, 128, 128, 128, 128, 128};  // kNN tile heights
  int64_t nrows = 0, nxs = 0, nv = 0;
  // workspace layout
  size_t o_probs, o_kprobs, o_plist[5], o_tiles[8], o_ranges, o_xs, o_v, o_b, o_ord, total, staged;
};

static int ro_plan(const sv_reorder_desc* D, const sv_reorder_prob* hp, RoPlan& L) {
  const int maxsm = ro_max_smem();
  const int64_t np = D->nprob;
  L.probs.resize(np);
  L.kprobs.resize(np);
  for (int64_t i = 0; i < np; ++i) {
    const sv_reorder_prob& U = hp[i];
    if (U.n < 0 || U.d < 1 || U.d > D->dmax || U.d > 64 || U.q < 0 || U.m < 0 || U.m > D->ldnbr ||
        (U.n > 0 && (U.first < 0 || U.first >= U.n)) || U.n > 0x7fffffffLL)
      return SV_EINVAL;
    RoProb& R = L.probs[i];
    R.n = U.n;
    R.xe_off = U.xe_off;
    R.ye_off = U.ye_off;
    R.ze_off = U.ze_off;
    R.x_off = U.x_off;
    R.y_off = U.y_off;
    R.z_off = U.z_off;
    R.blk_off = U.blk_off;
    R.first = U.first;
    R.d = U.d;
    R.q = U.q;
    R.m = U.m;
    R.flags = U.flags & 3;  // maximin test aids: exact roots always (1), full scans (2)
    R.DP = knn_pad_dim(U.d);
    R.C = mc_cluster_size(U.n, U.d, maxsm);
    if (R.C == 0) return SV_EINVAL;
    R.xs_off = L.nxs;
    L.nxs += 2 * U.n * U.d;  // scaled rows, then the same rows in maximin order
    R.v_off = L.nv;
    L.nv += U.n * R.DP;
    R.row_off = L.nrows;
    L.nrows += U.n;
    KnnBatchProb& K = L.kprobs[i];
    K.xs_off = R.xs_off + U.n * U.d;
    K.v_off = R.v_off;
    K.row_off = R.row_off;
    K.n = U.n;
    K.blk_off = U.blk_off;
    K.d = U.d;
    K.m = U.m;
  }
  // largest problems first in every launch
  std::vector<int32_t> byn(np);
  for (int64_t i = 0; i < np; ++i) byn[i] = (int32_t)i;
  std::stable_sort(byn.begin(), byn.end(),
                   [&](int32_t a, int32_t b) { return L.probs[a].n > L.probs[b].n; });
  for (int32_t i : byn) {
    const RoProb& R = L.probs[i];
    if (R.n < 1) continue;
    const int g = R.C == 1 ? 0 : R.C == 2 ? 1 : R.C == 4 ? 2 : R.C == 8 ? 3 : 4;
    L.plist[g].push_back(i);
    const size_t sm = (size_t)((R.n + R.C - 1) / R.C) * (size_t)mc_point_bytes(R.d) +
                      (size_t)mc_fixed_bytes(R.d);
    L.smem[g] = std::max(L.smem[g], sm);
    if (R.m < 1 || R.n < 2) continue;
    int gi = 0;
    while (L.DPs[gi] != R.DP) ++gi;
    L.kcap[gi] = std::max(L.kcap[gi], R.m);
  }
  // kNN tiles (largest problems and, within one, the last rows first), of the
  // height the search of each padded dimension takes
  for (int g = 0; g < 8; ++g)
    L.trows[g] = L.kcap[g] > 0 ? knn_batched_tile_rows(L.DPs[g], L.kcap[g]) : 128;
  for (int32_t i : byn) {
    const RoProb& R = L.probs[i];
    if (R.n < 1 || R.m < 1 || R.n < 2) continue;
    int gi = 0;
    while (L.DPs[gi] != R.DP) ++gi;
    const int64_t nt = (R.n + L.trows[gi] - 1) / L.trows[gi];
    for (int64_t t = nt - 1; t >= 0; --t) L.tiles[gi].push_back(make_int2(i, (int)t));
  }
  // workspace: staged tables first, then the arrays
  size_t off = 0;
  L.o_probs = off;
  off = ro_align(off + sizeof(RoProb) * (size_t)np);
  L.o_kprobs = off;
  off = ro_align(off + sizeof(KnnBatchProb) * (size_t)np);
  for (int g = 0; g < 5; ++g) {
    L.o_plist[g] = off;
    off = ro_align(off + sizeof(int32_t) * L.plist[g].size());
  }
  for (int g = 0; g < 8; ++g) {
    L.o_tiles[g] = off;
    off = ro_align(off + sizeof(int2) * L.tiles[g].size());
  }
  L.o_ranges = off;
  off = ro_align(off + sizeof(double) * (size_t)np * D->dmax);
  L.staged = off;
  L.o_xs = off;
  off = ro_align(off + sizeof(double) * (size_t)L.nxs);
  L.o_v = off;
  off = ro_align(off + sizeof(float) * (size_t)L.nv);
  L.o_b = off;
  off = ro_align(off + sizeof(float) * (size_t)L.nrows);
  L.o_ord = off;
  off = ro_align(off + sizeof(int64_t) * (size_t)L.nrows);
  L.total = off;
  return SV_OK;
}

static int launch_maximin_cluster(int C, size_t smem, unsigned nclusters, const RoProb* probs,
                                  const int32_t* plist, const double* Xs, int64_t* ord,
                                  int32_t* info, cudaStream_t st) {
  SV_CUDA_TRY(cudaFuncSetAttribute(k_maximin_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nclusters * (unsigned)C);
  cfg.blockDim = dim3(kMcThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SV_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_maximin_cluster, probs, plist, Xs, ord, info));
  return SV_OK;
}

// One problem through the cluster kernel (sv_maximin_order for n that fits
// one cluster).  ws: 256 bytes of device scratch.
int maximin_cluster_single(const double* X, int64_t n, int d, int64_t first, int64_t* order,
                           int32_t* info, char* ws, int flags, cudaStream_t st) {
  const int C = mc_cluster_size(n, d, ro_max_smem());
  if (C == 0) return SV_EINVAL;
  struct {
    RoProb p;
    int32_t plist[4];
  } h;
  memset(&h, 0, sizeof(h));
  h.p.n = n;
  h.p.first = first;
  h.p.d = d;
  h.p.C = C;
  h.p.flags = flags & 3;
  SV_CUDA_TRY(cudaMemcpyAsync(ws, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  const size_t smem = (size_t)((n + C - 1) / C) * (size_t)mc_point_bytes(d) + (size_t)mc_fixed_bytes(d);
  return launch_maximin_cluster(C, smem, 1, (const RoProb*)ws, (const int32_t*)(ws + sizeof(RoProb)),
                                X, order, info, st);
}

// grid form: CTAs (one per SM at most, >= 64 rows each) and rows per CTA
static int mg_plan(int64_t n, int d, int& G, int& per, size_t& smem) {
  const int nsm = sv_num_sms();
  const int64_t budget = (int64_t)ro_max_smem() - kMcStaticSmem - mc_fixed_bytes(d);
  G = (int)std::min<int64_t>(nsm, std::max<int64_t>(1, (n + 63) / 64));
  per = (int)((n + G - 1) / G);
  if ((int64_t)per * mc_point_bytes(d, true) > budget) return SV_EINVAL;
  smem = (size_t)per * (size_t)mc_point_bytes(d, true) + (size_t)mc_fixed_bytes(d);
  return SV_OK;
}

size_t maximin_grid_workspace_bytes() {
  const size_t g2 = 2 * (size_t)sv_num_sms();
  return ro_align(g2 * 32 * 8) + ro_align(g2 * 32 * 4) + ro_align(g2 * 8) + ro_align(g2 * 4) + 256;
}

int64_t maximin_grid_max_rows(int d) {
  if (d < 1 || d > 64) return 0;
  const int64_t budget = (int64_t)ro_max_smem() - kMcStaticSmem - mc_fixed_bytes(d);
  return (int64_t)sv_num_sms() * (budget / mc_point_bytes(d, true));
}

// One problem through the grid form (a cooperative launch, one CTA per SM).
int maximin_grid_single(const double* X, int64_t n, int d, int64_t first, int64_t* order,
                        int32_t* info, char* ws, size_t ws_bytes, int flags, cudaStream_t st) {
  int G = 0, per = 0;
  size_t smem = 0;
  if (mg_plan(n, d, G, per, smem) != SV_OK) return SV_EINVAL;
  if (ws_bytes < maximin_grid_workspace_bytes()) return SV_ENOSPC;
  SV_CUDA_TRY(cudaFuncSetAttribute(k_maximin_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int active = 0;
  SV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&active, k_maximin_grid, kMcThreads, smem));
  if (active < 1 || G > active * sv_num_sms()) return SV_EINVAL;
  const size_t g2 = 2 * (size_t)sv_num_sms();
  McRun Q = {};
  Q.X = X;
  Q.n = n;
  Q.first = first;
  Q.order = order;
  Q.info = info;
  Q.d = d;
  Q.flags = flags & 3;
  Q.skip_first_arrival = (flags & 8) ? 1 : 0;
  Q.spin_limit = (flags & 8) ? SV_SPIN_LIMIT_TEST : SV_SPIN_LIMIT;
  size_t off = 0;
  Q.gl_b = (long long*)(ws + off);
  off += ro_align(g2 * 32 * 8);
  Q.gl_i = (int*)(ws + off);
  off += ro_align(g2 * 32 * 4);
  Q.gl_Kb = (long long*)(ws + off);
  off += ro_align(g2 * 8);
  Q.gl_Ki = (int*)(ws + off);
  off += ro_align(g2 * 4);
  Q.arrive = (unsigned*)(ws + off);
  SV_CUDA_TRY(cudaMemsetAsync(Q.arrive, 0, sizeof(unsigned), st));
  void* args[] = {&Q};
  SV_CUDA_TRY(cudaLaunchCooperativeKernel((void*)k_maximin_grid, dim3((unsigned)G), dim3(kMcThreads), args,
                                          smem, st));
  return SV_OK;
}

// Helper streams for launches that do not depend on one another (the
// maximin launches of the cluster sizes, the neighbour-search launches of the
// dimension classes): each launch lasts as long as its largest problem, so
// running them side by side costs the longest instead of the sum.  Created
// once per device; every call forks them off its own stream with an event and
// joins them back before the work that needs their results.  Calls from
// several host threads at once may serialise on the helpers, never misorder.
constexpr int kRoHelpers = 7;
constexpr int kRoMaxDevices = 64;
static cudaStream_t g_ro_helper[kRoMaxDevices][kRoHelpers];
static bool g_ro_helper_made[kRoMaxDevices];
static std::mutex g_ro_mu;

static int ro_helper_streams(cudaStream_t* out) {
  std::lock_guard<std::mutex> lk(g_ro_mu);
  int dev = 0;
  SV_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kRoMaxDevices) return SV_EINVAL;
  if (!g_ro_helper_made[dev]) {
    for (int i = 0; i < kRoHelpers; ++i)
      SV_CUDA_TRY(cudaStreamCreateWithFlags(&g_ro_helper[dev][i], cudaStreamNonBlocking));
    g_ro_helper_made[dev] = true;
  }
  for (int i = 0; i < kRoHelpers; ++i) out[i] = g_ro_helper[dev][i];
  return SV_OK;
}

// helpers hs[0 .. n-1] wait for the work enqueued on st so far
static int ro_fork(cudaStream_t st, const cudaStream_t* hs, int n) {
  if (n <= 0) return SV_OK;
  cudaEvent_t e;
  SV_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  SV_CUDA_TRY(cudaEventRecord(e, st));
  for (int i = 0; i < n; ++i) SV_CUDA_TRY(cudaStreamWaitEvent(hs[i], e, 0));
  SV_CUDA_TRY(cudaEventDestroy(e));
  return SV_OK;
}

// st waits for the work enqueued on hs[0 .. n-1] so far
static int ro_join(cudaStream_t st, const cudaStream_t* hs, int n) {
  for (int i = 0; i < n; ++i) {
    cudaEvent_t e;
    SV_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    SV_CUDA_TRY(cudaEventRecord(e, hs[i]));
    SV_CUDA_TRY(cudaStreamWaitEvent(st, e, 0));
    SV_CUDA_TRY(cudaEventDestroy(e));
  }
  return SV_OK;
}

int64_t maximin_cluster_max_rows(int d) {
  if (d < 1 || d > 64) return 0;
  const int64_t budget = (int64_t)ro_max_smem() - kMcStaticSmem - mc_fixed_bytes(d);
  return (int64_t)mc_max_cluster() * (budget / mc_point_bytes(d));
}

}  // namespace sv

using namespace sv;

extern "C" int64_t sv_maximin_cluster_max_rows(int32_t d) { return maximin_cluster_max_rows(d); }

extern "C" size_t sv_reorder_batched_workspace_bytes(const sv_reorder_desc* D,
                                                     const sv_reorder_prob* probs) {
  if (!D || (D->nprob > 0 && !probs) || D->nprob < 0) return 0;
  RoPlan L;
  if (ro_plan(D, probs, L) != SV_OK) return 0;
  return L.total;
}

extern "C" int sv_reorder_batched(const sv_reorder_desc* D, const sv_reorder_prob* probs,
                                  const double* ranges, const double* Xe, const double* ye,
                                  const double* Ze, double* X, double* y, double* Z, int32_t* nbr,
                                  int64_t* order, int32_t* info, void* workspace,
                                  size_t workspace_bytes, sv_stream_t stream) {
  if (!D || D->nprob < 0 || D->dmax < 1 || D->dmax > 64 || D->ldnbr < 0 || !info) return SV_EINVAL;
  if (D->nprob == 0) return SV_OK;
  if (!probs || !ranges || !Xe || !ye || !X || !y) return SV_EINVAL;
  RoPlan L;
  int rc = ro_plan(D, probs, L);
  if (rc != SV_OK) return rc;
  bool anyq = false, anym = false;
  for (const RoProb& R : L.probs) {
    anyq = anyq || R.q > 0;
    anym = anym || (R.m > 0 && R.n > 1);
  }
  if ((anyq && (!Ze || !Z)) || (anym && (!nbr || D->ldnbr < 1))) return SV_EINVAL;
  if (!workspace || workspace_bytes < L.total) return SV_ENOSPC;
  cudaStream_t st = (cudaStream_t)stream;
  char* ws = (char*)workspace;
  const int np = (int)D->nprob;

  // one staged copy of every table
  std::vector<char> host(L.staged, 0);
  memcpy(host.data() + L.o_probs, L.probs.data(), sizeof(RoProb) * np);
  memcpy(host.data() + L.o_kprobs, L.kprobs.data(), sizeof(KnnBatchProb) * np);
  for (int g = 0; g < 5; ++g)
    if (!L.plist[g].empty())
      memcpy(host.data() + L.o_plist[g], L.plist[g].data(), sizeof(int32_t) * L.plist[g].size());
  for (int g = 0; g < 8; ++g)
    if (!L.tiles[g].empty())
      memcpy(host.data() + L.o_tiles[g], L.tiles[g].data(), sizeof(int2) * L.tiles[g].size());
  memcpy(host.data() + L.o_ranges, ranges, sizeof(double) * (size_t)np * D->dmax);
  SV_CUDA_TRY(cudaMemcpyAsync(ws, host.data(), L.staged, cudaMemcpyHostToDevice, st));
  const RoProb* dprobs = (const RoProb*)(ws + L.o_probs);
  double* Xs = (double*)(ws + L.o_xs);
  float* v = (float*)(ws + L.o_v);
  float* B = (float*)(ws + L.o_b);
  int64_t* ord = (int64_t*)(ws + L.o_ord);

  k_ro_info_init<<<(np + 255) / 256, 256, 0, st>>>(info, np);
  SV_CUDA_TRY(cudaGetLastError());
  int64_t maxn = 0;
  for (const RoProb& R : L.probs) maxn = std::max(maxn, R.n);
  int64_t gx = (maxn * D->dmax + 255) / 256;
  gx = std::max<int64_t>(1, std::min<int64_t>(gx, 64));
  k_ro_scale<<<dim3((unsigned)gx, np), 256, 0, st>>>(dprobs, (const double*)(ws + L.o_ranges),
                                                      D->dmax, Xe, Xs);
  SV_CUDA_TRY(cudaGetLastError());

  cudaStream_t hs[kRoHelpers];
  if ((rc = ro_helper_streams(hs)) != SV_OK) return rc;
  // maximin: one launch per cluster size, side by side (the first on st)
  {
    int used = 0;
    for (int g = 0; g < 5; ++g) used += L.plist[g].empty() ? 0 : 1;
    const int nh = used > 1 ? used - 1 : 0;
    if ((rc = ro_fork(st, hs, nh)) != SV_OK) return rc;
    int slot = 0;
    for (int g = 0; g < 5; ++g) {
      if (L.plist[g].empty()) continue;
      cudaStream_t sg = slot == 0 ? st : hs[slot - 1];
      ++slot;
      rc = launch_maximin_cluster(1 << g, L.smem[g], (unsigned)L.plist[g].size(), dprobs,
                                  (const int32_t*)(ws + L.o_plist[g]), (const double*)Xs, ord, info, sg);
      if (rc != SV_OK) return rc;
    }
    if ((rc = ro_join(st, hs, nh)) != SV_OK) return rc;
  }

  gx = (maxn + 255) / 256;
  gx = std::max<int64_t>(1, std::min<int64_t>(gx, 64));
  k_ro_permute<<<dim3((unsigned)gx, np), 256, 0, st>>>(dprobs, ord, Xe, ye, Ze, Xs, X, y, Z, Xs, order);
  SV_CUDA_TRY(cudaGetLastError());
  k_ro_knn_prep<<<dim3((unsigned)gx, np), 256, 0, st>>>(dprobs, Xs, v, B);
  SV_CUDA_TRY(cudaGetLastError());
  // neighbour search: one launch per dimension class, side by side
  {
    int used = 0;
    for (int g = 0; g < 8; ++g) used += L.tiles[g].empty() ? 0 : 1;
    const int nh = used > 1 ? used - 1 : 0;
    if ((rc = ro_fork(st, hs, nh)) != SV_OK) return rc;
    int slot = 0;
    for (int g = 0; g < 8; ++g) {
      if (L.tiles[g].empty()) continue;
      cudaStream_t sg = slot == 0 ? st : hs[slot - 1];
      ++slot;
      rc = launch_knn_batched(L.DPs[g], (const KnnBatchProb*)(ws + L.o_kprobs),
                              (const int2*)(ws + L.o_tiles[g]), (int64_t)L.tiles[g].size(), Xs, v, B,
                              nbr, D->ldnbr, L.kcap[g], sg);
      if (rc != SV_OK) return rc;
    }
    if ((rc = ro_join(st, hs, nh)) != SV_OK) return rc;
  }
  return SV_OK;
}
