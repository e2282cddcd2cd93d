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
//  * argmax: candidates compare squared bits, then indices.  Distinct squares
//    can round to the same root only within a few ulps, so whenever a loser
//    within 4 ulps of the winner has a smaller index, the step resolves its
//    winner again from the exact roots of every point within 4 ulps (one
//    more cluster exchange; rare).  Per step the CTAs' candidates (distance bits, index)
// meet through distributed shared memory after one hardware cluster barrier
// (double-buffered by step parity), so there is no spin-wait at all.
// Problems are grouped by cluster size (1, 2, 4 or 8 CTAs, the smallest
// whose shared memory holds the problem), one launch per group, largest
// problems first.
#include <cooperative_groups.h>

#include <algorithm>
#include <vector>

#include "sv_reorder.cuh"

namespace cg = cooperative_groups;

namespace sv {

constexpr int kMcThreads = 512;
// static shared memory of k_maximin_cluster (3.7 KB), rounded up: the
// capacity of a cluster is computed from what is left of 227 KB
constexpr int kMcStaticSmem = 4096;
constexpr int kMcMaxCluster = 16;

struct RoProb {
  int64_t n, xe_off, ye_off, ze_off, x_off, y_off, z_off, blk_off, first;
  int64_t xs_off;   // doubles: this call's scaled rows (and their maximin-order copy)
  int64_t v_off;    // floats: centred float32 rows [n][DP]
  int64_t row_off;  // rows: order, B
  int32_t d, q, m, DP, C, pad;
};

// per-point shared memory of the cluster maximin: dist f64, exact coordinates
// f64[d], thr f32, B f32, float32 centred coordinates f32[d]
__host__ __device__ inline int64_t mc_point_bytes(int d) { return 16 + 12 * (int64_t)d; }

__device__ __forceinline__ void cand_better(long long ob, long long oi, long long& bb, long long& bi) {
  if (ob > bb || (ob == bb && oi < bi)) {
    bb = ob;
    bi = oi;
  }
}

// merge of (squared-distance bits, index, near-tie flag) candidates: larger
// bits win, then the smaller index; a loser within 4 ulps below the winner
// with a smaller index may share the winner's square root
__device__ __forceinline__ void cand_merge(long long ob, long long oi, int of, long long& bb,
                                           long long& bi, int& bf) {
  const bool ow = ob > bb || (ob == bb && oi < bi);
  const long long wb = ow ? ob : bb, wi = ow ? oi : bi;
  const long long lb = ow ? bb : ob, li = ow ? bi : oi;
  int f = of | bf;
  if (lb >= 0 && wb - lb <= 4 && li < wi) f = 1;
  bb = wb;
  bi = wi;
  bf = f;
}

// float32 screening threshold from a squared distance: an upper bound of
// (fl(sqrt(s)) (1 + (d+4) 2^-53) + B_p) (1 + 2^-40), d <= 64
__device__ __forceinline__ float thr_sq(double s, float Bp) {
  const float r = __fsqrt_ru(__double2float_ru(s));  // >= sqrt(s)
  return __fmul_ru(__fadd_ru(r, Bp), 1.0f + 0x1p-20f);
}

// (1+2^-24)^(d+2) (1+2^-20) as a float32 rounded up
__device__ __forceinline__ float mc_growth(int d) {
  double g = 1.0;
  for (int i = 0; i < d + 2; ++i) g *= (1.0 + 0x1p-24);
  return __double2float_ru(g * (1.0 + 0x1p-20));
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

// warp 0: exact pivot row, its float32 image and rounding bound
__device__ __forceinline__ void mc_load_pivot(const double* X, long long j, int d, const double* cen,
                                              double* xj, float* vj, float* Bj) {
  const int lane = threadIdx.x & 31;
  double e2 = 0.0;
  for (int l = lane; l < d; l += 32) {
    const double x = X[j * d + l];
    const double c = x - cen[l];
    xj[l] = x;
    vj[l] = __double2float_rn(c);
    e2 += c * c;
  }
  for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
  if (lane == 0) *Bj = __double2float_ru(1.01 * 0x1p-24 * sqrt(e2));
}

// warp 0: pivot row from a row of d doubles (shared or distributed shared memory)
__device__ __forceinline__ void mc_pivot_from(const double* src, int d, const double* cen, double* xj,
                                              float* vj, float* Bj) {
  const int lane = threadIdx.x & 31;
  double e2 = 0.0;
  for (int l = lane; l < d; l += 32) {
    const double x = src[l];
    const double c = x - cen[l];
    xj[l] = x;
    vj[l] = __double2float_rn(c);
    e2 += c * c;
  }
  for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
  if (lane == 0) *Bj = __double2float_ru(1.01 * 0x1p-24 * sqrt(e2));
}

__global__ void __launch_bounds__(kMcThreads) k_maximin_cluster(const RoProb* probs,
                                                                const int32_t* plist,
                                                                const double* Xs, int64_t* ord,
                                                                int32_t* info) {
  extern __shared__ unsigned char smraw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int r = (int)cluster.block_rank();
  const int pid = plist[blockIdx.x / C];
  const RoProb& P = probs[pid];
  const int64_t n = P.n;
  const int d = P.d;
  const double* X = Xs + P.xs_off;
  int64_t* order = ord + P.row_off;
  const int64_t per = (n + C - 1) / C;
  const int64_t p0 = (int64_t)r * per;
  const int64_t p1 = min(n, p0 + per);
  const int S = (int)max((int64_t)0, p1 - p0);
  const int Sc = (int)per;
  double* dist = (double*)smraw;
  double* xs = dist + Sc;  // exact coordinates of the CTA's points, row-major
  float* thr = (float*)(xs + (int64_t)Sc * d);
  float* Bp = thr + Sc;
  float* v = Bp + Sc;
  __shared__ double xj[64], cen[64];
  __shared__ float vj[64];
  __shared__ float Bj_f;
  __shared__ long long red_bits[kMcThreads / 32], red_idx[kMcThreads / 32];
  __shared__ int red_flag[kMcThreads / 32];
  __shared__ long long cand_bits[2], cand_idx[2];
  __shared__ int cand_flag[2];
  __shared__ double cand_x[2][64];  // the CTA candidate's exact coordinates
  __shared__ long long res_bits[2], res_idx[2];  // exact-root resolution
  __shared__ double res_x[2][64];
  __shared__ long long s_pivot;
  __shared__ int s_flag;
  const bool force_roots = (P.pad & 1) != 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarp = blockDim.x >> 5;
  const float growth = mc_growth(d);

  // centre: the first row (any shift serves the float32 screen)
  for (int l = threadIdx.x; l < d; l += blockDim.x) cen[l] = X[P.first * d + l];
  __syncthreads();
  for (int e = threadIdx.x; e < S * d; e += blockDim.x) xs[e] = X[p0 * d + e];
  for (int p = threadIdx.x; p < S; p += blockDim.x) {
    const double* xp = X + (p0 + p) * d;
    double e2 = 0.0;
    for (int l = 0; l < d; ++l) {
      const double c = xp[l] - cen[l];
      v[l * Sc + p] = __double2float_rn(c);
      e2 += c * c;
    }
    Bp[p] = __double2float_ru(1.01 * 0x1p-24 * sqrt(e2));
    dist[p] = __longlong_as_double(0x7ff0000000000000LL);  // +inf: first pass is exact
    thr[p] = __int_as_float(0x7f800000);
  }
  if (threadIdx.x == 0) {
    s_pivot = P.first;
    if (r == 0) order[0] = P.first;
  }
  if (warp == 0) mc_load_pivot(X, P.first, d, cen, xj, vj, &Bj_f);
  __syncthreads();

  for (int64_t t = 0; t + 1 < n; ++t) {
    const long long j = s_pivot;
    const float bj = Bj_f;
    long long best_bits = -1LL;  // below every non-negative double
    long long best_idx = 0x7fffffffffffffffLL;
    int best_flag = 0;
    for (int p = threadIdx.x; p < S; p += blockDim.x) {
      double dp = dist[p];  // squared distance
      if (__double_as_longlong(dp) < 0) continue;  // already ordered (ordering.py:50-51)
      const long long gp = p0 + p;
      if (gp == j) {
        dist[p] = -1.0;  // ordering.py:58
        continue;
      }
      float s32 = 0.0f;
      for (int l = 0; l < d; ++l) {
        const float df = __fsub_rn(v[l * Sc + p], vj[l]);
        s32 = __fmaf_rn(df, df, s32);
      }
      const float tb = __fadd_ru(thr[p], bj);
      const float bound = __fmul_ru(__fmul_ru(tb, tb), growth);
      if (!(s32 >= bound)) {
        // possible update: the reference's squared distance (ordering.py:52-57)
        const double sn = sqdist_exact(xs + (int64_t)p * d, xj, d);
        if (__double_as_longlong(sn) < __double_as_longlong(dp)) {
          dp = sn;
          dist[p] = sn;
          thr[p] = thr_sq(sn, Bp[p]);
        }
      }
      const long long bits = __double_as_longlong(dp);
      if (bits <= 0x7ff0000000000000LL) cand_merge(bits, gp, 0, best_bits, best_idx, best_flag);
    }
    for (int o = 16; o > 0; o >>= 1)
      cand_merge(__shfl_xor_sync(0xffffffffu, best_bits, o), __shfl_xor_sync(0xffffffffu, best_idx, o),
                 __shfl_xor_sync(0xffffffffu, best_flag, o), best_bits, best_idx, best_flag);
    if (lane == 0) {
      red_bits[warp] = best_bits;
      red_idx[warp] = best_idx;
      red_flag[warp] = best_flag;
    }
    __syncthreads();
    const int par = (int)(t & 1);
    long long bb = -1LL, bi = 0x7fffffffffffffffLL;
    int bf = 0;
    if (warp == 0) {
      if (lane < nwarp) {
        bb = red_bits[lane];
        bi = red_idx[lane];
        bf = red_flag[lane];
      }
      for (int o = 16; o > 0; o >>= 1)
        cand_merge(__shfl_xor_sync(0xffffffffu, bb, o), __shfl_xor_sync(0xffffffffu, bi, o),
                   __shfl_xor_sync(0xffffffffu, bf, o), bb, bi, bf);
      if (C > 1) {
        if (lane == 0) {
          cand_bits[par] = bb;
          cand_idx[par] = bi;
          cand_flag[par] = bf;
        }
        if (bi != 0x7fffffffffffffffLL)
          for (int l = lane; l < d; l += 32) cand_x[par][l] = xs[(bi - p0) * d + l];
      }
    }
    if (C > 1) {
      // every CTA's candidate of this step is visible after the barrier; the
      // slots of step t are rewritten at t + 2, after the next barrier, which
      // no CTA passes before all have read them
      cluster.sync();
      if (warp == 0) {
        bb = -1LL;
        bi = 0x7fffffffffffffffLL;
        bf = 0;
        if (lane < C) {
          bb = cluster.map_shared_rank(cand_bits, lane)[par];
          bi = cluster.map_shared_rank(cand_idx, lane)[par];
          bf = cluster.map_shared_rank(cand_flag, lane)[par];
        }
        for (int o = 16; o > 0; o >>= 1)
          cand_merge(__shfl_xor_sync(0xffffffffu, bb, o), __shfl_xor_sync(0xffffffffu, bi, o),
                     __shfl_xor_sync(0xffffffffu, bf, o), bb, bi, bf);
      }
    }
    if (threadIdx.x == 0) {
      s_pivot = bi;
      s_flag = (bf || force_roots) && bi != 0x7fffffffffffffffLL;
      red_bits[0] = bb;  // the winner's squared bits for the resolution below
    }
    __syncthreads();
    const double* src = nullptr;  // the winner's exact row (warp 0)
    if (s_flag) {
      // exact-root resolution among the points within 4 ulps of the winner
      const long long wb = red_bits[0];
      long long rb = -1LL, ri = 0x7fffffffffffffffLL;
      for (int p = threadIdx.x; p < S; p += blockDim.x) {
        const long long bits = __double_as_longlong(dist[p]);
        if (bits < 0 || bits > wb || bits < wb - 4) continue;
        const long long rbits = __double_as_longlong(__dsqrt_rn(dist[p]));
        if (rbits > rb || (rbits == rb && p0 + p < ri)) {
          rb = rbits;
          ri = p0 + p;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const long long ob = __shfl_xor_sync(0xffffffffu, rb, o), oi = __shfl_xor_sync(0xffffffffu, ri, o);
        if (ob > rb || (ob == rb && oi < ri)) {
          rb = ob;
          ri = oi;
        }
      }
      __syncthreads();  // red_bits[0] has been read by every thread
      if (lane == 0) {
        red_bits[warp] = rb;
        red_idx[warp] = ri;
      }
      __syncthreads();
      if (warp == 0) {
        rb = -1LL;
        ri = 0x7fffffffffffffffLL;
        if (lane < nwarp) {
          rb = red_bits[lane];
          ri = red_idx[lane];
        }
        for (int o = 16; o > 0; o >>= 1) {
          const long long ob = __shfl_xor_sync(0xffffffffu, rb, o), oi = __shfl_xor_sync(0xffffffffu, ri, o);
          if (ob > rb || (ob == rb && oi < ri)) {
            rb = ob;
            ri = oi;
          }
        }
        if (C > 1) {
          if (lane == 0) {
            res_bits[par] = rb;
            res_idx[par] = ri;
          }
          if (ri != 0x7fffffffffffffffLL)
            for (int l = lane; l < d; l += 32) res_x[par][l] = xs[(ri - p0) * d + l];
        }
      }
      if (C > 1) {
        cluster.sync();
        if (warp == 0) {
          rb = -1LL;
          ri = 0x7fffffffffffffffLL;
          if (lane < C) {
            rb = cluster.map_shared_rank(res_bits, lane)[par];
            ri = cluster.map_shared_rank(res_idx, lane)[par];
          }
          for (int o = 16; o > 0; o >>= 1) {
            const long long ob = __shfl_xor_sync(0xffffffffu, rb, o), oi = __shfl_xor_sync(0xffffffffu, ri, o);
            if (ob > rb || (ob == rb && oi < ri)) {
              rb = ob;
              ri = oi;
            }
          }
        }
      }
      if (warp == 0) {
        bi = ri;
        const int owner = (int)(bi / per);
        src = (C == 1 || owner == r) ? xs + (bi - p0) * d : cluster.map_shared_rank(&res_x[par][0], owner);
      }
    } else if (warp == 0 && bi != 0x7fffffffffffffffLL) {
      const int owner = (int)(bi / per);
      src = (C == 1 || owner == r) ? xs + (bi - p0) * d : cluster.map_shared_rank(&cand_x[par][0], owner);
    }
    if (warp == 0) {
      if (lane == 0) s_pivot = bi;
      if (bi != 0x7fffffffffffffffLL) {
        if (r == 0 && lane == 0) order[t + 1] = bi;
        mc_pivot_from(src, d, cen, xj, vj, &Bj_f);
      } else if (r == 0 && lane == 0) {
        // no finite candidate left (NaN inputs): report and stop
        set_error(info + 4 * pid + SV_INFO_STATUS, SV_EINVAL);
        info[4 * pid + SV_INFO_BLOCK] = (int)t;
      }
    }
    __syncthreads();
    if (s_pivot == 0x7fffffffffffffffLL) break;  // the same value in every CTA
  }
  // keep this CTA's shared memory alive until every remote read is done
  if (C > 1) cluster.sync();
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
  const int64_t budget = (int64_t)maxsm - kMcStaticSmem;
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
    R.pad = U.flags & 1;  // bit 0: resolve every maximin step from exact roots
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
    const size_t sm = (size_t)((R.n + R.C - 1) / R.C) * (size_t)mc_point_bytes(R.d);
    L.smem[g] = std::max(L.smem[g], sm);
    if (R.m < 1 || R.n < 2) continue;
    int gi = 0;
    while (L.DPs[gi] != R.DP) ++gi;
    L.kcap[gi] = std::max(L.kcap[gi], R.m);
    const int64_t nt = (R.n + 127) / 128;
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
                           int32_t* info, char* ws, cudaStream_t st) {
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
  SV_CUDA_TRY(cudaMemcpyAsync(ws, &h, sizeof(h), cudaMemcpyHostToDevice, st));
  const size_t smem = (size_t)((n + C - 1) / C) * (size_t)mc_point_bytes(d);
  return launch_maximin_cluster(C, smem, 1, (const RoProb*)ws, (const int32_t*)(ws + sizeof(RoProb)),
                                X, order, info, st);
}

int64_t maximin_cluster_max_rows(int d) {
  if (d < 1 || d > 64) return 0;
  const int64_t budget = (int64_t)ro_max_smem() - kMcStaticSmem;
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

  // maximin: one launch per cluster size
  for (int g = 0; g < 5; ++g) {
    if (L.plist[g].empty()) continue;
    rc = launch_maximin_cluster(1 << g, L.smem[g], (unsigned)L.plist[g].size(), dprobs,
                                (const int32_t*)(ws + L.o_plist[g]), (const double*)Xs, ord, info, st);
    if (rc != SV_OK) return rc;
  }

  gx = (maxn + 255) / 256;
  gx = std::max<int64_t>(1, std::min<int64_t>(gx, 64));
  k_ro_permute<<<dim3((unsigned)gx, np), 256, 0, st>>>(dprobs, ord, Xe, ye, Ze, Xs, X, y, Z, Xs, order);
  SV_CUDA_TRY(cudaGetLastError());
  k_ro_knn_prep<<<dim3((unsigned)gx, np), 256, 0, st>>>(dprobs, Xs, v, B);
  SV_CUDA_TRY(cudaGetLastError());
  for (int g = 0; g < 8; ++g) {
    if (L.tiles[g].empty()) continue;
    rc = launch_knn_batched(L.DPs[g], (const KnnBatchProb*)(ws + L.o_kprobs),
                            (const int2*)(ws + L.o_tiles[g]), (int64_t)L.tiles[g].size(), Xs, v, B,
                            nbr, D->ldnbr, L.kcap[g], st);
    if (rc != SV_OK) return rc;
  }
  return SV_OK;
}
