// Exact maximin ordering for any n, by a tree over the points: ordering.py:
// 27-73 (maximin_order / _maximin_core), bit for bit.  The cluster and grid
// forms (sv_reorder.cu) keep every point in shared memory and visit all of
// them in every pass (O(n^2 d) work, at most 581k rows at d = 10); this form
// keeps the points in global memory and visits only what a pass can change.
//
// It runs the pass algorithm of k_maximin_cluster (many pivots per pass, each
// provably the reference's next choice, a tie pass when none is certain)
// with every O(n) step replaced by a descent of a 32-ary tree, on the
// observation of Schaefer, Sullivan and Owhadi (2021) that a pivot at
// distance l from the ordered set can lower only points within l of it:
//  * the points are put in k-d order (segments halved along their widest
//    coordinate, level by level, by radix sorts of (segment, coordinate)
//    keys); 32 consecutive points form a leaf, 32 consecutive nodes a node
//    of the next level, up to a level of at most 32 nodes.  A node at level
//    h holds the points [32^h j, 32^h (j+1));
//  * a node keeps the bounding box of its points' float32 images, an upper
//    bound of its live points' float32 screening thresholds and its largest
//    point key (squared-distance bits, then the smaller row index);
//  * apply: a pass's pivots descend the tree; a node is left for a pivot when
//    a rigorous lower bound of the squared distance from the pivot's image to
//    the node's box is beyond the node's threshold bound (the float32 screen
//    of the point kernels, applied to the box); the points of the leaves
//    reached take the screen and the exact update of the point kernels;
//    the leaves touched and their ancestors are keyed again;
//  * candidates: the 31 largest point keys lie in the 31 leaves with the
//    largest keys, which lie below the 31 level-2 nodes with the largest keys,
//    and so on: 31 nodes per level from the top, then the points of 31
//    leaves; R, the largest key of anything not chosen, is the largest 32nd
//    key over the levels;
//  * tie pass: the subtrees whose largest key lies within 4 ulps of the top.
// One thread-block cluster (16 CTAs of 1024 threads where the device allows,
// else 8 or fewer) runs the whole ordering, phases separated by the hardware
// cluster barrier (no spin-wait of any kind); the tree lives in global memory.
#include <cooperative_groups.h>

#include <cub/device/device_radix_sort.cuh>

#include "sv_maximin_ops.cuh"
#include "sv_reorder.cuh"

namespace cg = cooperative_groups;

namespace sv {

constexpr int kMtThreads = 1024;
constexpr int kMtWarps = kMtThreads / 32;
constexpr int kMtMaxLevels = 7;  // 32^7 > 2^31 rows
constexpr int kMtLeaf = 32;      // points per leaf, children per node

struct MtRun {
  int64_t n;
  int d, DV, H, flags;
  int hdesc;             // the level the descent starts at
  int hcand;             // the level the candidate rounds start at (0: the rows)
  int cdist;             // the first candidate round split over the cluster's CTAs
  int64_t first;         // original index of the first row (ordering.py:72)
  const int* first_pos;  // its position in tree order (device word)
  int64_t* order;
  int32_t* info;
  const double* xs;      // [n][d] exact rows, tree order
  const float* v;        // [n][DV] float32 images centred on the first row, zero padded
  const float* Bp;       // [n] image rounding bounds
  const int* gidx;       // [n] original row index of each position
  const int* posof;      // [n] position of each original row
  double* dist;          // [n] squared distance to the ordered set; -1 once ordered
  float* thr;            // [n] float32 screening thresholds
  int64_t nn[kMtMaxLevels + 1];  // nodes per level (1: leaves)
  const float* lo[kMtMaxLevels + 1];  // [nn][DV] boxes of the images
  const float* hi[kMtMaxLevels + 1];
  long long* kb[kMtMaxLevels + 1];    // [nn] largest key: squared bits (-1: none)
  int* ki[kMtMaxLevels + 1];          //      and original index
  float* tmax[kMtMaxLevels + 1];      // [nn] threshold bound of the live points (-1: none)
  int* dflag[kMtMaxLevels + 1];       // [nn] keyed-again marks (all zero between passes)
  int* q[2];                          // queues of nodes, 32 nn[1] entries each
  unsigned* qm[2];                    // with a pivot index (descent) or mask
  int* cnt;                           // [24] counters of the cluster's queues
  long long* cl_b;                    // [16][32] each CTA's largest keys of level hcand
  int* cl_i;
  long long* cl_Kb;                   // [16] and the bound of the rest
  int* cl_Ki;
  int* leaves;                        // [nn[1]] leaves reached by a pass
  unsigned* lmask;                    // [nn[1]] their pivot masks (zero between passes)
};

// lower bound of the squared distance from image p to the box [lo, hi] (zero
// padded to DV, like the images), rounded down
__device__ __forceinline__ float mt_box_lb(const float* lo, const float* hi, const float* p, int DV) {
  float s = 0.0f;
  for (int l = 0; l < DV; ++l) {
    const float a = lo[l], b = hi[l], x = p[l];
    float g = 0.0f;
    if (x < a)
      g = __fsub_rd(a, x);
    else if (x > b)
      g = __fsub_rd(x, b);
    s = __fmaf_rd(g, g, s);
  }
  return s;
}

__global__ void __launch_bounds__(kMtThreads, 1) k_maximin_tree(MtRun Q) {
  extern __shared__ __align__(16) unsigned char mt_raw[];
  const int d = Q.d, DV = Q.DV, H = Q.H;
  const int64_t n = Q.n;
  double* Ux = (double*)mt_raw;                         // [32][d] candidates' rows
  double* Px = Ux + 32 * d;                             // [32][d] pivots' rows
  double* pairS = Px + 32 * d;                          // [31][31]
  long long* wlb = (long long*)(pairS + kMcU * kMcU);   // [warps][32] lists
  int* wli = (int*)(wlb + kMtWarps * 32);
  float* Uv = (float*)(wli + kMtWarps * 32);            // [32][DV] candidates' images
  float* Pv = Uv + 32 * DV;                             // [32][DV] pivots' images
  __shared__ long long Ub[32], w_Kb[kMtWarps], s_Kb, s_top;
  __shared__ int Ui[32], Upos[32], w_Ki[kMtWarps], s_Ki, s_sel[32], piv_slot[32], P_pos[32];
  __shared__ float UB[32], Uthr[32], P_B[32];
  __shared__ int s_k, s_tie, s_err, s_qn[2];
  const unsigned FULL = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float growth = mc_growth(d);
  const bool roots_always = (Q.flags & 1) != 0;
  const bool scan_always = (Q.flags & 2) != 0;

  // slots 0..31 (Ub, Ui) <- the 32 largest of every thread's three keys;
  // (Kb, Ki) <- the largest key that may be outside slots 0..30
  auto collect = [&](long long b1, int i1, long long b2, int i2, long long b3, int i3,
                     long long& Kb, int& Ki) {
    mc_warp_sort2(b1, i1, b2, i2);
    mc_warp_merge(b1, i1, b2, i2);
    mc_warp_max(b3, i3);
    wlb[warp * 32 + lane] = b1;
    wli[warp * 32 + lane] = i1;
    if (lane == 0) {
      w_Kb[warp] = b3;
      w_Ki[warp] = i3;
    }
    __syncthreads();
    for (int s = kMtWarps >> 1; s >= 1; s >>= 1) {
      if (warp < s) {
        mc_warp_merge(b1, i1, wlb[(warp + s) * 32 + lane], wli[(warp + s) * 32 + lane]);
        if (s > 1) {
          wlb[warp * 32 + lane] = b1;
          wli[warp * 32 + lane] = i1;
        }
      }
      if (s > 1) __syncthreads();
    }
    if (warp == 0) {
      long long kb = w_Kb[lane];
      int ki = w_Ki[lane];
      mc_warp_max(kb, ki);
      const long long b32 = __shfl_sync(FULL, b1, 31);
      const int i32 = __shfl_sync(FULL, i1, 31);
      if (mc_greater(b32, i32, kb, ki)) {
        kb = b32;
        ki = i32;
      }
      Ub[lane] = b1;
      Ui[lane] = i1;
      if (lane == 0) {
        s_Kb = kb;
        s_Ki = ki;
      }
    }
    __syncthreads();
    Kb = s_Kb;
    Ki = s_Ki;
  };

  // queue push of cnt entries (node ids first .. first + cnt - 1, one mask)
  auto push_run = [&](int side, int64_t first, int cnt, unsigned mask) {
    const int base = atomicAdd(&s_qn[side], cnt);
    for (int c = 0; c < cnt; ++c) {
      Q.q[side][base + c] = (int)(first + c);
      Q.qm[side][base + c] = mask;
    }
  };

  // warp-wide: node itself (h == 1: a leaf, to the leaf list) or its
  // children (h > 1) to queue `side`, all with pivot mask m
  auto push_children = [&](int side, int h, int node, unsigned m) {
    int cnt = 1;
    int64_t c0 = node;
    if (h > 1) {
      c0 = (int64_t)node * kMtLeaf;
      cnt = (int)(min(c0 + kMtLeaf, Q.nn[h - 1]) - c0);
    }
    int base = 0;
    if (lane == 0) base = atomicAdd(&s_qn[side], cnt);
    base = __shfl_sync(FULL, base, 0);
    if (lane < cnt) {
      Q.q[side][base + lane] = (int)(c0 + lane);
      Q.qm[side][base + lane] = m;
    }
  };

  // ---- the 31 largest point keys (slots 0..30, positions Upos) and R.
  //      The first round takes every node of level hc (the lowest level with
  //      at most 32 nodes per thread), each thread keeping its three largest;
  //      later rounds the children of the 31 nodes chosen, then their points.
  //      Whatever a round leaves out is bounded by its Kb (a key left in a
  //      thread's third place included).
  const int hc = Q.hcand;
  const int ncta = (int)cg::this_cluster().num_blocks();
  auto candidates = [&](long long& Rb, int& Ri) {
    Rb = -1LL;
    Ri = kMcNone;
    int nsel = 0;
    for (int h = hc; h >= 0; --h) {
      long long b = -1LL, b2 = -1LL, b3 = -1LL;
      int i = kMcNone, i2 = kMcNone, i3 = kMcNone;
      if (h == hc && Q.cdist) {
        // the CTAs' lists of this round (step 5a): warp w merges CTA w's
        if (warp < ncta) {
          b = __ldcg(Q.cl_b + warp * 32 + lane);
          i = __ldcg(Q.cl_i + warp * 32 + lane);
          if (lane == 0) {
            b3 = __ldcg(Q.cl_Kb + warp);
            i3 = __ldcg(Q.cl_Ki + warp);
          }
        }
      } else if (h == hc) {
        for (int64_t id = threadIdx.x; id < Q.nn[h]; id += blockDim.x) {
          const long long kb = __ldcg(Q.kb[h] + id);
          if (kb >= 0) mc_insert3(kb, __ldcg(Q.ki[h] + id), b, i, b2, i2, b3, i3);
        }
      } else {
        int64_t id = -1;
        if (warp < nsel) {
          id = (int64_t)s_sel[warp] * kMtLeaf + lane;
          if (id >= (h > 0 ? Q.nn[h] : n)) id = -1;
        }
        if (id >= 0) {
          if (h > 0) {
            b = __ldcg(Q.kb[h] + id);
            i = __ldcg(Q.ki[h] + id);
          } else {
            const long long bits = dbits(__ldcg(Q.dist + id));
            if (bits >= 0 && bits < kBitsInf) {
              b = bits;
              i = Q.gidx[id];
            }
          }
          if (b < 0) {
            b = -1LL;
            i = kMcNone;
          }
        }
      }
      long long Kb;
      int Ki;
      collect(b, i, b2, i2, b3, i3, Kb, Ki);
      if (mc_greater(Kb, Ki, Rb, Ri)) {
        Rb = Kb;
        Ri = Ki;
      }
      // the chosen nodes (points): from the position of their largest point
      if (threadIdx.x < kMcU) {
        const int u = threadIdx.x;
        const int pos = Ub[u] >= 0 ? Q.posof[Ui[u]] : -1;
        s_sel[u] = pos >= 0 ? (pos >> (5 * h)) : -1;
        if (h == 0) Upos[u] = pos;
      }
      __syncthreads();
      nsel = 0;
      while (nsel < kMcU && Ub[nsel] >= 0) ++nsel;
    }
  };

  // ---- the candidates' rows and their pairwise exact squared distances
  // (float32-screened: +inf where neither can lower the other; -1 where a
  // float32 upper bound already puts either below R once the other is a pivot)
  auto fetch_pairs = [&](double Rv) {
    for (int e = threadIdx.x; e < kMcU * DV; e += blockDim.x) {
      const int u = e / DV, l = e - u * DV;
      if (Ub[u] >= 0) {
        Uv[u * DV + l] = Q.v[(size_t)Upos[u] * DV + l];
        if (l < d) Ux[u * d + l] = Q.xs[(size_t)Upos[u] * d + l];
      }
    }
    __syncthreads();
    if (threadIdx.x < kMcU && Ub[threadIdx.x] >= 0) {
      const int u = threadIdx.x;
      const float B = Q.Bp[Upos[u]];
      UB[u] = B;
      Uthr[u] = thr_sq(__longlong_as_double(Ub[u]), B);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kMcU * kMcU; t += blockDim.x) {
      const int a = t / kMcU, b = t - a * kMcU;
      if (a >= b || Ub[a] < 0 || Ub[b] < 0) continue;
      float s32 = 0.0f;
      for (int l = 0; l < d; ++l) {
        const float df = __fsub_rn(Uv[a * DV + l], Uv[b * DV + l]);
        s32 = __fmaf_rn(df, df, s32);
      }
      double sp = __longlong_as_double(kBitsInf);  // cannot update
      if (mc_may_update(s32, Uthr[a], UB[b], growth) || mc_may_update(s32, Uthr[b], UB[a], growth)) {
        if (Rv >= 0.0 && (double)mc_sq_upper(s32, UB[a], UB[b], growth) < Rv)
          sp = -1.0;  // either, once the other is a pivot, falls below R: out of this pass
        else
          sp = sqdist_exact(Ux + a * d, Ux + b * d, d);
      }
      pairS[a * kMcU + b] = sp;
      pairS[b * kMcU + a] = sp;
    }
    __syncthreads();
  };

  // warp 0: the pivot table from slots piv_slot[0..kk), their rows in order
  auto build_pivots = [&](int kk, int64_t nsel) {
    __syncwarp();
    for (int e = lane; e < kk * DV; e += 32) {
      const int t = e / DV, l = e - t * DV;
      Pv[e] = Uv[piv_slot[t] * DV + l];
    }
    for (int e = lane; e < kk * d; e += 32) {
      const int t = e / d, l = e - t * d;
      Px[e] = Ux[piv_slot[t] * d + l];
    }
    if (lane < kk) {
      const int u = piv_slot[lane];
      P_pos[lane] = Upos[u];
      P_B[lane] = UB[u];
      Q.order[nsel + lane] = Ui[u];
    }
    __syncwarp();
  };

  // ---- a cluster of C CTAs: every CTA takes a share of the (node, pivot)
  //      items, the points and the keys; CTA 0 alone chooses the pivots and
  //      the others copy its pivot table.  Counters in global memory: cdesc[h]
  //      items at level h, cleaf leaves reached, ckey[h] nodes to key at level
  //      h.  Data other CTAs write in the same call are read past L1 (__ldcg).
  cg::cluster_group cl = cg::this_cluster();
  const int r = (int)cl.block_rank(), C = (int)cl.num_blocks();
  const int64_t gt = (int64_t)r * blockDim.x + threadIdx.x;
  const int64_t gs = (int64_t)C * blockDim.x;
  const int gw = r * kMtWarps + warp, gws = C * kMtWarps;
  int* cdesc = Q.cnt;
  int* cleaf = Q.cnt + 8;
  int* ckey = Q.cnt + 9;

  // the first pivot: row `first`
  if (threadIdx.x == 0) {
    const int fp = *Q.first_pos;
    P_pos[0] = fp;
    P_B[0] = Q.Bp[fp];
    if (r == 0) Q.order[0] = Q.first;
    s_k = 1;
    s_err = 0;
    s_tie = 0;
  }
  __syncthreads();
  for (int l = threadIdx.x; l < DV; l += blockDim.x) Pv[l] = Q.v[(size_t)P_pos[0] * DV + l];
  for (int l = threadIdx.x; l < d; l += blockDim.x) Px[l] = Q.xs[(size_t)P_pos[0] * d + l];
  __syncthreads();

  const int hd = Q.hdesc;
  int64_t nsel = 1;
  while (nsel < n) {
    const int k = s_k;
    // 1. (CTA 0) the pivots are ordered (ordering.py:58) and their leaves
    //    listed (mask bit 31: to be keyed again, no pivot); the first items:
    //    every node of level hd with every pivot (hd: the highest level whose
    //    nodes times 31 pivots are at most two items per thread of the
    //    cluster, which saves the barriers of the levels above)
    if (r == 0) {
      if (threadIdx.x < 24) Q.cnt[threadIdx.x] = 0;
      __syncthreads();
      if (threadIdx.x < k) {
        const int p = P_pos[threadIdx.x];
        Q.dist[p] = -1.0;
        const int leaf = p / kMtLeaf;
        if (atomicOr(&Q.lmask[leaf], 0x80000000u) == 0u) Q.leaves[atomicAdd(cleaf, 1)] = leaf;
      }
      for (int e = threadIdx.x; e < (int)Q.nn[hd] * k; e += blockDim.x) {
        Q.q[0][e] = e / k;
        Q.qm[0][e] = (unsigned)(e % k);
      }
      if (threadIdx.x == 0) cdesc[hd] = (int)Q.nn[hd] * k;
    }
    cl.sync();
    // 2. the descent from level hd, a thread per (node, pivot) item; a leaf
    //    reached takes the pivot into its mask (the first bit puts it on the
    //    list)
    for (int h = hd; h >= 1; --h) {
      const int buf = (hd - h) & 1;
      const int nin = __ldcg(cdesc + h);
      for (int64_t e = gt; e < nin; e += gs) {
        const int node = __ldcg(Q.q[buf] + e);
        const int t = (int)__ldcg(Q.qm[buf] + e);
        const float tm = __ldcg(Q.tmax[h] + node);
        if (tm < 0.0f) continue;
        const float* lo = Q.lo[h] + (size_t)node * DV;
        const float* hi = Q.hi[h] + (size_t)node * DV;
        if (!mc_may_update(mt_box_lb(lo, hi, Pv + t * DV, DV), tm, P_B[t], growth)) continue;
        if (h == 1) {
          if (atomicOr(&Q.lmask[node], 1u << t) == 0u) Q.leaves[atomicAdd(cleaf, 1)] = node;
        } else {
          const int64_t c0 = (int64_t)node * kMtLeaf;
          const int cnt = (int)(min(c0 + kMtLeaf, Q.nn[h - 1]) - c0);
          const int base = atomicAdd(cdesc + h - 1, cnt);
          for (int c = 0; c < cnt; ++c) {
            Q.q[buf ^ 1][base + c] = (int)(c0 + c);
            Q.qm[buf ^ 1][base + c] = (unsigned)t;
          }
        }
      }
      cl.sync();
    }
    // 3. the points of the leaves reached: float32 screen against the leaf's
    //    pivots with the pass-start threshold, then the exact squared
    //    distances of the pivots left, in pivot order (ordering.py:49-58)
    const int nleaf = __ldcg(cleaf);
    for (int64_t e = gt; e < (int64_t)nleaf * kMtLeaf; e += gs) {
      const int leaf = __ldcg(Q.leaves + (e >> 5));
      const int64_t pos = (int64_t)leaf * kMtLeaf + (e & 31);
      if (pos >= n) continue;
      const unsigned mask = __ldcg(Q.lmask + leaf) & 0x7fffffffu;
      if (!mask) continue;
      double dp = __ldcg(Q.dist + pos);
      if (dbits(dp) < 0) continue;  // ordered (ordering.py:50-51)
      const float th = __ldcg(Q.thr + pos);
      const float* vp = Q.v + (size_t)pos * DV;
      unsigned m3 = 0;
      for (unsigned mm = mask; mm; mm &= mm - 1) {
        const int t = __ffs(mm) - 1;
        float s32 = 0.0f;
        for (int l = 0; l < d; ++l) {
          const float df = __fsub_rn(vp[l], Pv[t * DV + l]);
          s32 = __fmaf_rn(df, df, s32);
        }
        if (mc_may_update(s32, th, P_B[t], growth)) m3 |= 1u << t;
      }
      if (!m3) continue;
      const long long b0 = dbits(dp);
      const double* xp = Q.xs + (size_t)pos * d;
      for (unsigned mm = m3; mm; mm &= mm - 1) {
        const int t = __ffs(mm) - 1;
        const double sn = sqdist_exact(xp, Px + t * d, d);
        if (dbits(sn) < dbits(dp)) dp = sn;
      }
      if (dbits(dp) != b0) {
        Q.dist[pos] = dp;
        Q.thr[pos] = thr_sq(dp, Q.Bp[pos]);
      }
    }
    cl.sync();
    // 4. the listed leaves keyed again (a warp per leaf, a lane per point),
    //    then their ancestors (a lane per child)
    for (int e = gw; e < nleaf; e += gws) {
      const int node = __ldcg(Q.leaves + e);
      long long kb = -1LL;
      int ki = kMcNone;
      float tm = -1.0f;
      const int64_t c = (int64_t)node * kMtLeaf + lane;
      if (c < n) {
        const long long bits = dbits(__ldcg(Q.dist + c));
        if (bits >= 0) {
          tm = __ldcg(Q.thr + c);
          if (bits < kBitsInf) {
            kb = bits;
            ki = Q.gidx[c];
          }
        }
      }
      mc_warp_max(kb, ki);
      for (int o = 16; o > 0; o >>= 1) tm = fmaxf(tm, __shfl_xor_sync(FULL, tm, o));
      if (lane == 0) {
        Q.kb[1][node] = kb;
        Q.ki[1][node] = ki;
        Q.tmax[1][node] = tm;
        Q.lmask[node] = 0u;
        if (H > 1) {
          const int parent = node / kMtLeaf;
          if (atomicExch(&Q.dflag[2][parent], 1) == 0) Q.q[0][atomicAdd(ckey + 2, 1)] = parent;
        }
      }
    }
    cl.sync();
    for (int h = 2; h <= H; ++h) {
      const int buf = h & 1;
      const int nin = __ldcg(ckey + h);
      for (int e = gw; e < nin; e += gws) {
        const int node = __ldcg(Q.q[buf] + e);
        long long kb = -1LL;
        int ki = kMcNone;
        float tm = -1.0f;
        const int64_t c = (int64_t)node * kMtLeaf + lane;
        if (c < Q.nn[h - 1]) {
          kb = __ldcg(Q.kb[h - 1] + c);
          ki = __ldcg(Q.ki[h - 1] + c);
          tm = __ldcg(Q.tmax[h - 1] + c);
          if (kb < 0) {
            kb = -1LL;
            ki = kMcNone;
          }
        }
        mc_warp_max(kb, ki);
        for (int o = 16; o > 0; o >>= 1) tm = fmaxf(tm, __shfl_xor_sync(FULL, tm, o));
        if (lane == 0) {
          Q.dflag[h][node] = 0;
          Q.kb[h][node] = kb;
          Q.ki[h][node] = ki;
          Q.tmax[h][node] = tm;
          if (h < H) {
            const int parent = node / kMtLeaf;
            if (atomicExch(&Q.dflag[h + 1][parent], 1) == 0) Q.q[buf ^ 1][atomicAdd(ckey + h + 1, 1)] = parent;
          }
        }
      }
      cl.sync();
    }

    if (Q.cdist) {
      // 5a. the first candidate round, every node of level hc, split over
      //     the CTAs: each keeps its 32 largest keys and the bound of the rest
      const int64_t per = (Q.nn[hc] + C - 1) / C;
      const int64_t i0 = (int64_t)r * per, i1 = min(i0 + per, Q.nn[hc]);
      long long b1 = -1LL, b2 = -1LL, b3 = -1LL;
      int x1 = kMcNone, x2 = kMcNone, x3 = kMcNone;
      for (int64_t id = i0 + threadIdx.x; id < i1; id += blockDim.x) {
        const long long kb = __ldcg(Q.kb[hc] + id);
        if (kb >= 0) mc_insert3(kb, __ldcg(Q.ki[hc] + id), b1, x1, b2, x2, b3, x3);
      }
      long long Kb;
      int Ki;
      collect(b1, x1, b2, x2, b3, x3, Kb, Ki);
      if (threadIdx.x < 32) {
        Q.cl_b[r * 32 + threadIdx.x] = Ub[threadIdx.x];
        Q.cl_i[r * 32 + threadIdx.x] = Ui[threadIdx.x];
      }
      if (threadIdx.x == 0) {
        Q.cl_Kb[r] = Kb;
        Q.cl_Ki[r] = Ki;
      }
      cl.sync();
    }
    if (r == 0) {
      // 5. candidates U = slots 0..30; R bounds every other point's bits
      long long R;
      int Ri;
      candidates(R, Ri);
      fetch_pairs(R >= 0 ? __longlong_as_double(R) : -1.0);
      //    pivots from the candidates (warp 0, one candidate per lane)
      if (warp == 0) {
        long long sb = lane < kMcU ? Ub[lane] : -1LL;
        const int si = lane < kMcU ? Ui[lane] : kMcNone;
        bool alive = sb >= 0;
        const long long top = __shfl_sync(FULL, sb, 0);  // the largest square
        int kk = 0;
        if (!scan_always && !roots_always) {
          // the leading run of slots that are certain in list order: each is
          // above R + 4 ulps, more than 4 ulps above the next slot (no equal
          // root below it) and not lowered by a slot before it
          bool red = false;
          for (int i = 0; i < lane && i < kMcU; ++i)
            red = red || __double_as_longlong(pairS[lane * kMcU + i]) < sb;  // (knock-outs are < 0)
          const long long nb = __shfl_down_sync(FULL, sb, 1);
          const bool near = lane + 1 < kMcU && nb >= 0 && nb >= sb - 4;
          const bool bad = lane >= kMcU || !alive || red || near || !(R < 0 || sb > R + 4);
          const int m = (int)min((int64_t)(__ffs(__ballot_sync(FULL, bad)) - 1), n - nsel);
          if (m > 0) {
            if (lane < m) {
              piv_slot[lane] = lane;
              alive = false;
            }
            for (int i = 0; alive && i < m; ++i) {
              const long long sn = __double_as_longlong(pairS[lane * kMcU + i]);
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
          const unsigned mh = __reduce_max_sync(FULL, hi);
          if (mh == 0) break;  // none left
          const unsigned lo = alive && hi == mh ? (unsigned)sb : 0u;
          const unsigned ml = __reduce_max_sync(FULL, lo);
          const long long mb = ((long long)(mh - 1u) << 32) | (long long)ml;
          if (!(R < 0 || mb > R + 4)) break;  // not certain
          const bool is_max = alive && hi == mh && (unsigned)sb == ml;
          int mi = (int)__reduce_min_sync(FULL, is_max ? (unsigned)si : (unsigned)kMcNone);
          const unsigned nearm = __ballot_sync(FULL, alive && sb >= mb - 4 && si < mi);
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
          const int ws = __ffs(__ballot_sync(FULL, alive && si == mi)) - 1;
          if (lane == 0) piv_slot[kk] = ws;
          if (lane == ws) alive = false;
          if (alive) {
            const long long sn = __double_as_longlong(pairS[lane * kMcU + ws]);
            if (sn < 0)
              alive = false;  // below R after this pivot: cannot be chosen in this pass
            else if (sn < sb)
              sb = sn;
          }
          ++kk;
        }
        build_pivots(kk, nsel);
        if (lane == 0) {
          s_k = kk;
          s_tie = kk == 0;
          s_top = top;
        }
      }
      __syncthreads();
      if (s_tie) {
        //    tie pass: no choice was certain, so many squares lie within 4 ulps
        //    of the largest, top.  The largest root is fl(sqrt(top)); the points
        //    with that root, T, are the reference's next choices in index order
        //    (ordering.py:45) while they keep it.  Slots 0..30 take the 31
        //    smallest indices of T (found below the nodes whose largest key is
        //    within 4 ulps of top); any other member of T has an index >= the
        //    bound Ki.
        const long long top = s_top;
        if (top < 0) {
          // no finite candidate left (NaN inputs): report and stop
          if (threadIdx.x == 0) {
            s_err = 1;
            set_error(Q.info + SV_INFO_STATUS, SV_EINVAL);
            Q.info[SV_INFO_BLOCK] = (int)nsel;
          }
        } else {
          const long long rmax = __double_as_longlong(__dsqrt_rn(__longlong_as_double(top)));
          if (threadIdx.x == 0) {
            s_qn[0] = 0;
            s_qn[1] = 0;
          }
          __syncthreads();
          int tc = 0;
          if (threadIdx.x == 0) push_run(0, 0, (int)Q.nn[H], 0u);
          for (int h = H; h >= 1; --h) {
            __syncthreads();
            const int nin = s_qn[tc];
            __syncthreads();
            if (threadIdx.x == 0) s_qn[tc ^ 1] = 0;
            __syncthreads();
            for (int e = warp; e < nin; e += kMtWarps) {
              const int node = Q.q[tc][e];
              if (__ldcg(Q.kb[h] + node) >= top - 4) push_children(tc ^ 1, h, node, 0u);
            }
            tc ^= 1;
          }
          __syncthreads();
          long long b1 = -1, b2 = -1, b3 = -1;
          int i1 = kMcNone, i2 = kMcNone, i3 = kMcNone;
          const int nl = s_qn[tc];
          for (int64_t e = threadIdx.x; e < (int64_t)nl * kMtLeaf; e += blockDim.x) {
            const int64_t pos = (int64_t)Q.q[tc][e >> 5] * kMtLeaf + (e & 31);
            if (pos >= n) continue;
            const double dp = __ldcg(Q.dist + pos);
            const long long bits = dbits(dp);
            if (bits < 0 || bits > top || bits < top - 4) continue;
            if (dbits(__dsqrt_rn(dp)) != rmax) continue;
            // key: the smaller index first; the low 3 bits carry top - bits
            const int gi = Q.gidx[pos];
            mc_insert3(((1LL << 40) - gi) * 8 + (top - bits), gi, b1, i1, b2, i2, b3, i3);
          }
          long long Kb;
          int Ki;
          collect(b1, i1, b2, i2, b3, i3, Kb, Ki);
          const int bound = Kb >= 0 ? Ki : kMcNone;
          // the slots' squares from their keys, their positions
          if (threadIdx.x < kMcU && Ub[threadIdx.x] >= 0) {
            Ub[threadIdx.x] = top - (Ub[threadIdx.x] & 7);
            Upos[threadIdx.x] = Q.posof[Ui[threadIdx.x]];
          }
          __syncthreads();
          fetch_pairs(-1.0);
          if (warp == 0) {
            long long sb = lane < kMcU ? Ub[lane] : -1LL;
            const int si = lane < kMcU ? Ui[lane] : kMcNone;
            bool alive = sb >= 0, tied = alive;
            int kk = 0;
            while (kk < kMcU && nsel + kk < n) {
              const int mi = (int)__reduce_min_sync(FULL, alive && tied ? (unsigned)si : (unsigned)kMcNone);
              if (mi == kMcNone || mi >= bound) break;
              const int ws = __ffs(__ballot_sync(FULL, alive && si == mi)) - 1;
              if (lane == 0) piv_slot[kk] = ws;
              if (lane == ws) alive = false;
              if (alive) {
                const double sn = pairS[lane * kMcU + ws];
                if (__double_as_longlong(sn) < sb) {
                  sb = __double_as_longlong(sn);
                  if (tied) tied = __double_as_longlong(__dsqrt_rn(sn)) == rmax;
                }
              }
              ++kk;
            }
            build_pivots(kk, nsel);
            if (lane == 0) s_k = kk;
          }
        }
        __syncthreads();
      }
    }
    cl.sync();
    // 6. the other CTAs take CTA 0's pivot table
    if (r != 0) {
      if (threadIdx.x == 0) {
        s_k = *cl.map_shared_rank(&s_k, 0);
        s_err = *cl.map_shared_rank(&s_err, 0);
      }
      __syncthreads();
      const int kk = s_k;
      if (threadIdx.x < kk) {
        P_pos[threadIdx.x] = cl.map_shared_rank(P_pos, 0)[threadIdx.x];
        P_B[threadIdx.x] = cl.map_shared_rank(P_B, 0)[threadIdx.x];
      }
      const float* rPv = cl.map_shared_rank(Pv, 0);
      const double* rPx = cl.map_shared_rank(Px, 0);
      for (int e = threadIdx.x; e < kk * DV; e += blockDim.x) Pv[e] = rPv[e];
      for (int e = threadIdx.x; e < kk * d; e += blockDim.x) Px[e] = rPx[e];
      __syncthreads();
    }
    if (s_err) break;
    if (s_k < 1) {
      // every pass orders at least one row (the tie pass always takes the
      // smallest index of T); anything else stops the kernel with an error
      if (r == 0 && threadIdx.x == 0) {
        set_error(Q.info + SV_INFO_STATUS, SV_EINVAL);
        Q.info[SV_INFO_BLOCK] = (int)nsel;
      }
      break;
    }
    nsel += s_k;
    __syncthreads();
  }
  // CTA 0's shared memory stays until every CTA has copied from it
  cl.sync();
}

// ---------------------------------------------------------------------------
// the tree: k-d order and the node levels
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned mt_ord(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float mt_unord(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// images centred on the first row, zero padded to DV, in original order
__global__ void k_mt_images(const double* X, int64_t n, int d, int DV, int64_t first, float* v0,
                            int* ids) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * DV;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / DV;
    const int l = (int)(e - i * DV);
    v0[e] = l < d ? __double2float_rn(X[i * d + l] - X[first * d + l]) : 0.0f;
    if (l == 0) ids[i] = (int)i;
  }
}

__global__ void k_mt_fill_u32(unsigned* p, int64_t cnt, unsigned val) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x)
    p[e] = val;
}

// segment s of S holds positions [s n / S, (s+1) n / S)
__device__ __forceinline__ int64_t mt_seg(int64_t pos, int64_t n, int64_t S) { return ((pos + 1) * S - 1) / n; }

// per segment and coordinate: min and max of the images (order-preserving
// unsigned codes, atomics once per warp run of equal segments)
__global__ void k_mt_seg_minmax(const float* v0, const int* ids, int64_t n, int d, int DV, int64_t S,
                                unsigned* mn, unsigned* mx) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) & ~(int64_t)31; base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pos = base + lane;
    const bool ok = pos < n;
    const int64_t seg = ok ? mt_seg(pos, n, S) : -1;
    const int64_t seg0 = __shfl_sync(0xffffffffu, seg, 0);
    const bool uni = __all_sync(0xffffffffu, !ok || seg == seg0);
    for (int l = 0; l < d; ++l) {
      unsigned a = 0xffffffffu, b = 0u;
      if (ok) {
        const unsigned c = mt_ord(v0[(size_t)ids[pos] * DV + l]);
        a = c;
        b = c;
      }
      if (uni) {
        a = __reduce_min_sync(0xffffffffu, a);
        b = __reduce_max_sync(0xffffffffu, b);
        if (lane == 0) {
          atomicMin(mn + seg0 * d + l, a);
          atomicMax(mx + seg0 * d + l, b);
        }
      } else if (ok) {
        atomicMin(mn + seg * d + l, a);
        atomicMax(mx + seg * d + l, b);
      }
    }
  }
}

// sort keys: (segment, code of the coordinate along the segment's widest extent)
__global__ void k_mt_keys(const float* v0, const int* ids, int64_t n, int d, int DV, int64_t S,
                          const unsigned* mn, const unsigned* mx, unsigned long long* keys) {
  for (int64_t pos = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pos < n;
       pos += (int64_t)gridDim.x * blockDim.x) {
    const int64_t seg = mt_seg(pos, n, S);
    int best = 0;
    float wbest = -1.0f;
    for (int l = 0; l < d; ++l) {
      const float w = mt_unord(mx[seg * d + l]) - mt_unord(mn[seg * d + l]);
      if (w > wbest) {
        wbest = w;
        best = l;
      }
    }
    keys[pos] = ((unsigned long long)seg << 32) | mt_ord(v0[(size_t)ids[pos] * DV + best]);
  }
}

// tree-order rows, images, bounds, indices; distances and thresholds +inf
__global__ void k_mt_gather(const double* X, const float* v0, const int* ids, int64_t n, int d, int DV,
                            int64_t first, double* xs, float* v, float* Bp, int* gidx, int* posof,
                            double* dist, float* thr, int* first_pos) {
  for (int64_t pos = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pos < n;
       pos += (int64_t)gridDim.x * blockDim.x) {
    const int id = ids[pos];
    for (int l = 0; l < d; ++l) xs[pos * d + l] = X[(int64_t)id * d + l];
    for (int l = 0; l < DV; ++l) v[pos * DV + l] = v0[(int64_t)id * DV + l];
    Bp[pos] = mc_img_bound(v + pos * DV, d);
    gidx[pos] = id;
    posof[id] = (int)pos;
    dist[pos] = __longlong_as_double(kBitsInf);
    thr[pos] = __int_as_float(0x7f800000);
    if (id == first) *first_pos = (int)pos;
  }
}

// boxes of level h from level h-1 (h = 1: from the points); keys none,
// threshold bounds +inf, marks clear
__global__ void k_mt_level(const float* clo, const float* chi, int64_t nc, int DV, int64_t nn,
                           float* lo, float* hi, long long* kb, int* ki, float* tmax, int* dflag) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn * DV;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / DV;
    const int l = (int)(e - j * DV);
    const int64_t c0 = j * kMtLeaf, c1 = min(c0 + kMtLeaf, nc);
    float a = __int_as_float(0x7f800000), b = -a;
    for (int64_t c = c0; c < c1; ++c) {
      a = fminf(a, clo[c * DV + l]);
      b = fmaxf(b, chi[c * DV + l]);
    }
    lo[e] = a;
    hi[e] = b;
    if (l == 0) {
      kb[j] = -1LL;
      ki[j] = kMcNone;
      tmax[j] = __int_as_float(0x7f800000);
      dflag[j] = 0;
    }
  }
}

static size_t mt_align(size_t x) { return (x + 255) & ~(size_t)255; }

static int mt_levels(int64_t n, int64_t* nn) {
  int H = 1;
  nn[0] = n;
  nn[1] = (n + kMtLeaf - 1) / kMtLeaf;
  while (nn[H] > kMtLeaf) {
    nn[H + 1] = (nn[H] + kMtLeaf - 1) / kMtLeaf;
    ++H;
  }
  return H;
}

// binary k-d levels: segments of at most 32 rows at the last one
static int mt_kd_levels(int64_t n) {
  int L = 0;
  while (((n + ((int64_t)1 << L) - 1) >> L) > kMtLeaf) ++L;
  return L;
}

// bytes of scratch CUB's radix sort may ask for on top of its key and value
// buffers; checked at run time
static size_t mt_sort_reserve(int64_t n) { return ((size_t)32 << 20) + 16 * (size_t)n; }

size_t maximin_tree_workspace_bytes(int64_t n, int d) {
  if (n < 1) n = 1;
  const int DV = d <= 4 ? 4 : d <= 8 ? 8 : d <= 16 ? 16 : d <= 32 ? 32 : 64;
  int64_t nn[kMtMaxLevels + 2] = {0};
  const int H = mt_levels(n, nn);
  if (H > kMtMaxLevels) return 0;
  const int64_t S = (int64_t)1 << mt_kd_levels(n);
  size_t b = 0;
  b += 2 * mt_align(8 * (size_t)n);            // sort keys
  b += 2 * mt_align(4 * (size_t)n);            // ids
  b += mt_align(4 * (size_t)n * DV);           // v0
  b += 2 * mt_align(4 * (size_t)S * d);        // segment min / max
  b += mt_align(mt_sort_reserve(n));
  b += mt_align(8 * (size_t)n * d);            // xs
  b += mt_align(4 * (size_t)n * DV);           // v
  b += 4 * mt_align(4 * (size_t)n);            // Bp, gidx, posof, thr
  b += mt_align(8 * (size_t)n);                // dist
  for (int h = 1; h <= H; ++h)
    b += 2 * mt_align(4 * (size_t)nn[h] * DV) + mt_align(8 * (size_t)nn[h]) + 3 * mt_align(4 * (size_t)nn[h]);
  b += 4 * mt_align(4 * 32 * (size_t)nn[1]);   // queues and their pivots / masks
  b += 2 * mt_align(4 * (size_t)nn[1]);        // leaf list and leaf masks
  b += mt_align(4 * 24);                       // queue counters
  b += 4 * mt_align(16 * 32 * 8);              // the CTAs' candidate lists
  b += 256;                                    // first position
  return b;
}

// the largest cluster (16, non-portable, else 8, 4, 2, 1) of k_maximin_tree
// CTAs with smem bytes of dynamic shared memory the device can schedule
static int mt_cluster_size(size_t smem) {
  cudaFuncSetAttribute(k_maximin_tree, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  for (int C = 16; C > 1; C /= 2) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C);
    cfg.blockDim = dim3(kMtThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclus = 0;
    if (cudaOccupancyMaxActiveClusters(&nclus, (void*)k_maximin_tree, &cfg) == cudaSuccess && nclus > 0) {
      cudaGetLastError();
      return C;
    }
  }
  cudaGetLastError();  // a refused query leaves no error behind
  return 1;
}

int maximin_tree_single(const double* X, int64_t n, int d, int64_t first, int64_t* order, int32_t* info,
                        char* ws, size_t ws_bytes, int flags, cudaStream_t st) {
  if (n < 2 || n > 0x7fffffffLL || d < 1 || d > 64) return SV_EINVAL;
  const size_t need = maximin_tree_workspace_bytes(n, d);
  if (need == 0) return SV_EINVAL;
  if (ws_bytes < need) return SV_ENOSPC;
  const int DV = d <= 4 ? 4 : d <= 8 ? 8 : d <= 16 ? 16 : d <= 32 ? 32 : 64;
  MtRun Q = {};
  const int H = mt_levels(n, Q.nn);
  const int L = mt_kd_levels(n);
  const int64_t Smax = (int64_t)1 << L;
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = ws + off;
    off += mt_align(bytes);
    return p;
  };
  unsigned long long* keys0 = (unsigned long long*)take(8 * (size_t)n);
  unsigned long long* keys1 = (unsigned long long*)take(8 * (size_t)n);
  int* ids0 = (int*)take(4 * (size_t)n);
  int* ids1 = (int*)take(4 * (size_t)n);
  float* v0 = (float*)take(4 * (size_t)n * DV);
  unsigned* mn = (unsigned*)take(4 * (size_t)Smax * d);
  unsigned* mx = (unsigned*)take(4 * (size_t)Smax * d);
  const size_t sort_bytes = mt_sort_reserve(n);
  void* sort_tmp = take(sort_bytes);
  double* xs = (double*)take(8 * (size_t)n * d);
  float* v = (float*)take(4 * (size_t)n * DV);
  float* Bp = (float*)take(4 * (size_t)n);
  int* gidx = (int*)take(4 * (size_t)n);
  int* posof = (int*)take(4 * (size_t)n);
  float* thr = (float*)take(4 * (size_t)n);
  double* dist = (double*)take(8 * (size_t)n);
  for (int h = 1; h <= H; ++h) {
    Q.lo[h] = (float*)take(4 * (size_t)Q.nn[h] * DV);
    Q.hi[h] = (float*)take(4 * (size_t)Q.nn[h] * DV);
    Q.kb[h] = (long long*)take(8 * (size_t)Q.nn[h]);
    Q.ki[h] = (int*)take(4 * (size_t)Q.nn[h]);
    Q.tmax[h] = (float*)take(4 * (size_t)Q.nn[h]);
    Q.dflag[h] = (int*)take(4 * (size_t)Q.nn[h]);
  }
  for (int s = 0; s < 2; ++s) {
    Q.q[s] = (int*)take(4 * 32 * (size_t)Q.nn[1]);
    Q.qm[s] = (unsigned*)take(4 * 32 * (size_t)Q.nn[1]);
  }
  Q.leaves = (int*)take(4 * (size_t)Q.nn[1]);
  int* mt_cnt = (int*)take(4 * 24);
  Q.cl_b = (long long*)take(16 * 32 * 8);
  Q.cl_i = (int*)take(16 * 32 * 8);
  Q.cl_Kb = (long long*)take(16 * 32 * 8);
  Q.cl_Ki = (int*)take(16 * 32 * 8);
  Q.lmask = (unsigned*)take(4 * (size_t)Q.nn[1]);
  int* first_pos = (int*)take(4);
  if (off > ws_bytes) return SV_ENOSPC;

  const int nsm = sv_num_sms();
  const unsigned grid = (unsigned)std::min<int64_t>(8LL * nsm, (n * DV + 255) / 256 + 1);
  k_mt_images<<<grid, 256, 0, st>>>(X, n, d, DV, first, v0, ids0);
  SV_CUDA_TRY(cudaGetLastError());
  // k-d order: L levels of halving
  cub::DoubleBuffer<unsigned long long> kbuf(keys0, keys1);
  cub::DoubleBuffer<int> ibuf(ids0, ids1);
  size_t tmp_need = 0;
  SV_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmp_need, kbuf, ibuf, (int)n, 0, 64, st));
  if (tmp_need > sort_bytes) return SV_ENOSPC;
  for (int lev = 0; lev < L; ++lev) {
    const int64_t S = (int64_t)1 << lev;
    k_mt_fill_u32<<<grid, 256, 0, st>>>(mn, S * d, 0xffffffffu);
    k_mt_fill_u32<<<grid, 256, 0, st>>>(mx, S * d, 0u);
    k_mt_seg_minmax<<<grid, 256, 0, st>>>(v0, ibuf.Current(), n, d, DV, S, mn, mx);
    k_mt_keys<<<grid, 256, 0, st>>>(v0, ibuf.Current(), n, d, DV, S, mn, mx, kbuf.Current());
    SV_CUDA_TRY(cudaGetLastError());
    int end_bit = 32;
    while (((int64_t)1 << (end_bit - 32)) < S) ++end_bit;
    size_t tb = sort_bytes;
    SV_CUDA_TRY(cub::DeviceRadixSort::SortPairs(sort_tmp, tb, kbuf, ibuf, (int)n, 0, end_bit, st));
  }
  SV_CUDA_TRY(cudaMemsetAsync(Q.lmask, 0, 4 * (size_t)Q.nn[1], st));
  k_mt_gather<<<grid, 256, 0, st>>>(X, v0, ibuf.Current(), n, d, DV, first, xs, v, Bp, gidx, posof, dist,
                                    thr, first_pos);
  SV_CUDA_TRY(cudaGetLastError());
  for (int h = 1; h <= H; ++h) {
    const float* clo = h == 1 ? v : Q.lo[h - 1];
    k_mt_level<<<grid, 256, 0, st>>>(clo, clo == v ? v : Q.hi[h - 1], Q.nn[h - 1], DV, Q.nn[h],
                                     const_cast<float*>(Q.lo[h]), const_cast<float*>(Q.hi[h]), Q.kb[h],
                                     Q.ki[h], Q.tmax[h], Q.dflag[h]);
    SV_CUDA_TRY(cudaGetLastError());
  }
  Q.n = n;
  Q.d = d;
  Q.DV = DV;
  Q.H = H;
  Q.flags = flags & 3;
  Q.first = first;
  Q.first_pos = first_pos;
  Q.order = order;
  Q.info = info;
  Q.xs = xs;
  Q.v = v;
  Q.Bp = Bp;
  Q.gidx = gidx;
  Q.posof = posof;
  Q.dist = dist;
  Q.thr = thr;
  Q.cnt = mt_cnt;
  const size_t smem = (size_t)(2 * 32 * d + kMcU * kMcU) * 8 + (size_t)kMtWarps * 32 * 12 +
                      (size_t)2 * 32 * DV * 4;
  SV_CUDA_TRY(cudaFuncSetAttribute(k_maximin_tree, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int C = mt_cluster_size(smem);
  // the descent starts at the lowest level whose nodes times 31 pivots are at
  // most two items per thread of the cluster, the candidate rounds at the
  // lowest level of at most 32 nodes per thread (the top level always
  // qualifies: at most 32 nodes)
  Q.hdesc = H;
  for (int h = 1; h <= H; ++h)
    if (Q.nn[h] * kMcU <= 2LL * C * kMtThreads) {
      Q.hdesc = h;
      break;
    }
  Q.hcand = H;
  for (int h = 1; h <= H; ++h)
    if (Q.nn[h] <= 32LL * kMtThreads) {
      Q.hcand = h;
      break;
    }
  // with more than 8 nodes per thread there, the first round is split over
  // the cluster (one more barrier per pass)
  Q.cdist = (C > 1 && Q.nn[Q.hcand] > 8LL * kMtThreads) ? 1 : 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)C);
  cfg.blockDim = dim3(kMtThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SV_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_maximin_tree, Q));
  return SV_OK;
}

}  // namespace sv
