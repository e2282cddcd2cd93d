// Exact k-nearest-neighbour searches on the GPU.
//
//   ordered : ordering.py:76-116 (find_ordered_nn): row i takes the min(i, m)
//             nearest rows j < i;
//   query   : gp.py:253-255 (cKDTree.query): each query row takes the k
//             nearest reference rows.
//
// Tiled brute force.  A CTA owns a tile of Q query rows (one thread each,
// coordinates in registers) and streams candidate tiles of C rows through
// shared memory.  The screening distance is float32 on coordinates centred on
// the centroid; a candidate whose float32 lower bound (same error analysis as
// the maximin kernel: s32 >= (sqrt(s64_k)(1+(d+4)2^-53) + B_i + B_j)^2
// (1+2^-24)^(D+2), formed with upward rounding) cannot beat the current k-th
// best is skipped, every other one is measured exactly (IEEE sequential
// float64, no FMA) and inserted into the thread's sorted list.  Candidates
// are visited in increasing index order, so equal float64 distances keep the
// smaller index: the selected set is the exact (distance, index) order.
#include "sv_reorder.cuh"

namespace sv {

constexpr int kKnnQ = 128;  // queries per CTA (one per thread)
constexpr int kKnnC = 128;  // candidates per shared-memory tile
constexpr int kKnnHeapMin = 48;  // lists of at least this many neighbours are kept as heaps

// Max-heap on (squared distance, index) in a thread's column of the list
// arrays (element e at [e * kKnnQ + tid]); the root is the current k-th.
__device__ __forceinline__ bool knn_key_less(double a, int ia, double b, int ib) {
  return a < b || (a == b && ia < ib);
}
__device__ __forceinline__ void knn_heap_swap(double* lsd, int* lsi, int e, int f, int tid) {
  const double td = lsd[e * kKnnQ + tid];
  const int ti = lsi[e * kKnnQ + tid];
  lsd[e * kKnnQ + tid] = lsd[f * kKnnQ + tid];
  lsi[e * kKnnQ + tid] = lsi[f * kKnnQ + tid];
  lsd[f * kKnnQ + tid] = td;
  lsi[f * kKnnQ + tid] = ti;
}
__device__ __forceinline__ void knn_sift_down(double* lsd, int* lsi, int e, int size, int tid) {
  while (true) {
    const int l = 2 * e + 1;
    if (l >= size) break;
    int c = l;
    if (l + 1 < size && knn_key_less(lsd[l * kKnnQ + tid], lsi[l * kKnnQ + tid],
                                     lsd[(l + 1) * kKnnQ + tid], lsi[(l + 1) * kKnnQ + tid]))
      c = l + 1;
    if (!knn_key_less(lsd[e * kKnnQ + tid], lsi[e * kKnnQ + tid], lsd[c * kKnnQ + tid],
                      lsi[c * kKnnQ + tid]))
      break;
    knn_heap_swap(lsd, lsi, e, c, tid);
    e = c;
  }
}

// prologue: centred float32 coordinates (zero padded to DP) and their bound
__global__ void k_knn_prep(const double* X, int64_t n, int d, int DP, const double* centroid,
                           float* v, float* B) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double e2 = 0.0;
    for (int l = 0; l < DP; ++l) {
      float f = 0.0f;
      if (l < d) {
        const double c = X[i * d + l] - centroid[l];
        f = __double2float_rn(c);
        e2 += c * c;
      }
      v[i * DP + l] = f;
    }
    B[i] = __double2float_ru(1.01 * 0x1p-24 * sqrt(e2));
  }
}

__global__ void k_centroid2(const double* X, int64_t n, int d, double* c) {
  const int l = blockIdx.x;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += X[i * d + l];
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) c[l] = n > 0 ? red[0] / (double)n : 0.0;
}

struct KnnArgs {
  const double* Xq;    // query rows (float64)
  const double* Xr;    // reference rows (float64)
  const float* vq;     // query rows, centred float32 [nq][DP]
  const float* vr;     // reference rows [nr][DP]
  const float* Bq;
  const float* Br;
  int64_t nq, nr;
  int d, k, m;
  int64_t start;       // ordered: first row to fill
  int64_t* out;        // ordered: (n, m+1); query: (nq, k)
  float growth;        // (1+2^-24)^(DP+2) (1+2^-20), rounded up
  int ordered;
  int32_t* nbr;        // ordered, block form: neighbour columns of blocks b0 + i
  int64_t b0;
  int ldnbr;
  int wq_cap, wq_sort;  // large k: superset capacity and sort width per warp
};

__device__ __forceinline__ float knn_thr(double s64k, float Bi, int d) {
  const double t = (sqrt(s64k) * (1.0 + (double)(d + 4) * 0x1p-53) + (double)Bi) * (1.0 + 0x1p-40);
  return __double2float_ru(t);
}

// One query tile: qt = tile index, rows [qt Q, qt Q + Q) of the query set.
// Ordered searches write the reference's (n, m+1) rows, or, when A.nbr is
// set, the neighbour columns of the likelihood blocks (block b0 + i holds
// row i's neighbours, -1 padded to ldnbr).
template <int DP>
__device__ __forceinline__ void knn_tile(const KnnArgs& A, int64_t qt, unsigned char* smraw) {
  float* tile = (float*)smraw;                     // [C][DP]
  float* tileB = tile + kKnnC * DP;                // [C]
  double* lsd = (double*)(tileB + kKnnC);          // [k][Q] squared distances
  int* lsi = (int*)(lsd + (size_t)A.k * kKnnQ);    // [k][Q] indices

  const int64_t i = qt * kKnnQ + threadIdx.x;
  const bool valid = i < A.nq;
  const int tid = threadIdx.x;

  int kq = A.k;
  if (A.ordered) kq = (int)min((int64_t)A.m, i);
  bool active = valid && kq > 0;
  if (A.ordered && i < A.start) active = false;

  float qv[DP];
  float Bi = 0.0f;
  const double* xq = A.Xq + (valid ? i : 0) * A.d;
#pragma unroll
  for (int l = 0; l < DP; ++l) qv[l] = valid ? A.vq[i * DP + l] : 0.0f;
  if (valid) Bi = A.Bq[i];

  int cnt = 0;
  float T = __int_as_float(0x7f800000);  // +inf until the list is full
  const bool heap = A.k >= kKnnHeapMin;

  // candidate range
  int64_t cend = A.nr;
  if (A.ordered) cend = min(A.nq, (qt + 1) * kKnnQ);  // rows < last query of the tile
  for (int64_t c0 = 0; c0 < cend; c0 += kKnnC) {
    __syncthreads();
    const int nc = (int)min((int64_t)kKnnC, cend - c0);
    for (int e = tid; e < nc * DP; e += blockDim.x) tile[e] = A.vr[c0 * DP + e];
    for (int e = tid; e < nc; e += blockDim.x) tileB[e] = A.Br[c0 + e];
    __syncthreads();
    if (!active) continue;
    int cmax = nc;
    if (A.ordered) {
      const int64_t lim = i - c0;  // candidates j < i
      if (lim <= 0) continue;
      if (lim < cmax) cmax = (int)lim;
    }
    for (int c = 0; c < cmax; ++c) {
      const float* tv = tile + c * DP;
      float s32 = 0.0f;
#pragma unroll
      for (int l = 0; l < DP; l += 4) {
        const float4 t4 = *reinterpret_cast<const float4*>(tv + l);
        float df = __fsub_rn(qv[l], t4.x);
        s32 = __fmaf_rn(df, df, s32);
        df = __fsub_rn(qv[l + 1], t4.y);
        s32 = __fmaf_rn(df, df, s32);
        df = __fsub_rn(qv[l + 2], t4.z);
        s32 = __fmaf_rn(df, df, s32);
        df = __fsub_rn(qv[l + 3], t4.w);
        s32 = __fmaf_rn(df, df, s32);
      }
      const float tb = __fadd_ru(T, tileB[c]);
      const float bound = __fmul_ru(__fmul_ru(tb, tb), A.growth);
      if (s32 >= bound) continue;
      // exact float64 squared distance (IEEE sequential, no FMA)
      const int64_t j = c0 + c;
      const double* xr = A.Xr + j * A.d;
      double s = 0.0;
      for (int l = 0; l < A.d; ++l) {
        const double df = __dsub_rn(xq[l], xr[l]);
        s = __dadd_rn(s, __dmul_rn(df, df));
      }
      if (heap) {
        // later index loses ties: only a strictly smaller distance displaces the root
        if (cnt == kq) {
          if (!(s < lsd[tid])) continue;
          lsd[tid] = s;
          lsi[tid] = (int)j;
          knn_sift_down(lsd, lsi, 0, kq, tid);
        } else {
          int e = cnt++;
          lsd[e * kKnnQ + tid] = s;
          lsi[e * kKnnQ + tid] = (int)j;
          while (e > 0) {
            const int par = (e - 1) >> 1;
            if (!knn_key_less(lsd[par * kKnnQ + tid], lsi[par * kKnnQ + tid], s, (int)j)) break;
            knn_heap_swap(lsd, lsi, e, par, tid);
            e = par;
          }
        }
        if (cnt == kq) T = knn_thr(lsd[tid], Bi, A.d);
        continue;
      }
      if (cnt == kq) {
        if (!(s < lsd[(kq - 1) * kKnnQ + tid])) continue;  // later index loses ties
        --cnt;
      }
      int p = cnt;
      while (p > 0 && lsd[(p - 1) * kKnnQ + tid] > s) {
        lsd[p * kKnnQ + tid] = lsd[(p - 1) * kKnnQ + tid];
        lsi[p * kKnnQ + tid] = lsi[(p - 1) * kKnnQ + tid];
        --p;
      }
      lsd[p * kKnnQ + tid] = s;
      lsi[p * kKnnQ + tid] = (int)j;
      ++cnt;
      if (cnt == kq) T = knn_thr(lsd[(kq - 1) * kKnnQ + tid], Bi, A.d);
    }
  }
  if (!valid) return;
  if (heap)  // heap sort: ascending (distance, index)
    for (int end = cnt - 1; end > 0; --end) {
      knn_heap_swap(lsd, lsi, 0, end, tid);
      knn_sift_down(lsd, lsi, 0, end, tid);
    }
  if (A.nbr) {
    int32_t* row = A.nbr + (A.b0 + i) * (int64_t)A.ldnbr;
    for (int c = 0; c < A.ldnbr; ++c) row[c] = (active && c < cnt) ? lsi[c * kKnnQ + tid] : -1;
  } else if (A.ordered) {
    int64_t* row = A.out + i * (int64_t)(A.m + 1);
    row[0] = i;
    for (int c = 0; c < A.m; ++c) row[1 + c] = (active && c < cnt) ? (int64_t)lsi[c * kKnnQ + tid] : -1;
  } else {
    int64_t* row = A.out + i * (int64_t)A.k;
    for (int c = 0; c < A.k; ++c) row[c] = (c < cnt) ? (int64_t)lsi[c * kKnnQ + tid] : -1;
  }
}

template <int DP>
__global__ void __launch_bounds__(kKnnQ) k_knn(KnnArgs A) {
  extern __shared__ unsigned char smraw[];
  const int64_t ntile = (A.nq + kKnnQ - 1) / kKnnQ;
  // largest tiles first (ordered search work grows with the row index)
  const int64_t qt = A.ordered ? (ntile - 1 - blockIdx.x) : blockIdx.x;
  knn_tile<DP>(A, qt, smraw);
}

// ---------------------------------------------------------------------------
// Large k (kKnnHeapMin <= k <= kWqMaxK, DP <= 16): one warp per query.
// The warps of a CTA (up to 8 queries) stream the same candidate tiles.  A
// candidate's exact key (the float64 squared distance of the reference, IEEE
// sequential) is bracketed by float32 bounds on its root,
//   lo = sqrt(s32 / g) - B_q - B_c  <=  sqrt(key) (1 -+ tiny)  <=  hi = sqrt(s32 g) + B_q + B_c,
// (s32 the float32 squared distance of the centred images, g the growth
// factor of the screen above).  Each warp keeps in shared memory a superset
// of its query's k nearest: every candidate whose lo does not exceed tau, the
// k-th smallest hi kept so far (raised by 2^-20 for the root's rounding); no
// candidate outside it can reach the k nearest.  When the buffer fills it is
// filtered against the new tau, and if ties keep it full the exact keys of
// its entries decide (sorted by (key, index), the first k kept).  At the end
// the exact keys of the superset are sorted by (key, index): the reference's
// k nearest in order.  float64 work is dense (one entry per lane) and limited
// to about k entries per query.
constexpr int kWqC = 256;      // candidates per tile
constexpr int kWqMaxK = 1024;  // largest k of this path

// superset capacity (k + 160 rounded to 32, at least 384) and sort width
// (the power of two above it) per warp
__host__ __device__ inline int wq_cap(int k) { return max(384, ((k + 160 + 31) / 32) * 32); }
__host__ __device__ inline int wq_sort(int cap) {
  int s = 32;
  while (s < cap) s <<= 1;
  return s;
}

struct WqSmem {
  float* tv;      // [kWqC][DP] candidate images
  float* tB;      // [kWqC] their bounds
  float* bh;      // [warps][cap] hi of the superset entries
  float* bl;      // [warps][cap] lo
  int* bi;        // [warps][cap] index
  double* bs;     // [warps][sort width] exact keys while sorting
  int* bsi;       // [warps][sort width] their indices
};

__host__ __device__ inline size_t wq_smem_bytes(int DP, int warps, int cap, int sortw) {
  return (size_t)kWqC * DP * 4 + (size_t)kWqC * 4 + (size_t)warps * ((size_t)cap * 12 + (size_t)sortw * 12);
}

// k-th smallest (k >= 1) of the n non-negative floats x[0..n) (warp):
// radix search on the bit patterns, which order like the values
__device__ __forceinline__ float wq_kth(const float* x, int n, int k) {
  const int lane = threadIdx.x & 31;
  unsigned res = 0;
  for (int b = 30; b >= 0; --b) {
    const unsigned trial = res | (1u << b);
    int c = 0;
    for (int e = lane; e < n; e += 32) c += __float_as_uint(x[e]) < trial;
    c = __reduce_add_sync(0xffffffffu, c);
    if (c < k) res = trial;  // fewer than k lie below: the k-th is >= trial
  }
  return __uint_as_float(res);
}

// exact keys of the n entries, sorted by (key, index); returns them in
// S.bs/S.bsi[0..n) of this warp (warp-collective)
__device__ __forceinline__ void wq_exact_sort(const WqSmem& S, int w, int n, const double* xq,
                                              const double* Xr, int d, int cap, int sortw) {
  const int lane = threadIdx.x & 31;
  double* bs = S.bs + (size_t)w * sortw;
  int* bsi = S.bsi + (size_t)w * sortw;
  const int* bi = S.bi + (size_t)w * cap;
  int np = 32;
  while (np < n) np <<= 1;
  for (int e = lane; e < np; e += 32) {
    if (e < n) {
      const int j = bi[e];
      const double* xr = Xr + (size_t)j * d;
      double s = 0.0;
      for (int l = 0; l < d; ++l) {
        const double df = __dsub_rn(xq[l], xr[l]);
        s = __dadd_rn(s, __dmul_rn(df, df));
      }
      bs[e] = s;
      bsi[e] = j;
    } else {
      bs[e] = __longlong_as_double(0x7ff0000000000000LL);
      bsi[e] = 0x7fffffff;
    }
  }
  __syncwarp();
  // bitonic sort, ascending in (key, index)
  for (int k = 2; k <= np; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < np / 2; t += 32) {
        const int lo = 2 * t - (t & (j - 1));  // index with bit j clear
        const int hi = lo + j;
        const bool up = (lo & k) == 0;
        const double a = bs[lo], b = bs[hi];
        const int ia = bsi[lo], ib = bsi[hi];
        const bool agt = a > b || (a == b && ia > ib);
        if (agt == up) {
          bs[lo] = b;
          bs[hi] = a;
          bsi[lo] = ib;
          bsi[hi] = ia;
        }
      }
      __syncwarp();
    }
}

// One tile of nw = blockDim.x / 32 query rows: rows [qt nw, qt nw + nw), a
// warp each.
template <int DP>
__device__ __forceinline__ void knn_wq_tile(const KnnArgs& A, int64_t qt, unsigned char* smraw) {
  const int nw = blockDim.x >> 5;
  const int cap = A.wq_cap, sortw = A.wq_sort;
  WqSmem S;
  S.tv = (float*)smraw;
  S.tB = S.tv + (size_t)kWqC * DP;
  S.bh = S.tB + kWqC;
  S.bl = S.bh + (size_t)nw * cap;
  S.bi = (int*)(S.bl + (size_t)nw * cap);
  S.bs = (double*)(S.bi + (size_t)nw * cap);  // 8-byte aligned: cap is a multiple of 32
  S.bsi = (int*)(S.bs + (size_t)nw * sortw);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* bh = S.bh + (size_t)w * cap;
  float* bl = S.bl + (size_t)w * cap;
  int* bi = S.bi + (size_t)w * cap;
  const int64_t i = qt * nw + w;
  const bool valid = i < A.nq;
  int kq = A.k;
  if (A.ordered) kq = (int)min((int64_t)A.m, i);
  bool active = valid && kq > 0;
  if (A.ordered && i < A.start) active = false;

  float qv[DP];
  float Bi = 0.0f;
#pragma unroll
  for (int l = 0; l < DP; ++l) qv[l] = valid ? A.vq[i * DP + l] : 0.0f;
  if (valid) Bi = A.Bq[i];
  const double* xq = A.Xq + (valid ? i : 0) * A.d;
  int cnt = 0;
  float Tq = __int_as_float(0x7f800000);  // tau' + B_q: +inf until a filter
  const float g = A.growth;

  // filter the superset against tau (the kq-th smallest hi); if ties keep it
  // nearly full, keep the kq first by exact (key, index)
  auto compact = [&]() {
    const float tau = wq_kth(bh, cnt, kq);
    const float taum = __fmul_ru(tau, 1.0f + 0x1p-20f);
    int nc = 0;
    for (int e0 = 0; e0 < cnt; e0 += 32) {
      const int e = e0 + lane;
      float h = 0.0f, l = 0.0f;
      int ix = 0;
      bool keep = false;
      if (e < cnt) {
        h = bh[e];
        l = bl[e];
        ix = bi[e];
        keep = !(l > taum);
      }
      const unsigned km = __ballot_sync(0xffffffffu, keep);
      __syncwarp();
      if (keep) {
        const int p = nc + __popc(km & ((1u << lane) - 1));
        bh[p] = h;
        bl[p] = l;
        bi[p] = ix;
      }
      nc += __popc(km);
      __syncwarp();
    }
    cnt = nc;
    Tq = __fadd_ru(taum, Bi);
    if (cnt > cap - 2 * 32) {
      wq_exact_sort(S, w, cnt, xq, A.Xr, A.d, cap, sortw);
      const double* bs = S.bs + (size_t)w * sortw;
      const int* bsi = S.bsi + (size_t)w * sortw;
      for (int e = lane; e < kq; e += 32) {
        const double r = sqrt(bs[e]);
        bh[e] = __double2float_ru(r * (1.0 + 0x1p-40));
        bl[e] = __double2float_rd(r * (1.0 - 0x1p-40));
        bi[e] = bsi[e];
      }
      __syncwarp();
      cnt = kq;
      const float tau2 = bh[kq - 1];  // the kq-th exact root, rounded up
      Tq = __fadd_ru(__fmul_ru(tau2, 1.0f + 0x1p-20f), Bi);
    }
  };

  int64_t cend = A.nr;
  if (A.ordered) cend = min(A.nq, (qt + 1) * nw);  // rows < last query of the tile
  for (int64_t c0 = 0; c0 < cend; c0 += kWqC) {
    __syncthreads();
    const int nc = (int)min((int64_t)kWqC, cend - c0);
    for (int e = threadIdx.x; e < nc * DP; e += blockDim.x) S.tv[e] = A.vr[c0 * DP + e];
    for (int e = threadIdx.x; e < nc; e += blockDim.x) S.tB[e] = A.Br[c0 + e];
    __syncthreads();
    if (!active) continue;
    int cmax = nc;
    if (A.ordered) {
      const int64_t lim = i - c0;  // candidates j < i
      if (lim <= 0) continue;
      if (lim < cmax) cmax = (int)lim;
    }
    for (int cc0 = 0; cc0 < cmax; cc0 += 32) {
      const int cc = cc0 + lane;
      float s32 = 0.0f, Bc = 0.0f;
      const bool in = cc < cmax;
      if (in) {
        const float* tv = S.tv + cc * DP;
#pragma unroll
        for (int l = 0; l < DP; l += 4) {
          const float4 t4 = *reinterpret_cast<const float4*>(tv + l);
          float df = __fsub_rn(qv[l], t4.x);
          s32 = __fmaf_rn(df, df, s32);
          df = __fsub_rn(qv[l + 1], t4.y);
          s32 = __fmaf_rn(df, df, s32);
          df = __fsub_rn(qv[l + 2], t4.z);
          s32 = __fmaf_rn(df, df, s32);
          df = __fsub_rn(qv[l + 3], t4.w);
          s32 = __fmaf_rn(df, df, s32);
        }
        Bc = S.tB[cc];
      }
      // keep unless lo > tau': sqrt(s32 / g) > Tq + B_c
      auto keep_of = [&]() {
        if (!in) return false;
        const float tb = __fadd_ru(Tq, Bc);
        return !(s32 > __fmul_ru(__fmul_ru(tb, tb), g));
      };
      bool keep = keep_of();
      unsigned km = __ballot_sync(0xffffffffu, keep);
      if (!km) continue;
      if (cnt + __popc(km) > cap) {
        compact();
        keep = keep_of();
        km = __ballot_sync(0xffffffffu, keep);
      }
      if (keep) {
        const int p = cnt + __popc(km & ((1u << lane) - 1));
        const float bsum = __fadd_ru(Bi, Bc);
        bh[p] = __fadd_ru(__fsqrt_ru(__fmul_ru(s32, g)), bsum);
        bl[p] = __fsub_rd(__fsqrt_rd(__fdiv_rd(s32, g)), bsum);
        bi[p] = (int)(c0 + cc);
      }
      cnt += __popc(km);
      __syncwarp();
    }
  }
  if (!valid) return;
  int nout = 0;
  if (active && cnt > 0) {
    wq_exact_sort(S, w, cnt, xq, A.Xr, A.d, cap, sortw);
    nout = min(cnt, kq);
  }
  const int* bsi = S.bsi + (size_t)w * sortw;
  if (A.nbr) {
    int32_t* row = A.nbr + (A.b0 + i) * (int64_t)A.ldnbr;
    for (int c = lane; c < A.ldnbr; c += 32) row[c] = c < nout ? bsi[c] : -1;
  } else if (A.ordered) {
    int64_t* row = A.out + i * (int64_t)(A.m + 1);
    if (lane == 0) row[0] = i;
    for (int c = lane; c < A.m; c += 32) row[1 + c] = c < nout ? (int64_t)bsi[c] : -1;
  } else {
    int64_t* row = A.out + i * (int64_t)A.k;
    for (int c = lane; c < A.k; c += 32) row[c] = c < nout ? (int64_t)bsi[c] : -1;
  }
}

template <int DP>
__global__ void __launch_bounds__(256) k_knn_wq(KnnArgs A) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nw = blockDim.x >> 5;
  const int64_t ntile = (A.nq + nw - 1) / nw;
  // ordered searches: largest rows first (their work grows with the row index)
  knn_wq_tile<DP>(A, A.ordered ? (ntile - 1 - blockIdx.x) : blockIdx.x, smraw);
}

// batched ordered search, one warp per query row: entry t of the tile table
// is (problem, tile of blockDim.x / 32 rows)
template <int DP>
__global__ void __launch_bounds__(256) k_knn_wq_batched(const KnnBatchProb* probs, const int2* tiles,
                                                         const double* Xs, const float* v,
                                                         const float* B, int32_t* nbr, int ldnbr,
                                                         int kcap, float growth, int cap, int sortw) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int2 te = tiles[blockIdx.x];
  const KnnBatchProb& P = probs[te.x];
  KnnArgs A;
  A.Xq = Xs + P.xs_off;
  A.Xr = A.Xq;
  A.vq = v + P.v_off;
  A.vr = A.vq;
  A.Bq = B + P.row_off;
  A.Br = A.Bq;
  A.nq = P.n;
  A.nr = P.n;
  A.d = P.d;
  A.k = kcap;
  A.m = P.m;
  A.start = 1;
  A.out = nullptr;
  A.growth = growth;
  A.ordered = 1;
  A.nbr = nbr;
  A.b0 = P.blk_off;
  A.ldnbr = ldnbr;
  A.wq_cap = cap;
  A.wq_sort = sortw;
  knn_wq_tile<DP>(A, te.y, smraw);
}

static int pad_dim(int d) {
  if (d <= 4) return 4;
  if (d <= 8) return 8;
  if (d <= 12) return 12;
  if (d <= 16) return 16;
  if (d <= 24) return 24;
  if (d <= 32) return 32;
  if (d <= 48) return 48;
  return 64;
}

static float growth_factor(int DP) {
  double g = 1.0;
  for (int i = 0; i < DP + 2; ++i) g *= (1.0 + 0x1p-24);
  g *= (1.0 + 0x1p-20);
  float gf = (float)g;
  if ((double)gf < g) gf = nextafterf(gf, 2.0f);
  return gf;
}

static int knn_max_smem() {
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return maxsm;
}

// whether k takes the warp-per-query path, with its warps per CTA and shared memory
static bool wq_plan(int k, int DP, int* warps, size_t* smem) {
  if (k < 1 || k > kWqMaxK || DP > 16) return false;
  const int cap = wq_cap(k), sw = wq_sort(cap);
  int w = 8;
  while (w > 1 && wq_smem_bytes(DP, w, cap, sw) > (size_t)knn_max_smem()) --w;
  if (wq_smem_bytes(DP, w, cap, sw) > (size_t)knn_max_smem()) return false;
  if (warps) *warps = w;
  if (smem) *smem = wq_smem_bytes(DP, w, cap, sw);
  return true;
}

// the warp-per-query search: for large k, and for moderate k while the
// candidate sets are small enough that list insertions, not the screen,
// dominate the per-thread search (measured: 4x faster at n = 20k, m = 20;
// 15 % slower at n = 200k, m = 30)
static bool use_wq(int k, int64_t nr, int DP) {
  if (!wq_plan(k, DP, nullptr, nullptr)) return false;
  return k >= kKnnHeapMin || (k >= 16 && nr <= 65536);
}

static int launch_knn(const KnnArgs& A, int DP, int64_t grid, size_t smem, cudaStream_t st) {
  if (use_wq(A.k, A.nr, DP)) {
    // large k: one warp per query, as many warps per CTA (up to 8) as fit
    KnnArgs W = A;
    int warps = 0;
    size_t wsm = 0;
    wq_plan(A.k, DP, &warps, &wsm);
    W.wq_cap = wq_cap(A.k);
    W.wq_sort = wq_sort(W.wq_cap);
    const int64_t wgrid = (A.nq + warps - 1) / warps;
    switch (DP) {
#define SV_WQ_CASE(V)                                                                          \
  case V:                                                                                      \
    SV_CUDA_TRY(cudaFuncSetAttribute(k_knn_wq<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)wsm));                                               \
    k_knn_wq<V><<<(unsigned)wgrid, warps * 32, wsm, st>>>(W);                                 \
    break;
      SV_WQ_CASE(4)
      SV_WQ_CASE(8)
      SV_WQ_CASE(12)
      SV_WQ_CASE(16)
#undef SV_WQ_CASE
      default:
        return SV_EINVAL;
    }
    SV_CUDA_TRY(cudaGetLastError());
    return SV_OK;
  }
  switch (DP) {
#define SV_KNN_CASE(V)                                                                          \
  case V:                                                                                       \
    SV_CUDA_TRY(cudaFuncSetAttribute(k_knn<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)smem));                                               \
    k_knn<V><<<(unsigned)grid, kKnnQ, smem, st>>>(A);                                          \
    break;
    SV_KNN_CASE(4)
    SV_KNN_CASE(8)
    SV_KNN_CASE(12)
    SV_KNN_CASE(16)
    SV_KNN_CASE(24)
    SV_KNN_CASE(32)
    SV_KNN_CASE(48)
    SV_KNN_CASE(64)
#undef SV_KNN_CASE
    default:
      return SV_EINVAL;
  }
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// batched ordered search: entry t of the tile table is (problem, query tile)
template <int DP>
__global__ void __launch_bounds__(kKnnQ) k_knn_batched(const KnnBatchProb* probs, const int2* tiles,
                                                        const double* Xs, const float* v,
                                                        const float* B, int32_t* nbr, int ldnbr,
                                                        int kcap, float growth) {
  extern __shared__ unsigned char smraw[];
  const int2 te = tiles[blockIdx.x];
  const KnnBatchProb& P = probs[te.x];
  KnnArgs A;
  A.Xq = Xs + P.xs_off;
  A.Xr = A.Xq;
  A.vq = v + P.v_off;
  A.vr = A.vq;
  A.Bq = B + P.row_off;
  A.Br = A.Bq;
  A.nq = P.n;
  A.nr = P.n;
  A.d = P.d;
  A.k = kcap;
  A.m = P.m;
  A.start = 1;
  A.out = nullptr;
  A.growth = growth;
  A.ordered = 1;
  A.nbr = nbr;
  A.b0 = P.blk_off;
  A.ldnbr = ldnbr;
  knn_tile<DP>(A, te.y, smraw);
}

int knn_pad_dim(int d) { return pad_dim(d); }

int knn_batched_tile_rows(int DP, int kcap) {
  int warps = 0;
  return wq_plan(kcap, DP, &warps, nullptr) ? warps : kKnnQ;
}

int launch_knn_batched(int DP, const KnnBatchProb* probs, const int2* tiles, int64_t ntiles,
                       const double* Xs, const float* v, const float* B, int32_t* nbr, int ldnbr,
                       int kcap, cudaStream_t st) {
  if (ntiles <= 0) return SV_OK;
  int warps = 0;
  size_t wsm = 0;
  if (wq_plan(kcap, DP, &warps, &wsm)) {
    // one warp per row: the table's tiles are knn_batched_tile_rows(DP, kcap) = warps rows
    const float g = growth_factor(DP);
    const int cap = wq_cap(kcap), sw = wq_sort(cap);
    switch (DP) {
#define SV_WQB_CASE(V)                                                                                \
  case V:                                                                                             \
    SV_CUDA_TRY(cudaFuncSetAttribute(k_knn_wq_batched<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)wsm));                                                      \
    k_knn_wq_batched<V><<<(unsigned)ntiles, warps * 32, wsm, st>>>(probs, tiles, Xs, v, B, nbr, ldnbr, \
                                                                   kcap, g, cap, sw);               \
    break;
      SV_WQB_CASE(4)
      SV_WQB_CASE(8)
      SV_WQB_CASE(12)
      SV_WQB_CASE(16)
#undef SV_WQB_CASE
      default:
        return SV_EINVAL;
    }
    SV_CUDA_TRY(cudaGetLastError());
    return SV_OK;
  }
  const size_t smem = sizeof(float) * (size_t)kKnnC * DP + sizeof(float) * kKnnC +
                      (sizeof(double) + sizeof(int)) * (size_t)kcap * kKnnQ;
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > (size_t)maxsm) return SV_EINVAL;
  const float g = growth_factor(DP);
  switch (DP) {
#define SV_KNNB_CASE(V)                                                                           \
  case V:                                                                                        \
    SV_CUDA_TRY(cudaFuncSetAttribute(k_knn_batched<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)smem));                                                \
    k_knn_batched<V><<<(unsigned)ntiles, kKnnQ, smem, st>>>(probs, tiles, Xs, v, B, nbr, ldnbr,  \
                                                             kcap, g);                           \
    break;
    SV_KNNB_CASE(4)
    SV_KNNB_CASE(8)
    SV_KNNB_CASE(12)
    SV_KNNB_CASE(16)
    SV_KNNB_CASE(24)
    SV_KNNB_CASE(32)
    SV_KNNB_CASE(48)
    SV_KNNB_CASE(64)
#undef SV_KNNB_CASE
    default:
      return SV_EINVAL;
  }
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

}  // namespace sv

using namespace sv;

extern "C" size_t sv_ordered_knn_workspace_bytes(int64_t n, int32_t d) {
  const int DP = pad_dim(d > 0 ? d : 1);
  return al256(sizeof(double) * 64) + al256(sizeof(float) * (size_t)(n > 0 ? n : 1) * DP) +
         al256(sizeof(float) * (size_t)(n > 0 ? n : 1));
}

extern "C" size_t sv_knn_query_workspace_bytes(int64_t nref, int64_t nq, int32_t d) {
  return sv_ordered_knn_workspace_bytes(nref, d) + sv_ordered_knn_workspace_bytes(nq, d);
}

static int knn_smem_ok(int DP, int k, size_t* smem) {
  *smem = sizeof(float) * (size_t)kKnnC * DP + sizeof(float) * kKnnC +
          (sizeof(double) + sizeof(int)) * (size_t)k * kKnnQ;
  if (k >= kKnnHeapMin && wq_plan(k, DP, nullptr, smem)) return 1;
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return *smem <= (size_t)maxsm;
}

extern "C" int sv_ordered_knn(const double* X, int64_t n, int32_t d, int32_t m, int64_t start,
                              int64_t* nn, int32_t* info, void* workspace, size_t workspace_bytes,
                              sv_stream_t stream) {
  if (n < 0 || d < 1 || d > 64 || m < 0 || start < 0 || (n > 0 && (!X || !nn)) || !info)
    return SV_EINVAL;
  if (n > 0x7fffffffLL) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  if (n == 0) return SV_OK;
  if (!workspace || workspace_bytes < sv_ordered_knn_workspace_bytes(n, d)) return SV_ENOSPC;
  const int DP = pad_dim(d);
  size_t smem;
  if (!knn_smem_ok(DP, m > 0 ? m : 1, &smem)) return SV_EINVAL;
  char* ws = (char*)workspace;
  double* centroid = (double*)ws;
  float* v = (float*)(ws + al256(sizeof(double) * 64));
  float* B = (float*)((char*)v + al256(sizeof(float) * (size_t)n * DP));
  k_centroid2<<<d, 256, 0, st>>>(X, n, d, centroid);
  SV_CUDA_TRY(cudaGetLastError());
  int64_t g = (n + 255) / 256;
  if (g > 8LL * sv_num_sms()) g = 8LL * sv_num_sms();
  k_knn_prep<<<(unsigned)g, 256, 0, st>>>(X, n, d, DP, centroid, v, B);
  SV_CUDA_TRY(cudaGetLastError());
  KnnArgs A;
  A.Xq = X;
  A.Xr = X;
  A.vq = v;
  A.vr = v;
  A.Bq = B;
  A.Br = B;
  A.nq = n;
  A.nr = n;
  A.d = d;
  A.k = m > 0 ? m : 1;
  A.m = m;
  A.start = start > 1 ? start : 1;
  A.out = nn;
  A.growth = growth_factor(DP);
  A.ordered = 1;
  A.nbr = nullptr;
  A.b0 = 0;
  A.ldnbr = 0;
  const int64_t ntile = (n + kKnnQ - 1) / kKnnQ;
  return launch_knn(A, DP, ntile, smem, st);
}

extern "C" int sv_knn_query(const double* Xref, int64_t nref, const double* Xq, int64_t nq,
                            int32_t d, int32_t k, int64_t* nb, int32_t* info, void* workspace,
                            size_t workspace_bytes, sv_stream_t stream) {
  if (nref < 0 || nq < 0 || d < 1 || d > 64 || k < 1 || (nq > 0 && (!Xq || !nb)) ||
      (nref > 0 && !Xref) || !info)
    return SV_EINVAL;
  if (nref > 0x7fffffffLL || nq > 0x7fffffffLL) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  if (nq == 0) return SV_OK;
  if (!workspace || workspace_bytes < sv_knn_query_workspace_bytes(nref, nq, d)) return SV_ENOSPC;
  const int DP = pad_dim(d);
  size_t smem;
  if (!knn_smem_ok(DP, k, &smem)) return SV_EINVAL;
  char* ws = (char*)workspace;
  double* centroid = (double*)ws;
  float* vr = (float*)(ws + al256(sizeof(double) * 64));
  float* Br = (float*)((char*)vr + al256(sizeof(float) * (size_t)(nref > 0 ? nref : 1) * DP));
  char* ws2 = ws + sv_ordered_knn_workspace_bytes(nref, d);
  float* vq = (float*)(ws2 + al256(sizeof(double) * 64));
  float* Bq = (float*)((char*)vq + al256(sizeof(float) * (size_t)nq * DP));
  // one shift for both sets (the reference rows' centroid)
  if (nref > 0) {
    k_centroid2<<<d, 256, 0, st>>>(Xref, nref, d, centroid);
  } else {
    SV_CUDA_TRY(cudaMemsetAsync(centroid, 0, sizeof(double) * d, st));
  }
  SV_CUDA_TRY(cudaGetLastError());
  int64_t g = (nref + 255) / 256;
  if (g > 8LL * sv_num_sms()) g = 8LL * sv_num_sms();
  if (nref > 0) k_knn_prep<<<(unsigned)(g > 0 ? g : 1), 256, 0, st>>>(Xref, nref, d, DP, centroid, vr, Br);
  g = (nq + 255) / 256;
  if (g > 8LL * sv_num_sms()) g = 8LL * sv_num_sms();
  k_knn_prep<<<(unsigned)g, 256, 0, st>>>(Xq, nq, d, DP, centroid, vq, Bq);
  SV_CUDA_TRY(cudaGetLastError());
  KnnArgs A;
  A.Xq = Xq;
  A.Xr = Xref;
  A.vq = vq;
  A.vr = vr;
  A.Bq = Bq;
  A.Br = Br;
  A.nq = nq;
  A.nr = nref;
  A.d = d;
  A.k = k;
  A.m = k;
  A.start = 0;
  A.out = nb;
  A.growth = growth_factor(DP);
  A.ordered = 0;
  A.nbr = nullptr;
  A.b0 = 0;
  A.ldnbr = 0;
  const int64_t ntile = (nq + kKnnQ - 1) / kKnnQ;
  return launch_knn(A, DP, ntile, smem, st);
}
