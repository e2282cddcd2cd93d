// Exact maximin ordering on the GPU: ordering.py:27-59 (_maximin_core).
//
// A persistent cooperative kernel.  Each CTA owns a contiguous slice of the
// points and keeps, in shared memory, per point: its coordinates centred on
// the data centroid and rounded to float32, its current distance dist[p]
// (float64, exactly as the reference computes it) and a float32 skip
// threshold.  One step of the reference loop (pivot j):
//   for every remaining point p: dj = sqrt(sum_l (x_pl - x_jl)^2) in IEEE
//   sequential float64 (no FMA); if dj < dist[p]: dist[p] = dj;
//   dist[j] = -1; next pivot = argmax dist (strict '>', smallest index wins).
// The float64 distance is only evaluated when a float32 lower bound of it
// could be below dist[p]: the float32 squared distance s32 of the rounded,
// centred coordinates obeys
//   D >= sqrt(s32) (1+u)^-(d+2)/2 - B_p - B_j,   u = 2^-24,
// with B_p >= |fl32(x_p - c) - (x_p - c)|_2 (computed per point), and
//   fl64(sqrt(s64)) >= D (1 - (d+4) 2^-53),
// so s32 >= (dist[p](1+(d+4)2^-53) + B_p + B_j)^2 (1+u)^(d+2) proves that
// the reference would not update p; the threshold is formed with upward
// rounding.  Every update decision is therefore the reference's own.
//
// The per-CTA candidates (dist bits, index) meet through a double-buffered
// slot array and a monotone arrival counter; waits are bounded
// (SV_ETIMEOUT).  Every CTA reduces the same candidates in the same way, so
// all agree on the next pivot.
#include "sv_reorder.cuh"

namespace sv {

constexpr int kMmThreads = 512;

struct MmArgs {
  const double* X;
  int64_t n;
  int d;
  int64_t first;
  int64_t* order;
  int32_t* info;
  const double* centroid;  // d doubles (device)
  long long* slot_bits;    // [2][G]
  long long* slot_idx;     // [2][G]
  unsigned* arrive;
  int64_t per_cta;         // points per CTA
  float growth;            // (1+2^-24)^(d+2) (1+2^-20), rounded up
};


__global__ void __launch_bounds__(kMmThreads) k_maximin(MmArgs A) {
  extern __shared__ unsigned char smraw[];
  const int d = A.d;
  const int G = gridDim.x;
  const int64_t p0 = (int64_t)blockIdx.x * A.per_cta;
  const int64_t p1 = min(A.n, p0 + A.per_cta);
  const int S = (int)max((int64_t)0, p1 - p0);
  const int Sc = (int)A.per_cta;
  // shared layout: dist[Sc] f64 | Bp[Sc] f64 | thr[Sc] f32 | v[d][Sc] f32 | misc
  double* dist = (double*)smraw;
  double* Bp = dist + Sc;
  float* thr = (float*)(Bp + Sc);
  float* v = thr + Sc;
  __shared__ double xj[64];
  __shared__ float vj[64];
  __shared__ float Bj_f;
  __shared__ long long red_bits[kMmThreads / 32];
  __shared__ long long red_idx[kMmThreads / 32];
  __shared__ long long s_pivot;
  __shared__ int s_abort;

  // ---- init: centred float32 coordinates and their rounding bound
  for (int p = threadIdx.x; p < S; p += blockDim.x) {
    const double* xp = A.X + (p0 + p) * d;
    double e2 = 0.0;
    for (int l = 0; l < d; ++l) {
      const double c = xp[l] - A.centroid[l];
      v[l * Sc + p] = __double2float_rn(c);
      e2 += c * c;
    }
    Bp[p] = 1.01 * 0x1p-24 * sqrt(e2);
    dist[p] = __longlong_as_double(0x7ff0000000000000LL);  // +inf: first pass is exact
    thr[p] = __int_as_float(0x7f800000);
  }
  if (threadIdx.x == 0) {
    s_pivot = A.first;
    s_abort = 0;
    if (blockIdx.x == 0) A.order[0] = A.first;
  }
  __syncthreads();

  for (int64_t t = 0; t + 1 < A.n; ++t) {
    const long long j = s_pivot;
    // pivot coordinates (exact) and its float32 image
    if (threadIdx.x < d) {
      const double x = A.X[j * d + threadIdx.x];
      xj[threadIdx.x] = x;
      vj[threadIdx.x] = __double2float_rn(x - A.centroid[threadIdx.x]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double e2 = 0.0;
      for (int l = 0; l < d; ++l) {
        const double c = xj[l] - A.centroid[l];
        e2 += c * c;
      }
      Bj_f = __double2float_ru(1.01 * 0x1p-24 * sqrt(e2));
    }
    __syncthreads();
    const float bj = Bj_f;

    // ---- update + local argmax
    long long best_bits = -1LL;  // below every non-negative double
    long long best_idx = 0x7fffffffffffffffLL;
    for (int p = threadIdx.x; p < S; p += blockDim.x) {
      double dp = dist[p];
      // already ordered (ordering.py:50-51); sign test on the bits keeps the
      // common path off the float64 pipe
      if (__double_as_longlong(dp) < 0) continue;
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
      const float bound = __fmul_ru(__fmul_ru(tb, tb), A.growth);
      if (!(s32 >= bound)) {
        // possible update: decide exactly (ordering.py:52-57)
        const double dj = __dsqrt_rn(sqdist_exact(A.X + gp * d, xj, d));
        if (dj < dp) {
          dp = dj;
          dist[p] = dj;
          thr[p] = thr_base(dj, Bp[p], d);
        }
      }
      const long long bits = __double_as_longlong(dp);
      if (bits > best_bits && bits <= 0x7ff0000000000000LL) {
        best_bits = bits;
        best_idx = gp;
      }
    }
    // CTA reduction: larger distance wins, then smaller index
    for (int o = 16; o > 0; o >>= 1) {
      const long long ob = __shfl_down_sync(0xffffffffu, best_bits, o);
      const long long oi = __shfl_down_sync(0xffffffffu, best_idx, o);
      if (ob > best_bits || (ob == best_bits && oi < best_idx)) {
        best_bits = ob;
        best_idx = oi;
      }
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
      red_bits[w] = best_bits;
      red_idx[w] = best_idx;
    }
    __syncthreads();
    const int par = (int)(t & 1);
    if (threadIdx.x == 0) {
      long long bb = red_bits[0], bi = red_idx[0];
      for (int k = 1; k < (int)(blockDim.x >> 5); ++k)
        if (red_bits[k] > bb || (red_bits[k] == bb && red_idx[k] < bi)) {
          bb = red_bits[k];
          bi = red_idx[k];
        }
      if (G == 1) {
        s_pivot = bi;
      } else {
        A.slot_bits[par * G + blockIdx.x] = bb;
        A.slot_idx[par * G + blockIdx.x] = bi;
        __threadfence();
        atomicAdd(A.arrive, 1u);
        const unsigned target = (unsigned)G * (unsigned)(t + 1);
        unsigned it = 0;
        while (ld_acquire_u32(A.arrive) < target) {
          if (++it > (SV_SPIN_LIMIT >> 4)) {
            set_error(A.info + SV_INFO_STATUS, SV_ETIMEOUT);
            A.info[SV_INFO_BLOCK] = (int)t;
            s_abort = 1;
            break;
          }
        }
        __threadfence();
      }
    }
    __syncthreads();
    if (s_abort) return;
    if (G > 1) {
      // every CTA reduces all candidates identically
      long long bb = -1LL, bi = 0x7fffffffffffffffLL;
      for (int c = threadIdx.x; c < G; c += blockDim.x) {
        const long long cb = __ldcg(A.slot_bits + par * G + c);
        const long long ci = __ldcg(A.slot_idx + par * G + c);
        if (cb > bb || (cb == bb && ci < bi)) {
          bb = cb;
          bi = ci;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const long long ob = __shfl_down_sync(0xffffffffu, bb, o);
        const long long oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > bb || (ob == bb && oi < bi)) {
          bb = ob;
          bi = oi;
        }
      }
      if ((threadIdx.x & 31) == 0) {
        red_bits[w] = bb;
        red_idx[w] = bi;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        long long b2 = red_bits[0], i2 = red_idx[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k)
          if (red_bits[k] > b2 || (red_bits[k] == b2 && red_idx[k] < i2)) {
            b2 = red_bits[k];
            i2 = red_idx[k];
          }
        s_pivot = i2;
      }
      __syncthreads();
    }
    // no finite candidate left (NaN inputs): report instead of indexing with it
    if (s_pivot == 0x7fffffffffffffffLL) {
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        set_error(A.info + SV_INFO_STATUS, SV_EINVAL);
        A.info[SV_INFO_BLOCK] = (int)t;
      }
      return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) A.order[t + 1] = s_pivot;
  }
}

__global__ void k_centroid(const double* X, int64_t n, int d, double* c) {
  // mean of each column (only a shift for the float32 filter; any value works)
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

}  // namespace sv

using namespace sv;

static size_t mm_align(size_t x) { return (x + 255) & ~(size_t)255; }

extern "C" size_t sv_maximin_workspace_bytes(int64_t n, int32_t d) {
  (void)n;
  const int G = 4 * sv_num_sms();
  return mm_align(sizeof(double) * (size_t)(d > 0 ? d : 1)) + mm_align(2 * sizeof(long long) * 2 * G) +
         256;
}

extern "C" int sv_maximin_order(const double* X, int64_t n, int32_t d, int64_t first,
                                int64_t* order, int32_t* info, void* workspace,
                                size_t workspace_bytes, sv_stream_t stream) {
  if (n < 0 || d < 1 || d > 64 || (n > 0 && (!X || !order)) || !info) return SV_EINVAL;
  if (n > 0 && (first < 0 || first >= n)) return SV_EINVAL;
  if (n > 0x7fffffffLL) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  if (n == 0) return SV_OK;
  if (n == 1) {
    SV_CUDA_TRY(cudaMemcpyAsync(order, &first, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    return SV_OK;
  }
  if (!workspace || workspace_bytes < sv_maximin_workspace_bytes(n, d)) return SV_ENOSPC;
  // problems that fit one thread-block cluster: hardware cluster barrier per
  // step instead of the grid-wide exchange below
  if (n <= maximin_cluster_max_rows(d))
    return maximin_cluster_single(X, n, d, first, order, info, (char*)workspace, st);
  const int nsm = sv_num_sms();
  char* ws = (char*)workspace;
  double* centroid = (double*)ws;
  size_t off = mm_align(sizeof(double) * d);
  long long* slots = (long long*)(ws + off);
  const int Gmax_ws = 4 * nsm;
  off += mm_align(2 * sizeof(long long) * 2 * Gmax_ws);
  unsigned* arrive = (unsigned*)(ws + off);

  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t static_smem = 64 * 8 + 64 * 4 + 4 + 2 * 8 * (kMmThreads / 32) + 16;
  const size_t per_pt = 8 + 8 + 4 + 4 * (size_t)d;
  // points per CTA: spread over the SMs, at least 64 per CTA
  int64_t G = nsm;
  int64_t per = (n + G - 1) / G;
  if (per < 64) {
    per = 64;
    G = (n + per - 1) / per;
  }
  size_t dyn = per * per_pt;
  if (dyn + static_smem > (size_t)maxsm) return SV_EINVAL;  // too many points for one pass
  SV_CUDA_TRY(cudaFuncSetAttribute(k_maximin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  int active = 0;
  SV_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&active, k_maximin, kMmThreads, dyn));
  if (active < 1 || G > (int64_t)active * nsm || G > Gmax_ws) return SV_EINVAL;

  k_centroid<<<d, 256, 0, st>>>(X, n, d, centroid);
  SV_CUDA_TRY(cudaGetLastError());
  SV_CUDA_TRY(cudaMemsetAsync(arrive, 0, sizeof(unsigned), st));

  MmArgs A;
  A.X = X;
  A.n = n;
  A.d = d;
  A.first = first;
  A.order = order;
  A.info = info;
  A.centroid = centroid;
  A.slot_bits = slots;
  A.slot_idx = slots + 2 * G;
  A.arrive = arrive;
  A.per_cta = per;
  {
    double g = 1.0;
    for (int i = 0; i < d + 2; ++i) g *= (1.0 + 0x1p-24);
    g *= (1.0 + 0x1p-20);
    float gf = (float)g;
    if ((double)gf < g) gf = nextafterf(gf, 2.0f);
    A.growth = gf;
  }
  void* args[] = {&A};
  SV_CUDA_TRY(cudaLaunchCooperativeKernel((void*)k_maximin, dim3((unsigned)G), dim3(kMmThreads), args,
                                          dyn, st));
  return SV_OK;
}
