// Device helpers shared by the pass maximin kernels (sv_reorder.cu: cluster
// and grid forms; sv_maximin_tree.cu: the tree form): candidate keys and
// their warp-level sorting, the rigorous float32 screen and its thresholds.
// Keys order points as ordering.py:42-47 does: the larger squared distance
// first (bit patterns of non-negative float64 values order like the values),
// then the smaller row index.
#pragma once
#include "sv_common.cuh"

namespace sv {

constexpr int kMcU = 31;  // candidates per pass: lanes 0..30 of the merged list
constexpr int kMcNone = 0x7fffffff;

// candidate order: larger squared-distance bits first, then the smaller index
__device__ __forceinline__ bool mc_greater(long long ab, int ai, long long bb, int bi) {
  return ab > bb || (ab == bb && ai < bi);
}

// two bitonic sorts of one key per lane, descending in mc_greater order, at
// once (independent chains, one latency)
__device__ __forceinline__ void mc_warp_sort2(long long& b, int& i, long long& c, int& j) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
    for (int s = k >> 1; s > 0; s >>= 1) {
      const long long ob = __shfl_xor_sync(0xffffffffu, b, s);
      const int oi = __shfl_xor_sync(0xffffffffu, i, s);
      const long long oc = __shfl_xor_sync(0xffffffffu, c, s);
      const int oj = __shfl_xor_sync(0xffffffffu, j, s);
      const bool take_greater = ((lane & k) == 0) == ((lane & s) == 0);
      if (mc_greater(ob, oi, b, i) == take_greater) {
        b = ob;
        i = oi;
      }
      if (mc_greater(oc, oj, c, j) == take_greater) {
        c = oc;
        j = oj;
      }
    }
}

// top 32 of two descending lists (own keys and (ob, oi), in lane order),
// descending; every key left out is below the 32nd key kept
__device__ __forceinline__ void mc_warp_merge(long long& b, int& i, long long ob, int oi) {
  const int lane = threadIdx.x & 31;
  const long long rb = __shfl_sync(0xffffffffu, ob, 31 - lane);
  const int ri = __shfl_sync(0xffffffffu, oi, 31 - lane);
  if (mc_greater(rb, ri, b, i)) {
    b = rb;
    i = ri;
  }
#pragma unroll
  for (int j = 16; j > 0; j >>= 1) {
    const long long xb = __shfl_xor_sync(0xffffffffu, b, j);
    const int xi = __shfl_xor_sync(0xffffffffu, i, j);
    if (mc_greater(xb, xi, b, i) == ((lane & j) == 0)) {
      b = xb;
      i = xi;
    }
  }
}

// largest key of the warp, in every lane
__device__ __forceinline__ void mc_warp_max(long long& b, int& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long ob = __shfl_xor_sync(0xffffffffu, b, o);
    const int oi = __shfl_xor_sync(0xffffffffu, i, o);
    if (mc_greater(ob, oi, b, i)) {
      b = ob;
      i = oi;
    }
  }
}

__device__ __forceinline__ long long mc_warp_max_bits(long long b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  return b;
}

// float32 screening threshold from a squared distance: an upper bound of
// (fl(sqrt(s)) (1 + (d+4) 2^-53) + B_p) (1 + 2^-40), d <= 64
__device__ __forceinline__ float thr_sq(double s, float Bp) {
  const float r = __fsqrt_ru(__double2float_ru(s));  // >= sqrt(s)
  return __fmul_ru(__fadd_ru(r, Bp), 1.0f + 0x1p-20f);
}

// float32 screen: false only when the pivot cannot lower the stored distance
// (s32 = float32 squared distance of the centred images, th = the point's
// threshold, Bj = the pivot's rounding bound)
__device__ __forceinline__ bool mc_may_update(float s32, float th, float Bj, float growth) {
  const float tb = __fadd_ru(th, Bj);
  return !(s32 >= __fmul_ru(__fmul_ru(tb, tb), growth));
}

// upper bound of the exact squared distance (ordering.py:52-57) between two
// rows from their images' float32 squared distance s32 and rounding bounds
// Ba, Bb: (sqrt(s32 growth^2) + Ba + Bb)^2 (1 + 2^-20), rounded up
__device__ __forceinline__ float mc_sq_upper(float s32, float Ba, float Bb, float growth) {
  const float t = __fadd_ru(__fadd_ru(__fsqrt_ru(__fmul_ru(__fmul_ru(s32, growth), growth)), Ba), Bb);
  return __fmul_ru(__fmul_ru(t, t), 1.0f + 0x1p-20f);
}

// rounding bound of a float32 image v = fl32(c) of a centred row c:
// ||c - v|| <= 2^-24 (1 + 2^-23) ||v||, formed with upward rounding
__device__ __forceinline__ float mc_img_bound(const float* v, int d) {
  float e2 = 0.0f;
  for (int l = 0; l < d; ++l) e2 = __fmaf_ru(v[l], v[l], e2);
  return __fmul_ru(__fsqrt_ru(e2), 1.01f * 0x1p-24f);
}

// (1+2^-24)^(d+2) (1+2^-20) as a float32 rounded up
__device__ __forceinline__ float mc_growth(int d) {
  double g = 1.0;
  for (int i = 0; i < d + 2; ++i) g *= (1.0 + 0x1p-24);
  return __double2float_ru(g * (1.0 + 0x1p-20));
}

// keep the three largest keys b1 > b2 > b3 (mc_greater order)
__device__ __forceinline__ void mc_insert3(long long b, int i, long long& b1, int& i1, long long& b2,
                                           int& i2, long long& b3, int& i3) {
  if (mc_greater(b, i, b1, i1)) {
    b3 = b2;
    i3 = i2;
    b2 = b1;
    i2 = i1;
    b1 = b;
    i1 = i;
  } else if (mc_greater(b, i, b2, i2)) {
    b3 = b2;
    i3 = i2;
    b2 = b;
    i2 = i;
  } else if (mc_greater(b, i, b3, i3)) {
    b3 = b;
    i3 = i;
  }
}

}  // namespace sv
