// Shared definitions for the scaled Vecchia sm_103a kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/svgpu.h"

#ifndef SV_HOST_DEVICE
#define SV_HOST_DEVICE __host__ __device__ __forceinline__
#endif

#define SV_CUDA_TRY(expr)                                   \
  do {                                                      \
    cudaError_t e_ = (expr);                                \
    if (e_ != cudaSuccess) return sv_record_cuda_error(e_); \
  } while (0)

// Bounded spin-waits: a wait that runs out of iterations sets SV_ETIMEOUT in
// the kernel's error word and the kernel returns instead of hanging.  2^22
// polls of a word in L2 (each a few hundred nanoseconds) take about a second,
// far beyond any wait these kernels have when they work (microseconds).
#define SV_SPIN_LIMIT (1u << 22)
// the limit under the test aids that make a wait run out on purpose
#define SV_SPIN_LIMIT_TEST (1u << 12)

int sv_record_cuda_error(cudaError_t e);
int sv_num_sms();

namespace sv {

__device__ __forceinline__ void set_error(int32_t* err, int32_t code) {
  if (err) atomicCAS(err, 0, code);
}

// acquire / release accessors for inter-CTA flags (PTX memory model)
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_s32(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_release_u32(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// Row/column of the t-th entry of a packed lower triangle (row-major, i >= j).
__device__ __forceinline__ void tri_index(int t, int& i, int& j) {
  int r = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  // correct the float estimate
  while ((r + 1) * (r + 2) / 2 <= t) ++r;
  while (r * (r + 1) / 2 > t) --r;
  i = r;
  j = t - r * (r + 1) / 2;
}
__device__ __forceinline__ int tri_off(int i, int j) { return i * (i + 1) / 2 + j; }

// Order tests on the bit patterns of positive numbers (integer pipe): for
// x, y >= 0, x < y <=> bits(x) < bits(y).
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
constexpr long long kBitsTiny = 0x39B4484BFEEBC2A0LL;  // 1e-30
constexpr long long kBitsHuge = 0x46293E5939A08CEALL;  // 1e30
constexpr long long kBitsInf = 0x7FF0000000000000LL;
constexpr int kFBitsInf = 0x7F800000;

// |x| < 1e30 for a float64 x (bit test; NaN fails)
__device__ __forceinline__ bool in_f32_range(double x) {
  return (dbits(x) & 0x7FFFFFFFFFFFFFFFLL) < kBitsHuge;
}

// float32 -> float64 by bit manipulation (integer pipe; a float64 conversion
// instruction would occupy the slow float64 pipe): exact for zero and normal
// numbers, subnormals become a signed zero, infinities and NaN stay so.
__device__ __forceinline__ double f2d_int(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned s = b & 0x80000000u;
  const unsigned e64 = e == 0xffu ? 0x7ffu : e + 896u;
  const unsigned hi = e == 0u ? s : (s | (e64 << 20) | ((b & 0x7fffffu) >> 3));
  const unsigned lo = e == 0u ? 0u : (b << 29);
  return __hiloint2double((int)hi, (int)lo);
}

// float64 -> float32 rounded to nearest (halfway cases away from zero) by
// bit manipulation (integer pipe): magnitudes below float32's normal range
// give a signed zero, above it infinity; NaN stays NaN.
__device__ __forceinline__ float d2f_int(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned s = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long r = mag + 0x10000000ull;  // half a float32 ulp
  const unsigned e = (unsigned)(r >> 52);
  const unsigned m = (unsigned)(r >> 29) & 0x7fffffu;
  unsigned f;
  if (e <= 896u)
    f = s;
  else if (e >= 1151u)
    f = s | 0x7f800000u | (mag > 0x7FF0000000000000ull ? 0x400000u : 0u);
  else
    f = s | ((e - 896u) << 23) | m;
  return __uint_as_float(f);
}

// exact maximin / kNN arithmetic (ordering.py:52-57): squared distance in
// IEEE sequential float64, no FMA contraction
__device__ __forceinline__ double sqdist_exact(const double* a, const double* b, int d) {
  double s = 0.0;
  for (int l = 0; l < d; ++l) {
    const double df = __dsub_rn(a[l], b[l]);
    s = __dadd_rn(s, __dmul_rn(df, df));
  }
  return s;
}

// maximin float32 skip threshold: an upper bound of
// dist * (1 + (d+4) 2^-53) + B_p as a float32, rounded up
__device__ __forceinline__ float thr_base(double dist, double Bp, int d) {
  if (isinf(dist)) return __int_as_float(0x7f800000);
  const double t = (dist * (1.0 + (double)(d + 4) * 0x1p-53) + Bp) * (1.0 + 0x1p-40);
  return __double2float_ru(t);
}

}  // namespace sv
