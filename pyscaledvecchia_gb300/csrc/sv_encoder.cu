// Learned warm start: a DeepSets set encoder mapping a subsample of a
// problem's standardised (x, y) to initial log-parameters for Fisher
// scoring.  No counterpart in the reference; it only moves the starting
// point of gp.py:169-177 (the default start stays the fallback).
//
//   per point  (32 bfloat16 features, see sv_encoder_* in svgpu.h)
//     h1 = GELU(W1 x + b1)        128       (h1 rounded to bfloat16)
//     h2 = GELU(W2 h1 + b2)       128
//   pool = mean over the set's points of h2
//   head  g = GELU(W3 pool + b3)  128,   out = W4 g + b4   16 (14 used)
//
// Weights are bfloat16 copies of float32 master weights; every product
// accumulates in float32.  The per-point layers run on the tensor cores, one
// CTA per 128-point tile: the inference forward on tcgen05 (operands in
// shared memory, accumulators in tensor memory), the training forward and
// backward on mma.sync m16n8k16 (8 warps of 16 points, float32 fragments in
// registers, which the fused backward needs); the backward recomputes the tile's forward and produces
// per-tile weight-gradient partials that a separate kernel sums in a fixed
// order (no float atomics: results are bitwise reproducible).  The head is
// float32 SIMT, one CTA per set.
//
// Flat parameter layout (float32 master and bfloat16 copy alike):
//   W1[128][32] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] W4[16][128] b4[16]
#include <cuda_bf16.h>

#include "sv_common.cuh"

namespace sv {

constexpr int kEH = 128;   // hidden width
constexpr int kEF = 32;    // per-point features
constexpr int kEO = 16;    // head outputs
constexpr int kET = 128;   // points per tile (CTA)
constexpr int kELd = 136;  // bfloat16 row stride of 128-wide smem tiles
constexpr int kELx = 40;   // bfloat16 row stride of 32-wide smem tiles
constexpr int kEThreads = 256;

constexpr int64_t kOffW1 = 0;
constexpr int64_t kOffB1 = kOffW1 + kEH * kEF;
constexpr int64_t kOffW2 = kOffB1 + kEH;
constexpr int64_t kOffB2 = kOffW2 + kEH * kEH;
constexpr int64_t kOffW3 = kOffB2 + kEH;
constexpr int64_t kOffB3 = kOffW3 + kEH * kEH;
constexpr int64_t kOffW4 = kOffB3 + kEH;
constexpr int64_t kOffB4 = kOffW4 + kEO * kEH;
constexpr int64_t kEncParams = kOffB4 + kEO;
// per-tile backward partials: dW1, db1, dW2, db2
constexpr int64_t kEncTilePart = kEH * kEF + kEH + kEH * kEH + kEH;

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ float gelu_f(float z) {
  return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_d(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) +
         z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// D = A (16x16, row) * B (16x8, col) + D, bfloat16 inputs, float32 accumulate
__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }
// two bfloat16 from separate addresses: lo = p0[0], hi = p1[0]
__device__ __forceinline__ uint32_t ld2(const bf16* p0, const bf16* p1) {
  const uint32_t lo = *reinterpret_cast<const uint16_t*>(p0);
  const uint32_t hi = *reinterpret_cast<const uint16_t*>(p1);
  return lo | (hi << 16);
}
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const bf16 a = __float2bfloat16_rn(lo), b = __float2bfloat16_rn(hi);
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// Fragment helpers.  g = lane >> 2, t = lane & 3.  A row-major in smem
// (element (r, k) at A[r * lda + k]):
__device__ __forceinline__ void frag_a_row(uint32_t a[4], const bf16* A, int lda, int r0, int k0) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  a[0] = ld32(A + (r0 + g) * lda + k0 + 2 * t);
  a[1] = ld32(A + (r0 + g + 8) * lda + k0 + 2 * t);
  a[2] = ld32(A + (r0 + g) * lda + k0 + 8 + 2 * t);
  a[3] = ld32(A + (r0 + g + 8) * lda + k0 + 8 + 2 * t);
}
// A given transposed in smem (element (r, k) at At[k * lda + r])
__device__ __forceinline__ void frag_a_tr(uint32_t a[4], const bf16* At, int lda, int r0, int k0) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  const int r = r0 + g, k = k0 + 2 * t;
  a[0] = ld2(At + k * lda + r, At + (k + 1) * lda + r);
  a[1] = ld2(At + k * lda + r + 8, At + (k + 1) * lda + r + 8);
  a[2] = ld2(At + (k + 8) * lda + r, At + (k + 9) * lda + r);
  a[3] = ld2(At + (k + 8) * lda + r + 8, At + (k + 9) * lda + r + 8);
}
// B (k, n) = Bt[n * ldb + k] (B^T row-major, i.e. "col" operand)
__device__ __forceinline__ void frag_b_col(uint32_t b[2], const bf16* Bt, int ldb, int k0, int n0) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  b[0] = ld32(Bt + (n0 + g) * ldb + k0 + 2 * t);
  b[1] = ld32(Bt + (n0 + g) * ldb + k0 + 8 + 2 * t);
}
// B (k, n) = Bm[k * ldb + n] (row-major B)
__device__ __forceinline__ void frag_b_row(uint32_t b[2], const bf16* Bm, int ldb, int k0, int n0) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
  const int n = n0 + g, k = k0 + 2 * t;
  b[0] = ld2(Bm + k * ldb + n, Bm + (k + 1) * ldb + n);
  b[1] = ld2(Bm + (k + 8) * ldb + n, Bm + (k + 9) * ldb + n);
}

struct EncArgs {
  const bf16* x;       // [nset][S][16]
  const int32_t* cnt;  // [nset] points of each set (1..S)
  int S;               // set capacity, a multiple of 128
  int nset;
  const float* pf;     // float32 parameters (biases read here)
  const bf16* pb;      // bfloat16 parameters (weights read here)
  float* part;         // [nset][S/128][128] per-tile column sums of h2
  const float* dpool;  // [nset][128]
  float* gpart;        // [nset * S/128][kEncTilePart]
};

struct EncSmem {
  bf16 W1[kEH * kELx];
  bf16 W2[kEH * kELd];
  bf16 x[kET * kELx];
  bf16 h1[kET * kELd];
  bf16 dz2[kET * kELd];
  bf16 dz1[kET * kELd];
  float colsum[kEThreads / 32][kEH];
};

__device__ void enc_load_tile(const EncArgs& A, EncSmem& s, int set, int tile, bool need_w2) {
  for (int e = threadIdx.x; e < kEH * kEF / 2; e += blockDim.x) {
    const int r = e / (kEF / 2), c = 2 * (e % (kEF / 2));
    *reinterpret_cast<uint32_t*>(s.W1 + r * kELx + c) =
        *reinterpret_cast<const uint32_t*>(A.pb + kOffW1 + r * kEF + c);
  }
  if (need_w2)
    for (int e = threadIdx.x; e < kEH * kEH / 2; e += blockDim.x) {
      const int r = e / (kEH / 2), c = 2 * (e % (kEH / 2));
      *reinterpret_cast<uint32_t*>(s.W2 + r * kELd + c) =
          *reinterpret_cast<const uint32_t*>(A.pb + kOffW2 + r * kEH + c);
    }
  const bf16* xs = A.x + ((int64_t)set * A.S + (int64_t)tile * kET) * kEF;
  for (int e = threadIdx.x; e < kET * kEF / 2; e += blockDim.x) {
    const int r = e / (kEF / 2), c = 2 * (e % (kEF / 2));
    *reinterpret_cast<uint32_t*>(s.x + r * kELx + c) = *reinterpret_cast<const uint32_t*>(xs + r * kEF + c);
  }
}

// z1 for the warp's 16 points (rows r0..r0+15) into acc[16][4] (C layout, n = hidden)
__device__ __forceinline__ void enc_layer1(const EncSmem& s, const float* b1, int r0, float acc[16][4]) {
  const int t = threadIdx.x & 3;
#pragma unroll
  for (int nt = 0; nt < 16; ++nt) {
    const float bb0 = b1[nt * 8 + 2 * t], bb1 = b1[nt * 8 + 2 * t + 1];
    acc[nt][0] = bb0;
    acc[nt][1] = bb1;
    acc[nt][2] = bb0;
    acc[nt][3] = bb1;
  }
#pragma unroll
  for (int kt = 0; kt < kEF / 16; ++kt) {
    uint32_t a[4];
    frag_a_row(a, s.x, kELx, r0, kt * 16);
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
      uint32_t b[2];
      frag_b_col(b, s.W1, kELx, kt * 16, nt * 8);
      mma16816(acc[nt], a, b);
    }
  }
}

// z2 = W2 h1 + b2 for the warp's 16 points (h1 rows in smem)
__device__ __forceinline__ void enc_layer2(const EncSmem& s, const float* b2, int r0, float acc[16][4]) {
  const int t = threadIdx.x & 3;
#pragma unroll
  for (int nt = 0; nt < 16; ++nt) {
    const float bb0 = b2[nt * 8 + 2 * t], bb1 = b2[nt * 8 + 2 * t + 1];
    acc[nt][0] = bb0;
    acc[nt][1] = bb1;
    acc[nt][2] = bb0;
    acc[nt][3] = bb1;
  }
#pragma unroll
  for (int kt = 0; kt < 8; ++kt) {
    uint32_t a[4];
    frag_a_row(a, s.h1, kELd, r0, kt * 16);
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
      uint32_t b[2];
      frag_b_col(b, s.W2, kELd, kt * 16, nt * 8);
      mma16816(acc[nt], a, b);
    }
  }
}

// h1 = bf16(GELU(z1)) into smem rows of the warp
__device__ __forceinline__ void enc_store_h1(EncSmem& s, int r0, const float acc[16][4]) {
  const int g = (threadIdx.x & 31) >> 2, t = threadIdx.x & 3;
#pragma unroll
  for (int nt = 0; nt < 16; ++nt) {
    const int c = nt * 8 + 2 * t;
    *reinterpret_cast<uint32_t*>(s.h1 + (r0 + g) * kELd + c) = pack2(gelu_f(acc[nt][0]), gelu_f(acc[nt][1]));
    *reinterpret_cast<uint32_t*>(s.h1 + (r0 + g + 8) * kELd + c) =
        pack2(gelu_f(acc[nt][2]), gelu_f(acc[nt][3]));
  }
}

// column sums over the warp's valid rows of v (C layout) into s.colsum[warp]
__device__ __forceinline__ void enc_colsum(EncSmem& s, const float v[16][4], bool ok0, bool ok1) {
  const int lane = threadIdx.x & 31, t = lane & 3, warp = threadIdx.x >> 5;
#pragma unroll
  for (int nt = 0; nt < 16; ++nt) {
    float s0 = (ok0 ? v[nt][0] : 0.0f) + (ok1 ? v[nt][2] : 0.0f);
    float s1 = (ok0 ? v[nt][1] : 0.0f) + (ok1 ? v[nt][3] : 0.0f);
    // reduce over the 8 row groups (lanes with equal t)
    for (int o = 4; o < 32; o <<= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, o);
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if (lane < 4) {
      s.colsum[warp][nt * 8 + 2 * t] = s0;
      s.colsum[warp][nt * 8 + 2 * t + 1] = s1;
    }
  }
}

__global__ void __launch_bounds__(kEThreads, 1) k_enc_points_fwd(EncArgs A) {
  extern __shared__ __align__(16) unsigned char enc_smraw[];
  EncSmem& s = *reinterpret_cast<EncSmem*>(enc_smraw);
  const int tile = blockIdx.x, set = blockIdx.y;
  const int ntile = A.S / kET;
  const int warp = threadIdx.x >> 5, g = (threadIdx.x & 31) >> 2;
  const int cnt = A.cnt[set];
  enc_load_tile(A, s, set, tile, true);
  __syncthreads();
  const int r0 = warp * 16;
  float acc[16][4];
  enc_layer1(s, A.pf + kOffB1, r0, acc);
  enc_store_h1(s, r0, acc);
  __syncwarp();
  enc_layer2(s, A.pf + kOffB2, r0, acc);
#pragma unroll
  for (int nt = 0; nt < 16; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[nt][e] = gelu_f(acc[nt][e]);
  const int p0 = tile * kET + r0 + g;
  enc_colsum(s, acc, p0 < cnt, p0 + 8 < cnt);
  __syncthreads();
  if (threadIdx.x < kEH) {
    float v = 0.0f;
    for (int w = 0; w < kEThreads / 32; ++w) v += s.colsum[w][threadIdx.x];
    A.part[((int64_t)set * ntile + tile) * kEH + threadIdx.x] = v;
  }
}

__global__ void __launch_bounds__(kEThreads, 1) k_enc_points_bwd(EncArgs A) {
  extern __shared__ __align__(16) unsigned char enc_smraw[];
  EncSmem& s = *reinterpret_cast<EncSmem*>(enc_smraw);
  const int tile = blockIdx.x, set = blockIdx.y;
  const int ntile = A.S / kET;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int cnt = A.cnt[set];
  float* gp = A.gpart + ((int64_t)set * ntile + tile) * kEncTilePart;
  enc_load_tile(A, s, set, tile, true);
  __syncthreads();
  const int r0 = warp * 16;
  const int p0 = tile * kET + r0 + g;
  const bool ok0 = p0 < cnt, ok1 = p0 + 8 < cnt;
  float acc[16][4];
  enc_layer1(s, A.pf + kOffB1, r0, acc);
  enc_store_h1(s, r0, acc);
  __syncwarp();
  enc_layer2(s, A.pf + kOffB2, r0, acc);
  // dz2 = dpool / cnt * GELU'(z2) on valid points
  const float inv = 1.0f / (float)cnt;
  const float* dp = A.dpool + (int64_t)set * kEH;
#pragma unroll
  for (int nt = 0; nt < 16; ++nt) {
    const int c = nt * 8 + 2 * t;
    const float d0 = dp[c] * inv, d1 = dp[c + 1] * inv;
    acc[nt][0] = ok0 ? d0 * gelu_d(acc[nt][0]) : 0.0f;
    acc[nt][1] = ok0 ? d1 * gelu_d(acc[nt][1]) : 0.0f;
    acc[nt][2] = ok1 ? d0 * gelu_d(acc[nt][2]) : 0.0f;
    acc[nt][3] = ok1 ? d1 * gelu_d(acc[nt][3]) : 0.0f;
    *reinterpret_cast<uint32_t*>(s.dz2 + (r0 + g) * kELd + c) = pack2(acc[nt][0], acc[nt][1]);
    *reinterpret_cast<uint32_t*>(s.dz2 + (r0 + g + 8) * kELd + c) = pack2(acc[nt][2], acc[nt][3]);
  }
  // db2 partial (float32 dz2)
  enc_colsum(s, acc, true, true);
  __syncthreads();
  if (threadIdx.x < kEH) {
    float v = 0.0f;
    for (int w = 0; w < kEThreads / 32; ++w) v += s.colsum[w][threadIdx.x];
    gp[kEH * kEF + kEH + kEH * kEH + threadIdx.x] = v;
  }
  // dW2[o][i] = sum_p dz2[p][o] h1[p][i]: the warp's 16 rows of o
  {
    float w2[16][4];
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) w2[nt][0] = w2[nt][1] = w2[nt][2] = w2[nt][3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < 8; ++kt) {
      uint32_t a[4];
      frag_a_tr(a, s.dz2, kELd, r0, kt * 16);
#pragma unroll
      for (int nt = 0; nt < 16; ++nt) {
        uint32_t b[2];
        frag_b_row(b, s.h1, kELd, kt * 16, nt * 8);
        mma16816(w2[nt], a, b);
      }
    }
    float* dW2 = gp + kEH * kEF + kEH;
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
      const int c = nt * 8 + 2 * t;
      dW2[(r0 + g) * kEH + c] = w2[nt][0];
      dW2[(r0 + g) * kEH + c + 1] = w2[nt][1];
      dW2[(r0 + g + 8) * kEH + c] = w2[nt][2];
      dW2[(r0 + g + 8) * kEH + c + 1] = w2[nt][3];
    }
  }
  // dh1[p][i] = sum_o dz2[p][o] W2[o][i] for the warp's points
#pragma unroll
  for (int nt = 0; nt < 16; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
#pragma unroll
  for (int kt = 0; kt < 8; ++kt) {
    uint32_t a[4];
    frag_a_row(a, s.dz2, kELd, r0, kt * 16);
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
      uint32_t b[2];
      frag_b_row(b, s.W2, kELd, kt * 16, nt * 8);
      mma16816(acc[nt], a, b);
    }
  }
  // dz1 = dh1 * GELU'(z1), z1 recomputed in the same fragment layout
  {
    float z1[16][4];
    enc_layer1(s, A.pf + kOffB1, r0, z1);
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
      const int c = nt * 8 + 2 * t;
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[nt][e] *= gelu_d(z1[nt][e]);
      *reinterpret_cast<uint32_t*>(s.dz1 + (r0 + g) * kELd + c) = pack2(acc[nt][0], acc[nt][1]);
      *reinterpret_cast<uint32_t*>(s.dz1 + (r0 + g + 8) * kELd + c) = pack2(acc[nt][2], acc[nt][3]);
    }
  }
  __syncthreads();  // colsum reuse and dz1 rows of every warp
  enc_colsum(s, acc, true, true);
  __syncthreads();
  if (threadIdx.x < kEH) {
    float v = 0.0f;
    for (int w = 0; w < kEThreads / 32; ++w) v += s.colsum[w][threadIdx.x];
    gp[kEH * kEF + threadIdx.x] = v;  // db1
  }
  // dW1[o][i] = sum_p dz1[p][o] x[p][i]: the warp's 16 rows of o, 16 inputs
  {
    constexpr int NT1 = kEF / 8;
    float w1[NT1][4];
#pragma unroll
    for (int nt = 0; nt < NT1; ++nt) w1[nt][0] = w1[nt][1] = w1[nt][2] = w1[nt][3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < 8; ++kt) {
      uint32_t a[4];
      frag_a_tr(a, s.dz1, kELd, r0, kt * 16);
#pragma unroll
      for (int nt = 0; nt < NT1; ++nt) {
        uint32_t b[2];
        frag_b_row(b, s.x, kELx, kt * 16, nt * 8);
        mma16816(w1[nt], a, b);
      }
    }
#pragma unroll
    for (int nt = 0; nt < NT1; ++nt) {
      const int c = nt * 8 + 2 * t;
      gp[(r0 + g) * kEF + c] = w1[nt][0];
      gp[(r0 + g) * kEF + c + 1] = w1[nt][1];
      gp[(r0 + g + 8) * kEF + c] = w1[nt][2];
      gp[(r0 + g + 8) * kEF + c + 1] = w1[nt][3];
    }
  }
}

// ---------------------------------------------------------------------------
// Forward per-point layers on the 5th-generation tensor cores (tcgen05):
// one CTA of 4 warps per 128-point tile; operands in shared memory in the
// canonical no-swizzle K-major layout (8-row x 16-byte core matrices, core
// matrices along K 128 bytes apart, 8-row groups KG * 128 bytes apart),
// accumulators in tensor memory (128 lanes = points, 256 columns = two
// 128-wide float32 results), one thread issuing the MMAs, completion
// signalled through an mbarrier, epilogues read back with tcgen05.ld.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t umma_off(int r, int k, int KG) {
  return (uint32_t)((r >> 3) * (KG * 128) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets in 16-byte units, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor of kind::f16: D float32, A and B bfloat16, both
// K-major, M x N
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(mbar) : "memory");
}

// bounded wait for the mbarrier phase; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  for (uint32_t it = 0; it < (1u << 22); ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(mbar), "r"(phase) : "memory");
    if (done) return true;
  }
  return false;
}

#define SV_TC_LD32(taddr, v)                                                                      \
  asm volatile(                                                                                    \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14," \
      "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"              \
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),      \
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),  \
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),            \
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),            \
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])             \
      : "r"(taddr))

struct EncTcSmem {
  alignas(128) unsigned char x[kET * kEF * 2];   // canonical, KG = kEF / 8
  alignas(128) unsigned char w1[kEH * kEF * 2];  // canonical, KG = kEF / 8
  alignas(128) unsigned char w2[kEH * kEH * 2];  // canonical, KG = 16
  alignas(128) unsigned char h1[kET * kEH * 2];  // canonical, KG = 16
  float colsum[4][kEH];
  float tr[4][32][33];  // per-warp 32 x 32 transpose buffer of the pooling epilogue
  uint64_t mbar;
  uint32_t tmem_base;
};

// 16-byte chunk c of a row-major [rows][K] bfloat16 matrix into the canonical layout
__device__ __forceinline__ void umma_stage(unsigned char* dst, const bf16* src, int rows, int K) {
  const int KG = K / 8;
  for (int c = threadIdx.x; c < rows * KG; c += blockDim.x) {
    const int r = c / KG, kg = c - (c / KG) * KG;
    *reinterpret_cast<uint4*>(dst + umma_off(r, kg * 8, KG)) =
        *reinterpret_cast<const uint4*>(src + (int64_t)r * K + kg * 8);
  }
}

// Persistent: each CTA stages the weights once, then walks tiles t =
// blockIdx.x, blockIdx.x + gridDim.x, ... (set t / ntile, tile t % ntile).
// Two MMA groups per tile complete mbarrier phases of parity 0 and 1.
__global__ void __launch_bounds__(128, 1) k_enc_points_fwd_tc(EncArgs A, int32_t* err) {
  extern __shared__ __align__(16) unsigned char tc_smraw[];
  // 128-byte aligned base inside the launch's slack
  const uint32_t pad = (128u - (smem_u32(tc_smraw) & 127u)) & 127u;
  EncTcSmem& s = *reinterpret_cast<EncTcSmem*>(tc_smraw + pad);
  const int ntile = A.S / kET;
  const int64_t total = (int64_t)A.nset * ntile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t mbar = smem_u32(&s.mbar);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(&s.tmem_base)), "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(mbar), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma_stage(s.w1, A.pb + kOffW1, kEH, kEF);
  umma_stage(s.w2, A.pb + kOffW2, kEH, kEH);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tbase = s.tmem_base;
  const uint32_t idesc = umma_idesc_bf16(kET, kEH);
  const int row = warp * 32 + lane;  // this thread's point in the tile
  const uint32_t tlane = tbase + ((uint32_t)(warp * 32) << 16);
  bool ok = true;

  for (int64_t t = blockIdx.x; t < total && ok; t += gridDim.x) {
    const int set = (int)(t / ntile), tile = (int)(t - (t / ntile) * ntile);
    const int cnt = A.cnt[set];
    umma_stage(s.x, A.x + ((int64_t)set * A.S + (int64_t)tile * kET) * kEF, kET, kEF);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // layer 1: D1 = X W1^T (K = kEF, instructions of K = 16)
    if (threadIdx.x == 0) {
      for (int kk = 0; kk < kEF / 16; ++kk)
        umma_bf16(tbase, umma_desc(smem_u32(s.x) + kk * 256, 128, (kEF / 8) * 128),
                  umma_desc(smem_u32(s.w1) + kk * 256, 128, (kEF / 8) * 128), idesc, kk > 0 ? 1u : 0u);
      umma_commit(mbar);
    }
    ok = __all_sync(0xffffffffu, mbar_wait(mbar, 0));  // warp-uniform before tcgen05.ld
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
      // epilogue 1: h1 = bf16(GELU(z1 + b1)) into the canonical A operand of layer 2
      for (int c0 = 0; c0 < kEH; c0 += 32) {
        uint32_t v[32];
        SV_TC_LD32(tlane + c0, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int c = 0; c < 32; c += 8) {
          uint32_t w[4];
#pragma unroll
          for (int e = 0; e < 4; ++e)
            w[e] = pack2(gelu_f(__uint_as_float(v[c + 2 * e]) + A.pf[kOffB1 + c0 + c + 2 * e]),
                         gelu_f(__uint_as_float(v[c + 2 * e + 1]) + A.pf[kOffB1 + c0 + c + 2 * e + 1]));
          *reinterpret_cast<uint4*>(s.h1 + umma_off(row, c0 + c, kEH / 8)) =
              make_uint4(w[0], w[1], w[2], w[3]);
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // layer 2: D2 = H1 W2^T (K = 128, eight instructions of K = 16)
    if (ok && threadIdx.x == 0) {
      for (int kk = 0; kk < kEH / 16; ++kk)
        umma_bf16(tbase + kEH, umma_desc(smem_u32(s.h1) + kk * 256, 128, 2048),
                  umma_desc(smem_u32(s.w2) + kk * 256, 128, 2048), idesc, kk > 0 ? 1u : 0u);
      umma_commit(mbar);
    }
    if (ok) ok = __all_sync(0xffffffffu, mbar_wait(mbar, 1));
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool valid = tile * kET + row < cnt;
    for (int c0 = 0; c0 < kEH; c0 += 32) {
      uint32_t v[32];
      if (ok) {
        SV_TC_LD32(tlane + kEH + c0, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      }
      // column sums over the warp's 32 rows: transpose through shared memory,
      // then lane c adds up column c0 + c
#pragma unroll
      for (int c = 0; c < 32; ++c)
        s.tr[warp][c][lane] = (ok && valid) ? gelu_f(__uint_as_float(v[c]) + A.pf[kOffB2 + c0 + c]) : 0.0f;
      __syncwarp();
      float h = 0.0f;
#pragma unroll
      for (int r = 0; r < 32; ++r) h += s.tr[warp][lane][r];
      s.colsum[warp][c0 + lane] = h;
      __syncwarp();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    ok = __syncthreads_and(ok);
    if (threadIdx.x < kEH) {
      const float v = ((s.colsum[0][threadIdx.x] + s.colsum[1][threadIdx.x]) + s.colsum[2][threadIdx.x]) +
                      s.colsum[3][threadIdx.x];
      A.part[((int64_t)set * ntile + tile) * kEH + threadIdx.x] = v;
    }
    __syncthreads();  // colsum and x are rewritten by the next tile
  }
  if (!ok && threadIdx.x == 0) atomicExch(err, SV_ETIMEOUT);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(256));
  }
}

// head, one CTA (128 threads) per set: pool, g, out; with targets also the
// loss terms and the vectors the weight gradients need
struct HeadArgs {
  const int32_t* err;  // nonzero: the per-point forward failed (outputs NaN)
  const float* part;
  const int32_t* cnt;
  int ntile, nset;
  const float* pf;
  const bf16* pb;
  float* out;           // [nset][16]
  const float* target;  // [nset][16] or null
  const float* wts;     // [nset][16] loss weights (0 masks an output)
  float* pool;          // [nset][128]
  float* gv;            // [nset][128]  g
  float* dzg;           // [nset][128]
  float* dout;          // [nset][16]
  float* dpool;         // [nset][128]
  float* loss_set;      // [nset]
};

__global__ void __launch_bounds__(kEH) k_enc_head(HeadArgs H) {
  const int b = blockIdx.x, j = threadIdx.x;
  __shared__ float pool[kEH], gs[kEH], zs[kEH], dz[kEH], dout[kEO], lred[kEO];
  const float inv = 1.0f / (float)H.cnt[b];
  float pv = 0.0f;
  for (int t = 0; t < H.ntile; ++t) pv += H.part[((int64_t)b * H.ntile + t) * kEH + j];
  pv *= inv;
  pool[j] = pv;
  __syncthreads();
  float z = H.pf[kOffB3 + j];
  for (int i = 0; i < kEH; ++i) z += __bfloat162float(H.pb[kOffW3 + j * kEH + i]) * pool[i];
  zs[j] = z;
  gs[j] = gelu_f(z);
  __syncthreads();
  if (j < kEO) {
    float o = H.pf[kOffB4 + j];
    for (int i = 0; i < kEH; ++i) o += __bfloat162float(H.pb[kOffW4 + j * kEH + i]) * gs[i];
    H.out[(int64_t)b * kEO + j] = (H.err && *H.err) ? __int_as_float(0x7fc00000) : o;
    if (H.target) {
      const float w = H.wts[(int64_t)b * kEO + j];
      const float r = o - H.target[(int64_t)b * kEO + j];
      dout[j] = 2.0f * w * r;
      lred[j] = w * r * r;
    }
  }
  if (!H.target) return;
  __syncthreads();
  if (j == 0) {
    float l = 0.0f;
    for (int o = 0; o < kEO; ++o) l += lred[o];
    H.loss_set[b] = l;
  }
  float dg = 0.0f;
  for (int o = 0; o < kEO; ++o) dg += __bfloat162float(H.pb[kOffW4 + o * kEH + j]) * dout[o];
  const float dzj = dg * gelu_d(zs[j]);
  dz[j] = dzj;
  __syncthreads();
  float dpv = 0.0f;
  for (int i = 0; i < kEH; ++i) dpv += __bfloat162float(H.pb[kOffW3 + i * kEH + j]) * dz[i];
  H.dpool[(int64_t)b * kEH + j] = dpv;
  H.pool[(int64_t)b * kEH + j] = pool[j];
  H.gv[(int64_t)b * kEH + j] = gs[j];
  H.dzg[(int64_t)b * kEH + j] = dzj;
  if (j < kEO) H.dout[(int64_t)b * kEO + j] = dout[j];
}

// head weight gradients, summed over sets in a fixed order:
//   dW3[j][i] = sum_b dzg[b][j] pool[b][i], db3 = sum_b dzg,
//   dW4[o][j] = sum_b dout[b][o] g[b][j],   db4 = sum_b dout
__global__ void k_enc_head_wgrad(HeadArgs H, float* grad) {
  const int64_t nout = kEH * kEH + kEH + kEO * kEH + kEO;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nout;
       e += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    if (e < kEH * kEH) {
      const int jj = (int)(e / kEH), ii = (int)(e % kEH);
      for (int b = 0; b < H.nset; ++b) s += H.dzg[(int64_t)b * kEH + jj] * H.pool[(int64_t)b * kEH + ii];
      grad[kOffW3 + e] = s;
    } else if (e < kEH * kEH + kEH) {
      const int jj = (int)(e - kEH * kEH);
      for (int b = 0; b < H.nset; ++b) s += H.dzg[(int64_t)b * kEH + jj];
      grad[kOffB3 + jj] = s;
    } else if (e < kEH * kEH + kEH + kEO * kEH) {
      const int64_t f = e - kEH * kEH - kEH;
      const int o = (int)(f / kEH), jj = (int)(f % kEH);
      for (int b = 0; b < H.nset; ++b) s += H.dout[(int64_t)b * kEO + o] * H.gv[(int64_t)b * kEH + jj];
      grad[kOffW4 + f] = s;
    } else {
      const int o = (int)(e - kEH * kEH - kEH - kEO * kEH);
      for (int b = 0; b < H.nset; ++b) s += H.dout[(int64_t)b * kEO + o];
      grad[kOffB4 + o] = s;
    }
  }
}

// per-point layer gradients: sums of the per-tile partials, fixed order
__global__ void k_enc_reduce(const float* gpart, int64_t ntiles, float* grad) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < kEncTilePart;
       e += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int64_t t = 0; t < ntiles; ++t) s += gpart[t * kEncTilePart + e];
    // partial layout dW1 | db1 | dW2 | db2 is the parameter layout's prefix
    grad[e] = s;
  }
}

__global__ void k_enc_loss(const float* loss_set, int nset, float* loss) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    float l = 0.0f;
    for (int b = 0; b < nset; ++b) l += loss_set[b];
    loss[0] = l;
  }
}

// Adam on the float32 master weights; refreshes the bfloat16 copy
__global__ void k_enc_adam(float* p, const float* grad, float* m, float* v, bf16* pb, int64_t n,
                           float lr, float b1, float b2, float eps, float c1, float c2, float wd) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gr = grad[i] + wd * p[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gr;
    const float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    pb[i] = __float2bfloat16_rn(pi);
  }
}

__global__ void k_enc_to_bf16(const float* p, bf16* pb, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    pb[i] = __float2bfloat16_rn(p[i]);
}

// features: float64 -> float32 -> bfloat16 (round to nearest even each time)
__global__ void k_enc_pack(const double* f, bf16* x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = __float2bfloat16_rn(__double2float_rn(f[i]));
}

static size_t enc_align(size_t x) { return (x + 255) & ~(size_t)255; }

struct EncWs {
  size_t err, part, pool, gv, dzg, dout, dpool, loss_set, gpart, total;
};

static EncWs enc_ws(int64_t nset, int S, int train) {
  EncWs W;
  const int64_t ntile = S / kET;
  size_t off = 0;
  W.err = off;
  off = enc_align(off + sizeof(int32_t));
  W.part = off;
  off = enc_align(off + sizeof(float) * nset * ntile * kEH);
  W.pool = off;
  off = enc_align(off + sizeof(float) * nset * kEH);
  W.gv = off;
  off = enc_align(off + sizeof(float) * nset * kEH);
  W.dzg = off;
  off = enc_align(off + sizeof(float) * nset * kEH);
  W.dout = off;
  off = enc_align(off + sizeof(float) * nset * kEO);
  W.dpool = off;
  off = enc_align(off + sizeof(float) * nset * kEH);
  W.loss_set = off;
  off = enc_align(off + sizeof(float) * nset);
  W.gpart = off;
  if (train) off = enc_align(off + sizeof(float) * nset * ntile * kEncTilePart);
  W.total = off;
  return W;
}

}  // namespace sv

using namespace sv;

extern "C" int64_t sv_encoder_param_count(void) { return kEncParams; }

extern "C" size_t sv_encoder_workspace_bytes(int64_t nset, int32_t S, int32_t train) {
  if (nset < 1 || S < kET || S % kET) return 0;
  return enc_ws(nset, S, train).total;
}

extern "C" int sv_encoder_pack(const double* feats, int64_t n, uint16_t* x, sv_stream_t stream) {
  if (n < 0 || (n > 0 && (!feats || !x))) return SV_EINVAL;
  if (n == 0) return SV_OK;
  int64_t g = (n + 255) / 256;
  if (g > 4096) g = 4096;
  k_enc_pack<<<(unsigned)g, 256, 0, (cudaStream_t)stream>>>(feats, (bf16*)x, n);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

static int enc_common(int64_t nset, int32_t S, const uint16_t* x, const int32_t* cnt,
                      const float* pf, const uint16_t* pb, float* out, void* ws, size_t wsb,
                      int train, EncArgs& A, HeadArgs& H, EncWs& W) {
  if (nset < 1 || nset > 65535 || S < kET || S % kET || S / kET > 65535 || !x || !cnt || !pf ||
      !pb || !out || !ws)
    return SV_EINVAL;
  W = enc_ws(nset, S, train);
  if (wsb < W.total) return SV_ENOSPC;
  char* w = (char*)ws;
  A.x = (const bf16*)x;
  A.cnt = cnt;
  A.S = S;
  A.nset = (int)nset;
  A.pf = pf;
  A.pb = (const bf16*)pb;
  A.part = (float*)(w + W.part);
  A.dpool = (const float*)(w + W.dpool);
  A.gpart = (float*)(w + W.gpart);
  H.err = (const int32_t*)(w + W.err);
  H.part = A.part;
  H.cnt = cnt;
  H.ntile = S / kET;
  H.nset = (int)nset;
  H.pf = pf;
  H.pb = (const bf16*)pb;
  H.out = out;
  H.target = nullptr;
  H.wts = nullptr;
  H.pool = (float*)(w + W.pool);
  H.gv = (float*)(w + W.gv);
  H.dzg = (float*)(w + W.dzg);
  H.dout = (float*)(w + W.dout);
  H.dpool = (float*)(w + W.dpool);
  H.loss_set = (float*)(w + W.loss_set);
  return SV_OK;
}

extern "C" int sv_encoder_forward(int64_t nset, int32_t S, const uint16_t* x, const int32_t* cnt,
                                  const float* params, const uint16_t* params_bf16, float* out,
                                  int32_t variant, void* workspace, size_t workspace_bytes,
                                  sv_stream_t stream) {
  EncArgs A;
  HeadArgs H;
  EncWs W;
  if (variant != 0 && variant != 1) return SV_EINVAL;
  int rc = enc_common(nset, S, x, cnt, params, params_bf16, out, workspace, workspace_bytes, 0, A,
                      H, W);
  if (rc != SV_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 grid((unsigned)(S / kET), (unsigned)nset);
  int32_t* err = (int32_t*)((char*)workspace + W.err);
  SV_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int32_t), st));
  if (variant == 0) {
    const size_t smem = sizeof(EncTcSmem) + 128;  // + alignment slack of the dynamic base
    SV_CUDA_TRY(cudaFuncSetAttribute(k_enc_points_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // persistent: two CTAs per SM (256 tensor-memory columns each)
    int64_t ctas = (int64_t)nset * (S / kET);
    if (ctas > 2LL * sv_num_sms()) ctas = 2LL * sv_num_sms();
    k_enc_points_fwd_tc<<<(unsigned)ctas, 128, smem, st>>>(A, err);
  } else {
    const size_t smem = sizeof(EncSmem);
    SV_CUDA_TRY(cudaFuncSetAttribute(k_enc_points_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_enc_points_fwd<<<grid, kEThreads, smem, st>>>(A);
  }
  SV_CUDA_TRY(cudaGetLastError());
  k_enc_head<<<(unsigned)nset, kEH, 0, st>>>(H);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" int sv_encoder_backward(int64_t nset, int32_t S, const uint16_t* x, const int32_t* cnt,
                                   const float* params, const uint16_t* params_bf16,
                                   const float* target, const float* weights, float* out,
                                   float* loss, float* grad, void* workspace,
                                   size_t workspace_bytes, sv_stream_t stream) {
  EncArgs A;
  HeadArgs H;
  EncWs W;
  if (!target || !weights || !loss || !grad) return SV_EINVAL;
  int rc = enc_common(nset, S, x, cnt, params, params_bf16, out, workspace, workspace_bytes, 1, A,
                      H, W);
  if (rc != SV_OK) return rc;
  H.target = target;
  H.wts = weights;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t smem = sizeof(EncSmem);
  SV_CUDA_TRY(cudaFuncSetAttribute(k_enc_points_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SV_CUDA_TRY(cudaFuncSetAttribute(k_enc_points_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const dim3 grid((unsigned)(S / kET), (unsigned)nset);
  SV_CUDA_TRY(cudaMemsetAsync((char*)workspace + W.err, 0, sizeof(int32_t), st));
  k_enc_points_fwd<<<grid, kEThreads, smem, st>>>(A);
  SV_CUDA_TRY(cudaGetLastError());
  k_enc_head<<<(unsigned)nset, kEH, 0, st>>>(H);
  SV_CUDA_TRY(cudaGetLastError());
  k_enc_loss<<<1, 32, 0, st>>>(H.loss_set, (int)nset, loss);
  SV_CUDA_TRY(cudaGetLastError());
  k_enc_head_wgrad<<<64, 256, 0, st>>>(H, grad);
  SV_CUDA_TRY(cudaGetLastError());
  k_enc_points_bwd<<<grid, kEThreads, smem, st>>>(A);
  SV_CUDA_TRY(cudaGetLastError());
  k_enc_reduce<<<64, 256, 0, st>>>(A.gpart, nset * (int64_t)(S / kET), grad);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" int sv_encoder_adam(float* params, const float* grad, float* m, float* v,
                               uint16_t* params_bf16, int64_t n, float lr, float beta1,
                               float beta2, float eps, int32_t step, float weight_decay,
                               sv_stream_t stream) {
  if (!params || !grad || !m || !v || !params_bf16 || n < 0 || step < 1) return SV_EINVAL;
  if (n == 0) return SV_OK;
  const float c1 = 1.0f - powf(beta1, (float)step);
  const float c2 = 1.0f - powf(beta2, (float)step);
  int64_t g = (n + 255) / 256;
  if (g > 1024) g = 1024;
  k_enc_adam<<<(unsigned)g, 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, (bf16*)params_bf16, n,
                                                             lr, beta1, beta2, eps, c1, c2, weight_decay);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}

extern "C" int sv_encoder_to_bf16(const float* params, uint16_t* params_bf16, int64_t n,
                                  sv_stream_t stream) {
  if (n < 0 || (n > 0 && (!params || !params_bf16))) return SV_EINVAL;
  if (n == 0) return SV_OK;
  int64_t g = (n + 255) / 256;
  if (g > 1024) g = 1024;
  k_enc_to_bf16<<<(unsigned)g, 256, 0, (cudaStream_t)stream>>>(params, (bf16*)params_bf16, n);
  SV_CUDA_TRY(cudaGetLastError());
  return SV_OK;
}
