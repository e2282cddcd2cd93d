// Block table of the likelihood from the conditioning-set groups of
// ordering.py:119-127 (_nn_groups: rows with k neighbours each, and their
// neighbour rows), packed on the device so that the host only copies the
// groups' own arrays: rowb[o + r] = rows[r], kb[o + r] = k,
// nbr[o + r, c] = nb[r, c] for c < k and -1 beyond.  A row or neighbour index
// outside [0, n) raises the flag `bad` and is written as 0, so that no kernel
// ever reads outside the data; the caller reports the flag.
//
// The jitter-sharing chunks of the blocks (_covariance.py:255-259 sizes,
// likelihood.py:114 use): block r of group g lies in chunk base_g + r / step_g,
// the groups numbered in their own order.
//
// Group tables travel by value in the kernel parameters, up to kPackBatch
// groups per launch.
#include "sv_common.cuh"

namespace sv {

constexpr int kPackBatch = 32;

struct PackBatch {
  sv_pack_group g[kPackBatch];
  int ng;
};

struct ChunkBatch {
  sv_chunk_group g[kPackBatch];
  int ng;
};

// grid row y = group of the batch
__global__ void k_pack_groups(PackBatch PB, int64_t n, int32_t ldnbr, int32_t* rowb, int32_t* kb,
                              int32_t* nbr, int32_t* bad) {
  const sv_pack_group& G = PB.g[blockIdx.y];
  const int64_t tot = G.count * (int64_t)ldnbr;
  int flag = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / ldnbr;
    const int c = (int)(e - r * ldnbr);
    int32_t v = -1;
    if (c < G.k) {
      const int64_t x = G.nb[r * G.k + c];
      if (x < 0 || x >= n) {
        flag = 1;
        v = 0;
      } else {
        v = (int32_t)x;
      }
    }
    nbr[(G.out_off + r) * ldnbr + c] = v;
    if (c == 0) {
      const int64_t x = G.rows[r];
      if (x < 0 || x >= n) flag = 1;
      rowb[G.out_off + r] = (x < 0 || x >= n) ? 0 : (int32_t)x;
      kb[G.out_off + r] = G.k;
    }
  }
  if (flag) atomicOr(bad, 1);
}

__global__ void k_chunk_groups(ChunkBatch CB, int32_t* ids) {
  const sv_chunk_group& G = CB.g[blockIdx.y];
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < G.count;
       r += (int64_t)gridDim.x * blockDim.x)
    ids[G.out_off + r] = G.base + (int32_t)(r / G.step);
}

}  // namespace sv

using namespace sv;

extern "C" int sv_pack_blocks(const sv_pack_group* groups, int32_t ngroups, int64_t n, int32_t ldnbr,
                              int32_t* rowb, int32_t* kb, int32_t* nbr, int32_t* bad,
                              sv_stream_t stream) {
  if (ngroups < 0 || n < 0 || ldnbr < 1 || !bad || (ngroups > 0 && !groups)) return SV_EINVAL;
  // every group is checked before anything is launched, so a rejected call
  // leaves the block table untouched
  for (int g = 0; g < ngroups; ++g) {
    const sv_pack_group& G = groups[g];
    if (G.count < 0 || G.k < 0 || G.k > ldnbr || G.out_off < 0) return SV_EINVAL;
    if (G.count > 0 && (!G.rows || (G.k > 0 && !G.nb) || !rowb || !kb || !nbr)) return SV_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  SV_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int32_t), st));
  const int nsm = sv_num_sms();
  PackBatch PB;
  PB.ng = 0;
  int64_t maxtot = 0;
  auto flush = [&]() -> int {
    if (PB.ng == 0) return SV_OK;
    const int64_t bx = std::max<int64_t>(1, std::min<int64_t>((maxtot + 255) / 256, 4 * (int64_t)nsm));
    k_pack_groups<<<dim3((unsigned)bx, PB.ng), 256, 0, st>>>(PB, n, ldnbr, rowb, kb, nbr, bad);
    SV_CUDA_TRY(cudaGetLastError());
    PB.ng = 0;
    maxtot = 0;
    return SV_OK;
  };
  for (int g = 0; g < ngroups; ++g) {
    const sv_pack_group& G = groups[g];
    if (G.count == 0) continue;
    PB.g[PB.ng++] = G;
    maxtot = std::max<int64_t>(maxtot, G.count * (int64_t)ldnbr);
    if (PB.ng == kPackBatch) {
      const int rc = flush();
      if (rc != SV_OK) return rc;
    }
  }
  return flush();
}

extern "C" int sv_chunk_ids(const sv_chunk_group* groups, int32_t ngroups, int32_t* ids,
                            sv_stream_t stream) {
  if (ngroups < 0 || (ngroups > 0 && (!groups || !ids))) return SV_EINVAL;
  for (int g = 0; g < ngroups; ++g) {
    const sv_chunk_group& G = groups[g];
    if (G.count < 0 || G.out_off < 0 || G.step < 1 || G.base < 0) return SV_EINVAL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int nsm = sv_num_sms();
  ChunkBatch CB;
  CB.ng = 0;
  int64_t maxc = 0;
  auto flush = [&]() -> int {
    if (CB.ng == 0) return SV_OK;
    const int64_t bx = std::max<int64_t>(1, std::min<int64_t>((maxc + 255) / 256, 4 * (int64_t)nsm));
    k_chunk_groups<<<dim3((unsigned)bx, CB.ng), 256, 0, st>>>(CB, ids);
    SV_CUDA_TRY(cudaGetLastError());
    CB.ng = 0;
    maxc = 0;
    return SV_OK;
  };
  for (int g = 0; g < ngroups; ++g) {
    const sv_chunk_group& G = groups[g];
    if (G.count == 0) continue;
    CB.g[CB.ng++] = G;
    maxc = std::max<int64_t>(maxc, G.count);
    if (CB.ng == kPackBatch) {
      const int rc = flush();
      if (rc != SV_OK) return rc;
    }
  }
  return flush();
}
