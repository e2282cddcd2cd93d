// Block table of the likelihood from the conditioning-set groups of
// ordering.py:119-127 (_nn_groups: rows with k neighbours each, and their
// neighbour rows), packed on the device so that the host only copies the
// groups' own arrays: rowb[o + r] = rows[r], kb[o + r] = k,
// nbr[o + r, c] = nb[r, c] for c < k and -1 beyond.  A row or neighbour index
// outside [0, n) raises the flag `bad` and is written as 0, so that no kernel
// ever reads outside the data; the caller reports the flag.
#include "sv_common.cuh"

namespace sv {

__global__ void k_pack_group(sv_pack_group G, int64_t n, int32_t ldnbr, int32_t* rowb, int32_t* kb,
                             int32_t* nbr, int32_t* bad) {
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

}  // namespace sv

using namespace sv;

extern "C" int sv_pack_blocks(const sv_pack_group* groups, int32_t ngroups, int64_t n, int32_t ldnbr,
                              int32_t* rowb, int32_t* kb, int32_t* nbr, int32_t* bad,
                              sv_stream_t stream) {
  if (ngroups < 0 || n < 0 || ldnbr < 1 || !bad || (ngroups > 0 && !groups)) return SV_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  SV_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int32_t), st));
  const int nsm = sv_num_sms();
  for (int g = 0; g < ngroups; ++g) {
    const sv_pack_group& G = groups[g];
    if (G.count < 0 || G.k < 0 || G.k > ldnbr || G.out_off < 0) return SV_EINVAL;
    if (G.count == 0) continue;
    if (!G.rows || (G.k > 0 && !G.nb) || !rowb || !kb || !nbr) return SV_EINVAL;
    const int64_t tot = G.count * (int64_t)ldnbr;
    const int64_t blocks = std::min<int64_t>((tot + 255) / 256, 4 * (int64_t)nsm);
    k_pack_group<<<(unsigned)blocks, 256, 0, st>>>(G, n, ldnbr, rowb, kb, nbr, bad);
    SV_CUDA_TRY(cudaGetLastError());
  }
  return SV_OK;
}
