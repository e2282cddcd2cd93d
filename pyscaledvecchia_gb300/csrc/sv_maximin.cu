// Exact maximin ordering on the GPU: ordering.py:27-73 (maximin_order /
// _maximin_core), bit for bit.
//
// Both forms run the pass algorithm of k_maximin_cluster (sv_reorder.cu):
// many pivots per barrier, each provably the reference's next choice.
//  * n up to one thread-block cluster's shared memory (16 CTAs): the cluster
//    form, one hardware cluster barrier per pass;
//  * larger n: the grid form, one CTA per SM of a cooperative launch, the
//    CTAs' candidate lists exchanged through global memory behind a grid
//    barrier with bounded waits (SV_ETIMEOUT when a wait gives up).
#include "sv_reorder.cuh"

using namespace sv;

extern "C" size_t sv_maximin_workspace_bytes(int64_t n, int32_t d) {
  (void)n;
  (void)d;
  return std::max<size_t>(256, maximin_grid_workspace_bytes());
}

static int maximin_route(const double* X, int64_t n, int32_t d, int64_t first, int64_t* order,
                         int32_t* info, void* workspace, size_t workspace_bytes, int32_t flags,
                         sv_stream_t stream) {
  if (n < 0 || d < 1 || d > 64 || (n > 0 && (!X || !order)) || !info) return SV_EINVAL;
  if (n > 0 && (first < 0 || first >= n)) return SV_EINVAL;
  if (n > 0x7fffffffLL || flags < 0 || flags > 15) return SV_EINVAL;
  if ((flags & 8) && !(flags & 4)) return SV_EINVAL;  // the barrier test aid is the grid form's
  cudaStream_t st = (cudaStream_t)stream;
  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  if (n == 0) return SV_OK;
  if (n == 1) {
    SV_CUDA_TRY(cudaMemcpyAsync(order, &first, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    return SV_OK;
  }
  if (!workspace || workspace_bytes < sv_maximin_workspace_bytes(n, d)) return SV_ENOSPC;
  if (!(flags & 4) && n <= maximin_cluster_max_rows(d))
    return maximin_cluster_single(X, n, d, first, order, info, (char*)workspace, flags, st);
  return maximin_grid_single(X, n, d, first, order, info, (char*)workspace, workspace_bytes, flags, st);
}

extern "C" int sv_maximin_order(const double* X, int64_t n, int32_t d, int64_t first,
                                int64_t* order, int32_t* info, void* workspace,
                                size_t workspace_bytes, sv_stream_t stream) {
  return maximin_route(X, n, d, first, order, info, workspace, workspace_bytes, 0, stream);
}

extern "C" int sv_maximin_order_flags(const double* X, int64_t n, int32_t d, int64_t first,
                                      int64_t* order, int32_t* info, void* workspace,
                                      size_t workspace_bytes, int32_t flags, sv_stream_t stream) {
  return maximin_route(X, n, d, first, order, info, workspace, workspace_bytes, flags, stream);
}

extern "C" int64_t sv_maximin_max_rows(int32_t d) { return maximin_grid_max_rows(d); }
