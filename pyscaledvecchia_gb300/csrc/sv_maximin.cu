// Exact maximin ordering on the GPU: ordering.py:27-73 (maximin_order /
// _maximin_core), bit for bit.
//
// Every form runs the pass algorithm of k_maximin_cluster (sv_reorder.cu):
// many pivots per barrier, each provably the reference's next choice.
//  * n up to one thread-block cluster's shared memory (16 CTAs): the cluster
//    form, one hardware cluster barrier per pass;
//  * up to the shared memory of every SM: the grid form, one CTA per SM of a
//    cooperative launch, the CTAs' candidate lists exchanged through global
//    memory behind a grid barrier with bounded waits (SV_ETIMEOUT when a wait
//    gives up);
//  * beyond: the tree form (sv_maximin_tree.cu), one CTA over a 32-ary tree
//    of the rows in global memory, visiting only what a pass can change.
#include "sv_reorder.cuh"

using namespace sv;

// the route of n rows of dimension d under flags: 0 cluster, 1 grid, 2 tree
static int maximin_form(int64_t n, int32_t d, int32_t flags) {
  if (flags & 16) return 2;
  if (flags & 4) return 1;
  if (n <= maximin_cluster_max_rows(d)) return 0;
  return n <= maximin_grid_max_rows(d) ? 1 : 2;
}

extern "C" size_t sv_maximin_workspace_bytes_flags(int64_t n, int32_t d, int32_t flags) {
  size_t b = std::max<size_t>(256, maximin_grid_workspace_bytes());
  if (d >= 1 && d <= 64 && n >= 2 && maximin_form(n, d, flags) == 2)
    b = std::max(b, maximin_tree_workspace_bytes(n, d));
  return b;
}

extern "C" size_t sv_maximin_workspace_bytes(int64_t n, int32_t d) {
  return sv_maximin_workspace_bytes_flags(n, d, 0);
}

static int maximin_route(const double* X, int64_t n, int32_t d, int64_t first, int64_t* order,
                         int32_t* info, void* workspace, size_t workspace_bytes, int32_t flags,
                         sv_stream_t stream) {
  if (n < 0 || d < 1 || d > 64 || (n > 0 && (!X || !order)) || !info) return SV_EINVAL;
  if (n > 0 && (first < 0 || first >= n)) return SV_EINVAL;
  if (n > 0x7fffffffLL || flags < 0 || flags > 31) return SV_EINVAL;
  if ((flags & 8) && !(flags & 4)) return SV_EINVAL;  // the barrier test aid is the grid form's
  if ((flags & 16) && (flags & 4)) return SV_EINVAL;  // one forced form
  cudaStream_t st = (cudaStream_t)stream;
  int32_t init_info[4] = {0, -1, 0, 0};
  SV_CUDA_TRY(cudaMemcpyAsync(info, init_info, sizeof(init_info), cudaMemcpyHostToDevice, st));
  if (n == 0) return SV_OK;
  if (n == 1) {
    SV_CUDA_TRY(cudaMemcpyAsync(order, &first, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    return SV_OK;
  }
  if (!workspace || workspace_bytes < sv_maximin_workspace_bytes_flags(n, d, flags)) return SV_ENOSPC;
  switch (maximin_form(n, d, flags)) {
    case 0:
      return maximin_cluster_single(X, n, d, first, order, info, (char*)workspace, flags, st);
    case 1:
      return maximin_grid_single(X, n, d, first, order, info, (char*)workspace, workspace_bytes, flags, st);
    default:
      return maximin_tree_single(X, n, d, first, order, info, (char*)workspace, workspace_bytes, flags, st);
  }
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

// the cluster and grid forms hold every row in shared memory; the tree form
// takes any count the int32 row indices allow
extern "C" int64_t sv_maximin_max_rows(int32_t d) {
  (void)d;
  return 0x7fffffffLL;
}

extern "C" int64_t sv_maximin_grid_max_rows(int32_t d) { return maximin_grid_max_rows(d); }
