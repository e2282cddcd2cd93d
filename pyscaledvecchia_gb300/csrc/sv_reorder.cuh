// Internal interface between the batched reorder (sv_reorder.cu) and the kNN
// kernels (sv_knn.cu).
#pragma once
#include "sv_common.cuh"

namespace sv {

// one problem of a batched ordered kNN search
struct KnnBatchProb {
  int64_t xs_off;   // doubles: its rows (maximin order, scaled) in Xs
  int64_t v_off;    // floats: its centred float32 rows [n][DP] in v
  int64_t row_off;  // its rows in B
  int64_t n;
  int64_t blk_off;  // block of row 0 (row i -> block blk_off + i)
  int32_t d, m;
};

// padded dimension of the float32 screening rows (4, 8, 12, 16, 24, 32, 48, 64)
int knn_pad_dim(int d);

// rows per query tile of the batched ordered kNN for padded dimension DP and
// largest neighbour count kcap (the tile table must be built with it)
int knn_batched_tile_rows(int DP, int kcap);

// ordered kNN of every (problem, query tile) entry of tiles (one CTA each);
// all problems of the launch share DP; kcap >= every m
int launch_knn_batched(int DP, const KnnBatchProb* probs, const int2* tiles, int64_t ntiles,
                       const double* Xs, const float* v, const float* B, int32_t* nbr, int ldnbr,
                       int kcap, cudaStream_t st);

// single-problem maximin through the cluster kernel (n <= maximin_cluster_max_rows(d));
// ws: 256 bytes of device scratch; flags: the test aids of sv_reorder_prob
int maximin_cluster_single(const double* X, int64_t n, int d, int64_t first, int64_t* order,
                           int32_t* info, char* ws, int flags, cudaStream_t st);
int64_t maximin_cluster_max_rows(int d);
// single-problem maximin through the grid form (n <= maximin_grid_max_rows(d))
int maximin_grid_single(const double* X, int64_t n, int d, int64_t first, int64_t* order,
                        int32_t* info, char* ws, size_t ws_bytes, int flags, cudaStream_t st);
size_t maximin_grid_workspace_bytes();
int64_t maximin_grid_max_rows(int d);
// single-problem maximin through the tree form (any n >= 2)
int maximin_tree_single(const double* X, int64_t n, int d, int64_t first, int64_t* order,
                        int32_t* info, char* ws, size_t ws_bytes, int flags, cudaStream_t st);
size_t maximin_tree_workspace_bytes(int64_t n, int d);

}  // namespace sv
