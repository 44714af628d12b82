// Batched persistent y forward pass (image columns and kernel columns of every view).
#include "fc_batched_kern.cuh"

#define FC_BATCH_CASE_col_fwd_task(n_)                                            \
  case n_:                                                                        \
    fc::fast::col_fwd_task<n_>(tk, tile, (int)threadIdx.x, bsm);                  \
    break;

namespace fc {
namespace fast {
FC_DEFINE_BATCH_KERNEL(k_batch_cols_fwd, 2, FC_BATCH_COL_SIZES, col_fwd_task, , )
}  // namespace fast

long long batched_col_tiles(int n, int ncols, long long planes) {
  switch (n) {
#define FC_CASE(n_) \
  case n_:          \
    return (long long)((ncols + fast::ColGeom<n_>::B - 1) / fast::ColGeom<n_>::B) * planes;
    FC_BATCH_COL_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return 0;
  }
}

size_t batched_col_smem(int n, bool zconv) {
  (void)zconv;
  switch (n) {
#define FC_CASE(n_) \
  case n_:          \
    return sizeof(float2) * fast::ColGeom<n_>::SMEM;
    FC_BATCH_COL_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return 0;
  }
}

cudaError_t batched_cols_fwd(const BTask* tasks, int ntasks, long long total_tiles, int grid, size_t smem,
                             cudaStream_t st) {
  if (total_tiles <= 0) return cudaSuccess;
  cudaError_t e = fast::opt_in_smem((const void*)fast::k_batch_cols_fwd, smem);
  if (e != cudaSuccess) return e;
  fast::k_batch_cols_fwd<<<grid, kBatchThreads, smem, st>>>(tasks, ntasks, total_tiles);
  return cudaGetLastError();
}

int batched_occupancy_cols_fwd(size_t smem) {
  int n = 0;
  if (fast::opt_in_smem((const void*)fast::k_batch_cols_fwd, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fast::k_batch_cols_fwd, kBatchThreads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n < 1 ? 1 : n;
}

}  // namespace fc
