// Batched persistent x C2R pass of every view.
#include "fc_batched_kern.cuh"

#define FC_BATCH_CASE_row_inv_task(n_)                                            \
  case n_:                                                                        \
    fc::fast::row_inv_task<n_>(tk, tile, (int)threadIdx.x, bsm);                  \
    break;

namespace fc {
namespace fast {
FC_DEFINE_BATCH_KERNEL(k_batch_rows_inv, 2, FC_BATCH_ROW_SIZES, row_inv_task, , )
}  // namespace fast

cudaError_t batched_rows_inv(const BTask* tasks, int ntasks, long long total_tiles, int grid, size_t smem,
                             cudaStream_t st) {
  if (total_tiles <= 0) return cudaSuccess;
  cudaError_t e = fast::opt_in_smem((const void*)fast::k_batch_rows_inv, smem);
  if (e != cudaSuccess) return e;
  fast::k_batch_rows_inv<<<grid, kBatchThreads, smem, st>>>(tasks, ntasks, total_tiles);
  return cudaGetLastError();
}

int batched_occupancy_rows_inv(size_t smem) {
  int n = 0;
  if (fast::opt_in_smem((const void*)fast::k_batch_rows_inv, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fast::k_batch_rows_inv, kBatchThreads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n < 1 ? 1 : n;
}

}  // namespace fc
