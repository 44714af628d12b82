// Batched persistent x R2C pass (image rows and kernel-tap rows of every view).
#include "fc_batched_kern.cuh"

#define FC_BATCH_CASE_row_fwd_task(n_)                                            \
  case n_:                                                                        \
    fc::fast::row_fwd_task<n_>(tk, tile, (int)threadIdx.x, bsm);                  \
    break;

namespace fc {
namespace fast {
FC_DEFINE_BATCH_KERNEL(k_batch_rows_fwd, 2, FC_BATCH_ROW_SIZES, row_fwd_task, , )
}  // namespace fast

long long batched_row_tiles(int n, long long rows) {
  switch (n) {
#define FC_CASE(n_) \
  case n_:          \
    return fast::RowGeom<n_>::tiles(rows);
    FC_BATCH_ROW_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return 0;
  }
}

size_t batched_row_smem(int n) {
  switch (n) {
#define FC_CASE(n_) \
  case n_:          \
    return sizeof(float2) * fast::RowGeom<n_>::SMEM;
    FC_BATCH_ROW_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return 0;
  }
}

cudaError_t batched_rows_fwd(const BTask* tasks, int ntasks, long long total_tiles, int grid, size_t smem,
                             cudaStream_t st) {
  if (total_tiles <= 0) return cudaSuccess;
  cudaError_t e = fast::opt_in_smem((const void*)fast::k_batch_rows_fwd, smem);
  if (e != cudaSuccess) return e;
  fast::k_batch_rows_fwd<<<grid, kBatchThreads, smem, st>>>(tasks, ntasks, total_tiles);
  return cudaGetLastError();
}

int batched_occupancy_rows_fwd(size_t smem) {
  int n = 0;
  if (fast::opt_in_smem((const void*)fast::k_batch_rows_fwd, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fast::k_batch_rows_fwd, kBatchThreads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n < 1 ? 1 : n;
}

}  // namespace fc
