// Batched persistent fused z pass of every view.  The union of all lengths'
// code paths needs up to 255 registers, so this kernel runs one CTA per SM;
// the tuner may prefer one launch per view (fc_host.cpp, batched section).
#include "fc_batched_kern.cuh"

#define FC_BATCH_CASE_z_task(n_)                                                  \
  case n_:                                                                        \
    fc::fast::z_task<n_>(tk, tile, (int)threadIdx.x, bsm, bsm + stash_off);       \
    break;

namespace fc {
namespace fast {
FC_DEFINE_BATCH_KERNEL(k_batch_zconv, 1, FC_BATCH_COL_SIZES, z_task, FC_COMMA int stash_off, )
}  // namespace fast

cudaError_t batched_zconv(const BTask* tasks, int ntasks, long long total_tiles, int grid, size_t smem,
                          cudaStream_t st) {
  if (total_tiles <= 0) return cudaSuccess;
  const size_t stash = sizeof(float2) * kBatchThreads * fast::kVals;
  const size_t ex = smem > stash ? smem - stash : 0;
  cudaError_t e = fast::opt_in_smem((const void*)fast::k_batch_zconv, smem);
  if (e != cudaSuccess) return e;
  fast::k_batch_zconv<<<grid, kBatchThreads, smem, st>>>(tasks, ntasks, total_tiles, (int)(ex / sizeof(float2)));
  return cudaGetLastError();
}

int batched_occupancy_zconv(size_t smem) {
  int n = 0;
  if (fast::opt_in_smem((const void*)fast::k_batch_zconv, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fast::k_batch_zconv, kBatchThreads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n < 1 ? 1 : n;
}

}  // namespace fc
