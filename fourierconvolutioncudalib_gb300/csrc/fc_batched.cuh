// Work-list descriptors of the batched convolution (many volumes of uneven
// sizes, each with its own kernel).  Every pass of the batch is one
// persistent launch; its work-list holds one task per (view, pass role), and
// a task's tiles are numbered consecutively from tile0.  Host side:
// fc_host.cpp (batched section); device side: fc_batched_kern.cuh and the
// fc_batched_*.cu files.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fc {

enum BMode : int {
  kBRowsDense = 0,  // x R2C of an image: src float rows -> dst float2 rows
  kBRowsBox = 1,    // x R2C of kernel taps placed by the centred shift
  kBRowsC2R = 2,    // x C2R: src float2 rows -> dst float rows
  kBColsFwd = 3,    // y forward, in place
  kBColsInv = 4,    // y inverse, in place
  kBColsKX = 5,     // kernel y forward from the compact x-spectrum rows
  kBZconv = 6,      // fused z pass
};

struct BTask {
  long long tile0;   // first global tile of this task
  long long tiles;   // number of tiles
  long long rows;    // rows (x passes), planes (y passes), ny (z pass)
  long long p0, p1;  // x: in / out pitch; y: plane / element stride; z: row pitch
  const void* src;
  void* dst;
  const void* aux;   // z: kernel xy-spectrum
  const float2* W;   // twiddles of the pass axis
  int n;             // transform length of the pass axis
  int mode;          // BMode
  int ncols;         // columns (y and z passes)
  int i0, i1, i2;    // box: kx, hx | kernel y: krows, hy | z: kplanes, hz
  float scale;
  int pad_;
};

// launchers (device side, one translation unit each); tasks is a device array sorted by tile0
cudaError_t batched_rows_fwd(const BTask* tasks, int ntasks, long long total_tiles, int grid, size_t smem,
                             cudaStream_t st);
cudaError_t batched_rows_inv(const BTask* tasks, int ntasks, long long total_tiles, int grid, size_t smem,
                             cudaStream_t st);
cudaError_t batched_cols_fwd(const BTask* tasks, int ntasks, long long total_tiles, int grid, size_t smem,
                             cudaStream_t st);
cudaError_t batched_cols_inv(const BTask* tasks, int ntasks, long long total_tiles, int grid, size_t smem,
                             cudaStream_t st);
// smem = exchange bytes (max over the tasks) + the stash of kBatchThreads * 16 values
cudaError_t batched_zconv(const BTask* tasks, int ntasks, long long total_tiles, int grid, size_t smem,
                          cudaStream_t st);
// resident CTAs per SM of each batched kernel at the given dynamic shared memory
int batched_occupancy_rows_fwd(size_t smem);
int batched_occupancy_rows_inv(size_t smem);
int batched_occupancy_cols_fwd(size_t smem);
int batched_occupancy_cols_inv(size_t smem);
int batched_occupancy_zconv(size_t smem);
// per-length geometry, 0 when the length has no register-resident kernel
long long batched_row_tiles(int n, long long rows);
long long batched_col_tiles(int n, int ncols, long long planes);
size_t batched_row_smem(int n);
size_t batched_col_smem(int n, bool zconv);
constexpr int kBatchThreads = 256;

}  // namespace fc
