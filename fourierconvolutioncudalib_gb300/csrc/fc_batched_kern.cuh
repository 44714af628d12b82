// Device side of the batched persistent passes (templates; each fat kernel
// is instantiated in its own translation unit to keep the build parallel).
// A fat kernel covers one pass for every view: each CTA walks the global
// tile list with a grid stride and runs the register-resident body of its
// task's length (fc_fast_rows.cuh / fc_fast_cols.cuh).
#pragma once
#include "fc_batched.cuh"
#include "fc_fast_cols.cuh"
#include "fc_fast_rows.cuh"

namespace fc {
namespace fast {

// the task holding global tile g: the last task whose tile0 <= g (tasks sorted
// by tile0, tasks[0].tile0 == 0), by binary search
__device__ __forceinline__ int find_task(const BTask* __restrict__ tasks, int ntasks, long long g) {
  int lo = 0, hi = ntasks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tasks[mid].tile0 <= g)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

template <int N>
__device__ __forceinline__ void row_fwd_task(const BTask& tk, long long tile, int tid, float2* sm) {
  if (tk.mode == kBRowsDense)
    body_r2c<N>(SrcDense{(const float*)tk.src, tk.p0}, (float2*)tk.dst, tk.p1, tk.rows, tk.W, tile, tid, sm);
  else
    body_r2c<N>(SrcBox{(const float*)tk.src, tk.i0, tk.i1, N}, (float2*)tk.dst, tk.p1, tk.rows, tk.W, tile, tid,
                sm);
}

template <int N>
__device__ __forceinline__ void row_inv_task(const BTask& tk, long long tile, int tid, float2* sm) {
  body_c2r<N>((const float2*)tk.src, tk.p0, (float*)tk.dst, tk.p1, tk.rows, tk.W, tile, tid, sm);
}

template <int N>
__device__ __forceinline__ void col_fwd_task(const BTask& tk, long long tile, int tid, float2* sm) {
  constexpr int B = ColGeom<N>::B;
  const long long nbx = (tk.ncols + B - 1) / B;
  const int bx = (int)(tile % nbx);
  const int plane = (int)(tile / nbx);
  float2* S = (float2*)tk.dst;
  if (tk.mode == kBColsKX)
    body_cols<N, false>(ColKX{(const float2*)tk.src, tk.p1, tk.i0, tk.i1, N}, S, tk.p0, tk.p1, tk.ncols, tk.W, bx,
                        plane, tid, sm);
  else
    body_cols<N, false>(ColPlain{S, tk.p0, tk.p1}, S, tk.p0, tk.p1, tk.ncols, tk.W, bx, plane, tid, sm);
}

template <int N>
__device__ __forceinline__ void col_inv_task(const BTask& tk, long long tile, int tid, float2* sm) {
  constexpr int B = ColGeom<N>::B;
  const long long nbx = (tk.ncols + B - 1) / B;
  float2* S = (float2*)tk.dst;
  body_cols<N, true>(ColPlain{S, tk.p0, tk.p1}, S, tk.p0, tk.p1, tk.ncols, tk.W, (int)(tile % nbx),
                     (int)(tile / nbx), tid, sm);
}

template <int N>
__device__ __forceinline__ void z_task(const BTask& tk, long long tile, int tid, float2* sm, float2* stash) {
  constexpr int B = ColGeom<N>::B;
  const long long nbx = (tk.ncols + B - 1) / B;
  body_zconv<N, false>((float2*)tk.dst, (const float2*)tk.aux, tk.p0, (int)tk.rows, tk.ncols, tk.i0, tk.i1, tk.scale,
                       tk.W, (int)(tile % nbx), (int)(tile / nbx), tid, sm, stash, kBatchThreads);
}

static inline cudaError_t opt_in_smem(const void* k, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

}  // namespace fast
}  // namespace fc

// Defines a fat kernel NAME over SIZES(X) calling TASK<N>(tk, tile, tid, smem ARGS).
#define FC_COMMA ,
#define FC_DEFINE_BATCH_KERNEL(NAME, MINB, SIZES, TASK, EXTRA_PARAM, EXTRA_ARG)                  \
  __global__ void __launch_bounds__(fc::kBatchThreads, MINB)                                     \
      NAME(const fc::BTask* __restrict__ tasks, int ntasks, long long total EXTRA_PARAM) {       \
    extern __shared__ float2 bsm[];                                                              \
    for (long long g = blockIdx.x; g < total; g += gridDim.x) {                                  \
      const int i = fc::fast::find_task(tasks, ntasks, g);                                       \
      const fc::BTask tk = tasks[i];                                                             \
      const long long tile = g - tk.tile0;                                                       \
      switch (tk.n) {                                                                            \
        SIZES(FC_BATCH_CASE_##TASK)                                                              \
        default:                                                                                 \
          break;                                                                                 \
      }                                                                                          \
      __syncthreads();                                                                           \
    }                                                                                            \
  }
