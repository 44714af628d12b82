// Tensor-core precision mode: the register-resident pass kernels with their
// radix-16 stages on the tensor cores (fc_tc.cuh), for the power-of-two
// lengths FC_TC_SIZES.  This file is compiled twice, with FC_TC_MODE=1 (fp16
// hi+lo operands) and FC_TC_MODE=2 (bf16 hi+lo operands).
//
// Dynamic shared memory of every kernel: [exchange tile | stash (z pass) |
// A-fragment table (tc::kTableWords) | per-warp scratch (tc::kWarpWords each)];
// the table is built by the CTA at start.
#include "fc_fast_cols.cuh"
#include "fc_fast_rows.cuh"

#ifndef FC_TC_MODE
#define FC_TC_MODE 1
#endif
#define FC_TC_SIZES(X) X(128) X(256) X(512) X(1024)

namespace fc {
namespace fast {

constexpr int TCM = FC_TC_MODE;

__device__ __forceinline__ TcCtx tc_setup(float2* after, int tid, int nthreads) {
  uint32_t* tab = reinterpret_cast<uint32_t*>(after);
  tc::build_table<TCM>(tab, tid, nthreads);
  __syncthreads();
  return TcCtx{tab + tc::kTableWords + (tid >> 5) * tc::kWarpWords, tab};
}

static size_t tc_bytes(int nthreads) {
  return sizeof(uint32_t) * (size_t)(tc::kTableWords + ((nthreads + 31) / 32) * tc::kWarpWords);
}

template <int N, class Src>
__global__ void __launch_bounds__(RowGeom<N>::THREADS) k_r2c_tc(Src src, float2* __restrict__ out, long long out_pitch,
                                                                long long nrows, const float2* __restrict__ W) {
  extern __shared__ float2 dsm[];
  const TcCtx tcx = tc_setup(dsm + RowGeom<N>::SMEM, (int)threadIdx.x, (int)blockDim.x);
  body_r2c<N, Src, TCM>(src, out, out_pitch, nrows, W, (long long)blockIdx.x, (int)threadIdx.x, dsm, tcx);
}

template <int N>
__global__ void __launch_bounds__(RowGeom<N>::THREADS, 3) k_c2r_tc(const float2* __restrict__ in, long long in_pitch,
                                                                float* __restrict__ out, long long out_pitch,
                                                                long long nrows, const float2* __restrict__ W) {
  extern __shared__ float2 dsm[];
  const TcCtx tcx = tc_setup(dsm + RowGeom<N>::SMEM, (int)threadIdx.x, (int)blockDim.x);
  body_c2r<N, TCM, false>(in, in_pitch, out, out_pitch, nrows, W, (long long)blockIdx.x, (int)threadIdx.x, dsm, tcx);
}

template <int N, bool INV, class Src>
__global__ void __launch_bounds__(ColGeom<N>::THREADS, 3) k_cols_tc(Src src, float2* dst, long long ps, long long es,
                                                                 int ncols, const float2* __restrict__ W) {
  extern __shared__ float2 dsm[];
  const TcCtx tcx = tc_setup(dsm + ColGeom<N>::SMEM, (int)threadIdx.x, (int)blockDim.x);
  body_cols<N, INV, Src, TCM, ColGeom<N>, false>(src, dst, ps, es, ncols, W, (int)blockIdx.x, (int)blockIdx.y,
                                                 (int)threadIdx.x, dsm, tcx);
}

template <int N>
__global__ void __launch_bounds__(ColGeom<N>::THREADS) k_zconv_tc(float2* __restrict__ S,
                                                                  const float2* __restrict__ KXY, long long pitch,
                                                                  int ny, int ncols, int kplanes, int hz, float scale,
                                                                  const float2* __restrict__ W) {
  extern __shared__ float2 dsm[];
  constexpr int T = ColGeom<N>::THREADS;
  float2* stash = dsm + ColGeom<N>::SMEM;
  const TcCtx tcx = tc_setup(stash + T * kVals, (int)threadIdx.x, (int)blockDim.x);
  body_zconv<N, false, TCM>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, W, (int)blockIdx.x, (int)blockIdx.y,
                            (int)threadIdx.x, dsm, stash, T, tcx);
}

// opt the kernel in to more than 48 KiB of dynamic shared memory where it needs it
template <class K>
static cudaError_t allow_smem(K kernel, size_t smem) {
  if (smem > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaSuccess;
}

}  // namespace fast

#define FC_TC_NAME2(a, b) a##b
#define FC_TC_NAME(a, b) FC_TC_NAME2(a, b)
#if FC_TC_MODE == 1
#define FC_TC_SUFFIX _fp16
#else
#define FC_TC_SUFFIX _bf16
#endif

cudaError_t FC_TC_NAME(tc_x_r2c, FC_TC_SUFFIX)(const float* in, long long in_pitch, const float* taps, int kx, int hx,
                                              float2* out, long long out_pitch, long long nrows, const FcAxis& ax,
                                              cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  switch (ax.n) {
#define FC_CASE(n_)                                                                                             \
  case n_: {                                                                                                    \
    using G = fast::RowGeom<n_>;                                                                                \
    const size_t sm = sizeof(float2) * G::SMEM + fast::tc_bytes(G::THREADS);                                    \
    const dim3 grid((unsigned)G::tiles(nrows));                                                                 \
    cudaError_t e;                                                                                              \
    if (taps) {                                                                                                 \
      e = fast::allow_smem(fast::k_r2c_tc<n_, SrcBox>, sm);                               \
      if (e != cudaSuccess) return e;                                                                           \
      fast::k_r2c_tc<n_, SrcBox><<<grid, G::THREADS, sm, st>>>(SrcBox{taps, kx, hx, n_}, out, out_pitch, nrows, \
                                                                ax.W);                                          \
    } else {                                                                                                    \
      e = fast::allow_smem(fast::k_r2c_tc<n_, SrcDense>, sm);                             \
      if (e != cudaSuccess) return e;                                                                           \
      fast::k_r2c_tc<n_, SrcDense><<<grid, G::THREADS, sm, st>>>(SrcDense{in, in_pitch}, out, out_pitch, nrows, \
                                                                  ax.W);                                        \
    }                                                                                                           \
    return cudaGetLastError();                                                                                  \
  }
    FC_TC_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

cudaError_t FC_TC_NAME(tc_x_c2r, FC_TC_SUFFIX)(const float2* in, long long in_pitch, float* out, long long out_pitch,
                                              long long nrows, const FcAxis& ax, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  switch (ax.n) {
#define FC_CASE(n_)                                                                                  \
  case n_: {                                                                                         \
    using G = fast::RowGeom<n_>;                                                                     \
    const size_t sm = sizeof(float2) * G::SMEM + fast::tc_bytes(G::THREADS);                         \
    const dim3 grid((unsigned)G::tiles(nrows));                                                      \
    const cudaError_t e = fast::allow_smem(fast::k_c2r_tc<n_>, sm);            \
    if (e != cudaSuccess) return e;                                                                  \
    fast::k_c2r_tc<n_><<<grid, G::THREADS, sm, st>>>(in, in_pitch, out, out_pitch, nrows, ax.W);     \
    return cudaGetLastError();                                                                       \
  }
    FC_TC_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

// y passes: mode 0 forward, 1 inverse, 2 kernel forward from the compact x-spectrum rows
cudaError_t FC_TC_NAME(tc_cols, FC_TC_SUFFIX)(int mode, const float2* src, long long src_pitch, int krows, int hy,
                                             float2* dst, long long ps, long long es, int ncols, int nplanes,
                                             const FcAxis& ax, cudaStream_t st) {
  if (nplanes <= 0 || ncols <= 0) return cudaSuccess;
  switch (ax.n) {
#define FC_CASE(n_)                                                                                              \
  case n_: {                                                                                                     \
    using G = fast::ColGeom<n_>;                                                                                 \
    const size_t sm = sizeof(float2) * G::SMEM + fast::tc_bytes(G::THREADS);                                     \
    const dim3 grid((ncols + G::B - 1) / G::B, nplanes);                                                         \
    cudaError_t e;                                                                                               \
    if (mode == 2) {                                                                                             \
      e = fast::allow_smem(fast::k_cols_tc<n_, false, ColKX>, sm);                         \
      if (e != cudaSuccess) return e;                                                                            \
      fast::k_cols_tc<n_, false, ColKX><<<grid, G::THREADS, sm, st>>>(ColKX{src, src_pitch, krows, hy, n_}, dst, \
                                                                       ps, es, ncols, ax.W);                     \
    } else if (mode == 1) {                                                                                      \
      e = fast::allow_smem(fast::k_cols_tc<n_, true, ColPlain>, sm);                       \
      if (e != cudaSuccess) return e;                                                                            \
      fast::k_cols_tc<n_, true, ColPlain><<<grid, G::THREADS, sm, st>>>(ColPlain{src, ps, es}, dst, ps, es,      \
                                                                          ncols, ax.W);                          \
    } else {                                                                                                     \
      e = fast::allow_smem(fast::k_cols_tc<n_, false, ColPlain>, sm);                      \
      if (e != cudaSuccess) return e;                                                                            \
      fast::k_cols_tc<n_, false, ColPlain><<<grid, G::THREADS, sm, st>>>(ColPlain{src, ps, es}, dst, ps, es,     \
                                                                           ncols, ax.W);                         \
    }                                                                                                            \
    return cudaGetLastError();                                                                                   \
  }
    FC_TC_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

cudaError_t FC_TC_NAME(tc_zconv, FC_TC_SUFFIX)(float2* S, const float2* KXY, long long pitch, int ny, int ncols,
                                              int kplanes, int hz, float scale, const FcAxis& az, cudaStream_t st) {
  if (ny <= 0 || ncols <= 0) return cudaSuccess;
  switch (az.n) {
#define FC_CASE(n_)                                                                                              \
  case n_: {                                                                                                     \
    using G = fast::ColGeom<n_>;                                                                                 \
    const size_t sm = sizeof(float2) * (G::SMEM + G::THREADS * fast::kVals) + fast::tc_bytes(G::THREADS);        \
    const dim3 grid((ncols + G::B - 1) / G::B, ny);                                                              \
    const cudaError_t e = fast::allow_smem(fast::k_zconv_tc<n_>, sm);                      \
    if (e != cudaSuccess) return e;                                                                              \
    fast::k_zconv_tc<n_><<<grid, G::THREADS, sm, st>>>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az.W);       \
    return cudaGetLastError();                                                                                   \
  }
    FC_TC_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

}  // namespace fc
