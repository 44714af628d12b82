// Tensor-core precision mode: the register-resident pass kernels with their
// radix-16 stages on the fifth-generation tensor cores (tcgen05, fc_tc5.cuh),
// for the power-of-two lengths FC_TC_SIZES.  This file is compiled twice,
// with FC_TC_MODE=1 (fp16 hi+lo operands) and FC_TC_MODE=2 (bf16 hi+lo
// operands).
//
// Dynamic shared memory of every kernel: [exchange tile | stash (z pass) |
// tcgen05 area (tc::tc5_bytes, 128-byte aligned)].  Every kernel sets the
// mode up at start (DFT operands, mbarrier, TMEM allocation) and frees its
// TMEM at the end; no kernel of this file returns early.
#include "fc_fast_cols.cuh"
#include "fc_fast_rows.cuh"

#ifndef FC_TC_MODE
#define FC_TC_MODE 1
#endif
#define FC_TC_SIZES(X) X(128) X(256) X(512) X(1024)

namespace fc {
namespace fast {

constexpr int TCM = FC_TC_MODE;

// byte offset of the tcgen05 area after `floats2` float2 of the kernel's own buffers
__host__ __device__ constexpr size_t tc_area_off(size_t floats2) { return (floats2 * sizeof(float2) + 127) / 128 * 128; }

static size_t tc_smem(size_t floats2, int nthreads) { return tc_area_off(floats2) + (size_t)tc::tc5_bytes(nthreads); }

__device__ __forceinline__ tc::Tc5 tc_setup(float2* dsm, size_t floats2, int tid, int nthreads) {
  return tc::tc5_setup<TCM>(reinterpret_cast<unsigned char*>(dsm) + tc_area_off(floats2), tid, nthreads);
}

template <int N, class Src>
__global__ void __launch_bounds__(RowGeom<N>::THREADS) k_r2c_tc(Src src, float2* __restrict__ out, long long out_pitch,
                                                                long long nrows, const float2* __restrict__ W) {
  extern __shared__ __align__(128) float2 dsm[];
  const tc::Tc5 t5 = tc_setup(dsm, RowGeom<N>::SMEM, (int)threadIdx.x, (int)blockDim.x);
  body_r2c<N, Src, TCM>(src, out, out_pitch, nrows, W, (long long)blockIdx.x, (int)threadIdx.x, dsm, TcCtx{&t5});
  tc::tc5_teardown(t5, (int)threadIdx.x, (int)blockDim.x);
}

template <int N>
__global__ void __launch_bounds__(RowGeom<N>::THREADS, 3) k_c2r_tc(const float2* __restrict__ in, long long in_pitch,
                                                                float* __restrict__ out, long long out_pitch,
                                                                long long nrows, const float2* __restrict__ W) {
  extern __shared__ __align__(128) float2 dsm[];
  const tc::Tc5 t5 = tc_setup(dsm, RowGeom<N>::SMEM, (int)threadIdx.x, (int)blockDim.x);
  body_c2r<N, TCM, false>(in, in_pitch, out, out_pitch, nrows, W, (long long)blockIdx.x, (int)threadIdx.x, dsm,
                          TcCtx{&t5});
  tc::tc5_teardown(t5, (int)threadIdx.x, (int)blockDim.x);
}

template <int N, bool INV, class Src>
__global__ void __launch_bounds__(ColGeom<N>::THREADS, 3) k_cols_tc(Src src, float2* dst, long long ps, long long es,
                                                                 int ncols, const float2* __restrict__ W) {
  extern __shared__ __align__(128) float2 dsm[];
  const tc::Tc5 t5 = tc_setup(dsm, ColGeom<N>::SMEM, (int)threadIdx.x, (int)blockDim.x);
  body_cols<N, INV, Src, TCM, ColGeom<N>, false>(src, dst, ps, es, ncols, W, (int)blockIdx.x, (int)blockIdx.y,
                                                 (int)threadIdx.x, dsm, TcCtx{&t5});
  tc::tc5_teardown(t5, (int)threadIdx.x, (int)blockDim.x);
}

template <int N>
__global__ void __launch_bounds__(ColGeom<N>::THREADS) k_zconv_tc(float2* __restrict__ S,
                                                                  const float2* __restrict__ KXY, long long pitch,
                                                                  int ny, int ncols, int kplanes, int hz, float scale,
                                                                  const float2* __restrict__ W) {
  extern __shared__ __align__(128) float2 dsm[];
  constexpr int T = ColGeom<N>::THREADS;
  float2* stash = dsm + ColGeom<N>::SMEM;
  const tc::Tc5 t5 = tc_setup(dsm, ColGeom<N>::SMEM + T * kVals, (int)threadIdx.x, (int)blockDim.x);
  body_zconv<N, false, TCM>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, W, (int)blockIdx.x, (int)blockIdx.y,
                            (int)threadIdx.x, dsm, stash, T, TcCtx{&t5});
  tc::tc5_teardown(t5, (int)threadIdx.x, (int)blockDim.x);
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
    const size_t sm = fast::tc_smem(G::SMEM, G::THREADS);                                    \
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
    const size_t sm = fast::tc_smem(G::SMEM, G::THREADS);                         \
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
    const size_t sm = fast::tc_smem(G::SMEM, G::THREADS);                                     \
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
    const size_t sm = fast::tc_smem(G::SMEM + G::THREADS * fast::kVals, G::THREADS);        \
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

cudaError_t FC_TC_NAME(tc_timeouts_addr, FC_TC_SUFFIX)(unsigned int** p) {
  return cudaGetSymbolAddress((void**)p, tc::g_tc5_timeouts);
}
cudaError_t FC_TC_NAME(tc_timeouts_read_async, FC_TC_SUFFIX)(unsigned int* dst, cudaStream_t st) {
  return cudaMemcpyFromSymbolAsync(dst, tc::g_tc5_timeouts, sizeof(unsigned int), 0, cudaMemcpyDeviceToHost, st);
}
void FC_TC_NAME(tc_timeouts_clear, FC_TC_SUFFIX)() {
  const unsigned int zero = 0;
  cudaMemcpyToSymbol(tc::g_tc5_timeouts, &zero, sizeof(zero));
}

}  // namespace fc
