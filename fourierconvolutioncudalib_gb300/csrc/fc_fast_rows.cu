// Register-resident x passes (R2C / C2R) of one volume: thin kernels over the
// bodies of fc_fast_rows.cuh, one tile (2*LPB rows) per CTA.
#include "fc_fast_rows.cuh"

namespace fc {
namespace fast {

template <int N, class Src>
__global__ void __launch_bounds__(RowGeom<N>::THREADS) k_r2c(Src src, float2* __restrict__ out, long long out_pitch,
                                                             long long nrows, const float2* __restrict__ W) {
  __shared__ float2 sm[RowGeom<N>::SMEM];
  body_r2c<N>(src, out, out_pitch, nrows, W, (long long)blockIdx.x, (int)threadIdx.x, sm);
}

template <int N>
__global__ void __launch_bounds__(RowGeom<N>::THREADS) k_c2r(const float2* __restrict__ in, long long in_pitch,
                                                             float* __restrict__ out, long long out_pitch,
                                                             long long nrows, const float2* __restrict__ W) {
  __shared__ float2 sm[RowGeom<N>::SMEM];
  body_c2r<N, tc::kNone, false>(in, in_pitch, out, out_pitch, nrows, W, (long long)blockIdx.x, (int)threadIdx.x,
                                sm);
}

template <int N, class Src>
static cudaError_t run_r2c(Src src, float2* out, long long out_pitch, long long nrows, const float2* W,
                           cudaStream_t st) {
  using G = RowGeom<N>;
  const unsigned grid = (unsigned)G::tiles(nrows);
  k_r2c<N, Src><<<grid, G::THREADS, 0, st>>>(src, out, out_pitch, nrows, W);
  return cudaGetLastError();
}

template <int N>
static cudaError_t run_c2r(const float2* in, long long in_pitch, float* out, long long out_pitch, long long nrows,
                           const float2* W, cudaStream_t st) {
  using G = RowGeom<N>;
  const unsigned grid = (unsigned)G::tiles(nrows);
  k_c2r<N><<<grid, G::THREADS, 0, st>>>(in, in_pitch, out, out_pitch, nrows, W);
  return cudaGetLastError();
}

template <class Src>
static cudaError_t dispatch_r2c(int n, Src src, float2* out, long long out_pitch, long long nrows, const float2* W,
                                cudaStream_t st) {
  switch (n) {
#define FC_CASE(n_)                                                                          \
  case n_:                                                                                   \
    static_assert(Plan<n_>::supported() && Plan<n_>::T <= 256, "unsupported row length"); \
    return run_r2c<n_, Src>(src, out, out_pitch, nrows, W, st);
    FC_ROW_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

}  // namespace fast

bool fast_rows_supported(int n) {
  switch (n) {
#define FC_CASE(n_) case n_:
    FC_ROW_SIZES(FC_CASE)
#undef FC_CASE
    return true;
    default:
      return false;
  }
}

cudaError_t fast_x_r2c_dense(const float* in, long long in_pitch, float2* out, long long out_pitch, long long nrows,
                             const FcAxis& ax, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  return fast::dispatch_r2c(ax.n, SrcDense{in, in_pitch}, out, out_pitch, nrows, ax.W, st);
}

cudaError_t fast_x_r2c_box(const float* taps, int kx, int hx, float2* out, long long out_pitch, long long nrows,
                           const FcAxis& ax, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  return fast::dispatch_r2c(ax.n, SrcBox{taps, kx, hx, ax.n}, out, out_pitch, nrows, ax.W, st);
}

cudaError_t fast_x_c2r(const float2* in, long long in_pitch, float* out, long long out_pitch, long long nrows,
                       const FcAxis& ax, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  switch (ax.n) {
#define FC_CASE(n_) \
  case n_:          \
    return fast::run_c2r<n_>(in, in_pitch, out, out_pitch, nrows, ax.W, st);
    FC_ROW_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

}  // namespace fc
