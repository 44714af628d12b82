// Register-resident fused z pass of the subsampled-kernel convolution: a tile
// of B columns of one y row is transformed along z, multiplied by the
// nearest-neighbour kernel coefficient of each frequency (fc_sub.cuh) and
// transformed back, in registers; the spectrum is read and written once.
#include "fc_fast_cols.cuh"
#include "fc_sub.cuh"

namespace fc {
namespace fast {

// 16-column tiles (ZTile, as the fused z pass of the plain convolution): 73 us
// against 103 us for 32-column tiles at 512x512x128 on GB300 (more resident
// warps at these register counts, less work lost on the ragged last tile).
// Loading the coefficients before the forward transform measured twice as
// slow (the registers it holds cut the resident warps).
template <int N>
__global__ void __launch_bounds__(ZTile<N>::THREADS) k_zsub(float2* __restrict__ S, long long pitch, int ny,
                                                             int ncols, SubMap m, float scale,
                                                             const float2* __restrict__ W) {
  using G = ZTile<N>;
  constexpr int B = G::B;
  // the forward runs the forward chain, the inverse the reversed one, so the
  // forward's outputs are the inverse's first-stage inputs in registers
  constexpr int R0 = first_radix<N, false>(), RM = last_radix<N, false>(), RF = last_radix<N, true>();
  __shared__ float2 sm[G::SMEM];
  const int tid = threadIdx.x;
  const int c = tid % B;
  const int t = tid / B;
  const int col = blockIdx.x * B + c;
  const int y = blockIdx.y;
  const bool ok = col < ncols && t < G::T;
  const long long zs = (long long)ny * pitch;
  float2* base = S + (long long)y * pitch + col;
  const ColLay<B> lay{sm, c};
  float2 v[kVals];
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int z = stage_pos<N, R0>(t, q);
    v[q] = (ok && z >= 0) ? base[(long long)z * zs] : make_float2(0.f, 0.f);
  }
  fft<N, false>(v, lay, t, W);
  const SubCol kc(m, ok ? col : 0, y);
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int fz = stage_pos<N, RM>(t, q);
    if (ok && fz >= 0) v[q] = sub_product(kc.at(fz), v[q], scale);
  }
  fft<N, true>(v, lay, t, W);
  if (ok) {
#pragma unroll
    for (int q = 0; q < kVals; ++q) {
      const int z = stage_pos<N, RF>(t, q);
      if (z >= 0) base[(long long)z * zs] = v[q];
    }
  }
}

}  // namespace fast

cudaError_t fast_zsub(float2* S, long long pitch, int ny, int ncols, const SubMap& m, float scale, const FcAxis& az,
                      cudaStream_t st) {
  if (ny <= 0 || ncols <= 0) return cudaSuccess;
  switch (az.n) {
#define FC_CASE(n_)                                                                    \
  case n_: {                                                                           \
    using G = fast::ZTile<n_>;                                                         \
    dim3 grid((ncols + G::B - 1) / G::B, ny);                                          \
    fast::k_zsub<n_><<<grid, G::THREADS, 0, st>>>(S, pitch, ny, ncols, m, scale, az.W); \
    return cudaGetLastError();                                                         \
  }
    FC_COL_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

}  // namespace fc
