// Register-resident fused z pass of the convolution (kernel spectrum as is):
// instantiations and launcher (templates in fc_fast_cols.cuh; the
// conjugate-kernel and kernel-gradient variants are in fc_fast_zadj.cu).
#include "fc_fast_cols.cuh"

namespace fc {
namespace fast {
// opt in to more than 48 KiB of dynamic shared memory where a kernel needs it
template <class K>
static cudaError_t set_dyn_smem(K kernel, int bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <bool CONJ>
static cudaError_t zconv_launch(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                                float scale, const FcAxis& az, cudaStream_t st) {
  if (ny <= 0 || ncols <= 0) return cudaSuccess;
  switch (az.n) {
#define FC_CASE(n_)                                                                                             \
  case n_: {                                                                                                    \
    using G = ZTile<n_>;                                                                                        \
    constexpr int sm = ZGeom<n_>::SMEM_BYTES;                                                                   \
    dim3 grid((ncols + G::B - 1) / G::B, ny);                                                                   \
    const cudaError_t e = set_dyn_smem(k_zconv<n_, CONJ>, sm);                                                  \
    if (e != cudaSuccess) return e;                                                                             \
    k_zconv<n_, CONJ><<<grid, G::THREADS, sm, st>>>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az.W);        \
    return cudaGetLastError();                                                                                  \
  }
    FC_COL_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}
}  // namespace fast

cudaError_t fast_zconv_conj(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                            float scale, const FcAxis& az, cudaStream_t st);

cudaError_t fast_zconv(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                       float scale, bool conj_kernel, const FcAxis& az, cudaStream_t st) {
  if (conj_kernel) return fast_zconv_conj(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az, st);
  return fast::zconv_launch<false>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az, st);
}

}  // namespace fc
