// Register-resident fused z passes (convolution and kernel gradient):
// instantiations and launchers (templates in fc_fast_cols.cuh).
#include "fc_fast_cols.cuh"

namespace fc {
namespace fast {
// opt in to more than 48 KiB of dynamic shared memory where a kernel needs it
template <class K>
static cudaError_t set_dyn_smem(K kernel, int bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
}  // namespace fast

cudaError_t fast_zconv(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                       float scale, bool conj_kernel, const FcAxis& az, cudaStream_t st) {
  if (ny <= 0 || ncols <= 0) return cudaSuccess;
  switch (az.n) {
#define FC_CASE(n_)                                                                                             \
  case n_: {                                                                                                    \
    using G = fast::ColGeom<n_>;                                                                                \
    constexpr int sm = fast::ZGeom<n_>::SMEM_BYTES;                                                             \
    dim3 grid((ncols + G::B - 1) / G::B, ny);                                                                   \
    cudaError_t e;                                                                                              \
    if (conj_kernel) {                                                                                          \
      e = fast::set_dyn_smem(fast::k_zconv<n_, true>, sm);                                                      \
      if (e != cudaSuccess) return e;                                                                           \
      fast::k_zconv<n_, true><<<grid, G::THREADS, sm, st>>>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az.W);   \
    } else {                                                                                                    \
      e = fast::set_dyn_smem(fast::k_zconv<n_, false>, sm);                                                     \
      if (e != cudaSuccess) return e;                                                                           \
      fast::k_zconv<n_, false><<<grid, G::THREADS, sm, st>>>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az.W);  \
    }                                                                                                           \
    return cudaGetLastError();                                                                                  \
  }
    FC_COL_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

cudaError_t fast_zcorr(const float2* X, const float2* G_, float2* out, long long pitch, int ny, int ncols, int kz,
                       int hz, float scale, const FcAxis& az, cudaStream_t st) {
  if (ny <= 0 || ncols <= 0) return cudaSuccess;
  switch (az.n) {
#define FC_CASE(n_)                                                                                          \
  case n_: {                                                                                                 \
    using G = fast::ColGeom<n_>;                                                                             \
    constexpr int sm = fast::ZGeom<n_>::SMEM_BYTES;                                                          \
    dim3 grid((ncols + G::B - 1) / G::B, ny);                                                                \
    const cudaError_t e = fast::set_dyn_smem(fast::k_zcorr<n_>, sm);                                         \
    if (e != cudaSuccess) return e;                                                                          \
    fast::k_zcorr<n_><<<grid, G::THREADS, sm, st>>>(X, G_, out, pitch, ny, ncols, kz, hz, scale, az.W);       \
    return cudaGetLastError();                                                                               \
  }
    FC_COL_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

}  // namespace fc
