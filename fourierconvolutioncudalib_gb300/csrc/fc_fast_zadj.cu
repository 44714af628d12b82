// Register-resident fused z passes of the adjoint: the conjugate-kernel
// product (image gradient) and the kernel-gradient correlation
// (templates in fc_fast_cols.cuh).
#include "fc_fast_cols.cuh"

#include <cstring>

namespace fc {
namespace fast {
bool zstage_use_tma();
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
    bool used = false;                                                                                          \
    const cudaError_t ep = zconv_pipe_launch<n_, CONJ>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az.W, st,   \
                                                        &used);                                                 \
    if (ep != cudaSuccess || used) return ep;                                                                   \
    using G = ZTile<n_>;                                                                                        \
    constexpr int sm = ZGeom<n_>::SMEM_BYTES;                                                                   \
    dim3 grid((ncols + G::B - 1) / G::B, ny);                                                                   \
    const cudaError_t e = set_dyn_smem(k_zconv<n_, CONJ>, sm);                                                  \
    if (e != cudaSuccess) return e;                                                                             \
    CUtensorMap map;                                                                                            \
    std::memset(&map, 0, sizeof(map));                                                                          \
    const int tma = ZGeom<n_>::TMA_OK && zstage_use_tma() &&                                                    \
                    zstage_tensor_map(&map, S, pitch, ny, ncols, n_, G::B, ZGeom<n_>::ZBOX);                    \
    k_zconv<n_, CONJ><<<grid, G::THREADS, sm, st>>>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az.W, map,    \
                                                    tma);                                                       \
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
                            float scale, const FcAxis& az, cudaStream_t st) {
  return fast::zconv_launch<true>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az, st);
}

cudaError_t zadj_timeouts_addr(unsigned int** p) { return fast::zstage_timeouts_addr_tu(p); }
cudaError_t zadj_timeouts_read_async(unsigned int* dst, cudaStream_t st) {
  return fast::zstage_timeouts_read_async_tu(dst, st);
}
void zadj_timeouts_clear() { fast::zstage_timeouts_clear_tu(); }
cudaError_t zadj_wait_ctl_set(long long limit, int skip_copies) { return async::wait_ctl_set_tu(limit, skip_copies); }

cudaError_t fast_zcorr(const float2* X, const float2* G_, float2* out, long long pitch, int ny, int ncols, int kz,
                       int hz, float scale, const FcAxis& az, cudaStream_t st) {
  if (ny <= 0 || ncols <= 0) return cudaSuccess;
  switch (az.n) {
#define FC_CASE(n_)                                                                                          \
  case n_: {                                                                                                 \
    using G = fast::ColGeom<n_>;                                                                             \
    constexpr int sm = fast::CorrGeom<n_>::SMEM_BYTES;                                                          \
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
