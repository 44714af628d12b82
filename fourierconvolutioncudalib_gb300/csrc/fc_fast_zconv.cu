// Register-resident fused z pass of the convolution (kernel spectrum as is):
// instantiations and launcher (templates in fc_fast_cols.cuh; the
// conjugate-kernel and kernel-gradient variants are in fc_fast_zadj.cu).
#include "fc_fast_cols.cuh"

#include <cudaTypedefs.h>

#include <cstdlib>
#include <cstring>

namespace fc {
namespace fast {

// the driver's tensor-map encoder, looked up once (first from zstage_prepare,
// which the host calls when it creates a device context, outside any capture)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    cudaGetLastError();
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  return encode;
}

bool zstage_tensor_map(CUtensorMap* map, const float2* S, long long pitch, int ny, int ncols, int n, int box_cols,
                       int box_rows) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode || ((uintptr_t)S & 15) != 0 || (pitch * (long long)sizeof(float2)) % 16 != 0 || box_rows > 256 ||
      box_cols > 256 || (box_cols * sizeof(float2)) % 16 != 0)
    return false;
  const cuuint64_t dims[3] = {(cuuint64_t)ncols, (cuuint64_t)ny, (cuuint64_t)n};
  const cuuint64_t strides[2] = {(cuuint64_t)pitch * sizeof(float2), (cuuint64_t)pitch * sizeof(float2) * ny};
  const cuuint32_t box[3] = {(cuuint32_t)box_cols, 1u, (cuuint32_t)box_rows};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_INT64, 3, const_cast<float2*>(S), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// FC_ZSTAGE_TMA=0 stages the fused z pass's image tile with cp.async instead
// of the tensor-map copy
bool zstage_use_tma() {
  static const bool on = [] {
    const char* e = std::getenv("FC_ZSTAGE_TMA");
    return !e || std::atoi(e) != 0;
  }();
  return on;
}

bool tile_tensor_map(CUtensorMap* map, const float2* S, long long pitch, int ny, int ncols, int nz, int bx, int by,
                     int bz) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode || ((uintptr_t)S & 15) != 0 || (pitch * (long long)sizeof(float2)) % 16 != 0 || bx < 1 || by < 1 ||
      bz < 1 || bx > 256 || by > 256 || bz > 256 || (bx * sizeof(float2)) % 16 != 0 || ncols < 1 || ny < 1 || nz < 1)
    return false;
  const cuuint64_t dims[3] = {(cuuint64_t)ncols, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)pitch * sizeof(float2), (cuuint64_t)pitch * sizeof(float2) * ny};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_INT64, 3, const_cast<float2*>(S), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool ypipe_selected(int n) {
  // -1: by length (unset), 0: never (FC_YPIPE=0), 1: every length it applies to (FC_YPIPE=1)
  static const int mode = [] {
    const char* e = std::getenv("FC_YPIPE");
    return e ? (std::atoi(e) != 0 ? 1 : 0) : -1;
  }();
  if (mode >= 0) return mode == 1;
  // measured on GB300 over whole convolutions: faster at 512 and 1024
  // (512x512x128: 0.308 against 0.315 ms; 1024x1024x256: 2.356 against
  // 2.400 ms), slower at 448 (0.225 against 0.218 ms)
  return n >= 512 && (n & (n - 1)) == 0;
}

bool zpipe_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("FC_ZPIPE");
    return !e || std::atoi(e) != 0;
  }();
  return on;
}

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

cudaError_t zconv_timeouts_addr(unsigned int** p) { return fast::zstage_timeouts_addr_tu(p); }
cudaError_t zconv_timeouts_read_async(unsigned int* dst, cudaStream_t st) {
  return fast::zstage_timeouts_read_async_tu(dst, st);
}
void zconv_timeouts_clear() { fast::zstage_timeouts_clear_tu(); }
cudaError_t zconv_wait_ctl_set(long long limit, int skip_copies) { return async::wait_ctl_set_tu(limit, skip_copies); }

void zstage_prepare() { (void)fast::tensor_map_encoder(); }

cudaError_t fast_zconv_conj(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                            float scale, const FcAxis& az, cudaStream_t st);

cudaError_t fast_zconv(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                       float scale, bool conj_kernel, const FcAxis& az, cudaStream_t st) {
  if (conj_kernel) return fast_zconv_conj(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az, st);
  return fast::zconv_launch<false>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az, st);
}

}  // namespace fc
