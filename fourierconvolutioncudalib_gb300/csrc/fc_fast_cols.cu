// Register-resident y passes: instantiations and launchers (templates in fc_fast_cols.cuh).
#include "fc_fast_cols.cuh"

namespace fc {
namespace fast {

template <int N, bool INV, class Src>
static cudaError_t run_cols(Src src, float2* dst, long long ps, long long es, int ncols, int nplanes, const float2* W,
                            cudaStream_t st) {
  using G = ColGeom<N>;
  dim3 grid((ncols + G::B - 1) / G::B, nplanes);
  k_cols<N, INV, Src><<<grid, G::THREADS, 0, st>>>(src, dst, ps, es, ncols, W);
  return cudaGetLastError();
}

template <bool INV, class Src>
static cudaError_t dispatch_cols(int n, Src src, float2* dst, long long ps, long long es, int ncols, int nplanes,
                                 const float2* W, cudaStream_t st) {
  switch (n) {
#define FC_CASE(n_)                                                                               \
  case n_:                                                                                        \
    static_assert(Plan<n_>::supported() && ColGeom<n_>::THREADS <= 1024, "unsupported column length"); \
    return run_cols<n_, INV, Src>(src, dst, ps, es, ncols, nplanes, W, st);
    FC_COL_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

}  // namespace fast

bool fast_cols_supported(int n) {
  switch (n) {
#define FC_CASE(n_) case n_:
    FC_COL_SIZES(FC_CASE)
#undef FC_CASE
    return true;
    default:
      return false;
  }
}

cudaError_t fast_cols(const float2* src, float2* dst, long long ps, long long es, int ncols, int nplanes, bool inverse,
                      const FcAxis& ax, cudaStream_t st) {
  if (nplanes <= 0 || ncols <= 0) return cudaSuccess;
  const ColPlain s{src, ps, es};
  return inverse ? fast::dispatch_cols<true>(ax.n, s, dst, ps, es, ncols, nplanes, ax.W, st)
                 : fast::dispatch_cols<false>(ax.n, s, dst, ps, es, ncols, nplanes, ax.W, st);
}

cudaError_t fast_cols_kx(const float2* kx_spec, long long pitch, int krows, int hy, float2* dst, int ncols,
                         int nplanes, const FcAxis& ax, cudaStream_t st) {
  if (nplanes <= 0 || ncols <= 0) return cudaSuccess;
  const ColKX s{kx_spec, pitch, krows, hy, ax.n};
  return fast::dispatch_cols<false>(ax.n, s, dst, (long long)ax.n * pitch, pitch, ncols, nplanes, ax.W, st);
}

}  // namespace fc
