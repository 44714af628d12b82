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

// Fill the stage-twiddle tables of length N (layout: Plan<N>::tab_off) from
// the roots W[0..N) already in the table.
template <int N>
__global__ void k_stage_twiddles(float2* __restrict__ W) {
  constexpr ChainC C = Plan<N>::C;
  const int tid = (int)(blockIdx.x * blockDim.x + threadIdx.x), nth = (int)(gridDim.x * blockDim.x);
  for (int rev = 0; rev < 2; ++rev) {
    int ns = 1;
    int off = rev ? Plan<N>::tab_off(true, 1) : Plan<N>::tab_off(false, 1);
    for (int i = 0; i < Plan<N>::S; ++i) {
      const int R = C.r[rev ? Plan<N>::S - 1 - i : i];
      if (i >= 1) {
        for (int e = tid; e < ns * (R - 1); e += nth) {
          const int r = 1 + e / ns, k = e - (r - 1) * ns;
          W[off + e] = W[k * r * (N / (ns * R))];  // k*r*TWS < N
        }
        off += ns * (R - 1);
      }
      ns *= R;
    }
  }
}

}  // namespace fast

long long fast_twiddle_count(int n) {
  switch (n) {
#define FC_CASE(n_) \
  case n_:          \
    return fast::Plan<n_>::tab_total();
    FC_ROW_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return n;
  }
}

cudaError_t launch_stage_twiddles(float2* W, int n, cudaStream_t st) {
  switch (n) {
#define FC_CASE(n_)                                     \
  case n_:                                              \
    fast::k_stage_twiddles<n_><<<8, 256, 0, st>>>(W); \
    return cudaGetLastError();
    FC_ROW_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaSuccess;
  }
}

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

namespace fast {
// the persistent tensor-map y pass, for in-place passes over a spectrum whose
// planes are ny rows apart (ps == es * n); *used false: not selected or not applicable
template <bool INV>
static cudaError_t dispatch_cols_pipe(int n, float2* S, long long ps, long long es, int ncols, int nplanes,
                                      const float2* W, cudaStream_t st, bool* used) {
  *used = false;
  switch (n) {
#define FC_CASE(n_) \
  case n_:          \
    return cols_pipe_launch<n_, INV>(S, ps, es, ncols, nplanes, W, st, used);
    FC_COL_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaSuccess;
  }
}
}  // namespace fast

cudaError_t fast_cols(const float2* src, float2* dst, long long ps, long long es, int ncols, int nplanes, bool inverse,
                      const FcAxis& ax, cudaStream_t st) {
  if (nplanes <= 0 || ncols <= 0) return cudaSuccess;
  if (src == dst) {
    bool used = false;
    const cudaError_t e = inverse ? fast::dispatch_cols_pipe<true>(ax.n, dst, ps, es, ncols, nplanes, ax.W, st, &used)
                                  : fast::dispatch_cols_pipe<false>(ax.n, dst, ps, es, ncols, nplanes, ax.W, st, &used);
    if (e != cudaSuccess || used) return e;
  }
  const ColPlain s{src, ps, es};
  return inverse ? fast::dispatch_cols<true>(ax.n, s, dst, ps, es, ncols, nplanes, ax.W, st)
                 : fast::dispatch_cols<false>(ax.n, s, dst, ps, es, ncols, nplanes, ax.W, st);
}

namespace fast {
template <int N, bool INV, class Src>
static cudaError_t launch_cols_wide(Src src, float2* dst, long long ps, long long es, int ncols, int nplanes,
                                   const float2* W, cudaStream_t st) {
  using G = ColGeomWide<N>;
  constexpr int sm = G::SMEM * (int)sizeof(float2);
  if (sm > 48 * 1024) {
    const cudaError_t e =
        cudaFuncSetAttribute(k_cols_wide<N, INV, Src>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return e;
  }
  const dim3 grid((ncols + G::B - 1) / G::B, nplanes);
  k_cols_wide<N, INV, Src><<<grid, G::THREADS, sm, st>>>(src, dst, ps, es, ncols, W);
  return cudaGetLastError();
}

template <int N, bool INV>
static cudaError_t run_cols_wide(float2* S, long long ps, long long es, int ncols, int nplanes, const float2* W,
                                 cudaStream_t st) {
  using G = ColGeomWide<N>;
  // measured on GB300: wider tiles pay off for columns of 1024 (32-byte row
  // segments otherwise) and cost time at 512 and below; 2048 has only the
  // wide kernel (the 256-thread tile would not fit static shared memory)
  if constexpr ((G::B == ColGeom<N>::B || N < 1024) && N <= 1024) {
    return run_cols<N, INV, ColPlain>(ColPlain{S, ps, es}, S, ps, es, ncols, nplanes, W, st);
  } else {
    return launch_cols_wide<N, INV, ColPlain>(ColPlain{S, ps, es}, S, ps, es, ncols, nplanes, W, st);
  }
}
}  // namespace fast

bool fast_cols_wide_supported(int n) {
  switch (n) {
#define FC_CASE(n_) case n_:
    FC_COL_SIZES(FC_CASE)
    FC_WIDE_ONLY_SIZES(FC_CASE)
#undef FC_CASE
    return true;
    default:
      return false;
  }
}

cudaError_t fast_cols_wide(float2* S, long long ps, long long es, int ncols, int nplanes, bool inverse,
                           const FcAxis& ax, cudaStream_t st) {
  if (nplanes <= 0 || ncols <= 0) return cudaSuccess;
  {
    bool used = false;
    const cudaError_t e = inverse ? fast::dispatch_cols_pipe<true>(ax.n, S, ps, es, ncols, nplanes, ax.W, st, &used)
                                  : fast::dispatch_cols_pipe<false>(ax.n, S, ps, es, ncols, nplanes, ax.W, st, &used);
    if (e != cudaSuccess || used) return e;
  }
  switch (ax.n) {
#define FC_CASE(n_)                                                                      \
  case n_:                                                                               \
    return inverse ? fast::run_cols_wide<n_, true>(S, ps, es, ncols, nplanes, ax.W, st)  \
                   : fast::run_cols_wide<n_, false>(S, ps, es, ncols, nplanes, ax.W, st);
    FC_COL_SIZES(FC_CASE)
    FC_WIDE_ONLY_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

cudaError_t fast_cols_kx_wide(const float2* kx_spec, long long pitch, int krows, int hy, float2* dst, int ncols,
                              int nplanes, const FcAxis& ax, cudaStream_t st) {
  if (nplanes <= 0 || ncols <= 0) return cudaSuccess;
  const ColKX s{kx_spec, pitch, krows, hy, ax.n};
  switch (ax.n) {
#define FC_CASE(n_) \
  case n_:          \
    return fast::launch_cols_wide<n_, false, ColKX>(s, dst, (long long)ax.n * pitch, pitch, ncols, nplanes, ax.W, st);
    FC_WIDE_ONLY_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

cudaError_t fast_cols_kx(const float2* kx_spec, long long pitch, int krows, int hy, float2* dst, int ncols,
                         int nplanes, const FcAxis& ax, cudaStream_t st) {
  if (nplanes <= 0 || ncols <= 0) return cudaSuccess;
  const ColKX s{kx_spec, pitch, krows, hy, ax.n};
  return fast::dispatch_cols<false>(ax.n, s, dst, (long long)ax.n * pitch, pitch, ncols, nplanes, ax.W, st);
}

cudaError_t ycols_timeouts_addr(unsigned int** p) { return cudaGetSymbolAddress((void**)p, fast::g_ypipe_timeouts); }
cudaError_t ycols_timeouts_read_async(unsigned int* dst, cudaStream_t st) {
  return cudaMemcpyFromSymbolAsync(dst, fast::g_ypipe_timeouts, sizeof(unsigned int), 0, cudaMemcpyDeviceToHost, st);
}
void ycols_timeouts_clear() {
  const unsigned int zero = 0;
  cudaMemcpyToSymbol(fast::g_ypipe_timeouts, &zero, sizeof(zero));
}
cudaError_t ycols_wait_ctl_set(long long limit, int skip_copies) { return async::wait_ctl_set_tu(limit, skip_copies); }

}  // namespace fc
