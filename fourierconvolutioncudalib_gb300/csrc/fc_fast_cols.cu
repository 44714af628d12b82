// Register-resident column passes for power-of-two lengths: the y passes,
// the fused z pass (forward image and kernel columns, the reference's
// modulate-and-normalise, inverse) and the kernel-gradient z pass.
//
// A CTA owns B adjacent columns (kx) of one plane; thread (c, t) holds E
// values of column c at positions t + m*T.  Global loads and stores are
// B*8 contiguous bytes per row; shared memory is an N x B tile in a padded
// layout used only for the exchanges between radix stages.
#include "fc_fast.cuh"
#include "fc_internal.h"
#include "fc_sources.cuh"

namespace fc {
namespace fast {

template <int N>
struct ColGeom {
  static constexpr int E = P2<N>::E;
  static constexpr int T = P2<N>::T;
  // columns per tile: N*B ~ 4096 values, between 4 and 32
  static constexpr int B = (4096 / N) < 4 ? 4 : ((4096 / N) > 32 ? 32 : (4096 / N));
  static constexpr int THREADS = B * T;
  static constexpr int SMEM = N * B + (N * B) / 16;  // float2 elements
};

template <int N, bool INV, class Src>
__global__ void __launch_bounds__(ColGeom<N>::THREADS) k_cols(Src src, float2* dst, long long ps,
                                                              long long es, int ncols, const float2* __restrict__ W) {
  using G = ColGeom<N>;
  constexpr int E = G::E, T = G::T, B = G::B;
  __shared__ float2 sm[G::SMEM];
  const int c = threadIdx.x % B;
  const int t = threadIdx.x / B;
  const int col = blockIdx.x * B + c;
  const int plane = blockIdx.y;
  const bool ok = col < ncols;
  float2 v[E];
#pragma unroll
  for (int m = 0; m < E; ++m) v[m] = ok ? src.load(plane, t + m * T, col) : make_float2(0.f, 0.f);
  fft<N, INV>(v, ColLay<B>{sm, c}, t, W);
  if (ok) {
    float2* d = dst + (long long)plane * ps + col;
#pragma unroll
    for (int q = 0; q < E; ++q) d[(long long)out_pos<N>(t, q) * es] = v[q];
  }
}

// Fused z pass.  Kernel plane p of KXY holds z = (p - hz) mod nz.
template <int N, bool CONJ>
__global__ void __launch_bounds__(ColGeom<N>::THREADS) k_zconv(float2* __restrict__ S, const float2* __restrict__ KXY,
                                                               long long pitch, int ny, int ncols, int kplanes, int hz,
                                                               float scale, const float2* __restrict__ W) {
  using G = ColGeom<N>;
  constexpr int E = G::E, T = G::T, B = G::B;
  __shared__ float2 sm[G::SMEM];
  const int c = threadIdx.x % B;
  const int t = threadIdx.x / B;
  const int col = blockIdx.x * B + c;
  const int ky = blockIdx.y;
  const bool ok = col < ncols;
  const long long zs = (long long)ny * pitch;
  float2* base = S + (long long)ky * pitch + col;
  float2 v[E], w[E];
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const int z = t + m * T;
    v[m] = ok ? base[z * zs] : make_float2(0.f, 0.f);
    int p = z + hz;
    if (p >= N) p -= N;
    w[m] = (ok && p < kplanes) ? KXY[((long long)p * ny + ky) * pitch + col] : make_float2(0.f, 0.f);
  }
  const ColLay<B> lay{sm, c};
  fft<N, false>(w, lay, t, W);
  fft<N, false>(v, lay, t, W);
#pragma unroll
  for (int q = 0; q < E; ++q) {
    float2 a = w[q];        // kernel spectrum (d_Src of modulateAndNormalize_kernel)
    const float2 b = v[q];  // image spectrum  (d_Dst)
    if (CONJ) a.y = -a.y;
    v[q] = make_float2(scale * (a.x * b.x - a.y * b.y), scale * (a.y * b.x + a.x * b.y));
  }
  out_to_in<N>(v);
  fft<N, true>(v, lay, t, W);
  if (ok) {
#pragma unroll
    for (int q = 0; q < E; ++q) base[(long long)out_pos<N>(t, q) * zs] = v[q];
  }
}

// Kernel-gradient z pass: conj(X) * G * scale, inverse, keep kernel planes
// p < kz where z = (p - hz) mod nz, written to out plane p.
template <int N>
__global__ void __launch_bounds__(ColGeom<N>::THREADS) k_zcorr(const float2* __restrict__ X,
                                                               const float2* __restrict__ Gs, float2* __restrict__ out,
                                                               long long pitch, int ny, int ncols, int kz, int hz,
                                                               float scale, const float2* __restrict__ W) {
  using G = ColGeom<N>;
  constexpr int E = G::E, T = G::T, B = G::B;
  __shared__ float2 sm[G::SMEM];
  const int c = threadIdx.x % B;
  const int t = threadIdx.x / B;
  const int col = blockIdx.x * B + c;
  const int ky = blockIdx.y;
  const bool ok = col < ncols;
  const long long zs = (long long)ny * pitch;
  const long long off = (long long)ky * pitch + col;
  float2 v[E], w[E];
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const long long g = (long long)(t + m * T) * zs + off;
    v[m] = ok ? X[g] : make_float2(0.f, 0.f);
    w[m] = ok ? Gs[g] : make_float2(0.f, 0.f);
  }
  const ColLay<B> lay{sm, c};
  fft<N, false>(v, lay, t, W);
  fft<N, false>(w, lay, t, W);
#pragma unroll
  for (int q = 0; q < E; ++q) {
    const float2 a = make_float2(v[q].x, -v[q].y);
    const float2 b = w[q];
    v[q] = make_float2(scale * (a.x * b.x - a.y * b.y), scale * (a.y * b.x + a.x * b.y));
  }
  out_to_in<N>(v);
  fft<N, true>(v, lay, t, W);
  if (ok) {
#pragma unroll
    for (int q = 0; q < E; ++q) {
      const int z = out_pos<N>(t, q);
      int p = z + hz;
      if (p >= N) p -= N;
      if (p < kz) out[((long long)p * ny + ky) * pitch + col] = v[q];
    }
  }
}

#define FC_COL_SIZES(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024)

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
#define FC_CASE(n_) \
  case n_:          \
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

cudaError_t fast_zconv(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                       float scale, bool conj_kernel, const FcAxis& az, cudaStream_t st) {
  if (ny <= 0 || ncols <= 0) return cudaSuccess;
  switch (az.n) {
#define FC_CASE(n_)                                                                                             \
  case n_: {                                                                                                    \
    using G = fast::ColGeom<n_>;                                                                                \
    dim3 grid((ncols + G::B - 1) / G::B, ny);                                                                   \
    if (conj_kernel)                                                                                            \
      fast::k_zconv<n_, true><<<grid, G::THREADS, 0, st>>>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az.W); \
    else                                                                                                        \
      fast::k_zconv<n_, false><<<grid, G::THREADS, 0, st>>>(S, KXY, pitch, ny, ncols, kplanes, hz, scale,       \
                                                            az.W);                                              \
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
    dim3 grid((ncols + G::B - 1) / G::B, ny);                                                                \
    fast::k_zcorr<n_><<<grid, G::THREADS, 0, st>>>(X, G_, out, pitch, ny, ncols, kz, hz, scale, az.W);        \
    return cudaGetLastError();                                                                               \
  }
    FC_COL_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

}  // namespace fc
