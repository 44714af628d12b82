// Register-resident x passes (R2C / C2R) for row lengths in FC_ROW_SIZES.
//
// Two real rows a, b are transformed as one complex line z = a + i b.  A line
// is held by T = Plan<N>::T threads; a CTA carries LPB = max(1, 256/T) lines
// (2*LPB real rows) and has exactly LPB*T threads.  Loads and stores go
// straight between global memory and registers; shared memory carries only
// the exchanges between radix stages and, for the R2C, the final pairing of
// Z[k] with Z[N-k] that separates the two half spectra.
#include "fc_fast.cuh"
#include "fc_fast_sizes.h"
#include "fc_internal.h"
#include "fc_sources.cuh"

namespace fc {
namespace fast {

template <int N>
struct RowGeom {
  static constexpr int T = Plan<N>::T;
  static constexpr int LPB = (256 / T) < 1 ? 1 : 256 / T;  // lines per CTA
  static constexpr int THREADS = LPB * T;
  static constexpr int LS = N + N / 16 + 2;  // padded line stride
};

template <int N, class Src>
__global__ void __launch_bounds__(RowGeom<N>::THREADS) k_r2c(Src src, float2* __restrict__ out, long long out_pitch,
                                                             long long nrows, const float2* __restrict__ W) {
  using G = RowGeom<N>;
  constexpr int T = G::T;
  constexpr int R0 = first_radix<N, false>();
  constexpr int RF = last_radix<N, false>();
  __shared__ float2 sm[G::LPB * G::LS];
  const int line = threadIdx.x / T;
  const int t = threadIdx.x - line * T;
  const long long ra = ((long long)blockIdx.x * G::LPB + line) * 2, rb = ra + 1;
  const bool va = ra < nrows, vb = rb < nrows;
  float2* lbase = sm + line * G::LS;
  float2 v[kVals];
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int x = stage_pos<N, R0>(t, q);
    v[q] = make_float2(0.f, 0.f);
    if (x >= 0) v[q] = make_float2(va ? src.load(ra, x) : 0.f, vb ? src.load(rb, x) : 0.f);
  }
  fft<N, false>(v, RowLay{lbase}, t, W);
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int x = stage_pos<N, RF>(t, q);
    if (x >= 0) lbase[rpad(x)] = v[q];
  }
  __syncthreads();
  for (int k = t; k <= N / 2; k += T) {
    const float2 zk = lbase[rpad(k)];
    const float2 zn = lbase[rpad(k == 0 ? 0 : N - k)];
    if (va) out[ra * out_pitch + k] = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
    if (vb) out[rb * out_pitch + k] = make_float2(0.5f * (zk.y + zn.y), 0.5f * (zn.x - zk.x));
  }
}

template <int N>
__global__ void __launch_bounds__(RowGeom<N>::THREADS) k_c2r(const float2* __restrict__ in, long long in_pitch,
                                                             float* __restrict__ out, long long out_pitch,
                                                             long long nrows, const float2* __restrict__ W) {
  using G = RowGeom<N>;
  constexpr int T = G::T;
  constexpr int R0 = first_radix<N, true>();
  constexpr int RF = last_radix<N, true>();
  __shared__ float2 sm[G::LPB * G::LS];
  const int line = threadIdx.x / T;
  const int t = threadIdx.x - line * T;
  const long long ra = ((long long)blockIdx.x * G::LPB + line) * 2, rb = ra + 1;
  const bool va = ra < nrows, vb = rb < nrows;
  float2 v[kVals];
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int k = stage_pos<N, R0>(t, q);
    v[q] = make_float2(0.f, 0.f);
    if (k >= 0) {
      const bool lo = k <= N / 2;
      const int kk = lo ? k : N - k;
      float2 a = va ? in[ra * in_pitch + kk] : make_float2(0.f, 0.f);
      float2 b = vb ? in[rb * in_pitch + kk] : make_float2(0.f, 0.f);
      if (kk == 0 || 2 * kk == N) {
        a.y = 0.f;
        b.y = 0.f;
      }
      if (!lo) {
        a.y = -a.y;
        b.y = -b.y;
      }
      v[q] = make_float2(a.x - b.y, a.y + b.x);
    }
  }
  fft<N, true>(v, RowLay{sm + line * G::LS}, t, W);
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int x = stage_pos<N, RF>(t, q);
    if (x >= 0) {
      if (va) out[ra * out_pitch + x] = v[q].x;
      if (vb) out[rb * out_pitch + x] = v[q].y;
    }
  }
}

template <int N, class Src>
static cudaError_t run_r2c(Src src, float2* out, long long out_pitch, long long nrows, const float2* W,
                           cudaStream_t st) {
  using G = RowGeom<N>;
  const long long rows_per = 2LL * G::LPB;
  const unsigned grid = (unsigned)((nrows + rows_per - 1) / rows_per);
  k_r2c<N, Src><<<grid, G::THREADS, 0, st>>>(src, out, out_pitch, nrows, W);
  return cudaGetLastError();
}

template <int N>
static cudaError_t run_c2r(const float2* in, long long in_pitch, float* out, long long out_pitch, long long nrows,
                           const float2* W, cudaStream_t st) {
  using G = RowGeom<N>;
  const long long rows_per = 2LL * G::LPB;
  const unsigned grid = (unsigned)((nrows + rows_per - 1) / rows_per);
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
