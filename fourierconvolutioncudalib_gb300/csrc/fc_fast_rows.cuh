// Register-resident x-pass bodies (R2C / C2R) for row lengths in FC_ROW_SIZES,
// shared by the single-volume kernels (fc_fast_rows.cu) and the batched
// persistent kernels (fc_batched_rows_fwd.cu, fc_batched_rows_inv.cu).
//
// Two real rows a, b are transformed as one complex line z = a + i b.  A line
// is held by T = Plan<N>::T threads; a tile is LPB = max(1, 256/T) lines
// (2*LPB real rows) worked by RowGeom<N>::THREADS threads.  Loads and stores
// go straight between global memory and registers; shared memory carries only
// the exchanges between radix stages and, for the R2C, the final pairing of
// Z[k] with Z[N-k] that separates the two half spectra.  Threads with
// tid >= THREADS (a batched launch sized for the largest length) stay inert.
#pragma once
#include "fc_fast.cuh"
#include "fc_fast_sizes.h"
#include "fc_internal.h"
#include "fc_sources.cuh"

namespace fc {
namespace fast {

template <int N>
struct RowGeom {
  static constexpr int T = Plan<N>::T;
  static constexpr int LPB = (256 / T) < 1 ? 1 : 256 / T;  // lines per tile
  static constexpr int THREADS = LPB * T;
  static constexpr int LS = N + N / 16 + 2;  // padded line stride
  static constexpr int SMEM = LPB * LS;       // float2 elements
  static long long tiles(long long nrows) { return (nrows + 2LL * LPB - 1) / (2LL * LPB); }
};

template <int N, class Src, int TCM = tc::kNone>
__device__ __forceinline__ void body_r2c(const Src& src, float2* __restrict__ out, long long out_pitch,
                                         long long nrows, const float2* __restrict__ W, long long tile, int tid,
                                         float2* sm, const TcCtx& tcx = TcCtx{nullptr, nullptr}) {
  using G = RowGeom<N>;
  constexpr int R0 = first_radix<N, false>();
  constexpr int RF = last_radix<N, false>();
  const bool act = tid < G::THREADS;
  const int line = act ? tid / G::T : 0;
  const int t = act ? tid - line * G::T : G::T;  // inert threads own no butterfly
  const long long ra = (tile * G::LPB + line) * 2, rb = ra + 1;
  const bool va = act && ra < nrows, vb = act && rb < nrows;
  float2* lbase = sm + line * G::LS;
  float2 v[kVals];
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int x = stage_pos<N, R0>(t, q);
    v[q] = make_float2(0.f, 0.f);
    if (x >= 0) v[q] = make_float2(va ? src.load(ra, x) : 0.f, vb ? src.load(rb, x) : 0.f);
  }
  fft<N, false, TCM>(v, RowLay{lbase}, t, W, tcx);
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int x = stage_pos<N, RF>(t, q);
    if (x >= 0) lbase[rpad(x)] = v[q];
  }
  __syncthreads();
  if (act) {
    for (int k = t; k <= N / 2; k += G::T) {
      const float2 zk = lbase[rpad(k)];
      const float2 zn = lbase[rpad(k == 0 ? 0 : N - k)];
      if (va) out[ra * out_pitch + k] = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
      if (vb) out[rb * out_pitch + k] = make_float2(0.5f * (zk.y + zn.y), 0.5f * (zn.x - zk.x));
    }
  }
}

template <int N, int TCM = tc::kNone>
__device__ __forceinline__ void body_c2r(const float2* __restrict__ in, long long in_pitch, float* __restrict__ out,
                                         long long out_pitch, long long nrows, const float2* __restrict__ W,
                                         long long tile, int tid, float2* sm,
                                         const TcCtx& tcx = TcCtx{nullptr, nullptr}) {
  using G = RowGeom<N>;
  constexpr int R0 = first_radix<N, true>();
  constexpr int RF = last_radix<N, true>();
  const bool act = tid < G::THREADS;
  const int line = act ? tid / G::T : 0;
  const int t = act ? tid - line * G::T : G::T;
  const long long ra = (tile * G::LPB + line) * 2, rb = ra + 1;
  const bool va = act && ra < nrows, vb = act && rb < nrows;
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
  fft<N, true, TCM>(v, RowLay{sm + line * G::LS}, t, W, tcx);
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int x = stage_pos<N, RF>(t, q);
    if (x >= 0) {
      if (va) out[ra * out_pitch + x] = v[q].x;
      if (vb) out[rb * out_pitch + x] = v[q].y;
    }
  }
}

}  // namespace fast
}  // namespace fc
