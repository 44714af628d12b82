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
  __host__ __device__ static long long tiles(long long nrows) { return (nrows + 2LL * LPB - 1) / (2LL * LPB); }
};

// a line's T threads lie in one warp when T divides 32 (lines start at
// multiples of T); its exchanges then synchronise that warp only.  The
// tensor-core transforms keep CTA barriers.  FC_ROW_WARPSYNC=0 builds the CTA
// barriers everywhere, for comparison builds.
#ifndef FC_ROW_WARPSYNC
#define FC_ROW_WARPSYNC 1
#endif
template <int N, int TCM>
constexpr bool kLineWarp = FC_ROW_WARPSYNC && TCM == tc::kNone && 32 % RowGeom<N>::T == 0;
#ifndef FC_C2R_HALVES
#define FC_C2R_HALVES 1
#endif
// the R2C pairs Z[k] with Z[N-k] by warp shuffles: a line of 32 threads (one
// warp) whose last stage is radix 2 over 32 butterfly columns (N = 512);
// FC_ROW_SHFL=0 builds the shared-memory pairing, for comparison builds
#ifndef FC_ROW_SHFL
#define FC_ROW_SHFL 1
#endif
template <int N, int RF, int AF, bool WS>
constexpr bool kShflPair = FC_ROW_SHFL && WS && RowGeom<N>::T == 32 && RF == 2 && AF == 32 && N == 64 * (kVals / 2);

// line / thread split of a row tile: tile rows ra = 2*(tile*LPB + line), rb = ra + 1
template <int N>
struct RowSlot {
  bool act, va, vb;
  int line, t;
  long long ra, rb;
  __device__ __forceinline__ RowSlot(long long tile, int tid, long long nrows) {
    using G = RowGeom<N>;
    act = tid < G::THREADS;
    line = act ? tid / G::T : 0;
    t = act ? tid - line * G::T : G::T;  // inert threads own no butterfly
    ra = (tile * G::LPB + line) * 2;
    rb = ra + 1;
    va = act && ra < nrows;
    vb = act && rb < nrows;
  }
};

// first-stage values of the R2C: z = a + i b for real rows a, b of the slot
template <int N, class Src, bool REV = false>
__device__ __forceinline__ void load_r2c(float2 (&v)[kVals], const Src& src, const RowSlot<N>& s) {
  constexpr int R0 = first_radix<N, REV>();
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int x = stage_pos<N, R0>(s.t, q);
    v[q] = make_float2(0.f, 0.f);
    if (x >= 0) v[q] = make_float2(s.va ? src.load(s.ra, x) : 0.f, s.vb ? src.load(s.rb, x) : 0.f);
  }
}

// transform of the loaded values, separation of the two half spectra, stores
template <int N, int TCM = tc::kNone, bool REV = false, bool TWS = false>
__device__ __forceinline__ void finish_r2c(float2 (&v)[kVals], const RowSlot<N>& s, float2* __restrict__ out,
                                           long long out_pitch, const float2* __restrict__ W, float2* sm,
                                           const TcCtx& tcx = TcCtx{nullptr}) {
  using G = RowGeom<N>;
  constexpr int RF = last_radix<N, REV>();
  constexpr int NBF = N / RF, UF = kVals / RF, AF = Plan<N>::A(RF);
  constexpr bool WS = kLineWarp<N, TCM>;
  using Lay = RowLayT<WS>;
  float2* lbase = sm + s.line * G::LS;
  const Lay lay{lbase};
  fft<N, false, TCM, REV, TWS>(v, lay, s.t, W, tcx);
  if constexpr (kShflPair<N, RF, AF, WS>) {
    // The line is one warp and lane t holds Z[k] for k = t + 32 b + (N/2) m in
    // v[2b + m]; Z[N - k] sits in lane (32 - t) mod 32, in v[2(UF-1-b) + 1-m]
    // for t != 0 and in v[2(UF-b) + 1-m] for t == 0 (v[m] itself for k = 0,
    // N/2).  Each lane offers the register its partner lane asks for, so one
    // shuffle per value pairs the spectra without a trip through shared memory.
    const int lane = (int)(threadIdx.x & 31u);
    const int from = (32 - lane) & 31;
#pragma unroll
    for (int b = 0; b < UF; ++b) {
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        if (m == 1 && b != 0) continue;  // k > N/2: not stored
        const float2 mine = lane == 0 ? v[b == 0 ? m : 2 * (UF - b) + 1 - m] : v[2 * (UF - 1 - b) + 1 - m];
        const float2 zn = make_float2(__shfl_sync(0xffffffffu, mine.x, from), __shfl_sync(0xffffffffu, mine.y, from));
        const float2 zk = v[2 * b + m];
        const int k = lane + 32 * b + (N / 2) * m;
        if (s.act && (m == 0 || lane == 0)) {
          if (s.va) out[s.ra * out_pitch + k] = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
          if (s.vb) out[s.rb * out_pitch + k] = make_float2(0.5f * (zk.y + zn.y), 0.5f * (zn.x - zk.x));
        }
      }
    }
    return;
  }
  // natural-order outputs x = j + m*NBF of the last stage into the line
#pragma unroll
  for (int b = 0; b < UF; ++b) {
    const int j = s.t + b * AF;
    if (j < NBF && s.t < AF) {
      if constexpr (lin_read<Lay>(NBF)) {
        float2* p = lay.at(j);
#pragma unroll
        for (int m = 0; m < RF; ++m) p[run_off<Lay>(m, NBF)] = v[b * RF + m];
      } else {
#pragma unroll
        for (int m = 0; m < RF; ++m) lay[j + m * NBF] = v[b * RF + m];
      }
    }
  }
  if constexpr (WS)
    __syncwarp();
  else
    __syncthreads();
  if (s.act) {
    for (int k = s.t; k <= N / 2; k += G::T) {
      const float2 zk = lbase[rpad(k)];
      const float2 zn = lbase[rpad(k == 0 ? 0 : N - k)];
      if (s.va) out[s.ra * out_pitch + k] = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
      if (s.vb) out[s.rb * out_pitch + k] = make_float2(0.5f * (zk.y + zn.y), 0.5f * (zn.x - zk.x));
    }
  }
}

template <int N, class Src, int TCM = tc::kNone>
__device__ __forceinline__ void body_r2c(const Src& src, float2* __restrict__ out, long long out_pitch,
                                         long long nrows, const float2* __restrict__ W, long long tile, int tid,
                                         float2* sm, const TcCtx& tcx = TcCtx{nullptr}) {
  const RowSlot<N> s(tile, tid, nrows);
  float2 v[kVals];
  load_r2c<N>(v, src, s);
  finish_r2c<N, TCM>(v, s, out, out_pitch, W, sm, tcx);
}

// first-stage values of the C2R: the Hermitian extension of two half-spectrum
// rows a, b (read through `in` with row pitch in_pitch), packed as A + i B
// REV: radix order of the inverse transform (false: the forward chain with
// conjugate twiddles, which exchanges with fewer bank conflicts; true: the
// reversed chain)
template <int N, class In, bool REV = true>
__device__ __forceinline__ void load_c2r(float2 (&v)[kVals], const In& in, const RowSlot<N>& s) {
  constexpr int R0 = first_radix<N, REV>();
  constexpr int NB0 = N / R0, A0 = Plan<N>::A(R0);
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int k = stage_pos<N, R0>(s.t, q);
    v[q] = make_float2(0.f, 0.f);
    // position k = j + m N/R0 with j < N/R0: for an even R0 the half it lies in
    // is known from m alone except at m = R0/2 (k = N/2 + j), so those values
    // skip the runtime selection (FC_C2R_HALVES=0 builds the selection everywhere)
    constexpr bool kHalves = FC_C2R_HALVES && R0 % 2 == 0 && N % 2 == 0;
    const int m = q % R0;
    if (kHalves && q < (kVals / R0) * R0 && 2 * m < R0) {
      if (s.t < A0 && k >= 0) {  // low half: kk = k; the DC bin (m = 0, j = 0) is real
        float2 a = s.va ? in.load(s.ra, k) : make_float2(0.f, 0.f);
        float2 b = s.vb ? in.load(s.rb, k) : make_float2(0.f, 0.f);
        if (m == 0 && k == 0) {
          a.y = 0.f;
          b.y = 0.f;
        }
        v[q] = make_float2(a.x - b.y, a.y + b.x);
      }
      continue;
    }
    if (kHalves && q < (kVals / R0) * R0 && 2 * m > R0) {
      if (s.t < A0 && k >= 0) {  // high half: the conjugate of bin N - k (never DC or Nyquist)
        const float2 a = s.va ? in.load(s.ra, N - k) : make_float2(0.f, 0.f);
        const float2 b = s.vb ? in.load(s.rb, N - k) : make_float2(0.f, 0.f);
        v[q] = make_float2(a.x + b.y, b.x - a.y);
      }
      continue;
    }
    (void)NB0;
    if (k >= 0) {
      const bool lo = k <= N / 2;
      const int kk = lo ? k : N - k;
      float2 a = s.va ? in.load(s.ra, kk) : make_float2(0.f, 0.f);
      float2 b = s.vb ? in.load(s.rb, kk) : make_float2(0.f, 0.f);
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
}

template <int N, int TCM = tc::kNone, bool REV = true, bool TWS = false>
__device__ __forceinline__ void finish_c2r(float2 (&v)[kVals], const RowSlot<N>& s, float* __restrict__ out,
                                           long long out_pitch, const float2* __restrict__ W, float2* sm,
                                           const TcCtx& tcx = TcCtx{nullptr}) {
  using G = RowGeom<N>;
  constexpr int RF = last_radix<N, REV>();
  fft<N, true, TCM, REV, TWS>(v, RowLayT<kLineWarp<N, TCM>>{sm + s.line * G::LS}, s.t, W, tcx);
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int x = stage_pos<N, RF>(s.t, q);
    if (x >= 0) {
      if (s.va) out[s.ra * out_pitch + x] = v[q].x;
      if (s.vb) out[s.rb * out_pitch + x] = v[q].y;
    }
  }
}

// complex half-spectrum rows in global memory
struct HalfRows {
  const float2* p;
  long long pitch;
  __device__ __forceinline__ float2 load(long long row, int k) const { return p[row * pitch + k]; }
};

template <int N, int TCM = tc::kNone, bool REV = true>
__device__ __forceinline__ void body_c2r(const float2* __restrict__ in, long long in_pitch, float* __restrict__ out,
                                         long long out_pitch, long long nrows, const float2* __restrict__ W,
                                         long long tile, int tid, float2* sm,
                                         const TcCtx& tcx = TcCtx{nullptr}) {
  const RowSlot<N> s(tile, tid, nrows);
  float2 v[kVals];
  load_c2r<N, HalfRows, REV>(v, HalfRows{in, in_pitch}, s);
  finish_c2r<N, TCM, REV>(v, s, out, out_pitch, W, sm, tcx);
}

}  // namespace fast
}  // namespace fc
