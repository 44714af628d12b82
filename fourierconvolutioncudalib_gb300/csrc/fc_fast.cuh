// Register-resident FFT building blocks for lengths whose factors are all at
// most 16 (sm_103a).
//
// A length N has a compile-time radix chain R_0 .. R_{S-1} (largest radix
// first, radices 2..16 including the composite 6, 9, 10, 12, 14, 15).  At a
// stage of radix R each thread owns U = floor(16/R) butterflies
// j = t + b*A (b < U, A = ceil((N/R)/U)); register v[b*R + m] holds the
// butterfly input x[j + m*N/R] before the stage and the output
// y[(j - j%Ns)*R + j%Ns + m*Ns] after it (Stockham, natural order).  A line
// is held by T = max_s A_s threads with at most 16 values each.
//
// Consequences used by the pass kernels:
//   * first stage inputs are x[j + m*N/R_0]: loaded straight from global
//     memory (consecutive threads -> consecutive addresses);
//   * last stage outputs are y[j + m*N/R_last]: stored straight to global;
//   * between stages the values go once through shared memory (write,
//     barrier, read, barrier) in a padded layout;
//   * the inverse transform runs the reversed chain, so its first stage has
//     the forward's last radix, thread split and positions: a spectrum product
//     between a forward and an inverse transform happens in registers.
#pragma once
#include "fc_fft.cuh"
#include "fc_tc5.cuh"

namespace fc {
namespace fast {

constexpr int kVals = 16;  // values per thread

// tensor-core mode context: the CTA's tcgen05 state (operands, mbarrier, TMEM)
struct TcCtx {
  const tc::Tc5* t5;
};

__host__ __device__ constexpr int pick_radix(int rem) {
  return rem % 16 == 0   ? 16
         : rem % 15 == 0 ? 15
         : rem % 14 == 0 ? 14
         : rem % 13 == 0 ? 13
         : rem % 12 == 0 ? 12
         : rem % 11 == 0 ? 11
         : rem % 10 == 0 ? 10
         : rem % 9 == 0  ? 9
         : rem % 8 == 0  ? 8
         : rem % 7 == 0  ? 7
         : rem % 6 == 0  ? 6
         : rem % 5 == 0  ? 5
         : rem % 4 == 0  ? 4
         : rem % 3 == 0  ? 3
         : rem % 2 == 0  ? 2
                         : rem;
}

struct ChainC {
  int len;
  int r[12];
};

__host__ __device__ constexpr ChainC make_chain(int N) {
  ChainC c{0, {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}};
  int rem = N;
  while (rem > 1 && c.len < 12) {
    const int r = pick_radix(rem);
    c.r[c.len++] = r;
    rem /= r;
  }
  return c;
}

template <int N>
struct Plan {
  static constexpr ChainC C = make_chain(N);
  static constexpr int S = C.len;
  // stage i of the forward chain (REV = false) or of the reversed chain
  __host__ __device__ static constexpr int radix(int i, bool rev) { return C.r[rev ? S - 1 - i : i]; }
  __host__ __device__ static constexpr int U(int r) { return kVals / r; }
  __host__ __device__ static constexpr int A(int r) { return ((N / r) + U(r) - 1) / U(r); }
  __host__ __device__ static constexpr int max_a() {
    int t = 1;
    for (int i = 0; i < S; ++i) t = A(C.r[i]) > t ? A(C.r[i]) : t;
    return t;
  }
  static constexpr int T = max_a();
  // Stage-twiddle tables, stored after the n roots W[0..n) of the axis table:
  // for stage i >= 1 of a chain (NS = product of the earlier radices, radix R,
  // TWS = N / (NS R)) a block of R-1 rows of NS entries, entry (r, k) =
  // W[k r TWS] at (r-1)*NS + k (consecutive threads read consecutive k);
  // forward chain first, then the reversed chain.  The entries are copies of
  // W, so results do not depend on the layout.
  __host__ __device__ static constexpr int ns(int i, bool rev) {
    int p = 1;
    for (int k = 0; k < i; ++k) p *= radix(k, rev);
    return p;
  }
  __host__ __device__ static constexpr int tab_size(bool rev) {
    int s = 0;
    for (int i = 1; i < S; ++i) s += ns(i, rev) * (radix(i, rev) - 1);
    return s;
  }
  __host__ __device__ static constexpr int tab_off(bool rev, int i) {
    int o = N;
    if (rev) o += tab_size(false);
    for (int k = 1; k < i; ++k) o += ns(k, rev) * (radix(k, rev) - 1);
    return o;
  }
  __host__ __device__ static constexpr int tab_total() { return N + tab_size(false) + tab_size(true); }
  __host__ __device__ static constexpr bool supported() {
    if (N < 2) return false;
    for (int i = 0; i < S; ++i)
      if (C.r[i] > 16) return false;
    int p = 1;
    for (int i = 0; i < S; ++i) p *= C.r[i];
    return p == N;
  }
};

__device__ __forceinline__ int rpad(int i) { return i + (i >> 4); }

// Shared-memory layouts of a line: position i lives at at(i) = base + i*E +
// (D ? i / D : 0) (+ column offset), one pad word per D positions against bank
// conflicts.  A run i0 + m*step (m = 0, 1, ...) is at at(i0) + run_off(m, step)
// whenever no run crosses pad boundaries differently from its first element
// (lin_write / lin_read below), so its addresses fold into constant offsets.
// one line of a row tile; WS: the line's threads sit in one warp (T divides
// 32), so its exchanges synchronise the warp instead of the CTA
template <bool WS = false>
struct RowLayT {
  float2* base;
  static constexpr int E = 1, D = 16;
  static constexpr bool kWarpSync = WS;
  __device__ __forceinline__ float2* at(int i) const { return base + rpad(i); }
  __device__ __forceinline__ float2& operator[](int i) const { return base[rpad(i)]; }
};
using RowLay = RowLayT<false>;
// column tile: B adjacent columns, position i of column c
template <int B>
struct ColLay {
  float2* base;
  int c;
  static constexpr int E = B >= 16 ? B + B / 16 : B;
  static constexpr int D = B >= 16 ? 0 : 16 / B;
  static constexpr bool kWarpSync = false;
  __device__ __forceinline__ float2* at(int i) const {
    const int q = i * B;
    return base + q + c + (q >> 4);
  }
  __device__ __forceinline__ float2& operator[](int i) const { return *at(i); }
};

template <class L>
__host__ __device__ constexpr int run_off(int m, int step) {
  return m * step * L::E + (L::D ? (m * step) / L::D : 0);
}
// Stockham write run: base = (j - k) R + k with k = j mod NS < NS, elements
// base + m NS (m < R) inside the NS*R-aligned block of the butterfly
template <class L>
__host__ __device__ constexpr bool lin_write(int NS, int R) {
  if (L::D == 0) return true;  // no padding: every run is linear
  const int D = L::D ? L::D : 1;  // (not zero here; spelled so for the front end)
  return NS % D == 0 || (D % NS == 0 && ((NS * R) % D == 0 || D % (NS * R) == 0));
}
// read run: j + m NB (any j)
template <class L>
__host__ __device__ constexpr bool lin_read(int NB) {
  if (L::D == 0) return true;
  const int D = L::D ? L::D : 1;  // (not zero here; spelled so for the front end)
  return NB % D == 0;
}

// stage I of the forward chain (REV = false) or of the reversed chain (REV = true);
// INV selects the conjugate twiddles and DFT roots.  TWS: W is a copy of the
// chain's stage tables alone (its first entry is stage 1's), typically in
// shared memory, instead of the whole global table of the axis.
template <int N, int I, int R, int NS, bool INV, int TCM, bool REV = INV, bool TWS = false>
__device__ __forceinline__ void stage(float2 (&v)[kVals], const int t, const float2* __restrict__ W,
                                      const TcCtx& tcx) {
  constexpr int U = kVals / R;
  constexpr int A = Plan<N>::A(R);
  constexpr int NB = N / R;
  // butterflies a thread does not own compute on stale registers and are never
  // stored; their twiddle row k = (t + b*A) mod NS stays inside the table
#pragma unroll
  for (int b = 0; b < U; ++b) {
    if (NS > 1) {
      const int k = (t + b * A) % NS;
      if constexpr (TWS) {
        const float2* tw = W + (Plan<N>::tab_off(REV, I) - Plan<N>::tab_off(REV, 1)) + k;
#pragma unroll
        for (int r = 1; r < R; ++r) v[b * R + r] = c_tw<INV>(v[b * R + r], tw[(r - 1) * NS]);
      } else {
        const float2* tw = W + Plan<N>::tab_off(REV, I) + k;
#pragma unroll
        for (int r = 1; r < R; ++r) v[b * R + r] = c_tw<INV>(v[b * R + r], __ldg(tw + (r - 1) * NS));
      }
    }
    if constexpr (TCM != tc::kNone && R == 16)
      tc::dft16<INV, TCM>(&v[b * R], *tcx.t5);
    else
      Dft<R, INV>::run(&v[b * R]);
  }
  (void)NB;
  (void)tcx;
}

// TAIL: end with the barrier that lets the exchange area be written again;
// false where the caller passes a CTA barrier before its next write there
template <int N, int R, int NS, int R2, bool TAIL = true, class L>
__device__ __forceinline__ void exchange(float2 (&v)[kVals], const L& sm, const int t) {
  constexpr int U = kVals / R, A = Plan<N>::A(R), NB = N / R;
  constexpr int U2 = kVals / R2, A2 = Plan<N>::A(R2), NB2 = N / R2;
#pragma unroll
  for (int b = 0; b < U; ++b) {
    const int j = t + b * A;
    if (j < NB && t < A) {
      const int k = j % NS;
      const int base = (j - k) * R + k;
      if constexpr (lin_write<L>(NS, R)) {
        float2* p = sm.at(base);
#pragma unroll
        for (int m = 0; m < R; ++m) p[run_off<L>(m, NS)] = v[b * R + m];
      } else {
#pragma unroll
        for (int m = 0; m < R; ++m) sm[base + m * NS] = v[b * R + m];
      }
    }
  }
  if constexpr (L::kWarpSync)
    __syncwarp();
  else
    __syncthreads();
#pragma unroll
  for (int b = 0; b < U2; ++b) {
    const int j = t + b * A2;
    if (j < NB2 && t < A2) {
      if constexpr (lin_read<L>(NB2)) {
        const float2* p = sm.at(j);
#pragma unroll
        for (int m = 0; m < R2; ++m) v[b * R2 + m] = p[run_off<L>(m, NB2)];
      } else {
#pragma unroll
        for (int m = 0; m < R2; ++m) v[b * R2 + m] = sm[j + m * NB2];
      }
    }
  }
  if constexpr (TAIL) {
    if constexpr (L::kWarpSync)
      __syncwarp();
    else
      __syncthreads();
  }
}

// stages I .. S-1 of the forward chain (INV = false) or of the reversed chain (INV = true).
// LASTSYNC false: the last exchange leaves out its closing barrier (the caller
// passes a CTA barrier before it next writes the exchange area).
template <int N, int I, int NS, bool INV, int TCM, bool REV = INV, bool TWS = false, bool LASTSYNC = true>
struct Chain {
  template <class L>
  static __device__ __forceinline__ void run(float2 (&v)[kVals], const L& sm, const int t,
                                             const float2* __restrict__ W, const TcCtx& tcx) {
    constexpr int R = Plan<N>::radix(I, REV);
    stage<N, I, R, NS, INV, TCM, REV, TWS>(v, t, W, tcx);
    if constexpr (I + 1 < Plan<N>::S) {
      constexpr int R2 = Plan<N>::radix(I + 1, REV);
      exchange<N, R, NS, R2, (LASTSYNC || I + 2 < Plan<N>::S)>(v, sm, t);
      Chain<N, I + 1, NS * R, INV, TCM, REV, TWS, LASTSYNC>::run(v, sm, t, W, tcx);
    }
  }
};

// full transform; inputs per first_pos, outputs per last_pos.  TCM selects
// the tensor-core 16-point DFT for the radix-16 stages (tc::kFp16 / kBf16).
// REV: radix order (false: the forward chain, true: the reversed chain).  A
// transform that consumes another's outputs in registers runs the other's
// order reversed; a standalone pass may run either.  LASTSYNC as in Chain.
template <int N, bool INV, int TCM = tc::kNone, bool REV = INV, bool TWS = false, bool LASTSYNC = true, class L>
__device__ __forceinline__ void fft(float2 (&v)[kVals], const L& sm, const int t, const float2* __restrict__ W,
                                    const TcCtx& tcx = TcCtx{nullptr}) {
  Chain<N, 0, 1, INV, TCM, REV, TWS, LASTSYNC>::run(v, sm, t, W, tcx);
}

// Stage tables of one chain: Plan<N>::tab_size(REV) entries starting at the
// axis table's tab_off(REV, 1); copy_stage_tables copies them (all threads of
// the CTA take part; a barrier must follow before use) for fft<..., TWS=true>.
template <int N, bool REV>
__device__ __forceinline__ void copy_stage_tables(float2* dst, const float2* __restrict__ W, int tid, int nthreads) {
  constexpr int n = Plan<N>::tab_size(REV);
  const float2* src = W + Plan<N>::tab_off(REV, 1);
  for (int i = tid; i < n; i += nthreads) dst[i] = __ldg(src + i);
}

// radix of the first / last stage of the forward (INV=false) or inverse chain
template <int N, bool INV>
__host__ __device__ constexpr int first_radix() {
  return Plan<N>::radix(0, INV);
}
template <int N, bool INV>
__host__ __device__ constexpr int last_radix() {
  return Plan<N>::radix(Plan<N>::S - 1, INV);
}

// Register q = b*R + m of a stage of radix R (first stage: input position;
// last stage: output position) is position j + m*N/R with j = t + b*A(R);
// returns -1 when the butterfly does not exist for this thread.
template <int N, int R>
__device__ __forceinline__ int stage_pos(const int t, const int q) {
  constexpr int A = Plan<N>::A(R);
  const int b = q / R, m = q % R;
  const int j = t + b * A;
  if (q >= (kVals / R) * R || t >= A || j >= N / R) return -1;
  return j + m * (N / R);
}

}  // namespace fast
}  // namespace fc
