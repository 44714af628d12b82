// Register-resident FFT building blocks for power-of-two lengths (sm_103a).
//
// A line of length N is held by T = N/E threads, E = min(16, N) complex values
// per thread.  The stage chain is radix E, E, ..., then the remainder
// (e.g. 512 = 16*16*2, 128 = 16*8).  At a stage of radix R the thread owns the
// E/R butterflies j = t + b*T (b < E/R); register v[b*R + m] holds the
// butterfly input x[j + m*N/R] before the stage and its output
// y[(j - j%Ns)*R + j%Ns + m*Ns] after it (Stockham, natural order).
//
// Consequences used by the pass kernels:
//   * first stage inputs are x[t + m*T]: thread t loads them straight from
//     global memory (consecutive t -> consecutive addresses);
//   * last stage outputs are y[t + b*T + m*N/Rf]: stored straight to global
//     memory, also coalesced;
//   * between stages the values go once through shared memory (one write,
//     one barrier, one read, one barrier), in a padded layout that is free of
//     bank conflicts for both the row and the column tiles;
//   * a forward transform's outputs are, up to a compile-time permutation of
//     registers, exactly the inputs of the inverse transform's first stage, so
//     a spectrum product between them never touches shared memory.
#pragma once
#include "fc_fft.cuh"

namespace fc {
namespace fast {

template <int N>
struct P2 {
  static constexpr int E = N >= 16 ? 16 : N;
  static constexpr int T = N / E;
  // radix of the last stage
  static constexpr int last_radix() {
    int ns = 1;
    while (true) {
      const int rem = N / ns;
      const int r = rem >= E ? E : rem;
      if (ns * r >= N) return r;
      ns *= r;
    }
  }
  static constexpr int RF = last_radix();
};

__device__ __forceinline__ int rpad(int i) { return i + (i >> 4); }

// shared-memory index of logical position i of a row line (line base added by caller)
struct RowLay {
  float2* base;
  __device__ __forceinline__ float2& operator[](int i) const { return base[rpad(i)]; }
};
// column tile: B adjacent columns, position i of column c
template <int B>
struct ColLay {
  float2* base;
  int c;
  __device__ __forceinline__ float2& operator[](int i) const {
    const int q = i * B;
    return base[q + c + (q >> 4)];
  }
};

template <int N, int E, int R, int NS, bool INV>
__device__ __forceinline__ void stage(float2 (&v)[E], const int t, const float2* __restrict__ W) {
  constexpr int T = N / E;
  constexpr int TWS = N / (NS * R);
#pragma unroll
  for (int b = 0; b < E / R; ++b) {
    if (NS > 1) {
      const int j = t + b * T;
      const int k = j & (NS - 1);
#pragma unroll
      for (int r = 1; r < R; ++r) v[b * R + r] = c_tw<INV>(v[b * R + r], __ldg(W + k * r * TWS));
    }
    Dft<R, INV>::run(&v[b * R]);
  }
}

template <int N, int E, int R, int NS, int R2, class L>
__device__ __forceinline__ void exchange(float2 (&v)[E], const L& sm, const int t) {
  constexpr int T = N / E;
#pragma unroll
  for (int b = 0; b < E / R; ++b) {
    const int j = t + b * T;
    const int k = j & (NS - 1);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int m = 0; m < R; ++m) sm[base + m * NS] = v[b * R + m];
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < E / R2; ++b) {
    const int j = t + b * T;
#pragma unroll
    for (int m = 0; m < R2; ++m) v[b * R2 + m] = sm[j + m * (N / R2)];
  }
  __syncthreads();
}

// Run the stages from sub-transform size NS to the end.
template <int N, int NS, bool INV>
struct Chain {
  static constexpr int E = P2<N>::E;
  template <class L>
  static __device__ __forceinline__ void run(float2 (&v)[E], const L& sm, const int t,
                                             const float2* __restrict__ W) {
    constexpr int REM = N / NS;
    constexpr int R = REM >= E ? E : REM;
    stage<N, E, R, NS, INV>(v, t, W);
    if constexpr (NS * R < N) {
      constexpr int NS2 = NS * R;
      constexpr int REM2 = N / NS2;
      constexpr int R2 = REM2 >= E ? E : REM2;
      exchange<N, E, R, NS, R2>(v, sm, t);
      Chain<N, NS2, INV>::run(v, sm, t, W);
    }
  }
};

// full transform: v[m] = x[t + m*T] in, v[b*RF + m] = X[t + b*T + m*N/RF] out
template <int N, bool INV, class L>
__device__ __forceinline__ void fft(float2 (&v)[P2<N>::E], const L& sm, const int t, const float2* __restrict__ W) {
  Chain<N, 1, INV>::run(v, sm, t, W);
}

// logical position of output register index q (= b*RF + m)
template <int N>
__device__ __forceinline__ int out_pos(const int t, const int q) {
  constexpr int RF = P2<N>::RF;
  return t + (q / RF) * P2<N>::T + (q % RF) * (N / RF);
}

// reorder forward outputs into the inverse's first-stage input order:
// out register b*RF + m holds position t + T*(b + m*E/RF), the inverse's input m' = b + m*E/RF
template <int N>
__device__ __forceinline__ void out_to_in(float2 (&v)[P2<N>::E]) {
  constexpr int E = P2<N>::E;
  constexpr int RF = P2<N>::RF;
  if constexpr (RF != E) {
    float2 w[E];
#pragma unroll
    for (int b = 0; b < E / RF; ++b)
#pragma unroll
      for (int m = 0; m < RF; ++m) w[b + m * (E / RF)] = v[b * RF + m];
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = w[i];
  }
}

}  // namespace fast
}  // namespace fc
