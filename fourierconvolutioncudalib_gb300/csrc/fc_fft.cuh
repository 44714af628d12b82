// In-shared-memory mixed-radix Stockham FFT engine for sm_103a.
//
// A CTA holds a set of "lines" (1D signals of length n) in shared memory and
// runs the stages of a radix plan over all of them at once.  Each stage reads
// R values at stride n/R, applies the stage twiddles, does an in-register
// R-point DFT and writes the R outputs at stride Ns (Stockham auto-sort, so the
// result comes out in natural order and no bit reversal is needed).  The
// element (line l, index j) lives at smem[l*ls + j*es]: row tiles use es=1 and
// an odd ls (no bank conflicts), column tiles use es=B (lines = B adjacent
// columns) and ls=1 so that consecutive threads touch consecutive words.
//
// Twiddles come from a per-length table W[k] = exp(-2*pi*i*k/n) that the host
// computes in double precision and rounds once to float.  Inverse transforms
// use conj(W) and are unnormalised (the 1/N of a convolution is applied once,
// in the spectrum multiply, exactly as the reference does in
// modulateAndNormalize_kernel, src/convolution3Dfft.cu:41-62).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "fc_consts.cuh"

#include "fc_axis.h"

__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 c_mulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by the DFT's quarter-turn root: -i for the forward direction, +i for the inverse
template <bool INV>
__device__ __forceinline__ float2 c_rot(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
template <bool INV>
__device__ __forceinline__ float2 c_tw(float2 a, float2 w) {
  return INV ? c_mulc(a, w) : c_mul(a, w);
}

// ---------------------------------------------------------------- butterflies
template <int R, bool INV> struct Dft;

template <bool INV> struct Dft<2, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 a = v[0];
    v[0] = c_add(a, v[1]);
    v[1] = c_sub(a, v[1]);
  }
};

template <bool INV> struct Dft<4, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 t0 = c_add(v[0], v[2]), t1 = c_sub(v[0], v[2]);
    float2 t2 = c_add(v[1], v[3]), t3 = c_rot<INV>(c_sub(v[1], v[3]));
    v[0] = c_add(t0, t2);
    v[2] = c_sub(t0, t2);
    v[1] = c_add(t1, t3);
    v[3] = c_sub(t1, t3);
  }
};

// exp(s*2*pi*i/8) * a, exp(s*2*pi*i*3/8) * a  (s = -1 forward, +1 inverse)
template <bool INV>
__device__ __forceinline__ float2 c_w8_1(float2 a) {
  const float c = FC_SQRT1_2;
  return INV ? make_float2((a.x - a.y) * c, (a.x + a.y) * c) : make_float2((a.x + a.y) * c, (a.y - a.x) * c);
}
template <bool INV>
__device__ __forceinline__ float2 c_w8_3(float2 a) {
  const float c = FC_SQRT1_2;
  return INV ? make_float2((-a.x - a.y) * c, (a.x - a.y) * c) : make_float2((a.y - a.x) * c, (-a.x - a.y) * c);
}

template <bool INV> struct Dft<8, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    o[1] = c_w8_1<INV>(o[1]);
    o[2] = c_rot<INV>(o[2]);
    o[3] = c_w8_3<INV>(o[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = c_add(e[k], o[k]);
      v[k + 4] = c_sub(e[k], o[k]);
    }
  }
};

// radix 16 as 4 x 4: X[k1 + 4 k2] = sum_m2 w16^(m2 k1) w4^(m2 k2) sum_m1 x[4 m1 + m2] w4^(m1 k1)
template <bool INV> struct Dft<16, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    float2 y[4][4];
#pragma unroll
    for (int m2 = 0; m2 < 4; ++m2) {
      float2 t[4] = {v[m2], v[4 + m2], v[8 + m2], v[12 + m2]};
      Dft<4, INV>::run(t);
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1) y[m2][k1] = t[k1];
    }
    const float s = INV ? 1.0f : -1.0f;
    const float2 w1 = make_float2(FC_C16_1, s * FC_S16_1);   // w16^1
    const float2 w3 = make_float2(FC_S16_1, s * FC_C16_1);   // w16^3
    const float2 w9 = make_float2(-FC_C16_1, -s * FC_S16_1); // w16^9
    // m2 = 1: k1 = 1,2,3 -> w^1, w^2, w^3
    y[1][1] = c_mul(y[1][1], w1);
    y[1][2] = c_w8_1<INV>(y[1][2]);
    y[1][3] = c_mul(y[1][3], w3);
    // m2 = 2: w^2, w^4, w^6
    y[2][1] = c_w8_1<INV>(y[2][1]);
    y[2][2] = c_rot<INV>(y[2][2]);
    y[2][3] = c_w8_3<INV>(y[2][3]);
    // m2 = 3: w^3, w^6, w^9
    y[3][1] = c_mul(y[3][1], w3);
    y[3][2] = c_w8_3<INV>(y[3][2]);
    y[3][3] = c_mul(y[3][3], w9);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      float2 t[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
      Dft<4, INV>::run(t);
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
    }
  }
};

// odd prime P: pair x[m] with x[P-m];
//   X[k]   = x0 + sum_m cos(2pi mk/P)(x_m + x_{P-m}) + s*i*sin(2pi mk/P)(x_m - x_{P-m})
//   X[P-k] = x0 + sum_m cos(...)(x_m + x_{P-m})     - s*i*sin(...)(x_m - x_{P-m})
template <int P, bool INV> struct DftOdd {
  static __device__ __forceinline__ void run(float2* v) {
    constexpr int H = (P - 1) / 2;
    float2 sm[H], df[H];
    float2 x0 = v[0];
    float2 X0 = x0;
#pragma unroll
    for (int m = 1; m <= H; ++m) {
      sm[m - 1] = c_add(v[m], v[P - m]);
      df[m - 1] = c_sub(v[m], v[P - m]);
      X0 = c_add(X0, sm[m - 1]);
    }
#pragma unroll
    for (int k = 1; k <= H; ++k) {
      float2 re = x0, im = make_float2(0.f, 0.f);
#pragma unroll
      for (int m = 1; m <= H; ++m) {
        const float c = fc_dft_cos<P>((m * k) % P);
        const float sn = fc_dft_sin<P>((m * k) % P);
        re.x += c * sm[m - 1].x;
        re.y += c * sm[m - 1].y;
        im.x += sn * df[m - 1].x;
        im.y += sn * df[m - 1].y;
      }
      // s*i*im with s = -1 (forward) or +1 (inverse)
      const float2 rim = INV ? make_float2(-im.y, im.x) : make_float2(im.y, -im.x);
      v[k] = c_add(re, rim);
      v[P - k] = c_sub(re, rim);
    }
    v[0] = X0;
  }
};
// composite R = A*B: X[k1 + A k2] = sum_n2 wB^(n2 k2) wR^(n2 k1) sum_n1 x[B n1 + n2] wA^(n1 k1)
template <int A, int B, bool INV> struct DftCT {
  static constexpr int R = A * B;
  static __device__ __forceinline__ void run(float2* v) {
    float2 y[B][A];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      float2 t[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) t[n1] = v[B * n1 + n2];
      Dft<A, INV>::run(t);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) {
        const int e = (n2 * k1) % R;
        if (e == 0) {
          y[n2][k1] = t[k1];
        } else {
          const float2 w = make_float2(fc_tw_cos<R>(e), (INV ? 1.0f : -1.0f) * fc_tw_sin<R>(e));
          y[n2][k1] = c_mul(t[k1], w);
        }
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      float2 t[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) t[n2] = y[n2][k1];
      Dft<B, INV>::run(t);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = t[k2];
    }
  }
};

template <bool INV> struct Dft<3, INV> : DftOdd<3, INV> {};
template <bool INV> struct Dft<5, INV> : DftOdd<5, INV> {};
template <bool INV> struct Dft<7, INV> : DftOdd<7, INV> {};
template <bool INV> struct Dft<11, INV> : DftOdd<11, INV> {};
template <bool INV> struct Dft<13, INV> : DftOdd<13, INV> {};
template <bool INV> struct Dft<6, INV> : DftCT<2, 3, INV> {};
template <bool INV> struct Dft<9, INV> : DftCT<3, 3, INV> {};
template <bool INV> struct Dft<10, INV> : DftCT<2, 5, INV> {};
template <bool INV> struct Dft<12, INV> : DftCT<4, 3, INV> {};
template <bool INV> struct Dft<14, INV> : DftCT<2, 7, INV> {};
template <bool INV> struct Dft<15, INV> : DftCT<3, 5, INV> {};

// ---------------------------------------------------------------- stages
// One Stockham stage of radix R over all lines of a tile.
template <int R, bool INV>
__device__ __forceinline__ void fc_stage(const float2* __restrict__ a, float2* __restrict__ b, const int n,
                                         const int Ns, const float2* __restrict__ W, const int lines_log2,
                                         const int es, const int ls) {
  const int nb = n / R;
  const int tws = n / (Ns * R);
  const int lmask = (1 << lines_log2) - 1;
  const int total = nb << lines_log2;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int line = t & lmask;
    const int j = t >> lines_log2;
    const float2* src = a + line * ls + j * es;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[r * nb * es];
    const int k = j % Ns;
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = c_tw<INV>(v[r], __ldg(W + k * r * tws));
    }
    Dft<R, INV>::run(v);
    float2* dst = b + line * ls + ((j - k) * R + k) * es;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[r * Ns * es] = v[r];
  }
}

// Any radix (primes above 13, e.g. 17, 19, 37, 79, 109): direct O(R^2) DFT per
// butterfly, with twiddle and DFT root folded into one table lookup:
//   out_q = sum_m a[j + m nb] * W[(m * (k*tws + q*nb)) mod n]
template <bool INV>
__device__ __noinline__ void fc_stage_generic(const float2* __restrict__ a, float2* __restrict__ b, const int n,
                                              const int R, const int Ns, const float2* __restrict__ W,
                                              const int lines_log2, const int es, const int ls) {
  const int nb = n / R;
  const int tws = n / (Ns * R);
  const int lmask = (1 << lines_log2) - 1;
  const int total = (nb * R) << lines_log2;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int line = t & lmask;
    const int u = t >> lines_log2;  // u = q * nb + j
    const int q = u / nb;
    const int j = u - q * nb;
    const int k = j % Ns;
    int e = (k * tws + q * nb) % n;
    const float2* src = a + line * ls + j * es;
    float2 acc = make_float2(0.f, 0.f);
    int idx = 0;
    for (int m = 0; m < R; ++m) {
      const float2 x = src[m * nb * es];
      const float2 w = __ldg(W + idx);
      const float2 p = c_tw<INV>(x, w);
      acc.x += p.x;
      acc.y += p.y;
      idx += e;
      if (idx >= n) idx -= n;
    }
    b[line * ls + ((j - k) * R + k + q * Ns) * es] = acc;
  }
}

// Run every stage of the plan.  a holds the input; b is scratch of the same
// layout.  Returns the buffer that holds the result.  Ends with a barrier.
template <bool INV>
__device__ float2* fc_fft_lines(float2* a, float2* b, const FcAxis& ax, const int lines_log2, const int es,
                                const int ls) {
  int Ns = 1;
  for (int s = 0; s < ax.nst; ++s) {
    const int R = ax.radix[s];
    switch (R) {
      case 2: fc_stage<2, INV>(a, b, ax.n, Ns, ax.W, lines_log2, es, ls); break;
      case 3: fc_stage<3, INV>(a, b, ax.n, Ns, ax.W, lines_log2, es, ls); break;
      case 4: fc_stage<4, INV>(a, b, ax.n, Ns, ax.W, lines_log2, es, ls); break;
      case 5: fc_stage<5, INV>(a, b, ax.n, Ns, ax.W, lines_log2, es, ls); break;
      case 7: fc_stage<7, INV>(a, b, ax.n, Ns, ax.W, lines_log2, es, ls); break;
      case 8: fc_stage<8, INV>(a, b, ax.n, Ns, ax.W, lines_log2, es, ls); break;
      case 11: fc_stage<11, INV>(a, b, ax.n, Ns, ax.W, lines_log2, es, ls); break;
      case 13: fc_stage<13, INV>(a, b, ax.n, Ns, ax.W, lines_log2, es, ls); break;
      case 16: fc_stage<16, INV>(a, b, ax.n, Ns, ax.W, lines_log2, es, ls); break;
      default: fc_stage_generic<INV>(a, b, ax.n, R, Ns, ax.W, lines_log2, es, ls); break;
    }
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}
