// Tensor-core 16-point DFT for the radix-16 stages of the register-resident
// engine (opt-in precision mode, FC_FLAG_TC_FP16 / FC_FLAG_TC_BF16).
//
// At a radix-16 stage every lane of a warp owns one butterfly: 16 complex
// inputs x (after the stage twiddles).  The warp's 32 butterflies are the
// columns of a real 32 x 32 matrix X = [Re x; Im x], and the DFT is the real
// product Y = F X with F = [[Re W, -Im W], [Im W, Re W]], W[r][c] =
// exp(-+2 pi i r c / 16).  Each column is scaled by its own power of two
// (|x| < 1 after scaling, so fp16 cannot overflow), split into hi + lo
// halves of the 16-bit type, and multiplied on the tensor cores with
// mma.sync m16n8k16 as F_hi X_hi + F_hi X_lo + F_lo X_hi with fp32
// accumulation (the F_lo X_lo term is below fp32 rounding).  The columns go
// to the MMA operand layout and back through a per-warp shared tile.  The
// entries of F come from the exact values cos(2 pi a / 16), a = 0..4; a column
// whose largest magnitude is below 2^-126 (subnormal taps at the edge of a
// PSF) is scaled by 2^126 only, so scale and unscale stay finite.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace fc {
namespace tc {

// modes
constexpr int kNone = 0, kFp16 = 1, kBf16 = 2;

// per-warp scratch: two arrays of 32 columns x 17 words (hi, lo), reused for
// the 32 x 33-float output tile
constexpr int kColWords = 17;
constexpr int kWarpWords = 2 * 32 * kColWords;  // 1088 words (>= 32*33 floats)
// per-CTA table of the A fragments: [dir 2][i 2][kk 2][lane 32][4 regs] x (hi, lo)
constexpr int kTableWords = 2 * 2 * 2 * 32 * 4 * 2;  // 1024 words

template <int TCM>
__device__ __forceinline__ uint32_t pack2(float a, float b) {
  if (TCM == kFp16) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  } else {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  }
}

template <int TCM>
__device__ __forceinline__ float round16(float a) {
  if (TCM == kFp16) return __half2float(__float2half_rn(a));
  return __bfloat162float(__float2bfloat16_rn(a));
}

template <int TCM>
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  if (TCM == kFp16) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
  } else {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
  }
}

// cos(2 pi k / 16) for any integer k, from the exact values cos(2 pi a / 16), a = 0..4
__device__ __forceinline__ float cos16(int k) {
  k &= 15;
  const int a = k <= 8 ? k : 16 - k;  // cos(2 pi (16 - k) / 16) = cos(2 pi k / 16)
  const int b = a <= 4 ? a : 8 - a;   // cos(2 pi (8 - a) / 16) = -cos(2 pi a / 16)
  const float c = b == 0 ? 1.0f
                  : b == 1 ? 0.92387953251128675613f   // cos(pi/8)  = sqrt(2 + sqrt 2) / 2
                  : b == 2 ? 0.70710678118654752440f   // cos(pi/4)  = sqrt 2 / 2
                  : b == 3 ? 0.38268343236508977173f   // cos(3pi/8) = sqrt(2 - sqrt 2) / 2
                           : 0.0f;
  return a <= 4 ? c : -c;
}

// entry (r, c) of the real 32 x 32 DFT matrix; dir 0 forward (exp(-i...)), 1 inverse
__device__ __forceinline__ float dft_real(int r, int c, int dir) {
  const int k = (r & 15) * (c & 15);
  const float cs = cos16(k);
  const float sn = cos16(k - 4);  // sin(2 pi k / 16) = cos(2 pi (k - 4) / 16)
  const float im = dir ? sn : -sn;  // Im W
  if (r < 16) return (c < 16) ? cs : -im;
  return (c < 16) ? im : cs;
}

// Fill the A-fragment table (call with all threads of the CTA, then barrier).
template <int TCM>
__device__ __forceinline__ void build_table(uint32_t* tab, int tid, int nthreads) {
  for (int e = tid; e < 2 * 2 * 2 * 32; e += nthreads) {
    const int lane = e & 31, kk = (e >> 5) & 1, i = (e >> 6) & 1, dir = e >> 7;
    const int g = lane >> 2, q = lane & 3;
    const int rows[4] = {16 * i + g, 16 * i + g + 8, 16 * i + g, 16 * i + g + 8};
    const int cols[4] = {16 * kk + 2 * q, 16 * kk + 2 * q, 16 * kk + 2 * q + 8, 16 * kk + 2 * q + 8};
    for (int reg = 0; reg < 4; ++reg) {
      const float f0 = dft_real(rows[reg], cols[reg], dir);
      const float f1 = dft_real(rows[reg], cols[reg] + 1, dir);
      const float h0 = round16<TCM>(f0), h1 = round16<TCM>(f1);
      tab[(e * 4 + reg) * 2 + 0] = pack2<TCM>(h0, h1);
      tab[(e * 4 + reg) * 2 + 1] = pack2<TCM>(f0 - h0, f1 - h1);
    }
  }
}

// In-place 16-point DFT of every lane's v[0..15] (all 32 lanes must call).
template <bool INV, int TCM>
__device__ __forceinline__ void dft16(float2* v, uint32_t* ws, const uint32_t* tab) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, q = lane & 3;
  // power-of-two scale of this column
  float m = 0.f;
#pragma unroll
  for (int k = 0; k < 16; ++k) m = fmaxf(m, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
  // m < 2^e from the biased exponent E of m (E = 0 for zero and subnormal m),
  // e clamped to [-126, 126] so that both 2^-e and 2^e are normal floats
  const int e = min(max(((__float_as_int(m) >> 23) & 255) - 126, -126), 126);
  const float s = __int_as_float((127 - e) << 23), inv_s = __int_as_float((127 + e) << 23);
  uint32_t* hi = ws;
  uint32_t* lo = ws + 32 * kColWords;
#pragma unroll
  for (int w = 0; w < 16; ++w) {  // word w holds reals 2w, 2w+1 of the column (0..15 Re, 16..31 Im)
    const int k0 = (2 * w) & 15, k1 = (2 * w + 1) & 15;
    const float x0 = (w < 8 ? v[k0].x : v[k0].y) * s;
    const float x1 = (w < 8 ? v[k1].x : v[k1].y) * s;
    const float h0 = round16<TCM>(x0), h1 = round16<TCM>(x1);
    hi[lane * kColWords + w] = pack2<TCM>(h0, h1);
    lo[lane * kColWords + w] = pack2<TCM>(x0 - h0, x1 - h1);
  }
  __syncwarp();
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[i][j][c] = 0.f;
  const int dir = INV ? 1 : 0;
#pragma unroll
  for (int kk = 0; kk < 2; ++kk) {
    uint32_t ah[2][4], al[2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const uint32_t* t = tab + ((((dir * 2 + i) * 2 + kk) * 32 + lane) * 4) * 2;
#pragma unroll
      for (int reg = 0; reg < 4; ++reg) {
        ah[i][reg] = t[reg * 2 + 0];
        al[i][reg] = t[reg * 2 + 1];
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = 8 * j + g;
      const uint32_t bh0 = hi[n * kColWords + 8 * kk + q], bh1 = hi[n * kColWords + 8 * kk + q + 4];
      const uint32_t bl0 = lo[n * kColWords + 8 * kk + q], bl1 = lo[n * kColWords + 8 * kk + q + 4];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        mma16816<TCM>(acc[i][j], ah[i], bh0, bh1);
        mma16816<TCM>(acc[i][j], ah[i], bl0, bl1);
        mma16816<TCM>(acc[i][j], al[i], bh0, bh1);
      }
    }
  }
  __syncwarp();
  // D tile (i, j): rows 16i + g (+8), columns 8j + 2q (+1)  ->  out[col][row], stride 33
  float* out = reinterpret_cast<float*>(ws);
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = 16 * i + g, n = 8 * j + 2 * q;
      out[n * 33 + r] = acc[i][j][0];
      out[(n + 1) * 33 + r] = acc[i][j][1];
      out[n * 33 + r + 8] = acc[i][j][2];
      out[(n + 1) * 33 + r + 8] = acc[i][j][3];
    }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = make_float2(out[lane * 33 + k] * inv_s, out[lane * 33 + 16 + k] * inv_s);
  __syncwarp();
}

}  // namespace tc
}  // namespace fc
