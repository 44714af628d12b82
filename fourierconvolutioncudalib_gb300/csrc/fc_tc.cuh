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
// per-CTA table of the A fragments of the two distinct 16 x 16 blocks of the
// real DFT matrix, C[r][c] = cos(2 pi r c / 16) and S[r][c] = sin(2 pi r c / 16):
// [block 2][lane 32][4 regs] x (hi, lo)
constexpr int kTableWords = 2 * 32 * 4 * 2;  // 512 words

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

// Fill the A-fragment table (call with all threads of the CTA, then barrier).
// Fragment layout of m16n8k16 (row-major A): register reg of lane (g = lane/4,
// q = lane%4) holds A[g + 8*(reg&1)][2q + 8*(reg>>1) + {0,1}].
template <int TCM>
__device__ __forceinline__ void build_table(uint32_t* tab, int tid, int nthreads) {
  for (int e = tid; e < 2 * 32; e += nthreads) {
    const int lane = e & 31, blk = e >> 5;  // blk 0: C, 1: S
    const int g = lane >> 2, q = lane & 3;
    for (int reg = 0; reg < 4; ++reg) {
      const int r = g + 8 * (reg & 1), c = 2 * q + 8 * (reg >> 1);
      const float f0 = blk ? cos16(r * c - 4) : cos16(r * c);  // sin(x) = cos(x - pi/2)
      const float f1 = blk ? cos16(r * (c + 1) - 4) : cos16(r * (c + 1));
      const float h0 = round16<TCM>(f0), h1 = round16<TCM>(f1);
      tab[(e * 4 + reg) * 2 + 0] = pack2<TCM>(h0, h1);
      tab[(e * 4 + reg) * 2 + 1] = pack2<TCM>(f0 - h0, f1 - h1);
    }
  }
}

// x0, x1 rounded to the 16-bit type (hi) and their rounding errors (lo), packed
template <int TCM>
__device__ __forceinline__ void split2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
  if constexpr (TCM == kFp16) {
    const __half2 h = __floats2half2_rn(x0, x1);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(x0 - hf.x, x1 - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  } else {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  }
}

// D += A_hi B_hi + A_hi B_lo + A_lo B_hi for one 16 x 8 output tile
template <int TCM>
__device__ __forceinline__ void mma3(float (&d)[4], const uint32_t (&ah)[4], const uint32_t (&al)[4], uint32_t bh0,
                                     uint32_t bh1, uint32_t bl0, uint32_t bl1) {
  mma16816<TCM>(d, ah, bh0, bh1);
  mma16816<TCM>(d, ah, bl0, bl1);
  mma16816<TCM>(d, al, bh0, bh1);
}

// In-place 16-point DFT of every lane's v[0..15] (all 32 lanes must call).
template <bool INV, int TCM>
__device__ __forceinline__ void dft16(float2* v, uint32_t* ws, const uint32_t* tab) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, q = lane & 3;
  // fp16: power-of-two scale of this column (bf16 has the float exponent range)
  float s = 1.f, inv_s = 1.f;
  if constexpr (TCM == kFp16) {
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) m = fmaxf(m, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
    // m < 2^e from the biased exponent E of m (E = 0 for zero and subnormal m),
    // e clamped to [-126, 126] so that both 2^-e and 2^e are normal floats
    const int e = min(max(((__float_as_int(m) >> 23) & 255) - 126, -126), 126);
    s = __int_as_float((127 - e) << 23);
    inv_s = __int_as_float((127 + e) << 23);
  }
  uint32_t* hi = ws;
  uint32_t* lo = ws + 32 * kColWords;
#pragma unroll
  for (int w = 0; w < 16; ++w) {  // word w holds reals 2w, 2w+1 of the column (0..15 Re, 16..31 Im)
    const int k0 = (2 * w) & 15, k1 = (2 * w + 1) & 15;
    const float x0 = (w < 8 ? v[k0].x : v[k0].y) * s;
    const float x1 = (w < 8 ? v[k1].x : v[k1].y) * s;
    split2<TCM>(x0, x1, hi[lane * kColWords + w], lo[lane * kColWords + w]);
  }
  __syncwarp();
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[i][j][c] = 0.f;
  // A blocks (i, kk): (0,0) and (1,1) are C; (0,1) is -Im W = +S forward, -S inverse;
  // (1,0) is Im W = -S forward, +S inverse.  Negation flips the sign bits of both halves.
  uint32_t ch[4], cl[4], sh[4], sl[4], nh[4], nl[4];
#pragma unroll
  for (int reg = 0; reg < 4; ++reg) {
    ch[reg] = tab[(lane * 4 + reg) * 2 + 0];
    cl[reg] = tab[(lane * 4 + reg) * 2 + 1];
    sh[reg] = tab[((32 + lane) * 4 + reg) * 2 + 0];
    sl[reg] = tab[((32 + lane) * 4 + reg) * 2 + 1];
    nh[reg] = sh[reg] ^ 0x80008000u;
    nl[reg] = sl[reg] ^ 0x80008000u;
  }
#pragma unroll
  for (int kk = 0; kk < 2; ++kk) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = 8 * j + g;
      const uint32_t bh0 = hi[n * kColWords + 8 * kk + q], bh1 = hi[n * kColWords + 8 * kk + q + 4];
      const uint32_t bl0 = lo[n * kColWords + 8 * kk + q], bl1 = lo[n * kColWords + 8 * kk + q + 4];
      if (kk == 0) {
        mma3<TCM>(acc[0][j], ch, cl, bh0, bh1, bl0, bl1);
        if (INV)
          mma3<TCM>(acc[1][j], sh, sl, bh0, bh1, bl0, bl1);
        else
          mma3<TCM>(acc[1][j], nh, nl, bh0, bh1, bl0, bl1);
      } else {
        if (INV)
          mma3<TCM>(acc[0][j], nh, nl, bh0, bh1, bl0, bl1);
        else
          mma3<TCM>(acc[0][j], sh, sl, bh0, bh1, bl0, bl1);
        mma3<TCM>(acc[1][j], ch, cl, bh0, bh1, bl0, bl1);
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
