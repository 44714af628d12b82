// Nearest-neighbour kernel coefficient of the subsampled-kernel convolution
// (src/convolution3Dfft.cu:65-125, modulateAndNormalizeSubsampled_kernel).
//
// The kernel is transformed at its own size (kx, ky, kz), without padding or
// centring.  Image frequency f along an axis of length n reads kernel
// frequency (int)(r * f + 0.5) mod k with r = k / n (float32, one rounding of
// the multiply-add, as the reference's contracted expression at :106-108,
// with r from :68-70); the coefficient (:110-111) is negated where the three
// kernel indices sum to an odd number (:113-117), the reference's stand-in
// for the phase of the centre shift.
//
// One deliberate difference: for an odd kx the image's x Nyquist frequency
// maps to x index (kx+1)/2, one past the kx/2+1 stored columns; the reference
// then reads the first element of the next row (past the buffer's end at the
// last row).  Here that index takes the value the full spectrum holds there,
// the conjugate of the mirrored coefficient (K real).
#pragma once
#include "fc_internal.h"

namespace fc {

// (int)(r * f + 0.5) mod k; the kernel is no longer than the image (r <= 1,
// f < n), so the truncated value is at most k and the modulo one subtraction
__device__ __forceinline__ int sub_index(float r, int f, int k) {
  const int i = __float2int_rz(__fmaf_rn(r, (float)f, 0.5f));
  return i >= k ? i - k : i;
}

// The lookup for one spectrum column (fx, fy): its x and y kernel indices are
// fixed, only the z index varies along the column.
struct SubCol {
  const float2* p;  // the column's coefficient in kernel plane 0
  long long ps;     // kernel plane stride
  float rz;
  int kz, par;      // par: parity of ix + iy
  bool mir;         // x index past the stored half: mirrored, conjugated column

  __device__ __forceinline__ SubCol(const SubMap& m, int fx, int fy) {
    const int ix = sub_index(m.rx, fx, m.kx);
    const int iy = sub_index(m.ry, fy, m.ky);
    mir = ix >= m.kxh;
    const int jy = mir ? (iy ? m.ky - iy : 0) : iy;
    p = m.K + (long long)jy * m.kpitch + (mir ? m.kx - ix : ix);
    ps = (long long)m.ky * m.kpitch;
    rz = m.rz;
    kz = m.kz;
    par = (ix + iy) & 1;
  }
  // coefficient for z frequency fz, in the product's operand order
  __device__ __forceinline__ float2 at(int fz) const {
    const int iz = sub_index(rz, fz, kz);
    const int pz = mir ? (iz ? kz - iz : 0) : iz;
    float2 a = p[pz * ps];
    if (mir) a.y = -a.y;
    if ((iz + par) & 1) a = make_float2(-a.x, -a.y);
    return a;
  }
};

// scale * (a * b) in the operation order of the reference's mulAndScale (:41-45)
__device__ __forceinline__ float2 sub_product(float2 a, float2 b, float scale) {
  return make_float2(scale * (a.x * b.x - a.y * b.y), scale * (a.y * b.x + a.x * b.y));
}

}  // namespace fc
