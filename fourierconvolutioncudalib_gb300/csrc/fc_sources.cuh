// Load functors shared by the generic and the register-resident pass kernels.
#pragma once
#include <cuda_runtime.h>

namespace fc {

// real rows for the x passes
struct SrcDense {  // real rows of a dense volume
  const float* p;
  long long pitch;
  __device__ __forceinline__ float load(long long row, int x) const { return __ldg(p + row * pitch + x); }
};

struct SrcBox {  // kernel taps [kz][ky][kx]; row = plane*ky + iy; x -> ix = (x + hx) mod nx
  const float* k;
  int kx, hx, nx;
  __device__ __forceinline__ float load(long long row, int x) const {
    int ix = x + hx;
    if (ix >= nx) ix -= nx;
    return ix < kx ? __ldg(k + row * kx + ix) : 0.f;
  }
};

// complex columns for the y passes: element (plane, j, c)
struct ColPlain {
  const float2* p;
  long long ps, es;
  __device__ __forceinline__ float2 load(int plane, int j, int c) const {
    return p[(long long)plane * ps + (long long)j * es + c];
  }
};

struct ColKX {  // compact kernel x-spectrum rows: plane*krows + iy, y -> iy = (y + hy) mod ny
  const float2* p;
  long long pitch;
  int krows, hy, ny;
  __device__ __forceinline__ float2 load(int plane, int y, int c) const {
    int iy = y + hy;
    if (iy >= ny) iy -= ny;
    return iy < krows ? p[((long long)plane * krows + iy) * pitch + c] : make_float2(0.f, 0.f);
  }
};

}  // namespace fc
