// Radix plan of one transform axis, shared by host and device code.
#pragma once
#include <cuda_runtime.h>

#define FC_MAX_STAGES 24

struct FcAxis {
  int n;                      // transform length
  int nst;                    // number of stages
  int radix[FC_MAX_STAGES];   // radix of each stage; product == n
  const float2* W;            // n roots exp(-2*pi*i*k/n), device memory
};
