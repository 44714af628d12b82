// Host driver for the reference's subsampled-kernel product -- TEST
// INFRASTRUCTURE ONLY (built by oracle/build_ref.sh into
// oracle/_ref/libfc_reference_sub.so; never linked into the product).
//
// The reference keeps the device product of its memory-saving variant,
// modulateAndNormalizeSubsampled_kernel (src/convolution3Dfft.cu:65-125), but
// comments its host entry out (src/convolution3Dfft.h:58-64).  This file
// compiles the reference's unmodified convolution3Dfft.cu into the same
// translation unit (it is included, not copied) and drives that kernel the
// way the header describes the entry: the image and the kernel are each
// transformed at their own size with cuFFT R2C (no padding, no shift), the
// reference's kernel multiplies the image spectrum by the nearest kernel
// coefficients and 1/N, and a cuFFT C2R returns the result.  The kernel
// spectrum buffer is padded past its end: for an odd kernel x extent the
// reference reads one coefficient past a row (the next row's first; past
// the buffer at the last row), and the padding keeps that read inside the
// allocation.  Dims are slowest-first ({nz, ny, nx}); every CUDA or cuFFT
// failure returns a nonzero code instead of ending the process.
#include "convolution3Dfft.cu"

#include <cstdio>

namespace {
struct Bufs {
  cufftComplex* spec = nullptr;
  cufftComplex* kspec = nullptr;
  float* img = nullptr;
  float* ker = nullptr;
  cufftHandle fwd = 0, kfwd = 0, inv = 0;
  bool f = false, kf = false, i = false;
  ~Bufs() {
    if (f) cufftDestroy(fwd);
    if (kf) cufftDestroy(kfwd);
    if (i) cufftDestroy(inv);
    cudaFree(spec);
    cudaFree(kspec);
    cudaFree(img);
    cudaFree(ker);
  }
};
}  // namespace

extern "C" __attribute__((visibility("default"))) int fcref_subsampled(const float* im, int nz, int ny, int nx,
                                                                        const float* k, int kz, int ky, int kx,
                                                                        float* out, int dev) {
  if (cudaSetDevice(dev) != cudaSuccess) return 1;
  Bufs b;
  const long long n = (long long)nz * ny * nx, kn = (long long)kz * ky * kx;
  const long long mc = (long long)nz * ny * (nx / 2 + 1), kmc = (long long)kz * ky * (kx / 2 + 1);
  if (cudaMalloc(&b.spec, sizeof(cufftComplex) * mc) != cudaSuccess) return 2;
  if (cudaMalloc(&b.kspec, sizeof(cufftComplex) * (kmc + kx + 1)) != cudaSuccess) return 2;
  if (cudaMemset(b.kspec, 0, sizeof(cufftComplex) * (kmc + kx + 1)) != cudaSuccess) return 2;
  if (cudaMalloc(&b.img, sizeof(float) * n) != cudaSuccess) return 2;
  if (cudaMalloc(&b.ker, sizeof(float) * kn) != cudaSuccess) return 2;
  if (cudaMemcpy(b.img, im, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess) return 3;
  if (cudaMemcpy(b.ker, k, sizeof(float) * kn, cudaMemcpyHostToDevice) != cudaSuccess) return 3;
  if (cufftPlan3d(&b.fwd, nz, ny, nx, CUFFT_R2C) != CUFFT_SUCCESS) return 4;
  b.f = true;
  if (cufftPlan3d(&b.kfwd, kz, ky, kx, CUFFT_R2C) != CUFFT_SUCCESS) return 4;
  b.kf = true;
  if (cufftPlan3d(&b.inv, nz, ny, nx, CUFFT_C2R) != CUFFT_SUCCESS) return 4;
  b.i = true;
  if (cufftExecR2C(b.fwd, b.img, b.spec) != CUFFT_SUCCESS) return 5;
  if (cufftExecR2C(b.kfwd, b.ker, b.kspec) != CUFFT_SUCCESS) return 5;
  // launch shape as the reference's InPlace entry sizes its product (src/convolution3Dfft.cu:527-531)
  const int threads = (int)std::min((long long)MAX_THREADS_CUDA, mc);
  const int blocks = (int)std::min((long long)MAX_BLOCKS_CUDA, (mc + threads - 1) / threads);
  modulateAndNormalizeSubsampled_kernel<<<blocks, threads>>>(b.spec, b.kspec, kz, ky, kx, nz, ny, nx, mc,
                                                             1.0f / (float)n);
  if (cudaGetLastError() != cudaSuccess) return 6;
  if (cufftExecC2R(b.inv, b.spec, b.img) != CUFFT_SUCCESS) return 7;
  if (cudaMemcpy(out, b.img, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return 8;
  return 0;
}
