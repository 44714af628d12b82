// The reference's convolution3DfftCUDAInPlace restated on cuFFT -- a timing
// baseline and parity harness only, never part of the product library.
//
// The reference sources are not part of this repository, so this file
// re-expresses the same host and device sequence of
// src/convolution3Dfft.cu:399-578 in its own code:
//   host pad of the image into R2C rows (:495-510), H2D (:512-515),
//   fftShiftKernel scatter (:442-461) + per-row D2D copies (:474-486),
//   cufftPlan3d(nz,ny,nx) R2C, exec on image and kernel (:519-525),
//   modulateAndNormalize with 1/N (:527-536), C2R plan + exec (:544-547),
//   D2H (:551-554), host un-pad (:565-575).
// refseq_device_only() runs just the device part (R2C x2, modulate, C2R) on
// pre-padded device buffers with pre-built plans, for kernel-level timing.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define RS_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

int g_err = 0;
char g_msg[256];

bool ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_err = 1;
  snprintf(g_msg, sizeof(g_msg), "%s: %s", what, cudaGetErrorString(e));
  return false;
}
bool okf(cufftResult r, const char* what) {
  if (r == CUFFT_SUCCESS) return true;
  g_err = 2;
  snprintf(g_msg, sizeof(g_msg), "%s: cufft error %d", what, (int)r);
  return false;
}

int closest_multiplier(int a, int m) {
  int value = 1;
  const int mx = (a + m - 1) / m;
  for (int i = 1; i <= mx; ++i) {
    const int d = a - i * m;
    if ((d < 0 ? -d : d) < 1) value = i;
  }
  return value * m;
}

__global__ void __launch_bounds__(1024) rs_modulate(cufftComplex* dst, const cufftComplex* src, long long n,
                                                    float c) {
  long long i = (long long)blockDim.x * blockIdx.x + threadIdx.x;
  const long long step = (long long)blockDim.x * gridDim.x;
  for (; i < n; i += step) {
    const cufftComplex a = src[i];
    const cufftComplex b = dst[i];
    cufftComplex t;
    t.x = c * (a.x * b.x - a.y * b.y);
    t.y = c * (a.y * b.x + a.x * b.y);
    dst[i] = t;
  }
}

__global__ void __launch_bounds__(1024) rs_shift(const float* k, float* out, int kD0, int kD1, int kD2, int iD0,
                                                 int iD1, int iD2, int centered) {
  const int K = kD0 * kD1 * kD2;
  const int tid = blockDim.x * blockIdx.x + threadIdx.x;
  if (tid >= K) return;
  long long x, y, z;
  if (centered) {  // kernel [kz][ky][kx] with kD = {kx,ky,kz}, image {nx,ny,nz}: correct placement
    const long long ix = tid % kD0, r = tid / kD0, iy = r % kD1, iz = r / kD1;
    x = ix - kD0 / 2;
    y = iy - kD1 / 2;
    z = iz - kD2 / 2;
    if (x < 0) x += iD0;
    if (y < 0) y += iD1;
    if (z < 0) z += iD2;
    out[(z * iD1 + y) * iD0 + x] = k[tid];
  } else {  // the reference's arithmetic
    z = tid % kD2;
    const long long aux = (tid - z) / kD2;
    y = aux % kD1;
    x = (aux - y) / kD1;
    x -= kD0 / 2;
    y -= kD1 / 2;
    z -= kD2 / 2;
    if (x < 0) x += iD0;
    if (y < 0) y += iD1;
    if (z < 0) z += iD2;
    out[z + (long long)iD2 * (y + (long long)iD1 * x)] = k[tid];
  }
}

void launch_modulate(cufftComplex* img, const cufftComplex* ker, long long n, float scale, cudaStream_t st) {
  const int threads = (int)(n < 1024 ? n : 1024);
  long long blocks = (n + threads - 1) / threads;
  if (blocks > 65535) blocks = 65535;
  rs_modulate<<<(unsigned)blocks, threads, 0, st>>>(img, ker, n, scale);
}

}  // namespace

RS_EXPORT const char* refseq_last_error() { return g_msg; }

// Full host-to-host sequence of the reference InPlace entry.
// imDim {nx,ny,nz}, kernelDim {kx,ky,kz}; centered != 0 uses the correct
// placement instead of the reference's arithmetic.  Returns 0 on success.
RS_EXPORT int refseq_inplace(float* im, const int* imDim, const float* kernel, const int* kernelDim, int centered) {
  g_err = 0;
  const size_t nx = imDim[0], ny = imDim[1], nz = imDim[2];
  const size_t nxh = nx / 2 + 1;
  const size_t K = (size_t)kernelDim[0] * kernelDim[1] * kernelDim[2];
  const size_t N = nx * ny * nz, Mc = nxh * ny * nz;
  float* shifted = nullptr;
  float* dker = nullptr;
  cufftComplex* kpad = nullptr;
  cufftComplex* dimg = nullptr;
  cufftHandle pf = 0, pi = 0;
  int rc = 0;
  do {
    if (!ok(cudaMalloc(&shifted, N * 4), "malloc") || !ok(cudaMemset(shifted, 0, N * 4), "memset")) break;
    if (!ok(cudaMalloc(&dker, K * 4), "malloc") || !ok(cudaMemcpy(dker, kernel, K * 4, cudaMemcpyHostToDevice), "h2d"))
      break;
    int threads = (int)(K < 1024 ? K : 1024);
    threads = closest_multiplier(threads, 32);
    long long blocks = ((long long)K + threads - 1) / threads;
    if (blocks > 65535) blocks = 65535;
    rs_shift<<<(unsigned)blocks, threads>>>(dker, shifted, kernelDim[0], kernelDim[1], kernelDim[2], (int)nx, (int)ny,
                                            (int)nz, centered);
    if (!ok(cudaGetLastError(), "shift") || !ok(cudaDeviceSynchronize(), "sync")) break;
    cudaFree(dker);
    dker = nullptr;
    if (!ok(cudaMalloc(&kpad, Mc * 8), "malloc") || !ok(cudaMemset(kpad, 0, Mc * 8), "memset")) break;
    bool good = true;
    for (size_t z = 0; z < nz && good; ++z)
      for (size_t y = 0; y < ny && good; ++y)
        good = ok(cudaMemcpy(kpad + (z * ny + y) * nxh, shifted + (z * ny + y) * nx, nx * 4, cudaMemcpyDeviceToDevice),
                  "row copy");
    if (!good || !ok(cudaDeviceSynchronize(), "sync")) break;
    cudaFree(shifted);
    shifted = nullptr;
    if (!ok(cudaMalloc(&dimg, Mc * 8), "malloc")) break;
    std::vector<cufftComplex> padded(Mc);
    for (size_t z = 0; z < nz; ++z)
      for (size_t y = 0; y < ny; ++y)
        std::memcpy(&padded[(z * ny + y) * nxh], im + (z * ny + y) * nx, nx * 4);
    if (!ok(cudaMemcpy(dimg, padded.data(), Mc * 8, cudaMemcpyHostToDevice), "h2d")) break;
    if (!okf(cufftPlan3d(&pf, (int)nz, (int)ny, (int)nx, CUFFT_R2C), "plan r2c")) break;
    if (!okf(cufftExecR2C(pf, (cufftReal*)dimg, dimg), "exec r2c")) break;
    if (!okf(cufftExecR2C(pf, (cufftReal*)kpad, kpad), "exec r2c")) break;
    launch_modulate(dimg, kpad, (long long)Mc, 1.0f / (float)N, 0);
    if (!ok(cudaGetLastError(), "modulate")) break;
    cufftDestroy(pf);
    pf = 0;
    cudaFree(kpad);
    kpad = nullptr;
    if (!okf(cufftPlan3d(&pi, (int)nz, (int)ny, (int)nx, CUFFT_C2R), "plan c2r")) break;
    if (!okf(cufftExecC2R(pi, dimg, (cufftReal*)dimg), "exec c2r")) break;
    if (!ok(cudaMemcpy(padded.data(), dimg, Mc * 8, cudaMemcpyDeviceToHost), "d2h")) break;
    for (size_t z = 0; z < nz; ++z)
      for (size_t y = 0; y < ny; ++y)
        std::memcpy(im + (z * ny + y) * nx, &padded[(z * ny + y) * nxh], nx * 4);
  } while (0);
  if (pf) cufftDestroy(pf);
  if (pi) cufftDestroy(pi);
  cudaFree(shifted);
  cudaFree(dker);
  cudaFree(kpad);
  cudaFree(dimg);
  rc = g_err;
  return rc;
}

// Device-only sequence with pre-built plans (created on first use per shape).
// d_img, d_ker: Mc complex each in the R2C in-place padded layout; the result
// overwrites d_img (real rows with pitch 2*(nx/2+1) floats).
struct RsPlans {
  int nx = 0, ny = 0, nz = 0;
  cufftHandle f = 0, i = 0;
};
static RsPlans g_plans;

RS_EXPORT int refseq_device_only(float* d_img, float* d_ker, int nx, int ny, int nz, void* stream) {
  g_err = 0;
  cudaStream_t st = (cudaStream_t)stream;
  if (g_plans.nx != nx || g_plans.ny != ny || g_plans.nz != nz) {
    if (g_plans.f) cufftDestroy(g_plans.f);
    if (g_plans.i) cufftDestroy(g_plans.i);
    g_plans = RsPlans();
    if (!okf(cufftPlan3d(&g_plans.f, nz, ny, nx, CUFFT_R2C), "plan r2c")) return g_err;
    if (!okf(cufftPlan3d(&g_plans.i, nz, ny, nx, CUFFT_C2R), "plan c2r")) return g_err;
    g_plans.nx = nx;
    g_plans.ny = ny;
    g_plans.nz = nz;
  }
  cufftSetStream(g_plans.f, st);
  cufftSetStream(g_plans.i, st);
  const long long Mc = (long long)(nx / 2 + 1) * ny * nz;
  if (!okf(cufftExecR2C(g_plans.f, (cufftReal*)d_img, (cufftComplex*)d_img), "exec r2c")) return g_err;
  if (!okf(cufftExecR2C(g_plans.f, (cufftReal*)d_ker, (cufftComplex*)d_ker), "exec r2c")) return g_err;
  launch_modulate((cufftComplex*)d_img, (const cufftComplex*)d_ker, Mc, 1.0f / (float)((long long)nx * ny * nz), st);
  if (!ok(cudaGetLastError(), "modulate")) return g_err;
  if (!okf(cufftExecC2R(g_plans.i, (cufftComplex*)d_img, (cufftReal*)d_img), "exec c2r")) return g_err;
  return 0;
}

RS_EXPORT void refseq_release() {
  if (g_plans.f) cufftDestroy(g_plans.f);
  if (g_plans.i) cufftDestroy(g_plans.i);
  g_plans = RsPlans();
}
