// Allocation-free convolution entry point.
//
// Some callers cannot allocate device memory at the time they convolve: a
// host application whose framework has already reserved the GPU's memory in
// its own caching pool, a real-time acquisition loop that cannot afford
// cudaMalloc's implicit synchronisation, or a deployment that forbids dynamic
// device allocation after start-up.  For them, fc_conv3d_device_noalloc runs
// the plain fp32 convolution with every byte of scratch (the twiddle tables
// and the spectrum workspace) taken from one file-scope __device__ array of
// FC_NOALLOC_SCRATCH_BYTES.  It calls no cudaMalloc, cudaFree or allocating
// library routine; the caller still provides the image, kernel and output.
//
// The array exists once per device in every process that loads the library
// and is held until the process exits.  In host code its name is only a
// host-side stand-in: the device address is obtained once per device, with
// that device current, by cudaGetSymbolAddress on the first call made on
// that device (so that first call should come before any stream capture).
// All calls share the array and it keeps the previous call's contents; the
// passes overwrite every scratch byte they read, except the reference-
// placement buffer, which is cleared on the stream before use.  Calls whose
// executions overlap on the GPU (different streams, or different host
// threads on the same device) race on the array and must be serialised by
// the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/convolution3Dfft.h"
#include "fc_internal.h"

static __device__ __align__(256) unsigned char g_fc_noalloc_scratch[FC_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;
}  // namespace

extern "C" int fc_conv3d_device_noalloc(const float* d_image, float* d_out, const int* imDim, const float* d_kernel,
                                        const int* kernelDim, int flags, void* stream) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    fc::record_status(FC_ERR_CUDA, "fc_conv3d_device_noalloc: no usable current device");
    return FC_ERR_CUDA;
  }
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_fc_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        fc::record_status(FC_ERR_CUDA, "fc_conv3d_device_noalloc: cudaGetSymbolAddress of the static scratch failed");
        return FC_ERR_CUDA;
      }
      g_scratch_addr[dev] = p;
    }
    scratch = g_scratch_addr[dev];
  }
  return fc::conv_in_scratch(d_image, d_out, imDim, d_kernel, kernelDim, flags, (char*)scratch,
                             (size_t)FC_NOALLOC_SCRATCH_BYTES, (cudaStream_t)stream);
}
