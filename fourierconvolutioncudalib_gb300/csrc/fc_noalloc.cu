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
// The array belongs to this file's module.  With CUDA's lazy module loading
// (the default since CUDA 12.2) the driver loads the module, and reserves the
// array on the device, when the first call on that device asks for the
// array's address; from then on the array is held until the process exits.
// That first call should therefore come at start-up, before a memory pool
// takes the device's memory and before any stream capture.  In host code the
// array's name is only a host-side stand-in: the device address is looked up
// with cudaGetSymbolAddress, with the device current, once per device and
// CUDA context (the set-up of the first call there), and cached under the
// context's unique id, so that a context that was destroyed (cudaDeviceReset)
// and created again gets its own lookup rather than a stale address.  All
// calls share the array and it keeps the previous call's contents; the passes
// overwrite every scratch byte they read, except the reference-placement
// buffer, which is cleared on the stream before use.  Calls whose executions
// overlap on the GPU (different streams, or different host threads on the
// same device) race on the array and must be serialised by the caller.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "../../include/convolution3Dfft.h"
#include "fc_internal.h"

static __device__ __align__(256) unsigned char g_fc_noalloc_scratch[FC_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_scratch_mu;
std::map<std::pair<int, unsigned long long>, void*> g_scratch_addr;  // (device, context id) -> address

// unique id of the current thread's CUDA context (the runtime has made the
// device's primary context current); false if the driver cannot say
bool current_context_id(unsigned long long* id) {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(fn);
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(fn);
    cudaGetLastError();
  });
  CUcontext ctx = nullptr;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}
}  // namespace

extern "C" int fc_conv3d_device_noalloc(const float* d_image, float* d_out, const int* imDim, const float* d_kernel,
                                        const int* kernelDim, int flags, void* stream) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
    cudaGetLastError();
    fc::record_status(FC_ERR_CUDA, "fc_conv3d_device_noalloc: no usable current device");
    return FC_ERR_CUDA;
  }
  unsigned long long ctx_id = 0;
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    auto it = current_context_id(&ctx_id) ? g_scratch_addr.find({dev, ctx_id}) : g_scratch_addr.end();
    if (it != g_scratch_addr.end()) {
      scratch = it->second;
    } else {
      // set-up on this device and context (the lookup also makes the runtime
      // create the device's primary context, if this is its first CUDA call)
      const cudaError_t e = cudaGetSymbolAddress(&scratch, g_fc_noalloc_scratch);
      if (e != cudaSuccess || !scratch) {
        cudaGetLastError();
        const std::string msg = std::string("fc_conv3d_device_noalloc: cudaGetSymbolAddress of the static "
                                             "scratch failed: ") + cudaGetErrorString(e);
        fc::record_status(FC_ERR_CUDA, msg.c_str());
        return FC_ERR_CUDA;
      }
      // without a context id the address is looked up again on the next call
      if (current_context_id(&ctx_id)) g_scratch_addr[{dev, ctx_id}] = scratch;
    }
  }
  return fc::conv_in_scratch(d_image, d_out, imDim, d_kernel, kernelDim, flags, (char*)scratch,
                             (size_t)FC_NOALLOC_SCRATCH_BYTES, (cudaStream_t)stream);
}
