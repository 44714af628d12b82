// Bulk asynchronous copies (TMA, cp.async.bulk) into shared memory with
// mbarrier completion, for the pipelined pass kernels (sm_90 and later PTX).
//
// One elected thread arms the barrier with the byte count and issues the
// copy; every thread waits on the barrier's phase.  Waits are bounded: after
// about a second of clock cycles the wait gives up and returns false, and the
// caller records the timeout and leaves its loop instead of hanging the GPU.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fc {
namespace async {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// make the initialised barrier visible to the async proxy (before the CTA barrier that follows)
__device__ __forceinline__ void bar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// order this thread's earlier generic-proxy shared-memory accesses before later async-proxy ones
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// arm the barrier for one arrival carrying `bytes` of transaction count
__device__ __forceinline__ void bar_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// global -> shared tile copy through a tensor map (TMA, tile mode): the box
// at element coordinates (x, y, z) of a 3-D map.  dst 128-byte aligned; x *
// element size a multiple of 16 bytes; elements outside the map's extents
// arrive as zeros (and count towards the barrier's bytes).
__device__ __forceinline__ void tensor_load_3d(void* dst, const void* tmap, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// shared -> global tile copy through a tensor map (TMA store, bulk-group
// completion): the box at non-negative element coordinates (x, y, z); the
// parts of the box outside the map's extents are not written.  src 128-byte
// aligned and written before a proxy_fence() and a barrier.
__device__ __forceinline__ void tensor_store_3d(const void* tmap, int x, int y, int z, const void* src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(tmap),
               "r"(x), "r"(y), "r"(z), "r"(smem_addr(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the bulk groups this thread committed have read their shared-memory sources
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// ... and their writes are complete
__device__ __forceinline__ void bulk_wait() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ bool bar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

constexpr long long kWaitCycles = 1LL << 31;  // about one second at GB300 clocks

// Control of the bounded waits, one copy per translation unit and device (set
// from the host by wait_ctl_set_tu): the clock-cycle limit of one wait (0:
// kWaitCycles), and a test switch under which the kernels arm their barriers
// for the copies' bytes but issue no copy, so that every wait runs out with
// nothing in flight and the kernel returns its timeout status.
struct WaitCtl {
  long long limit;
  int skip_copies;
};
[[maybe_unused]] static __device__ WaitCtl g_wait_ctl = {0, 0};

__device__ __forceinline__ bool copies_skipped() { return *(volatile int*)&g_wait_ctl.skip_copies != 0; }

// wait for the phase with the given parity to complete; false on timeout
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity) {
  if (bar_try_wait(bar, parity)) return true;
  const long long lim = g_wait_ctl.limit > 0 ? g_wait_ctl.limit : kWaitCycles;
  const long long t0 = clock64();
  while (!bar_try_wait(bar, parity)) {
    if (clock64() - t0 > lim) return false;
  }
  return true;
}

// host: set this translation unit's wait control on the current device
static inline cudaError_t wait_ctl_set_tu(long long limit, int skip_copies) {
  const WaitCtl w{limit, skip_copies ? 1 : 0};
  return cudaMemcpyToSymbol(g_wait_ctl, &w, sizeof(w));
}

// Programmatic dependent launch (sm_90 and later).  A kernel launched with
// launch_pdl may start while the kernel before it on the stream is still
// running: it sets up its shared memory, then waits for its predecessor to
// complete and its memory to be visible (pdl_wait) before it reads anything
// that kernel wrote, and signals when its own successor may launch
// (pdl_launch_dependents).  Both are no-ops for a kernel launched
// without the attribute.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// pass kinds of launch_pdl; FC_PDL is a mask of them (0: none)
constexpr int kPdlX = 1, kPdlY = 2, kPdlZ = 4;

// Where a persistent pass lets its successor launch, per pass kind
// (FC_PDL_TRIGGER_X / _Y / _Z): 2, the default, once the CTA has no tile left
// (pdl_trigger_at_end); 1 when the CTA begins its last tile
// (pdl_trigger_last_tile); 0 at its start (pdl_trigger_at_start).  With the
// trigger at the end, a successor's CTAs take only the SM slots of CTAs that
// are done, and a chain of passes does not launch grids three deep whose
// waiting CTAs hold slots the running pass needs (measured on the chain of five
// passes against a ready kernel spectrum, 512x512x128: 0.308 ms with every
// trigger at the start, 0.263 ms at the end; 1024x1024x256: 2.314 against
// 2.247 ms; the x passes' trigger at the start measured 0.8 % faster at
// 512x512x128 and 2.3 % slower at 1024x1024x256).  Wherever it is, the
// successor's pdl_wait covers this whole grid and its memory.
#ifndef FC_PDL_TRIGGER_X
#define FC_PDL_TRIGGER_X 2
#endif
#ifndef FC_PDL_TRIGGER_Y
#define FC_PDL_TRIGGER_Y 2
#endif
#ifndef FC_PDL_TRIGGER_Z
#define FC_PDL_TRIGGER_Z 2
#endif
template <int KIND>
constexpr int kPdlTrigger = KIND == 1 ? FC_PDL_TRIGGER_X : KIND == 2 ? FC_PDL_TRIGGER_Y : FC_PDL_TRIGGER_Z;
template <int KIND>
__device__ __forceinline__ void pdl_trigger_at_start() {
  if constexpr (kPdlTrigger<KIND> == 0) pdl_launch_dependents();
}
// call at the top of each tile with last = (this is the CTA's last tile);
// true when it signalled
template <int KIND>
__device__ __forceinline__ bool pdl_trigger_last_tile(bool last) {
  if constexpr (kPdlTrigger<KIND> == 1) {
    if (last) {
      pdl_launch_dependents();
      return true;
    }
  }
  return false;
}
// call after the tile loop (also reached by CTAs without tiles and on an
// expired wait), with whether pdl_trigger_last_tile has signalled
template <int KIND>
__device__ __forceinline__ void pdl_trigger_at_end(bool signalled) {
  if constexpr (kPdlTrigger<KIND> != 0) {
    if (!signalled) pdl_launch_dependents();
  }
}

#ifndef FC_PDL_DEFAULT
#define FC_PDL_DEFAULT 7
#endif
// whether kernels of this pass kind launch with programmatic dependent launch
bool pdl_enabled(int kind);

template <class K, class... Args>
static inline cudaError_t launch_pdl(int kind, K kern, unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                                     Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_enabled(kind) ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

// per-thread 16-byte asynchronous copy global -> shared (cp.async, L1 bypass);
// both addresses 16-byte aligned.  Completion: commit(), then wait_all() in the
// issuing thread, then a CTA barrier before other threads read the data.
__device__ __forceinline__ void copy16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

}  // namespace async
}  // namespace fc
