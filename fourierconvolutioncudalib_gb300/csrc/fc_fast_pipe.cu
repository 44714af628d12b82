// Pipelined x passes (R2C of dense real rows, C2R of half-spectrum rows).
//
// Persistent CTAs walk the row tiles with a stride of the grid size.  A tile
// (2*LPB consecutive rows) is one contiguous block of global memory, so one
// elected thread brings it into shared memory with a single bulk asynchronous
// copy (TMA, cp.async.bulk) completing on an mbarrier.  The copy of the CTA's
// next tile is issued as soon as the current tile's values are in registers,
// so it lands while the CTA transforms and stores the current tile.  The
// transform itself is the register-resident engine of fc_fast_rows.cuh.
#include <atomic>
#include <cstdlib>

#include "fc_async.cuh"
#include "fc_fast_rows.cuh"

namespace fc {
namespace fast {

// bounded mbarrier waits that gave up (read and cleared by the host)
__device__ unsigned int g_pipe_timeouts;

template <int N>
struct PipeRows {
  using G = RowGeom<N>;
  static constexpr int ROWS = 2 * G::LPB;
  static constexpr int XBYTES = ((G::SMEM * (int)sizeof(float2) + 127) / 128) * 128;  // exchange area
};

// rows of the tile in shared memory: element x of global row r is b[(r - row0) * pitch + x]
template <class T>
struct TileRows {
  const T* b;
  long long row0;
  int pitch;
  __device__ __forceinline__ T load(long long row, int x) const { return b[(int)(row - row0) * pitch + x]; }
};

template <int N, bool C2R>
__global__ void __launch_bounds__(RowGeom<N>::THREADS, 3) k_rows_pipe(const char* __restrict__ in, long long in_pitch,
                                                                   void* __restrict__ out, long long out_pitch,
                                                                   long long nrows, const float2* __restrict__ W) {
  using P = PipeRows<N>;
  extern __shared__ __align__(128) unsigned char dsm[];
  __shared__ uint64_t bar;
  float2* sm = reinterpret_cast<float2*>(dsm);
  unsigned char* buf = dsm + P::XBYTES;
  const int tid = (int)threadIdx.x;
  const long long ntiles = RowGeom<N>::tiles(nrows);
  const long long row_bytes = in_pitch * (C2R ? (long long)sizeof(float2) : (long long)sizeof(float));
  const bool skip = async::copies_skipped();  // read once: a global load per tile would delay warp 0
  async::pdl_trigger_at_start<async::kPdlX>();
  if (tid == 0) {
    async::bar_init(&bar, 1);
    async::bar_init_fence();
  }
  __syncthreads();
  async::pdl_wait();  // the previous pass's output is complete and visible
  long long tile = blockIdx.x;
  auto issue = [&](long long tl) {
    const long long r0 = tl * P::ROWS;
    const long long nr = (nrows - r0) < P::ROWS ? (nrows - r0) : P::ROWS;
    const uint32_t bytes = (uint32_t)(nr * row_bytes);
    async::bar_expect(&bar, bytes);
    if (!skip) async::bulk_load(buf, in + r0 * row_bytes, bytes, &bar);
  };
  if (tid == 0 && tile < ntiles) issue(tile);
  uint32_t phase = 0;
  bool signalled = false;  // the successor may launch (programmatic dependent launch)
  for (; tile < ntiles; tile += gridDim.x) {
    signalled |= async::pdl_trigger_last_tile<async::kPdlX>(tile + gridDim.x >= ntiles);
    const bool ok = async::bar_wait(&bar, phase);
    if (!__syncthreads_and(ok)) {
      if (tid == 0) atomicAdd(&g_pipe_timeouts, 1u);
      break;
    }
    phase ^= 1u;
    const RowSlot<N> s(tile, tid, nrows);
    float2 v[kVals];
    if constexpr (C2R)
      load_c2r<N, TileRows<float2>, false>(
          v, TileRows<float2>{reinterpret_cast<const float2*>(buf), tile * P::ROWS, (int)in_pitch}, s);
    else
      load_r2c<N>(v, TileRows<float>{reinterpret_cast<const float*>(buf), tile * P::ROWS, (int)in_pitch}, s);
    __syncthreads();  // every thread's reads of the buffer are done
    if (tid == 0 && tile + gridDim.x < ntiles) {
      async::proxy_fence();
      issue(tile + gridDim.x);
    }
    if constexpr (C2R)
      finish_c2r<N, tc::kNone, false>(v, s, reinterpret_cast<float*>(out), out_pitch, W, sm);
    else
      finish_r2c<N>(v, s, reinterpret_cast<float2*>(out), out_pitch, W, sm);
  }
  async::pdl_trigger_at_end<async::kPdlX>(signalled);
}

template <int N, bool C2R>
static cudaError_t run_rows_pipe(const void* in, long long in_pitch, void* out, long long out_pitch, long long nrows,
                                 const float2* W, cudaStream_t st) {
  using P = PipeRows<N>;
  using G = RowGeom<N>;
  const size_t buf_bytes = (size_t)P::ROWS * in_pitch * (C2R ? sizeof(float2) : sizeof(float));
  const size_t smem = P::XBYTES + buf_bytes;
  auto kern = k_rows_pipe<N, C2R>;
  // (dynamic bytes << 8 | resident CTAs per SM) of the last launch configuration
  static std::atomic<long long> s_occ{0};
  long long cached = s_occ.load(std::memory_order_relaxed);
  int occ = (cached >> 8) == (long long)smem ? (int)(cached & 255) : 0;
  if (occ == 0) {
    if (smem > 48 * 1024) {
      const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, G::THREADS, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorNotSupported;
    s_occ.store(((long long)smem << 8) | (occ & 255), std::memory_order_relaxed);
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long ntiles = G::tiles(nrows);
  const long long grid = std::min<long long>(ntiles, (long long)occ * sms);
  return async::launch_pdl(async::kPdlX, kern, (unsigned)grid, G::THREADS, smem, st, reinterpret_cast<const char*>(in),
                           in_pitch, out, out_pitch, nrows, W);
}

}  // namespace fast

// in: 16-byte aligned, rows of in_pitch elements contiguous (checked by the caller)
cudaError_t pipe_x_r2c_dense(const float* in, long long in_pitch, float2* out, long long out_pitch, long long nrows,
                             const FcAxis& ax, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  switch (ax.n) {
#define FC_CASE(n_) \
  case n_:          \
    return fast::run_rows_pipe<n_, false>(in, in_pitch, out, out_pitch, nrows, ax.W, st);
    FC_ROW_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

cudaError_t pipe_x_c2r(const float2* in, long long in_pitch, float* out, long long out_pitch, long long nrows,
                       const FcAxis& ax, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  switch (ax.n) {
#define FC_CASE(n_) \
  case n_:          \
    return fast::run_rows_pipe<n_, true>(in, in_pitch, out, out_pitch, nrows, ax.W, st);
    FC_ROW_SIZES(FC_CASE)
#undef FC_CASE
    default:
      return cudaErrorNotSupported;
  }
}

cudaError_t pipe_timeouts_addr(unsigned int** p) { return cudaGetSymbolAddress((void**)p, fast::g_pipe_timeouts); }

cudaError_t pipe_timeouts_read_async(unsigned int* dst, cudaStream_t st) {
  return cudaMemcpyFromSymbolAsync(dst, fast::g_pipe_timeouts, sizeof(unsigned int), 0, cudaMemcpyDeviceToHost, st);
}

void pipe_timeouts_clear() {
  const unsigned int zero = 0;
  cudaMemcpyToSymbol(fast::g_pipe_timeouts, &zero, sizeof(zero));
}

cudaError_t pipe_wait_ctl_set(long long limit, int skip_copies) { return async::wait_ctl_set_tu(limit, skip_copies); }

namespace async {
bool pdl_enabled(int kind) {
  // FC_PDL: a mask of kPdlX | kPdlY | kPdlZ (0: none); default FC_PDL_DEFAULT
  static const int mask = [] {
    const char* e = std::getenv("FC_PDL");
    return e ? std::atoi(e) : FC_PDL_DEFAULT;
  }();
  return (mask & kind) != 0;
}
}  // namespace async

}  // namespace fc
