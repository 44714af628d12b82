// Register-resident column-pass kernel templates (lengths in FC_COL_SIZES):
// the y passes, the fused z pass (forward image and kernel columns, the
// reference's modulate-and-normalise, inverse) and the kernel-gradient z
// pass.  Instantiated by fc_fast_cols.cu and fc_fast_zconv.cu.
//
// A CTA owns B adjacent columns (kx) of one plane; thread (c, t) holds up to
// 16 values of column c (positions per the stage split of fc_fast.cuh).
// Global loads and stores are B*8 contiguous bytes per row; shared memory is
// an N x B tile in a padded layout used only for the exchanges between radix
// stages.
#pragma once
#ifndef FC_ZCONV_MIN_BLOCKS
#define FC_ZCONV_MIN_BLOCKS 2
#endif
#include <cuda.h>

#include <algorithm>

#include "fc_async.cuh"
#include "fc_fast.cuh"
#include "fc_fast_sizes.h"
#include "fc_internal.h"
#include "fc_sources.cuh"

namespace fc {
namespace fast {

// columns per tile: the largest power of two <= BMAX with N*B <= VMAX values
// and B*T <= TMAX threads (4 at least)
template <int N, int BMAX = 32, int TMAX = 256, int VMAX = 4096>
struct ColGeomB {
  static constexpr int T = Plan<N>::T;
  static constexpr int B0a = VMAX / N, B0b = TMAX / T;
  static constexpr int B0 = (B0a < B0b ? B0a : B0b) < BMAX ? (B0a < B0b ? B0a : B0b) : BMAX;
  static constexpr int B = B0 >= 32 ? 32 : B0 >= 16 ? 16 : B0 >= 8 ? 8 : 4;
  static constexpr int THREADS = B * T;
  static constexpr int SMEM = N * B + (N * B) / 16;  // float2 elements of the exchange tile
};
template <int N>
using ColGeom = ColGeomB<N, 32>;
// wide tiles for the image y passes: up to 512 threads and 8192 values, so that
// long columns still read rows of 8-16 columns (64-128 contiguous bytes);
// the exchange tile then needs dynamic shared memory
template <int N>
using ColGeomWide = ColGeomB<N, 32, 512, 8192>;

// rows per tensor-map box of a column of N values: the largest divisor of N of
// at most 256 (a box dimension is at most 256, and equal boxes cover N exactly)
constexpr int zbox_rows(int n) {
  int nb = (n + 255) / 256;
  while (n % nb) ++nb;
  return n / nb;
}

// y pass body: tile (bx, plane) = columns [bx*B, bx*B + B) of one plane.
// REV: radix order of the transform (a standalone pass may run the inverse in
// the forward order, which exchanges with fewer shared-memory bank conflicts)
template <int N, bool INV, class Src, int TCM = tc::kNone, class G = ColGeom<N>, bool REV = INV>
__device__ __forceinline__ void body_cols(const Src& src, float2* dst, long long ps, long long es, int ncols,
                                          const float2* __restrict__ W, int bx, int plane, int tid, float2* sm,
                                          const TcCtx& tcx = TcCtx{nullptr}) {
  constexpr int B = G::B;
  constexpr int R0 = first_radix<N, REV>(), RF = last_radix<N, REV>();
  const int c = tid % B;
  const int t = tid / B;  // >= T for threads beyond the tile: they own no butterfly
  const int col = bx * B + c;
  const bool ok = col < ncols && t < G::T;
  float2 v[kVals];
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int j = stage_pos<N, R0>(t, q);
    v[q] = (ok && j >= 0) ? src.load(plane, j, col) : make_float2(0.f, 0.f);
  }
  fft<N, INV, TCM, REV>(v, ColLay<B>{sm, c}, t, W, tcx);
  if (ok) {
    float2* d = dst + (long long)plane * ps + col;
#pragma unroll
    for (int q = 0; q < kVals; ++q) {
      const int j = stage_pos<N, RF>(t, q);
      if (j >= 0) d[(long long)j * es] = v[q];
    }
  }
}

// y pass on wide tiles (dynamic shared memory of ColGeomWide<N>::SMEM float2)
template <int N, bool INV, class Src>
__global__ void __launch_bounds__(ColGeomWide<N>::THREADS, 1024 / ColGeomWide<N>::THREADS)
    k_cols_wide(Src src, float2* dst, long long ps, long long es, int ncols, const float2* __restrict__ W) {
  extern __shared__ __align__(16) float2 wsm[];
  body_cols<N, INV, Src, tc::kNone, ColGeomWide<N>, false>(src, dst, ps, es, ncols, W, (int)blockIdx.x,
                                                           (int)blockIdx.y, (int)threadIdx.x, wsm);
}

template <int N, bool INV, class Src>
__global__ void __launch_bounds__(ColGeom<N>::THREADS) k_cols(Src src, float2* dst, long long ps, long long es,
                                                              int ncols, const float2* __restrict__ W) {
  __shared__ float2 sm[ColGeom<N>::SMEM];
  body_cols<N, INV, Src, tc::kNone, ColGeom<N>, false>(src, dst, ps, es, ncols, W, (int)blockIdx.x, (int)blockIdx.y,
                                                      (int)threadIdx.x, sm);
}

// ---------------------------------------------------------------------------
// Persistent in-place y pass on tensor-map tiles (default for power-of-two lengths >= 512).  The
// spectrum S is [nz][ny][pitch]; a tile is B adjacent columns of one plane,
// all N = ny rows.  Each CTA walks the tiles with a stride of the grid size; a
// tile arrives in shared memory (ISTAGE, rows of B columns) by tensor-map
// copies of YBOX rows each, and the copy of the CTA's next tile is issued as
// soon as every thread has read the current one into registers, so it lands
// behind the current tile's transform and stores.  The stage tables of the
// radix chain sit in shared memory.  Every box starts 128-byte aligned
// (lengths that fail it keep k_cols); waits are bounded as in the fused z
// pass.
// tiles written back by tensor-map stores staged in shared memory (bit 0: the
// persistent y pass, bit 1: the persistent fused z pass) instead of per-thread
// global stores; 0 for comparison builds
#ifndef FC_STORE_TMA
#define FC_STORE_TMA 3
#endif
// the persistent fused z pass leaves out a transform's closing barrier where a
// CTA barrier follows before the exchange area is written again (0 for comparison builds)
#ifndef FC_TAIL_SKIP
#define FC_TAIL_SKIP 1
#endif
// the fused z pass issues the next image copy together with the next kernel copy (0 for comparison builds)
#ifndef FC_ZIMG_LATE
#define FC_ZIMG_LATE 1
#endif
// the fused z pass takes the last spectrum column in 8-row tiles (0 for comparison builds)
#ifndef FC_ZNYQ
#define FC_ZNYQ 1
#endif

template <int N>
struct YPipe {
  using G = ColGeom<N>;
  static constexpr int B = G::B;
  static constexpr int THREADS = G::THREADS;
  static constexpr int XCH_BYTES = ((G::SMEM * (int)sizeof(float2) + 127) / 128) * 128;
  static constexpr int YBOX = zbox_rows(N);
  static constexpr int NBOX = N / YBOX;
  static constexpr int IBYTES = N * B * (int)sizeof(float2);
  static constexpr int ISTAGE_OFF = XCH_BYTES;
  static constexpr int TWN = Plan<N>::tab_size(false);
  static constexpr int TW_OFF = ISTAGE_OFF + ((IBYTES + 127) / 128) * 128;
  static constexpr int BAR_OFF = TW_OFF + ((TWN * (int)sizeof(float2) + 127) / 128) * 128;
  static constexpr int SMEM_BYTES = BAR_OFF + 128;
  static_assert(YBOX <= 256 && YBOX * NBOX == N, "boxes must tile the column");
  static constexpr bool OK = (YBOX * B * (int)sizeof(float2)) % 128 == 0 && (B * (int)sizeof(float2)) % 16 == 0 &&
                             SMEM_BYTES <= 227 * 1024;
};

// expired waits of the persistent y pass (per translation unit)
[[maybe_unused]] static __device__ unsigned int g_ypipe_timeouts;

template <int N, bool INV>
__global__ void __launch_bounds__(YPipe<N>::THREADS) k_cols_pipe(float2* __restrict__ S, long long ps, long long es,
                                                                  int ncols, int nplanes, const float2* __restrict__ W,
                                                                  const __grid_constant__ CUtensorMap map) {
  using P = YPipe<N>;
  constexpr int B = P::B;
  constexpr int R0 = first_radix<N, false>(), RF = last_radix<N, false>();
  // rows of 64 bytes or more: the tensor store measured faster than the
  // per-thread stores for 512-long columns (8-column tiles) and slower for
  // 1024-long ones (4-column tiles, 32-byte rows)
  constexpr bool kStore = (FC_STORE_TMA & 1) != 0 && B * (int)sizeof(float2) >= 64;
  extern __shared__ __align__(128) unsigned char ypsm[];
  float2* xch = reinterpret_cast<float2*>(ypsm);
  float2* ist = reinterpret_cast<float2*>(ypsm + P::ISTAGE_OFF);
  float2* tws = reinterpret_cast<float2*>(ypsm + P::TW_OFF);
  uint64_t* bar = reinterpret_cast<uint64_t*>(ypsm + P::BAR_OFF);
  const int tid = (int)threadIdx.x;
  const int c = tid % B;
  const int t = tid / B;
  const int ntx = (ncols + B - 1) / B;
  const int ntiles = ntx * nplanes;  // tile counts fit an int for every supported shape
  const bool skip = async::copies_skipped();
  async::pdl_trigger_at_start<async::kPdlY>();
  auto issue = [&](int ti) {
    const int bx = ti % ntx, plane = ti / ntx;
    async::bar_expect(bar, (unsigned)P::IBYTES);
    if (!skip)
#pragma unroll
      for (int b = 0; b < P::NBOX; ++b)
        async::tensor_load_3d(ist + b * P::YBOX * B, &map, bx * B, b * P::YBOX, plane, bar);
  };
  copy_stage_tables<N, false>(tws, W, tid, P::THREADS);  // the twiddle tables are not written by any pass
  if (tid == 0) {
    async::bar_init(bar, 1);
    async::bar_init_fence();
  }
  __syncthreads();
  async::pdl_wait();  // the previous pass's output is complete and visible
  int ti = (int)blockIdx.x;
  if (tid == 0 && ti < ntiles) issue(ti);
  bool pend = ti < ntiles;
  bool expired = false;
  uint32_t ph = 0;
  const ColLay<B> lay{xch, c};
  bool signalled = false;  // the successor may launch (programmatic dependent launch)
  for (; ti < ntiles; ti += (int)gridDim.x, ph ^= 1u) {
    signalled |= async::pdl_trigger_last_tile<async::kPdlY>(ti + (int)gridDim.x >= ntiles);
    const int plane = ti / ntx;
    const int col = (ti % ntx) * B + c;
    const bool ok = col < ncols && t < P::G::T;
    float2 v[kVals];
    if (!__syncthreads_and(async::bar_wait(bar, ph))) {
      expired = true;
      break;
    }
    pend = false;
#pragma unroll
    for (int q = 0; q < kVals; ++q) {
      const int j = stage_pos<N, R0>(t, q);
      v[q] = (ok && j >= 0) ? ist[j * B + c] : make_float2(0.f, 0.f);
    }
    async::proxy_fence();
    if (kStore && tid == 0) async::bulk_wait_read();  // the previous tile's store has read XCH
    __syncthreads();  // every thread has read ISTAGE (and XCH is free)
    if (ti + (int)gridDim.x < ntiles) {
      if (tid == 0) issue(ti + (int)gridDim.x);
      pend = true;
    }
    // the closing barrier stays: the staged stores write the exchange area
    // next, and without it the per-thread stores of 1024-long columns
    // measured 8-13 % slower (1024x1024x256)
    fft<N, INV, tc::kNone, false, true>(v, lay, t, tws);
    if constexpr (kStore) {
      // the tile as rows of B columns in XCH (the transform's last exchange
      // has been read), then one tensor store per box; the store leaves out
      // the columns past ncols
#pragma unroll
      for (int q = 0; q < kVals; ++q) {
        const int j = stage_pos<N, RF>(t, q);
        if (j >= 0) xch[j * B + c] = v[q];
      }
      async::proxy_fence();
      __syncthreads();
      if (tid == 0) {
        const int bx = ti % ntx;
#pragma unroll
        for (int b = 0; b < P::NBOX; ++b)
          async::tensor_store_3d(&map, bx * B, b * P::YBOX, plane, xch + b * P::YBOX * B);
        async::bulk_commit();
      }
    } else if (ok) {
      float2* d = S + (long long)plane * ps + col;
#pragma unroll
      for (int q = 0; q < kVals; ++q) {
        const int j = stage_pos<N, RF>(t, q);
        if (j >= 0) d[(long long)j * es] = v[q];
      }
    }
  }
  async::pdl_trigger_at_end<async::kPdlY>(signalled);
  if (expired) {
    if (tid == 0) atomicAdd(&g_ypipe_timeouts, 1u);
    if (pend) (void)async::bar_wait(bar, ph);
  }
  if (kStore && tid == 0) async::bulk_wait();  // the tile stores are complete before the CTA ends
}

// Host: encode a 3-D tensor map of a spectrum of ncols columns (row pitch
// `pitch` float2), ny rows and nz planes, box bx x by x bz elements of 8
// bytes; false when the driver entry point is missing or a rule is broken.
bool tile_tensor_map(CUtensorMap* map, const float2* S, long long pitch, int ny, int ncols, int nz, int bx, int by,
                     int bz);
// Whether the persistent tensor-map y pass runs for columns of length n: by
// default for power-of-two lengths from 512 (the one-tile-per-CTA pass is
// faster below); FC_YPIPE=0 never, FC_YPIPE=1 wherever its geometry applies
bool ypipe_selected(int n);

// Host: launch the persistent in-place y pass when selected and its geometry applies (sets *used)
template <int N, bool INV>
static cudaError_t cols_pipe_launch(float2* S, long long ps, long long es, int ncols, int nplanes, const float2* W,
                                    cudaStream_t st, bool* used) {
  using P = YPipe<N>;
  *used = false;
  if constexpr (!P::OK) {
    return cudaSuccess;
  } else {
    if (!ypipe_selected(N) || ncols < 1 || nplanes < 1 || ps != es * N) return cudaSuccess;
    CUtensorMap map;
    if (!tile_tensor_map(&map, S, es, N, ncols, nplanes, P::B, P::YBOX, 1)) return cudaSuccess;
    auto kern = k_cols_pipe<N, INV>;
    static int s_occ = 0;  // resident CTAs per SM of this instantiation (a benign race: same value)
    int occ = s_occ;
    if (occ == 0) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM_BYTES);
      if (e != cudaSuccess) return e;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, P::THREADS, P::SMEM_BYTES);
      if (e != cudaSuccess) return e;
      if (occ < 1) return cudaSuccess;
      s_occ = occ;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long ntiles = (long long)((ncols + P::B - 1) / P::B) * nplanes;
    const long long grid = std::min<long long>(ntiles, (long long)occ * sms);
    *used = true;
    return async::launch_pdl(async::kPdlY, kern, (unsigned)grid, P::THREADS, P::SMEM_BYTES, st, S, ps, es, ncols,
                             nplanes, W, map);
  }
}

// Fused z pass.  Kernel plane p of KXY holds z = (p - hz) mod nz.  The
// kernel column is transformed first and parked in a per-thread private
// shared-memory stash (stash[q*nstash + tid], no barrier needed), so only one
// column's values are live in registers during the image transform.  With a
// stage buffer, the image tile (N rows of B columns) is copied into shared
// memory asynchronously at the start, while the kernel column is loaded and
// transformed.
//
// The single-volume kernel uses tiles of at most 16 columns: the spectrum has
// nx/2+1 columns, and narrower tiles waste less work on the ragged last tile.
template <int N>
using ZTile = ColGeomB<N, 16>;
// radix order of the fused z pass: its forward transforms run the reversed
// chain and its inverse the forward chain (either pairing hands the spectrum
// over in registers; this one measured 0.4-2 % faster on GB300)
constexpr bool kZRev = true;
template <int N>
struct ZGeom {
  // exchange tile, stash, image stage buffer, mbarrier (float2 elements); the
  // stash starts on a 16-byte boundary (the exchange tile has N*B + N*B/16
  // entries, odd for some lengths), and the stage buffer, the target of the
  // tensor-map copy (or of the 16-byte cp.async copies), on a 128-byte one
  static constexpr int XCH = (ZTile<N>::SMEM + 1) & ~1;
  static constexpr int STAGE_OFF = (XCH + ZTile<N>::THREADS * kVals + 15) & ~15;
  static constexpr int STAGE = N * ZTile<N>::B;
  static constexpr int BAR_OFF = STAGE_OFF + STAGE;
  static constexpr int SMEM_BYTES = (BAR_OFF + 2) * (int)sizeof(float2);
  static constexpr int ZBOX = zbox_rows(N);
  static constexpr int NBOX = N / ZBOX;
  static constexpr unsigned STAGE_BYTES = (unsigned)STAGE * sizeof(float2);
  static_assert(ZBOX <= 256 && ZBOX * NBOX == N, "tensor-map boxes must tile the column");
  // the tensor-map stage is used for one box of 16 columns (z lengths up to
  // 256); a stage of two 8-column boxes (z = 500) raised a GPU exception on its
  // first run, with no cause found in its addresses, sizes or barrier count,
  // so longer columns keep the cp.async stage
  static constexpr bool TMA_OK = NBOX == 1 && ZTile<N>::B == 16;
  static_assert(ZTile<N>::B * sizeof(float2) % 16 == 0, "box rows must be multiples of 16 bytes");
  // resident CTAs requested from the register allocator (256 threads: 2 -> <= 128 registers)
  static constexpr int MIN_BLOCKS =
      ZTile<N>::THREADS <= 256 ? FC_ZCONV_MIN_BLOCKS * (256 / ZTile<N>::THREADS) : 1;
};

// expired waits of the fused z pass's tensor-map stage (one count per
// translation unit that instantiates k_zconv)
static __device__ unsigned int g_zstage_timeouts;

// fused z pass body: tile (bx, ky); stash holds nstash >= THREADS slots per value index;
// stage (optional) holds N*B float2 for the prefetched image tile.  With
// `bar`, the stage was filled by a tensor-map copy on that mbarrier (issued by
// the caller); the wait is bounded and a timeout ends the tile (counted in
// g_zstage_timeouts).  Without it the body stages the tile with cp.async.
template <int N, bool CONJ, int TCM = tc::kNone, class G = ColGeom<N>>
__device__ __forceinline__ void body_zconv(float2* __restrict__ S, const float2* __restrict__ KXY, long long pitch,
                                           int ny, int ncols, int kplanes, int hz, float scale,
                                           const float2* __restrict__ W, int bx, int ky, int tid, float2* sm,
                                           float2* stash, int nstash, const TcCtx& tcx = TcCtx{nullptr},
                                           float2* stage = nullptr, uint64_t* bar = nullptr) {
  constexpr int B = G::B;
  constexpr int R0 = first_radix<N, kZRev>(), RF = last_radix<N, !kZRev>();
  const int c = tid % B;
  const int t = tid / B;
  const int col0 = bx * B;
  const int col = col0 + c;
  const bool ok = col < ncols && t < G::T;
  const long long zs = (long long)ny * pitch;
  float2* base = S + (long long)ky * pitch + col;
  if (stage && !bar) {
    // 16-byte pieces (two columns) of the N x B image tile; pieces starting at
    // or beyond ncols are skipped (the row pitch covers the second column)
    const float2* src0 = S + (long long)ky * pitch + col0;
    for (int e = tid; e < N * (B / 2); e += G::THREADS) {
      const int z = e / (B / 2), part = e - z * (B / 2);
      if (col0 + 2 * part < ncols) async::copy16(stage + z * B + 2 * part, src0 + z * zs + 2 * part);
    }
    async::commit();
  }
  const ColLay<B> lay{sm, c};
  float2 v[kVals];
  const float2* kbase = KXY + (long long)ky * pitch + col;
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int z = stage_pos<N, R0>(t, q);
    int p = z + hz;
    if (p >= N) p -= N;
    v[q] = (ok && z >= 0 && p < kplanes) ? kbase[p * zs] : make_float2(0.f, 0.f);
  }
  fft<N, false, TCM, kZRev>(v, lay, t, W, tcx);
#pragma unroll
  for (int q = 0; q < kVals; ++q) stash[q * nstash + tid] = v[q];
  if (bar) {
    const bool ready = async::bar_wait(bar, 0);
    if (!__syncthreads_and(ready)) {
      if (tid == 0) atomicAdd(&g_zstage_timeouts, 1u);
      return;
    }
  } else if (stage) {
    async::wait_all();
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int z = stage_pos<N, R0>(t, q);
    if (stage)
      v[q] = (ok && z >= 0) ? stage[z * B + c] : make_float2(0.f, 0.f);
    else
      v[q] = (ok && z >= 0) ? base[z * zs] : make_float2(0.f, 0.f);
  }
  fft<N, false, TCM, kZRev>(v, lay, t, W, tcx);
  // the forward outputs sit where the inverse's first stage reads them
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    float2 a = stash[q * nstash + tid];  // kernel spectrum (d_Src of modulateAndNormalize_kernel)
    const float2 b = v[q];               // image spectrum  (d_Dst)
    if (CONJ) a.y = -a.y;
    v[q] = make_float2(scale * (a.x * b.x - a.y * b.y), scale * (a.y * b.x + a.x * b.y));
  }
  fft<N, true, TCM, !kZRev>(v, lay, t, W, tcx);
  if (ok) {
#pragma unroll
    for (int q = 0; q < kVals; ++q) {
      const int z = stage_pos<N, RF>(t, q);
      if (z >= 0) base[(long long)z * zs] = v[q];
    }
  }
}

// tmap: the spectrum as a 3-D tensor map (x: ncols columns, y: ny rows, z: N
// planes; 8-byte elements, box B x 1 x N) when use_tma and ZGeom::TMA_OK,
// else the image tile is staged with cp.async.  A stage that is not 128-byte
// aligned also takes the cp.async path.
template <int N, bool CONJ>
__global__ void __launch_bounds__(ZTile<N>::THREADS, ZGeom<N>::MIN_BLOCKS) k_zconv(
    float2* __restrict__ S, const float2* __restrict__ KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
    float scale, const float2* __restrict__ W, const __grid_constant__ CUtensorMap tmap, int use_tma) {
  using G = ZTile<N>;
  using Z = ZGeom<N>;
  extern __shared__ __align__(128) float2 zsm[];
  float2* stash = zsm + Z::XCH;
  float2* stage = zsm + Z::STAGE_OFF;
  uint64_t* bar = nullptr;
  if (Z::TMA_OK && use_tma && (async::smem_addr(stage) & 127u) == 0) {
    bar = reinterpret_cast<uint64_t*>(zsm + Z::BAR_OFF);
    if (threadIdx.x == 0) {
      async::bar_init(bar, 1);
      async::bar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      async::bar_expect(bar, Z::STAGE_BYTES);
      if (!async::copies_skipped())
        async::tensor_load_3d(stage, &tmap, (int)blockIdx.x * G::B, (int)blockIdx.y, 0, bar);
    }
  }
  body_zconv<N, CONJ, tc::kNone, G>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, W, (int)blockIdx.x,
                                    (int)blockIdx.y, (int)threadIdx.x, zsm, stash, G::THREADS,
                                    TcCtx{nullptr}, stage, bar);
}

// ---------------------------------------------------------------------------
// Persistent fused z pass.  Each CTA walks the tiles (B columns x N planes of
// one row ky) with a stride of the grid size; both operands of a tile arrive
// in shared memory by tensor-map copies (TMA) issued one tile ahead:
//   * the image tile (N rows of B columns) into ISTAGE, in NBOX boxes of
//     ZBOX rows; the next tile's copy is issued as soon as every thread has
//     read the current one into registers, so it lands behind the current
//     tile's three transforms;
//   * the kernel column tile (the kplanes planes of KXY that hold taps) into
//     KSTAGE, in boxes of kbox rows (host-chosen, <= 256); once transformed,
//     the kernel spectrum is parked in the same buffer (per-thread private
//     slots), and the next tile's kernel copy is issued after the product has
//     read it, so it lands behind the inverse transform and the stores.
// The stage tables of both radix chains sit in shared memory, copied once per
// CTA.  Every copy's destination is 128-byte aligned and every box lies
// inside its buffer: lengths whose image boxes would start off a 128-byte
// boundary (e.g. z = 500 on 4-column tiles, whose second 250-row box would
// start 8000 bytes in) keep the one-tile-per-CTA kernel.  Waits are bounded:
// a wait that runs out is counted, the CTA waits (bounded) for any copy it
// still has in flight, and returns.
// columns per tile of the persistent fused z pass (at most; 16 by default,
// other widths for comparison builds)
#ifndef FC_ZPIPE_B
#define FC_ZPIPE_B 16
#endif
template <int N>
struct ZPipe {
  using G = ColGeomB<N, FC_ZPIPE_B>;
  static constexpr int B = G::B;
  static constexpr int THREADS = G::THREADS;
  static constexpr int XCH_BYTES = ((G::SMEM * (int)sizeof(float2) + 127) / 128) * 128;
  static constexpr int ZBOX = zbox_rows(N);
  static constexpr int NBOX = N / ZBOX;
  static constexpr int IBYTES = N * B * (int)sizeof(float2);
  static constexpr int ISTAGE_OFF = XCH_BYTES;
  // kernel planes: at most N rows in boxes of kbox rows, each box's bytes a
  // multiple of 128 (kbox a multiple of 16/B); capacity N + 16 rows covers the
  // rounding; the parked kernel spectrum needs THREADS*16 slots
  static constexpr int KROW_ALIGN = B >= 16 ? 1 : 16 / B;
  static constexpr int KCAP = (N + 16) * B > THREADS * kVals ? (N + 16) * B : THREADS * kVals;  // float2
  static constexpr int KSTAGE_OFF = ISTAGE_OFF + ((IBYTES + 127) / 128) * 128;
  // stage tables of both chains (forward transforms: REV = kZRev; inverse: !kZRev)
  static constexpr int TWF_N = Plan<N>::tab_size(kZRev), TWI_N = Plan<N>::tab_size(!kZRev);
  static constexpr int TWF_OFF = KSTAGE_OFF + ((KCAP * (int)sizeof(float2) + 127) / 128) * 128;
  static constexpr int TWI_OFF = TWF_OFF + ((TWF_N * (int)sizeof(float2) + 127) / 128) * 128;
  static constexpr int BAR_OFF = TWI_OFF + ((TWI_N * (int)sizeof(float2) + 127) / 128) * 128;
  static constexpr int SMEM_BYTES = BAR_OFF + 128;
  static_assert(ZBOX <= 256 && ZBOX * NBOX == N, "image boxes must tile the column");
  static_assert((B * (int)sizeof(float2)) % 16 == 0, "box rows must be multiples of 16 bytes");
  static_assert(ISTAGE_OFF % 128 == 0 && KSTAGE_OFF % 128 == 0 && BAR_OFF % 128 == 0, "stage alignment");
  static constexpr bool OK = (ZBOX * B * (int)sizeof(float2)) % 128 == 0 && SMEM_BYTES <= 227 * 1024;
  // resident CTAs asked of the register allocator: 512 threads per SM (at most 128 registers)
  static constexpr int MIN_BLOCKS = THREADS <= 512 ? 512 / THREADS : 1;
};

template <int N, bool CONJ>
__global__ void __launch_bounds__(ZPipe<N>::THREADS, ZPipe<N>::MIN_BLOCKS)
    k_zconv_pipe(float2* __restrict__ S, long long pitch, int ny, int ncols, int kplanes, int hz, float scale,
                 const float2* __restrict__ W, const __grid_constant__ CUtensorMap imap,
                 const __grid_constant__ CUtensorMap kmap, int kbox, int nkbox,
                 const __grid_constant__ CUtensorMap nimap, const __grid_constant__ CUtensorMap nkmap, int nyq_tiles) {
  using P = ZPipe<N>;
  constexpr int B = P::B;
  constexpr int R0 = first_radix<N, kZRev>(), RF = last_radix<N, !kZRev>();
  constexpr bool kStore = (FC_STORE_TMA & 2) != 0;
  // the next tile's image copy is issued with its kernel copy, after the
  // product's barrier, instead of after a barrier of its own
  constexpr bool kLateImage = FC_ZIMG_LATE != 0;
  extern __shared__ __align__(128) unsigned char zpsm[];
  float2* xch = reinterpret_cast<float2*>(zpsm);
  float2* ist = reinterpret_cast<float2*>(zpsm + P::ISTAGE_OFF);
  float2* kst = reinterpret_cast<float2*>(zpsm + P::KSTAGE_OFF);
  float2* twf = reinterpret_cast<float2*>(zpsm + P::TWF_OFF);
  float2* twi = reinterpret_cast<float2*>(zpsm + P::TWI_OFF);
  uint64_t* ibar = reinterpret_cast<uint64_t*>(zpsm + P::BAR_OFF);
  uint64_t* kbar = ibar + 1;
  const int tid = (int)threadIdx.x;
  const int c = tid % B;
  const int t = tid / B;
  // nyq_tiles > 0: the last column of the spectrum (ncols = B k + 1 or + 2)
  // goes in tiles of B/2 rows x 2 columns (boxes of nimap / nkmap, laid out as
  // a B-column tile: column c of the tile is row c / 2, column c % 2 of the
  // box; the second column is past the spectrum: zeros in, not stored),
  // after the full B-column tiles, instead of one tile of 1 column per row
  const int ntx = nyq_tiles > 0 ? ncols / B : (ncols + B - 1) / B;
  const long long nmain = (long long)ntx * ny;
  const long long ntiles = nmain + nyq_tiles;
  const int nyq_col = ntx * B;
  const long long zs = (long long)ny * pitch;
  const unsigned kbytes = (unsigned)(nkbox * kbox * B * (int)sizeof(float2));
  const bool skip = async::copies_skipped();
  async::pdl_trigger_at_start<async::kPdlZ>();
  auto issue_image = [&](long long ti) {
    async::bar_expect(ibar, (unsigned)P::IBYTES);
    if (skip) return;
    if (ti < nmain) {
      const int bx = (int)(ti % ntx), ky = (int)(ti / ntx);
#pragma unroll
      for (int b = 0; b < P::NBOX; ++b)
        async::tensor_load_3d(ist + b * P::ZBOX * B, &imap, bx * B, ky, b * P::ZBOX, ibar);
    } else {
      const int ky0 = (int)(ti - nmain) * (B / 2);
#pragma unroll
      for (int b = 0; b < P::NBOX; ++b)
        async::tensor_load_3d(ist + b * P::ZBOX * B, &nimap, nyq_col, ky0, b * P::ZBOX, ibar);
    }
  };
  auto issue_kernel = [&](long long ti) {
    async::bar_expect(kbar, kbytes);
    if (skip) return;
    if (ti < nmain) {
      const int bx = (int)(ti % ntx), ky = (int)(ti / ntx);
      for (int b = 0; b < nkbox; ++b) async::tensor_load_3d(kst + b * kbox * B, &kmap, bx * B, ky, b * kbox, kbar);
    } else {
      const int ky0 = (int)(ti - nmain) * (B / 2);
      for (int b = 0; b < nkbox; ++b)
        async::tensor_load_3d(kst + b * kbox * B, &nkmap, nyq_col, ky0, b * kbox, kbar);
    }
  };
  // the twiddle tables are not written by any pass
  copy_stage_tables<N, kZRev>(twf, W, tid, P::THREADS);
  copy_stage_tables<N, !kZRev>(twi, W, tid, P::THREADS);
  if (tid == 0) {
    async::bar_init(ibar, 1);
    async::bar_init(kbar, 1);
    async::bar_init_fence();
  }
  __syncthreads();
  async::pdl_wait();  // the previous pass's output is complete and visible
  long long ti = blockIdx.x;
  if (tid == 0 && ti < ntiles) {
    issue_kernel(ti);
    issue_image(ti);
  }
  bool kpend = ti < ntiles, ipend = ti < ntiles;  // copies in flight (uniform)
  bool expired = false;
  uint32_t ph = 0;  // parity of the barriers' current phase (one phase per tile)
  const ColLay<B> lay{xch, c};
  bool signalled = false;  // the successor may launch (programmatic dependent launch)
  for (; ti < ntiles; ti += gridDim.x, ph ^= 1u) {
    const bool nyq = ti >= nmain;
    const int ky = nyq ? 0 : (int)(ti / ntx);
    const int col = nyq ? 0 : (int)(ti % ntx) * B + c;
    const bool ok = (nyq || col < ncols) && t < P::G::T;
    const long long next = ti + gridDim.x;
    signalled |= async::pdl_trigger_last_tile<async::kPdlZ>(next >= ntiles);
    float2 v[kVals];
    // ---- kernel column: load from KSTAGE, forward transform, park in KSTAGE
    if (kStore && tid == 0) async::bulk_wait_read();  // the previous tile's store has read XCH
    if (!__syncthreads_and(async::bar_wait(kbar, ph))) {
      expired = true;
      break;
    }
    kpend = false;
#pragma unroll
    for (int q = 0; q < kVals; ++q) {
      const int z = stage_pos<N, R0>(t, q);
      int p = z + hz;
      if (p >= N) p -= N;
      v[q] = (ok && z >= 0 && p < kplanes) ? kst[p * B + c] : make_float2(0.f, 0.f);
    }
    if constexpr (Plan<N>::S == 1) __syncthreads();  // no exchange barrier inside the transform
    // (the image wait below is the CTA barrier before the exchange area is next written)
    fft<N, false, tc::kNone, kZRev, true, !FC_TAIL_SKIP>(v, lay, t, twf);
#pragma unroll
    for (int q = 0; q < kVals; ++q) kst[q * P::THREADS + tid] = v[q];
    // ---- image tile: load from ISTAGE, then the next tile's image copy
    if (!__syncthreads_and(async::bar_wait(ibar, ph))) {
      expired = true;
      break;
    }
    ipend = false;
#pragma unroll
    for (int q = 0; q < kVals; ++q) {
      const int z = stage_pos<N, R0>(t, q);
      v[q] = (ok && z >= 0) ? ist[z * B + c] : make_float2(0.f, 0.f);
    }
    if constexpr (!kLateImage) {
      async::proxy_fence();
      __syncthreads();  // every thread has read ISTAGE
      if (next < ntiles) {
        if (tid == 0) issue_image(next);
        ipend = true;
      }
    }
    // (the barrier after the product is the one before the next write of the exchange area)
    fft<N, false, tc::kNone, kZRev, true, !FC_TAIL_SKIP>(v, lay, t, twf);
#pragma unroll
    for (int q = 0; q < kVals; ++q) {
      float2 a = kst[q * P::THREADS + tid];  // kernel spectrum (d_Src of modulateAndNormalize_kernel)
      const float2 b = v[q];                  // image spectrum  (d_Dst)
      if (CONJ) a.y = -a.y;
      v[q] = make_float2(scale * (a.x * b.x - a.y * b.y), scale * (a.y * b.x + a.x * b.y));
    }
    async::proxy_fence();
    __syncthreads();  // every thread has read its parked kernel spectrum (and ISTAGE)
    if (next < ntiles) {
      if (tid == 0) {
        issue_kernel(next);
        if (kLateImage) issue_image(next);
      }
      kpend = true;
      if (kLateImage) ipend = true;
    }
    // staged stores write the exchange area next: keep the closing barrier;
    // per-thread stores reach the next tile's first barrier before it
    fft<N, true, tc::kNone, !kZRev, true, kStore || !FC_TAIL_SKIP>(v, lay, t, twi);
    if constexpr (kStore) {
      // the tile as rows of B columns in XCH (the inverse's last exchange has
      // been read), then one tensor store per box; the store leaves out the
      // columns past ncols.  The next tile's first exchange waits for the
      // store to have read XCH (the wait before its first barrier).
#pragma unroll
      for (int q = 0; q < kVals; ++q) {
        const int z = stage_pos<N, RF>(t, q);
        if (z >= 0) xch[z * B + c] = v[q];
      }
      async::proxy_fence();
      __syncthreads();
      if (tid == 0) {
        if (!nyq) {
          const int bx = (int)(ti % ntx);
#pragma unroll
          for (int b = 0; b < P::NBOX; ++b)
            async::tensor_store_3d(&imap, bx * B, ky, b * P::ZBOX, xch + b * P::ZBOX * B);
        } else {
          const int ky0 = (int)(ti - nmain) * (B / 2);
#pragma unroll
          for (int b = 0; b < P::NBOX; ++b)
            async::tensor_store_3d(&nimap, nyq_col, ky0, b * P::ZBOX, xch + b * P::ZBOX * B);
        }
        async::bulk_commit();
      }
    } else if (ok) {
      float2* base = S + (long long)ky * pitch + col;
#pragma unroll
      for (int q = 0; q < kVals; ++q) {
        const int z = stage_pos<N, RF>(t, q);
        if (z >= 0) base[(long long)z * zs] = v[q];
      }
    }
  }
  async::pdl_trigger_at_end<async::kPdlZ>(signalled);
  if (expired) {
    // a wait ran out: count it, then let the copies still in flight (both of
    // the current phase) land, with the same bounded wait, before returning
    if (tid == 0) atomicAdd(&g_zstage_timeouts, 1u);
    if (kpend) (void)async::bar_wait(kbar, ph);
    if (ipend) (void)async::bar_wait(ibar, ph);
  }
  if (kStore && tid == 0) async::bulk_wait();  // the tile stores are complete before the CTA ends
}

// Host: encode the tensor map of k_zconv's image stage for a spectrum of ncols
// columns (row pitch `pitch` float2), ny rows and n planes; false when the
// driver entry point is missing or the layout breaks a tensor-map rule.
bool zstage_tensor_map(CUtensorMap* map, const float2* S, long long pitch, int ny, int ncols, int n, int box_cols,
                       int box_rows);
// FC_ZPIPE=0 selects the one-tile-per-CTA fused z pass instead of the persistent one
bool zpipe_enabled();

// Host: launch the persistent fused z pass when its geometry applies (sets
// *used); otherwise enqueue nothing and leave *used false.  The kernel planes
// come in boxes of kbox <= 256 rows, kbox a multiple of KROW_ALIGN (so that
// every box starts 128-byte aligned), within KSTAGE's capacity.
template <int N, bool CONJ>
static cudaError_t zconv_pipe_launch(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes,
                                     int hz, float scale, const float2* W, cudaStream_t st, bool* used) {
  using P = ZPipe<N>;
  *used = false;
  if constexpr (!P::OK) {
    return cudaSuccess;
  } else {
    if (!zpipe_enabled() || kplanes < 1 || kplanes > N || ny < 1 || ncols < 1) return cudaSuccess;
    const int nkb = (kplanes + 255) / 256;
    int kbox = (kplanes + nkb - 1) / nkb;
    kbox = (kbox + P::KROW_ALIGN - 1) / P::KROW_ALIGN * P::KROW_ALIGN;
    if (kbox > 256 || (long long)nkb * kbox * P::B > P::KCAP) return cudaSuccess;
    CUtensorMap imap, kmap, nimap, nkmap;
    if (!zstage_tensor_map(&imap, S, pitch, ny, ncols, N, P::B, P::ZBOX) ||
        !zstage_tensor_map(&kmap, KXY, pitch, ny, ncols, kplanes, P::B, kbox))
      return cudaSuccess;
    // the last one or two columns in tiles of 8 rows x 2 columns (the fused
    // pass writes its tiles back by tensor-map stores, which leave out what
    // lies past the spectrum)
    int nyq_tiles = 0;
    const int rem = ncols % P::B;
    if (FC_ZNYQ && (FC_STORE_TMA & 2) && P::B >= 4 && (rem == 1 || rem == 2) && ncols > P::B &&
        tile_tensor_map(&nimap, S, pitch, ny, ncols, N, 2, P::B / 2, P::ZBOX) &&
        tile_tensor_map(&nkmap, KXY, pitch, ny, ncols, kplanes, 2, P::B / 2, kbox))
      nyq_tiles = (ny + P::B / 2 - 1) / (P::B / 2);
    else
      nimap = imap, nkmap = kmap;
    auto kern = k_zconv_pipe<N, CONJ>;
    static int s_occ = 0;  // resident CTAs per SM of this instantiation (a benign race: same value)
    int occ = s_occ;
    if (occ == 0) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM_BYTES);
      if (e != cudaSuccess) return e;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, P::THREADS, P::SMEM_BYTES);
      if (e != cudaSuccess) return e;
      if (occ < 1) return cudaSuccess;
      s_occ = occ;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long ntiles = nyq_tiles > 0 ? (long long)(ncols / P::B) * ny + nyq_tiles
                                           : (long long)((ncols + P::B - 1) / P::B) * ny;
    const long long grid = std::min<long long>(ntiles, (long long)occ * sms);
    *used = true;
    return async::launch_pdl(async::kPdlZ, kern, (unsigned)grid, P::THREADS, P::SMEM_BYTES, st, S, pitch, ny, ncols,
                             kplanes, hz, scale, W, imap, kmap, kbox, nkb, nimap, nkmap, nyq_tiles);
  }
}
// Host: enqueue a read of this translation unit's count of expired stage
// waits into dst (page-locked host memory) on st; clear the count
static inline cudaError_t zstage_timeouts_read_async_tu(unsigned int* dst, cudaStream_t st) {
  return cudaMemcpyFromSymbolAsync(dst, g_zstage_timeouts, sizeof(unsigned int), 0, cudaMemcpyDeviceToHost, st);
}
static inline cudaError_t zstage_timeouts_addr_tu(unsigned int** p) {
  return cudaGetSymbolAddress((void**)p, g_zstage_timeouts);
}
static inline void zstage_timeouts_clear_tu() {
  const unsigned int zero = 0;
  cudaMemcpyToSymbol(g_zstage_timeouts, &zero, sizeof(zero));
}

template <int N>
struct CorrGeom {  // k_zcorr: exchange tile and stash of the 32-column geometry
  static constexpr int SMEM_BYTES = (ColGeom<N>::SMEM + ColGeom<N>::THREADS * kVals) * (int)sizeof(float2);
};

// Kernel-gradient z pass: conj(X) * G * scale, inverse, keep kernel planes
// p < kz where z = (p - hz) mod nz, written to out plane p.
template <int N>
__global__ void __launch_bounds__(ColGeom<N>::THREADS) k_zcorr(const float2* __restrict__ X,
                                                               const float2* __restrict__ Gs, float2* __restrict__ out,
                                                               long long pitch, int ny, int ncols, int kz, int hz,
                                                               float scale, const float2* __restrict__ W) {
  using G = ColGeom<N>;
  constexpr int B = G::B;
  constexpr int R0 = first_radix<N, false>(), RF = last_radix<N, true>();
  extern __shared__ float2 zsm[];
  float2* sm = zsm;
  float2* stash = zsm + G::SMEM;
  const int tid = threadIdx.x;
  const int c = tid % B;
  const int t = tid / B;
  const int col = blockIdx.x * B + c;
  const int ky = blockIdx.y;
  const bool ok = col < ncols && t < G::T;
  const long long zs = (long long)ny * pitch;
  const long long off = (long long)ky * pitch + col;
  float2 v[kVals];
  const ColLay<B> lay{sm, c};
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int z = stage_pos<N, R0>(t, q);
    v[q] = (ok && z >= 0) ? X[(long long)z * zs + off] : make_float2(0.f, 0.f);
  }
  fft<N, false>(v, lay, t, W);
#pragma unroll
  for (int q = 0; q < kVals; ++q) stash[q * G::THREADS + tid] = v[q];
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const int z = stage_pos<N, R0>(t, q);
    v[q] = (ok && z >= 0) ? Gs[(long long)z * zs + off] : make_float2(0.f, 0.f);
  }
  fft<N, false>(v, lay, t, W);
#pragma unroll
  for (int q = 0; q < kVals; ++q) {
    const float2 x = stash[q * G::THREADS + tid];
    const float2 a = make_float2(x.x, -x.y);
    const float2 b = v[q];
    v[q] = make_float2(scale * (a.x * b.x - a.y * b.y), scale * (a.y * b.x + a.x * b.y));
  }
  fft<N, true>(v, lay, t, W);
  if (ok) {
#pragma unroll
    for (int q = 0; q < kVals; ++q) {
      const int z = stage_pos<N, RF>(t, q);
      if (z < 0) continue;
      int p = z + hz;
      if (p >= N) p -= N;
      if (p < kz) out[((long long)p * ny + ky) * pitch + col] = v[q];
    }
  }
}


}  // namespace fast
}  // namespace fc
