// Fifth-generation tensor-core (tcgen05) 16-point DFT for the radix-16 stages
// of the register-resident engine: the opt-in precision mode
// (FC_FLAG_TC_FP16 / FC_FLAG_TC_BF16), sm_100-family inline PTX.
//
// At a radix-16 stage every thread of a CTA owns one butterfly: 16 complex
// inputs x (after the stage twiddles).  Each group of 128 threads is one
// M = 128 tile: thread r of the group writes its butterfly as row r of A,
//   A[r] = [Re x_0 .. Re x_15, Im x_0 .. Im x_15]   (K = 32 reals),
// and one elected thread issues the product D = A * B^T on the tensor cores,
// where B^T[n][k] (N = 32 rows, K = 32) is the real form of the DFT matrix
// W[n][k] = exp(-+2 pi i n k / 16), with C = cos(2 pi n k / 16) and
// S = sin(2 pi n k / 16):
//   rows n < 16 (Re y):  [ C | +S ] forward, [ C | -S ] inverse;
//   rows n >= 16 (Im y): [ -S | C ] forward, [ +S | C ] inverse.
// D (128 lanes x 32 fp32 columns) lives in tensor memory (TMEM); thread r
// reads its lane's 32 columns back with tcgen05.ld, so the outputs y_0..y_15
// land in the same registers that held the inputs.
//
// Precision: each row is scaled by its own power of two (fp16 only; bf16 has
// the float exponent range), split into 16-bit hi + lo parts, and the tensor
// cores accumulate A_hi B_hi + A_lo B_hi + A_hi B_lo in fp32 (the A_lo B_lo
// term lies below fp32 rounding).  The DFT entries come from the exact
// values cos(2 pi a / 16), a = 0..4.
//
// Operands in shared memory use the no-swizzle K-major layout of 8 x 16-byte
// core matrices: element (row, k) at base + (row/8)*SBO + (k/8)*LBO +
// (row%8)*16 + (k%8)*2 with LBO = 128 and SBO = 512 bytes, so a 128 x 32
// matrix of 16-bit values is 8 KiB and every address a descriptor can reach
// lies inside it (whichever of the two strides the hardware applies along K).
// One K step of kind::f16 covers 16 values; the two steps start at base and
// base + 2*LBO.
//
// Protocol per stage: rows written, fence.proxy.async, CTA barrier, the
// elected thread issues 6 MMAs per group and commits them to an mbarrier,
// every thread waits (bounded) on the barrier's phase, loads its lane, waits
// for the load; before the next stage's MMAs overwrite D, the threads'
// loads are ordered before the barrier by tcgen05.fence::before_thread_sync.
// TMEM is allocated by warp 0 at kernel start and freed by warp 0 at the end
// of every kernel that sets it up (tc5_teardown), on every exit path.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "fc_async.cuh"

namespace fc {
namespace tc {

// modes
constexpr int kNone = 0, kFp16 = 1, kBf16 = 2;

constexpr int kGroup = 128;                 // rows of one MMA tile (threads per group)
constexpr int kLBO = 128, kSBO = 512;       // core-matrix strides of the operand layout (bytes)
constexpr int kMatBytes = kGroup * 32 * 2;  // one 128 x 32 operand of 16-bit values
constexpr int kBBytes = 32 * 32 * 2;        // one 32 x 32 DFT operand

// Shared memory of the mode, after the kernel's own buffers (bytes, 128-aligned):
// B (forward hi, lo; inverse hi, lo), then per group A hi and A lo, then the
// mbarrier and the TMEM address slot.
__host__ __device__ constexpr int tc5_bytes(int threads) {
  return 4 * kBBytes + ((threads + kGroup - 1) / kGroup) * 2 * kMatBytes + 128;
}
// TMEM columns: 32 per group, allocated as a power of two >= 32
__host__ __device__ constexpr int tc5_cols(int threads) {
  return ((threads + kGroup - 1) / kGroup) <= 1 ? 32 : ((threads + kGroup - 1) / kGroup) <= 2 ? 64 : 128;
}

// expired waits on the MMA barrier (per translation unit; read with the other counts)
[[maybe_unused]] static __device__ unsigned int g_tc5_timeouts;

struct Tc5 {
  uint32_t b;         // shared address of the four B operands
  uint32_t a;         // shared address of this thread's group's A hi (A lo follows)
  uint32_t bar;       // shared address of the mbarrier
  uint32_t tmem;      // TMEM address of this group's accumulator, this warp's lane quarter
  uint32_t tmem_mma;  // TMEM address of this group's accumulator (lane 0)
  int ngroups;
  mutable uint32_t phase;
  mutable bool failed;
};

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(kLBO >> 4) << 16) | ((uint64_t)(kSBO >> 4) << 32) |
         (1ull << 46);  // descriptor version for the sm_100 family; no swizzle, base offset 0
}

// instruction descriptor of kind::f16: D fp32, A and B fp16 (0) or bf16 (1),
// both K-major, N = 32, M = 128
template <int TCM>
__device__ __forceinline__ uint32_t idesc() {
  constexpr uint32_t fmt = TCM == kBf16 ? 1u : 0u;
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&d)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) d[i] = __uint_as_float(r[i]);
}

// cos(2 pi k / 16) for any integer k, from the exact values cos(2 pi a / 16), a = 0..4
__device__ __forceinline__ float cos16(int k) {
  k &= 15;
  const int a = k <= 8 ? k : 16 - k;  // cos(2 pi (16 - k) / 16) = cos(2 pi k / 16)
  const int b = a <= 4 ? a : 8 - a;   // cos(2 pi (8 - a) / 16) = -cos(2 pi a / 16)
  const float c = b == 0 ? 1.0f
                  : b == 1 ? 0.92387953251128675613f   // cos(pi/8)  = sqrt(2 + sqrt 2) / 2
                  : b == 2 ? 0.70710678118654752440f   // cos(pi/4)  = sqrt 2 / 2
                  : b == 3 ? 0.38268343236508977173f   // cos(3pi/8) = sqrt(2 - sqrt 2) / 2
                           : 0.0f;
  return a <= 4 ? c : -c;
}

template <int TCM>
__device__ __forceinline__ uint16_t to16(float x) {
  if constexpr (TCM == kFp16)
    return __half_as_ushort(__float2half_rn(x));
  else
    return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
template <int TCM>
__device__ __forceinline__ float from16(uint16_t h) {
  if constexpr (TCM == kFp16)
    return __half2float(__ushort_as_half(h));
  else
    return __bfloat162float(__ushort_as_bfloat16(h));
}

// byte offset of element (row, k) in the operand layout
__host__ __device__ __forceinline__ constexpr int opnd_off(int row, int k) {
  return (row >> 3) * kSBO + (k >> 3) * kLBO + (row & 7) * 16 + (k & 7) * 2;
}

// Set up the mode (all threads of the CTA call it): B operands, mbarrier,
// TMEM allocation by warp 0.  `smem` is the mode's 128-aligned area of
// tc5_bytes(threads) bytes.
template <int TCM>
__device__ __forceinline__ Tc5 tc5_setup(unsigned char* smem, int tid, int threads) {
  Tc5 c;
  const uint32_t base = async::smem_addr(smem);
  c.ngroups = (threads + kGroup - 1) / kGroup;
  c.b = base;
  c.a = base + 4 * kBBytes + (tid / kGroup) * 2 * kMatBytes;
  c.bar = base + 4 * kBBytes + c.ngroups * 2 * kMatBytes;
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + 4 * kBBytes + c.ngroups * 2 * kMatBytes + 16);
  // B^T[n][k] in hi and lo parts, forward then inverse
  for (int e = tid; e < 2 * 32 * 32; e += threads) {
    const int inv = e >> 10, n = (e >> 5) & 31, k = e & 31;
    const int nn = n & 15, kk = k & 15;
    float f;
    if ((n < 16) == (k < 16)) {
      f = cos16(nn * kk);
    } else {
      const float s = cos16(nn * kk - 4);  // sin(x) = cos(x - pi/2)
      // rows n < 16 take +S (forward) / -S (inverse) on the Im inputs; rows n >= 16 the opposite on the Re inputs
      f = (n < 16) == (inv == 0) ? s : -s;
    }
    const uint16_t hi = to16<TCM>(f);
    const uint16_t lo = to16<TCM>(f - from16<TCM>(hi));
    unsigned char* bm = smem + inv * 2 * kBBytes;
    *reinterpret_cast<uint16_t*>(bm + opnd_off(n, k)) = hi;
    *reinterpret_cast<uint16_t*>(bm + kBBytes + opnd_off(n, k)) = lo;
  }
  if (tid == 0) {
    async::bar_init(reinterpret_cast<uint64_t*>(smem + 4 * kBBytes + c.ngroups * 2 * kMatBytes), 1);
    async::bar_init_fence();
  }
  if (tid < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(async::smem_addr(slot)),
                 "r"(tc5_cols(threads))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  async::proxy_fence();  // the B operands, written by the generic proxy, are read by the MMAs
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t t0 = *slot;
  const int g = tid / kGroup;
  c.tmem_mma = t0 + (uint32_t)(g * 32);
  c.tmem = c.tmem_mma + ((uint32_t)(32 * ((tid % kGroup) / 32)) << 16);
  c.phase = 0;
  c.failed = false;
  return c;
}

// Free the TMEM (all threads of the CTA call it, after their last use)
__device__ __forceinline__ void tc5_teardown(const Tc5& c, int tid, int threads) {
  fence_before();
  __syncthreads();
  if (tid < 32) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem_mma), "r"(tc5_cols(threads))
                 : "memory");
  }
}

// In-place 16-point DFT of v[0..15] of every thread of the CTA (all call it).
template <bool INV, int TCM>
__device__ __forceinline__ void dft16(float2* v, const Tc5& c) {
  // fp16: power-of-two scale of this row (bf16 has the float exponent range)
  float s = 1.f, inv_s = 1.f;
  if constexpr (TCM == kFp16) {
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) m = fmaxf(m, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
    // m < 2^e from the biased exponent E of m (E = 0 for zero and subnormal m),
    // e clamped to [-126, 126] so that both 2^-e and 2^e are normal floats
    const int e = min(max(((__float_as_int(m) >> 23) & 255) - 126, -126), 126);
    s = __int_as_float((127 - e) << 23);
    inv_s = __int_as_float((127 + e) << 23);
  }
  // row of A: reals 0..15 = Re x, 16..31 = Im x; hi and lo parts, 16 bytes per
  // core-matrix row segment of 8 values
  const int row = (int)threadIdx.x % kGroup;
#pragma unroll
  for (int kc = 0; kc < 4; ++kc) {
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const int k0 = 8 * kc + 2 * p;
      const float x0 = (k0 < 16 ? v[k0 & 15].x : v[k0 & 15].y) * s;
      const float x1 = (k0 + 1 < 16 ? v[(k0 + 1) & 15].x : v[(k0 + 1) & 15].y) * s;
      const uint16_t h0 = to16<TCM>(x0), h1 = to16<TCM>(x1);
      const uint16_t l0 = to16<TCM>(x0 - from16<TCM>(h0)), l1 = to16<TCM>(x1 - from16<TCM>(h1));
      hw[p] = (uint32_t)h0 | ((uint32_t)h1 << 16);
      lw[p] = (uint32_t)l0 | ((uint32_t)l1 << 16);
    }
    const uint32_t off = (uint32_t)opnd_off(row, 8 * kc);
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(c.a + off), "r"(hw[0]), "r"(hw[1]), "r"(hw[2]),
                 "r"(hw[3])
                 : "memory");
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(c.a + kMatBytes + off), "r"(lw[0]), "r"(lw[1]),
                 "r"(lw[2]), "r"(lw[3])
                 : "memory");
  }
  async::proxy_fence();  // A rows written by the generic proxy are read by the MMAs
  fence_before();        // this thread's earlier TMEM loads precede the next MMAs
  __syncthreads();
  if (threadIdx.x == 0) {
    fence_after();
    const uint32_t id = idesc<TCM>();
    const uint32_t bh = c.b + (INV ? 2 * kBBytes : 0), bl = bh + kBBytes;
    for (int g = 0; g < c.ngroups; ++g) {
      const uint32_t ah = c.b + 4 * kBBytes + g * 2 * kMatBytes, al = ah + kMatBytes;
      const uint32_t d = c.tmem_mma + (uint32_t)(g * 32);  // thread 0 belongs to group 0
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        const uint32_t ko = (uint32_t)(ks * 2 * kLBO);
        mma_f16(d, sdesc(ah + ko), sdesc(bh + ko), id, ks > 0 ? 1u : 0u);
        mma_f16(d, sdesc(al + ko), sdesc(bh + ko), id, 1u);
        mma_f16(d, sdesc(ah + ko), sdesc(bl + ko), id, 1u);
      }
    }
    mma_commit(c.bar);
  }
  // every thread waits for the MMAs (bounded); a wait that runs out is
  // counted and waited for once more, so no MMA is left running into the
  // next stage or past the TMEM release
  uint64_t* bar = reinterpret_cast<uint64_t*>(__cvta_shared_to_generic(c.bar));
  if (!async::bar_wait(bar, c.phase & 1u)) {
    if ((threadIdx.x & 31) == 0) atomicAdd(&g_tc5_timeouts, 1u);
    c.failed = true;
    (void)async::bar_wait(bar, c.phase & 1u);
  }
  c.phase++;
  fence_after();
  float d[32];
  tmem_ld32(c.tmem, d);
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = make_float2(d[k] * inv_s, d[16 + k] * inv_s);
}

}  // namespace tc
}  // namespace fc
