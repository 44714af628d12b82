// Host orchestration and C ABI of libFourierConvolutionCUDALib.so (GB300).
//
// Replaces the reference's host layer (src/convolution3Dfft.cu:216-603 and
// src/standardCUDAfunctions.cu:13-71).  Differences by design:
//   * no exit() and no exception crosses the C ABI: failures set a
//     thread-local status/message (fc_last_status / fc_last_error);
//   * one context per device holds a stream, a grow-only workspace, device
//     buffers for the host entry points and the twiddle tables per length;
//     calls on the same device serialise on the context's mutex;
//   * the FFT is this library's own (fc_fft.cuh); the spectrum product and the
//     kernel padding/shift are fused into the passes (fc_kernels.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <fstream>
#include <functional>
#include <sstream>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "../../include/convolution3Dfft.h"
#include "fc_batched.cuh"
#include "fc_internal.h"

namespace fc {

// ------------------------------------------------------------------ status
static thread_local int t_status = FC_OK;
static thread_local std::string t_error;
static thread_local int t_launches = 0;
static thread_local bool t_no_events = false;  // set while enqueuing for the allocation-free entry point

struct FcError {
  int code;
  std::string msg;
};

static void set_status(int code, const std::string& msg) {
  t_status = code;
  t_error = msg;
}
static void clear_status() {
  t_status = FC_OK;
  t_error.clear();
  t_launches = 0;
}

#define FC_THROW(code, msg)      \
  do {                           \
    throw FcError{(code), (msg)}; \
  } while (0)

static void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    const int code = (e == cudaErrorMemoryAllocation) ? FC_ERR_NOMEM : FC_ERR_CUDA;
    FC_THROW(code, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

// ------------------------------------------------------------------ allocation fault injection
// FC_FAULT_INJECT=alloc:n, or fc_fault_inject("alloc:n"), makes the n-th
// device or page-locked allocation of this library from then on fail as if
// the device were out of memory (n >= 1; "off" disables it).  The failure is
// made on the host before the CUDA call, so nothing of it reaches the GPU; it
// exercises the error paths that a real allocation failure takes.
static std::mutex g_fault_mu;
static long long g_fault_alloc_at = -1;  // -1: environment not read yet; 0: off
static long long g_fault_alloc_seen = 0;

// 0 on success with *n set (0 = off), -1 for a malformed specification
static int parse_fault_spec(const char* spec, long long* n) {
  *n = 0;
  if (!spec || !*spec || std::strcmp(spec, "off") == 0 || std::strcmp(spec, "0") == 0) return 0;
  if (std::strncmp(spec, "alloc:", 6) != 0) return -1;
  char* end = nullptr;
  const long long v = std::strtoll(spec + 6, &end, 10);
  if (end == spec + 6 || *end != '\0' || v < 1) return -1;
  *n = v;
  return 0;
}

static bool fault_alloc_now() {
  std::lock_guard<std::mutex> lk(g_fault_mu);
  if (g_fault_alloc_at < 0) {
    long long n = 0;
    g_fault_alloc_at = parse_fault_spec(std::getenv("FC_FAULT_INJECT"), &n) == 0 ? n : 0;
  }
  if (g_fault_alloc_at == 0) return false;
  if (++g_fault_alloc_seen < g_fault_alloc_at) return false;
  g_fault_alloc_at = 0;  // one failure per arming
  return true;
}

static void dev_malloc(void** p, size_t bytes, const char* what) {
  if (fault_alloc_now()) FC_THROW(FC_ERR_NOMEM, std::string(what) + ": injected allocation failure (FC_FAULT_INJECT)");
  cuda_check(cudaMalloc(p, bytes), what);
}

static void host_alloc(void** p, size_t bytes, const char* what) {
  if (fault_alloc_now()) FC_THROW(FC_ERR_NOMEM, std::string(what) + ": injected allocation failure (FC_FAULT_INJECT)");
  cuda_check(cudaHostAlloc(p, bytes, 0), what);
}

// ------------------------------------------------------------------ radix plans
static const int kMaxAxis = 4096;

// Factor n into stages: powers of two as evenly sized radix-16/8/4/2 stages,
// then 3, 5, 7, 11, 13 butterflies, then any remaining prime as a generic stage.
static int plan_radices(int n, int* out, int maxs) {
  if (n < 1) return -1;
  std::vector<int> r;
  int m = n, a = 0;
  while ((m & 1) == 0) {
    m >>= 1;
    ++a;
  }
  if (a > 0) {
    const int s = (a + 3) / 4;
    int rem = a;
    for (int i = 0; i < s; ++i) {
      const int e = (rem + (s - i) - 1) / (s - i);  // ceil(rem / stages left)
      r.push_back(1 << e);
      rem -= e;
    }
  }
  const int small[] = {3, 5, 7, 11, 13};
  for (int p : small) {
    while (m % p == 0) {
      r.push_back(p);
      m /= p;
    }
  }
  for (int p = 17; (long long)p * p <= m; p += 2) {
    while (m % p == 0) {
      r.push_back(p);
      m /= p;
    }
  }
  if (m > 1) r.push_back(m);
  if (r.empty()) r.push_back(1);  // n == 1: identity stage handled as radix 1 -> generic
  if ((int)r.size() > maxs) return -1;
  // larger radices first: fewer twiddle multiplies in the early stages
  for (size_t i = 0; i < r.size(); ++i) out[i] = r[i];
  return (int)r.size();
}

// ------------------------------------------------------------------ device context
struct DevCtx {
  int dev = -1;
  std::mutex mu;
  cudaStream_t stream = nullptr;
  void* ws = nullptr;
  size_t ws_cap = 0;
  float* d_img = nullptr;
  size_t img_cap = 0;
  float* d_ker = nullptr;
  size_t ker_cap = 0;
  std::map<int, float2*> twiddles;  // per transform length
  // side stream and events of the kernel-spectrum fork (created on first use)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_aux = nullptr, ev_done = nullptr;
  // streams and events of the view-concurrent batched schedule (created on first use)
  std::vector<cudaStream_t> bstreams;
  std::vector<cudaEvent_t> bevents;
  // page-locked counts of expired bounded device waits, read on the stream
  // before a synchronous entry's final synchronisation (created on first use)
  unsigned int* h_timeouts = nullptr;
};

// The kernel-spectrum passes depend only on the kernel, so they can run on a
// side stream while the image x and y passes run on the caller's stream; the
// fused z pass waits for them.
struct Fork {
  cudaStream_t side;
  cudaEvent_t forked, joined, aux, done;
};

static std::mutex g_ctx_mu;
static std::map<int, std::unique_ptr<DevCtx>> g_ctx;
static int g_shift_compat = -1;  // -1: not yet read from the environment

static bool shift_compat_default() {
  if (g_shift_compat < 0) {
    const char* e = std::getenv("FC_SHIFT_COMPAT");
    g_shift_compat = (e && std::atoi(e) != 0) ? 1 : 0;
  }
  return g_shift_compat == 1;
}

static int current_device() {
  int d = 0;
  cuda_check(cudaGetDevice(&d), "cudaGetDevice");
  return d;
}

static DevCtx& ctx_for(int dev) {
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  auto it = g_ctx.find(dev);
  if (it != g_ctx.end()) return *it->second;
  auto c = std::make_unique<DevCtx>();
  c->dev = dev;
  DevCtx& ref = *c;
  g_ctx[dev] = std::move(c);
  zstage_prepare();  // a driver entry-point lookup: here, not inside a later stream capture
  return ref;
}

static cudaStream_t ctx_stream(DevCtx& c) {
  if (!c.stream) cuda_check(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking), "cudaStreamCreate");
  return c.stream;
}

static void grow(void** p, size_t* cap, size_t need, const char* what) {
  if (need <= *cap) return;
  if (*p) {
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
  }
  dev_malloc(p, need, what);
  *cap = need;
}

// twiddle table W[k] = exp(-2 pi i k / n), double precision rounded once
static const float2* twiddles_for(DevCtx& c, int n) {
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  auto it = c.twiddles.find(n);
  if (it != c.twiddles.end()) return it->second;
  std::vector<float2> h(n);
  for (int k = 0; k < n; ++k) {
    const double ang = -2.0 * M_PI * (double)k / (double)n;
    h[k] = make_float2((float)std::cos(ang), (float)std::sin(ang));
  }
  float2* d = nullptr;
  dev_malloc((void**)&d, sizeof(float2) * (size_t)fast_twiddle_count(n), "cudaMalloc(twiddles)");
  cuda_check(cudaMemcpy(d, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice), "cudaMemcpy(twiddles)");
  cuda_check(launch_stage_twiddles(d, n, nullptr), "stage twiddles");
  cuda_check(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize(twiddles)");
  c.twiddles[n] = d;
  return d;
}

static FcAxis make_axis(DevCtx& c, int n) {
  FcAxis ax;
  std::memset(&ax, 0, sizeof(ax));
  ax.n = n;
  int r[FC_MAX_STAGES];
  const int s = plan_radices(n, r, FC_MAX_STAGES);
  if (s < 0) FC_THROW(FC_ERR_UNSUPPORTED, "no radix plan for length " + std::to_string(n));
  ax.nst = (n == 1) ? 0 : s;
  for (int i = 0; i < s; ++i) ax.radix[i] = r[i];
  ax.W = twiddles_for(c, n);
  return ax;
}

// ------------------------------------------------------------------ geometry
static int ilog2_floor(long long v) {
  int l = 0;
  while ((2LL << l) <= v) ++l;
  return l;
}

static Tiles choose_tiles(const Geom& g) {
  Tiles t;
  t.threads = 256;
  // x passes: about 2048 complex values per CTA (two real rows per line)
  long long P = std::max(1LL, 2048LL / std::max(1, g.nx));
  P = std::min(P, 64LL);
  // small volumes (a kernel transformed at its own size): fewer line pairs
  // per CTA, so that the grid still gives every SM two CTAs (each line's
  // transform does not depend on the tiling)
  const long long kMinCtas = 2 * 152;
  const long long rows = (long long)g.ny * g.nz;
  while (P > 1 && (rows + 2 * P - 1) / (2 * P) < kMinCtas) P >>= 1;
  t.x_pairs_log2 = ilog2_floor(P);
  // y passes: about 4096 complex values per tile (64 KiB of shared memory for 2 buffers),
  // no wider than the spectrum's columns
  long long By = std::max(1LL, std::min(32LL, 4096LL / std::max(1, g.ny)));
  while (By > 1 && By / 2 >= g.nxh) By >>= 1;
  while (By > 1 && (g.nxh + By - 1) / By * g.nz < kMinCtas) By >>= 1;
  t.y_cols_log2 = ilog2_floor(By);
  // z pass holds image and kernel columns: about 2048 columns x rows
  long long Bz = std::max(1LL, std::min(32LL, 2048LL / std::max(1, g.nz)));
  while (Bz > 1 && Bz / 2 >= g.nxh) Bz >>= 1;
  while (Bz > 1 && (g.nxh + Bz - 1) / Bz * g.ny < kMinCtas) Bz >>= 1;
  t.z_cols_log2 = ilog2_floor(Bz);
  return t;
}

static long long spectrum_pitch(int nxh) {
  if (nxh >= 64) return ((long long)nxh + 15) / 16 * 16;
  return ((long long)nxh + 1) / 2 * 2;
}

static size_t align256(size_t v) { return (v + 255) / 256 * 256; }

static void validate_dims(int nx, int ny, int nz) {
  if (nx < 1 || ny < 1 || nz < 1) FC_THROW(FC_ERR_ARG, "image dimensions must be positive");
  if (nx > kMaxAxis || ny > kMaxAxis || nz > kMaxAxis)
    FC_THROW(FC_ERR_UNSUPPORTED, "axis longer than " + std::to_string(kMaxAxis) + " is not supported by this build");
}

static Geom make_geom(int nx, int ny, int nz, int kx, int ky, int kz, bool dense) {
  validate_dims(nx, ny, nz);
  Geom g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.nxh = nx / 2 + 1;
  g.pitch = spectrum_pitch(g.nxh);
  g.kbox = !dense;
  if (dense) {
    g.kx = nx;
    g.ky = ny;
    g.kz = nz;
    g.kplanes = nz;
    g.krows = ny;
  } else {
    if (kx < 1 || ky < 1 || kz < 1) FC_THROW(FC_ERR_ARG, "kernel dimensions must be positive");
    if (kx > nx || ky > ny || kz > nz) FC_THROW(FC_ERR_ARG, "kernel larger than the image along an axis");
    g.kx = kx;
    g.ky = ky;
    g.kz = kz;
    g.kplanes = kz;
    g.krows = ky;
  }
  return g;
}

// Plain convolution workspace: S (image spectrum), KX (kernel x-spectrum rows,
// box mode only), KXY (kernel xy-spectrum planes), dense (materialised kernel
// for the reference-arithmetic placement).
static Layout conv_layout(const Geom& g, bool compat_dense) {
  Layout L;
  size_t o = 0;
  const size_t row = (size_t)g.pitch * sizeof(float2);
  L.off_S = o;
  o = align256(o + row * g.ny * g.nz);
  L.off_KX = o;
  if (g.kbox) o = align256(o + row * g.krows * g.kplanes);
  L.off_KXY = o;
  o = align256(o + row * g.ny * g.kplanes);
  L.off_dense = o;
  if (compat_dense) o = align256(o + sizeof(float) * (size_t)g.N());
  L.off_aux = o;
  L.total = o;
  return L;
}

// ------------------------------------------------------------------ profiling
struct ProfRec {
  std::string name;
  cudaEvent_t a, b;
  double bytes;
};
static std::mutex g_prof_mu;
static bool g_prof_on = false;
static std::string g_prof_only;  // record only the pass of this name (empty: all)
static std::vector<ProfRec> g_prof;

static bool prof_wants(const char* name) {
  if (!g_prof_on || t_no_events) return false;
  std::lock_guard<std::mutex> lk(g_prof_mu);
  return g_prof_only.empty() || g_prof_only == name;
}

struct PassScope {
  bool on;
  cudaEvent_t a = nullptr, b = nullptr;
  const char* name;
  double bytes;
  cudaStream_t st;
  PassScope(const char* nm, double by, cudaStream_t s) : on(prof_wants(nm)), name(nm), bytes(by), st(s) {
    if (on) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, st);
    }
  }
  ~PassScope() {
    if (on) {
      cudaEventRecord(b, st);
      std::lock_guard<std::mutex> lk(g_prof_mu);
      g_prof.push_back(ProfRec{name, a, b, bytes});
    }
  }
};

#define FC_PASS(name, bytes, st, call)                \
  do {                                                \
    PassScope _ps((name), (double)(bytes), (st));     \
    cuda_check((call), name);                         \
    ++t_launches;                                     \
  } while (0)

// ------------------------------------------------------------------ fast / generic dispatch
// The register-resident kernels cover power-of-two lengths; every other
// length runs on the generic shared-memory kernels.  FC_GENERIC=1 forces the
// generic kernels everywhere (used by the tests to cover both).
static int g_generic_only = -1;
static bool use_fast() {
  if (g_generic_only < 0) {
    const char* e = std::getenv("FC_GENERIC");
    g_generic_only = (e && std::atoi(e) != 0) ? 1 : 0;
  }
  return g_generic_only == 0;
}

// tensor-core mode of the enqueue in progress on this thread: 0 off, 1 fp16, 2 bf16
static thread_local int t_tc_mode = 0;
static bool tc_len(int n) { return n == 128 || n == 256 || n == 512 || n == 1024; }
#define FC_TC_CALL(fn, ...) (t_tc_mode == 1 ? fn##_fp16(__VA_ARGS__) : fn##_bf16(__VA_ARGS__))

// Pipelined x passes (fc_fast_pipe.cu); FC_PIPE=0 selects the one-tile-per-CTA kernels.
static int g_pipe = -1;
// set while the enqueue in progress on this thread targets a stream that runs
// beside a persistent pass (whose CTAs take a static share of the tiles and
// should not have to wait for SMs held by this stream's work)
static thread_local bool t_no_pipe = false;
struct NoPipeScope {
  bool prev;
  NoPipeScope() : prev(t_no_pipe) { t_no_pipe = true; }
  ~NoPipeScope() { t_no_pipe = prev; }
};
static bool use_pipe() {
  if (g_pipe < 0) {
    const char* e = std::getenv("FC_PIPE");
    g_pipe = e ? std::atoi(e) : 1;
  }
  return g_pipe != 0 && !t_no_pipe;
}
// in-place y passes on wide tiles (FC_COLS_WIDE=0: the 256-thread tiles)
static int g_cols_wide = -1;
static bool cols_wide() {
  if (g_cols_wide < 0) {
    const char* e = std::getenv("FC_COLS_WIDE");
    g_cols_wide = e ? std::atoi(e) : 1;
  }
  return g_cols_wide != 0;
}
// set while the enqueue in progress on this thread reads the image from host memory
static thread_local bool t_host_src = false;
struct HostSrcScope {
  bool prev;
  explicit HostSrcScope(bool on) : prev(t_host_src) { t_host_src = on; }
  ~HostSrcScope() { t_host_src = prev; }
};
static bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

static cudaError_t d_x_r2c_dense(const float* in, long long ip, float2* out, long long op, long long rows,
                                 const FcAxis& ax, const Tiles& t, cudaStream_t st) {
  if (t_tc_mode && tc_len(ax.n)) return FC_TC_CALL(tc_x_r2c, in, ip, nullptr, 0, 0, out, op, rows, ax, st);
  if (use_fast() && fast_rows_supported(ax.n)) {
    if (use_pipe() && !t_host_src && aligned16(in) && ip % 4 == 0) return pipe_x_r2c_dense(in, ip, out, op, rows, ax, st);
    return fast_x_r2c_dense(in, ip, out, op, rows, ax, st);
  }
  return launch_x_r2c_dense(in, ip, out, op, rows, ax, t, st);
}
static cudaError_t d_x_r2c_box(const float* taps, int kx, int hx, float2* out, long long op, long long rows,
                               const FcAxis& ax, const Tiles& t, cudaStream_t st) {
  if (t_tc_mode && tc_len(ax.n)) return FC_TC_CALL(tc_x_r2c, nullptr, 0, taps, kx, hx, out, op, rows, ax, st);
  if (use_fast() && fast_rows_supported(ax.n)) return fast_x_r2c_box(taps, kx, hx, out, op, rows, ax, st);
  return launch_x_r2c_box(taps, kx, hx, out, op, rows, ax, t, st);
}
static cudaError_t d_x_c2r(const float2* in, long long ip, float* out, long long op, long long rows, const FcAxis& ax,
                           const Tiles& t, cudaStream_t st) {
  if (t_tc_mode && tc_len(ax.n)) return FC_TC_CALL(tc_x_c2r, in, ip, out, op, rows, ax, st);
  if (use_fast() && fast_rows_supported(ax.n)) {
    if (use_pipe() && aligned16(in) && ip % 2 == 0) return pipe_x_c2r(in, ip, out, op, rows, ax, st);
    return fast_x_c2r(in, ip, out, op, rows, ax, st);
  }
  return launch_x_c2r(in, ip, out, op, rows, ax, t, st);
}
static cudaError_t d_cols(const float2* src, float2* dst, long long ps, long long es, int ncols, int nplanes, bool inv,
                          const FcAxis& ax, int cols_log2, int threads, cudaStream_t st) {
  if (t_tc_mode && tc_len(ax.n))
    return FC_TC_CALL(tc_cols, inv ? 1 : 0, src, 0, 0, 0, dst, ps, es, ncols, nplanes, ax, st);
  if (use_fast() && fast_cols_supported(ax.n)) {
    if (src == dst && cols_wide()) return fast_cols_wide(dst, ps, es, ncols, nplanes, inv, ax, st);
    return fast_cols(src, dst, ps, es, ncols, nplanes, inv, ax, st);
  }
  if (use_fast() && src == dst && fast_cols_wide_supported(ax.n))
    return fast_cols_wide(dst, ps, es, ncols, nplanes, inv, ax, st);
  return launch_cols(src, dst, ps, es, ncols, nplanes, inv, ax, cols_log2, threads, st);
}
static cudaError_t d_cols_kx(const float2* kx_spec, long long pitch, int krows, int hy, float2* dst, int ncols,
                             int nplanes, const FcAxis& ax, int cols_log2, int threads, cudaStream_t st) {
  if (t_tc_mode && tc_len(ax.n))
    return FC_TC_CALL(tc_cols, 2, kx_spec, pitch, krows, hy, dst, (long long)ax.n * pitch, pitch, ncols, nplanes, ax,
                      st);
  if (use_fast() && fast_cols_supported(ax.n)) return fast_cols_kx(kx_spec, pitch, krows, hy, dst, ncols, nplanes, ax, st);
  if (use_fast() && fast_cols_wide_supported(ax.n))
    return fast_cols_kx_wide(kx_spec, pitch, krows, hy, dst, ncols, nplanes, ax, st);
  return launch_cols_kx(kx_spec, pitch, krows, hy, dst, ncols, nplanes, ax, cols_log2, threads, st);
}
static cudaError_t d_zconv(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                           float scale, bool conj, const FcAxis& az, int cols_log2, int threads, cudaStream_t st) {
  if (t_tc_mode && !conj && tc_len(az.n))
    return FC_TC_CALL(tc_zconv, S, KXY, pitch, ny, ncols, kplanes, hz, scale, az, st);
  if (use_fast() && fast_cols_supported(az.n)) return fast_zconv(S, KXY, pitch, ny, ncols, kplanes, hz, scale, conj, az, st);
  return launch_zconv(S, KXY, pitch, ny, ncols, kplanes, hz, scale, conj, az, cols_log2, threads, st);
}
static cudaError_t d_zcorr(const float2* X, const float2* G, float2* out, long long pitch, int ny, int ncols, int kz,
                           int hz, float scale, const FcAxis& az, int cols_log2, int threads, cudaStream_t st) {
  if (use_fast() && fast_cols_supported(az.n)) return fast_zcorr(X, G, out, pitch, ny, ncols, kz, hz, scale, az, st);
  return launch_zcorr_crop(X, G, out, pitch, ny, ncols, kz, hz, scale, az, cols_log2, threads, st);
}

// ------------------------------------------------------------------ pass chains
struct Axes {
  FcAxis x, y, z;
};

static Axes axes_for(DevCtx& c, const Geom& g) {
  Axes a;
  a.x = make_axis(c, g.nx);
  a.y = make_axis(c, g.ny);
  a.z = make_axis(c, g.nz);
  return a;
}

// kernel spectrum: x pass of the taps (box) or of the dense kernel
static void enqueue_kernel_x(const Geom& g, const Axes& a, const Tiles& t, const float* d_kernel, char* ws,
                             const Layout& L, cudaStream_t st) {
  if (g.kbox) {
    const long long rows = (long long)g.kplanes * g.krows;
    FC_PASS("kernel_x_r2c", 4.0 * g.kx * rows + 8.0 * g.nxh * rows, st,
            d_x_r2c_box(d_kernel, g.kx, g.kx / 2, (float2*)(ws + L.off_KX), g.pitch, rows, a.x, t, st));
  } else {
    const long long rows = (long long)g.ny * g.nz;
    FC_PASS("kernel_x_r2c", 4.0 * g.nx * rows + 8.0 * g.nxh * rows, st,
            d_x_r2c_dense(d_kernel, g.nx, (float2*)(ws + L.off_KXY), g.pitch, rows, a.x, t, st));
  }
}

// kernel spectrum: y pass over spectrum columns [c0, c0 + w)
static void enqueue_kernel_y(const Geom& g, const Axes& a, const Tiles& t, char* ws, const Layout& L, int c0, int w,
                             cudaStream_t st) {
  float2* KXY = (float2*)(ws + L.off_KXY) + c0;
  if (g.kbox) {
    const double rows = (double)g.kplanes * g.krows;
    FC_PASS("kernel_y_fwd", 8.0 * w * (rows + (double)g.ny * g.kplanes), st,
            d_cols_kx((float2*)(ws + L.off_KX) + c0, g.pitch, g.krows, g.ky / 2, KXY, w, g.kplanes, a.y,
                      t.y_cols_log2, t.threads, st));
  } else {
    FC_PASS("kernel_y_fwd", 16.0 * w * (double)g.ny * g.nz, st,
            d_cols(KXY, KXY, (long long)g.ny * g.pitch, g.pitch, w, g.nz, false, a.y, t.y_cols_log2, t.threads, st));
  }
}

// kernel spectrum for all columns (used where no chunking applies)
static void enqueue_kernel_spectrum(const Geom& g, const Axes& a, const Tiles& t, const float* d_kernel, char* ws,
                                    const Layout& L, cudaStream_t st) {
  enqueue_kernel_x(g, a, t, d_kernel, ws, L, st);
  enqueue_kernel_y(g, a, t, ws, L, 0, g.nxh, st);
}

// Spectrum columns per L2 chunk.  The y-forward, fused z and y-inverse
// passes (and the kernel's y pass) can run chunk by chunk over kx, each chunk
// sized so that its image and kernel spectra fit in a budget of L2 bytes, so
// that a chunk's intermediate results could be re-read from L2 rather than
// HBM.  Measured on GB300 at 512x512x128 this is slower than one launch per
// pass at every budget from 24 to 96 MB (smaller grids, shorter row segments,
// no visible L2 reuse), so it is off unless asked for: FC_L2_CHUNK_MB or
// fc_set_l2_chunk_bytes (-1 = half the device's L2).
static long long g_l2_chunk_bytes = -2;  // -2: read env (default 0 = off)
static int chunk_cols(const Geom& g) {
  if (g_l2_chunk_bytes == -2) {
    const char* e = std::getenv("FC_L2_CHUNK_MB");
    g_l2_chunk_bytes = e ? (long long)(std::atof(e) * 1048576.0) : 0;
  }
  long long budget = g_l2_chunk_bytes;
  if (budget < 0) {
    int dev = 0, l2 = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess) {
      cudaGetLastError();
      l2 = 0;
    }
    budget = (long long)l2 / 2;
  }
  if (budget <= 0) return g.nxh;
  const long long per_col = 8LL * g.ny * (g.nz + g.kplanes);
  long long cw = budget / per_col;
  if (cw >= g.nxh) return g.nxh;
  if (cw < 16) cw = 16;
  const long long n = (g.nxh + cw - 1) / cw;
  cw = ((g.nxh + n - 1) / n + 7) / 8 * 8;
  return (int)std::min<long long>(cw, g.nxh);
}

// forward x and y passes of a real volume into spectrum S
static void enqueue_xy_fwd(const Geom& g, const Axes& a, const Tiles& t, const float* d_in, float2* S,
                           cudaStream_t st, const char* xname, const char* yname) {
  const long long rows = (long long)g.ny * g.nz;
  FC_PASS(xname, 4.0 * g.N() + 8.0 * g.nxh * rows, st, d_x_r2c_dense(d_in, g.nx, S, g.pitch, rows, a.x, t, st));
  FC_PASS(yname, 16.0 * g.nxh * rows, st,
          d_cols(S, S, (long long)g.ny * g.pitch, g.pitch, g.nxh, g.nz, false, a.y, t.y_cols_log2, t.threads,
                      st));
}

// Set by a synchronous host entry point around its enqueue: called just before
// the pass that writes the result, so that the entry can check the earlier
// passes' bounded waits before the caller's buffer is touched.
static thread_local const std::function<void()>* t_before_result_pass = nullptr;
static void before_result_pass() {
  if (t_before_result_pass) (*t_before_result_pass)();
}

static void enqueue_yx_inv(const Geom& g, const Axes& a, const Tiles& t, float2* S, float* d_out, cudaStream_t st,
                           const char* yname, const char* xname) {
  const long long rows = (long long)g.ny * g.nz;
  FC_PASS(yname, 16.0 * g.nxh * rows, st,
          d_cols(S, S, (long long)g.ny * g.pitch, g.pitch, g.nxh, g.nz, true, a.y, t.y_cols_log2, t.threads,
                      st));
  before_result_pass();
  FC_PASS(xname, 4.0 * g.N() + 8.0 * g.nxh * rows, st, d_x_c2r(S, g.pitch, d_out, g.nx, rows, a.x, t, st));
}


// The geometry the passes run on: the reference-arithmetic placement is
// materialised into a dense buffer and then treated as a dense kernel.
static Geom effective_geom(const Geom& g, bool compat) {
  return (compat && g.kbox) ? make_geom(g.nx, g.ny, g.nz, 0, 0, 0, true) : g;
}
static Layout plain_layout(const Geom& g, bool compat) { return conv_layout(effective_geom(g, compat), compat && g.kbox); }

// Enqueue a full convolution.  d_kernel: taps (box) or dense N floats.
static void enqueue_conv_core(const Geom& g0, const Axes& a, const float* d_image, float* d_out,
                              const float* d_kernel, bool compat, char* ws, size_t ws_bytes, cudaStream_t st,
                              const Fork* fork = nullptr);

// FC_FORK=0 keeps the kernel-spectrum passes on the caller's stream
static int g_fork = -1;
static bool use_fork() {
  if (g_fork < 0) {
    const char* e = std::getenv("FC_FORK");
    g_fork = e ? std::atoi(e) : 1;
  }
  return g_fork != 0;
}

static Fork ctx_fork(DevCtx& c) {
  if (!c.side) {
    int lo = 0, hi = 0;
    cuda_check(cudaDeviceGetStreamPriorityRange(&lo, &hi), "cudaDeviceGetStreamPriorityRange");
    // the kernel passes are short and latency-bound: their CTAs go first (measured
    // 2-5% faster per convolution than the default priority on GB300)
    cuda_check(cudaStreamCreateWithPriority(&c.side, cudaStreamNonBlocking, hi), "cudaStreamCreate(side)");
    cuda_check(cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming), "cudaEventCreate");
    cuda_check(cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming), "cudaEventCreate");
    cuda_check(cudaEventCreateWithFlags(&c.ev_aux, cudaEventDisableTiming), "cudaEventCreate");
    cuda_check(cudaEventCreateWithFlags(&c.ev_done, cudaEventDisableTiming), "cudaEventCreate");
  }
  return Fork{c.side, c.ev_fork, c.ev_join, c.ev_aux, c.ev_done};
}

static void enqueue_conv(DevCtx& c, const Geom& g0, const float* d_image, float* d_out, const float* d_kernel,
                         bool compat, char* ws, size_t ws_bytes, cudaStream_t st) {
  if (!use_fork()) {
    enqueue_conv_core(g0, axes_for(c, g0), d_image, d_out, d_kernel, compat, ws, ws_bytes, st);
    return;
  }
  const Fork f = ctx_fork(c);
  enqueue_conv_core(g0, axes_for(c, g0), d_image, d_out, d_kernel, compat, ws, ws_bytes, st, &f);
}

// The pass sequence of one convolution, with the twiddle tables given by the
// caller (a.x.W, a.y.W, a.z.W): enqueues kernels and one memset, allocates
// nothing and creates no CUDA object (profiling events aside).  With a fork,
// the kernel-spectrum passes run on fork->side between two event edges.
static void enqueue_conv_core(const Geom& g0, const Axes& a, const float* d_image, float* d_out,
                              const float* d_kernel, bool compat, char* ws, size_t ws_bytes, cudaStream_t st,
                              const Fork* fork) {
  const Geom g = effective_geom(g0, compat);
  const Layout L = conv_layout(g, compat && g0.kbox);
  if (ws_bytes < L.total) FC_THROW(FC_ERR_NOMEM, "workspace too small");
  const float* ksrc = d_kernel;
  if (compat && g0.kbox) {
    float* dense = (float*)(ws + L.off_dense);
    cuda_check(cudaMemsetAsync(dense, 0, sizeof(float) * (size_t)g.N(), st), "cudaMemsetAsync");
    FC_PASS("kernel_pad_shift_compat", 8.0 * g0.kx * g0.ky * g0.kz, st,
            launch_pad_shift(d_kernel, g0.kx, g0.ky, g0.kz, g0.nx, g0.ny, g0.nz, true, dense, st));
    ksrc = dense;
  }
  const Tiles t = choose_tiles(g);
  float2* S = (float2*)(ws + L.off_S);
  const long long rows = (long long)g.ny * g.nz;
  const long long ps = (long long)g.ny * g.pitch;
  const int cw = chunk_cols(g);
  // the fork point follows the image x pass, whose persistent CTAs take a
  // static share of the tiles each and so must all start together; the
  // kernel passes then overlap the image y pass
  const bool split = fork && cw == g.nxh;
  if (!split) enqueue_kernel_x(g, a, t, ksrc, ws, L, st);
  FC_PASS("image_x_r2c", 4.0 * g.N() + 8.0 * g.nxh * rows, st,
          d_x_r2c_dense(d_image, g.nx, S, g.pitch, rows, a.x, t, st));
  if (split) {
    cuda_check(cudaEventRecord(fork->forked, st), "cudaEventRecord(fork)");
    cuda_check(cudaStreamWaitEvent(fork->side, fork->forked, 0), "cudaStreamWaitEvent(fork)");
    enqueue_kernel_x(g, a, t, ksrc, ws, L, fork->side);
    enqueue_kernel_y(g, a, t, ws, L, 0, g.nxh, fork->side);
    cuda_check(cudaEventRecord(fork->joined, fork->side), "cudaEventRecord(join)");
  }
  for (int c0 = 0; c0 < g.nxh; c0 += cw) {
    const int w = std::min(cw, g.nxh - c0);
    if (!split) enqueue_kernel_y(g, a, t, ws, L, c0, w, st);
    FC_PASS("image_y_fwd", 16.0 * w * (double)rows, st,
            d_cols(S + c0, S + c0, ps, g.pitch, w, g.nz, false, a.y, t.y_cols_log2, t.threads, st));
    if (split) cuda_check(cudaStreamWaitEvent(st, fork->joined, 0), "cudaStreamWaitEvent(join)");
    FC_PASS("zconv", 16.0 * w * (double)rows + 8.0 * w * (double)g.ny * g.kplanes, st,
            d_zconv(S + c0, (const float2*)(ws + L.off_KXY) + c0, g.pitch, g.ny, w, g.kplanes,
                    g.kbox ? g.kz / 2 : 0, 1.0f / (float)g.N(), false, a.z, t.z_cols_log2, t.threads, st));
    FC_PASS("image_y_inv", 16.0 * w * (double)rows, st,
            d_cols(S + c0, S + c0, ps, g.pitch, w, g.nz, true, a.y, t.y_cols_log2, t.threads, st));
  }
  before_result_pass();
  FC_PASS("image_x_c2r", 4.0 * g.N() + 8.0 * g.nxh * rows, st,
          d_x_c2r(S, g.pitch, d_out, g.nx, rows, a.x, t, st));
}

// ------------------------------------------------------------------ adjoint
// Workspace: SG (gradient spectrum), SX (image spectrum), KX/KXY (kernel
// spectrum), GK (kernel-gradient spectrum, kernel planes only) and GKR (its
// real rows before the crop).
struct AdjLayout {
  size_t off_SG, off_SX, off_KX, off_KXY, off_GK, off_GKR, total;
};
static AdjLayout adj_layout(const Geom& g) {
  AdjLayout L;
  const size_t row = (size_t)g.pitch * sizeof(float2);
  size_t o = 0;
  L.off_SG = o;
  o = align256(o + row * g.ny * g.nz);
  L.off_SX = o;
  o = align256(o + row * g.ny * g.nz);
  L.off_KX = o;
  if (g.kbox) o = align256(o + row * g.krows * g.kplanes);
  L.off_KXY = o;
  o = align256(o + row * g.ny * g.kplanes);
  L.off_GK = o;
  o = align256(o + row * g.ny * g.kplanes);
  L.off_GKR = o;
  o = align256(o + sizeof(float) * (size_t)g.nx * g.ny * g.kplanes);
  L.total = o;
  return L;
}

static void enqueue_adjoint(DevCtx& c, const Geom& g, const float* d_x, const float* d_k, const float* d_g,
                            float* d_gx, float* d_gk, char* ws, size_t ws_bytes, cudaStream_t st) {
  const AdjLayout L = adj_layout(g);
  if (ws_bytes < L.total) FC_THROW(FC_ERR_NOMEM, "workspace too small");
  const Tiles t = choose_tiles(g);
  const Axes a = axes_for(c, g);
  float2* SG = (float2*)(ws + L.off_SG);
  float2* SX = (float2*)(ws + L.off_SX);
  float2* GK = (float2*)(ws + L.off_GK);
  float* GKR = (float*)(ws + L.off_GKR);
  const float scale = 1.0f / (float)g.N();
  const int hz = g.kbox ? g.kz / 2 : 0;
  // The kernel spectrum and the kernel-gradient tail run on the side stream:
  // the spectrum from after the gradient's x pass until the fused z pass
  // needs it, the tail once the correlation has produced GK.
  const bool split = use_fork();
  Fork f{};
  if (split) f = ctx_fork(c);
  const cudaStream_t ks = split ? f.side : st;
  const long long rows_all = (long long)g.ny * g.nz;
  FC_PASS("grad_x_r2c", 4.0 * g.N() + 8.0 * g.nxh * rows_all, st,
          d_x_r2c_dense(d_g, g.nx, SG, g.pitch, rows_all, a.x, t, st));
  if (split) {
    cuda_check(cudaEventRecord(f.forked, st), "cudaEventRecord(fork)");
    cuda_check(cudaStreamWaitEvent(f.side, f.forked, 0), "cudaStreamWaitEvent(fork)");
  }
  if (d_gx) {
    Layout kl;
    kl.off_KX = L.off_KX;
    kl.off_KXY = L.off_KXY;
    enqueue_kernel_spectrum(g, a, t, d_k, ws, kl, ks);
    if (split) cuda_check(cudaEventRecord(f.joined, ks), "cudaEventRecord(join)");
  }
  FC_PASS("grad_y_fwd", 16.0 * g.nxh * rows_all, st,
          d_cols(SG, SG, (long long)g.ny * g.pitch, g.pitch, g.nxh, g.nz, false, a.y, t.y_cols_log2, t.threads, st));
  if (d_gk) {
    enqueue_xy_fwd(g, a, t, d_x, SX, st, "image_x_r2c", "image_y_fwd");
    FC_PASS("zcorr_crop", 16.0 * g.nxh * (double)g.ny * g.nz + 8.0 * g.nxh * (double)g.ny * g.kplanes, st,
            d_zcorr(SX, SG, GK, g.pitch, g.ny, g.nxh, g.kplanes, hz, scale, a.z, t.z_cols_log2, t.threads,
                              st));
    if (split) {
      cuda_check(cudaEventRecord(f.aux, st), "cudaEventRecord");
      cuda_check(cudaStreamWaitEvent(ks, f.aux, 0), "cudaStreamWaitEvent");
    }
    NoPipeScope np;
    const long long rows = (long long)g.ny * g.kplanes;
    FC_PASS("grad_kernel_y_inv", 16.0 * g.nxh * rows, ks,
            d_cols(GK, GK, (long long)g.ny * g.pitch, g.pitch, g.nxh, g.kplanes, true, a.y, t.y_cols_log2,
                        t.threads, ks));
    float* dst = g.kbox ? GKR : d_gk;
    FC_PASS("grad_kernel_x_c2r", 8.0 * g.nxh * rows + 4.0 * g.nx * rows, ks,
            d_x_c2r(GK, g.pitch, dst, g.nx, rows, a.x, t, ks));
    if (g.kbox)
      FC_PASS("grad_kernel_crop", 8.0 * g.kx * g.ky * g.kz, ks,
              launch_crop_kernel(GKR, g.nx, g.ny, g.nx, g.kx, g.ky, g.kz, d_gk, ks));
  }
  if (d_gx) {
    if (split) cuda_check(cudaStreamWaitEvent(st, f.joined, 0), "cudaStreamWaitEvent(join)");
    FC_PASS("zconv_conj", 16.0 * g.nxh * (double)g.ny * g.nz + 8.0 * g.nxh * (double)g.ny * g.kplanes, st,
            d_zconv(SG, (const float2*)(ws + L.off_KXY), g.pitch, g.ny, g.nxh, g.kplanes, hz, scale, true, a.z,
                         t.z_cols_log2, t.threads, st));
    enqueue_yx_inv(g, a, t, SG, d_gx, st, "grad_image_y_inv", "grad_image_x_c2r");
  }
  if (split) {
    cuda_check(cudaEventRecord(f.done, ks), "cudaEventRecord");
    cuda_check(cudaStreamWaitEvent(st, f.done, 0), "cudaStreamWaitEvent");
  }
}

// ------------------------------------------------------------------ kernel-spectrum reuse
// The kernel's pruned xy-spectrum KXY ([kplanes][ny][pitch], plane p = image
// plane (p - kz/2) mod nz) depends only on the kernel and the image shape.
// Callers that convolve many images with one kernel (Richardson-Lucy
// iterations, multi-view fusion) compute it once and then run only the five
// image passes.  Buffer: KXY, then the KX rows used while computing it.
static Layout kspec_layout(const Geom& g) {
  Layout L;
  const size_t row = (size_t)g.pitch * sizeof(float2);
  L.off_KXY = 0;
  size_t o = align256(row * g.ny * g.kplanes);
  L.off_KX = o;
  if (g.kbox) o = align256(o + row * g.krows * g.kplanes);
  L.off_S = L.off_dense = L.off_aux = o;
  L.total = o;
  return L;
}
static size_t image_ws_bytes(const Geom& g) { return align256((size_t)g.pitch * sizeof(float2) * g.ny * g.nz); }

static void enqueue_kspec(const Geom& g, const Axes& a, const float* d_kernel, char* kbuf, cudaStream_t st) {
  const Tiles t = choose_tiles(g);
  const Layout L = kspec_layout(g);
  enqueue_kernel_x(g, a, t, d_kernel, kbuf, L, st);
  enqueue_kernel_y(g, a, t, kbuf, L, 0, g.nxh, st);
}

// the five image passes against a ready kernel spectrum (conj: correlation)
static void enqueue_conv_kspec(const Geom& g, const Axes& a, const float* d_image, float* d_out, const float2* KXY,
                               bool conj, char* ws, cudaStream_t st) {
  const Tiles t = choose_tiles(g);
  float2* S = (float2*)ws;
  const long long rows = (long long)g.ny * g.nz;
  const long long ps = (long long)g.ny * g.pitch;
  FC_PASS("image_x_r2c", 4.0 * g.N() + 8.0 * g.nxh * rows, st,
          d_x_r2c_dense(d_image, g.nx, S, g.pitch, rows, a.x, t, st));
  FC_PASS("image_y_fwd", 16.0 * g.nxh * (double)rows, st,
          d_cols(S, S, ps, g.pitch, g.nxh, g.nz, false, a.y, t.y_cols_log2, t.threads, st));
  FC_PASS(conj ? "zconv_conj" : "zconv", 16.0 * g.nxh * (double)rows + 8.0 * g.nxh * (double)g.ny * g.kplanes, st,
          d_zconv(S, KXY, g.pitch, g.ny, g.nxh, g.kplanes, g.kbox ? g.kz / 2 : 0, 1.0f / (float)g.N(), conj, a.z,
                  t.z_cols_log2, t.threads, st));
  FC_PASS("image_y_inv", 16.0 * g.nxh * (double)rows, st,
          d_cols(S, S, ps, g.pitch, g.nxh, g.nz, true, a.y, t.y_cols_log2, t.threads, st));
  FC_PASS("image_x_c2r", 4.0 * g.N() + 8.0 * g.nxh * rows, st, d_x_c2r(S, g.pitch, d_out, g.nx, rows, a.x, t, st));
}

// ------------------------------------------------------------------ Richardson-Lucy deconvolution
// x <- x * correlate(y / conv(x, k), k), the multiplicative update for
// Poisson data with a kernel of unit sum.  The kernel spectrum is computed
// once per call; each iteration is two convolutions against it and two
// pointwise passes.  Workspace: kernel spectrum, image spectrum, one volume.
struct RlLayout {
  size_t off_K, off_S, off_V, total;
};
static RlLayout rl_layout(const Geom& g) {
  RlLayout L;
  L.off_K = 0;
  L.off_S = align256(kspec_layout(g).total);
  L.off_V = align256(L.off_S + image_ws_bytes(g));
  L.total = align256(L.off_V + sizeof(float) * (size_t)g.N());
  return L;
}

static void enqueue_rl(DevCtx& c, const Geom& g, const float* d_y, float* d_x, const float* d_k, int iters,
                       char* ws, size_t wsb, cudaStream_t st) {
  const RlLayout L = rl_layout(g);
  if (wsb < L.total) FC_THROW(FC_ERR_NOMEM, "workspace too small");
  const Axes a = axes_for(c, g);
  char* kbuf = ws + L.off_K;
  const float2* KXY = (const float2*)(kbuf + kspec_layout(g).off_KXY);
  char* S = ws + L.off_S;
  float* V = (float*)(ws + L.off_V);
  const long long n = g.N();
  enqueue_kspec(g, a, d_k, kbuf, st);
  for (int it = 0; it < iters; ++it) {
    enqueue_conv_kspec(g, a, d_x, V, KXY, false, S, st);  // V = conv(x, k)
    FC_PASS("rl_ratio", 12.0 * n, st, launch_rl_ratio(d_y, V, n, st));  // V = y / V
    enqueue_conv_kspec(g, a, V, V, KXY, true, S, st);  // V = correlate(V, k)
    FC_PASS("rl_update", 12.0 * n, st, launch_rl_update(d_x, V, n, st));  // x *= V
  }
}

// ------------------------------------------------------------------ raw transforms
static size_t fft_ws_bytes(const Geom& g) { return align256((size_t)g.pitch * sizeof(float2) * g.ny * g.nz); }

static void enqueue_rfft3d(DevCtx& c, const Geom& g, const float* d_in, float* d_spec, char* ws, size_t wsb,
                           cudaStream_t st) {
  if (wsb < fft_ws_bytes(g)) FC_THROW(FC_ERR_NOMEM, "workspace too small");
  const Tiles t = choose_tiles(g);
  const Axes a = axes_for(c, g);
  float2* S = (float2*)ws;
  enqueue_xy_fwd(g, a, t, d_in, S, st, "fft_x_r2c", "fft_y_fwd");
  // z pass as a column pass over planes of constant y; the result is written
  // into the caller's dense layout (pitch nxh) by a final strided z pass
  FC_PASS("fft_z_fwd", 16.0 * g.nxh * (double)g.ny * g.nz, st,
          d_cols(S, S, g.pitch, (long long)g.ny * g.pitch, g.nxh, g.ny, false, a.z, t.z_cols_log2, t.threads,
                      st));
  cuda_check(cudaMemcpy2DAsync(d_spec, sizeof(float2) * g.nxh, S, sizeof(float2) * g.pitch, sizeof(float2) * g.nxh,
                               (size_t)g.ny * g.nz, cudaMemcpyDeviceToDevice, st),
             "cudaMemcpy2DAsync");
}

static void enqueue_irfft3d(DevCtx& c, const Geom& g, const float* d_spec, float* d_out, char* ws, size_t wsb,
                            cudaStream_t st) {
  if (wsb < fft_ws_bytes(g)) FC_THROW(FC_ERR_NOMEM, "workspace too small");
  const Tiles t = choose_tiles(g);
  const Axes a = axes_for(c, g);
  float2* S = (float2*)ws;
  cuda_check(cudaMemcpy2DAsync(S, sizeof(float2) * g.pitch, d_spec, sizeof(float2) * g.nxh, sizeof(float2) * g.nxh,
                               (size_t)g.ny * g.nz, cudaMemcpyDeviceToDevice, st),
             "cudaMemcpy2DAsync");
  FC_PASS("fft_z_inv", 16.0 * g.nxh * (double)g.ny * g.nz, st,
          d_cols(S, S, g.pitch, (long long)g.ny * g.pitch, g.nxh, g.ny, true, a.z, t.z_cols_log2, t.threads, st));
  enqueue_yx_inv(g, a, t, S, d_out, st, "fft_y_inv", "fft_x_c2r");
}

// ------------------------------------------------------------------ subsampled kernel
// The memory-saving variant whose device product the reference keeps
// (src/convolution3Dfft.cu:65-125) behind a commented-out entry point
// (src/convolution3Dfft.h:58-64): the kernel is transformed at its own size,
// unpadded and unshifted, and each image frequency takes the nearest kernel
// frequency (fc_sub.cuh).  Workspace: S (image spectrum), then K (the
// kernel's spectrum, kx/2+1 columns of its own pitch, ky rows, kz planes).
struct SubLayout {
  size_t off_K, total;
};
static Geom sub_kernel_geom(const Geom& g) { return make_geom(g.kx, g.ky, g.kz, 0, 0, 0, true); }
static SubLayout sub_layout(const Geom& g) {
  SubLayout L;
  L.off_K = image_ws_bytes(g);
  L.total = L.off_K + image_ws_bytes(sub_kernel_geom(g));
  return L;
}

static void enqueue_conv_sub(DevCtx& c, const Geom& g, const float* d_image, float* d_out, const float* d_kernel,
                             char* ws, size_t ws_bytes, cudaStream_t st) {
  const SubLayout L = sub_layout(g);
  if (ws_bytes < L.total) FC_THROW(FC_ERR_NOMEM, "workspace too small");
  const Geom kg = sub_kernel_geom(g);
  const Tiles t = choose_tiles(g), tk = choose_tiles(kg);
  const Axes a = axes_for(c, g), ak = axes_for(c, kg);
  float2* S = (float2*)ws;
  float2* K = (float2*)(ws + L.off_K);
  // the kernel's passes (a few latency-bound launches) run on the side stream
  // beside the image y pass, forked after the image x pass as in the plain
  // convolution, and without the persistent x kernel
  auto kernel_passes = [&](cudaStream_t ks) {
    NoPipeScope np;
    enqueue_xy_fwd(kg, ak, tk, d_kernel, K, ks, "sub_kernel_x_r2c", "sub_kernel_y_fwd");
    FC_PASS("sub_kernel_z_fwd", 16.0 * kg.nxh * (double)kg.ny * kg.nz, ks,
            d_cols(K, K, kg.pitch, (long long)kg.ny * kg.pitch, kg.nxh, kg.ny, false, ak.z, tk.z_cols_log2,
                   tk.threads, ks));
  };
  const long long rows = (long long)g.ny * g.nz;
  FC_PASS("image_x_r2c", 4.0 * g.N() + 8.0 * g.nxh * rows, st,
          d_x_r2c_dense(d_image, g.nx, S, g.pitch, rows, a.x, t, st));
  const bool fork = use_fork();
  Fork f{};
  if (fork) {
    f = ctx_fork(c);
    cuda_check(cudaEventRecord(f.forked, st), "cudaEventRecord(fork)");
    cuda_check(cudaStreamWaitEvent(f.side, f.forked, 0), "cudaStreamWaitEvent(fork)");
    kernel_passes(f.side);
    cuda_check(cudaEventRecord(f.joined, f.side), "cudaEventRecord(join)");
  } else {
    kernel_passes(st);
  }
  FC_PASS("image_y_fwd", 16.0 * g.nxh * (double)rows, st,
          d_cols(S, S, (long long)g.ny * g.pitch, g.pitch, g.nxh, g.nz, false, a.y, t.y_cols_log2, t.threads, st));
  if (fork) cuda_check(cudaStreamWaitEvent(st, f.joined, 0), "cudaStreamWaitEvent(join)");
  SubMap m;
  m.K = K;
  m.kpitch = kg.pitch;
  m.kx = g.kx;
  m.ky = g.ky;
  m.kz = g.kz;
  m.kxh = kg.nxh;
  // r = kernel extent / image extent (src/convolution3Dfft.cu:68-70), IEEE division
  m.rx = (float)g.kx / (float)g.nx;
  m.ry = (float)g.ky / (float)g.ny;
  m.rz = (float)g.kz / (float)g.nz;
  const float scale = 1.0f / (float)g.N();
  const double zbytes = 16.0 * g.nxh * (double)g.ny * g.nz;
  if (use_fast() && fast_cols_supported(g.nz)) {
    FC_PASS("zsub", zbytes, st, fast_zsub(S, g.pitch, g.ny, g.nxh, m, scale, a.z, st));
  } else {
    const long long es = (long long)g.ny * g.pitch;
    FC_PASS("sub_z_fwd", zbytes, st,
            d_cols(S, S, g.pitch, es, g.nxh, g.ny, false, a.z, t.z_cols_log2, t.threads, st));
    FC_PASS("sub_modulate", zbytes, st, launch_sub_modulate(S, g.pitch, g.ny, g.nz, g.nxh, m, scale, st));
    FC_PASS("sub_z_inv", zbytes, st, d_cols(S, S, g.pitch, es, g.nxh, g.ny, true, a.z, t.z_cols_log2, t.threads, st));
  }
  enqueue_yx_inv(g, a, t, S, d_out, st, "image_y_inv", "image_x_c2r");
}

// ------------------------------------------------------------------ host entry points
static void set_device(int dev) {
  int n = 0;
  cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
  if (dev < 0 || dev >= n) FC_THROW(FC_ERR_ARG, "invalid device index " + std::to_string(dev));
  cuda_check(cudaSetDevice(dev), "cudaSetDevice");
}

// Host I/O of the reference-compatible entry points.
//   copy   (0): H2D of image and kernel into device buffers, D2H of the result;
//   direct (1): the image x pass reads the caller's host buffer and the last
//               pass writes the result into it, over the CPU-GPU link, with no
//               staging copies -- for GPUs that access pageable host memory
//               through the host page tables (GB300 with NVLink-C2C); used by
//               the in-place entry only, whose buffer the caller has filled;
//   auto   (2): the default; direct for page-locked (pinned or registered)
//               host buffers, copy for pageable ones -- measured on GB300 at
//               512x512x128: pinned direct 1.67 ms vs copy 1.78 ms, pageable
//               direct 2.24 ms vs copy 1.88 ms per call.
// direct never touches host memory through the GPU on a device that lacks
// pageable-memory access: it falls back to copy there.
// FC_HOST_IO=copy|direct|auto or fc_set_host_io() select it.
static int g_host_io = -1;
static int host_io_mode() {
  if (g_host_io < 0) {
    const char* e = std::getenv("FC_HOST_IO");
    g_host_io = !e ? 2 : (std::strcmp(e, "direct") == 0 ? 1 : (std::strcmp(e, "copy") == 0 ? 0 : 2));
  }
  return g_host_io;
}
static bool device_reads_pageable(int dev) {
  int a = 0, b = 0;
  if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a == 1 && b == 1;
}

static bool host_buffer_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Bounded device waits (pipelined x passes, tensor-map stage of the fused z
// passes): enqueue reads of their expiry counts on st, to be checked after
// the stream's synchronisation by check_device_timeouts.
// The six counts reach c.h_timeouts by one gather kernel writing the
// page-locked buffer through its device address (instead of six small
// device-to-host copies); the addresses are looked up on every call, so that
// nothing stale survives a context that was torn down.  FC_GATHER_COUNTS=0
// builds the copies, for comparison builds.
#ifndef FC_GATHER_COUNTS
#define FC_GATHER_COUNTS 1
#endif
static void enqueue_timeout_reads(DevCtx& c, cudaStream_t st) {
  if (!c.h_timeouts) host_alloc((void**)&c.h_timeouts, 8 * sizeof(unsigned int), "cudaHostAlloc(wait counts)");
  if (FC_GATHER_COUNTS) {
    unsigned int* src[6] = {};
    unsigned int* dst = nullptr;
    if (pipe_timeouts_addr(&src[0]) == cudaSuccess && zconv_timeouts_addr(&src[1]) == cudaSuccess &&
        zadj_timeouts_addr(&src[2]) == cudaSuccess && tc_timeouts_addr_fp16(&src[3]) == cudaSuccess &&
        tc_timeouts_addr_bf16(&src[4]) == cudaSuccess && ycols_timeouts_addr(&src[5]) == cudaSuccess &&
        cudaHostGetDevicePointer((void**)&dst, c.h_timeouts, 0) == cudaSuccess) {
      cuda_check(gather_counts_async(src, 6, dst, st), "timeout count gather");
      return;
    }
    (void)cudaGetLastError();  // a failed lookup falls back to the copies
  }
  cuda_check(pipe_timeouts_read_async(c.h_timeouts, st), "timeout count read");
  cuda_check(zconv_timeouts_read_async(c.h_timeouts + 1, st), "timeout count read");
  cuda_check(zadj_timeouts_read_async(c.h_timeouts + 2, st), "timeout count read");
  cuda_check(tc_timeouts_read_async_fp16(c.h_timeouts + 3, st), "timeout count read");
  cuda_check(tc_timeouts_read_async_bf16(c.h_timeouts + 4, st), "timeout count read");
  cuda_check(ycols_timeouts_read_async(c.h_timeouts + 5, st), "timeout count read");
}
static void check_device_timeouts(DevCtx& c) {
  if (!(c.h_timeouts[0] | c.h_timeouts[1] | c.h_timeouts[2] | c.h_timeouts[3] | c.h_timeouts[4] |
        c.h_timeouts[5]))
    return;
  pipe_timeouts_clear();
  zconv_timeouts_clear();
  zadj_timeouts_clear();
  tc_timeouts_clear_fp16();
  tc_timeouts_clear_bf16();
  ycols_timeouts_clear();
  FC_THROW(FC_ERR_TIMEOUT, "a bounded device wait expired in an asynchronous copy");
}

// Host-pointer convolution used by the three reference-compatible entry points.
static void host_conv(const float* im, float* out, int nx, int ny, int nz, const float* kernel, int kx, int ky,
                      int kz, bool dense, int dev, bool allow_direct = false, bool subsampled = false) {
  if (!im || !out || !kernel) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
  const Geom g = make_geom(nx, ny, nz, kx, ky, kz, dense);
  set_device(dev);
  const bool compat = !subsampled && shift_compat_default() && g.kbox;
  DevCtx& c = ctx_for(dev);
  std::lock_guard<std::mutex> lk(c.mu);
  cudaStream_t st = ctx_stream(c);
  const size_t wsb = subsampled ? sub_layout(g).total : plain_layout(g, compat).total;
  auto run = [&](const float* src, float* dst) {
    if (subsampled)
      enqueue_conv_sub(c, g, src, dst, c.d_ker, (char*)c.ws, c.ws_cap, st);
    else
      enqueue_conv(c, g, src, dst, c.d_ker, compat, (char*)c.ws, c.ws_cap, st);
  };
  const size_t nimg = sizeof(float) * (size_t)g.N();
  const size_t nker = sizeof(float) * (dense ? (size_t)g.N() : (size_t)kx * ky * kz);
  grow(&c.ws, &c.ws_cap, wsb, "cudaMalloc(workspace)");
  grow((void**)&c.d_ker, &c.ker_cap, nker, "cudaMalloc(kernel)");
  cuda_check(cudaMemcpyAsync(c.d_ker, kernel, nker, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync(kernel H2D)");
  // every bounded device wait is checked before the result reaches `out`, so
  // that a failed call leaves the caller's buffer as it was
  auto check_waits = [&] {
    enqueue_timeout_reads(c, st);
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    check_device_timeouts(c);
  };
  const int mode = host_io_mode();
  if (allow_direct && mode != 0 && device_reads_pageable(dev) && (mode == 1 || host_buffer_pinned(im))) {
    // direct: the last pass writes `out` itself; the waits of the passes
    // before it are checked first (one extra synchronisation).  The last
    // pass's own waits (on copies from device memory) are checked after it:
    // a pass whose first wait expires stores nothing, so `out` stays as it
    // was unless a wait expires part-way through that pass.
    const std::function<void()> hook = check_waits;
    {
      HostSrcScope hs(true);
      struct HookScope {
        explicit HookScope(const std::function<void()>* h) { t_before_result_pass = h; }
        ~HookScope() { t_before_result_pass = nullptr; }
      } hk(&hook);
      run(im, out);
    }
    check_waits();
    return;
  }
  grow((void**)&c.d_img, &c.img_cap, nimg, "cudaMalloc(image)");
  cuda_check(cudaMemcpyAsync(c.d_img, im, nimg, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync(image H2D)");
  run(c.d_img, c.d_img);
  check_waits();
  cuda_check(cudaMemcpyAsync(out, c.d_img, nimg, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync(result D2H)");
  cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
}

template <class F>
static int guarded(F&& f) {
  try {
    f();
    return FC_OK;
  } catch (const FcError& e) {
    set_status(e.code, e.msg);
    return e.code;
  } catch (const std::bad_alloc&) {
    set_status(FC_ERR_NOMEM, "host allocation failed");
    return FC_ERR_NOMEM;
  } catch (const std::exception& e) {
    set_status(FC_ERR_CUDA, e.what());
    return FC_ERR_CUDA;
  } catch (...) {
    set_status(FC_ERR_CUDA, "unknown failure");
    return FC_ERR_CUDA;
  }
}

static void* resolve_ws(DevCtx& c, void* d_ws, size_t* bytes, size_t need) {
  if (d_ws) {
    if (*bytes < need) FC_THROW(FC_ERR_NOMEM, "workspace smaller than required");
    if (((uintptr_t)d_ws & 255) != 0) FC_THROW(FC_ERR_ARG, "workspace must be 256-byte aligned");
    return d_ws;
  }
  grow(&c.ws, &c.ws_cap, need, "cudaMalloc(workspace)");
  *bytes = c.ws_cap;
  return c.ws;
}

static void dims3(const int* d, int* a, int* b, int* cc) {
  if (!d) FC_THROW(FC_ERR_ARG, "NULL dimension array");
  *a = d[0];
  *b = d[1];
  *cc = d[2];
}

// ------------------------------------------------------------------ batched convolution
// Many volumes of uneven sizes, each with its own kernel.  Views whose three
// axis lengths all have register-resident kernels run as five passes over the
// whole batch -- x R2C (kernels and images), y forward (kernels and images),
// fused z, y inverse, x C2R -- each pass one persistent launch over a device
// work-list (BTask, fc_batched.cuh) or, where the tuner measured it faster,
// one launch per view.  Other views run the single-volume sequence.  The
// whole sequence is captured once per call signature (shapes, pointers,
// workspace, stream) into a CUDA graph and replayed.

enum BChoice : int { kFatOcc = 0, kFatOne = 1, kPerView = 2 };
constexpr int kBatchStreams = 4;  // streams of the view-concurrent schedule
static const char* const kBPassName[5] = {"batch_x_r2c", "batch_y_fwd", "batch_zconv", "batch_y_inv", "batch_x_c2r"};

struct BatchEntry {
  std::vector<BTask> tasks[5];
  long long total[5] = {0, 0, 0, 0, 0};
  size_t smem[5] = {0, 0, 0, 0, 0};
  double bytes[5] = {0, 0, 0, 0, 0};
  std::vector<int> slow_views;
  std::vector<Geom> g;
  std::vector<size_t> off;
  BTask* d_tasks = nullptr;
  size_t task_off[5] = {0, 0, 0, 0, 0};
  int choice[5] = {kFatOcc, kFatOcc, kFatOcc, kFatOcc, kFatOcc};
  // 0: pass-major (one launch per pass over all views); 1: view-major (each
  // view's passes in turn, its spectra stay in L2); 2: view-concurrent (the
  // views' pass chains on kBatchStreams streams, parallel graph branches);
  // 3: the single-volume pass sequence per view (kernel spectrum forked);
  // 4: those sequences on kBatchStreams streams (parallel graph branches)
  int schedule = 0;
  std::vector<std::vector<std::pair<int, int>>> view_tasks;  // per fast view: (pass, task index)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~BatchEntry() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (d_tasks) cudaFree(d_tasks);
  }
};

static std::mutex g_batch_mu;
static std::map<std::string, std::unique_ptr<BatchEntry>> g_batch;
static int g_use_graphs = -1;
static bool use_graphs() {
  if (g_use_graphs < 0) {
    const char* e = std::getenv("FC_GRAPH");
    g_use_graphs = (e && std::atoi(e) == 0) ? 0 : 1;
  }
  return g_use_graphs == 1;
}

static FcAxis task_axis(const BTask& t) {
  FcAxis a;
  std::memset(&a, 0, sizeof(a));
  a.n = t.n;
  a.W = t.W;
  return a;
}

// one view's tasks of the five passes
static void add_view_tasks(BatchEntry& E, const Geom& g, const Axes& a, const float* img, float* out,
                           const float* taps, char* w, const Layout& L) {
  float2* S = (float2*)(w + L.off_S);
  float2* KX = (float2*)(w + L.off_KX);
  float2* KXY = (float2*)(w + L.off_KXY);
  const long long rows = (long long)g.ny * g.nz;
  const double mc = 8.0 * g.nxh * (double)rows;
  auto mk = [](int mode, int n, const float2* W) {
    BTask t;
    std::memset(&t, 0, sizeof(t));
    t.mode = mode;
    t.n = n;
    t.W = W;
    return t;
  };
  // x R2C: kernel taps (box) and image
  BTask kx = mk(kBRowsBox, g.nx, a.x.W);
  kx.rows = (long long)g.kplanes * g.krows;
  kx.src = taps;
  kx.dst = KX;
  kx.p1 = g.pitch;
  kx.i0 = g.kx;
  kx.i1 = g.kx / 2;
  kx.tiles = batched_row_tiles(g.nx, kx.rows);
  BTask ix = mk(kBRowsDense, g.nx, a.x.W);
  ix.rows = rows;
  ix.src = img;
  ix.p0 = g.nx;
  ix.dst = S;
  ix.p1 = g.pitch;
  ix.tiles = batched_row_tiles(g.nx, rows);
  E.tasks[0].push_back(kx);
  E.tasks[0].push_back(ix);
  E.bytes[0] += 4.0 * g.kx * kx.rows + 8.0 * g.nxh * kx.rows + 4.0 * g.N() + mc;
  // y forward: kernel (from the compact x-spectrum rows) and image
  BTask ky = mk(kBColsKX, g.ny, a.y.W);
  ky.src = KX;
  ky.dst = KXY;
  ky.p0 = (long long)g.ny * g.pitch;
  ky.p1 = g.pitch;
  ky.i0 = g.krows;
  ky.i1 = g.ky / 2;
  ky.ncols = g.nxh;
  ky.rows = g.kplanes;
  ky.tiles = batched_col_tiles(g.ny, g.nxh, g.kplanes);
  BTask iy = mk(kBColsFwd, g.ny, a.y.W);
  iy.dst = S;
  iy.p0 = (long long)g.ny * g.pitch;
  iy.p1 = g.pitch;
  iy.ncols = g.nxh;
  iy.rows = g.nz;
  iy.tiles = batched_col_tiles(g.ny, g.nxh, g.nz);
  E.tasks[1].push_back(ky);
  E.tasks[1].push_back(iy);
  E.bytes[1] += 8.0 * g.nxh * ((double)g.krows * g.kplanes + (double)g.ny * g.kplanes) + 2.0 * mc;
  // fused z
  BTask z = mk(kBZconv, g.nz, a.z.W);
  z.dst = S;
  z.aux = KXY;
  z.p0 = g.pitch;
  z.rows = g.ny;
  z.ncols = g.nxh;
  z.i0 = g.kplanes;
  z.i1 = g.kz / 2;
  z.scale = 1.0f / (float)g.N();
  z.tiles = batched_col_tiles(g.nz, g.nxh, g.ny);
  E.tasks[2].push_back(z);
  E.bytes[2] += 2.0 * mc + 8.0 * g.nxh * (double)g.ny * g.kplanes;
  // y inverse
  BTask yi = iy;
  yi.mode = kBColsInv;
  E.tasks[3].push_back(yi);
  E.bytes[3] += 2.0 * mc;
  // x C2R
  BTask xc = mk(kBRowsC2R, g.nx, a.x.W);
  xc.rows = rows;
  xc.src = S;
  xc.p0 = g.pitch;
  xc.dst = out;
  xc.p1 = g.nx;
  xc.tiles = ix.tiles;
  E.tasks[4].push_back(xc);
  E.bytes[4] += mc + 4.0 * g.N();
}

static int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    n = 1;
  }
  return n;
}

static void launch_task(const BTask& t, int p, cudaStream_t st, bool pipe);

static void launch_pass(BatchEntry& E, int p, int choice, cudaStream_t st) {
  const std::vector<BTask>& T = E.tasks[p];
  if (T.empty()) return;
  if (choice == kPerView) {
    for (const BTask& t : T) launch_task(t, p, st, true);
    return;
  }
  const BTask* d = E.d_tasks + E.task_off[p];
  const int nt = (int)T.size();
  int occ = 1;
  switch (p) {
    case 0: occ = batched_occupancy_rows_fwd(E.smem[p]); break;
    case 1: occ = batched_occupancy_cols_fwd(E.smem[p]); break;
    case 2: occ = batched_occupancy_zconv(E.smem[p]); break;
    case 3: occ = batched_occupancy_cols_inv(E.smem[p]); break;
    default: occ = batched_occupancy_rows_inv(E.smem[p]); break;
  }
  const long long want = (long long)sm_count() * (choice == kFatOne ? 1 : occ);
  const int grid = (int)std::max<long long>(1, std::min<long long>(want, E.total[p]));
  cudaError_t e;
  switch (p) {
    case 0: e = batched_rows_fwd(d, nt, E.total[p], grid, E.smem[p], st); break;
    case 1: e = batched_cols_fwd(d, nt, E.total[p], grid, E.smem[p], st); break;
    case 2: e = batched_zconv(d, nt, E.total[p], grid, E.smem[p], st); break;
    case 3: e = batched_cols_inv(d, nt, E.total[p], grid, E.smem[p], st); break;
    default: e = batched_rows_inv(d, nt, E.total[p], grid, E.smem[p], st); break;
  }
  cuda_check(e, kBPassName[p]);
  ++t_launches;
}

// one task on the single-volume kernel of its length; pipe: the pipelined x
// kernels where they apply (not when views run concurrently: their CTAs take
// a static share of the tiles and must all start together)
static void launch_task(const BTask& t, int p, cudaStream_t st, bool pipe) {
  const FcAxis ax = task_axis(t);
  cudaError_t e = cudaSuccess;
  switch (t.mode) {
    case kBRowsBox:
      e = fast_x_r2c_box((const float*)t.src, t.i0, t.i1, (float2*)t.dst, t.p1, t.rows, ax, st);
      break;
    case kBRowsDense:
      if (pipe && use_pipe() && aligned16(t.src) && t.p0 % 4 == 0)
        e = pipe_x_r2c_dense((const float*)t.src, t.p0, (float2*)t.dst, t.p1, t.rows, ax, st);
      else
        e = fast_x_r2c_dense((const float*)t.src, t.p0, (float2*)t.dst, t.p1, t.rows, ax, st);
      break;
    case kBRowsC2R:
      if (pipe && use_pipe() && aligned16(t.src) && t.p0 % 2 == 0)
        e = pipe_x_c2r((const float2*)t.src, t.p0, (float*)t.dst, t.p1, t.rows, ax, st);
      else
        e = fast_x_c2r((const float2*)t.src, t.p0, (float*)t.dst, t.p1, t.rows, ax, st);
      break;
    case kBColsKX:
      e = fast_cols_kx((const float2*)t.src, t.p1, t.i0, t.i1, (float2*)t.dst, t.ncols, (int)t.rows, ax, st);
      break;
    case kBColsFwd:
    case kBColsInv:
      e = fast_cols((float2*)t.dst, (float2*)t.dst, t.p0, t.p1, t.ncols, (int)t.rows, t.mode == kBColsInv, ax,
                    st);
      break;
    case kBZconv:
      e = fast_zconv((float2*)t.dst, (const float2*)t.aux, t.p0, (int)t.rows, t.ncols, t.i0, t.i1, t.scale, false,
                     ax, st);
      break;
    default:
      break;
  }
  cuda_check(e, kBPassName[p]);
  ++t_launches;
}

static void run_batch(DevCtx& c, BatchEntry& E, const float* const* imgs, float* const* outs,
                      const float* const* kers, char* ws, cudaStream_t st) {
  if (E.schedule == 1) {
    for (const auto& vt : E.view_tasks)
      for (const auto& pt : vt) launch_task(E.tasks[pt.first][pt.second], pt.first, st, true);
  } else if (E.schedule == 3) {
    for (size_t v = 0; v < E.g.size(); ++v)
      if (std::find(E.slow_views.begin(), E.slow_views.end(), (int)v) == E.slow_views.end())
        enqueue_conv(c, E.g[v], imgs[v], outs[v], kers[v], false, ws + E.off[v], plain_layout(E.g[v], false).total,
                     st);
  } else if (E.schedule == 2 || E.schedule == 4) {
    const int P = kBatchStreams;
    while ((int)c.bstreams.size() < P) {
      cudaStream_t s2;
      cuda_check(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking), "cudaStreamCreate(batch)");
      c.bstreams.push_back(s2);
    }
    while ((int)c.bevents.size() < P + 1) {
      cudaEvent_t e2;
      cuda_check(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming), "cudaEventCreate(batch)");
      c.bevents.push_back(e2);
    }
    cuda_check(cudaEventRecord(c.bevents[P], st), "cudaEventRecord");
    for (int i = 0; i < P; ++i) cuda_check(cudaStreamWaitEvent(c.bstreams[i], c.bevents[P], 0), "cudaStreamWaitEvent");
    if (E.schedule == 2) {
      for (size_t v = 0; v < E.view_tasks.size(); ++v)
        for (const auto& pt : E.view_tasks[v])
          launch_task(E.tasks[pt.first][pt.second], pt.first, c.bstreams[v % P], false);
    } else {
      NoPipeScope np;  // the views' x passes run beside each other
      int k = 0;
      for (size_t v = 0; v < E.g.size(); ++v)
        if (std::find(E.slow_views.begin(), E.slow_views.end(), (int)v) == E.slow_views.end())
          enqueue_conv(c, E.g[v], imgs[v], outs[v], kers[v], false, ws + E.off[v],
                       plain_layout(E.g[v], false).total, c.bstreams[k++ % P]);
    }
    for (int i = 0; i < P; ++i) {
      cuda_check(cudaEventRecord(c.bevents[i], c.bstreams[i]), "cudaEventRecord");
      cuda_check(cudaStreamWaitEvent(st, c.bevents[i], 0), "cudaStreamWaitEvent");
    }
  } else {
    for (int p = 0; p < 5; ++p) {
      PassScope ps(kBPassName[p], E.bytes[p], st);
      launch_pass(E, p, E.choice[p], st);
    }
  }
  for (int v : E.slow_views)
    enqueue_conv(c, E.g[v], imgs[v], outs[v], kers[v], false, ws + E.off[v], plain_layout(E.g[v], false).total, st);
}

// ---- tuner: per pass, the fastest of {persistent launch at full occupancy,
// persistent launch with one CTA per SM, one launch per view}, then the
// faster of that pass-major schedule and the view-major one, measured with
// CUDA events on the first call of a new (GPU, view shapes) signature and
// cached in memory and in FC_TUNE_CACHE (default ~/.cache/fc_gb300_tune.txt);
// FC_AUTOTUNE=0 keeps the persistent launches untimed, FC_TUNE_LOG=1 prints
// the measurements.
static std::string tune_path() {
  const char* e = std::getenv("FC_TUNE_CACHE");
  if (e && *e) return e;
  const char* h = std::getenv("HOME");
  return std::string(h ? h : ".") + "/.cache/fc_gb300_tune.txt";
}

static bool tune_lookup(const std::string& sig, int* choice, int* schedule) {
  std::ifstream f(tune_path());
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    std::string k;
    int ch[6];
    if (!(is >> k)) continue;
    if (k != sig) continue;
    bool ok = true;
    for (int i = 0; i < 6; ++i) ok = ok && (bool)(is >> ch[i]);
    if (!ok) continue;
    for (int i = 0; i < 5; ++i) choice[i] = ch[i];
    if (ch[5] < 0 || ch[5] > 4) continue;
    *schedule = ch[5];
    return true;
  }
  return false;
}

static void tune_store(const std::string& sig, const int* choice, int schedule) {
  const std::string path = tune_path();
  const size_t slash = path.find_last_of('/');
  if (slash != std::string::npos) {
    const std::string dir = path.substr(0, slash);
    std::string cmd;  // create the directory without a shell: walk the components
    for (size_t i = 1; i <= dir.size(); ++i)
      if (i == dir.size() || dir[i] == '/') {
        const std::string part = dir.substr(0, i);
        mkdir(part.c_str(), 0755);
      }
  }
  std::ofstream f(path, std::ios::app);
  if (!f) return;
  f << sig;
  for (int i = 0; i < 5; ++i) f << ' ' << choice[i];
  f << ' ' << schedule << '\n';
}

// on unless FC_AUTOTUNE=0
static bool autotune_enabled() {
  const char* e = std::getenv("FC_AUTOTUNE");
  return !e || std::atoi(e) != 0;
}
static bool tune_log() {
  const char* e = std::getenv("FC_TUNE_LOG");
  return e && std::atoi(e) != 0;
}

static void autotune_batch(DevCtx& c, BatchEntry& E, const float* const* imgs, float* const* outs,
                           const float* const* kers, char* ws, cudaStream_t st) {
  cudaEvent_t a, b;
  cuda_check(cudaEventCreate(&a), "cudaEventCreate");
  cuda_check(cudaEventCreate(&b), "cudaEventCreate");
  run_batch(c, E, imgs, outs, kers, ws, st);  // warm: every kernel loaded, caches primed
  for (int p = 0; p < 5; ++p) {
    if (E.tasks[p].empty()) continue;
    float best = 1e30f;
    int best_choice = E.choice[p];
    for (int ch = 0; ch < 3; ++ch) {
      float tmin = 1e30f;
      for (int r = 0; r < 4; ++r) {
        cuda_check(cudaEventRecord(a, st), "cudaEventRecord");
        launch_pass(E, p, ch, st);
        cuda_check(cudaEventRecord(b, st), "cudaEventRecord");
        cuda_check(cudaEventSynchronize(b), "cudaEventSynchronize");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (r > 0) tmin = std::min(tmin, ms);
      }
      if (tune_log()) std::fprintf(stderr, "fc tune %s choice %d: %.1f us\n", kBPassName[p], ch, 1e3 * tmin);
      if (tmin < best) {
        best = tmin;
        best_choice = ch;
      }
    }
    E.choice[p] = best_choice;
  }
  // whole batch: the tuned pass-major schedule against the view-major and view-concurrent ones
  static const char* const kSchedName[5] = {"pass-major", "view-major", "view-concurrent", "plain-per-view",
                                             "plain-concurrent"};
  float t_sched[5] = {1e30f, 1e30f, 1e30f, 1e30f, 1e30f};
  for (int sc = 0; sc < 5; ++sc) {
    E.schedule = sc;
    for (int r = 0; r < 4; ++r) {
      cuda_check(cudaEventRecord(a, st), "cudaEventRecord");
      run_batch(c, E, imgs, outs, kers, ws, st);
      cuda_check(cudaEventRecord(b, st), "cudaEventRecord");
      cuda_check(cudaEventSynchronize(b), "cudaEventSynchronize");
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      if (r > 0) t_sched[sc] = std::min(t_sched[sc], ms);
    }
    if (tune_log()) std::fprintf(stderr, "fc tune schedule %s: %.1f us\n", kSchedName[sc], 1e3 * t_sched[sc]);
  }
  E.schedule = 0;
  for (int sc = 1; sc < 5; ++sc)
    if (t_sched[sc] < t_sched[E.schedule]) E.schedule = sc;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
}

static std::string batch_signature(int nv, const int* dims) {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  std::string name = "gpu";
  if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) name = prop.name;
  for (char& ch : name)
    if (ch == ' ') ch = '_';
  std::ostringstream os;
  os << name << ":v3";  // bumped when the kernels or the schedule set change
  for (int i = 0; i < 6 * nv; ++i) os << (i % 6 == 0 ? ':' : 'x') << dims[i];
  return os.str();
}

// plan of the most recent batched call on this thread (schedule, per-pass choices)
static thread_local int t_batch_schedule = -1;
static thread_local int t_batch_choice[5] = {-1, -1, -1, -1, -1};

static void enqueue_batched(DevCtx& c, int nv, const float* const* imgs, float* const* outs,
                            const float* const* kers, const int* dims, bool compat, char* ws, size_t wsb,
                            cudaStream_t st) {
  // key: shapes, pointers, workspace, stream, device
  std::ostringstream ks;
  ks << c.dev << '|' << (const void*)st << '|' << (const void*)ws << '|' << compat;
  for (int v = 0; v < nv; ++v) {
    for (int i = 0; i < 6; ++i) ks << ',' << dims[6 * v + i];
    ks << '|' << (const void*)imgs[v] << (const void*)outs[v] << (const void*)kers[v];
  }
  const std::string key = ks.str();
  std::lock_guard<std::mutex> lk(g_batch_mu);
  auto it = g_batch.find(key);
  BatchEntry* E = nullptr;
  if (it == g_batch.end() && g_batch.size() >= 32) {
    // bounded cache: drop every entry once 32 signatures have accumulated
    cudaStreamSynchronize(st);
    g_batch.clear();
  }
  if (it == g_batch.end()) {
    auto e = std::make_unique<BatchEntry>();
    size_t off = 0;
    for (int v = 0; v < nv; ++v) {
      const int* d = dims + 6 * v;
      const Geom g = make_geom(d[0], d[1], d[2], d[3], d[4], d[5], false);
      const Layout L = conv_layout(g, false);
      e->g.push_back(g);
      e->off.push_back(off);
      const Axes a = axes_for(c, g);  // twiddles exist before any capture
      // lengths the persistent batched kernels cover (a subset of the single-volume ones)
      const bool fast = !compat && use_fast() && batched_row_tiles(g.nx, 1) > 0 && batched_col_tiles(g.ny, 1, 1) > 0 &&
                        batched_col_tiles(g.nz, 1, 1) > 0;
      if (fast) {
        size_t before[5];
        for (int p = 0; p < 5; ++p) before[p] = e->tasks[p].size();
        add_view_tasks(*e, g, a, imgs[v], outs[v], kers[v], ws + off, L);
        std::vector<std::pair<int, int>> mine;
        for (int p = 0; p < 5; ++p)
          for (size_t i = before[p]; i < e->tasks[p].size(); ++i) mine.push_back({p, (int)i});
        e->view_tasks.push_back(mine);
      } else {
        e->slow_views.push_back(v);
      }
      off += plain_layout(g, compat).total;
    }
    if (off > wsb) FC_THROW(FC_ERR_NOMEM, "workspace too small");
    size_t ntask = 0;
    for (int p = 0; p < 5; ++p) {
      long long t0 = 0;
      size_t sm = 0;
      for (BTask& t : e->tasks[p]) {
        t.tile0 = t0;
        t0 += t.tiles;
        size_t need = (p == 0 || p == 4) ? batched_row_smem(t.n) : batched_col_smem(t.n, p == 2);
        sm = std::max(sm, need);
      }
      if (p == 2) sm += sizeof(float2) * kBatchThreads * 16;
      e->total[p] = t0;
      e->smem[p] = sm;
      e->task_off[p] = ntask;
      ntask += e->tasks[p].size();
    }
    if (ntask) {
      std::vector<BTask> all;
      for (int p = 0; p < 5; ++p) all.insert(all.end(), e->tasks[p].begin(), e->tasks[p].end());
      dev_malloc((void**)&e->d_tasks, sizeof(BTask) * ntask, "cudaMalloc(work-list)");
      cuda_check(cudaMemcpy(e->d_tasks, all.data(), sizeof(BTask) * ntask, cudaMemcpyHostToDevice),
                 "cudaMemcpy(work-list)");
    }
    const std::string sig = batch_signature(nv, dims);
    if (!tune_lookup(sig, e->choice, &e->schedule) && autotune_enabled()) {
      autotune_batch(c, *e, imgs, outs, kers, ws, st);
      tune_store(sig, e->choice, e->schedule);
    }
    E = e.get();
    g_batch[key] = std::move(e);
  } else {
    E = it->second.get();
  }
  t_batch_schedule = E->schedule;
  for (int p = 0; p < 5; ++p) t_batch_choice[p] = E->choice[p];
  if (!use_graphs() || g_prof_on) {
    run_batch(c, *E, imgs, outs, kers, ws, st);
    return;
  }
  if (!E->exec) {
    // capture on the library's own stream (the caller's may be the legacy
    // default stream, which cannot be captured); the graph is then launched
    // on the caller's stream
    struct NoEvents {
      NoEvents() { t_no_events = true; }
      ~NoEvents() { t_no_events = false; }
    } no_events;
    cudaStream_t cs = ctx_stream(c);
    cuda_check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    try {
      run_batch(c, *E, imgs, outs, kers, ws, cs);
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(cs, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    cuda_check(cudaStreamEndCapture(cs, &E->graph), "cudaStreamEndCapture");
    cuda_check(cudaGraphInstantiate(&E->exec, E->graph, 0), "cudaGraphInstantiate");
  }
  cuda_check(cudaGraphLaunch(E->exec, st), "cudaGraphLaunch");
  t_launches += 1;
}

// ------------------------------------------------------------------ scratch-only convolution
// Used by the allocation-free entry point (fc_noalloc.cu).  Layout of the
// scratch: the three twiddle tables, then the convolution workspace.
void record_status(int code, const char* msg) { set_status(code, msg ? msg : ""); }

int conv_in_scratch(const float* d_image, float* d_out, const int* imDim, const float* d_kernel,
                    const int* kernelDim, int flags, char* scratch, size_t scratch_bytes, cudaStream_t st) {
  clear_status();
  return guarded([&] {
    if (!d_image || !d_out || !d_kernel || !scratch) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
    if (flags & (FC_FLAG_TC_FP16 | FC_FLAG_TC_BF16))
      FC_THROW(FC_ERR_UNSUPPORTED, "the allocation-free entry point runs the fp32 path only");
    int nx, ny, nz, kx = 0, ky = 0, kz = 0;
    dims3(imDim, &nx, &ny, &nz);
    const bool dense = flags & FC_FLAG_DENSE_KERNEL;
    if (!dense) dims3(kernelDim, &kx, &ky, &kz);
    const Geom g = make_geom(nx, ny, nz, kx, ky, kz, dense);
    const bool compat = (flags & FC_FLAG_SHIFT_COMPAT) && g.kbox;
    const size_t tw =
        align256(sizeof(float2) * (size_t)(fast_twiddle_count(nx) + fast_twiddle_count(ny) + fast_twiddle_count(nz)));
    const size_t need = tw + plain_layout(g, compat).total;
    if (need > scratch_bytes)
      FC_THROW(FC_ERR_NOMEM, "this convolution needs " + std::to_string(need) + " bytes of scratch; the static scratch "
                             "of the allocation-free entry point holds " + std::to_string(scratch_bytes));
    float2* W = (float2*)scratch;
    Axes a;
    const int n3[3] = {nx, ny, nz};
    FcAxis* ax3[3] = {&a.x, &a.y, &a.z};
    size_t off = 0;
    for (int i = 0; i < 3; ++i) {
      FcAxis& ax = *ax3[i];
      std::memset(&ax, 0, sizeof(ax));
      ax.n = n3[i];
      int r[FC_MAX_STAGES];
      const int ns = plan_radices(n3[i], r, FC_MAX_STAGES);
      if (ns < 0) FC_THROW(FC_ERR_UNSUPPORTED, "no radix plan for length " + std::to_string(n3[i]));
      ax.nst = (n3[i] == 1) ? 0 : ns;
      for (int k = 0; k < ns; ++k) ax.radix[k] = r[k];
      ax.W = W + off;
      cuda_check(launch_make_twiddles(W + off, n3[i], st), "twiddles");
      cuda_check(launch_stage_twiddles(W + off, n3[i], st), "stage twiddles");
      t_launches += 2;
      off += (size_t)fast_twiddle_count(n3[i]);
    }
    struct NoEvents {
      NoEvents() { t_no_events = true; }
      ~NoEvents() { t_no_events = false; }
    } no_events;
    enqueue_conv_core(g, a, d_image, d_out, d_kernel, compat, scratch + tw, scratch_bytes - tw, st);
  });
}

}  // namespace fc

using namespace fc;

// ====================================================================== C ABI
extern "C" {

int fc_last_status(void) { return t_status; }
const char* fc_last_error(void) { return t_error.c_str(); }
void fc_free_result(imageType* p) { delete[] p; }
void fc_set_shift_compat(int on) { g_shift_compat = on ? 1 : 0; }
void fc_set_generic_kernels(int on) { g_generic_only = on ? 1 : 0; }
void fc_set_host_io(int mode) { g_host_io = (mode >= 0 && mode <= 2) ? mode : 2; }
void fc_set_l2_chunk_bytes(long long bytes) { g_l2_chunk_bytes = bytes < 0 ? -1 : bytes; }
const char* fc_version(void) { return "fc-gb300 0.1.0 (sm_103a)"; }
int fc_launch_count(void) { return t_launches; }

int fc_fault_inject(const char* spec) {
  clear_status();
  long long n = 0;
  if (parse_fault_spec(spec, &n) != 0) {
    set_status(FC_ERR_ARG, "fault specification must be \"alloc:n\" (n >= 1) or \"off\"");
    return FC_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_fault_mu);
  g_fault_alloc_at = n;
  g_fault_alloc_seen = 0;
  return FC_OK;
}

int fc_device_wait_status(void* stream) {
  clear_status();
  return guarded([&] {
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    const cudaStream_t st = (cudaStream_t)stream;
    enqueue_timeout_reads(c, st);
    cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    check_device_timeouts(c);
  });
}

int fc_test_set_wait_fault(long long limit_cycles, int skip_copies) {
  clear_status();
  return guarded([&] {
    if (limit_cycles < 0) FC_THROW(FC_ERR_ARG, "limit_cycles must be >= 0 (0 selects the default)");
    (void)ctx_for(current_device());
    cuda_check(pipe_wait_ctl_set(limit_cycles, skip_copies), "wait control (x passes)");
    cuda_check(zconv_wait_ctl_set(limit_cycles, skip_copies), "wait control (fused z pass)");
    cuda_check(zadj_wait_ctl_set(limit_cycles, skip_copies), "wait control (adjoint z pass)");
    cuda_check(ycols_wait_ctl_set(limit_cycles, skip_copies), "wait control (y passes)");
  });
}

int fc_plan_radices(int n, int* radices, int max_stages) {
  if (!radices || max_stages < 1) return -1;
  return plan_radices(n, radices, max_stages);
}

imageType* convolution3DfftCUDA_test(imageType* im, int* imDim, imageType* kernel, int devCUDA) {
  clear_status();
  imageType* out = nullptr;
  const int rc = guarded([&] {
    int d0, d1, d2;
    dims3(imDim, &d0, &d1, &d2);
    if (d0 < 1 || d1 < 1 || d2 < 1) FC_THROW(FC_ERR_ARG, "image dimensions must be positive");
    out = new imageType[(size_t)d0 * d1 * d2];
    host_conv(im, out, d2, d1, d0, kernel, 0, 0, 0, true, devCUDA);
  });
  if (rc != FC_OK) {
    delete[] out;
    return nullptr;
  }
  return out;
}

imageType* convolution3DfftCUDA(imageType* im, int* imDim, imageType* kernel, int* kernelDim, int devCUDA) {
  clear_status();
  imageType* out = nullptr;
  const int rc = guarded([&] {
    int d0, d1, d2, k0, k1, k2;
    dims3(imDim, &d0, &d1, &d2);
    dims3(kernelDim, &k0, &k1, &k2);
    if (d0 < 1 || d1 < 1 || d2 < 1) FC_THROW(FC_ERR_ARG, "image dimensions must be positive");
    out = new imageType[(size_t)d0 * d1 * d2];
    // dims are slowest-first here (index 2 fastest): x = d2, y = d1, z = d0
    host_conv(im, out, d2, d1, d0, kernel, k2, k1, k0, false, devCUDA);
  });
  if (rc != FC_OK) {
    delete[] out;
    return nullptr;
  }
  return out;
}

void convolution3DfftCUDAInPlace(imageType* im, int* imDim, imageType* kernel, int* kernelDim, int devCUDA) {
  clear_status();
  guarded([&] {
    int nx, ny, nz, kx, ky, kz;
    dims3(imDim, &nx, &ny, &nz);
    dims3(kernelDim, &kx, &ky, &kz);
    host_conv(im, im, nx, ny, nz, kernel, kx, ky, kz, false, devCUDA, true);
  });
}

void convolution3DfftCUDAInPlaceSaveMemory(imageType* im, int* imDim, imageType* kernel, int* kernelDim, int devCUDA) {
  clear_status();
  guarded([&] {
    int nx, ny, nz, kx, ky, kz;
    dims3(imDim, &nx, &ny, &nz);
    dims3(kernelDim, &kx, &ky, &kz);
    host_conv(im, im, nx, ny, nz, kernel, kx, ky, kz, false, devCUDA, true, true);
  });
}

int getNumDevicesCUDA(void) {
  clear_status();
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    set_status(FC_ERR_CUDA, "cudaGetDeviceCount failed");
    return 0;
  }
  return n;
}

static int cc_attr(int dev, cudaDeviceAttr which) {
  int v = -1;
  if (cudaDeviceGetAttribute(&v, which, dev) != cudaSuccess) {
    cudaGetLastError();
    set_status(FC_ERR_CUDA, "cudaDeviceGetAttribute failed");
    return -1;
  }
  return v;
}

int getCUDAcomputeCapabilityMajorVersion(int devCUDA) {
  clear_status();
  return cc_attr(devCUDA, cudaDevAttrComputeCapabilityMajor);
}

int getCUDAcomputeCapabilityMinorVersion(int devCUDA) {
  clear_status();
  return cc_attr(devCUDA, cudaDevAttrComputeCapabilityMinor);
}

int selectDeviceWithHighestComputeCapability(void) {
  clear_status();
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    set_status(FC_ERR_CUDA, "cudaGetDeviceCount failed");
    return -1;
  }
  int best = -1, best_cc = 0;
  for (int d = 0; d < n; ++d) {
    const int ma = cc_attr(d, cudaDevAttrComputeCapabilityMajor);
    const int mi = cc_attr(d, cudaDevAttrComputeCapabilityMinor);
    if (ma < 0 || mi < 0) continue;
    const int meta = 10 * ma + mi;  // same ordering as src/standardCUDAfunctions.cu:25
    if (meta > best_cc) {
      best_cc = meta;
      best = d;
    }
  }
  return best;
}

void getNameDeviceCUDA(int devCUDA, char* name) {
  clear_status();
  if (!name) {
    set_status(FC_ERR_ARG, "NULL name buffer");
    return;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, devCUDA) != cudaSuccess) {
    cudaGetLastError();
    std::memset(name, 0, 256);
    set_status(FC_ERR_CUDA, "cudaGetDeviceProperties failed");
    return;
  }
  std::memcpy(name, prop.name, 256);
}

long long int getMemDeviceCUDA(int devCUDA) {
  clear_status();
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, devCUDA) != cudaSuccess) {
    cudaGetLastError();
    set_status(FC_ERR_CUDA, "cudaGetDeviceProperties failed");
    return 0;
  }
  return (long long int)prop.totalGlobalMem;
}

int cuda_version(void) { return CUDART_VERSION; }

int gpu_mem_needed_mb(int* shape, int len) {
  clear_status();
  long long mb = -1;
  guarded([&] {
    if (!shape || len < 1 || len > 3) FC_THROW(FC_ERR_ARG, "shape must have 1 to 3 entries");
    const int nx = shape[len - 1];
    const int ny = len >= 2 ? shape[len - 2] : 1;
    const int nz = len == 3 ? shape[0] : 1;
    const Geom g = make_geom(nx, ny, nz, nx, ny, nz, false);
    const size_t b = plain_layout(g, false).total + 2 * sizeof(float) * (size_t)g.N();
    mb = (long long)(b >> 20);
  });
  return (int)mb;
}

int fc_release_device(int devCUDA) {
  clear_status();
  return guarded([&] {
    std::unique_ptr<DevCtx> c;
    {
      std::lock_guard<std::mutex> lk(g_ctx_mu);
      auto it = g_ctx.find(devCUDA);
      if (it == g_ctx.end()) return;
      c = std::move(it->second);
      g_ctx.erase(it);
    }
    std::lock_guard<std::mutex> lk(c->mu);
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(devCUDA);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->ws);
    cudaFree(c->d_img);
    cudaFree(c->d_ker);
    for (auto& kv : c->twiddles) cudaFree(kv.second);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_aux) cudaEventDestroy(c->ev_aux);
    if (c->ev_done) cudaEventDestroy(c->ev_done);
    for (cudaStream_t s2 : c->bstreams) cudaStreamDestroy(s2);
    for (cudaEvent_t e2 : c->bevents) cudaEventDestroy(e2);
    if (c->h_timeouts) cudaFreeHost(c->h_timeouts);
    cudaSetDevice(prev);
  });
}

size_t fc_conv3d_workspace_bytes(const int* imDim, const int* kernelDim, int flags) {
  clear_status();
  size_t r = 0;
  guarded([&] {
    int nx, ny, nz, kx = 0, ky = 0, kz = 0;
    dims3(imDim, &nx, &ny, &nz);
    const bool dense = flags & FC_FLAG_DENSE_KERNEL;
    if (!dense) dims3(kernelDim, &kx, &ky, &kz);
    const Geom g = make_geom(nx, ny, nz, kx, ky, kz, dense);
    r = plain_layout(g, (flags & FC_FLAG_SHIFT_COMPAT) != 0).total;
  });
  return r;
}

int fc_conv3d_device(const float* d_image, float* d_out, const int* imDim, const float* d_kernel,
                     const int* kernelDim, int flags, void* d_workspace, size_t workspace_bytes, void* stream) {
  clear_status();
  return guarded([&] {
    if (!d_image || !d_out || !d_kernel) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
    if ((flags & FC_FLAG_TC_FP16) && (flags & FC_FLAG_TC_BF16))
      FC_THROW(FC_ERR_ARG, "choose one of FC_FLAG_TC_FP16 and FC_FLAG_TC_BF16");
    struct TcScope {
      explicit TcScope(int m) { t_tc_mode = m; }
      ~TcScope() { t_tc_mode = 0; }
    } tc_scope((flags & FC_FLAG_TC_FP16) ? 1 : (flags & FC_FLAG_TC_BF16) ? 2 : 0);
    int nx, ny, nz, kx = 0, ky = 0, kz = 0;
    dims3(imDim, &nx, &ny, &nz);
    const bool dense = flags & FC_FLAG_DENSE_KERNEL;
    if (!dense) dims3(kernelDim, &kx, &ky, &kz);
    const Geom g = make_geom(nx, ny, nz, kx, ky, kz, dense);
    const bool compat = (flags & FC_FLAG_SHIFT_COMPAT) && g.kbox;
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    size_t wsb = workspace_bytes;
    void* ws = resolve_ws(c, d_workspace, &wsb, plain_layout(g, compat).total);
    enqueue_conv(c, g, d_image, d_out, d_kernel, compat, (char*)ws, wsb, (cudaStream_t)stream);
  });
}

size_t fc_conv3d_subsampled_workspace_bytes(const int* imDim, const int* kernelDim) {
  clear_status();
  size_t r = 0;
  guarded([&] {
    int nx, ny, nz, kx, ky, kz;
    dims3(imDim, &nx, &ny, &nz);
    dims3(kernelDim, &kx, &ky, &kz);
    r = sub_layout(make_geom(nx, ny, nz, kx, ky, kz, false)).total;
  });
  return r;
}

int fc_conv3d_subsampled_device(const float* d_image, float* d_out, const int* imDim, const float* d_kernel,
                                const int* kernelDim, void* d_workspace, size_t workspace_bytes, void* stream) {
  clear_status();
  return guarded([&] {
    if (!d_image || !d_out || !d_kernel) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
    int nx, ny, nz, kx, ky, kz;
    dims3(imDim, &nx, &ny, &nz);
    dims3(kernelDim, &kx, &ky, &kz);
    const Geom g = make_geom(nx, ny, nz, kx, ky, kz, false);
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    size_t wsb = workspace_bytes;
    void* ws = resolve_ws(c, d_workspace, &wsb, sub_layout(g).total);
    enqueue_conv_sub(c, g, d_image, d_out, d_kernel, (char*)ws, wsb, (cudaStream_t)stream);
  });
}

size_t fc_conv3d_adjoint_workspace_bytes(const int* imDim, const int* kernelDim, int flags) {
  clear_status();
  size_t r = 0;
  guarded([&] {
    int nx, ny, nz, kx = 0, ky = 0, kz = 0;
    dims3(imDim, &nx, &ny, &nz);
    const bool dense = flags & FC_FLAG_DENSE_KERNEL;
    if (!dense) dims3(kernelDim, &kx, &ky, &kz);
    r = adj_layout(make_geom(nx, ny, nz, kx, ky, kz, dense)).total;
  });
  return r;
}

// geometry of the kernel-spectrum entry points (no compat placement)
static Geom kspec_geom(const int* imDim, const int* kernelDim, int flags) {
  if (flags & FC_FLAG_SHIFT_COMPAT)
    FC_THROW(FC_ERR_UNSUPPORTED, "kernel-spectrum entry points use the centred placement (no FC_FLAG_SHIFT_COMPAT)");
  if ((flags & FC_FLAG_TC_FP16) && (flags & FC_FLAG_TC_BF16))
    FC_THROW(FC_ERR_ARG, "choose one of FC_FLAG_TC_FP16 and FC_FLAG_TC_BF16");
  int nx, ny, nz, kx = 0, ky = 0, kz = 0;
  dims3(imDim, &nx, &ny, &nz);
  const bool dense = flags & FC_FLAG_DENSE_KERNEL;
  if (!dense) dims3(kernelDim, &kx, &ky, &kz);
  return make_geom(nx, ny, nz, kx, ky, kz, dense);
}
struct TcFlags {
  explicit TcFlags(int flags) { t_tc_mode = (flags & FC_FLAG_TC_FP16) ? 1 : (flags & FC_FLAG_TC_BF16) ? 2 : 0; }
  ~TcFlags() { t_tc_mode = 0; }
};
static void check_align256(const void* p, const char* what) {
  if (((uintptr_t)p & 255) != 0) FC_THROW(FC_ERR_ARG, std::string(what) + " must be 256-byte aligned");
}

size_t fc_kernel_spectrum_bytes(const int* imDim, const int* kernelDim, int flags) {
  clear_status();
  size_t r = 0;
  guarded([&] { r = kspec_layout(kspec_geom(imDim, kernelDim, flags)).total; });
  return r;
}

int fc_kernel_spectrum_device(const float* d_kernel, const int* kernelDim, const int* imDim, int flags, void* d_kspec,
                              size_t kspec_bytes, void* stream) {
  clear_status();
  return guarded([&] {
    if (!d_kernel || !d_kspec) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
    const Geom g = kspec_geom(imDim, kernelDim, flags);
    if (kspec_bytes < kspec_layout(g).total) FC_THROW(FC_ERR_NOMEM, "kernel-spectrum buffer too small");
    check_align256(d_kspec, "kernel-spectrum buffer");
    TcFlags tc(flags);
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    enqueue_kspec(g, axes_for(c, g), d_kernel, (char*)d_kspec, (cudaStream_t)stream);
  });
}

size_t fc_conv3d_kspec_workspace_bytes(const int* imDim) {
  clear_status();
  size_t r = 0;
  guarded([&] {
    int nx, ny, nz;
    dims3(imDim, &nx, &ny, &nz);
    r = image_ws_bytes(make_geom(nx, ny, nz, 1, 1, 1, false));
  });
  return r;
}

int fc_conv3d_kspec_device(const float* d_image, float* d_out, const int* imDim, const void* d_kspec,
                           const int* kernelDim, int flags, void* d_workspace, size_t workspace_bytes, void* stream) {
  clear_status();
  return guarded([&] {
    if (!d_image || !d_out || !d_kspec) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
    const Geom g = kspec_geom(imDim, kernelDim, flags);
    check_align256(d_kspec, "kernel-spectrum buffer");
    TcFlags tc(flags);
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    size_t wsb = workspace_bytes;
    void* ws = resolve_ws(c, d_workspace, &wsb, image_ws_bytes(g));
    enqueue_conv_kspec(g, axes_for(c, g), d_image, d_out, (const float2*)((const char*)d_kspec + kspec_layout(g).off_KXY),
                       (flags & FC_FLAG_CORRELATE) != 0, (char*)ws, (cudaStream_t)stream);
  });
}

size_t fc_rl_workspace_bytes(const int* imDim, const int* kernelDim, int flags) {
  clear_status();
  size_t r = 0;
  guarded([&] { r = rl_layout(kspec_geom(imDim, kernelDim, flags)).total; });
  return r;
}

int fc_rl_deconvolve_device(const float* d_observed, float* d_estimate, const int* imDim, const float* d_kernel,
                            const int* kernelDim, int iterations, int flags, void* d_workspace, size_t workspace_bytes,
                            void* stream) {
  clear_status();
  return guarded([&] {
    if (!d_observed || !d_estimate || !d_kernel) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
    if (iterations < 0) FC_THROW(FC_ERR_ARG, "iterations must be >= 0");
    const Geom g = kspec_geom(imDim, kernelDim, flags);
    TcFlags tc(flags);
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    size_t wsb = workspace_bytes;
    void* ws = resolve_ws(c, d_workspace, &wsb, rl_layout(g).total);
    enqueue_rl(c, g, d_observed, d_estimate, d_kernel, iterations, (char*)ws, wsb, (cudaStream_t)stream);
  });
}

int fc_conv3d_adjoint_device(const float* d_image, const float* d_kernel, const float* d_grad_out,
                             float* d_grad_image, float* d_grad_kernel, const int* imDim, const int* kernelDim,
                             int flags, void* d_workspace, size_t workspace_bytes, void* stream) {
  clear_status();
  return guarded([&] {
    if (!d_grad_out) FC_THROW(FC_ERR_ARG, "NULL gradient");
    if (d_grad_image && !d_kernel) FC_THROW(FC_ERR_ARG, "the image gradient needs the kernel");
    if (d_grad_kernel && !d_image) FC_THROW(FC_ERR_ARG, "the kernel gradient needs the image");
    if (flags & FC_FLAG_SHIFT_COMPAT)
      FC_THROW(FC_ERR_UNSUPPORTED, "the adjoint is defined for the centred placement only");
    int nx, ny, nz, kx = 0, ky = 0, kz = 0;
    dims3(imDim, &nx, &ny, &nz);
    const bool dense = flags & FC_FLAG_DENSE_KERNEL;
    if (!dense) dims3(kernelDim, &kx, &ky, &kz);
    const Geom g = make_geom(nx, ny, nz, kx, ky, kz, dense);
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    size_t wsb = workspace_bytes;
    void* ws = resolve_ws(c, d_workspace, &wsb, adj_layout(g).total);
    if (!d_grad_image && !d_grad_kernel) return;
    enqueue_adjoint(c, g, d_image, d_kernel, d_grad_out, d_grad_image, d_grad_kernel, (char*)ws, wsb,
                    (cudaStream_t)stream);
  });
}

size_t fc_fft3d_workspace_bytes(const int* imDim) {
  clear_status();
  size_t r = 0;
  guarded([&] {
    int nx, ny, nz;
    dims3(imDim, &nx, &ny, &nz);
    r = fft_ws_bytes(make_geom(nx, ny, nz, 0, 0, 0, true));
  });
  return r;
}

int fc_rfft3d_device(const float* d_in, float* d_spec, const int* imDim, void* d_workspace, size_t workspace_bytes,
                     void* stream) {
  clear_status();
  return guarded([&] {
    if (!d_in || !d_spec) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
    int nx, ny, nz;
    dims3(imDim, &nx, &ny, &nz);
    const Geom g = make_geom(nx, ny, nz, 0, 0, 0, true);
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    size_t wsb = workspace_bytes;
    void* ws = resolve_ws(c, d_workspace, &wsb, fft_ws_bytes(g));
    enqueue_rfft3d(c, g, d_in, d_spec, (char*)ws, wsb, (cudaStream_t)stream);
  });
}

int fc_irfft3d_device(const float* d_spec, float* d_out, const int* imDim, void* d_workspace, size_t workspace_bytes,
                      void* stream) {
  clear_status();
  return guarded([&] {
    if (!d_spec || !d_out) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
    int nx, ny, nz;
    dims3(imDim, &nx, &ny, &nz);
    const Geom g = make_geom(nx, ny, nz, 0, 0, 0, true);
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    size_t wsb = workspace_bytes;
    void* ws = resolve_ws(c, d_workspace, &wsb, fft_ws_bytes(g));
    enqueue_irfft3d(c, g, d_spec, d_out, (char*)ws, wsb, (cudaStream_t)stream);
  });
}

int fc_pad_shift_kernel_device(const float* d_kernel, const int* kernelDim, const int* imDim, int flags,
                               float* d_out, void* stream) {
  clear_status();
  return guarded([&] {
    if (!d_kernel || !d_out) FC_THROW(FC_ERR_ARG, "NULL pointer argument");
    int nx, ny, nz, kx, ky, kz;
    dims3(imDim, &nx, &ny, &nz);
    dims3(kernelDim, &kx, &ky, &kz);
    const Geom g = make_geom(nx, ny, nz, kx, ky, kz, false);
    cudaStream_t st = (cudaStream_t)stream;
    cuda_check(cudaMemsetAsync(d_out, 0, sizeof(float) * (size_t)g.N(), st), "cudaMemsetAsync");
    FC_PASS("pad_shift", 8.0 * kx * ky * kz, st,
            launch_pad_shift(d_kernel, kx, ky, kz, nx, ny, nz, (flags & FC_FLAG_SHIFT_COMPAT) != 0, d_out, st));
  });
}

size_t fc_conv3d_batched_workspace_bytes(int n_views, const int* dims, int flags) {
  clear_status();
  size_t r = 0;
  guarded([&] {
    if (n_views < 1 || !dims) FC_THROW(FC_ERR_ARG, "no views");
    for (int v = 0; v < n_views; ++v) {
      const int* d = dims + 6 * v;
      const Geom g = make_geom(d[0], d[1], d[2], d[3], d[4], d[5], false);
      r += plain_layout(g, (flags & FC_FLAG_SHIFT_COMPAT) != 0).total;
    }
  });
  return r;
}

int fc_conv3d_batched_device(int n_views, const float* const* d_images, float* const* d_outs,
                             const float* const* d_kernels, const int* dims, int flags, void* d_workspace,
                             size_t workspace_bytes, void* stream) {
  clear_status();
  return guarded([&] {
    if (n_views < 1 || !d_images || !d_outs || !d_kernels || !dims) FC_THROW(FC_ERR_ARG, "NULL argument");
    const bool compat = (flags & FC_FLAG_SHIFT_COMPAT) != 0;
    std::vector<Geom> gs;
    size_t need = 0;
    for (int v = 0; v < n_views; ++v) {
      if (!d_images[v] || !d_outs[v] || !d_kernels[v])
        FC_THROW(FC_ERR_ARG, "NULL image, output or kernel pointer of view " + std::to_string(v));
      const int* d = dims + 6 * v;
      gs.push_back(make_geom(d[0], d[1], d[2], d[3], d[4], d[5], false));
      need += plain_layout(gs.back(), compat).total;
    }
    DevCtx& c = ctx_for(current_device());
    std::lock_guard<std::mutex> lk(c.mu);
    size_t wsb = workspace_bytes;
    char* ws = (char*)resolve_ws(c, d_workspace, &wsb, need);
    enqueue_batched(c, n_views, d_images, d_outs, d_kernels, dims, compat, ws, wsb, (cudaStream_t)stream);
  });
}

int fc_batched_last_plan(int* choices) {
  if (choices)
    for (int p = 0; p < 5; ++p) choices[p] = t_batch_choice[p];
  return t_batch_schedule;
}

void fc_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_on = on != 0;
}

void fc_profile_only(const char* pass_name) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof_only = pass_name ? pass_name : "";
}

int fc_profile_read(char* names, int name_stride, float* ms, double* bytes, int max) {
  std::vector<ProfRec> recs;
  {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    recs.swap(g_prof);
  }
  int n = 0;
  for (auto& r : recs) {
    cudaEventSynchronize(r.b);
    float t = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
    if (n < max) {
      if (names && name_stride > 0) {
        std::strncpy(names + (size_t)n * name_stride, r.name.c_str(), name_stride - 1);
        names[(size_t)n * name_stride + name_stride - 1] = 0;
      }
      if (ms) ms[n] = t;
      if (bytes) bytes[n] = r.bytes;
      ++n;
    }
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  return n;
}

}  // extern "C"
