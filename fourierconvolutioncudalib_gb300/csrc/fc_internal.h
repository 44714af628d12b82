// Internal declarations shared by the host orchestration (fc_host.cpp) and
// the kernel launchers (fc_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include "fc_axis.h"

namespace fc {

// Geometry of one circular convolution: image nx*ny*nz (x fastest), kernel
// source either a kx*ky*kz box of taps placed by the centred circular shift
// (kmode_box) or an image-sized dense real array (already shifted).
struct Geom {
  int nx, ny, nz;
  int kx, ky, kz;      // box dims (box mode); nx,ny,nz in dense mode
  int nxh;             // nx/2 + 1 complex values per spectrum row
  long long pitch;     // complex values between spectrum rows (>= nxh)
  bool kbox;           // true: box of taps, false: dense N-float kernel
  int kplanes;         // z-planes of the kernel spectrum actually computed (kz or nz)
  int krows;           // rows per kernel plane carried by the x pass (ky or ny)
  long long N() const { return (long long)nx * ny * nz; }
};

struct Tiles {
  int x_pairs_log2;   // row pairs per CTA in the x passes
  int y_cols_log2;    // columns per tile in the y passes
  int z_cols_log2;    // columns per tile in the fused z pass
  int threads;        // threads per CTA
};

// Workspace layout (byte offsets from the workspace base, 256-aligned)
struct Layout {
  size_t off_S, off_KX, off_KXY, off_dense, off_aux, total;
};

// Launch helpers (fc_kernels.cu).  All enqueue on `st`; none synchronise.
// Each returns cudaGetLastError() of its launch(es).
cudaError_t launch_x_r2c_dense(const float* in, long long in_pitch, float2* out, long long out_pitch, long long nrows,
                               const FcAxis& ax, const Tiles& t, cudaStream_t st);
cudaError_t launch_x_r2c_box(const float* taps, int kx, int hx, float2* out, long long out_pitch, long long nrows,
                             const FcAxis& ax, const Tiles& t, cudaStream_t st);
cudaError_t launch_x_c2r(const float2* in, long long in_pitch, float* out, long long out_pitch, long long nrows,
                         const FcAxis& ax, const Tiles& t, cudaStream_t st);
// Column FFT over axis `ax`: element (plane, j, c) at base + plane*ps + j*es + c,
// c in [0, ncols).  In place when src == dst.
cudaError_t launch_cols(const float2* src, float2* dst, long long ps, long long es, int ncols, int nplanes,
                        bool inverse, const FcAxis& ax, int cols_log2, int threads, cudaStream_t st);
// Kernel y pass: source rows are the compact x-spectrum rows iy in [0,krows) of
// each plane, y maps to iy = (y + hy) mod ny (rows outside are zero).
cudaError_t launch_cols_kx(const float2* kx_spec, long long pitch, int krows, int hy, float2* dst, int ncols,
                           int nplanes, const FcAxis& ax, int cols_log2, int threads, cudaStream_t st);
// Fused z pass: z-forward of the image column and the kernel column, the
// reference's modulate-and-normalise (kernel * image * scale), z-inverse.
// conj_kernel: multiply by conj(kernel spectrum) (adjoint / correlation).
cudaError_t launch_zconv(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                         float scale, bool conj_kernel, const FcAxis& az, int cols_log2, int threads,
                         cudaStream_t st);
// Kernel-gradient z pass: z-forward of image spectrum X and gradient spectrum G
// columns, conj(X) * G * scale, z-inverse, and keep only the kz planes of the
// kernel support: out plane p <- z = (p - hz) mod nz.
cudaError_t launch_zcorr_crop(const float2* X, const float2* G, float2* out, long long pitch, int ny, int ncols,
                              int kz, int hz, float scale, const FcAxis& az, int cols_log2, int threads,
                              cudaStream_t st);
// Scatter of the kernel taps into a dense zeroed N-float buffer (x fastest).
//   compat = false : centred circular shift
//   compat = true  : the reference's fftShiftKernel arithmetic as called from
//                    its in-place entry point
cudaError_t launch_pad_shift(const float* taps, int kx, int ky, int kz, int nx, int ny, int nz, bool compat,
                             float* out, cudaStream_t st);
// Crop/gather for the kernel gradient: out[iz][iy][ix] = vol[(iz-hz)%nz][(iy-hy)%ny][(ix-hx)%nx]
// from a real volume whose rows have `pitch` floats and whose planes are
// given by a compact array of kz planes (plane p holds z = (p - hz) mod nz).
// Richardson-Lucy pointwise steps over n floats: v = y / v where v > 0 (else
// 0); x = x * v
cudaError_t launch_rl_ratio(const float* y, float* v, long long n, cudaStream_t st);
cudaError_t launch_rl_update(float* x, const float* v, long long n, cudaStream_t st);
cudaError_t launch_crop_kernel(const float* vol, long long row_pitch, int ny_rows, int nx, int kx, int ky, int kz,
                               float* out, cudaStream_t st);

// Subsampled-kernel product (src/convolution3Dfft.cu:65-125): the kernel's
// spectrum at its own size (kx/2+1 columns of pitch kpitch, ky rows, kz
// planes; unshifted taps), read at the nearest kernel frequency of each image
// frequency (fc_sub.cuh).  r = k / n per axis, in float32.
struct SubMap {
  const float2* K;
  long long kpitch;
  int kx, ky, kz, kxh;
  float rx, ry, rz;
};
// S[z][y][x] = scale * (coeff * S) over nz planes of ny rows of ncols columns (pitch)
cudaError_t launch_sub_modulate(float2* S, long long pitch, int ny, int nz, int ncols, const SubMap& m, float scale,
                                cudaStream_t st);

// Register-resident fast path for power-of-two lengths (fc_fast_rows.cu,
// fc_fast_cols.cu).  Same contracts as the generic launchers above; they
// return cudaErrorNotSupported for lengths they do not cover.
bool fast_rows_supported(int n);
bool fast_cols_supported(int n);
cudaError_t fast_x_r2c_dense(const float* in, long long in_pitch, float2* out, long long out_pitch, long long nrows,
                             const FcAxis& ax, cudaStream_t st);
cudaError_t fast_x_r2c_box(const float* taps, int kx, int hx, float2* out, long long out_pitch, long long nrows,
                           const FcAxis& ax, cudaStream_t st);
cudaError_t fast_x_c2r(const float2* in, long long in_pitch, float* out, long long out_pitch, long long nrows,
                       const FcAxis& ax, cudaStream_t st);
cudaError_t fast_cols(const float2* src, float2* dst, long long ps, long long es, int ncols, int nplanes, bool inverse,
                      const FcAxis& ax, cudaStream_t st);
// Axis twiddle tables: W[0..n) followed, for lengths of the register-resident
// kernels, by their stage-twiddle tables (fc_fast.cuh, Plan<N>::tab_off).
// fast_twiddle_count(n) is the table length in float2 entries (n for other
// lengths); launch_stage_twiddles fills the stage part from W[0..n).
long long fast_twiddle_count(int n);
cudaError_t launch_stage_twiddles(float2* W, int n, cudaStream_t st);

// Pipelined x passes (fc_fast_pipe.cu): persistent CTAs with bulk
// asynchronous tile copies.  in must be device memory, 16-byte aligned, with
// rows of a multiple of 16 bytes.  pipe_timeouts_read_async() enqueues a read
// of the number of bounded waits that expired into page-locked host memory;
// pipe_timeouts_clear() resets it.
cudaError_t pipe_x_r2c_dense(const float* in, long long in_pitch, float2* out, long long out_pitch, long long nrows,
                             const FcAxis& ax, cudaStream_t st);
cudaError_t pipe_x_c2r(const float2* in, long long in_pitch, float* out, long long out_pitch, long long nrows,
                       const FcAxis& ax, cudaStream_t st);
cudaError_t pipe_timeouts_read_async(unsigned int* dst, cudaStream_t st);
void pipe_timeouts_clear();
// the device address of each translation unit's count (current device), for
// gather_counts_async
cudaError_t pipe_timeouts_addr(unsigned int** p);
cudaError_t zconv_timeouts_addr(unsigned int** p);
cudaError_t zadj_timeouts_addr(unsigned int** p);
cudaError_t ycols_timeouts_addr(unsigned int** p);
// one kernel copies n counts (device addresses) to dst (device-visible memory)
cudaError_t gather_counts_async(unsigned int* const* src, int n, unsigned int* dst, cudaStream_t st);
// the same for the fused z passes' tensor-map stage copies (plain and
// conjugate-kernel kernels)
cudaError_t zconv_timeouts_read_async(unsigned int* dst, cudaStream_t st);
void zconv_timeouts_clear();
cudaError_t zadj_timeouts_read_async(unsigned int* dst, cudaStream_t st);
void zadj_timeouts_clear();
// wait control of the bounded waits of each translation unit with bounded waits
// (limit in clock cycles, 0 = the default of about one second; skip_copies: the
// test switch that arms barriers without issuing their copies), current device
cudaError_t pipe_wait_ctl_set(long long limit, int skip_copies);
cudaError_t zconv_wait_ctl_set(long long limit, int skip_copies);
cudaError_t zadj_wait_ctl_set(long long limit, int skip_copies);
// the persistent tensor-map y passes (fc_fast_cols.cu; power-of-two lengths >= 512, FC_YPIPE=0/1 overrides)
cudaError_t ycols_timeouts_read_async(unsigned int* dst, cudaStream_t st);
void ycols_timeouts_clear();
cudaError_t ycols_wait_ctl_set(long long limit, int skip_copies);
// resolve the tensor-map encoder of the fused z pass's stage copy (host; call
// outside stream capture, e.g. when a device context is created)
void zstage_prepare();
// in-place y pass on wide tiles (fast::ColGeomWide); covers the column
// lengths plus FC_WIDE_ONLY_SIZES
bool fast_cols_wide_supported(int n);
// kernel y pass on wide tiles for the FC_WIDE_ONLY_SIZES lengths
cudaError_t fast_cols_kx_wide(const float2* kx_spec, long long pitch, int krows, int hy, float2* dst, int ncols,
                              int nplanes, const FcAxis& ax, cudaStream_t st);
cudaError_t fast_cols_wide(float2* S, long long ps, long long es, int ncols, int nplanes, bool inverse,
                           const FcAxis& ax, cudaStream_t st);
cudaError_t fast_cols_kx(const float2* kx_spec, long long pitch, int krows, int hy, float2* dst, int ncols,
                         int nplanes, const FcAxis& ax, cudaStream_t st);
cudaError_t fast_zconv(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                       float scale, bool conj_kernel, const FcAxis& az, cudaStream_t st);
cudaError_t fast_zcorr(const float2* X, const float2* G, float2* out, long long pitch, int ny, int ncols, int kz,
                       int hz, float scale, const FcAxis& az, cudaStream_t st);
// fused subsampled-kernel z pass: z forward, launch_sub_modulate's product, z inverse
cudaError_t fast_zsub(float2* S, long long pitch, int ny, int ncols, const SubMap& m, float scale, const FcAxis& az,
                      cudaStream_t st);

// Tensor-core precision mode (fc_tc.cu, compiled for fp16 and for bf16):
// register-resident kernels whose radix-16 stages run on the tcgen05 tensor
// cores, lengths 128, 256, 512, 1024.  tc_cols mode: 0 forward, 1 inverse,
// 2 kernel forward from the compact x-spectrum rows.  tc_x_r2c: taps != NULL
// selects the kernel-tap source (kx, hx), else the dense rows `in`.
// tc_timeouts_*: the count of expired waits on the MMA barrier.
#define FC_TC_DECL(sfx)                                                                                           \
  cudaError_t tc_x_r2c##sfx(const float* in, long long in_pitch, const float* taps, int kx, int hx, float2* out,   \
                            long long out_pitch, long long nrows, const FcAxis& ax, cudaStream_t st);               \
  cudaError_t tc_x_c2r##sfx(const float2* in, long long in_pitch, float* out, long long out_pitch, long long nrows, \
                            const FcAxis& ax, cudaStream_t st);                                                     \
  cudaError_t tc_cols##sfx(int mode, const float2* src, long long src_pitch, int krows, int hy, float2* dst,        \
                           long long ps, long long es, int ncols, int nplanes, const FcAxis& ax, cudaStream_t st);  \
  cudaError_t tc_zconv##sfx(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,  \
                            float scale, const FcAxis& az, cudaStream_t st);                                         \
  cudaError_t tc_timeouts_read_async##sfx(unsigned int* dst, cudaStream_t st);                                       \
  cudaError_t tc_timeouts_addr##sfx(unsigned int** p);                                                               \
  void tc_timeouts_clear##sfx();
FC_TC_DECL(_fp16)
FC_TC_DECL(_bf16)
#undef FC_TC_DECL

// W[k] = exp(-2 pi i k / n) computed on the device (double precision, rounded once)
cudaError_t launch_make_twiddles(float2* W, int n, cudaStream_t st);

// Plain convolution (fc_conv3d_device semantics) whose twiddle tables and
// workspace are carved out of caller-owned device scratch; allocates nothing.
// Sets the thread's status and returns it.
int conv_in_scratch(const float* d_image, float* d_out, const int* imDim, const float* d_kernel,
                    const int* kernelDim, int flags, char* scratch, size_t scratch_bytes, cudaStream_t st);
// record a failure of the caller's own set-up in the thread's status
void record_status(int code, const char* msg);

// reference thread-count helper (src/convolution3Dfft.cu:26-38) restated for
// the compat scatter's grid truncation
int ref_closest_multiplier(int a_number, int multiplier);

}  // namespace fc
