// Pass kernels of the 3D FFT convolution on sm_103a.
//
// A convolution is a chain of pencil passes over a half-spectrum S laid out as
// S[z][y][kx] (kx fastest, rows `pitch` complex values apart):
//   x pass  : real rows -> kx spectrum rows (two real rows per complex FFT)
//   y pass  : column tiles of B adjacent kx, FFT along y
//   z pass  : column tiles along z; the image column and the kernel column are
//             transformed together, multiplied (kernel * image / N, the
//             reference's modulateAndNormalize_kernel, src/convolution3Dfft.cu:41-62)
//             and transformed back, so the product spectrum never goes to HBM
//   y, x inverse passes mirror the forward ones.
// The kernel's zero padding and centre shift (the reference's fftShiftKernel,
// src/convolution3Dfft.cu:128-166) is folded into the loads of the kernel's x
// pass: only the rows and planes that hold taps are transformed.
#include <algorithm>

#include "fc_internal.h"
#include "fc_fft.cuh"
#include "fc_sources.cuh"
#include "fc_sub.cuh"

namespace fc {

// ------------------------------------------------------------------ x pass, R2C
// CTA: 2P real rows -> P complex lines z = a + i b -> FFT -> split into the two
// half spectra A[k] = (Z[k] + conj Z[n-k]) / 2, B[k] = (Z[k] - conj Z[n-k]) / (2i).
template <class Src>
__global__ void __launch_bounds__(256) k_x_r2c(Src src, float2* __restrict__ out, long long out_pitch,
                                               long long nrows, FcAxis ax, int pairs_log2) {
  extern __shared__ float2 smem[];
  const int n = ax.n;
  const int ls = n | 1;
  const int P = 1 << pairs_log2;
  float2* A = smem;
  float2* B = smem + P * ls;
  const long long row0 = (long long)blockIdx.x * 2 * P;

  // (line, x) flattened over the CTA: short rows keep every thread busy
  for (int e = threadIdx.x; e < P * n; e += blockDim.x) {
    const int p = e / n, x = e - p * n;
    const long long ra = row0 + 2 * p, rb = ra + 1;
    const float a = ra < nrows ? src.load(ra, x) : 0.f;
    const float b = rb < nrows ? src.load(rb, x) : 0.f;
    A[p * ls + x] = make_float2(a, b);
  }
  __syncthreads();
  const float2* R = fc_fft_lines<false>(A, B, ax, pairs_log2, 1, ls);
  const int nh = n / 2 + 1;
  for (int e = threadIdx.x; e < P * nh; e += blockDim.x) {
    const int p = e / nh, k = e - p * nh;
    const long long ra = row0 + 2 * p, rb = ra + 1;
    const bool va = ra < nrows, vb = rb < nrows;
    const float2 zk = R[p * ls + k];
    const float2 zn = R[p * ls + (k == 0 ? 0 : n - k)];
    const float2 Ak = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
    const float2 Bk = make_float2(0.5f * (zk.y + zn.y), 0.5f * (zn.x - zk.x));
    if (va) out[ra * out_pitch + k] = Ak;
    if (vb) out[rb * out_pitch + k] = Bk;
  }
}

// ------------------------------------------------------------------ x pass, C2R
// Rebuild the full Hermitian line Z[k] = A[k] + i B[k] of two rows (the
// imaginary parts of the DC and Nyquist bins are dropped, as a C2R transform
// does), inverse FFT, real part -> row a, imaginary part -> row b.
__global__ void __launch_bounds__(256) k_x_c2r(const float2* __restrict__ in, long long in_pitch,
                                               float* __restrict__ out, long long out_pitch, long long nrows,
                                               FcAxis ax, int pairs_log2) {
  extern __shared__ float2 smem[];
  const int n = ax.n;
  const int ls = n | 1;
  const int P = 1 << pairs_log2;
  float2* A = smem;
  float2* B = smem + P * ls;
  const long long row0 = (long long)blockIdx.x * 2 * P;
  const int nh = n / 2 + 1;
  const bool even = (n & 1) == 0;

  for (int e = threadIdx.x; e < P * n; e += blockDim.x) {
    const int p = e / n, k = e - p * n;
    const long long ra = row0 + 2 * p, rb = ra + 1;
    const bool va = ra < nrows, vb = rb < nrows;
    const bool lo = k < nh;
    const int kk = lo ? k : n - k;
    float2 a = va ? in[ra * in_pitch + kk] : make_float2(0.f, 0.f);
    float2 b = vb ? in[rb * in_pitch + kk] : make_float2(0.f, 0.f);
    if (kk == 0 || (even && kk == n / 2)) {
      a.y = 0.f;
      b.y = 0.f;
    }
    if (!lo) {
      a.y = -a.y;
      b.y = -b.y;
    }
    A[p * ls + k] = make_float2(a.x - b.y, a.y + b.x);
  }
  __syncthreads();
  const float2* R = fc_fft_lines<true>(A, B, ax, pairs_log2, 1, ls);
  for (int e = threadIdx.x; e < P * n; e += blockDim.x) {
    const int p = e / n, x = e - p * n;
    const long long ra = row0 + 2 * p, rb = ra + 1;
    const bool va = ra < nrows, vb = rb < nrows;
    const float2 z = R[p * ls + x];
    if (va) out[ra * out_pitch + x] = z.x;
    if (vb) out[rb * out_pitch + x] = z.y;
  }
}

template <bool INV, class Src>
__global__ void __launch_bounds__(256) k_cols(Src src, float2* dst, long long ps, long long es, int ncols,
                                              FcAxis ax, int cols_log2) {
  extern __shared__ float2 smem[];
  const int n = ax.n;
  const int Bc = 1 << cols_log2;
  float2* A = smem;
  float2* T = smem + n * Bc;
  const int c0 = blockIdx.x * Bc;
  const int plane = blockIdx.y;
  const int total = n << cols_log2;
#pragma unroll 4
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t & (Bc - 1), j = t >> cols_log2;
    A[t] = (c0 + c < ncols) ? src.load(plane, j, c0 + c) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2* R = fc_fft_lines<INV>(A, T, ax, cols_log2, Bc, 1);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t & (Bc - 1), j = t >> cols_log2;
    if (c0 + c < ncols) dst[(long long)plane * ps + (long long)j * es + c0 + c] = R[t];
  }
}

// ------------------------------------------------------------------ fused z pass
// Tile: Bc adjacent kx columns at one ky, all nz planes.  Smem lines 0..Bc-1 are
// the image columns, Bc..2Bc-1 the kernel columns (line-interleaved layout,
// es = 2Bc).  Kernel plane p of KXY sits at z = (p - hz) mod nz.
template <bool CONJ>
__global__ void __launch_bounds__(256) k_zconv(float2* S, const float2* __restrict__ KXY, long long pitch, int ny,
                                               int ncols, int kplanes, int hz, float scale, FcAxis az,
                                               int cols_log2) {
  extern __shared__ float2 smem[];
  const int nz = az.n;
  const int Bc = 1 << cols_log2;
  const int L = 2 * Bc;
  float2* A = smem;
  float2* T = smem + nz * L;
  const int c0 = blockIdx.x * Bc;
  const int ky = blockIdx.y;
  const long long zs = (long long)ny * pitch;
  const int total = nz << cols_log2;
#pragma unroll 4
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t & (Bc - 1), z = t >> cols_log2;
    const bool ok = c0 + c < ncols;
    A[z * L + c] = ok ? S[z * zs + (long long)ky * pitch + c0 + c] : make_float2(0.f, 0.f);
    int p = z + hz;
    if (p >= nz) p -= nz;
    A[z * L + Bc + c] =
        (ok && p < kplanes) ? KXY[((long long)p * ny + ky) * pitch + c0 + c] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* R = fc_fft_lines<false>(A, T, az, cols_log2 + 1, L, 1);
  float2* O = (R == A) ? T : A;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t & (Bc - 1), z = t >> cols_log2;
    const float2 b = R[z * L + c];        // image spectrum (d_Dst in the reference)
    float2 a = R[z * L + Bc + c];         // kernel spectrum (d_Src in the reference)
    if (CONJ) a.y = -a.y;
    // mulAndScale(a, b, c): {c*(a.x*b.x - a.y*b.y), c*(a.y*b.x + a.x*b.y)}
    R[z * L + c] = make_float2(scale * (a.x * b.x - a.y * b.y), scale * (a.y * b.x + a.x * b.y));
  }
  __syncthreads();
  const float2* Q = fc_fft_lines<true>(R, O, az, cols_log2, L, 1);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t & (Bc - 1), z = t >> cols_log2;
    if (c0 + c < ncols) S[z * zs + (long long)ky * pitch + c0 + c] = Q[z * L + c];
  }
}

// ------------------------------------------------------------------ kernel-gradient z pass
// conj(X) * G * scale along z, inverse z, keep the kz support planes:
// out plane p <- z = (p - hz) mod nz.
__global__ void __launch_bounds__(256) k_zcorr_crop(const float2* __restrict__ X, const float2* __restrict__ G,
                                                    float2* __restrict__ out, long long pitch, int ny, int ncols,
                                                    int kz, int hz, float scale, FcAxis az, int cols_log2) {
  extern __shared__ float2 smem[];
  const int nz = az.n;
  const int Bc = 1 << cols_log2;
  const int L = 2 * Bc;
  float2* A = smem;
  float2* T = smem + nz * L;
  const int c0 = blockIdx.x * Bc;
  const int ky = blockIdx.y;
  const long long zs = (long long)ny * pitch;
  const int total = nz << cols_log2;
#pragma unroll 4
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t & (Bc - 1), z = t >> cols_log2;
    const bool ok = c0 + c < ncols;
    const long long g = z * zs + (long long)ky * pitch + c0 + c;
    A[z * L + c] = ok ? X[g] : make_float2(0.f, 0.f);
    A[z * L + Bc + c] = ok ? G[g] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* R = fc_fft_lines<false>(A, T, az, cols_log2 + 1, L, 1);
  float2* O = (R == A) ? T : A;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int c = t & (Bc - 1), z = t >> cols_log2;
    float2 a = R[z * L + c];       // X
    const float2 b = R[z * L + Bc + c];  // G
    a.y = -a.y;
    R[z * L + c] = make_float2(scale * (a.x * b.x - a.y * b.y), scale * (a.y * b.x + a.x * b.y));
  }
  __syncthreads();
  const float2* Q = fc_fft_lines<true>(R, O, az, cols_log2, L, 1);
  const int totk = kz << cols_log2;
  for (int t = threadIdx.x; t < totk; t += blockDim.x) {
    const int c = t & (Bc - 1), p = t >> cols_log2;
    int z = p - hz;
    if (z < 0) z += nz;
    if (c0 + c < ncols) out[((long long)p * ny + ky) * pitch + c0 + c] = Q[z * L + c];
  }
}

// ------------------------------------------------------------------ pad + shift scatter
__global__ void k_pad_shift_centered(const float* __restrict__ taps, int kx, int ky, int kz, int nx, int ny, int nz,
                                     float* __restrict__ out) {
  const long long K = (long long)kx * ky * kz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < K; t += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(t % kx);
    const long long r = t / kx;
    const int iy = (int)(r % ky);
    const int iz = (int)(r / ky);
    int x = ix - kx / 2, y = iy - ky / 2, z = iz - kz / 2;
    if (x < 0) x += nx;
    if (y < 0) y += ny;
    if (z < 0) z += nz;
    out[((long long)z * ny + y) * nx + x] = taps[t];
  }
}

// The reference's fftShiftKernel (src/convolution3Dfft.cu:128-166) with the
// arguments its in-place entry passes (:454-461): kernelDim_0..2 = {kx,ky,kz},
// imDim_0..2 = {nx,ny,nz}; tap tid is decomposed with kernelDim_2 fastest and
// stored at z + imDim_2*(y + imDim_1*x); the row copy (:474-486) then reads the
// buffer as [nz][ny][nx].  Only taps below the reference's launch size are
// written (its grid is capped at 65535 blocks).
__global__ void k_pad_shift_compat(const float* __restrict__ taps, int kD0, int kD1, int kD2, int iD0, int iD1,
                                   int iD2, long long ntaps, float* __restrict__ out) {
  for (long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x; tid < ntaps;
       tid += (long long)gridDim.x * blockDim.x) {
    long long z = tid % kD2;
    long long aux = (tid - z) / kD2;
    long long y = aux % kD1;
    long long x = (aux - y) / kD1;
    x -= kD0 / 2;
    y -= kD1 / 2;
    z -= kD2 / 2;
    if (x < 0) x += iD0;
    if (y < 0) y += iD1;
    if (z < 0) z += iD2;
    out[z + (long long)iD2 * (y + (long long)iD1 * x)] = taps[tid];
  }
}

// ------------------------------------------------------------------ kernel-gradient crop
// vol: compact real rows; plane p (kz of them) holds z = (p - hz) mod nz, row y of
// plane p at vol + (p*ny_rows + y)*row_pitch.  out[iz][iy][ix] = vol[p=iz][(iy-hy) mod ny][(ix-hx) mod nx].
__global__ void k_crop_kernel(const float* __restrict__ vol, long long row_pitch, int ny, int nx, int kx, int ky,
                              int kz, float* __restrict__ out) {
  const long long K = (long long)kx * ky * kz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < K; t += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(t % kx);
    const long long r = t / kx;
    const int iy = (int)(r % ky);
    const int iz = (int)(r / ky);
    int x = ix - kx / 2, y = iy - ky / 2;
    if (x < 0) x += nx;
    if (y < 0) y += ny;
    out[t] = vol[((long long)iz * ny + y) * row_pitch + x];
  }
}

// ------------------------------------------------------------------ twiddles on the device
// W[k] = exp(-2 pi i k / n) evaluated in double precision (sincospi of the
// exact-as-possible ratio -2k/n) and rounded once to float: the device-side
// twin of the host table, for callers whose twiddles live in static memory.
__global__ void k_make_twiddles(float2* __restrict__ W, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    double sn, cs;
    sincospi(-2.0 * (double)k / (double)n, &sn, &cs);
    W[k] = make_float2((float)cs, (float)sn);
  }
}

// ------------------------------------------------------------------ launchers
static inline size_t row_smem(int n, int pairs_log2) { return (size_t)2 * (1 << pairs_log2) * (n | 1) * sizeof(float2); }

template <class K>
static cudaError_t set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return cudaSuccess;
}

cudaError_t launch_x_r2c_dense(const float* in, long long in_pitch, float2* out, long long out_pitch, long long nrows,
                               const FcAxis& ax, const Tiles& t, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  const size_t sm = row_smem(ax.n, t.x_pairs_log2);
  cudaError_t e = set_smem(k_x_r2c<SrcDense>, sm);
  if (e != cudaSuccess) return e;
  const long long rows_per = 2LL << t.x_pairs_log2;
  const unsigned grid = (unsigned)((nrows + rows_per - 1) / rows_per);
  k_x_r2c<SrcDense><<<grid, t.threads, sm, st>>>(SrcDense{in, in_pitch}, out, out_pitch, nrows, ax, t.x_pairs_log2);
  return cudaGetLastError();
}

cudaError_t launch_x_r2c_box(const float* taps, int kx, int hx, float2* out, long long out_pitch, long long nrows,
                             const FcAxis& ax, const Tiles& t, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  const size_t sm = row_smem(ax.n, t.x_pairs_log2);
  cudaError_t e = set_smem(k_x_r2c<SrcBox>, sm);
  if (e != cudaSuccess) return e;
  const long long rows_per = 2LL << t.x_pairs_log2;
  const unsigned grid = (unsigned)((nrows + rows_per - 1) / rows_per);
  k_x_r2c<SrcBox><<<grid, t.threads, sm, st>>>(SrcBox{taps, kx, hx, ax.n}, out, out_pitch, nrows, ax,
                                               t.x_pairs_log2);
  return cudaGetLastError();
}

cudaError_t launch_x_c2r(const float2* in, long long in_pitch, float* out, long long out_pitch, long long nrows,
                         const FcAxis& ax, const Tiles& t, cudaStream_t st) {
  if (nrows <= 0) return cudaSuccess;
  const size_t sm = row_smem(ax.n, t.x_pairs_log2);
  cudaError_t e = set_smem(k_x_c2r, sm);
  if (e != cudaSuccess) return e;
  const long long rows_per = 2LL << t.x_pairs_log2;
  const unsigned grid = (unsigned)((nrows + rows_per - 1) / rows_per);
  k_x_c2r<<<grid, t.threads, sm, st>>>(in, in_pitch, out, out_pitch, nrows, ax, t.x_pairs_log2);
  return cudaGetLastError();
}

cudaError_t launch_cols(const float2* src, float2* dst, long long ps, long long es, int ncols, int nplanes,
                        bool inverse, const FcAxis& ax, int cols_log2, int threads, cudaStream_t st) {
  if (nplanes <= 0 || ncols <= 0) return cudaSuccess;
  const size_t sm = (size_t)2 * ax.n * (1 << cols_log2) * sizeof(float2);
  dim3 grid((ncols + (1 << cols_log2) - 1) >> cols_log2, nplanes);
  cudaError_t e;
  if (inverse) {
    e = set_smem(k_cols<true, ColPlain>, sm);
    if (e != cudaSuccess) return e;
    k_cols<true, ColPlain><<<grid, threads, sm, st>>>(ColPlain{src, ps, es}, dst, ps, es, ncols, ax, cols_log2);
  } else {
    e = set_smem(k_cols<false, ColPlain>, sm);
    if (e != cudaSuccess) return e;
    k_cols<false, ColPlain><<<grid, threads, sm, st>>>(ColPlain{src, ps, es}, dst, ps, es, ncols, ax, cols_log2);
  }
  return cudaGetLastError();
}

cudaError_t launch_cols_kx(const float2* kx_spec, long long pitch, int krows, int hy, float2* dst, int ncols,
                           int nplanes, const FcAxis& ax, int cols_log2, int threads, cudaStream_t st) {
  if (nplanes <= 0 || ncols <= 0) return cudaSuccess;
  const size_t sm = (size_t)2 * ax.n * (1 << cols_log2) * sizeof(float2);
  cudaError_t e = set_smem(k_cols<false, ColKX>, sm);
  if (e != cudaSuccess) return e;
  dim3 grid((ncols + (1 << cols_log2) - 1) >> cols_log2, nplanes);
  const long long ps = (long long)ax.n * pitch;
  k_cols<false, ColKX><<<grid, threads, sm, st>>>(ColKX{kx_spec, pitch, krows, hy, ax.n}, dst, ps, pitch, ncols, ax,
                                                  cols_log2);
  return cudaGetLastError();
}

cudaError_t launch_zconv(float2* S, const float2* KXY, long long pitch, int ny, int ncols, int kplanes, int hz,
                         float scale, bool conj_kernel, const FcAxis& az, int cols_log2, int threads,
                         cudaStream_t st) {
  if (ny <= 0 || ncols <= 0) return cudaSuccess;
  const size_t sm = (size_t)2 * az.n * (2 << cols_log2) * sizeof(float2);
  dim3 grid((ncols + (1 << cols_log2) - 1) >> cols_log2, ny);
  cudaError_t e;
  if (conj_kernel) {
    e = set_smem(k_zconv<true>, sm);
    if (e != cudaSuccess) return e;
    k_zconv<true><<<grid, threads, sm, st>>>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az, cols_log2);
  } else {
    e = set_smem(k_zconv<false>, sm);
    if (e != cudaSuccess) return e;
    k_zconv<false><<<grid, threads, sm, st>>>(S, KXY, pitch, ny, ncols, kplanes, hz, scale, az, cols_log2);
  }
  return cudaGetLastError();
}

cudaError_t launch_zcorr_crop(const float2* X, const float2* G, float2* out, long long pitch, int ny, int ncols,
                              int kz, int hz, float scale, const FcAxis& az, int cols_log2, int threads,
                              cudaStream_t st) {
  if (ny <= 0 || ncols <= 0) return cudaSuccess;
  const size_t sm = (size_t)2 * az.n * (2 << cols_log2) * sizeof(float2);
  cudaError_t e = set_smem(k_zcorr_crop, sm);
  if (e != cudaSuccess) return e;
  dim3 grid((ncols + (1 << cols_log2) - 1) >> cols_log2, ny);
  k_zcorr_crop<<<grid, threads, sm, st>>>(X, G, out, pitch, ny, ncols, kz, hz, scale, az, cols_log2);
  return cudaGetLastError();
}

int ref_closest_multiplier(int a_number, int multiplier) {
  // src/convolution3Dfft.cu:26-38: the initial difference is abs(~0) == 1, so
  // only an exact multiple replaces the default of one multiplier.
  int value = 1;
  const int mx = (a_number + multiplier - 1) / multiplier;
  for (int i = 1; i <= mx; ++i) {
    const int d = a_number - i * multiplier;
    if ((d < 0 ? -d : d) < 1) value = i;
  }
  return value * multiplier;
}

cudaError_t launch_pad_shift(const float* taps, int kx, int ky, int kz, int nx, int ny, int nz, bool compat,
                             float* out, cudaStream_t st) {
  const long long K = (long long)kx * ky * kz;
  if (K <= 0) return cudaSuccess;
  if (!compat) {
    const unsigned grid = (unsigned)((K + 255) / 256 < 65535 ? (K + 255) / 256 : 65535);
    k_pad_shift_centered<<<grid, 256, 0, st>>>(taps, kx, ky, kz, nx, ny, nz, out);
  } else {
    // thread count and grid cap of src/convolution3Dfft.cu:448-453
    int nthreads = (int)(K < 1024 ? K : 1024);
    nthreads = ref_closest_multiplier(nthreads, 32);
    long long nblocks = (K + nthreads - 1) / nthreads;
    if (nblocks > 65535) nblocks = 65535;
    const long long covered = nblocks * nthreads < K ? nblocks * nthreads : K;
    const unsigned grid = (unsigned)((covered + 255) / 256 < 65535 ? (covered + 255) / 256 : 65535);
    k_pad_shift_compat<<<grid, 256, 0, st>>>(taps, kx, ky, kz, nx, ny, nz, covered, out);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------ Richardson-Lucy pointwise steps
__device__ __forceinline__ float rl_ratio1(float y, float e) { return e > 0.f ? y / e : 0.f; }

__global__ void k_rl_ratio(const float* __restrict__ y, float* __restrict__ v, long long n, bool vec) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long done = 0;
  if (vec) {
    const long long n4 = n / 4;
    const float4* y4 = reinterpret_cast<const float4*>(y);
    float4* v4 = reinterpret_cast<float4*>(v);
    for (long long i = i0; i < n4; i += stride) {
      const float4 a = y4[i];
      float4 e = v4[i];
      e.x = rl_ratio1(a.x, e.x);
      e.y = rl_ratio1(a.y, e.y);
      e.z = rl_ratio1(a.z, e.z);
      e.w = rl_ratio1(a.w, e.w);
      v4[i] = e;
    }
    done = n4 * 4;
  }
  for (long long i = done + i0; i < n; i += stride) v[i] = rl_ratio1(y[i], v[i]);
}

__global__ void k_rl_update(float* __restrict__ x, const float* __restrict__ v, long long n, bool vec) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long done = 0;
  if (vec) {
    const long long n4 = n / 4;
    float4* x4 = reinterpret_cast<float4*>(x);
    const float4* v4 = reinterpret_cast<const float4*>(v);
    for (long long i = i0; i < n4; i += stride) {
      float4 a = x4[i];
      const float4 c = v4[i];
      a.x *= c.x;
      a.y *= c.y;
      a.z *= c.z;
      a.w *= c.w;
      x4[i] = a;
    }
    done = n4 * 4;
  }
  for (long long i = done + i0; i < n; i += stride) x[i] *= v[i];
}

static unsigned pointwise_grid(long long n) {
  const long long b = (n / 4 + 255) / 256;
  return (unsigned)std::max<long long>(1, std::min<long long>(b, 152LL * 16));
}

cudaError_t launch_rl_ratio(const float* y, float* v, long long n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const bool vec = (((uintptr_t)y | (uintptr_t)v) & 15) == 0;
  k_rl_ratio<<<pointwise_grid(n), 256, 0, st>>>(y, v, n, vec);
  return cudaGetLastError();
}

cudaError_t launch_rl_update(float* x, const float* v, long long n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const bool vec = (((uintptr_t)x | (uintptr_t)v) & 15) == 0;
  k_rl_update<<<pointwise_grid(n), 256, 0, st>>>(x, v, n, vec);
  return cudaGetLastError();
}

// subsampled-kernel product over the spectrum (element (z, y, x) of the
// padded layout; the reference's flat index decomposition at :80-84)
__global__ void k_sub_modulate(float2* __restrict__ S, long long pitch, int ny, int nz, int ncols, SubMap m,
                               float scale) {
  const long long n = (long long)nz * ny * ncols;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int x = (int)(i % ncols);
    const long long r = i / ncols;  // row z * ny + y
    const int y = (int)(r % ny), z = (int)(r / ny);
    float2* p = S + r * pitch + x;
    *p = sub_product(SubCol(m, x, y).at(z), *p, scale);
  }
}

cudaError_t launch_sub_modulate(float2* S, long long pitch, int ny, int nz, int ncols, const SubMap& m, float scale,
                                cudaStream_t st) {
  const long long n = (long long)nz * ny * ncols;
  if (n <= 0) return cudaSuccess;
  k_sub_modulate<<<pointwise_grid(n), 256, 0, st>>>(S, pitch, ny, nz, ncols, m, scale);
  return cudaGetLastError();
}

cudaError_t launch_crop_kernel(const float* vol, long long row_pitch, int ny_rows, int nx, int kx, int ky, int kz,
                               float* out, cudaStream_t st) {
  const long long K = (long long)kx * ky * kz;
  if (K <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((K + 255) / 256 < 65535 ? (K + 255) / 256 : 65535);
  k_crop_kernel<<<grid, 256, 0, st>>>(vol, row_pitch, ny_rows, nx, kx, ky, kz, out);
  return cudaGetLastError();
}

namespace {
struct CountSrc {
  unsigned int* p[8];
  int n;
};
__global__ void k_gather_counts(CountSrc s, unsigned int* dst) {
  const int i = (int)threadIdx.x;
  if (i < s.n) dst[i] = *(volatile unsigned int*)s.p[i];
  __threadfence_system();
}
}  // namespace

cudaError_t gather_counts_async(unsigned int* const* src, int n, unsigned int* dst, cudaStream_t st) {
  if (n < 1 || n > 8) return cudaErrorInvalidValue;
  CountSrc s{};
  for (int i = 0; i < n; ++i) s.p[i] = src[i];
  s.n = n;
  k_gather_counts<<<1, 32, 0, st>>>(s, dst);
  return cudaGetLastError();
}

cudaError_t launch_make_twiddles(float2* W, int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_make_twiddles<<<(n + 255) / 256, 256, 0, st>>>(W, n);
  return cudaGetLastError();
}

}  // namespace fc
