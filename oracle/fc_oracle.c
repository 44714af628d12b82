/*
 * CPU oracle for the 3D FFT convolution -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the parts of FourierConvolutionCUDALib that the
 * parity tests check against.  Nothing in the product links or calls this
 * file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load it (through oracle/oracle.py).
 *
 * Every function cites the reference file:line it restates (paths are inside
 * the reference project).  Arrays are C-order float32, x fastest.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/convolution3Dfft.cu:26-38.  diff starts at abs(~0) == 1, so the loop
 * only replaces value when _a_number is an exact multiple; otherwise the
 * result is one multiplier. */
int fco_closest_multiplier(int a_number, int multiplier) {
  int value = 1;
  int max = (a_number + multiplier - 1) / multiplier;
  int diff = abs(~0);
  for (int i = 1; i <= max; ++i) {
    int temp_diff = a_number - (i * multiplier);
    if (abs(temp_diff) < diff) value = i;
  }
  return value * multiplier;
}

/* One thread of fftShiftKernel, src/convolution3Dfft.cu:128-166: tap tid is
 * decomposed with kernelDim_2 fastest, centred by kernelDim_d/2, negative
 * coordinates wrapped once by imDim_d, stored at z + imDim_2*(y + imDim_1*x).
 * Returns the destination index. */
static long long ref_shift_index(long long tid, int kD0, int kD1, int kD2, int iD0, int iD1, int iD2) {
  long long x, y, z, aux;
  z = tid % kD2;
  aux = (tid - z) / kD2;
  y = aux % kD1;
  x = (aux - y) / kD1;
  x -= kD0 / 2;
  y -= kD1 / 2;
  z -= kD2 / 2;
  if (x < 0) x += iD0;
  if (y < 0) y += iD1;
  if (z < 0) z += iD2;
  return z + (long long)iD2 * (y + (long long)iD1 * x);
}

/* The padded kernel of convolution3DfftCUDAInPlace in real [nz][ny][nx] layout:
 *   launch size   src/convolution3Dfft.cu:448-453 (closest_multiplier, 65535 cap)
 *   scatter       src/convolution3Dfft.cu:454-461 (kernelDim[0..2], stack_shape x,y,z)
 *   row copy      src/convolution3Dfft.cu:474-486 (buffer read as [nz][ny][nx])
 * kernelDim = {kx,ky,kz}, imDim = {nx,ny,nz}.  out (N floats) is zeroed here
 * (src/convolution3Dfft.cu:442-443).  Returns 0, or -1 if a tap would land
 * outside the buffer (the reference would write out of bounds). */
int fco_ref_inplace_padded_kernel(const float* kernel, const int* kernelDim, const int* imDim, float* out) {
  const long long K = (long long)kernelDim[0] * kernelDim[1] * kernelDim[2];
  const long long N = (long long)imDim[0] * imDim[1] * imDim[2];
  memset(out, 0, sizeof(float) * (size_t)N);
  long long nthreads = K < 1024 ? K : 1024;
  nthreads = fco_closest_multiplier((int)nthreads, 32);
  long long nblocks = (K + nthreads - 1) / nthreads;
  if (nblocks > 65535) nblocks = 65535;
  const long long covered = nblocks * nthreads < K ? nblocks * nthreads : K;
  for (long long tid = 0; tid < covered; ++tid) {
    const long long d = ref_shift_index(tid, kernelDim[0], kernelDim[1], kernelDim[2], imDim[0], imDim[1], imDim[2]);
    if (d < 0 || d >= N) return -1;
    out[d] = kernel[tid];
  }
  return 0;
}

/* The padded kernel of convolution3DfftCUDA (src/convolution3Dfft.cu:344-348):
 * same scatter with image and kernel dims both slowest-first (index 2 fastest),
 * packed into N floats.  Launch size min(1024,K) threads, 65535-block cap. */
int fco_ref_packed_padded_kernel(const float* kernel, const int* kernelDim, const int* imDim, float* out) {
  const long long K = (long long)kernelDim[0] * kernelDim[1] * kernelDim[2];
  const long long N = (long long)imDim[0] * imDim[1] * imDim[2];
  memset(out, 0, sizeof(float) * (size_t)N);
  const long long nthreads = K < 1024 ? K : 1024;
  long long nblocks = (K + nthreads - 1) / nthreads;
  if (nblocks > 65535) nblocks = 65535;
  const long long covered = nblocks * nthreads < K ? nblocks * nthreads : K;
  for (long long tid = 0; tid < covered; ++tid) {
    const long long d = ref_shift_index(tid, kernelDim[0], kernelDim[1], kernelDim[2], imDim[0], imDim[1], imDim[2]);
    if (d < 0 || d >= N) return -1;
    out[d] = kernel[tid];
  }
  return 0;
}

/* Centred circular placement (the intent of fftShiftKernel): tap (iz,iy,ix)
 * goes to ((iz-kz/2) mod nz, (iy-ky/2) mod ny, (ix-kx/2) mod nx).
 * kernelDim = {kx,ky,kz}, imDim = {nx,ny,nz}. */
int fco_centered_padded_kernel(const float* kernel, const int* kernelDim, const int* imDim, float* out) {
  const int kx = kernelDim[0], ky = kernelDim[1], kz = kernelDim[2];
  const int nx = imDim[0], ny = imDim[1], nz = imDim[2];
  if (kx > nx || ky > ny || kz > nz) return -1;
  memset(out, 0, sizeof(float) * (size_t)nx * ny * nz);
  for (int iz = 0; iz < kz; ++iz)
    for (int iy = 0; iy < ky; ++iy)
      for (int ix = 0; ix < kx; ++ix) {
        int x = ix - kx / 2, y = iy - ky / 2, z = iz - kz / 2;
        if (x < 0) x += nx;
        if (y < 0) y += ny;
        if (z < 0) z += nz;
        out[((long long)z * ny + y) * nx + x] = kernel[((long long)iz * ky + iy) * kx + ix];
      }
  return 0;
}

/* tests/test_algorithms.hpp:10-58: direct-sum convolution with the kernel
 * flipped (:43-45), float accumulator (:18-20, :50), result written only
 * inside [offset, shape-offset) per axis (:22-27).  shape/kshape are
 * {z,y,x} (Boost multi_array order); offset {z,y,x}.  periodic != 0 wraps the
 * image indices (circular convolution over the whole volume; offset ignored).
 * threads > 1 splits the outer z loop with OpenMP. */
void fco_convolve_direct(const float* image, const int* shape, const float* kernel, const int* kshape,
                         float* result, const int* offset, int periodic, int threads) {
  const int nz = shape[0], ny = shape[1], nx = shape[2];
  const int kz = kshape[0], ky = kshape[1], kx = kshape[2];
  const int hz = kz / 2, hy = ky / 2, hx = kx / 2;
  const int oz = periodic ? 0 : offset[0], oy = periodic ? 0 : offset[1], ox = periodic ? 0 : offset[2];
#ifdef _OPENMP
  if (threads < 1) threads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
  for (int image_z = oz; image_z < nz - oz; ++image_z) {
    for (int image_y = oy; image_y < ny - oy; ++image_y) {
      for (int image_x = ox; image_x < nx - ox; ++image_x) {
        float value = 0.f;
        for (int kernel_z = 0; kernel_z < kz; ++kernel_z) {
          int sz = image_z - hz + kernel_z;
          if (periodic) sz = ((sz % nz) + nz) % nz;
          for (int kernel_y = 0; kernel_y < ky; ++kernel_y) {
            int sy = image_y - hy + kernel_y;
            if (periodic) sy = ((sy % ny) + ny) % ny;
            const float* krow = kernel + ((long long)(kz - 1 - kernel_z) * ky + (ky - 1 - kernel_y)) * kx;
            const float* irow = image + ((long long)sz * ny + sy) * nx;
            for (int kernel_x = 0; kernel_x < kx; ++kernel_x) {
              int sx = image_x - hx + kernel_x;
              if (periodic) sx = ((sx % nx) + nx) % nx;
              const float kernel_value = krow[kx - 1 - kernel_x];
              const float image_value = irow[sx];
              value += kernel_value * image_value;
            }
          }
        }
        result[((long long)image_z * ny + image_y) * nx + image_x] = value;
      }
    }
  }
}

/* Direct-sum circular convolution on a crop of output voxels only (for timing
 * the CPU baseline on a bounded sample).  Output crop [z0,z0+cz) x [y0,y0+cy)
 * x [x0,x0+cx) written densely to result (cz*cy*cx floats).  Same arithmetic
 * as fco_convolve_direct with periodic != 0. */
void fco_convolve_direct_crop(const float* image, const int* shape, const float* kernel, const int* kshape,
                              const int* crop0, const int* cropn, float* result, int threads) {
  const int nz = shape[0], ny = shape[1], nx = shape[2];
  const int kz = kshape[0], ky = kshape[1], kx = kshape[2];
  const int hz = kz / 2, hy = ky / 2, hx = kx / 2;
#ifdef _OPENMP
  if (threads < 1) threads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
  for (int cz = 0; cz < cropn[0]; ++cz) {
    const int image_z = crop0[0] + cz;
    for (int cy = 0; cy < cropn[1]; ++cy) {
      const int image_y = crop0[1] + cy;
      for (int cx = 0; cx < cropn[2]; ++cx) {
        const int image_x = crop0[2] + cx;
        float value = 0.f;
        for (int kernel_z = 0; kernel_z < kz; ++kernel_z) {
          const int sz = (((image_z - hz + kernel_z) % nz) + nz) % nz;
          for (int kernel_y = 0; kernel_y < ky; ++kernel_y) {
            const int sy = (((image_y - hy + kernel_y) % ny) + ny) % ny;
            const float* krow = kernel + ((long long)(kz - 1 - kernel_z) * ky + (ky - 1 - kernel_y)) * kx;
            const float* irow = image + ((long long)sz * ny + sy) * nx;
            for (int kernel_x = 0; kernel_x < kx; ++kernel_x) {
              const int sx = (((image_x - hx + kernel_x) % nx) + nx) % nx;
              value += krow[kx - 1 - kernel_x] * irow[sx];
            }
          }
        }
        result[((long long)cz * cropn[1] + cy) * cropn[2] + cx] = value;
      }
    }
  }
}

/* src/convolution3Dfft.cu:41-62: d_Dst[i] = mulAndScale(d_Src[i], d_Dst[i], c)
 * with t = {c*(a.x*b.x - a.y*b.y), c*(a.y*b.x + a.x*b.y)}, a = kernel spectrum
 * (src), b = image spectrum (dst).  Interleaved complex float arrays. */
void fco_modulate_and_normalize(float* dst, const float* src, long long n, float c, int threads) {
#ifdef _OPENMP
  if (threads < 1) threads = 1;
#pragma omp parallel for schedule(static) num_threads(threads)
#endif
  for (long long i = 0; i < n; ++i) {
    const float ax = src[2 * i], ay = src[2 * i + 1];
    const float bx = dst[2 * i], by = dst[2 * i + 1];
    dst[2 * i] = c * (ax * bx - ay * by);
    dst[2 * i + 1] = c * (ay * bx + ax * by);
  }
}

/* src/convolution3Dfft.cu:68-70, :106-108: the kernel index read by image
 * frequencies f = 0..m-1 of an axis of length n, for a kernel of length k:
 * (int)(r*f + 0.5f) % k with r = (float)k / (float)n, the multiply-add rounded
 * once (fmaf) as in the reference's contracted device expression. */
void fco_subsampled_index(int n, int k, int m, int* out) {
  const float r = (float)k / (float)n;
  for (int f = 0; f < m; ++f) out[f] = ((int)fmaf(r, (float)f, 0.5f)) % k;
}

/* tests/test_utils.hpp:76-88: sqrt(sum (data-ref)^2) / n, accumulated in double */
double fco_l2norm(const float* reference, const float* data, long long n) {
  double s = 0.0;
  for (long long i = 0; i < n; ++i) {
    const double d = (double)(data[i] - reference[i]);
    s += d * d;
  }
  return sqrt(s) / (double)n;
}

/* tests/test_utils.hpp:90-108: sqrt(sum (data-ref)^2) / sqrt(sum data^2) */
double fco_l2norm_by_nvidia(const float* reference, const float* data, long long n) {
  double s = 0.0, r = 0.0;
  for (long long i = 0; i < n; ++i) {
    const double d = (double)(data[i] - reference[i]);
    s += d * d;
    r += (double)(data[i] * data[i]); /* float product, double sum (std::inner_product with init 0.) */
  }
  return sqrt(s) / sqrt(r);
}

int fco_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
