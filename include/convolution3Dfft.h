/*
 * Public C ABI of libFourierConvolutionCUDALib.so (GB300 / sm_103a build).
 *
 * The first block re-declares, with identical signatures and argument meaning,
 * every export of the reference header src/convolution3Dfft.h (lines 29-84 of
 * FourierConvolutionCUDALib), so that existing JNA / C / C++ callers link and
 * run unchanged.  Differences in behaviour are confined to error handling: no
 * function of this library calls exit() or lets a C++ exception cross the ABI.
 * A failed call records a status and message that fc_last_status() /
 * fc_last_error() return (thread-local).
 *
 * Layout (same as the reference): images are C-order float32, x fastest.
 *   convolution3DfftCUDAInPlace : imDim = {nx, ny, nz}, kernelDim = {kx, ky, kz}
 *                                  (reference src/convolution3Dfft.cu:394-421)
 *   convolution3DfftCUDA, _test : imDim = {d0, d1, d2}, d2 fastest
 *                                  (reference src/convolution3Dfft.h:26)
 * The convolution is circular; the kernel is zero-padded to the image and its
 * centre (k/2 on each axis) is moved to the origin before the transform.
 *
 * The second block (fc_*) is this library's own API: device-pointer entry
 * points with caller-provided workspace and stream, the adjoint (gradient)
 * operator, the batched multi-view operator, the tensor-core precision mode,
 * the raw 3D R2C/C2R transforms, and per-pass profiling.
 */
#ifndef FC_GB300_CONVOLUTION_3D_FFT_H
#define FC_GB300_CONVOLUTION_3D_FFT_H

#include <stddef.h>

#ifdef __cplusplus
#define FUNCTION_PREFIX extern "C" __attribute__((visibility("default")))
#else
#define FUNCTION_PREFIX extern __attribute__((visibility("default")))
#endif

typedef float imageType; /* reference src/convolution3Dfft.h:17 */

/* Compile-time constants of the reference header (src/convolution3Dfft.h:18-21),
 * kept with the same names, types and values for callers that use them.  This
 * library's kernels do not depend on them: their launch shapes are chosen per
 * transform length for sm_103a. */
static const int MAX_THREADS_CUDA = 1024;
static const int MAX_BLOCKS_CUDA = 65535;
static const int dimsImage = 3;

/* ------------------------------------------------------------------ *
 * Reference-compatible exports                                         *
 * ------------------------------------------------------------------ */

/* Replaces reference src/convolution3Dfft.h:29-32 (body src/convolution3Dfft.cu:216-292).
 * kernel is already image-sized and already shifted (N floats).  Returns a
 * new[]-allocated array of N floats owned by the caller (delete[] from C++,
 * or fc_free_result()), or NULL on error. */
FUNCTION_PREFIX imageType* convolution3DfftCUDA_test(imageType* im, int* imDim, imageType* kernel, int devCUDA);

/* Replaces reference src/convolution3Dfft.h:41-45 (body src/convolution3Dfft.cu:299-391).
 * Returns a new[]-allocated array of N floats owned by the caller, or NULL on
 * error.  im is not modified. */
FUNCTION_PREFIX imageType* convolution3DfftCUDA(imageType* im, int* imDim, imageType* kernel, int* kernelDim,
                                                 int devCUDA);

/* Replaces reference src/convolution3Dfft.h:56 (body src/convolution3Dfft.cu:399-578).
 * Overwrites im with the convolution.  On error im is left unchanged. */
FUNCTION_PREFIX void convolution3DfftCUDAInPlace(imageType* im, int* imDim, imageType* kernel, int* kernelDim,
                                                 int devCUDA);

/* Replaces reference src/convolution3Dfft.h:58-64, the commented-out
 * convolution3DfftCUDAInPlaceSaveMemory, whose device product survives as
 * modulateAndNormalizeSubsampled_kernel (src/convolution3Dfft.cu:65-125).
 * Same arguments and error behaviour as convolution3DfftCUDAInPlace; the
 * kernel is transformed at its own size (no padding, no centring) and each
 * image frequency takes the nearest kernel frequency, (int)(r*f + 0.5) mod k
 * per axis with r = k/n, negated where the three kernel indices sum to an odd
 * number (the phase of a shift by k/2: for an odd kernel edge the result
 * lies half a voxel off the centred convolution along that axis).  An
 * approximation of the convolution; for an odd kx the x index (kx+1)/2 takes
 * the Hermitian mirror of the stored half spectrum (the reference reads past
 * its row there). */
FUNCTION_PREFIX void convolution3DfftCUDAInPlaceSaveMemory(imageType* im, int* imDim, imageType* kernel,
                                                           int* kernelDim, int devCUDA);

/* Replace reference src/convolution3Dfft.h:66-72 (bodies src/standardCUDAfunctions.cu:13-71,
 * src/convolution3Dfft.cu:581-584).  On failure the int queries return -1
 * (selectDevice..., compute capability) or 0 (device count, memory). */
FUNCTION_PREFIX int selectDeviceWithHighestComputeCapability(void);
FUNCTION_PREFIX int getCUDAcomputeCapabilityMinorVersion(int devCUDA);
FUNCTION_PREFIX int getCUDAcomputeCapabilityMajorVersion(int devCUDA);
FUNCTION_PREFIX int getNumDevicesCUDA(void);
FUNCTION_PREFIX void getNameDeviceCUDA(int devCUDA, char* name); /* writes 256 bytes */
FUNCTION_PREFIX long long int getMemDeviceCUDA(int devCUDA);
FUNCTION_PREFIX int cuda_version(void);

/* Replaces reference src/convolution3Dfft.h:84 (body src/convolution3Dfft.cu:587-603).
 * shape is slowest-first (as for cufftEstimate{1,2,3}d); len is 1, 2 or 3.
 * Returns the device scratch this library needs for a plain convolution of
 * that image shape with a kernel of the same shape (the upper bound), in MiB,
 * or -1 for an invalid shape. */
FUNCTION_PREFIX int gpu_mem_needed_mb(int* shape, int len);

/* ------------------------------------------------------------------ *
 * Library extensions (no counterpart in the reference header)         *
 * ------------------------------------------------------------------ */

/* status codes */
#define FC_OK 0
#define FC_ERR_ARG 1         /* invalid argument (NULL, non-positive or oversized dims, kernel > image) */
#define FC_ERR_CUDA 2        /* a CUDA runtime call failed */
#define FC_ERR_NOMEM 3       /* device or host allocation failed, or workspace too small */
#define FC_ERR_UNSUPPORTED 4 /* shape or option outside what this build implements */
#define FC_ERR_TIMEOUT 5     /* a bounded device wait expired */

/* flags for the fc_* entry points */
#define FC_FLAG_SHIFT_COMPAT 1 /* place the kernel with the reference InPlace index arithmetic
                                  (src/convolution3Dfft.cu:128-166 called from :454-461); identical to the
                                  default when nx==nz and kx==kz */
#define FC_FLAG_DENSE_KERNEL 2 /* kernel is an image-sized, already shifted array of N floats */
#define FC_FLAG_TC_FP16 4      /* tensor-core DFT stages, fp16 hi+lo split operands, fp32 accumulate */
#define FC_FLAG_TC_BF16 8      /* tensor-core DFT stages, bf16 hi+lo split operands, fp32 accumulate */
#define FC_FLAG_CORRELATE 16   /* fc_conv3d_kspec_device: multiply by the conjugate kernel spectrum, i.e.
                                  convolve with the kernel flipped about its centre (the adjoint) */

FUNCTION_PREFIX int fc_last_status(void);
FUNCTION_PREFIX const char* fc_last_error(void);
/* release a buffer returned by convolution3DfftCUDA / convolution3DfftCUDA_test (delete[]) */
FUNCTION_PREFIX void fc_free_result(imageType* p);
/* set the kernel placement used by the reference-compatible host entry points:
   0 = centred circular shift (default), 1 = reference InPlace arithmetic.  The
   environment variable FC_SHIFT_COMPAT=1 sets 1 at load time. */
FUNCTION_PREFIX void fc_set_shift_compat(int on);
/* kernel selection: 0 = register-resident kernels for power-of-two axes and
   the generic shared-memory kernels elsewhere (default); 1 = generic kernels
   on every axis.  The environment variable FC_GENERIC=1 sets 1 at load time. */
FUNCTION_PREFIX void fc_set_generic_kernels(int on);
/* host I/O of convolution3DfftCUDAInPlace: 0 = copy the image to the device
   and back; 1 = direct: the first pass reads the caller's buffer and the last
   pass writes it over the CPU-GPU link, on GPUs that read pageable host memory
   through the host page tables (e.g. GB300), copy elsewhere; 2 = auto
   (default): direct for page-locked host buffers, copy for pageable ones.
   FC_HOST_IO=copy|direct|auto sets it at load time. */
FUNCTION_PREFIX void fc_set_host_io(int mode);
/* L2 budget of one column chunk of the y / fused-z / y-inverse passes:
   0 = no chunking (default), -1 = half the device L2, else bytes.  The
   environment variable FC_L2_CHUNK_MB sets it at load time. */
FUNCTION_PREFIX void fc_set_l2_chunk_bytes(long long bytes);
/* free the cached workspace, staging buffers and plans held for a device */
FUNCTION_PREFIX int fc_release_device(int devCUDA);
/* library version, e.g. "fc-gb300 0.1.0 (sm_103a)" */
FUNCTION_PREFIX const char* fc_version(void);

/* Device-pointer convolution on the caller's stream.
 *   d_image, d_out : N floats, x fastest; d_out may equal d_image
 *   imDim {nx,ny,nz}; kernelDim {kx,ky,kz} (ignored with FC_FLAG_DENSE_KERNEL)
 *   d_workspace    : at least fc_conv3d_workspace_bytes() bytes, 256-byte aligned,
 *                    or NULL to use a workspace the library allocates and caches
 *   stream         : a cudaStream_t (NULL = legacy default stream)
 * The call is asynchronous with respect to the host. */
FUNCTION_PREFIX size_t fc_conv3d_workspace_bytes(const int* imDim, const int* kernelDim, int flags);
FUNCTION_PREFIX int fc_conv3d_device(const float* d_image, float* d_out, const int* imDim, const float* d_kernel,
                                     const int* kernelDim, int flags, void* d_workspace, size_t workspace_bytes,
                                     void* stream);

/* Adjoint of the convolution y = conv(x, k) (same placement as fc_conv3d_device):
 *   d_grad_image  (N floats)  = correlation of d_grad_out with k   (may be NULL)
 *   d_grad_kernel (K floats)  = correlation of x with d_grad_out cropped to the
 *                               kernel support, in the kernel's own layout (may be NULL) */
FUNCTION_PREFIX size_t fc_conv3d_adjoint_workspace_bytes(const int* imDim, const int* kernelDim, int flags);
FUNCTION_PREFIX int fc_conv3d_adjoint_device(const float* d_image, const float* d_kernel, const float* d_grad_out,
                                             float* d_grad_image, float* d_grad_kernel, const int* imDim,
                                             const int* kernelDim, int flags, void* d_workspace,
                                             size_t workspace_bytes, void* stream);

/* Batched convolution of n_views independent volumes of uneven sizes, each
 * with its own kernel.  dims: 6 ints per view {nx,ny,nz,kx,ky,kz}.  Pointer
 * arrays are host arrays of device pointers. */
FUNCTION_PREFIX size_t fc_conv3d_batched_workspace_bytes(int n_views, const int* dims, int flags);
FUNCTION_PREFIX int fc_conv3d_batched_device(int n_views, const float* const* d_images, float* const* d_outs,
                                             const float* const* d_kernels, const int* dims, int flags,
                                             void* d_workspace, size_t workspace_bytes, void* stream);

/* Unnormalised 3D real-to-complex / complex-to-real transforms (cuFFT
 * conventions): d_spec holds nz*ny*(nx/2+1) complex values (interleaved
 * float pairs), x fastest.  The inverse overwrites neither input. */
FUNCTION_PREFIX size_t fc_fft3d_workspace_bytes(const int* imDim);
FUNCTION_PREFIX int fc_rfft3d_device(const float* d_in, float* d_spec, const int* imDim, void* d_workspace,
                                     size_t workspace_bytes, void* stream);
FUNCTION_PREFIX int fc_irfft3d_device(const float* d_spec, float* d_out, const int* imDim, void* d_workspace,
                                      size_t workspace_bytes, void* stream);

/* Materialise the zero-padded, shifted kernel (N floats, x fastest) exactly as
 * the convolution's first pass sees it; with FC_FLAG_SHIFT_COMPAT the buffer
 * equals the reference's shifted_kernel after its row copy
 * (src/convolution3Dfft.cu:442-486). */
FUNCTION_PREFIX int fc_pad_shift_kernel_device(const float* d_kernel, const int* kernelDim, const int* imDim,
                                               int flags, float* d_out, void* stream);

/* Radix plan of a transform length, for inspection: writes up to max_stages
 * radices and returns their count (or -1). Host-only, needs no GPU. */
FUNCTION_PREFIX int fc_plan_radices(int n, int* radices, int max_stages);

/* Kernel-spectrum reuse (no reference counterpart; the reference recomputes
 * the kernel's FFT on every call, its TODO at src/convolution3Dfft.cu:363).
 * fc_kernel_spectrum_device writes the kernel's spectrum for images of imDim
 * into a caller buffer of fc_kernel_spectrum_bytes (256-byte aligned; the
 * centred placement, flags FC_FLAG_DENSE_KERNEL / FC_FLAG_TC_* as for
 * fc_conv3d_device); fc_conv3d_kspec_device then convolves any number of
 * images with it, running only the image passes (FC_FLAG_CORRELATE:
 * correlation, i.e. the kernel flipped about its centre).  Workspace:
 * fc_conv3d_kspec_workspace_bytes, or NULL for the library's own.  Both
 * are asynchronous on `stream`. */
FUNCTION_PREFIX size_t fc_kernel_spectrum_bytes(const int* imDim, const int* kernelDim, int flags);
FUNCTION_PREFIX int fc_kernel_spectrum_device(const float* d_kernel, const int* kernelDim, const int* imDim, int flags,
                                              void* d_kspec, size_t kspec_bytes, void* stream);
FUNCTION_PREFIX size_t fc_conv3d_kspec_workspace_bytes(const int* imDim);
FUNCTION_PREFIX int fc_conv3d_kspec_device(const float* d_image, float* d_out, const int* imDim, const void* d_kspec,
                                           const int* kernelDim, int flags, void* d_workspace, size_t workspace_bytes,
                                           void* stream);

/* Richardson-Lucy deconvolution (no reference counterpart; the operator's
 * consumer named for this library): `iterations` updates
 * x <- x * correlate(y / conv(x, k), k) of the estimate d_estimate (holds the
 * starting estimate on entry, e.g. a copy of y), for a non-negative kernel of
 * unit sum; where conv(x, k) <= 0 the ratio is 0.  The kernel spectrum is
 * computed once per call.  Workspace: fc_rl_workspace_bytes, or NULL for the
 * library's own.  Asynchronous on `stream`. */
FUNCTION_PREFIX size_t fc_rl_workspace_bytes(const int* imDim, const int* kernelDim, int flags);
FUNCTION_PREFIX int fc_rl_deconvolve_device(const float* d_observed, float* d_estimate, const int* imDim,
                                            const float* d_kernel, const int* kernelDim, int iterations, int flags,
                                            void* d_workspace, size_t workspace_bytes, void* stream);

/* Device-pointer form of convolution3DfftCUDAInPlaceSaveMemory: d_out may
 * equal d_image; imDim = {nx, ny, nz}, kernelDim = {kx, ky, kz} with the
 * kernel no larger than the image along any axis.  Workspace:
 * fc_conv3d_subsampled_workspace_bytes (the image spectrum plus the kernel's
 * own-size spectrum), 256-byte aligned, or NULL for the library's own.
 * Asynchronous on `stream`. */
FUNCTION_PREFIX size_t fc_conv3d_subsampled_workspace_bytes(const int* imDim, const int* kernelDim);
FUNCTION_PREFIX int fc_conv3d_subsampled_device(const float* d_image, float* d_out, const int* imDim,
                                                const float* d_kernel, const int* kernelDim, void* d_workspace,
                                                size_t workspace_bytes, void* stream);

/* Plan the tuner chose for the most recent batched call on this thread:
 * returns the schedule (0 pass-major, 1 view-major, 2 view-concurrent,
 * 3 single-volume sequence per view, 4 those sequences concurrently; -1 if
 * no batched call yet) and, if choices != NULL, the 5 per-pass launch
 * choices (0 persistent work-list launch, 1 persistent with one CTA per SM,
 * 2 one launch per view) used by schedules 0-2. */
FUNCTION_PREFIX int fc_batched_last_plan(int* choices);

/* Per-pass timing: when enabled, every pass records CUDA events on the stream
 * it is launched on.  fc_profile_read synchronises and copies up to max
 * entries (name, milliseconds, algorithmic bytes) of the most recent call(s),
 * then clears the record. */
FUNCTION_PREFIX void fc_profile_enable(int on);
/* restrict the per-pass events to the pass of this name (NULL or "": all) */
FUNCTION_PREFIX void fc_profile_only(const char* pass_name);
FUNCTION_PREFIX int fc_profile_read(char* names, int name_stride, float* ms, double* bytes, int max);
/* number of kernel launches the most recent fc_* / reference call made */
FUNCTION_PREFIX int fc_launch_count(void);

/* Failure reporting of the asynchronous entry points (no reference
 * counterpart; the reference ends the process with exit() on any CUDA error,
 * src/book.h:22-30).  The pipelined x passes and the fused z passes wait on
 * asynchronous copies with a bounded wait (about one second); an expired wait
 * ends the kernel and is counted on the device.  The synchronous entry points
 * (convolution3DfftCUDA*, fc_* with a host buffer) check the counts before
 * the result reaches the caller's buffer and fail with FC_ERR_TIMEOUT, leaving
 * it unchanged.  The fc_*_device entry points return when their work is
 * enqueued; fc_device_wait_status synchronises `stream` and returns
 * FC_ERR_TIMEOUT if a wait on the current device has expired since the last
 * check (then the outputs of that work are undefined), else FC_OK. */
FUNCTION_PREFIX int fc_device_wait_status(void* stream);

/* Test controls of the failure paths (no reference counterpart).
 * fc_test_set_wait_fault sets, for the current device, the limit of the
 * bounded waits in clock cycles (0: the default) and, with skip_copies != 0,
 * makes the kernels arm their copy barriers without issuing the copies, so
 * that every wait runs out with no copy in flight and each kernel returns its
 * timeout status; (0, 0) restores normal operation.  fc_fault_inject("alloc:n")
 * makes the n-th device or page-locked allocation of this library from then on
 * fail with FC_ERR_NOMEM, on the host and before any CUDA call ("off"
 * disarms; the environment variable FC_FAULT_INJECT sets it at load time).
 * Both return FC_OK or FC_ERR_ARG. */
FUNCTION_PREFIX int fc_test_set_wait_fault(long long limit_cycles, int skip_copies);
FUNCTION_PREFIX int fc_fault_inject(const char* spec);

/* Allocation-free variant of fc_conv3d_device (no counterpart in the
 * reference).  For callers that cannot allocate device memory when they
 * convolve -- a framework that has reserved the GPU's memory in its own pool,
 * a real-time loop that cannot take cudaMalloc's implicit synchronisation, a
 * deployment that forbids device allocation after start-up.  Same arguments
 * and result as fc_conv3d_device (fp32 path, FC_FLAG_SHIFT_COMPAT and
 * FC_FLAG_DENSE_KERNEL honoured) but no workspace argument: all scratch,
 * including the twiddle tables, comes from one static device array of
 * FC_NOALLOC_SCRATCH_BYTES per device.  Under CUDA's lazy module loading (the
 * default since CUDA 12.2) the array is reserved when the first call on a
 * device loads it, and then held until the process exits: make that first
 * call at start-up, before a memory pool takes the GPU's memory and before any
 * stream capture.  A convolution needing more scratch than that is rejected
 * with FC_ERR_NOMEM and a message giving both sizes (e.g. a 256x256x128 image
 * with a 31x31x63 kernel needs about 56 MiB).  Each call looks up the array's
 * address for the current context.  Calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller. */
#define FC_NOALLOC_SCRATCH_BYTES (64ull << 20)
FUNCTION_PREFIX int fc_conv3d_device_noalloc(const float* d_image, float* d_out, const int* imDim,
                                             const float* d_kernel, const int* kernelDim, int flags, void* stream);

#endif /* FC_GB300_CONVOLUTION_3D_FFT_H */
