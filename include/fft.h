/*
 * fft.h -- muFFT public C API, served by the GB300 (sm_103a) implementation.
 *
 * Drop-in for the reference header fft.h: every function, type and constant
 * below has the reference's name, value and signature, so a program written
 * against muFFT recompiles and links against libmufft_gb300.so unchanged.
 * Each declaration cites the reference line it replaces.
 *
 * Semantics kept from the reference:
 *   - interleaved complex float {re, im} layout (README.md:33-42);
 *   - transforms are unnormalised in both directions (fft.h:66-76); the
 *     convolution output is normalised by 1/N (fft.h:187-195);
 *   - plan creation returns NULL for sizes the reference rejects
 *     (non-power-of-two, N == 1, r2c/c2r N == 2, fft.c:478-481, :628-631);
 *   - execute is synchronous: when it returns the output is written;
 *   - a plan owns scratch, so one plan must not run on two threads at once
 *     (fft.c:60, :78, :94); distinct plans are independent;
 *   - the MUFFT_FLAG_CPU_* bits are accepted and ignored: there is one GPU
 *     code path and no CPU fallback.
 *
 * Memory: buffers may live anywhere the CUDA driver can see -- device memory
 * (no copies), managed memory, or host memory (pinned or pageable; staged
 * through plan-owned device buffers).  mufft_alloc() returns pinned host
 * memory so that unmodified muFFT callers that fill buffers on the CPU work
 * and get fast host<->device transfers.  GPU-resident pipelines use the
 * extensions in mufft_gb300.h.
 */
#ifndef MUFFT_H__
#define MUFFT_H__

#ifdef __cplusplus
extern "C" {
#endif

#include <stddef.h>

#if defined(__STDC_VERSION__) && __STDC_VERSION__ >= 199901L
#define MUFFT_RESTRICT restrict
#else
#define MUFFT_RESTRICT
#endif

/* Directions (fft.h:44-46). */
#define MUFFT_FORWARD (-1)
#define MUFFT_INVERSE (1)

/* Planning flags (fft.h:52-65). */
#define MUFFT_FLAG_CPU_ANY (0)
#define MUFFT_FLAG_CPU_NO_SIMD ((1 << 16) - 1)
#define MUFFT_FLAG_CPU_NO_AVX (1 << 0)
#define MUFFT_FLAG_CPU_NO_SSE3 (1 << 1)
#define MUFFT_FLAG_CPU_NO_SSE (1 << 2)
/* r2c also writes the redundant upper bins X(N - k) = X(k)*. */
#define MUFFT_FLAG_FULL_R2C (1 << 16)
/* The upper half of a 1D input is zero and is neither read nor allocated. */
#define MUFFT_FLAG_ZERO_PAD_UPPER_HALF (1 << 17)

/* ---------------------------------------------------------------- 1D */

typedef struct mufft_plan_1d mufft_plan_1d;

/* fft.h:86 -- N: power of two >= 2; direction MUFFT_FORWARD or MUFFT_INVERSE. */
mufft_plan_1d *mufft_create_plan_1d_c2c(unsigned N, int direction, unsigned flags);
/* fft.h:99 -- N real samples -> N/2 + 1 bins (N with MUFFT_FLAG_FULL_R2C); N >= 4. */
mufft_plan_1d *mufft_create_plan_1d_r2c(unsigned N, unsigned flags);
/* fft.h:111 -- N/2 + 1 bins -> N real samples (scaled by N); N >= 4. */
mufft_plan_1d *mufft_create_plan_1d_c2r(unsigned N, unsigned flags);
/* fft.h:117 -- output and input must not overlap. */
void mufft_execute_plan_1d(mufft_plan_1d *plan, void *MUFFT_RESTRICT output, const void *MUFFT_RESTRICT input);
/* fft.h:121 -- NULL is a no-op. */
void mufft_free_plan_1d(mufft_plan_1d *plan);

/* ------------------------------------------------------- convolution */

/* Methods (fft.h:131-143). */
#define MUFFT_CONV_METHOD_FLAG_MONO_MONO 0
/* First block: interleaved stereo (L in re, R in im); second block: real filter. */
#define MUFFT_CONV_METHOD_FLAG_STEREO_MONO 1
#define MUFFT_CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST (1 << 2)
#define MUFFT_CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND (1 << 3)

/* Blocks (fft.h:146-150). */
#define MUFFT_CONV_BLOCK_FIRST 0
#define MUFFT_CONV_BLOCK_SECOND 1

typedef struct mufft_plan_conv mufft_plan_conv;

/* fft.h:168 -- circular convolution of length N (power of two >= 4). */
mufft_plan_conv *mufft_create_plan_conv(unsigned N, unsigned flags, unsigned method);
/* fft.h:179 -- forward transform of one block into a buffer of
 * mufft_conv_get_transformed_block_size() bytes. */
void mufft_execute_conv_input(mufft_plan_conv *plan, unsigned block, void *output, const void *input);
/* fft.h:185 -- (N/2 + 4) * 8 bytes for MONO_MONO, N * 8 for STEREO_MONO. */
size_t mufft_conv_get_transformed_block_size(mufft_plan_conv *plan);
/* fft.h:195 -- multiply the two transformed blocks, inverse transform, scale by 1/N. */
void mufft_execute_conv_output(mufft_plan_conv *plan, void *output, const void *input_first, const void *input_second);
/* fft.h:198 */
void mufft_free_plan_conv(mufft_plan_conv *plan);

/* fft.h:201-207 -- element-wise complex multiply out[i] = s * a[i] * b[i]
 * over `samples` complex values.  The returned function runs on the GPU and
 * returns when the result is written; pointers may be host or device memory. */
typedef void (*mufft_convolve_func)(void *output, const void *a, const void *b,
                                    float normalization, unsigned samples);
mufft_convolve_func mufft_get_convolve_func(unsigned flags);

/* ---------------------------------------------------------------- 2D */

typedef struct mufft_plan_2d mufft_plan_2d;

/* fft.h:232 -- row-major Ny x Nx complex grid. */
mufft_plan_2d *mufft_create_plan_2d_c2c(unsigned Nx, unsigned Ny, int direction, unsigned flags);
/* fft.h:249 -- Ny x Nx reals -> Ny rows of stride Nx complex, Nx/2 + 1 valid
 * (all Nx with MUFFT_FLAG_FULL_R2C).  Nx >= 4. */
mufft_plan_2d *mufft_create_plan_2d_r2c(unsigned Nx, unsigned Ny, unsigned flags);
/* fft.h:266 -- Ny rows of stride Nx complex (Nx/2 + 1 read) -> Ny x Nx reals.
 * The output buffer must hold 2 * Nx * Ny floats, as in the reference, but
 * only the first Nx * Ny are written. */
mufft_plan_2d *mufft_create_plan_2d_c2r(unsigned Nx, unsigned Ny, unsigned flags);
/* fft.h:272 */
void mufft_execute_plan_2d(mufft_plan_2d *plan, void *MUFFT_RESTRICT output, const void *MUFFT_RESTRICT input);
/* fft.h:276 */
void mufft_free_plan_2d(mufft_plan_2d *plan);

/* ------------------------------------------------------------ memory */

/* fft.h:286-297 -- pinned host memory, at least 64-byte aligned. */
void *mufft_alloc(size_t size);
void *mufft_calloc(size_t size);
void mufft_free(void *ptr);

#ifdef __cplusplus
}
#endif

#endif
