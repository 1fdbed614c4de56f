/*
 * mufft_oracle.h -- CPU restatement of muFFT's scalar FFT / convolution path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA library in
 * mufft_gb300/ is compared against.  Only tests/, __graft_entry__.smoke() and the CPU-baseline leg
 * of bench.py load it; the shipped library never links or calls it.
 *
 * The functions mirror the reference public API (fft.h) one for one, with an
 * "oracle_" prefix so both can live in one process.  Parity is pinned: with
 * MUFFT_FLAG_CPU_NO_SIMD the reference's scalar build produces bit-identical
 * outputs (tests/test_oracle.py against tests/golden/, which were generated by
 * the reference library compiled from its own sources by oracle/build_ref.sh).
 */
#ifndef MUFFT_ORACLE_H
#define MUFFT_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_plan_1d oracle_plan_1d;
typedef struct oracle_plan_2d oracle_plan_2d;
typedef struct oracle_plan_conv oracle_plan_conv;

/* fft.h:86, :99, :111, :117, :121 */
oracle_plan_1d *oracle_create_plan_1d_c2c(unsigned N, int direction, unsigned flags);
oracle_plan_1d *oracle_create_plan_1d_r2c(unsigned N, unsigned flags);
oracle_plan_1d *oracle_create_plan_1d_c2r(unsigned N, unsigned flags);
void oracle_execute_plan_1d(oracle_plan_1d *plan, void *output, const void *input);
void oracle_free_plan_1d(oracle_plan_1d *plan);

/* Step list chosen by the greedy planner (fft.c:325-379): radix[i], p[i]. */
unsigned oracle_plan_1d_steps(const oracle_plan_1d *plan, unsigned *radix, unsigned *p, unsigned max_steps);

/* Runs `count` independent transforms with one shared plan and per-thread
 * scratch: input i at in + i*in_stride bytes, output i at out + i*out_stride.
 * Used to time the CPU baseline over all host cores. */
void oracle_execute_plan_1d_many(oracle_plan_1d *plan, void *output, const void *input,
                                 unsigned count, size_t out_stride, size_t in_stride,
                                 unsigned nthreads);

/* fft.h:168-207 */
oracle_plan_conv *oracle_create_plan_conv(unsigned N, unsigned flags, unsigned method);
void oracle_execute_conv_input(oracle_plan_conv *plan, unsigned block, void *output, const void *input);
size_t oracle_conv_get_transformed_block_size(oracle_plan_conv *plan);
void oracle_execute_conv_output(oracle_plan_conv *plan, void *output, const void *first, const void *second);
void oracle_free_plan_conv(oracle_plan_conv *plan);
void oracle_convolve(void *output, const void *a, const void *b, float normalization, unsigned samples);

/* fft.h:232-276 */
oracle_plan_2d *oracle_create_plan_2d_c2c(unsigned Nx, unsigned Ny, int direction, unsigned flags);
oracle_plan_2d *oracle_create_plan_2d_r2c(unsigned Nx, unsigned Ny, unsigned flags);
oracle_plan_2d *oracle_create_plan_2d_c2r(unsigned Nx, unsigned Ny, unsigned flags);
void oracle_execute_plan_2d(oracle_plan_2d *plan, void *output, const void *input);
void oracle_free_plan_2d(oracle_plan_2d *plan);

/* Direct O(N^2) references in double precision: circular DFT and linear
 * convolution (the same role as test.c:375-403, but FP64). */
void oracle_dft_f64(double *out_interleaved, const double *in_interleaved, unsigned N, int direction);

#ifdef __cplusplus
}
#endif
#endif
