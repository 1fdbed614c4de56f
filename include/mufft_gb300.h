/*
 * mufft_gb300.h -- GB300 extensions to the muFFT C API.
 *
 * Nothing here has a counterpart in the reference, which is a single-threaded
 * CPU library: these entry points expose what a GPU caller needs on top of
 * fft.h -- batches, caller streams with device-resident buffers, error
 * reporting (the reference's execute functions return void and cannot fail),
 * and the GPU-only forms (ragged batched convolution, the convolution
 * adjoint).  All functions are C ABI; pointers are plain addresses, streams
 * are cudaStream_t passed as void*.
 */
#ifndef MUFFT_GB300_H__
#define MUFFT_GB300_H__

#include "fft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------- errors */

/* Error codes returned by the int-valued entry points and latched per thread
 * by every entry point (the fft.h functions return void or NULL).  Positive
 * values are cudaError_t codes from the CUDA runtime. */
#define MUFFT_GB_OK 0
#define MUFFT_GB_ERR_INVALID (-1)     /* bad size, flag, pointer or plan */
#define MUFFT_GB_ERR_UNSUPPORTED (-2) /* valid for muFFT but not built here */
#define MUFFT_GB_ERR_NO_DEVICE (-3)   /* no CUDA device visible */
#define MUFFT_GB_ERR_HOST_POINTER (-4)/* async call given host memory */
#define MUFFT_GB_ERR_ALLOC (-5)

/* Extension plan flags (bits the reference leaves unused, fft.h:52-65).
 * Split precision: c2c transforms of N = 256 or 4096 whose radix-16 stages
 * run as 16x16 DFT-matrix products on the tensor cores, with FP32 values
 * carried as BF16 limbs and FP32 accumulation.  No reference counterpart.
 *   BF16X3: three limbs, six products -- FP32-level error.
 *   BF16X2: two limbs, three products -- about 1e-5 relative error. */
#define MUFFT_GB_FLAG_SPLIT_BF16X3 (1u << 24)
#define MUFFT_GB_FLAG_SPLIT_BF16X2 (1u << 25)
/* Plan creation first times the candidate schedules of this shape on the
 * device (mufft_gb_autotune_1d) unless a choice for the shape is remembered;
 * the fastest is used and remembered.  The reference chose its passes from a
 * static table (fft.c:217-435); this flag makes the GPU choice measured. */
#define MUFFT_GB_FLAG_AUTOTUNE (1u << 26)

/* Last error of the calling thread (0 if none) and its text. */
int mufft_gb_last_error(void);
const char *mufft_gb_last_error_string(void);
void mufft_gb_clear_error(void);

/* ------------------------------------------------------------ batches */

/* `batch` independent transforms per execute.  idist / odist: distance
 * between consecutive transforms in elements of the input / output type
 * (complex for c2c input and output, r2c output and c2r input; float for
 * r2c input and c2r output).  0 selects the packed layout: c2c N (N/2 with
 * MUFFT_FLAG_ZERO_PAD_UPPER_HALF) in and N out; r2c N (N/2) in and N/2+1
 * (N with FULL_R2C) out; c2r N/2+1 in and N out.  Real distances must be
 * even. */
mufft_plan_1d *mufft_gb_create_plan_1d_c2c_batched(unsigned N, int direction, unsigned flags,
                                                   unsigned batch, size_t idist, size_t odist);
mufft_plan_1d *mufft_gb_create_plan_1d_r2c_batched(unsigned N, unsigned flags,
                                                   unsigned batch, size_t idist, size_t odist);
mufft_plan_1d *mufft_gb_create_plan_1d_c2r_batched(unsigned N, unsigned flags,
                                                   unsigned batch, size_t idist, size_t odist);

/* ------------------------------------------------------- plan options */

/* Schedule choices of one plan or batch.  The reference has no global state
 * (its choices come from CPUID and static tables, fft.c:217-435); here every
 * choice travels with the creation call that uses it, so threads creating
 * plans with different choices never interfere.  Initialise with
 * mufft_gb_options_init (the defaults below), change fields, pass the
 * address; NULL means the defaults (and, for 1D plans, the autotuner's
 * remembered choice for the shape, see mufft_gb_autotune_1d). */
typedef struct mufft_gb_tile_choice {
    unsigned L;             /* transform length of the tile */
    int load_across;        /* loads walk across neighbouring transforms (1) or along one (0) */
    int store_across;       /* the same for stores */
    unsigned transforms_per_tile, elems_per_thread, cluster_ctas;  /* 0 = any */
} mufft_gb_tile_choice;

#define MUFFT_GB_MAX_TILE_CHOICES 8

typedef struct mufft_gb_options {
    unsigned size;               /* sizeof(mufft_gb_options), set by mufft_gb_options_init */
    /* 1D transforms longer than one on-chip tile (16384 points): 0 automatic,
     * 2 four-step, 3 three-level decomposition with smaller tiles */
    int multipass_levels;
    /* inter-pass twiddles: -1 automatic, 0 sincospif per element, 1 FP64
     * table times a per-tile factor, 2 per-tile column powers */
    int twiddle_table;
    /* three-level N1 x 65536 transforms: last two passes as one persistent
     * launch with an L2-resident intermediate (1) or two launches (0) */
    int fused_passes;
    /* column passes staged by TMA: 0 off, 1 double-buffered persistent
     * CTAs, 2 single buffer */
    int tma;
    /* tile passes run at most this many CTAs per SM (0 = as many as fit) */
    int tile_occupancy;
    /* contiguous row passes as persistent CTAs prefetching their next tile (1) */
    int stream_tiles;
    /* split-precision products on tcgen05.mma with TMEM (0) or mma.sync (1) */
    int split_engine;
    /* 2D columns: 0 automatic (8192 points and more as a two-pass four-step
     * of short, wide column tiles, and 4096 points for grids at least 4096
     * (real) or 8192 (c2c) wide), 1 one pass, 2 two passes where possible */
    int columns_2d;
    /* ragged convolution batches: requests of at least conv_split complex
     * points run as phase tasks over many CTAs (0: none), of at least
     * conv_classes points as class pipelines (0: none); powers of two in
     * 16384..65536 */
    unsigned conv_split, conv_classes;
    /* streaming convolution: partition ranges of the multiply-accumulate (0
     * sized to the GPU) and one launch per block (1) or a graph (0) */
    unsigned stream_conv_ranges;
    int stream_conv_fused;
    /* ragged transform batches: requests of at least fft_split complex points
     * (a power of two in 8192..65536; 0: none) run as four-step phase tasks
     * over many CTAs, shorter ones above 4096 points whole in one CTA */
    unsigned fft_split;
    /* preferred tile kernels (mufft_gb_list_tiles), first ntiles entries */
    unsigned ntiles;
    mufft_gb_tile_choice tiles[MUFFT_GB_MAX_TILE_CHOICES];
    /* tile passes as a persistent grid of resident CTAs walking the pass's
     * tiles wherever the tile has that variant (the 1024-thread 4096-point
     * column tile): -1 automatic (on), 0 off, 1 on */
    int persistent_tiles;
    /* three-level transforms: the intermediate kept in L2 where it fits
     * (stores marked evict-last, the input and output streamed evict-first,
     * the intermediate dropped from L2 without write-back once the last pass
     * has read it): -1 automatic, 0 off, 1 on */
    int l2_residency;
} mufft_gb_options;

/* The defaults: levels 0, twiddles -1, fused 0, tma 0, occupancy 0, stream
 * tiles 0, split engine 0, 2D columns 0, conv_split 65536, conv_classes
 * 16384, stream ranges 0, stream fused 1, fft_split 8192, no tile choices,
 * persistent tiles -1, L2 residency -1. */
void mufft_gb_options_init(mufft_gb_options *opts);

/* 1D plans of every kind with options: kind 0 c2c, 1 r2c, 2 c2r (direction
 * is used by c2c only); the other arguments as the _batched creators, which
 * are this call with opts = NULL.  Invalid options return NULL with
 * MUFFT_GB_ERR_INVALID. */
mufft_plan_1d *mufft_gb_create_plan_1d(int kind, unsigned N, int direction, unsigned flags, unsigned batch,
                                       size_t idist, size_t odist, const mufft_gb_options *opts);
/* 2D plans with options: kind 0 c2c, 1 r2c, 2 c2r, as mufft_create_plan_2d_*. */
mufft_plan_2d *mufft_gb_create_plan_2d(int kind, unsigned Nx, unsigned Ny, int direction, unsigned flags,
                                       const mufft_gb_options *opts);
/* Convolution plans with options for their inner transforms, as
 * mufft_create_plan_conv. */
mufft_plan_conv *mufft_gb_create_plan_conv(unsigned N, unsigned flags, unsigned method, const mufft_gb_options *opts);

/* ------------------------------------------------- asynchronous execution */

/* Enqueue on `stream` (a cudaStream_t; NULL = the legacy default stream)
 * without synchronising.  Buffers must be device-accessible (device or
 * managed memory); host memory is rejected with MUFFT_GB_ERR_HOST_POINTER.
 * A plan's scratch is reused by every execute, so two executes of one plan
 * must not overlap on the GPU (enqueue them on one stream). */
int mufft_gb_execute_plan_1d_async(mufft_plan_1d *plan, void *output, const void *input, void *stream);
int mufft_gb_execute_plan_2d_async(mufft_plan_2d *plan, void *output, const void *input, void *stream);
/* Enqueues only launches first .. first + count - 1 of a 2D plan (device
 * buffers; for timing one pass at a time, like the 1D variant). */
int mufft_gb_execute_plan_2d_launches_async(mufft_plan_2d *plan, void *output, const void *input, unsigned first,
                                            unsigned count, void *stream);
int mufft_gb_execute_conv_input_async(mufft_plan_conv *plan, unsigned block, void *output,
                                      const void *input, void *stream);
int mufft_gb_execute_conv_output_async(mufft_plan_conv *plan, void *output, const void *input_first,
                                       const void *input_second, void *stream);

/* `count` executes of a 1D plan on buffers in any memory -- typically page-
 * locked host memory from mufft_alloc -- with the copies overlapped: input
 * i + 1 is copied to the device while transform i runs and output i - 1 is
 * copied back (two device slots of each, made on the plan's first call, and
 * a copy-in, a compute and a copy-out stream).  Returns when every output is
 * written, like mufft_execute_plan_1d called `count` times (fft.c:811-850),
 * which runs one transform's copies and kernels in turn.  Pageable host
 * memory works but its copies do not overlap.  Not for convolution output
 * plans.  No counterpart in the reference. */
int mufft_gb_execute_plan_1d_host_pipeline(mufft_plan_1d *plan, void *const *outputs, const void *const *inputs,
                                           unsigned count);

/* Enqueue only launches [first, first + count) of a 1D plan's schedule (see
 * mufft_gb_plan_1d_describe), for timing one kernel of a multi-pass plan.
 * Intermediate launches read and write the plan's scratch. */
int mufft_gb_execute_plan_1d_launches_async(mufft_plan_1d *plan, void *output, const void *input,
                                            unsigned first, unsigned count, void *stream);

/* ------------------------------------------------- convolution adjoints */

/* No counterpart in the reference.  Gradients of a convolution plan's output
 * out = (1/N) IFFT(FFT(first) . FFT(second)) (mufft_execute_conv_output,
 * fft.c:794-809) for an upstream gradient `grad_output` of `out` (N reals for
 * MONO_MONO, N complex for STEREO_MONO; full length, never zero-padded).
 * Complex gradients follow the dL/dRe + i dL/dIm convention.  Device
 * buffers; enqueued on `stream`; calls on one plan must not overlap (they
 * share its scratch).  The first call of each allocates the plan's adjoint
 * transforms and scratch. */

/* d out / d first, applied to grad_output:
 *   grad_input = (1/N) IFFT(FFT(grad_output) . conj(second_spectrum))
 * second_spectrum: the transformed second block (mufft_execute_conv_input
 * with MUFFT_CONV_BLOCK_SECOND).  grad_input: N reals (mono) / N complex
 * (stereo); with ZERO_PAD_UPPER_HALF_FIRST only its first N/2 entries belong
 * to real inputs. */
int mufft_gb_conv_adjoint_input(mufft_plan_conv *plan, void *grad_input, const void *grad_output,
                                const void *second_spectrum, void *stream);

/* d out / d second, summed over `batch` signals that share the second block:
 *   grad_filter = Re (1/N) IFFT(sum_b FFT(grad_output_b) . conj(first_spectrum_b))
 * The sum runs over spectra (one inverse transform in all).  grad_outputs:
 * batch blocks `output_dist` samples apart (floats for mono, complex for
 * stereo); first_spectra: the transformed first blocks (MUFFT_CONV_BLOCK_FIRST)
 * `spectrum_dist` complex apart.  grad_filter: N reals; with
 * ZERO_PAD_UPPER_HALF_SECOND only its first N/2 entries belong to taps. */
int mufft_gb_conv_adjoint_filter(mufft_plan_conv *plan, float *grad_filter, const void *grad_outputs,
                                 size_t output_dist, const void *first_spectra, size_t spectrum_dist,
                                 unsigned batch, void *stream);

/* Both gradients of `batch` signals sharing one second block, each output
 * gradient transformed once for both (batched launches over chunks of
 * signals): grad_filter as mufft_gb_conv_adjoint_filter (NULL: not computed)
 * and grad_inputs, batch blocks `input_dist` samples apart, each as
 * mufft_gb_conv_adjoint_input (NULL: not computed).  Device buffers. */
int mufft_gb_conv_adjoint(mufft_plan_conv *plan, float *grad_filter, void *grad_inputs, size_t input_dist,
                          const void *grad_outputs, size_t output_dist, const void *first_spectra,
                          size_t spectrum_dist, const void *second_spectrum, unsigned batch, void *stream);

/* mufft_execute_conv_output for `batch` signals sharing one second block:
 * outputs `output_dist` samples apart, first spectra `spectrum_dist` complex
 * apart, one filter spectrum for all (batched launches over chunks of
 * signals).  Device buffers. */
int mufft_gb_execute_conv_output_batched(mufft_plan_conv *plan, void *outputs, size_t output_dist,
                                         const void *first_spectra, size_t spectrum_dist, const void *second_spectrum,
                                         unsigned batch, void *stream);

/* --------------------------------------------- ragged batched convolution */

/* No counterpart in the reference, which convolves one block per call
 * (fft.c:794-809).  One request is what mufft_execute_conv_input(FIRST) +
 * mufft_execute_conv_output do for one block: transform `input`, multiply by
 * the already transformed second block `filter` (from
 * mufft_execute_conv_input(SECOND) of a plan of the same N and method), scale
 * by 1/N and transform back into `output`.
 *   N: power of two; MONO_MONO 32..65536, STEREO_MONO 16..65536.
 *   method: MUFFT_CONV_METHOD_FLAG_* (ZERO_PAD_UPPER_HALF_FIRST: input has N/2
 *     samples; the SECOND flag was applied when the filter was transformed).
 *   input: N (N/2) floats for mono, N (N/2) complex for stereo; filter: N/2+1
 *     (mono) or N (stereo) complex; output: N floats / N complex.  Device
 *     memory; the addresses are fixed when the batch is created. */
typedef struct mufft_gb_conv_request {
    unsigned N;
    unsigned method;
    const void *input;
    const void *filter;
    void *output;
} mufft_gb_conv_request;

typedef struct mufft_gb_conv_batch mufft_gb_conv_batch;

/* Prepares `count` requests of mixed sizes for one persistent launch,
 * captured in a CUDA graph.  Requests of at least opts->conv_classes complex
 * points run as class pipelines: the requests of one size, method and
 * zero-pad setting go through five ordinary batched launches (the four-step
 * phases) on parallel branches of the batch's graph.  The rest run longest
 * first in a persistent kernel, whole in one CTA each or -- from
 * opts->conv_split points -- as phase tasks spread over many CTAs.  flags: 0,
 * or MUFFT_GB_FLAG_AUTOTUNE to time the batch with every split / class size
 * (running it, so writing the outputs, a few times) and keep the fastest.
 * opts: NULL for the defaults (mufft_gb_options_init). */
mufft_gb_conv_batch *mufft_gb_create_conv_batch(const mufft_gb_conv_request *requests, unsigned count,
                                                unsigned flags, const mufft_gb_options *opts);
/* The split size in use (complex points; 0: no request is split). */
unsigned mufft_gb_conv_batch_split_size(const mufft_gb_conv_batch *batch);
/* The class-pipeline size in use (complex points; 0: none). */
unsigned mufft_gb_conv_batch_class_size(const mufft_gb_conv_batch *batch);
/* Synchronises the device and reports whether a bounded wait of the batch's
 * task dependencies timed out in an earlier execute (MUFFT_GB_ERR_UNSUPPORTED),
 * clearing the flag. */
int mufft_gb_conv_batch_status(mufft_gb_conv_batch *batch);
/* Replays the batch on `stream` (enqueued, not synchronised).  Executes of one
 * batch must not overlap on the GPU (they share its scratch). */
int mufft_gb_execute_conv_batch(mufft_gb_conv_batch *batch, void *stream);
void mufft_gb_free_conv_batch(mufft_gb_conv_batch *batch);

/* ---------------------------------------------- ragged batched transforms */

/* No counterpart in the reference, which runs one transform per plan execute
 * (fft.c:811-850).  One request is what a plan of its kind, N and flags does
 * in one mufft_execute_plan_1d: kind 0 c2c (direction MUFFT_FORWARD or
 * MUFFT_INVERSE), 1 r2c, 2 c2r; flags MUFFT_FLAG_ZERO_PAD_UPPER_HALF and (r2c)
 * MUFFT_FLAG_FULL_R2C, the CPU flags accepted and ignored; unnormalised.
 *   N: power of two; c2c 2..65536, r2c and c2r 4..131072.
 *   input / output: device memory, 8-byte aligned, sized as for a plan (c2c
 *     N complex in, N/2 with zero padding, N out; r2c N (N/2) reals in, N/2+1
 *     (N with FULL_R2C) complex out; c2r N/2+1 complex in, N reals out);
 *     the addresses are fixed when the batch is created. */
typedef struct mufft_gb_fft_request {
    unsigned N;
    int kind;
    int direction;
    unsigned flags;
    const void *input;
    void *output;
} mufft_gb_fft_request;

typedef struct mufft_gb_fft_batch mufft_gb_fft_batch;

/* Prepares `count` requests of mixed kinds and sizes for one persistent
 * launch captured in a CUDA graph.  Requests of up to 4096 complex points run
 * in groups of one class as the transforms of one tile; longer ones as
 * four-step phase tasks that any CTA may take.  flags: 0, or
 * MUFFT_GB_FLAG_AUTOTUNE to time the batch with every split size and grid
 * (running it, so writing the outputs, a few times) and keep the fastest.
 * opts: NULL for the defaults. */
mufft_gb_fft_batch *mufft_gb_create_fft_batch(const mufft_gb_fft_request *requests, unsigned count, unsigned flags,
                                              const mufft_gb_options *opts);
/* Replays the batch on `stream` (enqueued, not synchronised).  Executes of one
 * batch must not overlap on the GPU (they share its scratch and counters). */
int mufft_gb_execute_fft_batch(mufft_gb_fft_batch *batch, void *stream);
/* Synchronises the device and reports whether a bounded wait of the batch's
 * task dependencies timed out in an earlier execute (MUFFT_GB_ERR_UNSUPPORTED),
 * clearing the flag. */
int mufft_gb_fft_batch_status(mufft_gb_fft_batch *batch);
/* "requests=.. tasks=.. split=.. grid=.. resident=.. algorithmic_bytes=.." */
int mufft_gb_fft_batch_describe(const mufft_gb_fft_batch *batch, char *buf, size_t size);
void mufft_gb_free_fft_batch(mufft_gb_fft_batch *batch);

/* ---------------------------------------------- streaming convolution */

/* A stream of `block`-sample blocks convolved with a filter of any length
 * (the reference's block convolution, fft.c:794-809, extended to filters
 * longer than a block): uniformly partitioned overlap-save.  The filter is
 * cut into P = ceil(taps / block) partitions whose 2*block-point spectra are
 * computed once here; each block costs one forward transform of the last two
 * input blocks, a multiply-accumulate over the P partitions against the
 * spectra of the last P windows, and one inverse transform -- one CUDA graph
 * launch.  Output block k is samples k*block .. (k+1)*block - 1 of the linear
 * convolution of the whole input stream with the filter.
 *   method: MUFFT_CONV_METHOD_FLAG_MONO_MONO (real samples) or _STEREO_MONO
 *     (complex samples: interleaved left/right); the filter is real.
 *   filter: `taps` floats in host or device memory (copied here).
 * No counterpart in the reference. */
typedef struct mufft_gb_stream_conv mufft_gb_stream_conv;
/* opts: NULL for the defaults.  opts->stream_conv_ranges: partition ranges
 * the multiply-accumulate splits the P partitions into (each range a row of
 * CTAs whose partial sums are added in range order; 0 sizes it to the GPU;
 * clamped to P, or P - 1 for one-launch blocks, which also keep every CTA
 * resident at once).  opts->stream_conv_fused: convolvers whose windows one
 * 256-thread row tile transforms (64 .. 4096 complex points) run a block as
 * one launch -- the forward transform, the multiply-accumulate and the
 * inverse transform in one grid, ordered by tickets (1) -- or as a graph of
 * separate launches (0). */
mufft_gb_stream_conv *mufft_gb_create_stream_conv(unsigned block, unsigned method, const float *filter, unsigned taps,
                                                  unsigned flags, const mufft_gb_options *opts);
/* Device buffer the next input block goes into (block floats or complex).
 * Write it on the stream that runs mufft_gb_stream_conv_process, after the
 * previous process call. */
void *mufft_gb_stream_conv_input(mufft_gb_stream_conv *conv);
/* Device buffer holding the last processed output block. */
const void *mufft_gb_stream_conv_output(const mufft_gb_stream_conv *conv);
/* Convolves the block in the input buffer (one graph launch on `stream`). */
int mufft_gb_stream_conv_process(mufft_gb_stream_conv *conv, void *stream);
/* Forgets the input history (as if the stream restarted from silence). */
int mufft_gb_stream_conv_reset(mufft_gb_stream_conv *conv, void *stream);
void mufft_gb_free_stream_conv(mufft_gb_stream_conv *conv);
/* Partition ranges a convolver uses, and whether it runs a block as one
 * launch (1) or a graph of launches (0). */
unsigned mufft_gb_stream_conv_ranges(const mufft_gb_stream_conv *conv);
int mufft_gb_stream_conv_fused(const mufft_gb_stream_conv *conv);
/* Synchronises the device; MUFFT_GB_ERR_UNSUPPORTED if a one-launch block's
 * bounded wait timed out since the last call (clearing the flag).  The
 * output of that block and the convolver's input history are then not
 * valid: call mufft_gb_stream_conv_reset before relying on further output.
 * The launches themselves stay consistent, so processing may simply go on
 * after the reset. */
int mufft_gb_stream_conv_status(mufft_gb_stream_conv *conv);
/* For testing a caller's error handling: while enabled (1), every block
 * launch waits for a spectrum flag that is never published, gives up after
 * well under a millisecond and reports the timeout through
 * mufft_gb_stream_conv_status; 0 restores normal operation.  One-launch
 * convolvers only (MUFFT_GB_ERR_UNSUPPORTED otherwise). */
int mufft_gb_stream_conv_inject_timeout(mufft_gb_stream_conv *conv, int enable);

/* ------------------------------------------------- allocation-free execute */

/* No counterpart in the reference.  A forward or inverse c2c transform of N
 * complex points for callers that must not allocate memory when they
 * transform -- a real-time audio callback that cannot take cudaMalloc's
 * latency and implicit synchronisation, or a plugin whose host owns all
 * device memory.  No plan is needed: the scratch between the two passes of
 * long transforms and the twiddle table live in fixed device arrays of the
 * library (2^20 points of scratch, about 8.6 MB per GPU, held until exit).
 *   N: power of two, 2 <= N <= 2^20 (1048576); larger N returns
 *      MUFFT_GB_ERR_UNSUPPORTED -- use a plan.
 *   output, input: N complex each in device or managed memory, or in
 *      page-locked host memory mapped into the device's address space (other
 *      host memory returns MUFFT_GB_ERR_HOST_POINTER).  output == input
 *      transforms in place; partially overlapping buffers are not allowed.
 *   stream: cudaStream_t (NULL = legacy default stream); enqueued, not synchronised.
 * The first call on a device sets up (looks up the arrays' device addresses,
 * fills the twiddle table, synchronises the device): make it before any
 * stream capture.  Later calls take no lock.  All calls on a device share one scratch array, which keeps
 * the last call's contents; calls whose kernels overlap on the GPU race on it,
 * so serialise them (one stream).  Returns MUFFT_GB_OK or an error code. */
int mufft_gb_execute_c2c_noalloc(unsigned N, int direction, void *output, const void *input, void *stream);

/* ---------------------------------------------------------- introspection */

/* Kernel launches one execute enqueues, and a one-line description of the
 * GPU schedule (kernel, length, transforms per CTA, grid) into buf. */
unsigned mufft_gb_plan_1d_launches(const mufft_plan_1d *plan);
unsigned mufft_gb_plan_2d_launches(const mufft_plan_2d *plan);
int mufft_gb_plan_1d_describe(const mufft_plan_1d *plan, char *buf, size_t size);
int mufft_gb_plan_2d_describe(const mufft_plan_2d *plan, char *buf, size_t size);

/* The same description for a 1D plan that would be built from these
 * arguments and options, computed on the host without touching a GPU (kind:
 * 0 c2c, 1 r2c, 2 c2r).  Returns MUFFT_GB_OK or the error plan creation
 * would report. */
int mufft_gb_describe_schedule_1d(unsigned N, int kind, int direction, unsigned flags, unsigned batch,
                                  const mufft_gb_options *opts, char *buf, size_t size);

/* The same for a 2D plan (kind 0 c2c, 1 r2c, 2 c2r; Nx columns, Ny rows;
 * direction is used by c2c only), without touching a GPU. */
int mufft_gb_describe_schedule_2d(int kind, unsigned Nx, unsigned Ny, int direction, unsigned flags,
                                  const mufft_gb_options *opts, char *buf, size_t size);

/* --------------------------------------------------------- autotuning */

/* Times the candidate GPU schedules of a 1D plan shape (kind 0 c2c, 1 r2c,
 * 2 c2r; N, direction, flags and batch as for plan creation) on the current
 * device -- pass count, inter-pass twiddle scheme, fused last passes, then
 * every tile variant of the winning schedule's passes -- and remembers the
 * fastest for plans of that shape created afterwards (by any entry point,
 * including the reference's).  Allocates two N x batch complex buffers
 * while it runs.  `report` (optional) receives one line per candidate. */
int mufft_gb_autotune_1d(int kind, unsigned N, int direction, unsigned flags, unsigned batch, char *report,
                         size_t report_size);
/* The remembered choices as a text file, tied to the GPU model and SM count
 * (loading a file made on another GPU fails with MUFFT_GB_ERR_INVALID). */
int mufft_gb_autotune_save(const char *path);
int mufft_gb_autotune_load(const char *path);
void mufft_gb_autotune_clear(void);

/* Writes "L=.. R=.. C=.. Q=.. along/across threads=.. smem=..; ..." for every
 * compiled tile kernel; returns the full length. */
int mufft_gb_list_tiles(char *buf, size_t size);

/* ------------------------------------------------------ memory helpers */

/* Device memory for callers that do not link the CUDA runtime themselves. */
void *mufft_gb_device_alloc(size_t size);
void mufft_gb_device_free(void *ptr);
/* Synchronous copy between any two addresses the driver knows (host, pinned,
 * device, managed). */
int mufft_gb_memcpy(void *dst, const void *src, size_t size);
int mufft_gb_device_synchronize(void);

#ifdef __cplusplus
}
#endif

#endif
