// Ragged batched convolution kernel (conv_ragged.cu).
#pragma once

#include <stddef.h>

#include "common.h"

namespace mgb {

// One convolution request as the kernel sees it.
struct RaggedReq {
    const float2 *in;     // first block, time domain (reals read as pairs for mono)
    const float2 *h;      // transformed second block (mono: N/2 + 1 bins, stereo: N)
    float2 *out;          // N reals (mono) or N complex (stereo)
    float2 *spec;         // scratch: L + 1 complex
    float scale;          // 1 / N
    unsigned lg;          // log2 of the complex FFT length L (mono N/2, stereo N)
    unsigned stereo;
    unsigned zero_pad;    // first block zero-padded (upper half not read)
    unsigned split;       // 1: runs as phase tasks (four-step over several CTAs)
    unsigned counter;     // split requests: index of its completion counter
};

// Work item: a whole request, or one task of a phase of a split request.
struct RaggedTask {
    unsigned req;
    unsigned short phase;  // split: 0 F1 columns, 1 F2 rows, 2 multiply, 3 I1 rows, 4 I2 columns;
                           // kRaggedGroupTask: a group of whole requests of one class
    unsigned short index;  // tile / chunk within the phase; group: member count
    unsigned wait;         // tasks of this request that must be complete first
    unsigned pad;          // group: offset of its buffer tables in RaggedArgs::tab
};

// A group task runs up to C whole requests of one (size, method, zero-pad)
// class as the C transforms of one tile pair (C = the tile's transforms for
// that size); `req` is its first member.  Its tables in RaggedArgs::tab: count
// input, filter-spectrum, output and spectrum-scratch pointers, in that order.
constexpr unsigned short kRaggedGroupTask = 8;
unsigned ragged_group_size(unsigned lg);  // members per group task (1: whole requests run alone)

// Phase task counts of a split request of length 2^lg (four-step L1 x L2).
constexpr unsigned kRaggedMulChunks = 8;
unsigned ragged_phase_tasks(unsigned lg, unsigned phase);
constexpr unsigned kRaggedMinSplitLg = 14;  // split requests have L >= 16384

struct RaggedArgs {
    const RaggedReq *reqs;
    const RaggedTask *tasks;  // in dequeue order
    unsigned count;           // tasks
    unsigned *next;           // dequeue counter, zeroed before each launch
    unsigned *counters;       // per split request: completed tasks, zeroed before each launch
    int *err;                 // set when a bounded wait times out
    const float2 *tw;         // stage twiddle table
    const float2 *rtw;        // per size: r2c fix-up twiddles (L) then c2r ones (L)
    unsigned rtw_off[17];     // offset of size 2^lg in rtw
    const float2 *const *tab; // group tasks' buffer tables
};

const void *conv_ragged_fn();
int conv_ragged_threads();
size_t conv_ragged_smem();

// Class pipelines: requests of one (size, method, zero-pad) class whose
// five four-step phases run as ordinary batched launches over a table of the
// requests' buffers (blockIdx.y picks the request).
struct ClassEntry {
    const float2 *in;
    const float2 *h;
    float2 *out;
    float2 *spec;
};

struct ClassTile {
    const void *fn;  // kernel(TileArgs tmpl, const ClassEntry *tab, int phase)
    int L, C, threads;
    size_t smem;     // with the twiddle region
};
// Phase 0/4 (columns of L1) and 1/3 (rows of L2) tiles for a split L1 x L2.
ClassTile class_column_tile(int L1);
ClassTile class_row_tile(int L2);
// Phase 1 with the stereo spectral multiply fused, kernel(TileArgs tmpl,
// const ClassEntry *tab, int phase) with the template's in2_dist = 1,
// in2_stride = L1 and scale = 1 / L; the multiply launch is then skipped.
ClassTile class_row_mul_tile(int L2);
// Multiply phase of a mono class: kernel(const ClassEntry *tab, unsigned l1,
// unsigned l2, float scale, const float2 *rtw_fwd, const float2 *rtw_inv),
// grid (L1/32, L2/64, requests), 256 threads.
const void *class_multiply_fn();

}  // namespace mgb
