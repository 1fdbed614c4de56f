// Ragged batched transforms (fft_ragged.cu): many c2c / r2c / c2r requests
// of mixed power-of-two lengths in one persistent launch.
#pragma once

#include <stddef.h>

#include "common.h"

namespace mgb {

// Kinds of a request (the reference's three 1D plan kinds, fft.c:476-547, 626-662).
enum FftRaggedKind : unsigned { FR_C2C = 0, FR_R2C = 1, FR_C2R = 2 };

// One request as the kernel sees it.  Complex length L = 2^lg: N for c2c,
// N/2 for r2c and c2r (the real data is read or written as L complex pairs).
struct FftRaggedReq {
    const float2 *in;
    float2 *out;
    float2 *scratch;   // split requests: L complex between the two passes
    unsigned lg;
    unsigned kind;     // FftRaggedKind
    unsigned inverse;  // c2c: MUFFT_INVERSE (conjugated in and out)
    unsigned half;     // MUFFT_FLAG_ZERO_PAD_UPPER_HALF: inputs n >= L/2 are zero and not read
    unsigned full;     // r2c: MUFFT_FLAG_FULL_R2C (all 2L bins)
    unsigned split;    // 1: runs as phase tasks that any CTA may take
    unsigned counter;  // split requests: index of its completion counter
};

// Work item.  phase kFrGroup: a group of `index` whole requests of one class
// (length, kind, direction, zero padding, full output), the transforms of
// one tile, their buffers in FftRaggedArgs::tab from offset `tab`: `index`
// inputs, then `index` outputs.  Otherwise a task of a split request: phase
// 0 column tile `index` (first pass of the four-step), 1 row tile `index`
// (second pass, stored transposed into natural order), 2 r2c fix-up chunk
// `index`; `index` 0xFFFF runs the whole phase.  `wait`: tasks of the same
// request that must be complete first.
constexpr unsigned short kFrGroup = 8;
constexpr unsigned short kFrWholePhase = 0xFFFF;
struct FftRaggedTask {
    unsigned req;
    unsigned short phase;
    unsigned short index;
    unsigned wait;
    unsigned tab;
};

// Lengths: group tasks up to kFrMaxGroupLg, four-step phases from there on.
constexpr unsigned kFrMaxLg = 16;
constexpr unsigned kFrMaxGroupLg = 12;
constexpr unsigned kFrFixupChunks = 4;
// Requests per group task of length 2^lg (the tile's transforms).
unsigned fft_ragged_group_size(unsigned lg);
// Tasks of phase `phase` of a request of length 2^lg (lg > kFrMaxGroupLg).
unsigned fft_ragged_phase_tasks(unsigned lg, unsigned phase, unsigned kind);

struct FftRaggedArgs {
    const FftRaggedReq *reqs;
    const FftRaggedTask *tasks;  // in dequeue order
    unsigned count;              // tasks
    unsigned *next;              // [0] dequeue counter, [1 + c] completed tasks of split request c; zeroed per launch
    int *err;                    // set when a bounded wait times out
    const float2 *tw;            // stage twiddle table
    const float2 *rtw;           // per length: r2c fix-up twiddles (L), then the c2r ones (L)
    unsigned rtw_off[kFrMaxLg + 1];
    const float2 *const *tab;    // group tasks' buffer tables
};

const void *fft_ragged_fn();
int fft_ragged_threads();
size_t fft_ragged_smem();

}  // namespace mgb
