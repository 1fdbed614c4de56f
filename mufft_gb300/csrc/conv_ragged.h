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
};

struct RaggedArgs {
    const RaggedReq *reqs;  // sorted longest first
    unsigned count;
    unsigned *next;         // dequeue counter, zeroed before each launch
    const float2 *tw;       // stage twiddle table
    const float2 *rtw;      // per size: r2c fix-up twiddles (L) then c2r ones (L)
    unsigned rtw_off[17];   // offset of size 2^lg in rtw
};

const void *conv_ragged_fn();
int conv_ragged_threads();
size_t conv_ragged_smem();

}  // namespace mgb
