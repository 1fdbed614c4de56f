// One-launch block of the streaming partitioned convolution (stream_conv.cu).
#pragma once

#include <stddef.h>

#include "common.h"

namespace mgb {

struct UpolsBlockArgs {
    TileArgs fwd;        // forward transform: window -> xcur (256-thread row tile, one transform)
    TileArgs inv;        // inverse transform: y -> output window
    int inv_c2r_rows;    // the inverse's c2r fix-up stages y in shared memory (load_stage0_c2r_rows)
    float2 *xcur;        // nb bins: spectrum of the current window
    float2 *fdl;         // P rows of `pitch` bins: spectra of the last P windows (block j in slot j % P)
    const float2 *h;     // P rows of `pitch` bins: filter-partition spectra (pad bins zero)
    float2 *part;        // G rows of `pitch` bins: partial sums over partitions 1 .. P-1
    float2 *y;           // nb bins: output spectrum
    float4 *win;         // window [previous | input]; the input half becomes the previous half
    unsigned half16;     // bytes of one half / 16
    unsigned nb, pitch, P, G, groups;
    unsigned *tickets;   // upols_block_tickets(groups): [0] blocks processed, [1] groups finished,
                         // [2] spectrum of block k published (k + 1), [3 + x] range CTAs done with group x
    int *err;            // set when a bounded wait for the spectrum times out
    float s;             // 1 / transform length
    unsigned wait_polls; // bound of the wait for the spectrum (polls of ~32 ns and more)
    unsigned wait_skew;  // 0; 1 makes the wait look for a flag value nobody publishes
                         // (the timeout path, for tests of a caller's error handling)
};
// Polls of the spectrum wait before it gives up (half a second or more).
constexpr unsigned kUpolsWaitPolls = 1u << 24;
// The bound used while a timeout is injected: well under a millisecond.
constexpr unsigned kUpolsInjectedWaitPolls = 4096;
inline unsigned upols_block_tickets(unsigned groups) { return 3 + groups; }

// Row-tile length M (complex points) with a compiled fused kernel, and its
// launch shape: 1 + groups * G CTAs of 256 threads (G >= 1), all resident.
bool upols_block_supported(int M);
const void *upols_block_fn(int M);
size_t upols_block_smem(int M);
cudaError_t launch_upols_block(int M, const UpolsBlockArgs &a, cudaStream_t st);

}  // namespace mgb
