// Fused second and third passes of the three-level transform (bc_fused.cu).
#pragma once

#include <stddef.h>

#include "common.h"

namespace mgb {

struct BcArgs {
    const float2 *y;      // pass-A output: [batch][N1][65536]
    float2 *x;            // final output
    float2 *ring;         // ring_slots x 16 rows x 65536 points (L2-resident)
    unsigned *counters;   // doneB[nblk], doneC[nblk], next task; zeroed before each launch
    int *err;             // set to 1 when a bounded wait times out
    long long y_item;     // points between batch items of y
    long long x_item;     // points between batch items of x
    unsigned n1;          // N1 (rows of y per item)
    unsigned nblk;        // blocks of 16 rows over all items
    unsigned blk_per_item;
    unsigned ring_slots;
    TileArgs b;           // pass-B tile template (twiddles, conj)
    TileArgs c;           // pass-C tile template
};

size_t bc_smem_bytes();
const void *bc_kernel();
int bc_threads();

}  // namespace mgb
