// Split-precision tensor-core transforms (split_tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include <vector>

namespace mgb {

struct SplitArgs {
    const float2 *in;
    float2 *out;
    long long in_dist, out_dist;  // complex elements between transforms
    unsigned ntrans;
    int conj;                     // 1: inverse (conjugate in and out)
    const unsigned *afrag;        // DFT-16 matrix limbs in mma A-fragment order
    const float2 *tw;             // stage twiddle factors: W_256^(m*q) then W_4096^(m*r), m, q, r < 16
    const void *bfrag;            // tcgen05 form: DFT-16 limbs as B operands (core-matrix order)
    int *err;                     // tcgen05 form: set when a bounded wait times out
    int bulk;                     // tcgen05 form: inputs 16-byte aligned, prefetched by bulk async copies
};

constexpr int kSplitThreads = 256;
constexpr int kSplitPoints = 4096;  // complex points per CTA

// N = 16^stages (256 or 4096); limbs 2 (3 products) or 3 (6 products).
const void *split_kernel(int stages, int limbs);
size_t split_smem_bytes();
// Host tables (FP64, then split / rounded): A fragments (3 limbs x {Re F,
// Im F, -Im F} x 32 lanes x 4 registers) and the stage twiddles.
std::vector<unsigned> split_afrag_table();
std::vector<float2> split_twiddle_table();

// The same transforms with the products on tcgen05.mma (split_umma.cu):
// persistent CTAs, grid = 2 x SMs at most.
const void *split_umma_kernel(int stages, int limbs);
size_t split_umma_smem_bytes();
int split_umma_threads();
std::vector<unsigned short> split_umma_bfrag_table();

}  // namespace mgb
