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
    const float2 *tw;             // stage twiddles W_(16p)^(m*q): p = 16 at 0, p = 256 at 256
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

}  // namespace mgb
