// Shared host/device definitions for the GB300 muFFT kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mgb {

// Largest FFT length a tile can hold on chip (shared memory of a cluster of
// up to 8 CTAs), and the largest the planner runs as a single pass by
// default: beyond 16384 the four-step path measured faster on GB300 than
// cluster tiles, whose stage exchanges are bound by distributed-shared-memory
// bandwidth.
constexpr unsigned kMaxTileLog2 = 16;
constexpr unsigned kMaxTile = 1u << kMaxTileLog2;
constexpr unsigned kMaxSinglePass = 16384;

// Stage twiddle table.  A stage of radix r following sub-transforms of size p
// (p in {16, 256, 4096} inside a tile) needs W^(m*k), W = exp(-2*pi*i/(r*p)),
// for k < p and m < r.  For every (r, p) and k the table holds W^k, W^2k,
// W^4k and W^8k as four consecutive float2 (32 bytes, two float4 loads); the
// other powers are products of at most three of them.
constexpr int kStageTableK = 16 + 256 + 4096;
__host__ __device__ constexpr int stage_radix_index(int r) { return r == 2 ? 0 : r == 4 ? 1 : r == 8 ? 2 : 3; }
__host__ __device__ constexpr int stage_p_offset(int p) { return p == 16 ? 0 : p == 256 ? 16 : 272; }
__host__ __device__ constexpr int stage_table_base(int r, int p)
{
    return (stage_radix_index(r) * kStageTableK + stage_p_offset(p)) * 4;
}
constexpr int kStageTableFloat2 = 4 * kStageTableK * 4;

// Thread-to-work decomposition of a CTA: which index runs fastest across
// consecutive threads.  ALONG: consecutive threads walk along one transform
// (contiguous rows); ACROSS: consecutive threads walk across neighbouring
// transforms (columns of a row-major grid, transposed stores).
enum Map : int { ALONG = 0, ACROSS = 1 };

// How stage-0 inputs are produced from global memory.
enum Prologue : int {
    PRO_PLAIN = 0,      // x[n]
    PRO_C2R = 1,        // complex-to-real fix-up: (a + b*) + w_n (a - b*), a = X[n], b = X[M - n]
    PRO_MUL = 2,        // s * A[n] * B[n]            (stereo convolution output)
    PRO_MUL_C2R = 3,    // fix-up of s * A[n] * B[n]  (mono convolution output)
};

// How last-stage outputs are written.
enum Epilogue : int {
    EPI_PLAIN = 0,
    EPI_R2C = 1,        // real-to-complex fix-up, M + 1 bins
    EPI_R2C_FULL = 2,   // real-to-complex fix-up, all 2M bins
    EPI_TWIDDLE = 3,    // four-step inter-pass twiddle W_N^(k * column)
};

// Arguments of one tile-FFT launch.  A launch runs `ntrans` transforms of
// length L (times gridDim.y batches).  Element n of transform t lives at
//     base + t * dist + n * stride
// with base advanced by blockIdx.y * batch for batched multi-pass launches.
struct TileArgs {
    const float2 *in;
    float2 *out;
    long long in_stride, in_dist, in_batch;
    long long out_stride, out_dist, out_batch;
    // two-level batch: blockIdx.y = g + ysplit*b advances g*in_batch + b*in_batch2
    // (ysplit 0: one level, blockIdx.y*in_batch)
    unsigned ysplit;
    long long in_batch2, out_batch2;
    unsigned ntrans;
    int conj;                 // 1: inverse transform by conjugating in and out
    int prologue;
    int half;                 // inputs n >= L/2 are zero and not read (MUFFT_FLAG_ZERO_PAD_UPPER_HALF)
    int epilogue;
    const float2 *tw;         // stage twiddle table (stage_table_base)
    // real<->complex fix-ups: twiddles of length M, mirror length M
    const float2 *rtw;
    long long mirror_len;     // M for PRO_C2R / PRO_MUL_C2R
    long long mirror_ldist;   // see tile kernel: local index = t*ldist + n*stride
    // convolution prologues
    const float2 *in2;        // second spectrum (B)
    // multiply epilogue (class pipelines): output k of transform t times
    // scale * in2[t*in2_dist + k*in2_stride]
    long long in2_dist, in2_stride;
    // per-transform buffers (tile_body with TAB): transform t reads in_tab[t]
    // (and in2_tab[t]) and writes out_tab[t]; in_dist / out_dist are then 0
    const float2 *const *in_tab;
    const float2 *const *in2_tab;
    float2 *const *out_tab;
    // one in2 for the whole batch (a filter spectrum shared by many signals):
    // bit 0 -- not offset by the grid row's batch (multi-pass passes), bit 1 --
    // not offset by the transform index (single-pass batched tiles)
    int in2_bcast;
    float scale;
    int conj2;                // multiply by conj(B) instead (adjoint of the convolution)
    // four-step twiddle W_N^m = exp(-2*pi*i*m/N): tw_scale = 2/N, tw_mask = N - 1;
    // for column tiles of C transforms tw_lo[k*C + c] = W_N^(k*c) (or null:
    // then every twiddle comes from sincospif)
    float tw_scale;
    unsigned tw_mask;
    const float2 *tw_lo;
    // nonzero: per-tile column powers instead (W_N^(col*off) for the R output
    // offsets of each column in shared memory, times W_N^(col*base) per thread)
    int tw_colpow;
    // nonzero: the twiddle's column factor is the CTA's grid row instead of the
    // transform index (column passes of a 2D four-step: W_N^(k*row) for every
    // column of the tile, from a per-CTA table)
    int tw_by_y;
    // L2 residency of multi-pass intermediates (bits): L2_LOAD_FIRST plain
    // loads marked evict-first, L2_STORE_LAST / L2_STORE_FIRST stores marked
    // evict-last / evict-first, L2_DISCARD_IN the tile's input lines dropped
    // from L2 without write-back once read (row tiles over a dead intermediate)
    int l2;
};

constexpr int L2_LOAD_FIRST = 1, L2_STORE_LAST = 2, L2_STORE_FIRST = 4, L2_DISCARD_IN = 8;

}  // namespace mgb
