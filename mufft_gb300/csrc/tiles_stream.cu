// Batched contiguous transforms (and 2D row passes) as persistent CTAs that
// stream their tiles.
//
// A grid of ordinary tiles that fills the GPU only about once (4096 x 1024
// points, a 4096-row 2D pass) runs in lockstep: every CTA loads, then every
// CTA computes while HBM idles, then every CTA stores.  Here each CTA walks
// tiles blockIdx.x, blockIdx.x + gridDim.x, ... and issues the stage-0 loads
// of its next tile into a second register set before it transforms the
// current one, so reads stay in flight through the FFT stages and the
// stores.  Loads, stages, prologues and epilogues are the code of every other
// row tile (tile_body with preloaded registers).
#include "fft_device.cuh"
#include "tiles_stream.h"

namespace mgb {

namespace {

template <int L, int R, int C>
__global__ void __launch_bounds__(tile_threads<L, R, C, 1>()) tile_fft_stream(const TileArgs a, const unsigned ntiles)
{
    extern __shared__ float2 smem[];
    constexpr int TL = Tile<L, R, 1>::TL;
    unsigned t = blockIdx.x;
    if (t >= ntiles)
        return;
    int c, tl;
    split_tid<ALONG, C, TL>(threadIdx.x, c, tl);
    float2 v[R];
    load_stage0<L, R, 1, ALONG, false>(a, a.in, a.in2, t * C + c, 0, tl, v);
    for (;;) {
        const unsigned tn = t + gridDim.x;
        float2 vn[R];
        // the next tile's loads, in flight during this tile's stages and stores
        if (tn < ntiles)
            load_stage0<L, R, 1, ALONG, false>(a, a.in, a.in2, tn * C + c, 0, tl, vn);
        tile_body<L, R, C, 1, ALONG, ALONG, false, false, true>(a, t, 0, 0, 0, smem, nullptr, 0, v);
        if (tn >= ntiles)
            break;
        __syncthreads();  // the exchange slices are free for the next tile
#pragma unroll
        for (int q = 0; q < R; q++)
            v[q] = vn[q];
        t = tn;
    }
}

}  // namespace

void register_tiles_stream(std::vector<StreamTileKernel> &out)
{
#define STREAM_TILE(L, R, C)                                                                            \
    out.push_back(StreamTileKernel{L, R, C, (const void *)&tile_fft_stream<L, R, C>, tile_threads<L, R, C, 1>(), \
                                   tile_smem_bytes<L, R, C, 1, ALONG, ALONG>()})
    STREAM_TILE(256, 16, 16);
    STREAM_TILE(512, 16, 8);
    STREAM_TILE(1024, 16, 4);
    STREAM_TILE(1024, 16, 2);
    STREAM_TILE(1024, 16, 1);
    STREAM_TILE(2048, 16, 2);
    STREAM_TILE(2048, 16, 1);
    STREAM_TILE(4096, 16, 1);
#undef STREAM_TILE
}

}  // namespace mgb
