// Persistent column-tile kernels that prefetch their next tile into L2.
//
// A column tile reads C neighbouring columns of L points: L rows of C*8
// contiguous bytes, far apart in memory.  When a tile needs all the registers
// an SM has (4096-point columns: 1024 threads x 16 points), one CTA runs per
// SM and nothing overlaps its load, compute and store phases.  Here the CTA
// is persistent and, before it transforms tile t, asks L2 for the rows of
// tile t + gridDim.x (one prefetch per row segment, no registers held), so
// that the next tile's loads find their data in L2 instead of HBM.  The FFT
// stages, epilogues and stores are the register-tile code of every other pass.
#include "fft_device.cuh"
#include "tiles_stream.h"

namespace mgb {

namespace {

template <int L, int R, int C>
__global__ void __launch_bounds__(tile_threads<L, R, C, 1>(), tile_min_blocks<L, R, C, 1>())
    tile_fft_cols_pf(const TileArgs a, unsigned ntiles)
{
    extern __shared__ float2 smem[];
    constexpr int T = tile_threads<L, R, C, 1>();
    // rows that the tile reads: the upper half of a zero-padded input is not there
    const int rows = a.half ? L / 2 : L;
    for (unsigned t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const unsigned tn = t + gridDim.x;
        if (tn < ntiles) {
            // first column of the next tile (a valid column: tn * C < ntrans)
            const float2 *base = a.in + (long long)tn * C * a.in_dist;
            for (int n = threadIdx.x; n < rows; n += T)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (long long)n * a.in_stride));
        }
        tile_body<L, R, C, 1, ACROSS, ACROSS, false>(a, t, 0, 0, 0, smem);
        __syncthreads();
    }
}

}  // namespace

#define PF_TILE(L, R, C)                                                                                    \
    out.push_back(StreamTileKernel{L, R, C, (const void *)&tile_fft_cols_pf<L, R, C>, tile_threads<L, R, C, 1>(), \
                                   tile_smem_bytes<L, R, C, 1, ACROSS, ACROSS>()})

void register_tiles_prefetch(std::vector<StreamTileKernel> &out)
{
    PF_TILE(4096, 16, 4);
    PF_TILE(2048, 16, 4);
    PF_TILE(1024, 16, 8);
    PF_TILE(256, 16, 16);
}

}  // namespace mgb
