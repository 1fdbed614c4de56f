// Tile passes as a persistent grid: as many CTAs as are resident at once,
// each walking tiles blockIdx.x, blockIdx.x + gridDim.x, ... of the pass
// (tile t is column block t % tiles_x of grid row t / tiles_x, the
// blockIdx.x / blockIdx.y of the one-CTA-per-tile launch).  Same tile code,
// same results bit for bit; the CTAs start their next tile's loads right
// after their stores instead of leaving and being replaced.
//
// Only the 1024-thread 4096-point column tile has this variant: with one CTA
// per SM (16384 points fill the register file) it measured faster on GB300
// (4096^2 r2c 78.0 -> 77.2 us, c2r 94.4 -> 92.3 us, c2c 131.0 -> 127.6 us),
// while tiles that run several CTAs per SM lost (the three 256-point passes
// of 2^24: 137.5 -> 144.7 us; 2048-point row tiles: 37.1 -> 40.2 us for
// a 4096 x 2048 r2c).  Staging the next tile's first stage-0 values in
// shared memory by cp.async while the current tile runs was built and
// verified as well and measured slower the more it staged (2 of 16 values
// per thread 79.1 us, 6: 79.1, 11: 94.3 for the 4096^2 r2c): the staging
// slots take the shared memory that the L1 needs for the misses in flight
// of the 32-byte column segments.
#include "fft_device.cuh"
#include "tiles_persist.h"

namespace mgb {

namespace {

template <int L, int R, int C, int LMAP, int SMAP>
__global__ void __launch_bounds__(tile_threads<L, R, C, 1>(), tile_min_blocks<L, R, C, 1>())
    tile_fft_persist(const TileArgs a, const unsigned tiles_x, const unsigned ntiles)
{
    extern __shared__ float2 smem[];
    for (unsigned t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const unsigned tx = t % tiles_x, z = t / tiles_x;
        long long ioff, ooff;
        if (a.ysplit) {
            const unsigned g = z % a.ysplit, b = z / a.ysplit;
            ioff = (long long)g * a.in_batch + (long long)b * a.in_batch2;
            ooff = (long long)g * a.out_batch + (long long)b * a.out_batch2;
        } else {
            ioff = (long long)z * a.in_batch;
            ooff = (long long)z * a.out_batch;
        }
        tile_body<L, R, C, 1, LMAP, SMAP, false>(a, tx, 0, ioff, ooff, smem, nullptr, z);
        __syncthreads();  // the exchange slices and twiddle region are free for the next tile
    }
}

}  // namespace

void register_tiles_persist(std::vector<PersistTileKernel> &out)
{
#define PERSIST_TILE(L, R, C, LM, SM)                                                                       \
    out.push_back(PersistTileKernel{L, R, C, LM, SM, (const void *)&tile_fft_persist<L, R, C, LM, SM>, \
                                    tile_threads<L, R, C, 1>()})
    PERSIST_TILE(4096, 16, 4, ACROSS, ACROSS);
#undef PERSIST_TILE
}

}  // namespace mgb
