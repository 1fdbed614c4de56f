// Contiguous batched transforms: loads and stores walk along each transform.
#include "fft_device.cuh"
#include "registry.h"

namespace mgb {

#define TILE_Q(L, R, C, Q)                                                                            \
    out.push_back(TileKernel{L, R, C, Q, ALONG, ALONG, (const void *)&tile_fft<L, R, C, Q, ALONG, ALONG>, \
                             C *(L / (R * Q)), tile_smem_bytes<L, R, C, Q, ALONG, ALONG>(),                \
                             tile_has_thi<L, R, C, Q, ALONG, ALONG>(), tile_exchange_bytes<L, R, C, Q, ALONG, ALONG>(), \
                             tile_c2r_rows_fn<L, R, C, Q>()})
#define TILE(L, R, C) TILE_Q(L, R, C, 1)

void register_tiles_along(std::vector<TileKernel> &out)
{
    TILE(2, 2, 256);
    TILE(4, 4, 256);
    TILE(8, 8, 256);
    TILE(16, 16, 256);
    TILE(32, 16, 128);
    TILE(64, 16, 64);
    TILE(128, 16, 32);
    TILE(256, 16, 16);
    TILE(512, 16, 8);
    // one transform per tile from 1024 points: measured faster than several
    // on GB300 for batches of every size (c2c 2048 x 1024: 12.4 -> 10.4 us,
    // c2r 4096 x 16384: 140.2 -> 132.7 us, r2c 4096 x 16: 6.2 -> 4.3 us) and for
    // the row passes of 2D transforms (4096^2 c2r 94.4 -> 91.1 us)
    TILE(1024, 16, 1);
    TILE(2048, 16, 1);
    TILE(4096, 16, 1);
    TILE(8192, 16, 1);
    TILE(8192, 32, 1);
    TILE_Q(8192, 16, 1, 2);  // clusters: the transform is spread over Q SMs
    TILE(16384, 16, 1);
    TILE(16384, 32, 1);
    TILE_Q(16384, 16, 1, 4);
    TILE_Q(32768, 16, 1, 8);
    TILE_Q(65536, 16, 1, 8);
    // wider batched tiles (after the defaults above), for the autotuner and
    // explicit tile choices
    TILE(1024, 16, 4);
    TILE(1024, 16, 2);
    TILE(2048, 16, 2);
}

}  // namespace mgb
