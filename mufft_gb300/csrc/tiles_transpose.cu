// Row passes with transposed stores (second pass of the four-step FFT): loads
// walk along each row, stores walk across neighbouring rows.
#include "fft_device.cuh"
#include "registry.h"

namespace mgb {

#define TILE_Q(L, R, C, Q)                                                                            \
    out.push_back(TileKernel{L, R, C, Q, ALONG, ACROSS, (const void *)&tile_fft<L, R, C, Q, ALONG, ACROSS>, \
                             C *(L / (R * Q)), tile_smem_bytes<L, R, C, Q, ALONG, ACROSS>(),                \
                             tile_has_thi<L, R, C, Q, ALONG, ACROSS>(), tile_exchange_bytes<L, R, C, Q, ALONG, ACROSS>()})
#define TILE(L, R, C) TILE_Q(L, R, C, 1)

void register_tiles_transpose(std::vector<TileKernel> &out)
{
    TILE(32, 16, 128);
    TILE(64, 16, 64);
    TILE(128, 16, 32);
    TILE(256, 16, 16);
    TILE(256, 16, 32);
    TILE(512, 16, 8);
    TILE(1024, 16, 8);
    TILE(1024, 16, 16);
    TILE(2048, 16, 4);
    TILE(2048, 16, 8);
    TILE(4096, 16, 4);       // default: measured fastest for the 4096 x 4096 four-step
    TILE_Q(4096, 16, 4, 4);  // the same tile spread over a 4-CTA cluster
    TILE(4096, 16, 2);
    TILE(4096, 32, 4);
    TILE(4096, 32, 2);
    TILE(8192, 32, 2);
    TILE(16384, 32, 1);
}

}  // namespace mgb
