// Persistent row-tile kernels with register prefetch (tiles_stream.cu).
#pragma once

#include <stddef.h>
#include <vector>

namespace mgb {

struct StreamTileKernel {
    int L;           // transform length
    int R;           // elements per thread
    int C;           // transforms per tile
    const void *fn;  // kernel(TileArgs a, unsigned ntiles)
    int threads;
    size_t smem;
};

void register_tiles_stream(std::vector<StreamTileKernel> &out);

}  // namespace mgb
