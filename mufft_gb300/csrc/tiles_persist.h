// Persistent tile kernels: one grid of resident CTAs walks all tiles of a
// pass (tiles_persist.cu).
#pragma once

#include <stddef.h>
#include <vector>

namespace mgb {

struct PersistTileKernel {
    int L;           // transform length
    int R;           // elements per thread
    int C;           // transforms per tile
    int lmap, smap;  // thread maps of the load and store phases
    const void *fn;  // kernel(TileArgs a, unsigned tiles_x, unsigned ntiles)
    int threads;
};

void register_tiles_persist(std::vector<PersistTileKernel> &out);

}  // namespace mgb
