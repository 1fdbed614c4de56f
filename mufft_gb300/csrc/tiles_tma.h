// Column-pass kernels with TMA-staged inputs (tiles_tma.cu).
#pragma once

#include <stddef.h>
#include <vector>

namespace mgb {

struct TmaTileKernel {
    int L;             // column length (<= 256: one TMA box per tile)
    int R;             // elements per thread
    int C;             // columns per tile
    int nbuf;          // staging buffers (2: the next tile's copy overlaps this tile's work)
    const void *fn;    // kernel(const CUtensorMap map, TileArgs a, unsigned tiles_x, unsigned ntiles, int *err)
    int threads;
    size_t smem;
    bool has_thi;
    size_t buf_bytes;
};

void register_tiles_tma(std::vector<TmaTileKernel> &out);

}  // namespace mgb
