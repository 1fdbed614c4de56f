// Table of compiled tile-FFT instantiations, filled by the kernel translation
// units and searched by the planner.
#pragma once

#include <stddef.h>
#include <vector>

namespace mgb {

struct TileKernel {
    int L;          // transform length
    int R;          // elements per thread
    int C;          // transforms per tile
    int Q;          // CTAs per tile (thread-block cluster size)
    int lmap, smap; // thread maps of the load and store phases
    const void *fn;
    int threads;    // per CTA
    size_t smem;    // per CTA
    bool has_thi;   // column pass that takes the four-step twiddle table tw_lo
    size_t smem_ex; // per CTA without the four-step table region (launches with tw_lo == null)
    const void *fn_c2r = nullptr;  // row tiles: variant staging c2r fix-up rows in shared memory
};

void register_tiles_along(std::vector<TileKernel> &out);
void register_tiles_across(std::vector<TileKernel> &out);
void register_tiles_transpose(std::vector<TileKernel> &out);

// Returns the instantiation for (L, lmap, smap): the one matching the
// nonzero of C (transforms per tile), R (elements per thread) and Q (cluster
// size), else the one the options of the plan being built prefer, else the
// first registered.  nullptr if none exists.
const TileKernel *find_tile(int L, int lmap, int smap, int C = 0, int R = 0, int Q = 0);

}  // namespace mgb
