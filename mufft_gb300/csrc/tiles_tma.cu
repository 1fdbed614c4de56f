// Column passes with TMA-staged inputs.
//
// The column tiles of a multi-pass transform read C neighbouring columns of L
// points each: L rows of C*8 contiguous bytes, far apart in memory.  Here one
// thread moves the whole tile with a single cp.async.bulk.tensor (a 3D box
// {C columns, L rows, 1}) into shared memory, completing on an mbarrier, and
// the CTA is persistent: while it transforms tile i from one buffer, the copy
// of tile i + gridDim.x fills the other.  The FFT stages, the twiddle
// epilogue and the stores are the register-tile code of every other pass.
//
// Tile t covers columns x = (t % tiles_x) * C of row block z = t / tiles_x;
// the tensor map describes the pass input as {columns, L, blocks}.  Waits are
// bounded: on timeout the kernel records an error, waits (bounded) for its
// copies in flight and returns.
#include <cuda.h>

#include "fft_device.cuh"
#include "tiles_tma.h"

namespace mgb {

namespace {

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity)
{
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
    for (unsigned i = 0; i < (1u << 22); i++)
        if (mbar_try(bar, parity))
            return true;
    return false;
}

template <int L, int C>
__device__ __forceinline__ void tma_tile(const CUtensorMap *map, unsigned dst, unsigned bar, unsigned x, unsigned z)
{
    constexpr unsigned bytes = (unsigned)(L * C * sizeof(float2));
    // earlier generic-proxy reads of this buffer are ordered before the copy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            dst),
        "l"((unsigned long long)map), "r"(x), "r"(0u), "r"(z), "r"(bar)
        : "memory");
}

template <int L, int R, int C> __host__ __device__ constexpr size_t tma_buf_bytes() { return ((size_t)L * C * sizeof(float2) + 1023) & ~(size_t)1023; }
template <int L, int R, int C> __host__ __device__ constexpr size_t tma_region_bytes()
{
    return (tile_smem_bytes<L, R, C, 1, ACROSS, ACROSS>() + 15) & ~(size_t)15;
}

template <int L, int R, int C, int NBUF>
__global__ void __launch_bounds__(tile_threads<L, R, C, 1>(), 2)
    tile_fft_tma(const __grid_constant__ CUtensorMap map, const TileArgs a, const unsigned tiles_x,
                 const unsigned ntiles, int *err)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    constexpr size_t BUF = tma_buf_bytes<L, R, C>();
    float2 *ex = (float2 *)(sm + NBUF * BUF);
    unsigned long long *bars = (unsigned long long *)(sm + NBUF * BUF + tma_region_bytes<L, R, C>());
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int b = 0; b < NBUF; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&bars[b])), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    unsigned t = blockIdx.x;
    if (tid == 0 && t < ntiles)
        tma_tile<L, C>(&map, smem_addr(sm), smem_addr(&bars[0]), (t % tiles_x) * C, t / tiles_x);
    bool ok = true;
    bool prefetched = false;  // a copy for the next iteration is in flight
    unsigned i = 0;
    for (; t < ntiles; t += gridDim.x, i++) {
        const unsigned b = NBUF == 2 ? (i & 1) : 0;
        const unsigned tn = t + gridDim.x;
        prefetched = NBUF == 2 && tn < ntiles;
        if (prefetched && tid == 0)
            tma_tile<L, C>(&map, smem_addr(sm + (b ^ 1) * BUF), smem_addr(&bars[b ^ 1]), (tn % tiles_x) * C,
                           tn / tiles_x);
        const unsigned parity = (NBUF == 2 ? (i >> 1) : i) & 1;
        ok = __syncthreads_and(mbar_wait(smem_addr(&bars[b]), parity)) != 0;
        if (!ok)
            break;
        const unsigned tx = t % tiles_x, z = t / tiles_x;
        long long ooff;
        if (a.ysplit) {
            const unsigned g = z % a.ysplit, bb = z / a.ysplit;
            ooff = (long long)g * a.out_batch + (long long)bb * a.out_batch2;
        } else {
            ooff = (long long)z * a.out_batch;
        }
        tile_body<L, R, C, 1, ACROSS, ACROSS, false, true>(a, tx, 0, 0, ooff, ex, (const float2 *)(sm + b * BUF));
        __syncthreads();  // the buffer and the exchange region are free again
        if (NBUF == 1 && tid == 0 && tn < ntiles)
            tma_tile<L, C>(&map, smem_addr(sm), smem_addr(&bars[0]), (tn % tiles_x) * C, tn / tiles_x);
    }
    if (!ok) {
        if (tid == 0 && err)
            atomicExch(err, 1);
        // copies still in flight land before the CTA leaves (bounded): the one
        // that timed out, and the prefetch issued with it
        const unsigned b = NBUF == 2 ? (i & 1) : 0;
        mbar_wait(smem_addr(&bars[b]), (NBUF == 2 ? (i >> 1) : i) & 1);
        if (prefetched)
            mbar_wait(smem_addr(&bars[b ^ 1]), ((i + 1) >> 1) & 1);
    }
}

template <int L, int R, int C, int NBUF> constexpr size_t tma_smem()
{
    return NBUF * tma_buf_bytes<L, R, C>() + tma_region_bytes<L, R, C>() + 2 * sizeof(unsigned long long);
}

}  // namespace

void register_tiles_tma(std::vector<TmaTileKernel> &out)
{
#define TMA_TILE(L, R, C, NB)                                                                                    \
    out.push_back(TmaTileKernel{L, R, C, NB, (const void *)&tile_fft_tma<L, R, C, NB>, tile_threads<L, R, C, 1>(), \
                                tma_smem<L, R, C, NB>(), tile_has_thi<L, R, C, 1, ACROSS, ACROSS>(),              \
                                tma_buf_bytes<L, R, C>() * NB})
    TMA_TILE(256, 16, 16, 2);
    TMA_TILE(256, 16, 16, 1);
    TMA_TILE(128, 16, 32, 2);
    TMA_TILE(128, 16, 32, 1);
    TMA_TILE(64, 16, 64, 2);
    TMA_TILE(64, 16, 64, 1);
#undef TMA_TILE
}

}  // namespace mgb
