// Last two passes of a three-level transform in one persistent launch, with
// their intermediate kept in L2.
//
// A transform of M = N1 * 256 * 256 points is factored as M = N1 x (256 x 256).
// Pass A (a separate column-tile launch) leaves Y[k1][m], m < 65536.  For each
// row k1 the remaining 65536-point FFT is itself a four-step:
//   B: per row, column FFTs of length 256 over n3 < 256 (stride 256), with the
//      twiddle W_65536^(k2*n3), into Z[k1][k2][n3];
//   C: rows (k1, k2) of length 256, stored transposed to X[k1 + N1*(k2 + 256*k3)].
// A C tile needs 16 consecutive rows k1 for coalesced 128-byte stores, i.e.
// every B tile of a block of 16 rows.  Rows are therefore processed in blocks
// of 16: per block 256 B tasks (16 rows x 16 column tiles) then 256 C tasks
// (one per k2).  The block's Z (8 MiB) goes to a ring of RING slots that stays
// resident in L2, so HBM carries Y once in and X once out; run separately, B
// and C would add a full write and read of the intermediate.
//
// Scheduling: CTAs take task indices from a global counter in the order
// B0, B1, C0, B2, C1, ..., B(n-1), C(n-2), C(n-1).  A C task waits for all B
// tasks of its block; a B task waits for the C tasks of the block that last
// used its ring slot.  Every task a CTA waits for was dequeued earlier by a
// running CTA, and B tasks of a block never wait on later tasks, so the
// schedule cannot deadlock whether or not all CTAs are resident.  Waits are
// bounded: on timeout the kernel records an error and every CTA leaves.
#include "bc_fused.h"
#include "fft_device.cuh"

namespace mgb {

namespace {

constexpr int kBcL = 256;       // B and C tile length
constexpr int kBcC = 16;        // transforms per tile
constexpr int kBcR = 16;        // elements per thread
constexpr int kBcThreads = 256; // kBcC * kBcL / kBcR
constexpr unsigned kTasksPerGroup = 256;
constexpr long long kRowLen = 65536;

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Thread 0 waits until *ctr >= target (bounded); returns false on timeout.
__device__ bool wait_counter(const unsigned *ctr, unsigned target, int *err)
{
    __shared__ int ok;
    if (threadIdx.x == 0) {
        ok = 1;
        unsigned long long spins = 0;
        while (ld_acquire(ctr) < target) {
            if (++spins > (1ull << 24) || *((volatile int *)err)) {
                atomicExch(err, 1);
                ok = 0;
                break;
            }
            __nanosleep(256);
        }
    }
    __syncthreads();
    return ok != 0;
}

__device__ void signal_done(unsigned *ctr)
{
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
        atomicAdd(ctr, 1u);
}

}  // namespace

__global__ void __launch_bounds__(kBcThreads, 4) bc_persistent(const BcArgs p)
{
    extern __shared__ float2 smem[];
    __shared__ unsigned s_task;
    const unsigned ngroups = 2 * p.nblk;
    const unsigned total = ngroups * kTasksPerGroup;
    unsigned *doneB = p.counters;
    unsigned *doneC = p.counters + p.nblk;
    unsigned *next = p.counters + 2 * p.nblk;
    for (;;) {
        if (threadIdx.x == 0)
            s_task = atomicAdd(next, 1u);
        __syncthreads();
        const unsigned t = s_task;
        __syncthreads();
        if (t >= total)
            return;
        const unsigned g = t / kTasksPerGroup, local = t % kTasksPerGroup;
        bool isB;
        unsigned kb;
        if (g == 0) {
            isB = true;
            kb = 0;
        } else if (g & 1) {
            kb = (g + 1) / 2;
            isB = kb < p.nblk;
            if (!isB)
                kb = p.nblk - 1;
        } else {
            isB = false;
            kb = g / 2 - 1;
        }
        const unsigned b = kb / p.blk_per_item;          // batch item
        const unsigned r0 = (kb % p.blk_per_item) * kBcC; // first row k1 of the block
        float2 *slot = p.ring + (long long)(kb % p.ring_slots) * kBcC * kRowLen;
        if (isB) {
            if (kb >= p.ring_slots && !wait_counter(&doneC[kb - p.ring_slots], kTasksPerGroup, p.err))
                return;
            // 16 rows x 16 column tiles: row r0 + local/16, columns tile local%16
            const unsigned row = local / kBcC, ct = local % kBcC;
            TileArgs a = p.b;
            a.in = p.y + (long long)b * p.y_item + (long long)(r0 + row) * kRowLen;
            a.out = slot + (long long)row * kRowLen;
            tile_body<kBcL, kBcR, kBcC, 1, ACROSS, ACROSS, false>(a, ct, 0, 0, 0, smem);
            signal_done(&doneB[kb]);
        } else {
            if (!wait_counter(&doneB[kb], kTasksPerGroup, p.err))
                return;
            // one k2: rows (k1 = r0..r0+15, k2), each 256 contiguous points
            const unsigned k2 = local;
            TileArgs a = p.c;
            a.in = slot + (long long)k2 * kBcL;
            a.out = p.x + (long long)b * p.x_item + r0 + (long long)k2 * p.n1;
            tile_body<kBcL, kBcR, kBcC, 1, ALONG, ACROSS, true>(a, 0, 0, 0, 0, smem);
            signal_done(&doneC[kb]);
        }
        __syncthreads();  // smem is reused by the next task
    }
}

size_t bc_smem_bytes()
{
    const size_t sb = tile_smem_bytes<kBcL, kBcR, kBcC, 1, ACROSS, ACROSS>();
    const size_t sc = tile_smem_bytes<kBcL, kBcR, kBcC, 1, ALONG, ACROSS>();
    return sb > sc ? sb : sc;
}

const void *bc_kernel() { return (const void *)&bc_persistent; }

int bc_threads() { return kBcThreads; }

}  // namespace mgb
