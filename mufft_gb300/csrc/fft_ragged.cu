// Ragged batched transforms: many c2c / r2c / c2r requests of mixed
// power-of-two lengths in one persistent launch.
//
// Each request is what one reference plan execute does (fft.c:811-850): a
// c2c transform of N points, or an r2c / c2r transform of N reals through an
// N/2-point complex transform and the real fix-up (kernel.c:36-82), with the
// reference's zero-padding and full-output flags.  Every CTA (256 threads)
// takes the next work item from a global counter; the host orders the items
// longest first.
//   Complex length L <= 4096: requests of one class (length, kind,
//     direction, zero padding, full output) run in groups, the C transforms
//     of one tile (C = 4096 / L, or 256 for L < 16) each taking its request's
//     buffers from a table; the r2c fix-up is fused into the tile's store,
//     the c2r fix-up into its loads.
//   L = 8192 .. 65536: a four-step L = L1 x L2 as phase tasks that any CTA
//     may take -- column tiles of L1 points (stride L2, twiddle W_L^(n2*k1)
//     fused into their stores, the c2r fix-up into their loads) into the
//     request's scratch, then row tiles of L2 points stored transposed into
//     natural order, then (r2c) the in-place fix-up in chunks.  A task waits
//     (bounded) on its request's counter until the previous phase is done;
//     phases are queued phase-major across requests, group tasks in between,
//     and every awaited task was dequeued earlier by a running CTA.
#include "../../include/fft.h"
#include "fft_device.cuh"
#include "fft_ragged.h"

namespace mgb {

namespace {

constexpr int kThreads = 256;

template <int L> __host__ __device__ constexpr int grp_r() { return L < 16 ? L : 16; }
template <int L> __host__ __device__ constexpr int grp_c() { return kThreads * grp_r<L>() / L; }

// Four-step split of 2^lg points: L1 (columns) x L2 (rows).
__host__ __device__ constexpr unsigned fr_l1(unsigned lg) { return lg == 13 ? 64 : (lg == 16 ? 256 : 128); }
__host__ __device__ constexpr unsigned fr_l2(unsigned lg) { return lg >= 15 ? 256 : 128; }

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Thread 0 waits (bounded) until *ctr >= target; CTA-uniform result.
__device__ bool wait_tasks(const unsigned *ctr, unsigned target, int *err)
{
    int ok = 1;
    if (threadIdx.x == 0) {
        for (unsigned i = 0; ld_acquire_u32(ctr) < target; i++) {
            if (i > (1u << 24) || *(volatile int *)err) {
                atomicExch(err, 1);
                ok = 0;
                break;
            }
            __nanosleep(128);
        }
    }
    return __syncthreads_and(ok) != 0;
}

// A group of n whole requests of one class: the n transforms of one tile.
template <int L>
__device__ void fr_group(const FftRaggedReq &q, const float2 *const *tab, unsigned n, float2 *smem,
                         const float2 *tw, const float2 *rtw_fwd, const float2 *rtw_inv)
{
    constexpr int R = grp_r<L>(), C = grp_c<L>();
    TileArgs a{};
    a.in = q.in;
    a.out = q.out;
    a.in_tab = tab;
    a.out_tab = (float2 *const *)(tab + n);
    a.in_stride = a.out_stride = 1;
    a.ntrans = n;
    a.half = (int)q.half;
    a.tw = tw;
    a.scale = 1.0f;
    if (q.kind == FR_C2C) {
        a.conj = q.inverse ? 3 : 0;
    } else if (q.kind == FR_R2C) {
        a.epilogue = q.full ? EPI_R2C_FULL : EPI_R2C;
        a.rtw = rtw_fwd;
    } else {
        a.prologue = PRO_C2R;
        a.conj = 3;
        a.rtw = rtw_inv;
        a.mirror_len = L;
    }
    tile_body<L, R, C, 1, ALONG, ALONG, false, false, false, false, false, true>(a, 0, 0, 0, 0, smem);
    __syncthreads();
}

// Column tiles of the first pass: L1-point columns n2 (stride L2) of the
// input into the scratch, times W_L^(n2*k1).
template <int L1, int L2>
__device__ void fr_columns(const FftRaggedReq &q, float2 *smem, const float2 *tw, const float2 *rtw_inv, int index)
{
    constexpr int C1 = kThreads * 16 / L1, L = L1 * L2;
    TileArgs a{};
    a.in = q.in;
    a.out = q.scratch;
    a.in_stride = a.out_stride = L2;
    a.in_dist = a.out_dist = 1;
    a.ntrans = L2;
    a.half = (int)q.half;
    a.epilogue = EPI_TWIDDLE;
    a.tw_scale = 2.0f / (float)L;
    a.tw_mask = L - 1;
    a.tw_colpow = 1;
    a.tw = tw;
    a.scale = 1.0f;
    if (q.kind == FR_C2C) {
        a.conj = q.inverse ? 1 : 0;
    } else if (q.kind == FR_C2R) {
        // fix-up of X[n] and X[L - n] with n = n1*L2 + n2 (local = n2 + n1*L2)
        a.prologue = PRO_C2R;
        a.conj = 1;
        a.rtw = rtw_inv;
        a.mirror_len = L;
        a.mirror_ldist = 1;
    }
    const int t0 = index < 0 ? 0 : index, t1 = index < 0 ? L2 / C1 : index + 1;
    for (int t = t0; t < t1; t++) {
        tile_body<L1, 16, C1, 1, ACROSS, ACROSS, false>(a, t, 0, 0, 0, smem);
        __syncthreads();
    }
}

// Row tiles of the second pass: rows k1 of L2 points of the scratch, output
// k2 stored at k1 + L1*k2 (natural order).
template <int L1, int L2>
__device__ void fr_rows(const FftRaggedReq &q, float2 *smem, const float2 *tw, int index)
{
    constexpr int C2 = kThreads * 16 / L2;
    TileArgs a{};
    a.in = q.scratch;
    a.out = q.out;
    a.in_stride = 1;
    a.in_dist = L2;
    a.out_stride = L1;
    a.out_dist = 1;
    a.ntrans = L1;
    a.tw = tw;
    a.scale = 1.0f;
    a.conj = (q.kind == FR_C2R || (q.kind == FR_C2C && q.inverse)) ? 2 : 0;
    const int t0 = index < 0 ? 0 : index, t1 = index < 0 ? L1 / C2 : index + 1;
    for (int t = t0; t < t1; t++) {
        tile_body<L2, 16, C2, 1, ALONG, ACROSS, true>(a, t, 0, 0, 0, smem);
        __syncthreads();
    }
}

// In-place r2c fix-up of the L-point complex transform in q.out (kernel.c:47-82):
// bin pairs k, L - k for k in this chunk of 0 .. L/2.
__device__ void fr_fixup(const FftRaggedReq &q, const float2 *rtw_fwd, int index)
{
    const long long L = 1ll << q.lg, half = L / 2;
    const long long n = half + 1;
    const long long k0 = index < 0 ? 0 : n * index / kFrFixupChunks;
    const long long k1 = index < 0 ? n : n * (index + 1) / kFrFixupChunks;
    float2 *z = q.out;
    for (long long k = k0 + threadIdx.x; k < k1; k += kThreads) {
        if (k == 0) {
            const float2 z0 = __ldcg(&z[0]);
            z[0] = make_float2(z0.x + z0.y, 0.f);
            z[L] = make_float2(z0.x - z0.y, 0.f);
            continue;
        }
        const long long km = L - k;
        const float2 zk = __ldcg(&z[k]), zm = __ldcg(&z[km]);
        float2 lo_k, hi_k, lo_m, hi_m;
        r2c_bins(zk, zm, __ldg(&rtw_fwd[k]), lo_k, hi_k);
        r2c_bins(zm, zk, __ldg(&rtw_fwd[km]), lo_m, hi_m);
        z[k] = lo_k;
        if (q.full)
            z[k + L] = hi_k;
        if (km != k) {
            z[km] = lo_m;
            if (q.full)
                z[km + L] = hi_m;
        }
    }
}

template <int L1, int L2>
__device__ void fr_phase(const FftRaggedReq &q, float2 *smem, const float2 *tw, const float2 *rf, const float2 *ri,
                         int phase, int index)
{
    if (phase == 0)
        fr_columns<L1, L2>(q, smem, tw, ri, index);
    else if (phase == 1)
        fr_rows<L1, L2>(q, smem, tw, index);
    else
        fr_fixup(q, rf, index);
}

// A whole four-step request in one CTA (requests below the split size).
template <int L1, int L2>
__device__ void fr_whole(const FftRaggedReq &q, float2 *smem, const float2 *tw, const float2 *rf, const float2 *ri)
{
    fr_phase<L1, L2>(q, smem, tw, rf, ri, 0, -1);
    fr_phase<L1, L2>(q, smem, tw, rf, ri, 1, -1);
    if (q.kind == FR_R2C) {
        fr_fixup(q, rf, -1);
        __syncthreads();
    }
}

}  // namespace

unsigned fft_ragged_group_size(unsigned lg)
{
    return lg == 0 ? 1u : (unsigned)(kThreads * (lg < 4 ? (1 << lg) : 16)) >> lg;
}

unsigned fft_ragged_phase_tasks(unsigned lg, unsigned phase, unsigned kind)
{
    const unsigned l1 = fr_l1(lg), l2 = fr_l2(lg);
    switch (phase) {
    case 0: return l2 / (kThreads * 16 / l1);
    case 1: return l1 / (kThreads * 16 / l2);
    default: return kind == FR_R2C ? kFrFixupChunks : 0;
    }
}

__global__ void __launch_bounds__(kThreads, 4) fft_ragged_kernel(const FftRaggedArgs args)
{
    extern __shared__ float2 smem[];
    __shared__ unsigned s_idx;
    for (;;) {
        if (threadIdx.x == 0)
            s_idx = atomicAdd(args.next, 1u);
        __syncthreads();
        const unsigned i = s_idx;
        __syncthreads();
        if (i >= args.count)
            return;
        const FftRaggedTask task = args.tasks[i];
        const FftRaggedReq q = args.reqs[task.req];
        const float2 *rf = args.rtw + args.rtw_off[q.lg];
        const float2 *ri = rf + (1u << q.lg);
        if (task.phase == kFrGroup) {
            const float2 *const *tab = args.tab + task.tab;
            switch (q.lg) {
            case 1: fr_group<2>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 2: fr_group<4>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 3: fr_group<8>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 4: fr_group<16>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 5: fr_group<32>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 6: fr_group<64>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 7: fr_group<128>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 8: fr_group<256>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 9: fr_group<512>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 10: fr_group<1024>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 11: fr_group<2048>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 12: fr_group<4096>(q, tab, task.index, smem, args.tw, rf, ri); break;
            default: break;
            }
            continue;
        }
        if (!q.split) {
            switch (q.lg) {
            case 13: fr_whole<64, 128>(q, smem, args.tw, rf, ri); break;
            case 14: fr_whole<128, 128>(q, smem, args.tw, rf, ri); break;
            case 15: fr_whole<128, 256>(q, smem, args.tw, rf, ri); break;
            case 16: fr_whole<256, 256>(q, smem, args.tw, rf, ri); break;
            default: break;
            }
            continue;
        }
        unsigned *ctr = args.next + 1 + q.counter;
        if (task.wait && !wait_tasks(ctr, task.wait, args.err))
            return;
        const int index = task.index == kFrWholePhase ? -1 : (int)task.index;
        switch (q.lg) {
        case 13: fr_phase<64, 128>(q, smem, args.tw, rf, ri, task.phase, index); break;
        case 14: fr_phase<128, 128>(q, smem, args.tw, rf, ri, task.phase, index); break;
        case 15: fr_phase<128, 256>(q, smem, args.tw, rf, ri, task.phase, index); break;
        case 16: fr_phase<256, 256>(q, smem, args.tw, rf, ri, task.phase, index); break;
        default: break;
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0)
            atomicAdd(ctr, 1u);
    }
}

namespace {

template <int L> constexpr size_t grp_bytes()
{
    return tile_smem_bytes<L, grp_r<L>(), grp_c<L>(), 1, ALONG, ALONG>();
}
template <int L1, int L2> constexpr size_t split_bytes()
{
    constexpr size_t a = tile_smem_bytes<L1, 16, kThreads * 16 / L1, 1, ACROSS, ACROSS>();
    constexpr size_t b = tile_smem_bytes<L2, 16, kThreads * 16 / L2, 1, ALONG, ACROSS>();
    return a > b ? a : b;
}

}  // namespace

size_t fft_ragged_smem()
{
    const size_t v[] = {grp_bytes<2>(),    grp_bytes<4>(),    grp_bytes<8>(),    grp_bytes<16>(),
                        grp_bytes<32>(),   grp_bytes<64>(),   grp_bytes<128>(),  grp_bytes<256>(),
                        grp_bytes<512>(),  grp_bytes<1024>(), grp_bytes<2048>(), grp_bytes<4096>(),
                        split_bytes<64, 128>(), split_bytes<128, 128>(), split_bytes<128, 256>(),
                        split_bytes<256, 256>()};
    size_t m = 0;
    for (size_t x : v)
        m = x > m ? x : m;
    return m;
}

const void *fft_ragged_fn() { return (const void *)&fft_ragged_kernel; }
int fft_ragged_threads() { return kThreads; }

}  // namespace mgb
