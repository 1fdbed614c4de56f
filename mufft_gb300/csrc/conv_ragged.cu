// Ragged batched fast convolution: many muFFT convolution requests of mixed
// power-of-two sizes in one persistent launch.
//
// A request is the reference's per-block convolution (fft.c:794-809): the
// first block is transformed (zero-padded input allowed), multiplied by the
// already transformed second block (a filter spectrum from
// mufft_execute_conv_input), scaled by 1/N and transformed back.  MONO_MONO
// goes through an N/2-point complex FFT with the r2c/c2r fix-ups,
// STEREO_MONO through an N-point complex FFT (fft.c:585-599).
//
// Every CTA (512 threads) takes the next work item from a global counter.
// The host orders the items (longest requests first) and decides which
// requests are split: a split request of L = L1 x L2 >= 16384 points runs as
// five phases of tasks (F1 column tiles, F2 row tiles, multiply chunks, I1 row
// tiles, I2 column tiles) that any CTA may take, each task waiting (bounded)
// on a per-request counter until the previous phase is complete; phases are
// queued phase-major across requests, so the waits are rarely long, and every
// awaited task was dequeued earlier by a running CTA (no deadlock).  A request
// that is not split runs whole in one CTA:
//   L <= 8192 complex points: one forward tile (r2c fix-up fused into its
//     store for mono) writes the spectrum to the request's scratch, which
//     stays in L2; one inverse tile reads it back with the multiply and the
//     c2r pre-pass fused into its loads.
//   L = 16384 .. 65536: an in-CTA four-step over the request's scratch,
//     L = L1 x L2.  The forward half stops at the transposed spectrum
//     X^T[k1][k2] = X[k1 + L1*k2] (no transpose), the multiply (and for mono
//     the r2c fix-up, product and c2r pre-pass of each bin pair k, L-k) runs
//     on that layout, and the inverse four-step consumes it directly:
//       F1 columns of L1 with W_L^(n2*k1) -> F2 rows of L2 -> multiply ->
//       I1 rows of L2 (inverse) with W_L^(-n2*k1) -> I2 columns of L1 -> output.
#include "../../include/fft.h"
#include "conv_ragged.h"
#include "fft_device.cuh"

namespace mgb {

namespace {

constexpr int kThreads = 512;

template <int L> __host__ __device__ constexpr int single_r() { return L > 8192 ? 32 : 16; }
template <int L> __host__ __device__ constexpr int single_c() { return kThreads * single_r<L>() / L; }

// Forward tile into the spectrum scratch, then the fused multiply + inverse
// tile into the output.
template <int L>
__device__ void conv_single(const RaggedReq &q, float2 *smem, const float2 *tw, const float2 *rtw_fwd,
                            const float2 *rtw_inv)
{
    constexpr int C = single_c<L>(), R = single_r<L>();
    const bool mono = q.stereo == 0;
    TileArgs f{};
    f.in = q.in;
    f.out = q.spec;
    f.in_stride = f.out_stride = 1;
    f.in_dist = f.out_dist = L + 1;
    f.ntrans = 1;
    f.half = q.zero_pad;
    f.epilogue = mono ? EPI_R2C : EPI_PLAIN;
    f.tw = tw;
    f.rtw = rtw_fwd;
    f.scale = 1.0f;
    tile_body<L, R, C, 1, ALONG, ALONG, false>(f, 0, 0, 0, 0, smem);
    __syncthreads();  // spectrum complete and visible to the whole CTA

    TileArgs b{};
    b.in = q.spec;
    b.in2 = q.h;
    b.out = q.out;
    b.in_stride = b.out_stride = 1;
    b.in_dist = b.out_dist = L + 1;
    b.ntrans = 1;
    b.prologue = mono ? PRO_MUL_C2R : PRO_MUL;
    b.mirror_len = L;
    b.rtw = rtw_inv;
    b.scale = q.scale;
    b.conj = 3;
    b.tw = tw;
    tile_body<L, R, C, 1, ALONG, ALONG, true>(b, 0, 0, 0, 0, smem);
    __syncthreads();
}

// A group of n whole requests of one class: the n transforms of one tile pair
// (the tile's C transforms each take one request's buffers from the tables).
template <int L>
__device__ void conv_group(const RaggedReq &q, const float2 *const *tab, unsigned n, float2 *smem, const float2 *tw,
                           const float2 *rtw_fwd, const float2 *rtw_inv)
{
    constexpr int C = single_c<L>(), R = single_r<L>();
    const bool mono = q.stereo == 0;
    const float2 *const *t_in = tab, *const *t_h = tab + n;
    float2 *const *t_out = (float2 *const *)(tab + 2 * n), *const *t_spec = (float2 *const *)(tab + 3 * n);
    TileArgs f{};
    f.in = q.in;
    f.out = q.spec;
    f.in_tab = t_in;
    f.out_tab = t_spec;
    f.in_stride = f.out_stride = 1;
    f.ntrans = n;
    f.half = q.zero_pad;
    f.epilogue = mono ? EPI_R2C : EPI_PLAIN;
    f.tw = tw;
    f.rtw = rtw_fwd;
    f.scale = 1.0f;
    tile_body<L, R, C, 1, ALONG, ALONG, false, false, false, false, false, true>(f, 0, 0, 0, 0, smem);
    __syncthreads();  // spectra complete and visible to the whole CTA

    TileArgs b{};
    b.in = q.spec;
    b.in2 = q.h;
    b.out = q.out;
    b.in_tab = (const float2 *const *)t_spec;
    b.in2_tab = t_h;
    b.out_tab = t_out;
    b.in_stride = b.out_stride = 1;
    b.ntrans = n;
    b.prologue = mono ? PRO_MUL_C2R : PRO_MUL;
    b.mirror_len = L;
    b.rtw = rtw_inv;
    b.scale = q.scale;
    b.conj = 3;
    b.tw = tw;
    tile_body<L, R, C, 1, ALONG, ALONG, true, false, false, false, false, true>(b, 0, 0, 0, 0, smem);
    __syncthreads();
}

// Multiply phase of the four-step path on the transposed spectrum, for the
// chunk `chunk` of `nchunks` (pairs k, L-k for mono; elements for stereo).
template <int L1, int L2>
__device__ void conv_multiply(const RaggedReq &q, const float2 *rtw_fwd, const float2 *rtw_inv, unsigned chunk,
                              unsigned nchunks)
{
    constexpr int L = L1 * L2;
    float2 *s = q.spec;
    auto at = [](int k) { return (k % L1) * L2 + k / L1; };  // X[k] lives at X^T[k % L1][k / L1]
    if (q.stereo) {
        const int i0 = (int)((long long)L * chunk / nchunks), i1 = (int)((long long)L * (chunk + 1) / nchunks);
        for (int idx = i0 + threadIdx.x; idx < i1; idx += kThreads) {
            const int k = (idx / L2) + L1 * (idx % L2);
            s[idx] = cscale(cmul(__ldcg(&s[idx]), __ldcg(&q.h[k])), q.scale);
        }
        return;
    }
    // mono: Z (forward complex FFT of the packed reals) -> r2c bins X -> Y = s*X*H
    // -> c2r pre-pass Zi, pair by pair (kernel.c:36-82).
    constexpr int NP = L / 2 + 1;
    const int k0 = (int)((long long)NP * chunk / nchunks), k1 = (int)((long long)NP * (chunk + 1) / nchunks);
    for (int k = k0 + threadIdx.x; k < k1; k += kThreads) {
        if (k == 0) {
            const float2 z0 = __ldcg(&s[0]);
            const float2 x0 = make_float2(z0.x + z0.y, 0.f), xm = make_float2(z0.x - z0.y, 0.f);
            const float2 y0 = cscale(cmul(x0, __ldcg(&q.h[0])), q.scale);
            const float2 ym = cscale(cmul(xm, __ldcg(&q.h[L])), q.scale);
            s[0] = c2r_fixup(y0, ym, __ldg(&rtw_inv[0]));
            continue;
        }
        const int km = L - k;
        const int ik = at(k), im = at(km);
        const float2 zk = __ldcg(&s[ik]), zm = __ldcg(&s[im]);
        float2 xk, xk_hi, xm, xm_hi;
        r2c_bins(zk, zm, __ldg(&rtw_fwd[k]), xk, xk_hi);
        r2c_bins(zm, zk, __ldg(&rtw_fwd[km]), xm, xm_hi);
        const float2 yk = cscale(cmul(xk, __ldcg(&q.h[k])), q.scale);
        const float2 ym = cscale(cmul(xm, __ldcg(&q.h[km])), q.scale);
        s[ik] = c2r_fixup(yk, ym, __ldg(&rtw_inv[k]));
        if (km != k)
            s[im] = c2r_fixup(ym, yk, __ldg(&rtw_inv[km]));
    }
}

template <int L1, int L2> __host__ __device__ constexpr int c1_of() { return kThreads * 16 / L1; }
template <int L1, int L2> __host__ __device__ constexpr int c2_of() { return kThreads * 16 / L2; }

// Tile arguments of the four phases that transform (F1, F2, I1, I2).
template <int L1, int L2>
__device__ TileArgs multi_args(const RaggedReq &q, const float2 *tw, int phase)
{
    constexpr int L = L1 * L2;
    TileArgs a{};
    a.tw = tw;
    a.scale = 1.0f;
    a.tw_scale = 2.0f / (float)L;
    a.tw_mask = L - 1;
    if (phase == 0 || phase == 4) {
        // columns of length L1 (n1), stride L2, twiddle W_L^(k1*n2) on the way in
        a.in = phase == 0 ? q.in : q.spec;
        a.out = phase == 0 ? q.spec : q.out;
        a.in_stride = a.out_stride = L2;
        a.in_dist = a.out_dist = 1;
        a.ntrans = L2;
        a.half = phase == 0 ? q.zero_pad : 0;
        a.epilogue = phase == 0 ? EPI_TWIDDLE : EPI_PLAIN;
        a.conj = phase == 0 ? 0 : 2;  // I2: inverse over k1 of conj(Z), conjugated out
    } else {
        // rows of length L2, in place; I1: inverse over k2 (conj in, forward FFT,
        // W_L^(n2*k1)) -> conj(Z)
        a.in = q.spec;
        a.out = q.spec;
        a.in_stride = a.out_stride = 1;
        a.in_dist = a.out_dist = L2;
        a.ntrans = L1;
        a.conj = phase == 3 ? 1 : 0;
        a.epilogue = phase == 3 ? EPI_TWIDDLE : EPI_PLAIN;
    }
    return a;
}

// One phase task of a split request (or, with index < 0, the whole phase).
template <int L1, int L2>
__device__ void multi_phase(const RaggedReq &q, float2 *smem, const float2 *tw, const float2 *rtw_fwd,
                            const float2 *rtw_inv, int phase, int index)
{
    constexpr int C1 = c1_of<L1, L2>(), C2 = c2_of<L1, L2>();
    if (phase == 2) {
        if (index < 0)
            conv_multiply<L1, L2>(q, rtw_fwd, rtw_inv, 0, 1);
        else
            conv_multiply<L1, L2>(q, rtw_fwd, rtw_inv, (unsigned)index, kRaggedMulChunks);
        return;
    }
    const TileArgs a = multi_args<L1, L2>(q, tw, phase);
    if (phase == 0 || phase == 4) {
        const int t0 = index < 0 ? 0 : index, t1 = index < 0 ? L2 / C1 : index + 1;
        for (int t = t0; t < t1; t++) {
            if (phase == 0)
                tile_body<L1, 16, C1, 1, ACROSS, ACROSS, false>(a, t, 0, 0, 0, smem);
            else
                tile_body<L1, 16, C1, 1, ACROSS, ACROSS, true>(a, t, 0, 0, 0, smem);
            __syncthreads();
        }
    } else {
        const int t0 = index < 0 ? 0 : index, t1 = index < 0 ? L1 / C2 : index + 1;
        for (int t = t0; t < t1; t++) {
            tile_body<L2, 16, C2, 1, ALONG, ALONG, true>(a, t, 0, 0, 0, smem);
            __syncthreads();
        }
    }
}

// Whole request through the in-CTA four-step.
template <int L1, int L2>
__device__ void conv_multi(const RaggedReq &q, float2 *smem, const float2 *tw, const float2 *rtw_fwd,
                           const float2 *rtw_inv)
{
    for (int phase = 0; phase < 5; phase++) {
        multi_phase<L1, L2>(q, smem, tw, rtw_fwd, rtw_inv, phase, -1);
        __syncthreads();
    }
}

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

}  // namespace

unsigned ragged_phase_tasks(unsigned lg, unsigned phase)
{
    // four-step split L1 x L2 of the in-CTA path: 2^14 = 128 x 128, 2^15 = 128 x 256, 2^16 = 256 x 256
    const unsigned l1 = lg == 16 ? 256 : 128, l2 = lg == 14 ? 128 : 256;
    const unsigned c1 = kThreads * 16 / l1, c2 = kThreads * 16 / l2;
    switch (phase) {
    case 0:
    case 4: return l2 / c1;
    case 1:
    case 3: return l1 / c2;
    default: return kRaggedMulChunks;
    }
}

__global__ void __launch_bounds__(kThreads, 1) conv_ragged_kernel(const RaggedArgs args)
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
        const RaggedTask task = args.tasks[i];
        const RaggedReq q = args.reqs[task.req];
        const float2 *rf = args.rtw + args.rtw_off[q.lg];
        const float2 *ri = rf + (1u << q.lg);
        if (q.split) {
            if (task.wait && !wait_tasks(&args.counters[q.counter], task.wait, args.err))
                return;
            switch (q.lg) {
            case 14: multi_phase<128, 128>(q, smem, args.tw, rf, ri, task.phase, task.index); break;
            case 15: multi_phase<128, 256>(q, smem, args.tw, rf, ri, task.phase, task.index); break;
            case 16: multi_phase<256, 256>(q, smem, args.tw, rf, ri, task.phase, task.index); break;
            default: break;
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0)
                atomicAdd(&args.counters[q.counter], 1u);
            continue;
        }
        if (task.phase == kRaggedGroupTask) {
            const float2 *const *tab = args.tab + task.pad;
            switch (q.lg) {
            case 4: conv_group<16>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 5: conv_group<32>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 6: conv_group<64>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 7: conv_group<128>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 8: conv_group<256>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 9: conv_group<512>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 10: conv_group<1024>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 11: conv_group<2048>(q, tab, task.index, smem, args.tw, rf, ri); break;
            case 12: conv_group<4096>(q, tab, task.index, smem, args.tw, rf, ri); break;
            default: break;
            }
            continue;
        }
        // whole requests up to 4096 points always come as group tasks (above)
        switch (q.lg) {
        case 13: conv_single<8192>(q, smem, args.tw, rf, ri); break;
        case 14: conv_single<16384>(q, smem, args.tw, rf, ri); break;
        case 15: conv_multi<128, 256>(q, smem, args.tw, rf, ri); break;
        case 16: conv_multi<256, 256>(q, smem, args.tw, rf, ri); break;
        default: break;
        }
    }
}

unsigned ragged_group_size(unsigned lg)
{
    switch (lg) {
    case 4: return single_c<16>();
    case 5: return single_c<32>();
    case 6: return single_c<64>();
    case 7: return single_c<128>();
    case 8: return single_c<256>();
    case 9: return single_c<512>();
    case 10: return single_c<1024>();
    case 11: return single_c<2048>();
    case 12: return single_c<4096>();
    default: return 1;
    }
}

template <int L> constexpr size_t single_bytes()
{
    return tile_exchange_bytes<L, single_r<L>(), single_c<L>(), 1, ALONG, ALONG>();
}
template <int L1, int L2> constexpr size_t multi_bytes()
{
    constexpr size_t a = tile_exchange_bytes<L1, 16, kThreads * 16 / L1, 1, ACROSS, ACROSS>();
    constexpr size_t b = tile_exchange_bytes<L2, 16, kThreads * 16 / L2, 1, ALONG, ALONG>();
    return a > b ? a : b;
}

size_t conv_ragged_smem()
{
    // every tile conv_ragged_kernel instantiates
    const size_t v[] = {single_bytes<16>(),   single_bytes<32>(),   single_bytes<64>(),   single_bytes<128>(),
                        single_bytes<256>(),  single_bytes<512>(),  single_bytes<1024>(), single_bytes<2048>(),
                        single_bytes<4096>(), single_bytes<8192>(), single_bytes<16384>(),
                        multi_bytes<128, 128>(), multi_bytes<128, 256>(), multi_bytes<256, 256>()};
    size_t m = 0;
    for (size_t x : v)
        m = x > m ? x : m;
    return m;
}

namespace {

// Phase launches of class pipelines (see conv_ragged.h): F1 reads the request's
// input, I2 writes its output, the others work on its spectrum scratch.
template <int L, int C, int LMAP, int SMAP>
__global__ void __launch_bounds__(tile_threads<L, 16, C, 1>(), tile_min_blocks<L, 16, C, 1>())
    class_tile(const TileArgs tmpl, const ClassEntry *tab, int phase)
{
    extern __shared__ float2 smem[];
    const ClassEntry e = tab[blockIdx.y];
    TileArgs a = tmpl;
    a.in = phase == 0 ? e.in : e.spec;
    a.out = phase == 4 ? e.out : e.spec;
    tile_body<L, 16, C, 1, LMAP, SMAP, false>(a, blockIdx.x, 0, 0, 0, smem);
}

// Phase 1 of a stereo class with the spectral multiply fused into its
// epilogue: rows k1 of X^T[k1][k2] = X[k1 + L1*k2], times s * H[k1 + L1*k2]
// (the template's in2_dist = 1, in2_stride = L1); the multiply launch is
// skipped.  Neighbouring rows of a tile read H's neighbouring elements.
template <int L, int C>
__global__ void __launch_bounds__(tile_threads<L, 16, C, 1>(), tile_min_blocks<L, 16, C, 1>())
    class_tile_mul(const TileArgs tmpl, const ClassEntry *tab, int phase)
{
    extern __shared__ float2 smem[];
    const ClassEntry e = tab[blockIdx.y];
    TileArgs a = tmpl;
    a.in = e.spec;
    a.out = e.spec;
    a.in2 = e.h;
    (void)phase;
    tile_body<L, 16, C, 1, ALONG, ALONG, false, false, false, false, true>(a, blockIdx.x, 0, 0, 0, smem);
}

// The multiply phase of a mono class (stereo classes fuse it into F2), on the
// transposed spectrum X^T[k1][k2] = X[k1 + L1*k2] of the packed reals (as
// conv_multiply above): the r2c pair X[k], X[L-k] sits in rows k1 and L1-k1
// (row 0 pairs with itself, column L2-k2).  A CTA takes 32 rows x 32 columns
// of the lower half (k2 < L2/2, i.e. k < L/2) of request blockIdx.z and the
// mirror elements, staged in shared memory by row-contiguous loads; the
// filter spectrum and the twiddle tables, indexed by k, are then read along
// k1 -- contiguously too.  k = 0 (paired with X[L]) and the self-mirrored
// k = L/2 (row 0, column L2/2) are the special cases.
__global__ void __launch_bounds__(256) class_multiply(const ClassEntry *tab, unsigned l1, unsigned l2, float scale,
                                                      const float2 *rtw_fwd, const float2 *rtw_inv)
{
    __shared__ float2 lo[32][33], hi[32][33];
    const ClassEntry e = tab[blockIdx.z];
    const int L1 = 1 << l1, L2 = 1 << l2, L = L1 * L2;
    float2 *s = e.spec;
    const int a = blockIdx.x * 32, b = blockIdx.y * 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    auto mirror = [&](int k1, int k2) { return k1 == 0 ? ((L2 - k2) & (L2 - 1)) : (L1 - k1) * L2 + (L2 - 1 - k2); };
    for (int i = w; i < 32; i += 8) {
        lo[i][lane] = s[(a + i) * L2 + b + lane];
        hi[i][lane] = s[mirror(a + i, b + lane)];
    }
    __syncthreads();
    for (int jj = w; jj < 32; jj += 8) {
        const int k = a + lane + L1 * (b + jj);
        if (k == 0) {
            // s[0] holds Z[0]: X[0] and X[L] from its real and imaginary parts
            const float2 z0 = lo[lane][jj];
            const float2 x0 = make_float2(z0.x + z0.y, 0.f), xm = make_float2(z0.x - z0.y, 0.f);
            const float2 y0 = cscale(cmul(x0, __ldg(&e.h[0])), scale);
            const float2 ym = cscale(cmul(xm, __ldg(&e.h[L])), scale);
            lo[lane][jj] = hi[lane][jj] = c2r_fixup(y0, ym, __ldg(&rtw_inv[0]));  // both name s[0]
            continue;
        }
        const int km = L - k;
        const float2 zk = lo[lane][jj], zm = hi[lane][jj];
        float2 xk, xk_hi, xm, xm_hi;
        r2c_bins(zk, zm, __ldg(&rtw_fwd[k]), xk, xk_hi);
        r2c_bins(zm, zk, __ldg(&rtw_fwd[km]), xm, xm_hi);
        const float2 yk = cscale(cmul(xk, __ldg(&e.h[k])), scale);
        const float2 ym = cscale(cmul(xm, __ldg(&e.h[km])), scale);
        lo[lane][jj] = c2r_fixup(yk, ym, __ldg(&rtw_inv[k]));
        hi[lane][jj] = c2r_fixup(ym, yk, __ldg(&rtw_inv[km]));
    }
    __syncthreads();
    for (int i = w; i < 32; i += 8) {
        s[(a + i) * L2 + b + lane] = lo[i][lane];
        s[mirror(a + i, b + lane)] = hi[i][lane];
    }
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
        const int k = L / 2, idx = L2 / 2;  // row 0, column L2/2: X[L/2] pairs with itself
        const float2 zk = s[idx];
        float2 xk, xk_hi;
        r2c_bins(zk, zk, __ldg(&rtw_fwd[k]), xk, xk_hi);
        const float2 yk = cscale(cmul(xk, __ldg(&e.h[k])), scale);
        s[idx] = c2r_fixup(yk, yk, __ldg(&rtw_inv[k]));
    }
}

}  // namespace

ClassTile class_column_tile(int L1)
{
    if (L1 == 128)
        return ClassTile{(const void *)&class_tile<128, 32, ACROSS, ACROSS>, 128, 32, tile_threads<128, 16, 32, 1>(),
                         tile_smem_bytes<128, 16, 32, 1, ACROSS, ACROSS>()};
    return ClassTile{(const void *)&class_tile<256, 16, ACROSS, ACROSS>, 256, 16, tile_threads<256, 16, 16, 1>(),
                     tile_smem_bytes<256, 16, 16, 1, ACROSS, ACROSS>()};
}

ClassTile class_row_tile(int L2)
{
    if (L2 == 128)
        return ClassTile{(const void *)&class_tile<128, 32, ALONG, ALONG>, 128, 32, tile_threads<128, 16, 32, 1>(),
                         tile_smem_bytes<128, 16, 32, 1, ALONG, ALONG>()};
    return ClassTile{(const void *)&class_tile<256, 16, ALONG, ALONG>, 256, 16, tile_threads<256, 16, 16, 1>(),
                     tile_smem_bytes<256, 16, 16, 1, ALONG, ALONG>()};
}

ClassTile class_row_mul_tile(int L2)
{
    if (L2 == 128)
        return ClassTile{(const void *)&class_tile_mul<128, 32>, 128, 32, tile_threads<128, 16, 32, 1>(),
                         tile_smem_bytes<128, 16, 32, 1, ALONG, ALONG>()};
    return ClassTile{(const void *)&class_tile_mul<256, 16>, 256, 16, tile_threads<256, 16, 16, 1>(),
                     tile_smem_bytes<256, 16, 16, 1, ALONG, ALONG>()};
}

const void *class_multiply_fn() { return (const void *)&class_multiply; }

const void *conv_ragged_fn() { return (const void *)&conv_ragged_kernel; }
int conv_ragged_threads() { return kThreads; }

}  // namespace mgb
