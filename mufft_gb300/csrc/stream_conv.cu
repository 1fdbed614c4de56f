// One block of the uniformly partitioned overlap-save convolution as a single
// launch, for windows that one 256-thread row tile transforms.
//
// CTA 0 transforms the window [previous | input] (the forward row tile, the
// same code as every other row pass), moves the input half to the previous
// half and publishes the spectrum (flag = k + 1).  Every other CTA (bin group
// x of 64 bins, partition range g) multiply-accumulates the delay-line spectra
// of blocks k-1 .. k-P+1 with filter partitions 1 .. P-1 -- work that does not
// need the current spectrum -- and writes its partial.  The last range CTA of
// a group (ticket) waits for the spectrum, adds the partials in range order
// plus the current spectrum times partition 0, scales, writes y and stores the
// current spectrum in the delay line.  The CTA that finishes the last group
// runs the inverse row tile on y and advances the block count.
//
// Only a group's finishing CTA waits, and only for CTA 0, which waits for
// nobody; the grid is sized so that all CTAs are resident together.  The wait
// is bounded: on timeout the CTA records an error and leaves the group's
// output and delay-line bins unwritten, but still does the group's ticket
// bookkeeping (and, if it is the last group, the inverse transform and the
// block count), so the next launch starts from consistent tickets.
//   tickets[0] = k, [1] groups finished, [2] = k + 1 once the spectrum of
//   block k is out, [3 + x] range CTAs done with group x.
#include "fft_device.cuh"
#include "stream_conv.h"

namespace mgb {

namespace {

constexpr int kWarps = 8;
constexpr unsigned kBins = 64;  // per group: two per lane

__device__ __forceinline__ void cmac2(float4 &acc, const float4 a, const float4 b)
{
    acc.x += a.x * b.x - a.y * b.y;
    acc.y += a.x * b.y + a.y * b.x;
    acc.z += a.z * b.z - a.w * b.w;
    acc.w += a.z * b.w + a.w * b.z;
}

__device__ __forceinline__ float4 add4(float4 a, const float4 b)
{
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
    a.w += b.w;
    return a;
}

// Bins b, b + 1 of an nb-bin vector written earlier in this launch.
__device__ __forceinline__ float4 load_bins_cg(const float2 *v, unsigned b, unsigned nb)
{
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    if (b < nb) {
        const float2 v0 = __ldcg(&v[b]);
        r.x = v0.x;
        r.y = v0.y;
    }
    if (b + 1 < nb) {
        const float2 v1 = __ldcg(&v[b + 1]);
        r.z = v1.x;
        r.w = v1.y;
    }
    return r;
}

// Tickets and flags: one thread releases what its CTA wrote before a
// __syncthreads, or acquires what other CTAs released before it lets its CTA
// read (after a __syncthreads).
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *p, unsigned v)
{
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

template <int M>
__global__ void __launch_bounds__(256) upols_block(const UpolsBlockArgs a)
{
    extern __shared__ float2 smem[];
    __shared__ float4 red[kWarps][32];
    __shared__ unsigned flag;
    constexpr int C = 4096 / M;
    static_assert(C * (M / 16) == 256, "256-thread row tile");
    const unsigned k = *(volatile unsigned *)&a.tickets[0];
    const unsigned cur = k % a.P;
    const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;

    if (blockIdx.x == 0) {
        tile_body<M, 16, C, 1, ALONG, ALONG, false>(a.fwd, 0, 0, 0, 0, smem);
        __syncthreads();  // the spectrum is written and the whole window has been read
        if (threadIdx.x == 0)
            st_release(&a.tickets[2], k + 1);
        // the input half becomes the previous half (nobody else reads the window)
        for (unsigned i = threadIdx.x; i < a.half16; i += blockDim.x)
            a.win[i] = a.win[a.half16 + i];
        return;
    }

    const unsigned id = blockIdx.x - 1;
    const unsigned x = id % a.groups, g = id / a.groups;
    const unsigned np = a.P - 1;  // partitions 1 .. P-1
    const unsigned p0 = 1 + (unsigned)((unsigned long long)np * g / a.G);
    const unsigned p1 = 1 + (unsigned)((unsigned long long)np * (g + 1) / a.G);
    const unsigned b = x * kBins + 2 * lane;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 8
    for (unsigned p = p0 + w; p < p1; p += kWarps) {
        const unsigned slot = cur >= p ? cur - p : cur + a.P - p;  // block k - p
        cmac2(acc, __ldg((const float4 *)&a.fdl[(size_t)slot * a.pitch + b]),
              __ldg((const float4 *)&a.h[(size_t)p * a.pitch + b]));
    }
    red[w][lane] = acc;
    __syncthreads();
    if (w == 0) {
        float4 t = red[0][lane];
#pragma unroll
        for (int q = 1; q < kWarps; q++)
            t = add4(t, red[q][lane]);
        *(float4 *)&a.part[(size_t)g * a.pitch + b] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        flag = atom_add_acq_rel(&a.tickets[3 + x], 1u) == a.G - 1;
    __syncthreads();
    if (!flag)
        return;

    // finish group x: the partials of its range CTAs (all arrived) and
    // partition 0's filter bins load while thread 0 waits for the spectrum
    __shared__ unsigned ready;
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
    for (unsigned q = w; q < a.G; q += kWarps)
        t = add4(t, __ldcg((const float4 *)&a.part[(size_t)q * a.pitch + b]));
    const float4 h0 = __ldg((const float4 *)&a.h[b]);
    red[w][lane] = t;  // red was last read before the ticket
    if (threadIdx.x == 0) {
        // the current spectrum (CTA 0, which waits for nobody)
        const unsigned want = k + 1 + a.wait_skew;
        bool seen = ld_acquire(&a.tickets[2]) == want;
        for (unsigned i = 0; !seen && i < a.wait_polls; i++) {
            __nanosleep(32);
            seen = ld_acquire(&a.tickets[2]) == want;
        }
        ready = seen;
        if (!seen)
            atomicExch(a.err, 1);
    }
    __syncthreads();
    if (ready && w == 0) {
        float4 r = red[0][lane];
#pragma unroll
        for (int q = 1; q < kWarps; q++)
            r = add4(r, red[q][lane]);
        const float4 xv = load_bins_cg(a.xcur, b, a.nb);
        cmac2(r, xv, h0);
        if (b < a.nb)
            a.y[b] = make_float2(r.x * a.s, r.y * a.s);
        if (b + 1 < a.nb)
            a.y[b + 1] = make_float2(r.z * a.s, r.w * a.s);
        *(float4 *)&a.fdl[(size_t)cur * a.pitch + b] = xv;  // slot of block k - P: nobody reads it for block k
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a.tickets[3 + x] = 0;
        flag = atom_add_acq_rel(&a.tickets[1], 1u) == a.groups - 1;
    }
    __syncthreads();
    if (flag) {
        // every group is finished: y is complete (L2-coherent loads)
        if (a.inv_c2r_rows)
            tile_body<M, 16, C, 1, ALONG, ALONG, true, false, false, true>(a.inv, 0, 0, 0, 0, smem);
        else
            tile_body<M, 16, C, 1, ALONG, ALONG, true>(a.inv, 0, 0, 0, 0, smem);
        if (threadIdx.x == 0) {
            a.tickets[1] = 0;  // read again by the next launch only
            a.tickets[0] = k + 1;
        }
    }
}

template <int M> void *block_fn() { return (void *)&upols_block<M>; }

}  // namespace

bool upols_block_supported(int M) { return M >= 64 && M <= 4096 && (M & (M - 1)) == 0; }

size_t upols_block_smem(int M)
{
    switch (M) {
    case 64: return tile_smem_bytes<64, 16, 64, 1, ALONG, ALONG>();
    case 128: return tile_smem_bytes<128, 16, 32, 1, ALONG, ALONG>();
    case 256: return tile_smem_bytes<256, 16, 16, 1, ALONG, ALONG>();
    case 512: return tile_smem_bytes<512, 16, 8, 1, ALONG, ALONG>();
    case 1024: return tile_smem_bytes<1024, 16, 4, 1, ALONG, ALONG>();
    case 2048: return tile_smem_bytes<2048, 16, 2, 1, ALONG, ALONG>();
    case 4096: return tile_smem_bytes<4096, 16, 1, 1, ALONG, ALONG>();
    default: return 0;
    }
}

const void *upols_block_fn(int M)
{
    switch (M) {
    case 64: return block_fn<64>();
    case 128: return block_fn<128>();
    case 256: return block_fn<256>();
    case 512: return block_fn<512>();
    case 1024: return block_fn<1024>();
    case 2048: return block_fn<2048>();
    case 4096: return block_fn<4096>();
    default: return nullptr;
    }
}

cudaError_t launch_upols_block(int M, const UpolsBlockArgs &a, cudaStream_t st)
{
    const void *fn = upols_block_fn(M);
    if (!fn)
        return cudaErrorInvalidValue;
    UpolsBlockArgs args = a;
    void *params[] = {&args};
    const unsigned grid = 1 + a.groups * a.G;
    return cudaLaunchKernel(fn, dim3(grid), dim3(256), params, upols_block_smem(M), st);
}

}  // namespace mgb
